// ensemble.cpp -- see ensemble.hpp.
#include "ensemble.hpp"

#include <algorithm>
#include <map>

namespace cmm {

EnsembleSim::EnsembleSim(const std::vector<Settings>& members)
{
    for (auto& st : members) m_.emplace_back(new EulerSim(st));
}

EnsembleSim::~EnsembleSim()
{
    drop_graphs();
    for (auto& c : cls_) {
        fft::plan_destroy(c.pv);
        fft::plan_destroy(c.pp);
        if (c.real) cudaFree(c.real);
        if (c.spec) cudaFree(c.spec);
        if (c.spec4) cudaFree(c.spec4);
    }
    for (auto& p : d_cum_) if (p) cudaFree(p);
    for (int k = 0; k < 2; ++k) {
        if (d_mem_[k]) cudaFree(d_mem_[k]);
        if (h_mem_[k]) cudaFreeHost(h_mem_[k]);
    }
    if (d_einc_) cudaFree(d_einc_);
    if (h_einc_) cudaFreeHost(h_einc_);
    m_.clear();   // members before the stream they use
    if (own_stream_ && stream) cudaStreamDestroy(stream);
}

int EnsembleSim::check(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return kOk;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return kErrCuda;
}

#define ENS_CUDA(x) do { int rc_ = check((x), #x); if (rc_) return rc_; } while (0)

int EnsembleSim::set_initial_discrete(int i, const double* host, size_t n)
{
    if (i < 0 || i >= size()) { err = "no member " + std::to_string(i); return kErrParam; }
    int rc = m_[(size_t)i]->set_initial_discrete(host, n);
    if (rc) err = m_[(size_t)i]->err;
    return rc;
}

bool EnsembleSim::done() const
{
    for (auto& p : m_) if (!p->done()) return false;
    return true;
}

int EnsembleSim::init()
{
    if (initialised_) { err = "init called twice"; return kErrState; }
    if (m_.empty()) { err = "an ensemble needs members"; return kErrParam; }
    if (!stream) {
        ENS_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream_ = true;
    }
    const int M = size();
    for (int i = 0; i < M; ++i) {
        EulerSim& s = *m_[(size_t)i];
        s.set_stream(stream);
        int rc = s.init();
        if (rc) { err = "member " + std::to_string(i) + ": " + s.err; return rc; }
        std::string why;
        if (!s.ens_check(&why)) { err = "member " + std::to_string(i) + ": " + why; return kErrUnsupported; }
        if (i == 0) {
            ti_ = s.s.time_integration_num;
            lpn_log2_ = s.s.map_update_order_num <= 1 ? 3 : 4;
        } else if (s.s.time_integration_num != ti_ || (s.s.map_update_order_num <= 1 ? 3 : 4) != lpn_log2_) {
            err = "ensemble members share the map time integration and update order";
            return kErrParam;
        }
    }
    // size classes: members with the same vort and psi grids share batched transforms
    std::map<std::pair<int, int>, int> idx;
    for (int i = 0; i < M; ++i) {
        EulerSim& s = *m_[(size_t)i];
        auto key = std::make_pair(s.gv.NX, s.gp.NX);
        if (!idx.count(key)) {
            idx[key] = (int)cls_.size();
            SizeClass c;
            c.nv = s.gv.NX;
            c.np = s.gp.NX;
            cls_.push_back(c);
        }
        cls_[(size_t)idx[key]].members.push_back(i);
    }
    ENS_CUDA(cudaMalloc((void**)&d_einc_, sizeof(unsigned long long) * M));
    ENS_CUDA(cudaMallocHost((void**)&h_einc_, sizeof(double) * M));
    for (auto& c : cls_) {
        EulerSim& s0 = *m_[(size_t)c.members[0]];
        const long long nb = (long long)c.members.size();
        c.real_stride = std::max(s0.gv.N, 4 * s0.gp.N);
        c.spec_stride = s0.gv.Nfft;
        c.spec4_stride = 4 * s0.gp.Nfft;
        ENS_CUDA(cudaMalloc((void**)&c.real, sizeof(float) * c.real_stride * nb));
        ENS_CUDA(cudaMalloc((void**)&c.spec, sizeof(float2) * c.spec_stride * nb));
        ENS_CUDA(cudaMalloc((void**)&c.spec4, sizeof(float2) * c.spec4_stride * nb));
        // R2C: one transform per member (input stride real_stride, output stride Nv_fft);
        // C2R: four per member (input stride Np_fft, output stride Np, members contiguous)
        if (fft::plan_create(c.pv, s0.gv.NX, s0.gv.NY, false, stream) ||
            fft::plan_create(c.pp, s0.gp.NX, s0.gp.NY, false, stream)) {
            err = "FFT plan creation failed (ensemble size class)";
            return kErrCuda;
        }
        for (size_t k = 0; k < c.members.size(); ++k) {
            const int i = c.members[k];
            // one buffer, two views: member k's vort-grid sample at real + k real_stride (R2C
            // input) and its four psi planes at real + k 4 Np (C2R output, 4 transforms per
            // member back to back); the R2C has consumed every sample before the C2R writes
            m_[(size_t)i]->ens_bind(c.real + (long long)k * c.real_stride, c.spec + (long long)k * c.spec_stride,
                                    c.spec4 + (long long)k * c.spec4_stride, c.real + (long long)k * 4 * s0.gp.N,
                                    d_einc_ + i);
        }
    }
    // work lists: tiles of 256 threads per member and kernel kind
    std::vector<int> cum((size_t)M + 1);
    for (int kind = 0; kind < kEnsKinds; ++kind) {
        cum[0] = 0;
        for (int i = 0; i < M; ++i) {
            EulerSim& s = *m_[(size_t)i];
            long long items = 0;
            switch (kind) {
                case kEnsAdvect: items = s.gc.N << lpn_log2_; break;
                case kEnsIncomp: items = s.gc.N * (s.gf.NX / s.gc.NX); break;
                case kEnsSampleVort: items = s.gv.N; break;
                case kEnsSampleCoarse: items = s.gc.N; break;
                case kEnsSpec: items = (long long)s.gp.NX_fft * s.gp.NY; break;
                default: items = s.gp.N; break;
            }
            const long long t = (items + 255) / 256;
            if ((long long)cum[(size_t)i] + t > 0x7fffffffLL) { err = "ensemble work list too long"; return kErrParam; }
            cum[(size_t)i + 1] = cum[(size_t)i] + (int)t;
        }
        tiles[kind] = cum[(size_t)M];
        blocks[kind] = std::min(tiles[kind], 152 * 8);
        ENS_CUDA(cudaMalloc((void**)&d_cum_[kind], sizeof(int) * (M + 1)));
        ENS_CUDA(cudaMemcpyAsync(d_cum_[kind], cum.data(), sizeof(int) * (M + 1), cudaMemcpyHostToDevice, stream));
    }
    for (int k = 0; k < 2; ++k) {
        ENS_CUDA(cudaMallocHost((void**)&h_mem_[k], sizeof(EnsMember) * M));
        ENS_CUDA(cudaMalloc((void**)&d_mem_[k], sizeof(EnsMember) * M));
        std::fill(h_mem_[k], h_mem_[k] + M, EnsMember{});
    }
    ENS_CUDA(cudaStreamSynchronize(stream));
    initialised_ = true;
    return kOk;
}

int EnsembleSim::launch(int kind, int blocks_now)
{
    launches++;
    const bool a = kind == kEnsPrecombine || kind == kEnsAdvect || kind == kEnsIncomp;
    return check(launch_ens(kind, ti_, d_mem_[a ? 0 : 1], d_cum_[kind], size(), blocks_now, lpn_log2_, stream),
                 "launch_ens");
}

int EnsembleSim::phase_a()
{
    const int M = size();
    int rc;
    ENS_CUDA(cudaMemcpyAsync(d_mem_[0], h_mem_[0], sizeof(EnsMember) * M, cudaMemcpyHostToDevice, stream));
    ENS_CUDA(cudaMemsetAsync(d_einc_, 0, sizeof(unsigned long long) * M, stream));
    if ((rc = launch(kEnsPrecombine, blocks[kEnsPrecombine])) || (rc = launch(kEnsAdvect, blocks[kEnsAdvect])) ||
        (rc = launch(kEnsIncomp, blocks[kEnsIncomp])))
        return rc;
    ENS_CUDA(cudaMemcpyAsync(h_einc_, d_einc_, sizeof(double) * M, cudaMemcpyDeviceToHost, stream));
    return kOk;
}

int EnsembleSim::phase_b()
{
    const int M = size();
    int rc;
    ENS_CUDA(cudaMemcpyAsync(d_mem_[1], h_mem_[1], sizeof(EnsMember) * M, cudaMemcpyHostToDevice, stream));
    if ((rc = launch(kEnsSampleVort, blocks[kEnsSampleVort]))) return rc;
    for (auto& c : cls_) {
        if (!c.active) continue;
        launches += 2;   // row pass + column pass
        const int nb = (int)c.members.size();
        if ((rc = check(fft::r2c(c.pv, c.real, c.spec, nb, stream, c.real_stride, c.spec_stride), "FFT R2C (ensemble)")))
            return rc;
    }
    if ((rc = launch(kEnsSpec, blocks[kEnsSpec]))) return rc;
    for (auto& c : cls_) {
        if (!c.active) continue;
        launches += 2;
        const int nb = (int)c.members.size();
        if ((rc = check(fft::c2r(c.pp, c.spec4, c.real, 4 * nb, stream), "FFT C2R (ensemble)"))) return rc;
    }
    if ((rc = launch(kEnsNodes, blocks[kEnsNodes])) || (rc = launch(kEnsSampleCoarse, blocks[kEnsSampleCoarse])))
        return rc;
    return kOk;
}

int EnsembleSim::tune(const std::vector<int>& kinds)
{
    // time each batched kernel at each candidate grid on this iteration's real data and keep
    // the fastest.  Called for phase A's kernels right after phase A (the maps, levels and
    // combinations they read are unchanged, and what they write they write again with the
    // same values) and for phase B's right after phase B (the vort-sample trials overwrite the
    // class buffers that hold the psi planes, so the caller runs phase B once more)
    cudaEvent_t e0, e1;
    ENS_CUDA(cudaEventCreate(&e0));
    ENS_CUDA(cudaEventCreate(&e1));
    const int cand[] = {152, 304, 608, 1216, 2432, 4864, 9728};
    int rc = kOk;
    for (int kind : kinds) {
        float best = 1e30f;
        int pick = blocks[kind];
        for (int c : cand) {
            const int b = std::min(c, tiles[kind]);
            for (int rep = 0; rep < 2 && !rc; ++rep) {   // the first run warms the caches
                if (kind == kEnsIncomp) rc = check(cudaMemsetAsync(d_einc_, 0, sizeof(unsigned long long) * size(), stream), "memset");
                if (!rc) rc = check(cudaEventRecord(e0, stream), "event");
                if (!rc) rc = launch(kind, b);
                if (!rc) rc = check(cudaEventRecord(e1, stream), "event");
            }
            if (!rc) rc = check(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float ms = 0;
            if (!rc) rc = check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
            if (rc) break;
            if (ms < best) { best = ms; pick = b; }
            if (b == tiles[kind]) break;
        }
        if (rc) break;
        blocks[kind] = pick;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

void EnsembleSim::drop_graphs()
{
    for (auto& g : graph_)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

int EnsembleSim::capture(int which, cudaGraphExec_t* exec)
{
    cudaGraph_t g = nullptr;
    ENS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    long long before = launches;
    int rc = which == 0 ? phase_a() : phase_b();
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    launches = before;
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    ENS_CUDA(e);
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    return check(e, "cudaGraphInstantiate");
}

int EnsembleSim::step()
{
    if (!initialised_) { err = "step before init"; return kErrState; }
    const int M = size();
    stepping_.clear();
    int rc;
    for (int i = 0; i < M; ++i) {
        EnsMember& e = h_mem_[0][i];
        e = EnsMember{};
        rc = m_[(size_t)i]->ens_begin(e);
        if (rc < 0) { err = "member " + std::to_string(i) + ": " + m_[(size_t)i]->err; return rc; }
        if (rc == 0) stepping_.push_back(i);
    }
    if (stepping_.empty()) return 1;
    // a size class whose members are all done drops out of the transforms (and the graphs)
    for (auto& c : cls_) {
        bool any = false;
        for (int i : c.members) any = any || h_mem_[0][i].active;
        if (c.active && !any) { c.active = false; drop_graphs(); }
    }
    const bool graphs = use_graphs && tuned_;
    if (graphs && !graph_[0]) {
        if ((rc = capture(0, &graph_[0])) || (rc = capture(1, &graph_[1]))) return rc;
    }
    // phase A
    if (graphs) { ENS_CUDA(cudaGraphLaunch(graph_[0], stream)); launches += 3; }
    else if ((rc = phase_a())) return rc;
    ENS_CUDA(cudaStreamSynchronize(stream));
    if (!tuned_ && (rc = tune({kEnsPrecombine, kEnsAdvect, kEnsIncomp}))) return rc;
    for (int i = 0; i < M; ++i) h_mem_[1][i] = h_mem_[0][i];
    for (int i : stepping_) {
        rc = m_[(size_t)i]->ens_middle(h_einc_[i], h_mem_[1][i]);
        if (rc) { err = "member " + std::to_string(i) + ": " + m_[(size_t)i]->err; return rc; }
    }
    // phase B
    if (graphs) { ENS_CUDA(cudaGraphLaunch(graph_[1], stream)); launches += 4 + 2 * (int)cls_.size(); }
    else if ((rc = phase_b())) return rc;
    if (!tuned_) {
        if ((rc = tune({kEnsSampleVort, kEnsSpec, kEnsNodes, kEnsSampleCoarse})) || (rc = phase_b())) return rc;
        tuned_ = true;
    }
    for (int i : stepping_) {
        rc = m_[(size_t)i]->ens_end();
        if (rc && rc != kErrSaturated) { err = "member " + std::to_string(i) + ": " + m_[(size_t)i]->err; return rc; }
        member_steps++;
    }
    iterations++;
    return 0;
}

int EnsembleSim::run()
{
    int rc;
    while ((rc = step()) == 0) {}
    if (rc != 1) return rc;
    for (auto& p : m_) {
        rc = p->finish();
        if (rc) { err = p->err; return rc; }
    }
    return kOk;
}

}  // namespace cmm
