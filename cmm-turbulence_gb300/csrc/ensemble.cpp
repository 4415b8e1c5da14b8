// ensemble.cpp -- see ensemble.hpp.
#include "ensemble.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
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
        fft::plan_destroy(c.pf);
        if (c.real) cudaFree(c.real);
        if (c.spec) cudaFree(c.spec);
        if (c.spec4) cudaFree(c.spec4);
        if (c.freal) cudaFree(c.freal);
        if (c.fw1) cudaFree(c.fw1);
        if (c.fw2) cudaFree(c.fw2);
    }
    if (d_cls_) cudaFree(d_cls_);
    if (d_prof_) cudaFree(d_prof_);
    if (d_rem_) cudaFree(d_rem_);
    if (h_rem_) cudaFreeHost(h_rem_);
    if (d_fsh_) cudaFree(d_fsh_);
    if (h_fsh_) cudaFreeHost(h_fsh_);
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
    // size classes: members with the same vort, psi and fine grids share batched transforms
    std::map<std::pair<std::pair<int, int>, int>, int> idx;
    for (int i = 0; i < M; ++i) {
        EulerSim& s = *m_[(size_t)i];
        auto key = std::make_pair(std::make_pair(s.gv.NX, s.gp.NX), s.gf.NX);
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
    if (fused_mode != 0) {
        int rc = init_fused();
        if (rc) return rc;
    } else {
        fused_why = "off (set before init)";
    }
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
    if (fgraph_) { cudaGraphExecDestroy(fgraph_); fgraph_ = nullptr; }
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
    if (broken_) { err = "an earlier iteration stopped on the device; the ensemble cannot continue"; return kErrState; }
    if (!fused_ok_) return step_two_phase(false);
    // the autotuner: round robin over the candidate forms and shapes, the fastest median after
    const int K = (int)cands_.size();
    const int cand = fused_tuned_ ? -1 : tune_iter_ % K;
    const Shape sh = cand < 0 ? Shape{fused_minb, fused_blocks, fused_g, 0.0} : cands_[(size_t)cand];
    const bool clean = sh.minb != 0 || tuned_;   // the two-phase iteration's first run tunes its kernels
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = sh.minb == 0 ? step_two_phase(true) : step_fused(sh);
    if (rc) return rc;
    if (cand >= 0) {
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (clean) samples_[(size_t)cand].push_back((float)ms);
        tune_iter_++;
        bool enough = true;
        for (auto& v : samples_) enough = enough && v.size() >= 3;
        if (enough) {
            tuning.clear();
            double best = 1e300;
            for (int k = 0; k < K; ++k) {
                std::vector<float> v = samples_[(size_t)k];
                std::sort(v.begin(), v.end());
                Shape t = cands_[(size_t)k];
                t.ms = v[v.size() / 2];
                tuning.push_back(t);
                if (t.ms < best) { best = t.ms; fused_minb = t.minb; fused_blocks = t.blocks; fused_g = t.g; }
            }
            fused_tuned_ = true;
        }
    }
    return 0;
}

int EnsembleSim::remap_launch()
{
    // the remaps ens_middle described, in one launch of the fused kernel's remap stages
    const int M = size();
    ENS_CUDA(cudaMemcpyAsync(d_rem_, h_rem_, sizeof(EnsMember) * M, cudaMemcpyHostToDevice, stream));
    ENS_CUDA(cudaMemsetAsync(d_fsh_, 0, fsh_bytes_, stream));
    EnsFusedArgs a{};
    a.mem = d_rem_;
    a.cls = d_cls_;
    a.M = M;
    a.g = 1;
    a.lpn_log2 = lpn_log2_;
    a.tab_values = tab_values_;
    a.work_values = work_values_;
    a.wait_limit = wait_limit;
    a.sh = reinterpret_cast<EnsShared*>(d_fsh_);
    a.einc = d_einc_;
    a.remapped = reinterpret_cast<int*>(d_fsh_ + sizeof(EnsShared) + sizeof(unsigned long long) * (size_t)M);
    a.remaps_only = 1;
    const Shape& sh = cands_.front();
    ENS_CUDA(launch_ens_fused(ti_, sh.minb, a, sh.blocks, stream));
    ENS_CUDA(cudaMemcpyAsync(h_fsh_, d_fsh_, sizeof(EnsShared), cudaMemcpyDeviceToHost, stream));
    launches++;
    remap_pending_ = true;
    return kOk;
}

int EnsembleSim::step_two_phase(bool batched)
{
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
    int nremap = 0;
    for (int i : stepping_) {
        EnsMember* rem = nullptr;
        if (batched) {
            h_rem_[i] = EnsMember{};
            rem = &h_rem_[i];
        }
        rc = m_[(size_t)i]->ens_middle(h_einc_[i], h_mem_[1][i], rem);
        if (rc) { err = "member " + std::to_string(i) + ": " + m_[(size_t)i]->err; return rc; }
        if (rem && rem->active) nremap++;
    }
    if (batched) {
        for (int i = 0; i < M; ++i)
            if (std::find(stepping_.begin(), stepping_.end(), i) == stepping_.end()) h_rem_[i] = EnsMember{};
        if (nremap && (rc = remap_launch())) return rc;
    }
    // phase B
    if (graphs) { ENS_CUDA(cudaGraphLaunch(graph_[1], stream)); launches += 4 + 2 * (int)cls_.size(); }
    else if ((rc = phase_b())) return rc;
    if (!tuned_) {
        if ((rc = tune({kEnsSampleVort, kEnsSpec, kEnsNodes, kEnsSampleCoarse})) || (rc = phase_b())) return rc;
        tuned_ = true;
    }
    if (remap_pending_) {   // the remap launch's barriers: wait for it, read its status
        remap_pending_ = false;
        ENS_CUDA(cudaStreamSynchronize(stream));
        const EnsShared* sh = reinterpret_cast<const EnsShared*>(h_fsh_);
        if (sh->status != 0) {
            broken_ = true;
            err = "a grid barrier of the batched remap launch gave up waiting after wave " + std::to_string(sh->status - 1) +
                  " (wait limit " + std::to_string(wait_limit) + " polls); the members' states are partial";
            return kErrTimeout;
        }
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

// ---------------------------------------------------------------- single-launch iteration
static long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

int EnsembleSim::init_fused()
{
    // the single-launch iteration where every member and size class allows it; otherwise
    // fused_why says why and the two-phase iteration runs
    const int M = size();
    auto off = [&](const std::string& why) { fused_why = why; fused_ok_ = false; return kOk; };
    if (M > kEnsFusedMaxMembers) return off("more than " + std::to_string(kEnsFusedMaxMembers) + " members");
    if (ti_ != 10 && ti_ != 21 && ti_ != 30) return off("map time integration other than EulerExp, RK2, RK3");
    for (int i = 0; i < M; ++i) {
        std::string why;
        if (!m_[(size_t)i]->ens_fused_check(&why)) return off("member " + std::to_string(i) + ": " + why);
    }
    std::vector<EnsClass> hc(cls_.size());
    int tab = 0, work = 0;
    for (size_t k = 0; k < cls_.size(); ++k) {
        SizeClass& c = cls_[k];
        EulerSim& s0 = *m_[(size_t)c.members[0]];
        const Grid &gv = s0.gv, &gp = s0.gp, &gf = s0.gf;
        const int rc = fft::plan_create(c.pf, gf.NX, gf.NY, false, stream);
        if (rc == -2) { err = "FFT plan creation failed (fine grid)"; return kErrCuda; }
        if (rc) return off("fine-grid transform length not supported");
        if (gv.NX % 2 || gp.NX % 2 || gf.NX % 2) return off("odd grid width");
        const fft::RadixPlan* plans[6] = {&c.pv.rx, &c.pv.ry, &c.pp.rx, &c.pp.ry, &c.pf.rx, &c.pf.ry};
        bool pow2 = true;
        for (const fft::RadixPlan* p : plans) {
            // the launch carries the radix-2/4/8 and radix-3 passes only
            for (int q = 0; q < p->np; ++q) {
                const int r = p->r[q];
                if (r != 2 && r != 3 && r != 4 && r != 8) return off("transform lengths with prime factors above 3");
                pow2 = pow2 && r != 3;
            }
            if (p->n > 1024) return off("transform longer than 1024 points (vort/psi/fine grid above 2048 x 1024)");
        }
        EnsClass& e = hc[k];
        e.v_rx = c.pv.rx; e.v_ry = c.pv.ry; e.p_rx = c.pp.rx; e.p_ry = c.pp.ry; e.f_rx = c.pf.rx; e.f_ry = c.pf.ry;
        e.v_twx = static_cast<const float2*>(c.pv.twx); e.v_twy = static_cast<const float2*>(c.pv.twy);
        e.p_twx = static_cast<const float2*>(c.pp.twx); e.p_twy = static_cast<const float2*>(c.pp.twy);
        e.f_twx = static_cast<const float2*>(c.pf.twx); e.f_twy = static_cast<const float2*>(c.pf.twy);
        e.pow2 = pow2 ? 1 : 0;
        // the psi solve's kept columns (psi::make_layout's rule)
        const double freq = s0.s.freq_cut_psi;
        const int fc = freq >= (double)(1 << 30) ? (1 << 30) : (freq < 0 ? -1 : (int)std::floor(freq));
        e.ncols = std::min(gp.NX / 2, fc) + 1;
        if (e.ncols < 1) return off("psi cut-off below zero");
        e.kv = std::min(gv.NX / 2, e.ncols - 1) + 1;
        e.ld = round_up(e.ncols, 4);
        e.f_ld = round_up(gf.NX / 2 + 1, 4);
        // group shapes: one block_fft call holds kEnsFusedThreads x 8 values
        const int B = kEnsFusedThreads * 8;
        e.nb_frow = std::max(1, B / (gf.NX / 2));
        e.nb_prow = std::max(1, B / (gv.NX / 2));
        e.nb_finv = std::max(1, B / (4 * (gf.NX / 2)));   // the four planes' rows in one call when they fit
        e.nb_pinv = std::max(1, B / (4 * (gp.NX / 2)));
        e.C_f = std::min(8, std::max(1, B / gf.NY));
        e.C_p = std::min(8, std::max(1, B / std::max(gv.NY, gp.NY)));
        int t = 0, w = 0;
        ens_fused_smem_values(e, gv, gp, gf, &t, &w);
        tab = std::max(tab, t);
        work = std::max(work, w);
        // per-member work arrays (128-byte aligned member slots)
        const long long nb = (long long)c.members.size();
        c.freal_stride = round_up(std::max(gf.N, gv.N), 32);
        c.fw1_stride = round_up(std::max((long long)gf.NY * e.f_ld, (long long)gv.NY * e.ld), 16);
        c.fw2_stride = round_up(std::max(4ll * gf.NY * e.f_ld, 4ll * gp.NY * e.ld), 16);
        ENS_CUDA(cudaMalloc((void**)&c.freal, sizeof(float) * c.freal_stride * nb));
        ENS_CUDA(cudaMalloc((void**)&c.fw1, sizeof(float2) * c.fw1_stride * nb));
        ENS_CUDA(cudaMalloc((void**)&c.fw2, sizeof(float2) * c.fw2_stride * nb));
        for (size_t j = 0; j < c.members.size(); ++j)
            m_[(size_t)c.members[j]]->ens_fused_bind((int)k, c.freal + (long long)j * c.freal_stride,
                                                     c.fw1 + (long long)j * c.fw1_stride, c.fw2 + (long long)j * c.fw2_stride);
    }
    tab_values_ = tab;
    work_values_ = work;
    if (sizeof(float2) * (size_t)(tab + work) > 180 * 1024) return off("transform work does not fit in shared memory");
    ENS_CUDA(cudaMalloc((void**)&d_cls_, sizeof(EnsClass) * hc.size()));
    ENS_CUDA(cudaMemcpyAsync(d_cls_, hc.data(), sizeof(EnsClass) * hc.size(), cudaMemcpyHostToDevice, stream));
    fsh_bytes_ = sizeof(EnsShared) + (sizeof(unsigned long long) + sizeof(int)) * (size_t)M;
    ENS_CUDA(cudaMalloc((void**)&d_fsh_, fsh_bytes_));
    ENS_CUDA(cudaMallocHost((void**)&h_fsh_, fsh_bytes_));
    EnsFusedArgs a{};
    a.M = M;
    a.tab_values = tab_values_;
    a.work_values = work_values_;
    int dev = 0;
    ENS_CUDA(cudaGetDevice(&dev));
    ENS_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
    // autotuner candidates: register budget (64 registers for 4 resident blocks per SM, 40 for
    // 6) x resident blocks per SM x 256-thread tiles (or transform groups) per task
    cands_.clear();
    for (int minb : {4, 6}) {
        const int occ = ens_fused_blocks_per_sm(ti_, minb, a);
        for (int k = minb - 1; k <= std::min(occ, minb); ++k)
            for (int g : {2, 4, 8}) cands_.push_back(Shape{minb, k * sms_, g, 0.0});
    }
    if (cands_.empty()) return off("the launch does not fit on a multiprocessor");
    std::sort(cands_.begin(), cands_.end(), [](const Shape& x, const Shape& y) {   // the widest shape first
        return x.blocks != y.blocks ? x.blocks > y.blocks : x.g > y.g;
    });
    if (fused_mode == 2) cands_.push_back(Shape{0, 0, 0, 0.0});   // the two-phase iteration, batched remaps
    ENS_CUDA(cudaMallocHost((void**)&h_rem_, sizeof(EnsMember) * M));
    ENS_CUDA(cudaMalloc((void**)&d_rem_, sizeof(EnsMember) * M));
    samples_.assign(cands_.size(), std::vector<float>());
    tune_iter_ = 0;
    fused_tuned_ = false;
    fused_minb = cands_.front().minb;
    fused_blocks = cands_.front().blocks;
    fused_g = cands_.front().g;
    ENS_CUDA(cudaStreamSynchronize(stream));
    fused_ok_ = true;
    fused_why.clear();
    return kOk;
}

void EnsembleSim::set_wait_limit(long long polls)
{
    wait_limit = polls < 0 ? 0 : polls;
    if (fgraph_) { cudaGraphExecDestroy(fgraph_); fgraph_ = nullptr; }   // the limit is baked into the graph
}

int EnsembleSim::set_profiling(bool on)
{
    if (fgraph_) { cudaGraphExecDestroy(fgraph_); fgraph_ = nullptr; }   // the counters' address is baked into the graph
    if (!on) {
        if (d_prof_) cudaFree(d_prof_);
        d_prof_ = nullptr;
        return kOk;
    }
    if (!d_prof_) ENS_CUDA(cudaMalloc((void**)&d_prof_, sizeof(unsigned long long) * kProfValues));
    ENS_CUDA(cudaMemsetAsync(d_prof_, 0, sizeof(unsigned long long) * kProfValues, stream));
    return kOk;
}

int EnsembleSim::read_profile(unsigned long long* out)
{
    if (!d_prof_) { err = "profiling is off"; return kErrState; }
    ENS_CUDA(cudaMemcpyAsync(out, d_prof_, sizeof(unsigned long long) * kProfValues, cudaMemcpyDeviceToHost, stream));
    ENS_CUDA(cudaStreamSynchronize(stream));
    return kOk;
}

int EnsembleSim::fused_sequence(const Shape& sh)
{
    const int M = size();
    ENS_CUDA(cudaMemcpyAsync(d_mem_[0], h_mem_[0], sizeof(EnsMember) * M, cudaMemcpyHostToDevice, stream));
    ENS_CUDA(cudaMemsetAsync(d_fsh_, 0, fsh_bytes_, stream));
    EnsFusedArgs a{};
    a.mem = d_mem_[0];
    a.cls = d_cls_;
    a.M = M;
    a.g = sh.g;
    a.lpn_log2 = lpn_log2_;
    a.tab_values = tab_values_;
    a.work_values = work_values_;
    a.wait_limit = wait_limit;
    a.sh = reinterpret_cast<EnsShared*>(d_fsh_);
    a.einc = reinterpret_cast<unsigned long long*>(d_fsh_ + sizeof(EnsShared));
    a.remapped = reinterpret_cast<int*>(d_fsh_ + sizeof(EnsShared) + sizeof(unsigned long long) * (size_t)M);
    a.prof = d_prof_;
    ENS_CUDA(launch_ens_fused(ti_, sh.minb, a, sh.blocks, stream));
    ENS_CUDA(cudaMemcpyAsync(h_fsh_, d_fsh_, fsh_bytes_, cudaMemcpyDeviceToHost, stream));
    return kOk;
}

int EnsembleSim::step_fused(const Shape& shape)
{
    const int M = size();
    stepping_.clear();
    int rc;
    for (int i = 0; i < M; ++i) {
        EnsMember& e = h_mem_[0][i];
        e = EnsMember{};
        rc = m_[(size_t)i]->ens_begin(e);
        if (rc < 0) { err = "member " + std::to_string(i) + ": " + m_[(size_t)i]->err; return rc; }
        if (rc == 0) {
            stepping_.push_back(i);
            if ((rc = m_[(size_t)i]->ens_fused_prepare(e))) {
                err = "member " + std::to_string(i) + ": " + m_[(size_t)i]->err;
                return rc;
            }
        }
    }
    if (stepping_.empty()) return 1;
    // once tuned, the iteration is one CUDA graph (descriptors up, state zeroed, the launch, results down)
    if (fused_tuned_ && use_graphs) {
        if (!fgraph_) {
            cudaGraph_t gr = nullptr;
            ENS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            rc = fused_sequence(shape);
            cudaError_t e = cudaStreamEndCapture(stream, &gr);
            if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
            ENS_CUDA(e);
            e = cudaGraphInstantiate(&fgraph_, gr, 0);
            cudaGraphDestroy(gr);
            ENS_CUDA(e);
        }
        ENS_CUDA(cudaGraphLaunch(fgraph_, stream));
    } else if ((rc = fused_sequence(shape))) {
        return rc;
    }
    launches++;
    ENS_CUDA(cudaStreamSynchronize(stream));
    const EnsShared* sh = reinterpret_cast<const EnsShared*>(h_fsh_);
    if (sh->status != 0) {
        broken_ = true;
        err = "a grid barrier of the batched iteration gave up waiting after wave " + std::to_string(sh->status - 1) +
              " (wait limit " + std::to_string(wait_limit) + " polls); the members' states are partial";
        return kErrTimeout;
    }
    last_waves = sh->waves;
    const unsigned long long* einc = reinterpret_cast<const unsigned long long*>(h_fsh_ + sizeof(EnsShared));
    const int* remapped = reinterpret_cast<const int*>(h_fsh_ + sizeof(EnsShared) + sizeof(unsigned long long) * (size_t)M);
    for (int i : stepping_) {
        double ei;
        std::memcpy(&ei, einc + i, sizeof(double));
        EulerSim& s = *m_[(size_t)i];
        rc = s.ens_fused_finish(ei, remapped[i] != 0);
        if (!rc) rc = s.ens_end();
        if (rc && rc != kErrSaturated) { err = "member " + std::to_string(i) + ": " + s.err; return rc; }
        member_steps++;
    }
    iterations++;
    return 0;
}

}  // namespace cmm
