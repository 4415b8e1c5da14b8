// sim.cpp -- see sim.hpp.  Host orchestration of one Euler-2D CMM run:
// reference driver src/simulation/cmm-euler2d.cu:45-1099 and host layer
// src/simulation/cmm-simulation-host.cu.
#include "sim.hpp"

#include "mixed.hpp"

#include <cuda_runtime.h>
#include <curand.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>

namespace cmm {

namespace {
// get_L_coefficient (src/numerical/cmm-timestep.cu:474-484)
double lagrange_coefficient(const double* t, double t_next, int loop_ctr, int i_point, int l_order)
{
    double c = 1;
    for (int i_p = 0; i_p < l_order; ++i_p)
        if (i_p != i_point) c *= (t_next - t[loop_ctr - i_p]) / (t[loop_ctr - i_point] - t[loop_ctr - i_p]);
    return c;
}

bool has(const std::string& s, const char* k) { return s.find(k) != std::string::npos; }

std::string two(int i)
{
    char b[16];
    snprintf(b, sizeof(b), "%02d", i);
    return b;
}
}  // namespace

EulerSim::EulerSim(const Settings& st) : s(st) {}

EulerSim::~EulerSim()
{
    flush_monitor();
    learned_release();
    set_profiling(false);
    release();
}

const char* EulerSim::phase_name(int p)
{
    static const char* n[kNumPhases] = {"advect", "incomp", "remap", "psi", "coarse", "particles", "save"};
    return p >= 0 && p < kNumPhases ? n[p] : "";
}

void EulerSim::set_profiling(bool on)
{
    if (on && !prof_) {
        for (int p = 0; p < kNumPhases; ++p) {
            cudaEventCreate(&ev_[p][0]);
            cudaEventCreate(&ev_[p][1]);
            prof_ms[p] = 0;
            prof_count[p] = 0;
        }
    } else if (!on && prof_) {
        for (int p = 0; p < kNumPhases; ++p) {
            cudaEventDestroy(ev_[p][0]);
            cudaEventDestroy(ev_[p][1]);
        }
    }
    prof_ = on;
}

void EulerSim::ph_begin(int p)
{
    if (prof_) cudaEventRecord(ev_[p][0], stream);
}

void EulerSim::ph_end(int p)
{
    if (!prof_) return;
    cudaEventRecord(ev_[p][1], stream);
    ev_live_[p] = true;
}

void EulerSim::ph_collect()
{
    // one stream sync per profiled iteration; events of each phase timed once
    if (!prof_) return;
    cudaStreamSynchronize(stream);
    for (int p = 0; p < kNumPhases; ++p) {
        if (!ev_live_[p]) continue;
        float ms = 0;
        if (cudaEventElapsedTime(&ms, ev_[p][0], ev_[p][1]) == cudaSuccess) {
            prof_ms[p] += ms;
            prof_count[p] += 1;
        }
        ev_live_[p] = false;
    }
}

int EulerSim::check(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return kOk;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return kErrCuda;
}

#define CMM_CUDA(call) do { int rc_ = check((call), #call); if (rc_) return rc_; } while (0)
#define CMM_LAUNCH(k, call) do { kernel_launches += (k); int rc_ = check((call), #call); if (rc_) return rc_; } while (0)
#define CMM_FFT(call) do { fft_calls++; cudaError_t e_ = (call); if (e_ != cudaSuccess) { err = std::string("FFT: ") + #call + ": " + cudaGetErrorString(e_); return kErrCuda; } } while (0)

double EulerSim::wall() const
{
    return std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - begin_).count() / 1e6;
}

int EulerSim::set_stream(cudaStream_t st)
{
    if (initialised_) { err = "set_stream after init"; return kErrState; }
    stream = st;
    own_stream_ = false;
    return kOk;
}

int EulerSim::set_initial_discrete(const double* host, size_t n)
{
    if (initialised_) { err = "set_initial_discrete after init"; return kErrState; }
    size_t need = (size_t)s.initial_discrete_grid * s.initial_discrete_grid;
    if (n != need) { err = "discrete initial condition needs initial_discrete_grid^2 values"; return kErrParam; }
    host_discrete_.assign(host, host + n);
    return kOk;
}

int EulerSim::alloc()
{
    if (s.simulation_type != "cmm_euler_2d" && s.simulation_type != "cmm_vlasov_poisson_1d") {
        err = "unknown simulation_type " + s.simulation_type;
        return kErrParam;
    }
    vlasov_ = s.simulation_type == "cmm_vlasov_poisson_1d";
    if (s.initial_condition_num < 0) { err = "unknown initial condition " + s.initial_condition; return kErrParam; }
    auto levels_needed = [](int ti) {
        // Lagrange levels a scheme reads (settings.cu time-integration table)
        switch (ti) {
            case 10: return 1;
            case 20: case 21: return 2;
            case 30: case 31: return 3;
            case 40: case 41: return 4;
            default: return -1;
        }
    };
    if (levels_needed(s.time_integration_num) < 0) {
        err = "unknown map time integration " + s.time_integration;
        return kErrParam;
    }
    if (s.map_update_order_num < 0) { err = "unknown map_update_order " + s.map_update_order; return kErrParam; }
    if (s.scalar_discrete && !s.initial_discrete) {
        err = "scalar_discrete samples the discrete initial vorticity (as the reference does): it needs initial_discrete=1";
        return kErrUnsupported;
    }
    if (s.forward_map && s.precision == "mixed" && s.simulation_type == "cmm_vlasov_poisson_1d") {
        err = "forward_map with precision=mixed is built for 2D Euler (Vlasov-Poisson: precision=fp64)";
        return kErrUnsupported;
    }
    if (s.grid_coarse <= 0 || s.grid_fine <= 0 || s.grid_psi <= 0 || s.grid_vort <= 0) { err = "grid sizes must be positive"; return kErrParam; }

    dt = s.dt();
    L = s.effective_lagrange_order();
    if (L < 1 || L > kMaxLagrange) { err = "lagrange order out of range"; return kErrParam; }
    if (L < levels_needed(s.time_integration_num)) {
        err = "map time integration " + s.time_integration + " needs lagrange order >= " +
              std::to_string(levels_needed(s.time_integration_num));
        return kErrParam;
    }
    for (auto& p : s.particles_advected) {
        int need = p.time_integration_num == 20 ? 2 : levels_needed(p.time_integration_num);
        if (need < 0 || p.time_integration_num == 21) {
            err = "unknown particle time integration " + p.time_integration;
            return kErrParam;
        }
        if (L < need) {
            err = "particle time integration " + p.time_integration + " needs lagrange order >= " + std::to_string(need);
            return kErrParam;
        }
    }
    s.lagrange_order = L;
    s.file_name = s.derived_file_name();
    max_maps = s.cpu_map_num();
    if (s.precision == "mixed") {
        // the mixed kernels address every grid as integer multiples of the map grid
        bool ratios = s.grid_psi % s.grid_coarse == 0 && s.grid_vort % s.grid_coarse == 0 &&
                      s.grid_fine % s.grid_vort == 0 && s.grid_fine % s.grid_coarse == 0;
        if (!ratios) { err = "precision=mixed needs psi, vort and fine grids that are integer multiples of the map grid"; return kErrUnsupported; }
        if (s.molly_stencil != 0) { err = "precision=mixed does not build mollified sampling"; return kErrUnsupported; }
        if (vlasov_) {
            // the separable-psi kernels of the mixed Vlasov form carry EulerExp, Heun and RK3
            bool ok = s.time_integration_num == 10 || s.time_integration_num == 21 || s.time_integration_num == 30;
            for (auto& p : s.particles_advected)
                ok = ok && p.tau == 0 && (p.time_integration_num == 10 || p.time_integration_num == 20 ||
                                          p.time_integration_num == 30);
            if (!ok) {
                err = "precision=mixed for Vlasov-Poisson builds EulerExp, Heun and RK3 maps and fluid tracers only";
                return kErrUnsupported;
            }
        }
        mixed_ = true;
    } else if (s.precision != "fp64") {
        err = "precision must be fp64 or mixed";
        return kErrParam;
    }

    if (vlasov_) {
        // the Vlasov driver states its domain in units of pi (cmm-vlasov1d.cu:72)
        for (int i = 0; i < 4; ++i) s.domain_bounds[i] *= kTwoPi / 2;
        if (s.grid_vort > s.grid_psi) {
            // calc_phi's restriction (cmm-simulation-host.cu:457-460)
            err = "vorticity grid should be smaller than phi_out grid (grid_vort > grid_psi)";
            return kErrParam;
        }
    }
    const double* b = s.domain_bounds;
    gc = make_grid(s.grid_coarse, s.grid_coarse, b);
    gf = make_grid(s.grid_fine, s.grid_fine, b);
    gp = make_grid(s.grid_psi, s.grid_psi, b);
    gv = make_grid(s.grid_vort, s.grid_vort, b);
    int nd = s.initial_discrete ? s.initial_discrete_grid : 1;
    gd = make_grid(nd, nd, b);

    if (!stream) {
        CMM_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream_ = true;
    }
    auto dalloc = [&](double** p, long long n) { return check(cudaMalloc((void**)p, sizeof(double) * (size_t)std::max(n, 1ll)), "cudaMalloc"); };
    int rc;
    if ((rc = dalloc(&ChiX, 4 * gc.N)) || (rc = dalloc(&ChiY, 4 * gc.N)) || (rc = dalloc(&ChiX_new, 4 * gc.N)) ||
        (rc = dalloc(&ChiY_new, 4 * gc.N)) || (rc = dalloc(&vort, gc.N)) || (rc = dalloc(&wfine, 4 * gf.N)))
        return rc;
    for (int l = 0; l < L; ++l) if ((rc = dalloc(&psi[l], 4 * gp.N))) return rc;
    if (s.initial_discrete && (rc = dalloc(&wdisc, 4 * gd.N))) return rc;
    if (s.forward_map) {
        if ((rc = dalloc(&ChiX_f, 4 * gc.N)) || (rc = dalloc(&ChiY_f, 4 * gc.N))) return rc;
        for (auto& p : s.particles_forwarded) {
            double* d = nullptr;
            if ((rc = dalloc(&d, 2ll * std::max(p.num, 1)))) return rc;
            fparts_.push_back(d);
        }
        init_map_.assign(s.particles_forwarded.size(), 0);
        long long tot = 0;
        for (auto& p : s.particles_forwarded) tot += std::max(p.num, 0);
        if ((rc = dalloc(&fpos_, 2 * std::max(tot, 1ll)))) return rc;
    }
    stack_cap_ = std::max(0, std::min(max_maps, 16));
    if (!mixed_ && stack_cap_ > 0 && (rc = dalloc(&stack, 8 * gc.N * stack_cap_))) return rc;
    if (s.forward_map && stack_cap_ > 0 && (rc = dalloc(&stack_f, 8 * gc.N * stack_cap_))) return rc;
    long long rmax = std::max({gf.N, gv.N, gd.N, gc.N, gp.N});
    long long cmax = std::max({gf.Nfft, gv.Nfft, gd.Nfft, gc.Nfft, gp.Nfft});
    if ((rc = dalloc(&real_buf_, rmax))) return rc;
    CMM_CUDA(cudaMalloc((void**)&spec_, sizeof(double2) * (size_t)cmax));
    CMM_CUDA(cudaMalloc((void**)&spec4_, sizeof(double2) * 4 * (size_t)cmax));
    if ((rc = dalloc(&red_, 3 * kReduceBlocks)) || (rc = dalloc(&d_scal_, 16)) || (rc = dalloc(&d_einc2_, 2)) ||
        (rc = dalloc(&d_params_, 10)) ||
        (rc = dalloc(&d_rand_, kInitTable)))
        return rc;
    CMM_CUDA(cudaMemsetAsync(d_einc2_, 0, sizeof(double) * 2, stream));
    einc_slot_ = 0;
    CMM_CUDA(cudaMallocHost((void**)&h_scal_, sizeof(double) * 16));
    CMM_CUDA(cudaEventCreateWithFlags(&einc_ev_, cudaEventDisableTiming));
    CMM_CUDA(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming));
    CMM_CUDA(cudaEventCreateWithFlags(&join_ev_, cudaEventDisableTiming));
    CMM_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
    for (auto& p : s.particles_advected) {
        double* d = nullptr;
        if ((rc = dalloc(&d, 2ll * std::max(p.num, 1)))) return rc;
        parts.push_back(d);
        double* v = nullptr;
        if (p.tau != 0 && (rc = dalloc(&v, 2ll * std::max(p.num, 1)))) return rc;
        vels.push_back(v);
    }
    if (!make_plans(pf_, gf, stream) || !make_plans(pv_, gv, stream) || !make_plans(pp_, gp, stream) ||
        !make_plans(pc_, gc, stream) || (s.initial_discrete && !make_plans(pd_, gd, stream))) {
        err = "FFT plan creation failed (grid sizes need NX even, sides <= 8192, prime factors <= 13)";
        return kErrCuda;
    }
    if (vlasov_) {
        for (int l = 0; l < L; ++l) if ((rc = dalloc(&phi_lv_[l], 2 * (long long)gp.NX))) return rc;
        long long nchunks = (gv.NY + kVlasovRowChunk - 1) / kVlasovRowChunk;
        if ((rc = dalloc(&vl_h_, 2 * (long long)gp.NY)) || (rc = dalloc(&vl_rho_, gv.NX)) ||
            (rc = dalloc(&vl_part_, nchunks * gv.NX)))
            return rc;
        int cn = std::max(gv.NX_fft, gp.NX_fft);
        for (int k = 0; k < 3; ++k) CMM_CUDA(cudaMalloc((void**)&vl_c_[k], sizeof(double2) * cn));
        if (mixed_)
            for (int k = 0; k < 4; ++k) CMM_CUDA(cudaMalloc((void**)&vtab_[k], sizeof(double2) * std::max(gp.NX, gp.NY)));
        if (!make_vlasov_plans(vp_, gv, gp, stream)) { err = "FFT plan creation failed (1D, Vlasov)"; return kErrParam; }
    }
    if (mixed_) {
        auto falloc = [&](void** p, size_t bytes) { return check(cudaMalloc(p, std::max(bytes, (size_t)16)), "cudaMalloc"); };
        size_t mapb = sizeof(float4) * 2 * (size_t)gc.N, psib = sizeof(float4) * (size_t)gp.N;
        if ((rc = falloc((void**)&mapm_, mapb)) || (rc = falloc((void**)&mapm_new_, mapb)) ||
            (rc = falloc((void**)&psiA_, psib)) || (rc = falloc((void**)&psiB_, psib)) ||
            (rc = falloc((void**)&psiP_, psib)) ||
            (rc = falloc((void**)&wfm_, sizeof(float4) * (size_t)gf.N)) ||
            (rc = falloc((void**)&realf_, sizeof(float) * 4 * (size_t)std::max({gv.N, gp.N, gf.N}))) ||
            (rc = falloc((void**)&specf_, sizeof(float2) * (size_t)std::max(gv.Nfft, gf.Nfft))) ||
            (rc = falloc((void**)&spec4f_, sizeof(float2) * 4 * (size_t)std::max(gp.Nfft, gf.Nfft))))
            return rc;
        for (int l = 0; l < L; ++l) if ((rc = falloc((void**)&psim_[l], psib))) return rc;
        if (s.initial_discrete && (rc = falloc((void**)&wdiscm_, sizeof(float4) * (size_t)gd.N))) return rc;
        int tmax = 0;
        for (auto& p : s.particles_advected) {
            unsigned long long* d = nullptr;
            if ((rc = falloc((void**)&d, sizeof(unsigned long long) * 2 * (size_t)std::max(p.num, 1)))) return rc;
            partfix_.push_back(d);
            // large tracer sets of the Euler form are kept in spatial storage order
            int* perm = nullptr;
            if (!vlasov_ && p.num >= kReorderMin) {
                if ((rc = falloc((void**)&perm, sizeof(int) * (size_t)p.num))) return rc;
                tmax = std::max(tmax, p.num);
            }
            tperm_.push_back(perm);
            float2* v = nullptr;
            if (p.tau != 0 && (rc = falloc((void**)&v, sizeof(float2) * (size_t)std::max(p.num, 1)))) return rc;
            velm_.push_back(v);
        }
        if (tmax > 0) {
            TracerScratch& t = tscratch_;
            t.cap = tmax;
            t.nb_cap = ((gp.NX + 3) / 4) * ((gp.NY + 3) / 4);
            if ((rc = falloc((void**)&t.pos, sizeof(unsigned long long) * 2 * (size_t)tmax)) ||
                (rc = falloc((void**)&t.vel, sizeof(float2) * (size_t)tmax)) ||
                (rc = falloc((void**)&t.perm, sizeof(int) * (size_t)tmax)) ||
                (rc = falloc((void**)&t.key, sizeof(int) * (size_t)tmax)) ||
                (rc = falloc((void**)&t.rank, sizeof(int) * (size_t)tmax)) ||
                (rc = falloc((void**)&t.count, sizeof(int) * (size_t)t.nb_cap)))
                return rc;
        }
        if (stack_cap_ > 0 && (rc = falloc((void**)&stackm_, mapb * stack_cap_))) return rc;
        if (fft::plan_create(fv_, gv.NX, gv.NY, false, stream) || fft::plan_create(fp_, gp.NX, gp.NY, false, stream) ||
            fft::plan_create(ff_, gf.NX, gf.NY, false, stream)) {
            err = "FFT plan creation failed (grid sizes need NX even, sides <= 8192, prime factors <= 13)";
            return kErrParam;
        }
        // the psi solve keeps the columns kx <= freq_cut_psi of omega's spectrum only: a
        // row R2C of every row writing those columns, then a column transform of just them
        if (!vlasov_) vcols_ = std::min(gv.NX_fft, (int)std::floor(s.freq_cut_psi) + 1);
    }
    if (!vlasov_) {
        // the psi solve as four kernels (sample, kept row modes, column transforms with the
        // spectral step, inverse rows with the node pass) where the sizes allow it, else
        // sample, 2D transform, spectral step, 2D inverse transforms and node pass
        long long n1 = 0, n2 = 0;
        psi_fused_ = mixed_ ? psi_solve_m_fits(gc, gv, gp, s.freq_cut_psi, fv_, fp_, &n1, &n2)
                            : psi_solve_fits(gv, gp, s.freq_cut_psi, pv_.p, pp_.p, &n1, &n2);
        if (psi_fused_) {
            const size_t vb = mixed_ ? sizeof(float2) : sizeof(double2);
            CMM_CUDA(cudaMalloc(&psw1_, vb * (size_t)n1));
            CMM_CUDA(cudaMalloc(&psw2_, vb * (size_t)n2));
            if (mixed_) psi_solve_m_prepare();
            else psi_solve_prepare();
        }
    }
    // random table for gaussian_blobs (cmm-euler2d.cu:348-354)
    std::vector<double> rnd(1000);
    std::mt19937_64 gen(0);
    std::uniform_real_distribution<double> dist(-1.0, 1.0);
    for (auto& v : rnd) v = dist(gen);
    CMM_CUDA(cudaMemcpyAsync(d_rand_, rnd.data(), sizeof(double) * kRandTable, cudaMemcpyHostToDevice, stream));
    CMM_LAUNCH(1, launch_gaussienne_offsets(d_rand_ + kRandTable, stream));
    CMM_CUDA(cudaMemcpyAsync(d_params_, s.initial_params, sizeof(double) * 10, cudaMemcpyHostToDevice, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    return kOk;
}

void EulerSim::release()
{
    auto f = [](void* p) { if (p) cudaFree(p); };
    f(ChiX); f(ChiY); f(ChiX_new); f(ChiY_new); f(vort); f(wfine); f(wdisc); f(stack);
    f(ChiX_f); f(ChiY_f); f(stack_f); f(fpos_);
    ChiX_f = ChiY_f = stack_f = fpos_ = nullptr;
    for (auto p : fparts_) f(p);
    fparts_.clear();
    for (int l = 0; l < kMaxLagrange; ++l) f(psi[l]);
    f(real_buf_); f(spec_); f(spec4_); f(red_); f(d_scal_); f(d_einc2_); f(d_params_); f(d_rand_);
    for (auto p : parts) f(p);
    parts.clear();
    for (auto p : vels) f(p);
    vels.clear();
    for (auto p : partfix_) f(p);
    partfix_.clear();
    for (auto p : tperm_) f(p);
    tperm_.clear();
    f(tscratch_.pos); f(tscratch_.vel); f(tscratch_.perm); f(tscratch_.key); f(tscratch_.rank); f(tscratch_.count);
    tscratch_ = TracerScratch{};
    for (auto p : velm_) f(p);
    velm_.clear();
    for (int l = 0; l < kMaxLagrange; ++l) { f(phi_lv_[l]); phi_lv_[l] = nullptr; }
    f(vl_h_); f(vl_rho_); f(vl_part_);
    vl_h_ = vl_rho_ = vl_part_ = nullptr;
    for (int k = 0; k < 3; ++k) { f(vl_c_[k]); vl_c_[k] = nullptr; }
    for (int k = 0; k < 4; ++k) { f(vtab_[k]); vtab_[k] = nullptr; }
    destroy_vlasov_plans(vp_);
    f(wdiscm_); wdiscm_ = nullptr;
    for (auto& p : smp_) { f(p); p = nullptr; }
    for (auto& p : smp_c_) { f(p); p = nullptr; }
    destroy_plans(ps_);
    destroy_vlasov_plans(vps_);
    smp_n_ = smp_plan_n_ = vsmp_plan_n_ = 0;
    f(mapm_); f(mapm_new_); f(psiA_); f(psiB_); f(psiP_); f(wfm_); f(stackm_); f(realf_); f(specf_); f(spec4f_);
    f(d_stack_tau_); d_stack_tau_ = nullptr; stack_tau_cap_ = 0; stack_tau_.clear(); map_tau_ = 0.0;
    f(drift_rows_); drift_rows_ = nullptr;
    psiP_ = nullptr;
    fused_ = false;
    for (int l = 0; l < kMaxLagrange; ++l) { f(psim_[l]); psim_[l] = nullptr; }
    mapm_ = mapm_new_ = psiA_ = psiB_ = wfm_ = stackm_ = nullptr;
    realf_ = nullptr; specf_ = nullptr; spec4f_ = nullptr;
    fft::plan_destroy(fv_);
    fft::plan_destroy(fp_);
    fft::plan_destroy(ff_);
    f(psw1_); f(psw2_);
    psw1_ = psw2_ = nullptr;
    psi_fused_ = false;
    if (h_scal_) cudaFreeHost(h_scal_);
    h_scal_ = nullptr;
    if (einc_ev_) cudaEventDestroy(einc_ev_);
    einc_ev_ = nullptr;
    if (fork_ev_) cudaEventDestroy(fork_ev_);
    if (join_ev_) cudaEventDestroy(join_ev_);
    fork_ev_ = join_ev_ = nullptr;
    if (side_) cudaStreamDestroy(side_);
    side_ = nullptr;
    if (step_graph_) cudaGraphExecDestroy(step_graph_);
    step_graph_ = nullptr;
    destroy_plans(pf_); destroy_plans(pv_); destroy_plans(pp_); destroy_plans(pc_); destroy_plans(pd_);
    ChiX = ChiY = ChiX_new = ChiY_new = vort = wfine = wdisc = stack = nullptr;
    for (int l = 0; l < kMaxLagrange; ++l) psi[l] = nullptr;
    real_buf_ = nullptr; spec_ = nullptr; spec4_ = nullptr; red_ = d_scal_ = d_einc2_ = d_params_ = d_rand_ = nullptr;
    if (own_stream_ && stream) cudaStreamDestroy(stream);
    stream = nullptr;
    own_stream_ = false;
}

// ---------------------------------------------------------------- phases
int EulerSim::translate_ic()
{
    InitSource src{};
    src.kind = s.initial_discrete ? 3 : vlasov_ ? 2 : 0;   // ID_DIST_FUNC for Vlasov (cmm-vlasov1d.cu:538)
    src.ic_num = s.initial_condition_num;
    src.discrete = wdisc;
    src.gd = gd;
    src.params = d_params_;
    src.rand_table = d_rand_;
    if (mixed_ && !vlasov_) {
        // fixed-point positions through the FP32 displacement stack, then the
        // spectral Hermite planes in FP32, the precision of the nodes they are stored in
        CMM_LAUNCH(1, launch_compose_m(gc, gf, mapm_, stackm_, n_maps_, src, wdiscm_, nullptr, stream, realf_));
        CMM_FFT(fft::r2c(ff_, realf_, specf_, 1, stream));
        CMM_LAUNCH(1, launch_spec_hermite_f(specf_, gf, spec4f_, stream));
        CMM_FFT(fft::c2r(ff_, spec4f_, realf_, 4, stream));
        CMM_LAUNCH(1, launch_planes_to_float4(realf_, nullptr, gf.N, wfm_, stream));
        return kOk;
    }
    // plain form, and the Vlasov mixed form: there the kinetic energy weights f by v^2 over the
    // whole velocity range, where an FP32 transform's noise floor (~1e-7 of max f) would show
    SepDrift drift;
    if (mixed_)
        CMM_LAUNCH(1, launch_compose_m(gc, gf, mapm_, stackm_, n_maps_, src, wdiscm_, real_buf_, stream, nullptr,
                                       sep_drift(drift, map_tau_)));
    else CMM_LAUNCH(1, launch_compose_sample(gc, gf, ChiX, ChiY, stack, n_maps_, src, real_buf_, stream));
    CMM_FFT(fft_d2z(pf_, real_buf_, spec_, stream));
    CMM_LAUNCH(1, launch_spec_hermite(spec_, gf, spec4_, stream));
    CMM_FFT(fft_z2d(pf_, spec4_, wfine, 4, stream));
    if (mixed_) CMM_LAUNCH(1, launch_planes_to_float4(nullptr, wfine, gf.N, wfm_, stream));
    return kOk;
}

int EulerSim::evaluate_stream()
{
    if (vlasov_) return evaluate_potential();
    if (mixed_) {
        if (ups_ && in_step_) {
            int rc = learned_stream();
            if (rc) return rc;
        } else if (psi_fused_) {
            // sample, transforms, spectral step and node pass in four kernels; with three
            // Lagrange levels the node pass also writes the combinations below
            const bool combos = psi_lcl_ >= 0 && L == 3;
            fused_ = false;
            if (combos) predict_combinations();
            CMM_LAUNCH(4, launch_psi_solve_m(gc, gv, gf, mapm_, wfm_, gp, s.freq_cut_psi, fv_, fp_, realf_,
                                             static_cast<float2*>(psw1_), static_cast<float2*>(psw2_), psim_[0],
                                             psim_[1], psim_[2], combos ? fusedLp_ : nullptr, fusedL1_, fusedL12_,
                                             psiP_, psiA_, psiB_, stream));
            fused_ = combos;
            return kOk;
        } else {
            CMM_LAUNCH(1, launch_sample_m(gc, gv, gf, mapm_, wfm_, realf_, nullptr, stream));
            if (int rc = vort_spectrum()) return rc;
            CMM_LAUNCH(1, launch_spec_psi_f(specf_, gv, gp, s.freq_cut_psi, spec4f_, stream));
            if (int rc = psi_planes(spec4f_, realf_)) return rc;
        }
        fused_ = false;
        if (psi_lcl_ >= 0 && L == 3) {
            // one pass writes the new level and the Lagrange combinations this step's
            // tracers and the next step's advection will ask for (next dt predicted by
            // compute_next_timestep; the users check the coefficients bitwise)
            predict_combinations();
            CMM_LAUNCH(1, launch_psi_nodes3(realf_, gp.N, psim_[1], psim_[2], fusedLp_, fusedL1_, fusedL12_, psim_[0],
                                            psiP_, psiA_, psiB_, stream));
            fused_ = true;
        } else {
            CMM_LAUNCH(1, launch_planes_to_float4(realf_, nullptr, gp.N, psim_[0], stream));
        }
        return kOk;
    }
    if (psi_fused_) {
        CMM_LAUNCH(4, launch_psi_solve(gc, gv, gf, ChiX, ChiY, wfine, s.molly_stencil, gp, s.freq_cut_psi, pv_.p, pp_.p,
                                       real_buf_, static_cast<double2*>(psw1_), static_cast<double2*>(psw2_), psi[0],
                                       stream));
        return kOk;
    }
    CMM_LAUNCH(1, launch_sample_vort(gc, gv, gf, ChiX, ChiY, wfine, s.molly_stencil, real_buf_, gv.NX, stream));
    CMM_FFT(fft_d2z(pv_, real_buf_, spec_, stream));
    CMM_LAUNCH(1, launch_spec_psi(spec_, gv, gp, s.freq_cut_psi, spec4_, stream));
    CMM_FFT(fft_z2d(pp_, spec4_, psi[0], 4, stream));
    return kOk;
}

void EulerSim::predict_combinations()
{
    // the Lagrange combinations this step's tracers (t_{n+1/2}) and the next step's advection
    // (t_{n+1}, t_{n+1/2} for the dt compute_next_timestep predicts) ask for; their users
    // check the coefficients bitwise and recombine on a mismatch
    const int lcl = psi_lcl_;
    const double* t = t_vec_.data();
    const double tn = t[lcl + 1];
    double dtn = compute_next_timestep(tn);
    if (tn + dtn > s.final_time) dtn = s.final_time - tn;
    for (int i = 0; i < L; ++i) {
        fusedLp_[i] = lagrange_coefficient(t, t[lcl] + dt_vec_[lcl + 1] / 2.0, lcl + 1, i, L);
        fusedL1_[i] = lagrange_coefficient(t, tn + dtn, lcl + 1, i, L);
        fusedL12_[i] = lagrange_coefficient(t, tn + dtn / 2.0, lcl + 1, i, L);
    }
}

int EulerSim::vort_spectrum()
{
    // omega on the vorticity grid (realf_) -> the modes the psi solve keeps (specf_)
    if (vcols_ <= 0) {
        CMM_FFT(fft::r2c(fv_, realf_, specf_, 1, stream));
        return kOk;
    }
    CMM_FFT(fft::rows_r2c(fv_, realf_, gv.NX, gv.N, specf_, gv.NX_fft, gv.Nfft, gv.NY, 1, vcols_, stream));
    CMM_FFT(fft::cols_c2c(fv_, specf_, gv.NX_fft, gv.Nfft, vcols_, 1, false, stream));
    return kOk;
}

int EulerSim::psi_planes(float2* spec4, float* out)
{
    // the four Hermite spectra (gp layout) -> the planes on the psi grid
    CMM_FFT(fft::c2r(fp_, spec4, out, 4, stream));
    return kOk;
}

void EulerSim::scalar_source(InitSource& src) const
{
    // the passive scalar's initial field: the analytic scalar_name, or with scalar_discrete
    // the discrete initial *vorticity* (k_h_sample_from_init on Vort_discrete_init,
    // cmm-simulation-host.cu:803-805, 1160-1162: the reference has no discrete scalar input)
    if (s.scalar_discrete) {
        src.kind = 3;
        src.discrete = wdisc;
        src.gd = gd;
    } else {
        src.kind = 1;
        src.ic_num = s.scalar_num;
    }
}

int EulerSim::ensure_vort()
{
    if (!vort_stale_) return kOk;
    vort_stale_ = false;
    return coarse_vort();
}

int EulerSim::coarse_vort()
{
    if (mixed_) {
        SepDrift drift;
        CMM_LAUNCH(1, launch_sample_m(gc, gc, gf, mapm_, wfm_, nullptr, vort, stream, sep_drift(drift, map_tau_)));
        return kOk;
    }
    CMM_LAUNCH(1, launch_sample_vort(gc, gc, gf, ChiX, ChiY, wfine, 0, vort, gc.NX, stream));
    return kOk;
}

int EulerSim::sync_fp64_views()
{
    // mixed form: rebuild the reference-layout FP64 views (map planes, psi
    // levels, fine vorticity planes) used by the writers and cmm_get_field
    if (!mixed_) return kOk;
    SepDrift drift;
    CMM_LAUNCH(1, launch_map_to_planes(mapm_, gc, ChiX, ChiY, stream, sep_drift(drift, map_tau_)));
    for (int l = 0; l < L; ++l) CMM_LAUNCH(1, launch_float4_to_planes(psim_[l], gp.N, psi[l], stream));
    CMM_LAUNCH(1, launch_float4_to_planes(wfm_, gf.N, wfine, stream));
    for (size_t i = 0; i < partfix_.size(); ++i) {
        CMM_LAUNCH(1, launch_fix_to_pos(partfix_[i], s.particles_advected[i].num, gp, parts[i], stream, tperm_[i]));
        if (velm_[i])
            CMM_LAUNCH(1, launch_vel_to_f64(velm_[i], s.particles_advected[i].num, vels[i], stream, tperm_[i]));
    }
    if (vlasov_)   // psi levels are held as phi(x) and h(v): write their Hermite planes
        for (int l = 0; l < L; ++l)
            CMM_LAUNCH(1, launch_vlasov_assemble(phi_lv_[l], phi_lv_[l] + gp.NX, vl_h_, vl_h_ + gp.NY, gp, psi[l], stream));
    return kOk;
}

// ---------------------------------------------------------------- Vlasov-Poisson
int EulerSim::vlasov_setup_h()
{
    // compute_periodification_function (cmm-simulation-host.cu:534-571): the
    // normalised bump, integrated twice in v by 1D spectra; h and h' on the psi grid
    CMM_LAUNCH(1, launch_vlasov_bump(gp, real_buf_, stream));
    CMM_FFT(fft_d2z_1d(vp_.p, real_buf_, vl_c_[0], stream));
    CMM_LAUNCH(1, launch_vlasov_h_spec(vl_c_[0], gp, vl_c_[1], vl_c_[2], stream));
    CMM_FFT(fft_z2d_1d(vp_.p, vl_c_[1], vl_h_, stream));
    CMM_FFT(fft_z2d_1d(vp_.p, vl_c_[2], vl_h_ + gp.NY, stream));
    if (mixed_) {
        const double* lv[1] = {vl_h_};
        double one[1] = {1.0};
        CMM_LAUNCH(1, launch_vlasov_table(lv, one, 1, gp.NY, vtab_[3], stream));
    }
    return kOk;
}

int EulerSim::evaluate_potential()
{
    // evaluate_potential_from_density_hermite (cmm-simulation-host.cu:385-415):
    // f on the vort grid, rho = int f dv - 1, phi from the 1D Poisson solve,
    // psi = phi(x) - h(v) (its Hermite planes written directly, psi is separable)
    SepDrift drift;
    if (mixed_) CMM_LAUNCH(1, launch_sample_m(gc, gv, gf, mapm_, wfm_, realf_, nullptr, stream, sep_drift(drift, map_tau_)));
    else CMM_LAUNCH(1, launch_sample_vort(gc, gv, gf, ChiX, ChiY, wfine, s.molly_stencil, real_buf_, gv.NX, stream));
    CMM_LAUNCH(2, launch_vlasov_rho(mixed_ ? nullptr : real_buf_, mixed_ ? realf_ : nullptr, gv, vl_part_, vl_rho_, stream));
    CMM_FFT(fft_d2z_1d(vp_.v, vl_rho_, vl_c_[0], stream));
    CMM_LAUNCH(1, launch_vlasov_phi_spec(vl_c_[0], gv, gp, vl_c_[1], vl_c_[2], stream));
    double* phi = phi_lv_[0];
    CMM_FFT(fft_z2d_1d(vp_.p, vl_c_[1], phi, stream));
    CMM_FFT(fft_z2d_1d(vp_.p, vl_c_[2], phi + gp.NX, stream));
    if (!mixed_) CMM_LAUNCH(1, launch_vlasov_assemble(phi, phi + gp.NX, vl_h_, vl_h_ + gp.NY, gp, psi[0], stream));
    return kOk;
}

int EulerSim::vlasov_mesure(double* out)
{
    // Vlasov branch of compute_conservation_targets (cmm-simulation-host.cu:639-664),
    // Compute_* of src/numerical/cmm-mesure.cu:97-202
    CMM_LAUNCH(2, launch_vlasov_moments(vort, gc, red_, d_scal_, stream));
    CMM_LAUNCH(2, launch_sumsq(phi_lv_[0] + gp.NX, gp.NX, red_, d_scal_ + 3, stream));
    CMM_CUDA(cudaMemcpyAsync(real_buf_, phi_lv_[0] + gp.NX, sizeof(double) * gp.NX, cudaMemcpyDeviceToDevice, stream));
    CMM_FFT(fft_d2z_1d(vp_.p, real_buf_, vl_c_[0], stream));
    CMM_LAUNCH(1, launch_vlasov_modes(vl_c_[0], gp.NX, gp.NX_fft, d_scal_ + 4, stream));
    CMM_CUDA(cudaMemcpyAsync(h_scal_, d_scal_, sizeof(double) * 8, cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    double ekin = 0.5 * gc.hy * gc.hx * h_scal_[2];
    double epot = 0.5 * gp.hx * h_scal_[3];
    out[0] = ekin + epot;
    out[1] = ekin;
    out[2] = epot;
    out[3] = gc.hy * gc.hx * h_scal_[0];
    out[4] = gc.hy * gc.hx * h_scal_[1];
    for (int k = 0; k < 4; ++k) out[5 + k] = h_scal_[4 + k];
    return kOk;
}

int EulerSim::reset_map()
{
    map_tau_ = 0.0;
    if (mixed_) CMM_LAUNCH(1, launch_init_map_m(mapm_, gc, stream));
    else CMM_LAUNCH(1, launch_init_map(ChiX, ChiY, gc, stream));
    return kOk;
}

void EulerSim::swap_levels(int a, int b)
{
    std::swap(psi[a], psi[b]);
    std::swap(psim_[a], psim_[b]);
    std::swap(phi_lv_[a], phi_lv_[b]);
}

int EulerSim::advect_m(const double* t, const double* dtv, int lc, int ti_num, int l_order)
{
    int lcl = lc + l_order - 1;
    double L1[kMaxLagrange] = {0, 0, 0, 0}, L12[kMaxLagrange] = {0, 0, 0, 0};
    for (int i = 0; i < l_order; ++i) {
        L1[i] = lagrange_coefficient(t, t[lcl + 1], lcl, i, l_order);
        L12[i] = lagrange_coefficient(t, t[lcl] + dtv[lcl + 1] / 2.0, lcl, i, l_order);
    }
    AdvectMArgs a{};
    if (vlasov_) {
        // separable psi: 1D tables of the combined phi levels (and the static h)
        const double* lv[kMaxLagrange] = {phi_lv_[0], phi_lv_[1], phi_lv_[2], phi_lv_[3]};
        double one[1] = {1.0};
        CMM_LAUNCH(1, launch_vlasov_table(lv, L1, l_order, gp.NX, vtab_[0], stream));
        if (ti_num == 30) CMM_LAUNCH(1, launch_vlasov_table(lv, L12, l_order, gp.NX, vtab_[1], stream));
        CMM_LAUNCH(1, launch_vlasov_table(lv, one, 1, gp.NX, vtab_[2], stream));
        a.tA = vtab_[0]; a.tB = vtab_[1]; a.t0 = vtab_[2]; a.tv = vtab_[3];
    } else {
        // Lagrange extrapolation is linear in psi: combine the levels once per
        // step, then every RK stage interpolates a single field (already done by
        // the previous psi solve when its predicted coefficients are these)
        const bool half = ti_num == 30 || ti_num == 40 || ti_num == 41;   // schemes with a t_{n+1/2} stage
        bool have = fused_ && l_order == 3;
        for (int i = 0; i < l_order && have; ++i)
            have = L1[i] == fusedL1_[i] && (!half || L12[i] == fusedL12_[i]);
        if (!have && ti_num != 20)
            CMM_LAUNCH(1, launch_precombine(psim_, l_order, L1, half ? L12 : nullptr, gp.N, psiA_,
                                            half ? psiB_ : nullptr, stream));
    }
    a.gm = gc; a.gp = gp;
    a.map = mapm_; a.out = mapm_new_;
    a.psiA = psiA_; a.psiB = psiB_; a.psi0 = psim_[0]; a.psi1 = psim_[l_order > 1 ? 1 : 0];
    double coef[4][kMaxFoot];
    map_update_coefficients(s.map_update_order_num, s.map_epsilon, coef, &a.nfoot);
    for (int p = 0; p < 4; ++p)
        for (int k = 0; k < kMaxFoot; ++k) { a.coef[p][k] = (float)coef[p][k]; a.coef64[p][k] = coef[p][k]; }
    a.dt = (float)dtv[lcl + 1];
    a.ep = (float)s.map_epsilon;
    a.dt64 = dtv[lcl + 1];
    a.ep64 = s.map_epsilon;
    a.time_integration_num = ti_num;
    a.rp = gp.NX / gc.NX;
    a.nx_log2 = (gc.NX & (gc.NX - 1)) == 0 ? __builtin_ctz((unsigned)gc.NX) : -1;
    a.tau64 = map_tau_;
    a.drows = drift_rows_;
    CMM_LAUNCH(1, launch_advect_m(a, stream));
    std::swap(mapm_, mapm_new_);
    if (vlasov_) map_tau_ += a.dt64;   // the new map is one (signed) step older
    return kOk;
}

const SepDrift* EulerSim::sep_drift(SepDrift& d, double tau) const
{
    if (!(mixed_ && vlasov_)) return nullptr;
    d = SepDrift{};
    d.rows = drift_rows_;
    d.gm = gc;
    d.tau = tau;
    d.taus = d_stack_tau_;
    return &d;
}

int EulerSim::upload_stack_taus()
{
    // the stacked maps' ages, for the compositions (Vlasov mixed form)
    if (!(mixed_ && vlasov_)) return kOk;
    const int need = std::max(1, (int)stack_tau_.size());
    if (need > stack_tau_cap_) {
        if (d_stack_tau_) CMM_CUDA(cudaFree(d_stack_tau_));
        d_stack_tau_ = nullptr;
        const int cap = std::max({need, 2 * stack_tau_cap_, 16});
        CMM_CUDA(cudaMalloc((void**)&d_stack_tau_, sizeof(double) * cap));
        stack_tau_cap_ = cap;
    }
    if (!stack_tau_.empty())
        CMM_CUDA(cudaMemcpy(d_stack_tau_, stack_tau_.data(), sizeof(double) * stack_tau_.size(), cudaMemcpyHostToDevice));
    return kOk;
}

int EulerSim::advect(const double* t, const double* dtv, int lc, int ti_num, int l_order)
{
    if (mixed_) return advect_m(t, dtv, lc, ti_num, l_order);
    AdvectArgs a{};
    a.gm = gc; a.gp = gp;
    a.ChiX = ChiX; a.ChiY = ChiY; a.outX = ChiX_new; a.outY = ChiY_new;
    for (int l = 0; l < kMaxLagrange; ++l) a.psi[l] = psi[l];
    int lcl = lc + l_order - 1;
    for (int i = 0; i < l_order; ++i) {
        a.L1[i] = lagrange_coefficient(t, t[lcl + 1], lcl, i, l_order);
        a.L12[i] = lagrange_coefficient(t, t[lcl] + dtv[lcl + 1] / 2.0, lcl, i, l_order);
    }
    map_update_coefficients(s.map_update_order_num, s.map_epsilon, a.coef, &a.nfoot);
    a.dt = dtv[lcl + 1];
    a.ep = s.map_epsilon;
    a.time_integration_num = ti_num;
    a.l_order = l_order;
    CMM_LAUNCH(1, launch_advect(a, stream));
    std::swap(ChiX, ChiX_new);
    std::swap(ChiY, ChiY_new);
    return kOk;
}

int EulerSim::forward_step(int lcl, bool* forced_remap)
{
    // the forward map's part of a step (cmm-euler2d.cu:780-811): advect_using_stream_hermite
    // with direction 1 on the same psi history, then the invertibility check X_b(X_f(x)) ~ x
    // and the incompressibility check on the coarse grid, and a forced remap in the step
    // that reaches a forwarded set's start time (its particles are mapped from the sub-map
    // after that remap on)
    *forced_remap = false;
    if (!s.forward_map) return kOk;
    if (mixed_) {
        // mixed form: the forward map stays FP64; it is advected on FP64 copies of the FP32 psi
        // levels and checked against the FP64 planes of the FP32 backward map
        for (int l = 0; l < L; ++l) CMM_LAUNCH(1, launch_float4_to_planes(psim_[l], gp.N, psi[l], stream));
        CMM_LAUNCH(1, launch_map_to_planes(mapm_, gc, ChiX, ChiY, stream));
    }
    AdvectArgs a{};
    a.gm = gc; a.gp = gp;
    a.ChiX = ChiX_f; a.ChiY = ChiY_f; a.outX = ChiX_new; a.outY = ChiY_new;
    for (int l = 0; l < kMaxLagrange; ++l) a.psi[l] = psi[l];
    for (int i = 0; i < L; ++i) {
        a.L1[i] = lagrange_coefficient(t_vec_.data(), t_vec_[lcl + 1], lcl, i, L);
        a.L12[i] = lagrange_coefficient(t_vec_.data(), t_vec_[lcl] + dt_vec_[lcl + 1] / 2.0, lcl, i, L);
    }
    map_update_coefficients(s.map_update_order_num, s.map_epsilon, a.coef, &a.nfoot);
    a.dt = dt_vec_[lcl + 1];
    a.ep = s.map_epsilon;
    a.time_integration_num = s.time_integration_num;
    a.l_order = L;
    a.direction = 1;
    CMM_LAUNCH(1, launch_advect(a, stream));
    std::swap(ChiX_f, ChiX_new);
    std::swap(ChiY_f, ChiY_new);
    CMM_LAUNCH(1, launch_invert(gc, gc, ChiX, ChiY, ChiX_f, ChiY_f, d_scal_ + 14, stream));
    CMM_LAUNCH(1, launch_incomp(gc, gc, ChiX_f, ChiY_f, d_scal_ + 15, stream));
    CMM_CUDA(cudaMemcpyAsync(h_scal_ + 14, d_scal_ + 14, sizeof(double) * 2, cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    e_inv_ = h_scal_[14];
    e_inc_f_ = h_scal_[15];
    for (size_t i = 0; i < s.particles_forwarded.size(); ++i) {
        double d = t_vec_[lcl + 1] - s.particles_forwarded[i].init_time + dt * 1e-5;
        if (d < dt_vec_[lcl + 1] && d >= 0) {
            *forced_remap = true;
            init_map_[i] = n_maps_ + 1;
        }
    }
    return kOk;
}

int EulerSim::forwarded_positions(const double* frame, double* out)
{
    // apply_map_stack_points, direction 1 (cmm-simulation-host.cu:204-289): each set's
    // initial positions through the forward stack from its start map on, then the active
    // forward map; a set starting at t = 0 goes through every map; points leaving the frame
    // become NaN (k_h_sample_points_map)
    double* o = out;
    const int n = n_maps_f_;
    for (size_t i = 0; i < s.particles_forwarded.size(); ++i) {
        const int num = s.particles_forwarded[i].num;
        const double t0 = s.particles_forwarded[i].init_time;
        const int im = init_map_[i];
        if (num <= 0) continue;
        auto fmap = [&](int m) { return stack_f + (size_t)m * 8 * gc.N; };
        if (n > 0) {
            if (t0 == 0) CMM_LAUNCH(1, launch_map_points(gc, frame, fmap(0), fmap(0) + 4 * gc.N, fparts_[i], o, num, stream));
            else CMM_CUDA(cudaMemcpyAsync(o, fparts_[i], sizeof(double) * 2 * num, cudaMemcpyDeviceToDevice, stream));
            for (int m = 1; m < n; ++m)
                if ((m >= im && t0 != 0) || t0 == 0)
                    CMM_LAUNCH(1, launch_map_points(gc, frame, fmap(m), fmap(m) + 4 * gc.N, o, o, num, stream));
            if ((im != 0 && t0 != 0) || t0 == 0)
                CMM_LAUNCH(1, launch_map_points(gc, frame, ChiX_f, ChiY_f, o, o, num, stream));
        } else {
            CMM_LAUNCH(1, launch_map_points(gc, frame, ChiX_f, ChiY_f, fparts_[i], o, num, stream));
        }
        o += 2 * (size_t)num;
    }
    return kOk;
}

int EulerSim::incomp(double* out)
{
    SepDrift drift;
    if (mixed_) CMM_LAUNCH(1, launch_incomp_m(gc, gf.NX / gc.NX, mapm_, d_scal_, stream, sep_drift(drift, map_tau_)));
    else CMM_LAUNCH(1, launch_incomp(gf, gc, ChiX, ChiY, d_scal_, stream));
    CMM_CUDA(cudaMemcpyAsync(h_scal_, d_scal_, sizeof(double), cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    *out = h_scal_[0];
    return kOk;
}

void EulerSim::unrotate_psi(int n)
{
    // the inverse of rotate_psi(n)
    double* tmp = psi[0];
    for (int j = 0; j < n; ++j) psi[j] = psi[j + 1];
    psi[n] = tmp;
    float4* tmf = psim_[0];
    for (int j = 0; j < n; ++j) psim_[j] = psim_[j + 1];
    psim_[n] = tmf;
    double* tph = phi_lv_[0];
    for (int j = 0; j < n; ++j) phi_lv_[j] = phi_lv_[j + 1];
    phi_lv_[n] = tph;
}

void EulerSim::rotate_psi(int n)
{
    // levels 0..n-1 move to 1..n, the buffer of level n becomes the new level 0
    double* tmp = psi[n];
    for (int j = n; j >= 1; --j) psi[j] = psi[j - 1];
    psi[0] = tmp;
    float4* tmf = psim_[n];
    for (int j = n; j >= 1; --j) psim_[j] = psim_[j - 1];
    psim_[0] = tmf;
    double* tph = phi_lv_[n];
    for (int j = n; j >= 1; --j) phi_lv_[j] = phi_lv_[j - 1];
    phi_lv_[0] = tph;
}

int EulerSim::reserve_stack(int n)
{
    // the sub-map stack stays in HBM: grow it geometrically, up to the capacity
    // mem_RAM_CPU_remaps allows
    if (n <= stack_cap_) return kOk;
    int cap = std::min(max_maps, std::max({2 * stack_cap_, 16, n}));
    const size_t mapb = mixed_ ? sizeof(float4) * 2 * (size_t)gc.N : sizeof(double) * 8 * (size_t)gc.N;
    const size_t mapb_f = sizeof(double) * 8 * (size_t)gc.N;   // the forward stack is FP64 in both forms
    void* bigger = nullptr;
    CMM_CUDA(cudaMalloc(&bigger, mapb * cap));
    void* old = mixed_ ? (void*)stackm_ : (void*)stack;
    if (old && n_maps_ > 0) CMM_CUDA(cudaMemcpyAsync(bigger, old, mapb * n_maps_, cudaMemcpyDeviceToDevice, stream));
    void* bigger_f = nullptr;
    if (s.forward_map) {
        // the forward stack grows with the backward one (one forward sub-map per remap)
        CMM_CUDA(cudaMalloc(&bigger_f, mapb_f * cap));
        if (stack_f && n_maps_ > 0)
            CMM_CUDA(cudaMemcpyAsync(bigger_f, stack_f, mapb_f * n_maps_, cudaMemcpyDeviceToDevice, stream));
    }
    CMM_CUDA(cudaStreamSynchronize(stream));
    if (old) cudaFree(old);
    if (mixed_) stackm_ = (float4*)bigger;
    else stack = (double*)bigger;
    if (s.forward_map) {
        if (stack_f) cudaFree(stack_f);
        stack_f = (double*)bigger_f;
    }
    stack_cap_ = cap;
    return kOk;
}

int EulerSim::push_stack()
{
    int rc;
    if ((rc = reserve_stack(n_maps_ + 1))) return rc;
    if (mixed_) {
        size_t mapb = sizeof(float4) * 2 * (size_t)gc.N;
        CMM_CUDA(cudaMemcpyAsync(stackm_ + 2 * (size_t)n_maps_ * gc.N, mapm_, mapb, cudaMemcpyDeviceToDevice, stream));
        if (vlasov_) {
            stack_tau_.resize((size_t)n_maps_ + 1);
            stack_tau_[(size_t)n_maps_] = map_tau_;
            if ((rc = upload_stack_taus())) return rc;
        }
    } else {
        double* slot = stack + (size_t)n_maps_ * 8 * gc.N;
        CMM_CUDA(cudaMemcpyAsync(slot, ChiX, sizeof(double) * 4 * gc.N, cudaMemcpyDeviceToDevice, stream));
        CMM_CUDA(cudaMemcpyAsync(slot + 4 * gc.N, ChiY, sizeof(double) * 4 * gc.N, cudaMemcpyDeviceToDevice, stream));
    }
    if (s.forward_map) {
        // the forward map goes onto its own stack and restarts from the identity (cmm-euler2d.cu:847-851)
        double* fslot = stack_f + (size_t)n_maps_ * 8 * gc.N;
        CMM_CUDA(cudaMemcpyAsync(fslot, ChiX_f, sizeof(double) * 4 * gc.N, cudaMemcpyDeviceToDevice, stream));
        CMM_CUDA(cudaMemcpyAsync(fslot + 4 * gc.N, ChiY_f, sizeof(double) * 4 * gc.N, cudaMemcpyDeviceToDevice, stream));
        CMM_LAUNCH(1, launch_init_map(ChiX_f, ChiY_f, gc, stream));
        n_maps_f_++;
    }
    n_maps_++;
    return kOk;
}

// ---------------------------------------------------------------- MapStack folder
static std::string two_digits(int i) { return (i < 10 ? "0" : "") + std::to_string(i); }

int EulerSim::write_map_stack(int map_num, bool forward)
{
    // writeMapStack (src/ui/cmm-io.cu:611-635): one backward map in the reference's planar
    // FP64 layout under MapStack/Map_Chi{X,Y}_H_<n|coarse>.data, and psi for the restart.
    // The reference stores psi level 0 under every Stream_function_Psi_H_psi_<l> name
    // (l = 1..L-1, it passes Psi.Dev_var for each); a restart then starts with a flat
    // psi history.  Kept as is: the reference's restart goldens depend on it.
    const std::string dir = run_dir(s) + "/MapStack";
    if (!make_dir(dir)) { err = "cannot create " + dir; return kErrIO; }
    const std::string name = map_num < 0 ? std::string("coarse") : std::to_string(map_num);
    // forward maps go under Map_Chi{X,Y}_f_H_<n|coarse>, the names the reference's reader
    // expects (its writer puts a forward sub-map under the next backward name at a remap,
    // cmm-euler2d.cu:848, which a later restart would read as a backward sub-map)
    const std::string fw = forward ? "_f" : "";
    SepDrift drift;
    if (mixed_) CMM_LAUNCH(1, launch_map_to_planes(mapm_, gc, ChiX, ChiY, stream, sep_drift(drift, map_tau_)));
    std::vector<double> h((size_t)8 * gc.N);
    const double* MX = forward ? ChiX_f : ChiX;
    const double* MY = forward ? ChiY_f : ChiY;
    CMM_CUDA(cudaMemcpyAsync(h.data(), MX, sizeof(double) * 4 * gc.N, cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaMemcpyAsync(h.data() + 4 * gc.N, MY, sizeof(double) * 4 * gc.N, cudaMemcpyDeviceToHost, stream));
    const double* p0 = psi[0];
    if (mixed_ && vlasov_)
        CMM_LAUNCH(1, launch_vlasov_assemble(phi_lv_[0], phi_lv_[0] + gp.NX, vl_h_, vl_h_ + gp.NY, gp, psi[0], stream));
    else if (mixed_)
        CMM_LAUNCH(1, launch_float4_to_planes(psim_[0], gp.N, psi[0], stream));
    std::vector<double> hp(L > 1 ? (size_t)4 * gp.N : 0);
    if (L > 1) CMM_CUDA(cudaMemcpyAsync(hp.data(), p0, sizeof(double) * 4 * gp.N, cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    bool ok = write_f64(dir + "/Map_ChiX" + fw + "_H_" + name + ".data", h.data(), (size_t)4 * gc.N) &&
              write_f64(dir + "/Map_ChiY" + fw + "_H_" + name + ".data", h.data() + 4 * gc.N, (size_t)4 * gc.N);
    for (int l = 1; l < L && ok && !forward; ++l)
        ok = write_f64(dir + "/Stream_function_Psi_H_psi_" + std::to_string(l) + ".data", hp.data(), (size_t)4 * gp.N);
    if (!ok) { err = "cannot write the map stack under " + dir; return kErrIO; }
    return kOk;
}

int EulerSim::write_particles_state()
{
    // writeParticlesState (src/ui/cmm-io.cu:638-657): positions of every advected set and the
    // velocity state of the inertial ones
    const std::string dir = run_dir(s) + "/MapStack";
    if (!make_dir(dir)) { err = "cannot create " + dir; return kErrIO; }
    for (size_t i = 0; i < s.particles_advected.size(); ++i) {
        const int num = s.particles_advected[i].num;
        if (num <= 0) continue;
        if (mixed_) CMM_LAUNCH(1, launch_fix_to_pos(partfix_[i], num, gp, parts[i], stream, tperm_[i]));
        std::vector<double> h((size_t)2 * num);
        CMM_CUDA(cudaMemcpyAsync(h.data(), parts[i], sizeof(double) * 2 * num, cudaMemcpyDeviceToHost, stream));
        CMM_CUDA(cudaStreamSynchronize(stream));
        bool ok = write_f64(dir + "/Particles_advected_pos_P" + two_digits((int)i + 1) + ".data", h.data(), h.size());
        if (ok && s.particles_advected[i].tau != 0) {
            if (mixed_) CMM_LAUNCH(1, launch_vel_to_f64(velm_[i], num, vels[i], stream, tperm_[i]));
            CMM_CUDA(cudaMemcpyAsync(h.data(), vels[i], sizeof(double) * 2 * num, cudaMemcpyDeviceToHost, stream));
            CMM_CUDA(cudaStreamSynchronize(stream));
            ok = write_f64(dir + "/Particles_advected_vel_U" + two_digits((int)i + 1) + ".data", h.data(), h.size());
        }
        if (!ok) {
            err = "cannot write particle state under " + dir;
            return kErrIO;
        }
    }
    return kOk;
}

int EulerSim::restart_from_map_stack()
{
    // readMapStack (src/simulation/cmm-simulation-host.cu:1256-1302) and the rest of the
    // restart branch (src/simulation/cmm-euler2d.cu:634-685): every stored sub-map onto the
    // stack (their count: files named *Map_ChiX_H* minus the active map's), the initial
    // condition translated through them with the identity as the active map, then the
    // stored active map and psi levels 1..L-1; psi level 0 and the coarse vorticity are
    // computed from those, and the particle positions are read back.  Missing or short
    // files are reported together (the reference logs them and exits).
    const std::string dir = s.restart_location.empty() ? run_dir(s) + "/MapStack" : s.restart_location;
    if (s.verbose >= 2) log_.push("Initializing by loading previous state");
    std::string msg;
    auto read = [&](const std::string& file, double* dst, size_t n) {
        int r = read_f64(dir + "/" + file, dst, n);
        if (r == 1) msg += "Failed to read in " + file + " at location " + dir + "\n";
        if (r == 2) msg += "File " + dir + "/" + file + " holds fewer than " + std::to_string(n) + " values\n";
        return r == 0;
    };
    const int n = count_files_containing(dir, "Map_ChiX_H") - 1;
    if (n > max_maps) {
        err = "the map stack at " + dir + " holds " + std::to_string(n) + " maps, more than mem_RAM_CPU_remaps allows (" +
              std::to_string(max_maps) + ")";
        return kErrParam;
    }
    int rc;
    if (n > 0 && (rc = reserve_stack(n))) return rc;
    const size_t nc4 = (size_t)4 * gc.N, np4 = (size_t)4 * gp.N;
    std::vector<double> h(2 * nc4);
    auto upload_map = [&](double* X, double* Y, float4* M) -> int {
        // host planes -> the device map: a displacement map M of the mixed form (through the
        // FP64 scratch planes), or the FP64 planes X, Y (the plain form's maps, and the
        // forward maps of both forms: M null)
        double* dX = M ? ChiX_new : X;
        double* dY = M ? ChiY_new : Y;
        CMM_CUDA(cudaMemcpyAsync(dX, h.data(), sizeof(double) * nc4, cudaMemcpyHostToDevice, stream));
        CMM_CUDA(cudaMemcpyAsync(dY, h.data() + nc4, sizeof(double) * nc4, cudaMemcpyHostToDevice, stream));
        if (M) CMM_LAUNCH(1, launch_planes_to_map(dX, dY, gc, M, stream));
        CMM_CUDA(cudaStreamSynchronize(stream));
        return kOk;
    };
    for (int i = 0; i < n; ++i) {
        bool ok = read("Map_ChiX_H_" + std::to_string(i) + ".data", h.data(), nc4);
        ok = read("Map_ChiY_H_" + std::to_string(i) + ".data", h.data() + nc4, nc4) && ok;
        if (!ok) continue;
        if (mixed_) rc = upload_map(nullptr, nullptr, stackm_ + 2 * (size_t)i * gc.N);
        else rc = upload_map(stack + (size_t)i * 8 * gc.N, stack + (size_t)i * 8 * gc.N + nc4, nullptr);
        if (rc) return rc;
    }
    n_maps_ = std::max(n, 0);
    stack_tau_.assign((size_t)n_maps_, 0.0);   // stored maps are taken with age 0: X - x in full
    if ((rc = upload_stack_taus())) return rc;
    if (!msg.empty()) { log_.push(msg + "Exitting .."); err = msg; return kErrIO; }
    if (s.verbose >= 2) log_.push("Loaded " + std::to_string(n_maps_) + " maps to map stack");

    if ((rc = reset_map()) || (rc = translate_ic())) return rc;
    bool ok = read("Map_ChiX_H_coarse.data", h.data(), nc4);
    ok = read("Map_ChiY_H_coarse.data", h.data() + nc4, nc4) && ok;
    if (ok && (rc = upload_map(ChiX, ChiY, mapm_))) return rc;
    if (s.forward_map) {
        // the forward stack and active forward map (readMapStack with isForward, :1256-1302)
        const int nf = count_files_containing(dir, "Map_ChiX_f_H") - 1;
        if (nf > n_maps_) {
            err = "the forward map stack at " + dir + " holds more maps than the backward one";
            return kErrParam;
        }
        for (int i = 0; i < nf; ++i) {
            bool okf = read("Map_ChiX_f_H_" + std::to_string(i) + ".data", h.data(), nc4);
            okf = read("Map_ChiY_f_H_" + std::to_string(i) + ".data", h.data() + nc4, nc4) && okf;
            if (okf && (rc = upload_map(stack_f + (size_t)i * 8 * gc.N, stack_f + (size_t)i * 8 * gc.N + nc4, nullptr)))
                return rc;
        }
        n_maps_f_ = std::max(nf, 0);
        bool okf = read("Map_ChiX_f_H_coarse.data", h.data(), nc4);
        okf = read("Map_ChiY_f_H_coarse.data", h.data() + nc4, nc4) && okf;
        if (okf && (rc = upload_map(ChiX_f, ChiY_f, nullptr))) return rc;
        if (s.verbose >= 2) log_.push("Loaded " + std::to_string(n_maps_f_) + " maps to forward map stack");
    }
    std::vector<double> hp(np4);
    for (int l = 1; l < L; ++l) {
        if (!read("Stream_function_Psi_H_psi_" + std::to_string(l) + ".data", hp.data(), np4)) continue;
        CMM_CUDA(cudaMemcpyAsync(psi[l], hp.data(), sizeof(double) * np4, cudaMemcpyHostToDevice, stream));
        if (mixed_ && !vlasov_) CMM_LAUNCH(1, launch_planes_to_float4(nullptr, psi[l], gp.N, psim_[l], stream));
        if (vlasov_) CMM_LAUNCH(1, launch_vlasov_phi_from_psi(psi[l], vl_h_, gp, phi_lv_[l], stream));
        CMM_CUDA(cudaStreamSynchronize(stream));
    }
    if (!msg.empty()) { log_.push(msg + "Exitting .."); err = msg; return kErrIO; }
    if ((rc = evaluate_stream()) || (rc = coarse_vort())) return rc;

    // readParticlesState (src/ui/cmm-io.cu:659-688)
    for (size_t i = 0; i < s.particles_advected.size(); ++i) {
        const int num = s.particles_advected[i].num;
        if (num <= 0) continue;
        std::vector<double> pos((size_t)2 * num);
        if (!read("Particles_advected_pos_P" + two_digits((int)i + 1) + ".data", pos.data(), pos.size())) continue;
        CMM_CUDA(cudaMemcpyAsync(parts[i], pos.data(), sizeof(double) * pos.size(), cudaMemcpyHostToDevice, stream));
        if (mixed_) CMM_LAUNCH(1, launch_pos_to_fix(parts[i], num, gp, partfix_[i], stream));
        if (mixed_ && tperm_[i]) CMM_LAUNCH(1, launch_iota(tperm_[i], num, stream));
        CMM_CUDA(cudaStreamSynchronize(stream));
        if (s.particles_advected[i].tau == 0) continue;
        if (!read("Particles_advected_vel_U" + two_digits((int)i + 1) + ".data", pos.data(), pos.size())) continue;
        CMM_CUDA(cudaMemcpyAsync(vels[i], pos.data(), sizeof(double) * pos.size(), cudaMemcpyHostToDevice, stream));
        if (mixed_) CMM_LAUNCH(1, launch_vel_from_f64(vels[i], num, velm_[i], stream));
        CMM_CUDA(cudaStreamSynchronize(stream));
    }
    if (!msg.empty()) { log_.push(msg + "Exitting .."); err = msg; return kErrIO; }
    if (!s.particles_advected.empty() && s.verbose >= 2) log_.push("Loaded data for particle sets");
    return kOk;
}

int EulerSim::init_positions(double* dst, int num, unsigned long long seed, int init_num, const double* param,
                             const std::string& init_name)
{
    // init_particles (src/simulation/cmm-init.cu:311-389); bounds of the psi grid
    if (num <= 0) return kOk;
    if (init_num == 0 || init_num == 1) {
        curandGenerator_t g;
        if (curandCreateGenerator(&g, CURAND_RNG_PSEUDO_DEFAULT) != CURAND_STATUS_SUCCESS) { err = "cuRAND create"; return kErrCuda; }
        curandSetStream(g, stream);
        curandSetPseudoRandomGeneratorSeed(g, seed);
        curandStatus_t st = init_num == 0 ? curandGenerateUniformDouble(g, dst, 2 * (size_t)num)
                                          : curandGenerateNormalDouble(g, dst, 2 * (size_t)num, 0.5, 1.0);
        curandDestroyGenerator(g);
        if (st != CURAND_STATUS_SUCCESS) { err = "cuRAND generate"; return kErrCuda; }
        CMM_LAUNCH(1, launch_particle_rescale(dst, num, param, gp, stream));
    } else if (init_num >= 2 && init_num <= 4) {
        CMM_LAUNCH(1, launch_particle_layout(dst, num, init_num, param, gp, stream));
    } else {
        err = "unknown particle init_name " + init_name;
        return kErrParam;
    }
    return kOk;
}

int EulerSim::init_particles()
{
    int rc;
    for (size_t i = 0; i < s.particles_advected.size(); ++i) {
        auto& p = s.particles_advected[i];
        if ((rc = init_positions(parts[i], p.num, p.seed, p.init_num, p.init_param, p.init_name))) return rc;
    }
    for (size_t i = 0; i < fparts_.size(); ++i) {
        auto& p = s.particles_forwarded[i];
        if ((rc = init_positions(fparts_[i], p.num, p.seed, p.init_num, p.init_param, p.init_name))) return rc;
    }
    return kOk;
}

int EulerSim::init_inertial_velocity(size_t i)
{
    // Particle_advect_inertia_init (cmm-particles.cu:50-60) or a set at rest
    // (cmm-euler2d.cu:620-632, 883-895)
    auto& p = s.particles_advected[i];
    if (p.tau == 0 || p.num <= 0) return kOk;
    if (mixed_) {
        if (p.init_vel) CMM_LAUNCH(1, launch_particle_vel_init_m(gp, partfix_[i], p.num, psim_[0], velm_[i], stream));
        else CMM_CUDA(cudaMemsetAsync(velm_[i], 0, sizeof(float2) * (size_t)p.num, stream));
    } else {
        if (p.init_vel) CMM_LAUNCH(1, launch_particle_vel_init(parts[i], p.num, psi[0], gp, vels[i], stream));
        else CMM_CUDA(cudaMemsetAsync(vels[i], 0, sizeof(double) * 2 * (size_t)p.num, stream));
    }
    return kOk;
}

int EulerSim::advect_particles(int lcl)
{
    // particles_advect (src/numerical/cmm-particles.cu:63-87): Lp12 for t_n + dt/2 on
    // the history ending at the new psi; fluid tracers (tau == 0) and inertial sets
    double Lp12[kMaxLagrange] = {0, 0, 0, 0};
    for (int i = 0; i < L; ++i)
        Lp12[i] = lagrange_coefficient(t_vec_.data(), t_vec_[lcl] + dt_vec_[lcl + 1] / 2.0, lcl + 1, i, L);
    bool combined = false;
    for (size_t i = 0; i < s.particles_advected.size(); ++i) {
        auto& p = s.particles_advected[i];
        if (p.num <= 0) continue;
        if (!(t_vec_[lcl + 1] + 1e-5 * dt_vec_[lcl + 1] >= p.init_time)) continue;
        const int ti = p.time_integration_num;
        const bool half = ti == 30 || ti == 40 || ti == 41;   // schemes with a t_{n+1/2} stage
        if (mixed_) {
            if (!combined && vlasov_) {
                // separable psi: tables of level 1 (t_n), the t_{n+1/2} combination and level 0
                const double* lv[kMaxLagrange] = {phi_lv_[0], phi_lv_[1], phi_lv_[2], phi_lv_[3]};
                const double* l1[1] = {phi_lv_[L > 1 ? 1 : 0]};
                double one[1] = {1.0};
                CMM_LAUNCH(1, launch_vlasov_table(l1, one, 1, gp.NX, vtab_[0], stream));
                CMM_LAUNCH(1, launch_vlasov_table(lv, Lp12, L, gp.NX, vtab_[1], stream));
                CMM_LAUNCH(1, launch_vlasov_table(lv, one, 1, gp.NX, vtab_[2], stream));
                combined = true;
            } else if (half && !combined && !vlasov_) {
                bool have = fused_ && L == 3;
                for (int k = 0; k < L && have; ++k) have = Lp12[k] == fusedLp_[k];
                if (!have) CMM_LAUNCH(1, launch_precombine(psim_, L, Lp12, nullptr, gp.N, psiP_, nullptr, stream));
                combined = true;
            }
            if (tperm_[i] && loop_ctr_ % kReorderEvery == 0) {
                CMM_LAUNCH(3, launch_tracer_reorder(gp, partfix_[i], velm_[i], tperm_[i], p.num, tscratch_, stream));
            }
            cudaError_t e = vlasov_
                ? launch_particles_m(gp, partfix_[i], p.num, nullptr, nullptr, nullptr, dt_vec_[lcl + 1], ti, stream,
                                     vtab_[0], vtab_[1], vtab_[2], vtab_[3])
                : launch_particles_m(gp, partfix_[i], p.num, psim_[L > 1 ? 1 : 0], psiP_, psim_[0], dt_vec_[lcl + 1], ti,
                                     stream, nullptr, nullptr, nullptr, nullptr, L > 2 ? psim_[2] : nullptr, velm_[i],
                                     p.tau);
            kernel_launches++;
            if (e == cudaErrorInvalidValue) { err = "particle time integration " + p.time_integration + " is not built"; return kErrUnsupported; }
            CMM_CUDA(e);
            continue;
        }
        ParticleArgs a{};
        a.gp = gp; a.pos = parts[i]; a.vel = vels[i]; a.num = p.num; a.tau = p.tau;
        for (int l = 0; l < kMaxLagrange; ++l) a.psi[l] = psi[l];
        for (int l = 0; l < kMaxLagrange; ++l) a.Lp12[l] = Lp12[l];
        a.dt = dt_vec_[lcl + 1];
        a.time_integration_num = ti;
        a.l_order = L;
        cudaError_t e = launch_particles(a, stream);
        kernel_launches++;
        if (e == cudaErrorInvalidValue) { err = "particle time integration " + p.time_integration + " is not built"; return kErrUnsupported; }
        CMM_CUDA(e);
    }
    // an inertial set whose start time was crossed in this step restarts its velocity
    // (cmm-euler2d.cu:883-895)
    int rc;
    for (size_t i = 0; i < s.particles_advected.size(); ++i) {
        auto& p = s.particles_advected[i];
        if (p.tau != 0 && t_vec_[lcl] - p.init_time + dt * 1e-5 < 0 && t_vec_[lcl + 1] - p.init_time + dt * 1e-5 > 0)
            if ((rc = init_inertial_velocity(i))) return rc;
    }
    return kOk;
}

// ---------------------------------------------------------------- init
int EulerSim::init()
{
    if (initialised_) { err = "init called twice"; return kErrState; }
    begin_ = std::chrono::steady_clock::now();
    int rc = alloc();
    if (rc) return rc;
    if (!s.psi_upsampler.empty() && (rc = load_upsampler())) return rc;
    if (!create_directory_structure(s)) { err = "cannot create output folders under " + s.workspace; return kErrIO; }
    log_.start(run_dir(s) + "/log.txt", s.restart_time != 0, s.file_name);
    log_.quiet = s.verbose < 1;
    if (s.verbose >= 1) {
        if (vlasov_) log_.push(std::string("Starting Vlasov 1D simulation, initial condition ") + s.initial_condition);
        log_.push("Solving = " + s.simulation_type);
        log_.push("Initial condition = " + s.initial_condition);
        log_.push("Iter max = " + std::to_string(s.iter_max()));
        log_.push("Name of simulation = " + s.file_name);
        log_.push("Map stack length = " + std::to_string(max_maps) + " (device resident)");
    }
    s.save_param_file(run_dir(s) + "/params.txt");

    // discrete initial condition (cmm-euler2d.cu:325-344)
    if (s.initial_discrete) {
        if (host_discrete_.empty()) {
            host_discrete_.resize((size_t)gd.N);
            std::ifstream f(s.initial_discrete_location, std::ios::binary);
            if (!f) { err = "unable to read discrete initial condition " + s.initial_discrete_location; return kErrIO; }
            f.read(reinterpret_cast<char*>(host_discrete_.data()), sizeof(double) * gd.N);
            if (f.gcount() != (std::streamsize)(sizeof(double) * gd.N)) { err = "discrete initial condition too short"; return kErrIO; }
        }
        CMM_CUDA(cudaMemcpyAsync(real_buf_, host_discrete_.data(), sizeof(double) * gd.N, cudaMemcpyHostToDevice, stream));
        CMM_FFT(fft_d2z(pd_, real_buf_, spec_, stream));
        CMM_LAUNCH(1, launch_spec_hermite(spec_, gd, spec4_, stream));
        CMM_FFT(fft_z2d(pd_, spec4_, wdisc, 4, stream));
        if (mixed_) CMM_LAUNCH(1, launch_planes_to_float4(nullptr, wdisc, gd.N, wdiscm_, stream));
        CMM_CUDA(cudaStreamSynchronize(stream));   // host_discrete_ may be released by the caller
    }

    if ((rc = reset_map())) return rc;
    if (vlasov_ && (rc = vlasov_setup_h())) return rc;
    if (vlasov_ && mixed_) {   // the free-streaming frame's per-row drift table (SepDrift)
        if (!drift_rows_) CMM_CUDA(cudaMalloc((void**)&drift_rows_, sizeof(double2) * gc.NY));
        CMM_LAUNCH(1, launch_drift_rows(vtab_[3], gp, gc, drift_rows_, stream));
    }
    if (s.forward_map) CMM_LAUNCH(1, launch_init_map(ChiX_f, ChiY_f, gc, stream));
    n_maps_f_ = 0;
    const bool restart = s.restart_time != 0;
    if (restart) {
        if ((rc = restart_from_map_stack())) return rc;
    } else if ((rc = translate_ic()) || (rc = evaluate_stream()) || (rc = coarse_vort())) {
        return rc;
    }

    // Lagrange velocity history (cmm-euler2d.cu:520-619): alternate the
    // direction of time and raise the scheme order EulerExp -> RK2 -> RK3
    if (L > 1 && !restart) {
        double dt_now = dt * std::pow(-1.0, L);
        double t_init[5] = {0, dt_now, 2 * dt_now, 3 * dt_now, 4 * dt_now};
        double dt_init[5] = {dt_now, dt_now, dt_now, dt_now, dt_now};
        for (int io = 1; io <= L; ++io) {
            if (!s.lagrange_init_higher_order && io != L) {
                for (int i = 0; i < 5; ++i) { dt_init[i] = -dt_init[i]; t_init[i] = -t_init[i]; }
                continue;
            }
            int ti = 10, lo = 1;
            if (s.lagrange_init_higher_order) {
                ti = io == 1 ? 10 : io == 2 ? 21 : 30;
                lo = io;
                if (io == 4) ti = 40;
            }
            int nsteps = io - (io == L);
            for (int k = 1; k <= nsteps; ++k) {
                if ((rc = advect(t_init, dt_init, 0, ti, lo))) return rc;
                double inc;
                if ((rc = incomp(&inc))) return rc;
                rotate_psi(nsteps);
                if ((rc = evaluate_stream())) return rc;
                if (s.verbose >= 2)
                    log_.push("   Init step = " + std::to_string(k) + "/" + std::to_string(nsteps) + " \t IncompErr = " + to_str3(inc));
            }
            for (int i = 0; i < 5; ++i) { dt_init[i] = -dt_init[i]; t_init[i] = -t_init[i]; }
            swap_levels(0, nsteps);
            if (nsteps >= 3) swap_levels(1, 2);
            if ((rc = reset_map())) return rc;
        }
        if ((rc = reset_map())) return rc;
    }
    if (!restart) {
        if ((rc = init_particles())) return rc;
        for (size_t i = 0; i < partfix_.size(); ++i) {
            CMM_LAUNCH(1, launch_pos_to_fix(parts[i], s.particles_advected[i].num, gp, partfix_[i], stream));
            if (tperm_[i]) CMM_LAUNCH(1, launch_iota(tperm_[i], s.particles_advected[i].num, stream));
        }
        // inertial particles start at the fluid velocity of psi(t_0) or at rest (cmm-euler2d.cu:620-632)
        for (size_t i = 0; i < s.particles_advected.size(); ++i)
            if ((rc = init_inertial_velocity(i))) return rc;
    }

    t_vec_.assign((size_t)s.iter_max() + L + 8, 0.0);
    dt_vec_.assign(t_vec_.size(), dt);
    for (int i = 0; i < L; ++i) { t_vec_[i] = s.restart_time - (L - 1 - i) * dt; dt_vec_[i] = dt; }
    loop_ctr_ = 0; old_ctr_ = 0;
    if (!restart) n_maps_ = 0;   // a restart keeps the sub-maps it loaded
    initialised_ = true;

    if ((rc = save_functions(s.restart_time, dt))) return rc;
    double tc = wall();
    append_f64(run_dir(s) + "/Monitoring_data/Time_c.data", &tc, 1);
    if (s.verbose >= 1) log_.push("Simulation initialization finished \t C-Time = " + format_duration(tc));
    return kOk;
}

// ---------------------------------------------------------------- loop
double EulerSim::compute_next_timestep(double t) const
{
    // src/simulation/cmm-simulation-host.cu:1307-1374
    double dt_now = dt, e = dt * 1e-5;
    auto instant = [&](double start) {
        if (t + e - start < 0 && t + e + dt - start > 0) dt_now = std::fmin(dt_now, start - t);
    };
    auto interval = [&](double start, double end, double step) {
        double a = std::fmod(t + e - start, step), b2 = std::fmod(t + dt + e - start, step);
        if ((a > b2 || (a < 0 && b2 > 0)) && t + dt + e >= start && t - e <= end)
            dt_now = std::fmin(dt_now, step - std::fmod(t, step));
    };
    for (auto& p : s.particles_advected) instant(p.init_time);
    for (auto& p : s.particles_forwarded) instant(p.init_time);
    for (auto& r : s.save_computational) r.is_instant ? instant(r.time_start) : interval(r.time_start, r.time_end, r.time_step);
    for (auto& r : s.save_sample) r.is_instant ? instant(r.time_start) : interval(r.time_start, r.time_end, r.time_step);
    for (auto& r : s.save_zoom) r.is_instant ? instant(r.time_start) : interval(r.time_start, r.time_end, r.time_step);
    return dt_now;
}

bool EulerSim::done() const
{
    if (!initialised_) return false;
    int lcl = loop_ctr_ + L - 1;
    return !(s.final_time - t_vec_[lcl] > dt * 1e-5 && loop_ctr_ < s.iter_max() && continue_);
}

int EulerSim::step_once()
{
    if (!initialised_) { err = "step before init"; return kErrState; }
    if (done()) return 1;
    int rc;
    int lcl = loop_ctr_ + L - 1;
    double t = t_vec_[lcl];
    double dt_now = compute_next_timestep(t);
    if (t + dt_now > s.final_time) dt_now = s.final_time - t;
    t_vec_[lcl + 1] = t + dt_now;
    dt_vec_[lcl + 1] = dt_now;

    // mixed Euler: the psi of the advected map is enqueued before the host reads E_inc, so
    // the GPU computes while the host waits; a remap (a few steps in a hundred) undoes the
    // psi rotation and redoes the evaluation on the remapped state.  That front of the step
    // (advection, incompressibility check and its readback, psi solve) is captured as a CUDA
    // graph and replayed through one executable updated in place (no gaps between its
    // kernels); profiled steps launch plainly
    const bool spec = mixed_ && !vlasov_ && !ups_ && !s.forward_map;
    bool capturing = spec && use_graphs_ && !prof_ &&
                     cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    bool forked = false;   // the E_inc readback went to side_
    auto join = [&]() -> int {
        if (!forked) return kOk;
        forked = false;
        int rj = check(cudaEventRecord(join_ev_, side_), "cudaEventRecord");
        if (!rj) rj = check(cudaStreamWaitEvent(stream, join_ev_, 0), "cudaStreamWaitEvent");
        return rj;
    };
    auto end_capture = [&](int rc_in) -> int {
        const int rj = join();
        if (!rc_in) rc_in = rj;
        if (!capturing) return rc_in;
        capturing = false;
        cudaGraph_t g = nullptr;
        cudaError_t ec = cudaStreamEndCapture(stream, &g);
        if (rc_in) {
            if (g) cudaGraphDestroy(g);
            return rc_in;
        }
        if (ec != cudaSuccess || !g) return check(ec != cudaSuccess ? ec : cudaErrorUnknown, "cudaStreamEndCapture");
        if (step_graph_) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(step_graph_, g, &info) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(step_graph_);
                step_graph_ = nullptr;
            }
        }
        cudaError_t ei = step_graph_ ? cudaSuccess : cudaGraphInstantiate(&step_graph_, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) return check(ei, "cudaGraphInstantiate");
        ++graph_launches_;
        return check(cudaGraphLaunch(step_graph_, stream), "cudaGraphLaunch");
    };
    ph_begin(kPhAdvect);
    if ((rc = advect(t_vec_.data(), dt_vec_.data(), loop_ctr_, s.time_integration_num, L))) return end_capture(rc);
    bool forced_remap = false;
    if ((rc = forward_step(lcl, &forced_remap))) return end_capture(rc);
    ph_end(kPhAdvect);
    ph_begin(kPhIncomp);
    if (spec) {
        kernel_launches++;
        double* slot = d_einc2_ + einc_slot_;
        if ((rc = check(launch_incomp_m_pp(gc, gf.NX / gc.NX, mapm_, slot, d_einc2_ + (1 - einc_slot_), stream),
                        "launch_incomp_m")) ||
            (rc = check(cudaEventRecord(fork_ev_, stream), "cudaEventRecord")) ||
            (rc = check(cudaStreamWaitEvent(side_, fork_ev_, 0), "cudaStreamWaitEvent")))
            return end_capture(rc);
        einc_slot_ = 1 - einc_slot_;
        forked = true;
        if ((rc = check(cudaMemcpyAsync(h_scal_, slot, sizeof(double), cudaMemcpyDeviceToHost, side_), "cudaMemcpyAsync")) ||
            (rc = check(capturing ? cudaEventRecordWithFlags(einc_ev_, side_, cudaEventRecordExternal)
                                  : cudaEventRecord(einc_ev_, side_),
                        "cudaEventRecord")))
            return end_capture(rc);
    } else if ((rc = incomp(&e_inc_))) {
        return rc;
    }
    ph_end(kPhIncomp);
    bool psi_done = false;
    if (spec) {
        rotate_psi(L - 1);
        ph_begin(kPhPsi);
        psi_lcl_ = lcl;
        in_step_ = true;
        rc = evaluate_stream();
        in_step_ = false;
        psi_lcl_ = -1;
        if ((rc = end_capture(rc))) return rc;
        ph_end(kPhPsi);
        CMM_CUDA(cudaEventSynchronize(einc_ev_));
        e_inc_ = h_scal_[0];
        psi_done = !((e_inc_ > s.incomp_threshold && !s.skip_remapping) || forced_remap);
        if (!psi_done) unrotate_psi(L - 1);
    }
    if (vlasov_ && (e_inc_ <= 0 || e_inc_ > 1e15)) {
        // the Vlasov driver aborts on a vanishing or exploding incompressibility error (cmm-vlasov1d.cu:838-840)
        err = "incompressibility error out of range in the coarse grid (" + to_str3(e_inc_) + "): run aborted";
        log_.push(err);
        continue_ = false;
        return kErrState;
    }
    bool saturated = false;
    if ((e_inc_ > s.incomp_threshold && !s.skip_remapping) || forced_remap) {
        if (n_maps_ >= max_maps) {
            if (s.verbose >= 0) log_.push("Stack Saturated : Exitting");
            saturated = true;
            continue_ = false;
        } else {
            if (s.verbose >= 2)
                log_.push("Refining Map : Step = " + std::to_string(loop_ctr_) + " \t Maps = " + std::to_string(n_maps_ + 1) +
                          " \t Gap = " + std::to_string(loop_ctr_ - old_ctr_));
            old_ctr_ = loop_ctr_;
            ph_begin(kPhRemap);
            if ((rc = translate_ic())) return rc;
            if (s.save_map_stack && (rc = write_map_stack(n_maps_))) return rc;
            if (s.save_map_stack && s.forward_map && (rc = write_map_stack(n_maps_f_, true))) return rc;
            if ((rc = push_stack())) return rc;
            if ((rc = reset_map())) return rc;
            kernel_launches++;
            ph_end(kPhRemap);
        }
    }
    double gap = loop_ctr_ - old_ctr_, counter = n_maps_;
    if (!psi_done) {
        rotate_psi(L - 1);
        ph_begin(kPhPsi);
        psi_lcl_ = lcl;
        in_step_ = true;
        rc = evaluate_stream();
        in_step_ = false;
        psi_lcl_ = -1;
        if (rc) return rc;
        ph_end(kPhPsi);
    }
    // the coarse vorticity is read only by the diagnostics, the saves and get_field: the 2D Euler
    // form samples it when first read after a step (same map, same fine vorticity, same values)
    ph_begin(kPhCoarse);
    if (vlasov_) {
        if ((rc = coarse_vort())) return rc;
    } else {
        vort_stale_ = true;
    }
    ph_end(kPhCoarse);
    ph_begin(kPhParticles);
    if ((rc = advect_particles(lcl))) return rc;
    ph_end(kPhParticles);
    ph_begin(kPhSave);
    if ((rc = save_functions(t_vec_[lcl + 1], dt_now))) return rc;
    ph_end(kPhSave);
    ph_collect();
    loop_ctr_++;
    CMM_CUDA(cudaGetLastError());

    // the per-step Monitoring_data records are kept in host buffers and appended in blocks
    // (every 256 steps, at the final step, when the stack saturates, in finish and on destruction)
    mon_buf_[kMonTimeS].push_back(t_vec_[lcl + 1]);
    mon_buf_[kMonEinc].push_back(e_inc_);
    if (s.forward_map) {
        mon_buf_[kMonEincF].push_back(e_inc_f_);
        mon_buf_[kMonEinv].push_back(e_inv_);
    }
    mon_buf_[kMonGap].push_back(gap);
    mon_buf_[kMonCounter].push_back(counter);
    double tc = wall();
    if (s.verbose >= 2)
        log_.push("Step = " + std::to_string(loop_ctr_) + " \t S-Time = " + to_str3(t_vec_[lcl + 1]) + "/" +
                  to_str3(s.final_time) + " \t E-inc = " + to_str3(e_inc_) +
                  (s.forward_map ? " \t E-inc_f = " + to_str3(e_inc_f_) + " \t E-inv = " + to_str3(e_inv_) : std::string()) +
                  " \t C-Time = " + format_duration(tc));
    mon_buf_[kMonTimeC].push_back(tc);
    if (mon_buf_[kMonTimeS].size() >= 256 || saturated || done()) flush_monitor();
    return saturated ? kErrSaturated : kOk;
}

// ---------------------------------------------------------------- ensemble step pieces
int EulerSim::ens_check(std::string* why) const
{
    auto no = [&](const char* w) { if (why) *why = w; return 0; };
    if (!mixed_) return no("ensemble members run in the mixed form (precision=mixed)");
    if (vlasov_) return no("ensemble members are 2D Euler runs");
    if (ups_) return no("ensemble members evaluate psi exactly (no upsampler)");
    if (L != 3) return no("ensemble members use three Lagrange levels");
    if (s.time_integration_num != 10 && s.time_integration_num != 21 && s.time_integration_num != 30)
        return no("ensemble members advect their maps with EulerExp, RK2 or RK3");
    if (s.forward_map) return no("ensemble members have no forward map");
    if (s.map_update_order_num > 1) return no("ensemble members use 2nd or 4th order map updates");
    // the batched kernels keep per-member weight tables of the vort/map and fine/map ratios
    if (gv.NX / gc.NX > 32 || gf.NX / gc.NX > 32) return no("ensemble members need vort and fine grids at most 32x the map grid");
    return 1;
}

void EulerSim::ens_bind(float* sample_out, const float2* spec_v, float2* spec4, const float* planes,
                        unsigned long long* einc)
{
    ens_sample_ = sample_out;
    ens_spec_v_ = spec_v;
    ens_spec4_ = spec4;
    ens_planes_ = planes;
    ens_einc_ = einc;
}

void EulerSim::flush_monitor()
{
    static const char* names[kMonSeries] = {"Time_s", "Error_incompressibility", "Error_incompressibility_forward",
                                            "Error_invertibility", "Map_gaps", "Map_counter", "Time_c"};
    bool any = false;
    for (auto& b : mon_buf_) any = any || !b.empty();
    if (!any) return;
    std::string dir = run_dir(s) + "/Monitoring_data/";
    for (int k = 0; k < kMonSeries; ++k) {
        if (mon_buf_[k].empty()) continue;
        append_f64(dir + names[k] + ".data", mon_buf_[k].data(), mon_buf_[k].size());
        mon_buf_[k].clear();
    }
}

int EulerSim::ens_begin(EnsMember& e)
{
    // step_once up to the advection: the time step (compute_next_timestep, clipped to the
    // final time), the Lagrange coefficients and the advection's descriptor (advect_m)
    e.active = 0;
    if (done()) return 1;
    const int lcl = loop_ctr_ + L - 1;
    const double t = t_vec_[lcl];
    double dt_now = compute_next_timestep(t);
    if (t + dt_now > s.final_time) dt_now = s.final_time - t;
    t_vec_[lcl + 1] = t + dt_now;
    dt_vec_[lcl + 1] = dt_now;
    ens_lcl_ = lcl;
    ens_dt_ = dt_now;
    const double* tv = t_vec_.data();
    double L1[kMaxLagrange] = {0, 0, 0, 0}, L12[kMaxLagrange] = {0, 0, 0, 0};
    for (int i = 0; i < L; ++i) {
        L1[i] = lagrange_coefficient(tv, tv[lcl + 1], lcl, i, L);
        L12[i] = lagrange_coefficient(tv, tv[lcl] + dt_now / 2.0, lcl, i, L);
    }
    const int ti = s.time_integration_num;
    AdvectMArgs a{};
    a.gm = gc; a.gp = gp;
    a.map = mapm_; a.out = mapm_new_;
    a.psiA = psiA_; a.psiB = psiB_; a.psi0 = psim_[0]; a.psi1 = psim_[1];
    double coef[4][kMaxFoot];
    map_update_coefficients(s.map_update_order_num, s.map_epsilon, coef, &a.nfoot);
    for (int p = 0; p < 4; ++p)
        for (int k = 0; k < kMaxFoot; ++k) { a.coef[p][k] = (float)coef[p][k]; a.coef64[p][k] = coef[p][k]; }
    a.dt = (float)dt_now;
    a.ep = (float)s.map_epsilon;
    a.dt64 = dt_now;
    a.ep64 = s.map_epsilon;
    a.time_integration_num = ti;
    a.rp = gp.NX / gc.NX;
    a.nx_log2 = (gc.NX & (gc.NX - 1)) == 0 ? __builtin_ctz((unsigned)gc.NX) : -1;
    e.adv = a;
    e.active = 1;
    // the previous psi solve's fused combinations, if its predicted coefficients are these
    const bool half = ti == 30;
    bool have = fused_;
    for (int i = 0; i < L && have; ++i) have = L1[i] == fusedL1_[i] && (!half || L12[i] == fusedL12_[i]);
    e.precombine = !have;
    e.lv0 = psim_[0]; e.lv1 = psim_[1]; e.lv2 = psim_[2];
    e.pa = psiA_;
    e.pb = half ? psiB_ : nullptr;
    for (int i = 0; i < 3; ++i) { e.ca[i] = (float)L1[i]; e.cb[i] = (float)L12[i]; }
    e.r_check = gf.NX / gc.NX;
    e.ir_check = 1.0f / (float)e.r_check;
    e.einc = ens_einc_;
    e.fused = 0;
    return 0;
}

int EulerSim::ens_middle(double e_inc, EnsMember& e, EnsMember* remap)
{
    // step_once after the incompressibility check: the remap decision and remap, the
    // psi rotation, and the descriptor of the psi solve with its fused combinations
    std::swap(mapm_, mapm_new_);
    e_inc_ = e_inc;
    ens_saturated_ = false;
    int rc;
    if (e_inc_ > s.incomp_threshold && !s.skip_remapping) {
        if (n_maps_ >= max_maps) {
            if (s.verbose >= 0) log_.push("Stack Saturated : Exitting");
            ens_saturated_ = true;
            continue_ = false;
        } else if (remap) {
            // the remap runs in the ensemble's batched remap launch (launch_ens_fused, remaps
            // only): its descriptor, the stack's room; the map moves to the stack there
            old_ctr_ = loop_ctr_;
            if ((rc = reserve_stack(n_maps_ + 1))) return rc;
            *remap = EnsMember{};
            remap_fields(*remap, true);
            remap->active = 1;
            remap->threshold = -1.0;   // decided here: every member in the launch remaps
            remap->adv.gm = gc;
            remap->adv.gp = gp;
            remap->adv.out = mapm_;
            n_maps_++;
            kernel_launches++;
        } else {
            old_ctr_ = loop_ctr_;
            if ((rc = translate_ic())) return rc;
            if (s.save_map_stack && (rc = write_map_stack(n_maps_))) return rc;
            if ((rc = push_stack())) return rc;
            if ((rc = reset_map())) return rc;
            kernel_launches++;
        }
    }
    ens_gap_ = loop_ctr_ - old_ctr_;
    ens_counter_ = n_maps_;
    rotate_psi(L - 1);
    // the next advection's and this step's tracers' combinations, for the predicted next dt
    const int lcl = ens_lcl_;
    const double* t = t_vec_.data();
    const double tn = t[lcl + 1];
    double dtn = compute_next_timestep(tn);
    if (tn + dtn > s.final_time) dtn = s.final_time - tn;
    for (int i = 0; i < L; ++i) {
        fusedLp_[i] = lagrange_coefficient(t, t[lcl] + dt_vec_[lcl + 1] / 2.0, lcl + 1, i, L);
        fusedL1_[i] = lagrange_coefficient(t, tn + dtn, lcl + 1, i, L);
        fusedL12_[i] = lagrange_coefficient(t, tn + dtn / 2.0, lcl + 1, i, L);
    }
    fused_ = true;
    e.adv.map = mapm_;
    e.gv = gv;
    e.gf = gf;
    e.wfm = wfm_;
    e.sample_out = ens_sample_;
    e.spec_v = ens_spec_v_;
    e.spec4 = ens_spec4_;
    e.planes = ens_planes_;
    e.freq = (float)s.freq_cut_psi;
    e.inv_nv = (float)(1.0 / (double)gv.N);
    e.psi_new = psim_[0];
    e.lv1n = psim_[1];
    e.lv2n = psim_[2];
    e.o1 = psiP_; e.o2 = psiA_; e.o3 = psiB_;
    for (int l = 0; l < 3; ++l) {
        e.cm.c[0][l] = (float)fusedLp_[l];
        e.cm.c[1][l] = (float)fusedL1_[l];
        e.cm.c[2][l] = (float)fusedL12_[l];
    }
    e.fused = 1;
    e.vort = vort;
    e.precombine = 0;
    return kOk;
}

int EulerSim::ens_end()
{
    // step_once after the psi solve and the coarse vorticity
    int rc;
    const int lcl = ens_lcl_;
    if ((rc = advect_particles(lcl))) return rc;
    if ((rc = save_functions(t_vec_[lcl + 1], ens_dt_))) return rc;
    loop_ctr_++;
    mon_buf_[kMonTimeS].push_back(t_vec_[lcl + 1]);
    mon_buf_[kMonEinc].push_back(e_inc_);
    mon_buf_[kMonGap].push_back(ens_gap_);
    mon_buf_[kMonCounter].push_back(ens_counter_);
    if (mon_buf_[kMonTimeS].size() >= 1024) flush_monitor();
    return ens_saturated_ ? kErrSaturated : kOk;
}

int EulerSim::ens_fused_check(std::string* why) const
{
    auto no = [&](const char* w) { if (why) *why = w; return 0; };
    if (s.save_map_stack) return no("the map stack is written at remaps (save_map_stack)");
    if (gv.NX % gc.NX || gv.NY % gc.NY || gv.NX / gc.NX != gv.NY / gc.NY) return no("vort grid not a multiple of the map grid");
    if (gf.NX % gv.NX || gf.NY % gv.NY) return no("fine grid not a multiple of the vort grid");
    if (gf.b0 != gc.b0 || gf.b2 != gc.b2 || gf.Wx != gc.Wx || gf.Wy != gc.Wy) return no("fine and map grids span different domains");
    if (s.initial_discrete && (gd.b0 != gc.b0 || gd.b2 != gc.b2 || gd.Wx != gc.Wx || gd.Wy != gc.Wy))
        return no("discrete initial field on another domain");
    return 1;
}

void EulerSim::ens_fused_bind(int cls, float* real, float2* w1, float2* w2)
{
    ens_cls_ = cls;
    ens_real_ = real;
    ens_w1_ = w1;
    ens_w2_ = w2;
}

int EulerSim::ens_fused_prepare(EnsMember& e)
{
    // ens_middle's work that does not depend on the remap decision, done ahead of the launch:
    // room on the stack for a push, the psi rotation, the predicted combinations, and the
    // descriptor of the psi solve (on the advected map, mapm_new_ until the swap after it)
    int rc;
    const bool can = !s.skip_remapping && n_maps_ < max_maps;
    if (can && (rc = reserve_stack(n_maps_ + 1))) return rc;
    rotate_psi(L - 1);
    const int lcl = ens_lcl_;
    const double* t = t_vec_.data();
    const double tn = t[lcl + 1];
    double dtn = compute_next_timestep(tn);
    if (tn + dtn > s.final_time) dtn = s.final_time - tn;
    for (int i = 0; i < L; ++i) {
        fusedLp_[i] = lagrange_coefficient(t, t[lcl] + dt_vec_[lcl + 1] / 2.0, lcl + 1, i, L);
        fusedL1_[i] = lagrange_coefficient(t, tn + dtn, lcl + 1, i, L);
        fusedL12_[i] = lagrange_coefficient(t, tn + dtn / 2.0, lcl + 1, i, L);
    }
    fused_ = true;
    e.gv = gv;
    e.gf = gf;
    e.wfm = wfm_;
    e.wfm_out = wfm_;
    e.sample_out = ens_real_;
    e.real = ens_real_;
    e.w1 = ens_w1_;
    e.w2 = ens_w2_;
    e.freq = (float)s.freq_cut_psi;
    e.inv_nv = (float)(1.0 / (double)gv.N);
    e.inv_nf = (float)(1.0 / (double)gf.N);
    e.psi_new = psim_[0];
    e.lv1n = psim_[1];
    e.lv2n = psim_[2];
    e.o1 = psiP_; e.o2 = psiA_; e.o3 = psiB_;
    for (int l = 0; l < 3; ++l) {
        e.cm.c[0][l] = (float)fusedLp_[l];
        e.cm.c[1][l] = (float)fusedL1_[l];
        e.cm.c[2][l] = (float)fusedL12_[l];
    }
    e.fused = 1;
    e.vort = vort;
    remap_fields(e, can);
    return kOk;
}

void EulerSim::remap_fields(EnsMember& e, bool can)
{
    // what the batched remap (compose, fine-grid transforms, push, reset) reads: the stack, the
    // slot of the next map, omega_0 as translate_ic gives it to launch_compose_m, the work arrays
    e.gf = gf;
    e.wfm_out = wfm_;
    e.real = ens_real_;
    e.w1 = ens_w1_;
    e.w2 = ens_w2_;
    e.inv_nf = (float)(1.0 / (double)gf.N);
    e.cls = ens_cls_;
    e.can_remap = can ? 1 : 0;
    e.threshold = s.incomp_threshold;
    e.n_maps = n_maps_;
    e.stack = stackm_;
    e.push_slot = can ? stackm_ + 2 * (size_t)n_maps_ * gc.N : nullptr;
    e.src = InitSource{};
    e.src.kind = s.initial_discrete ? 3 : 0;
    e.src.ic_num = s.initial_condition_num;
    e.src.discrete = wdisc;
    e.src.gd = gd;
    e.src.params = d_params_;
    e.src.rand_table = d_rand_;
    e.disc = wdiscm_;
    fix_constants(gc, gf, &e.stx, &e.sty, &e.scx, &e.scy);
}

int EulerSim::ens_fused_finish(double e_inc, bool remapped)
{
    // ens_middle's bookkeeping for the decision the device made with the same comparison
    std::swap(mapm_, mapm_new_);
    e_inc_ = e_inc;
    ens_saturated_ = false;
    const bool wants = e_inc_ > s.incomp_threshold && !s.skip_remapping;
    if (remapped != (wants && n_maps_ < max_maps)) {
        err = "remap decision of the batched iteration differs from the host's";
        return kErrState;
    }
    if (wants && !remapped) {
        if (s.verbose >= 0) log_.push("Stack Saturated : Exitting");
        ens_saturated_ = true;
        continue_ = false;
    } else if (remapped) {
        old_ctr_ = loop_ctr_;
        n_maps_++;
        kernel_launches++;
    }
    ens_gap_ = loop_ctr_ - old_ctr_;
    ens_counter_ = n_maps_;
    return kOk;
}

int EulerSim::finish()
{
    if (!initialised_) { err = "finish before init"; return kErrState; }
    if (finished_) return kOk;
    flush_monitor();
    int rc = save_functions(kTMax, dt);
    if (rc) return rc;
    if (s.save_map_stack) {
        // cmm-euler2d.cu:1033-1051: the active map, psi and the particle state
        if (s.verbose >= 2) {
            std::ostringstream os;
            os.precision(16);
            os << "Saving last Map of MapStack : Maps = " << n_maps_ << " \t Total size = "
               << (n_maps_ + 1) * (8.0 * gc.N * 8 / 1e6) << "mb \t S-time = " << time();
            log_.push(os.str());
        }
        if ((rc = write_map_stack(-1)) || (rc = write_particles_state())) return rc;
        if (s.forward_map && (rc = write_map_stack(-1, true))) return rc;
    }
    CMM_CUDA(cudaStreamSynchronize(stream));
    double tc = wall();
    append_f64(run_dir(s) + "/Monitoring_data/Time_c.data", &tc, 1);
    if (s.verbose >= 1) log_.push("Finished simulation \t Last Cuda Error = cudaSuccess \t C-Time = " + format_duration(tc));
    finished_ = true;
    return kOk;
}

// ---------------------------------------------------------------- saves
static bool instant_fires(bool is_instant, double start, double end, double step, double t_now, double dt_now, double dt)
{
    // src/ui/cmm-io.cu:302-317
    if (is_instant) return t_now - start + dt * 1e-5 < dt_now && t_now - start + dt * 1e-5 >= 0;
    return (std::fmod(t_now - start + dt * 1e-5, step) < dt_now && t_now + dt * 1e-5 >= start && t_now - dt * 1e-5 <= end) ||
           t_now == end;
}

int EulerSim::save_functions(double t_now, double dt_now)
{
    int rc;
    if ((rc = write_time_step(t_now, dt_now))) return rc;
    if ((rc = conservation(t_now, dt_now))) return rc;
    if ((rc = sample_outputs(t_now, dt_now))) return rc;
    if ((rc = zoom_outputs(t_now, dt_now))) return rc;
    return kOk;
}

int EulerSim::sample_outputs(double t_now, double dt_now)
{
    // sample_compute_and_write, backward-map part (src/simulation/cmm-simulation-host.cu:706-893):
    // the full map on the sample grid, scalar and vorticity there, their spectral
    // derivatives, psi and velocity, the sample-grid conservation values
    if (vlasov_) return vlasov_sample_outputs(t_now, dt_now);
    for (auto& r : s.save_sample) {
        if (r.grid <= 0 || !instant_fires(r.is_instant, r.time_start, r.time_end, r.time_step, t_now, dt_now, dt)) continue;
        const int n = r.grid;
        Grid gs = make_grid(n, n, s.domain_bounds);
        int rb;
        if ((rb = reserve_sample_buffers(n))) return rb;
        if (n != smp_plan_n_) {
            destroy_plans(ps_);
            smp_plan_n_ = 0;
            if (!make_plans(ps_, gs, stream)) { err = "FFT plan creation failed (sample grid)"; return kErrParam; }
            smp_plan_n_ = n;
        }
        double *X = smp_[0], *Y = smp_[1], *S = smp_[2], *W = smp_[3], *P = smp_[4], *T = smp_[5];
        double2 *F0 = smp_c_[0], *F1 = smp_c_[1];
        const std::string ns = std::to_string(n), var = r.var;
        const bool all = has(var, "All"), dbg = s.verbose >= 4;
        const std::string tname = std::abs(t_now - kTMax) < 1 ? "final" : to_str3(t_now);
        const std::string sub = "/Time_data/Time_" + tname, mdir = run_dir(s) + "/Monitoring_data/";
        if (dbg) append_f64(mdir + "Debug_globals/Time_s_" + ns + ".data", &t_now, 1);
        else make_dir(run_dir(s) + sub);
        auto out = [&](const std::string& name, const double* v) {
            return dbg ? debug_globals(name + "_" + ns, v, gs.N, true, gs) : write_field(sub, name + "_" + ns, v, gs.N);
        };
        auto sumsq = [&](const double* v, double* hv) {
            int rc2 = check(launch_sumsq(v, gs.N, red_, d_scal_ + 12, stream), "sumsq");
            kernel_launches += 2;
            if (!rc2) rc2 = check(cudaMemcpyAsync(h_scal_ + 12, d_scal_ + 12, sizeof(double), cudaMemcpyDeviceToHost, stream), "copy");
            if (!rc2) rc2 = check(cudaStreamSynchronize(stream), "sync");
            *hv = h_scal_[12];
            return rc2;
        };
        // spectral operator op of the field whose half spectrum is in F0 -> T (F1 is consumed)
        auto spec = [&](int op, double* dst) {
            int rc2 = check(launch_spec_op(F0, gs, op, F1, stream), "spec_op");
            kernel_launches++;
            if (!rc2) rc2 = check(fft_z2d(ps_, F1, dst, 1, stream), "FFT Z2D (sample grid)");
            fft_calls++;
            return rc2;
        };
        int rc;
        if (s.forward_map && (has(var, "Map_f") || has(var, "Chi_f") || all || !s.particles_forwarded.empty())) {
            // forward part (cmm-simulation-host.cu:736-782): the forward map on the sample grid and
            // the forwarded particles, written raw to Particle_data at every verbosity
            CMM_LAUNCH(1, launch_compose_fwd(gc, gs, ChiX_f, ChiY_f, stack_f, n_maps_f_, X, Y, stream));
            if (has(var, "Map_f") || has(var, "Chi_f") || all)
                if ((rc = out("Map_ChiX_f", X)) || (rc = out("Map_ChiY_f", Y))) return rc;
            if ((rc = write_forwarded(s.domain_bounds, "/Particle_data/Time_" + tname, false, var))) return rc;
        }
        if (mixed_) {
            SepDrift drift;
            CMM_LAUNCH(1, launch_compose_pos_m(gc, gs, mapm_, stackm_, n_maps_, X, Y, stream,
                                               sep_drift(drift, map_tau_)));
        } else {
            CMM_LAUNCH(1, launch_compose_pos(gc, gs, ChiX, ChiY, stack, n_maps_, X, Y, stream));
        }
        if (has(var, "Map_b") || has(var, "Chi_b") || all) {
            if ((rc = out("Map_ChiX", X)) || (rc = out("Map_ChiY", Y))) return rc;
        }
        InitSource src{};
        src.params = d_params_;
        src.rand_table = d_rand_;
        if (has(var, "Scalar") || has(var, "Theta") || all) {
            scalar_source(src);
            CMM_LAUNCH(1, launch_eval_init(X, Y, gs.N, src, S, stream));
            if ((rc = out("Scalar_Theta", S))) return rc;
            // Compute_avg reduces with thrust::maximum: hx hy max(0, max theta) (cmm-mesure.cu:226-229)
            CMM_LAUNCH(2, launch_stats(S, gs.N, 1, red_, d_scal_ + 8, stream));
            CMM_CUDA(cudaMemcpyAsync(h_scal_ + 8, d_scal_ + 8, sizeof(double) * 4, cudaMemcpyDeviceToHost, stream));
            CMM_CUDA(cudaStreamSynchronize(stream));
            double si = gs.hx * gs.hy * h_scal_[10];
            append_f64(mdir + "Mesure/Scalar_integral_" + ns + ".data", &si, 1);
        }
        src.kind = s.initial_discrete ? 3 : 0;
        src.ic_num = s.initial_condition_num;
        src.discrete = wdisc;
        src.gd = gd;
        CMM_LAUNCH(1, launch_eval_init(X, Y, gs.N, src, W, stream));
        if (has(var, "Vorticity") || has(var, "W") || has(var, "F") || all)
            if ((rc = out("Vorticity_W", W))) return rc;
        double mes[4], a, b2;
        if ((rc = sumsq(W, &a))) return rc;
        mes[1] = 0.5 * gs.hx * gs.hy * a;
        CMM_FFT(fft_d2z(ps_, W, F0, stream));
        if ((rc = spec(1, T)) || (rc = sumsq(T, &a))) return rc;
        if (has(var, "Grad_W") || all) if ((rc = out("GradX_W", T))) return rc;
        if ((rc = spec(2, T)) || (rc = sumsq(T, &b2))) return rc;
        if (has(var, "Grad_W") || all) if ((rc = out("GradY_W", T))) return rc;
        mes[2] = 0.5 * gs.hx * gs.hy * a + 0.5 * gs.hx * gs.hy * b2;
        // both extremes are taken with Compute_max in the reference (cmm-simulation-host.cu:807-809)
        CMM_LAUNCH(2, launch_stats(W, gs.N, 1, red_, d_scal_ + 8, stream));
        CMM_CUDA(cudaMemcpyAsync(h_scal_ + 8, d_scal_ + 8, sizeof(double) * 4, cudaMemcpyDeviceToHost, stream));
        CMM_CUDA(cudaStreamSynchronize(stream));
        mes[3] = std::max(h_scal_[9], -h_scal_[9]);
        if (has(var, "Laplacian_W") || all) {
            if ((rc = spec(0, T)) || (rc = out("Laplacian_W", T))) return rc;
        }
        if ((rc = spec(3, P))) return rc;
        if (has(var, "Stream") || has(var, "Psi") || all) if ((rc = out("Stream_function_Psi", P))) return rc;
        CMM_FFT(fft_d2z(ps_, P, F0, stream));
        if ((rc = spec(1, T)) || (rc = sumsq(T, &a))) return rc;
        if (has(var, "Velocity") || has(var, "U") || all) if ((rc = out("Velocity_UX", T))) return rc;
        if ((rc = spec(2, T)) || (rc = sumsq(T, &b2))) return rc;
        if (has(var, "Velocity") || has(var, "U") || all) if ((rc = out("Velocity_UY", T))) return rc;
        mes[0] = 0.5 * gs.hx * gs.hy * a + 0.5 * gs.hx * gs.hy * b2;
        append_f64(mdir + "Mesure/Time_s_" + ns + ".data", &t_now, 1);
        append_f64(mdir + "Mesure/Energy_" + ns + ".data", &mes[0], 1);
        append_f64(mdir + "Mesure/Enstrophy_" + ns + ".data", &mes[1], 1);
        append_f64(mdir + "Mesure/Palinstrophy_" + ns + ".data", &mes[2], 1);
        append_f64(mdir + "Mesure/Max_vorticity_" + ns + ".data", &mes[3], 1);
        if (s.verbose >= 3)
            log_.push("Processed sample data on grid " + ns + ", Cons : Energ = " + to_str_prec(mes[0], 8) +
                      " \t Enstr = " + to_str_prec(mes[1], 8) + " \t Palinstr = " + to_str_prec(mes[2], 8) +
                      " \t Wmax = " + to_str_prec(mes[3], 8));
    }
    return kOk;
}

int EulerSim::vlasov_sample_outputs(double t_now, double dt_now)
{
    // sample_compute_and_write_vlasov, backward-map part (cmm-simulation-host.cu:898-1030): the
    // full map and the distribution function on the sample grid, its kinetic energy, momentum
    // and mass there (Compute_Kinetic_Energy / _Momentum / _Mass, cmm-mesure.cu:97-183), the
    // field e = d phi / dx of calc_phi on the sample grid itself (v-integral, 1D inverse
    // Laplacian, 1D derivative: cmm-simulation-host.cu:436-471, 1006-1009) and its potential
    // energy, and the four mode amplitudes of the run's own field (Compute_kth_Mode on psi_x
    // row 0).  The reference writes its sample buffer as Stream_function_Psi after those in-place
    // steps: e in the first n entries, the distribution from entry N / 8 on, left-over scratch
    // between (written here as 0).
    for (size_t i_save = 0; i_save < s.save_sample.size(); ++i_save) {
        auto& r = s.save_sample[i_save];
        if (r.grid <= 0 || !instant_fires(r.is_instant, r.time_start, r.time_end, r.time_step, t_now, dt_now, dt)) continue;
        const int n = r.grid;
        Grid gs = make_grid(n, n, s.domain_bounds);
        int rc;
        if ((rc = reserve_sample_buffers(n))) return rc;
        if (n != vsmp_plan_n_) {
            destroy_vlasov_plans(vps_);
            vsmp_plan_n_ = 0;
            if (!make_vlasov_plans(vps_, gs, gs, stream)) { err = "FFT plan creation failed (1D, sample grid)"; return kErrParam; }
            vsmp_plan_n_ = n;
        }
        double *X = smp_[0], *Y = smp_[1], *E = smp_[2], *F = smp_[3], *P = smp_[4], *T = smp_[5];
        double2 *F0 = smp_c_[0], *F1 = smp_c_[1];
        const std::string ns = std::to_string(n), var = r.var;
        const bool all = has(var, "All"), dbg = s.verbose >= 4;
        const std::string tname = std::abs(t_now - kTMax) < 1 ? "final" : to_str3(t_now);
        const std::string sub = "/Time_data/Time_" + tname, mdir = run_dir(s) + "/Monitoring_data/";
        if (dbg) append_f64(mdir + "Debug_globals/Time_s_" + ns + ".data", &t_now, 1);
        else make_dir(run_dir(s) + sub);
        auto out = [&](const std::string& name, const double* v) {
            return dbg ? debug_globals(name + "_" + ns, v, gs.N, true, gs) : write_field(sub, name + "_" + ns, v, gs.N);
        };
        if (s.forward_map && (has(var, "Map_f") || has(var, "Chi_f") || all)) {
            CMM_LAUNCH(1, launch_compose_fwd(gc, gs, ChiX_f, ChiY_f, stack_f, n_maps_f_, X, Y, stream));
            if ((rc = out("Map_ChiX_f", X)) || (rc = out("Map_ChiY_f", Y))) return rc;
        }
        if (mixed_) {
            SepDrift drift;
            CMM_LAUNCH(1, launch_compose_pos_m(gc, gs, mapm_, stackm_, n_maps_, X, Y, stream,
                                               sep_drift(drift, map_tau_)));
        } else {
            CMM_LAUNCH(1, launch_compose_pos(gc, gs, ChiX, ChiY, stack, n_maps_, X, Y, stream));
        }
        if (has(var, "Map_b") || has(var, "Chi_b") || all)
            if ((rc = out("Map_ChiX", X)) || (rc = out("Map_ChiY", Y))) return rc;
        InitSource src{};
        src.kind = s.initial_discrete ? 3 : 2;
        src.ic_num = s.initial_condition_num;
        src.discrete = wdisc;
        src.gd = gd;
        src.params = d_params_;
        src.rand_table = d_rand_;
        CMM_LAUNCH(1, launch_eval_init(X, Y, gs.N, src, F, stream));
        if (has(var, "Dist") || has(var, "F") || all)
            if ((rc = out("Distribution_F", F))) return rc;
        // moments of f on the sample grid -> d_scal_[0..2]
        CMM_LAUNCH(2, launch_vlasov_moments(F, gs, red_, d_scal_, stream));
        // e = d phi / dx from f on the sample grid: rho (partials in T) -> 1D spectra -> E
        CMM_LAUNCH(2, launch_vlasov_rho(F, nullptr, gs, T, P, stream));
        CMM_FFT(fft_d2z_1d(vps_.v, P, F0, stream));
        CMM_LAUNCH(1, launch_vlasov_phi_spec(F0, gs, gs, F1, reinterpret_cast<double2*>(T), stream));
        CMM_FFT(fft_z2d_1d(vps_.p, reinterpret_cast<const double2*>(T), E, stream));
        CMM_LAUNCH(2, launch_sumsq(E, n, red_, d_scal_ + 3, stream));
        // mode amplitudes of the run's field phi' (psi_x row 0)
        CMM_CUDA(cudaMemcpyAsync(real_buf_, phi_lv_[0] + gp.NX, sizeof(double) * gp.NX, cudaMemcpyDeviceToDevice, stream));
        CMM_FFT(fft_d2z_1d(vp_.p, real_buf_, vl_c_[0], stream));
        CMM_LAUNCH(1, launch_vlasov_modes(vl_c_[0], gp.NX, gp.NX_fft, d_scal_ + 4, stream));
        if (has(var, "Stream") || has(var, "Psi") || all) {
            const long long tail = std::max<long long>(gs.N / 8, (long long)n + 2);
            CMM_CUDA(cudaMemsetAsync(P, 0, sizeof(double) * gs.N, stream));
            CMM_CUDA(cudaMemcpyAsync(P, E, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
            if (tail < gs.N)
                CMM_CUDA(cudaMemcpyAsync(P + tail, F + tail, sizeof(double) * (gs.N - tail), cudaMemcpyDeviceToDevice,
                                         stream));
            if ((rc = out("Stream_function_Psi", P))) return rc;
        }
        CMM_CUDA(cudaMemcpyAsync(h_scal_, d_scal_, sizeof(double) * 8, cudaMemcpyDeviceToHost, stream));
        CMM_CUDA(cudaStreamSynchronize(stream));
        const double hh = gs.hx * gs.hy;
        double mes[9];
        mes[1] = 0.5 * hh * h_scal_[2];
        mes[2] = 0.5 * gs.hx * h_scal_[3];
        mes[0] = mes[1] + mes[2];
        mes[3] = hh * h_scal_[0];
        mes[4] = hh * h_scal_[1];
        for (int k = 0; k < 4; ++k) mes[5 + k] = h_scal_[4 + k];
        static const char* names[9] = {"Etot", "Ekin", "Epot", "Mass", "Momentum", "Emode1", "Emode2", "Emode3", "Emode4"};
        append_f64(mdir + "Mesure/Time_s_" + ns + ".data", &t_now, 1);
        for (int k = 0; k < 9; ++k) append_f64(mdir + "Mesure/" + names[k] + "_" + ns + ".data", &mes[k], 1);
        if (s.verbose >= 3)
            log_.push("Saved sample data " + std::to_string(i_save + 1) + " on grid " + ns + ", Cons : Etot = " +
                      to_str_prec(mes[0], 8) + " \t Momenta = " + to_str_prec(mes[4], 8) + " \t Ekin = " +
                      to_str_prec(mes[1], 8) + " \t Epot = " + to_str_prec(mes[2], 8) + " \t Mass = " +
                      to_str_prec(mes[3], 8));
    }
    return kOk;
}

int EulerSim::write_forwarded(const double* frame, const std::string& sub, bool zoom, const std::string& var)
{
    if (s.particles_forwarded.empty()) return kOk;
    int rc;
    if ((rc = forwarded_positions(frame, fpos_))) return rc;
    size_t off = 0;
    for (size_t i = 0; i < s.particles_forwarded.size(); ++i) {
        const int num = std::max(s.particles_forwarded[i].num, 0);
        const bool want = has(var, ("PartF_" + two((int)i + 1)).c_str()) || (!zoom && has(var, "All"));
        if (want && num > 0) {
            make_dir(run_dir(s) + sub.substr(0, sub.rfind('/')));
            make_dir(run_dir(s) + sub);
            if ((rc = write_field(sub, "Particles_forwarded_pos_P" + two(zoom ? (int)i : (int)i + 1), fpos_ + off, 2ll * num)))
                return rc;
        }
        off += 2 * (size_t)num;
    }
    return kOk;
}

int EulerSim::reserve_sample_buffers(int n)
{
    if (n <= smp_n_) return kOk;
    Grid g = make_grid(n, n, s.domain_bounds);
    auto f = [](void* p) { if (p) cudaFree(p); };
    for (auto& p : smp_) { f(p); p = nullptr; }
    for (auto& p : smp_c_) { f(p); p = nullptr; }
    smp_n_ = 0;
    for (auto& p : smp_) CMM_CUDA(cudaMalloc((void**)&p, sizeof(double) * (size_t)g.N));
    for (auto& p : smp_c_) CMM_CUDA(cudaMalloc((void**)&p, sizeof(double2) * (size_t)g.Nfft));
    smp_n_ = n;
    return kOk;
}

int EulerSim::zoom_outputs(double t_now, double dt_now)
{
    // compute_zoom, backward-map part (src/simulation/cmm-simulation-host.cu:1039-1201): for
    // each firing zoom record, rep windows of half-width width/2 * rep_fac^k around
    // (pos_x, pos_y); on each n x n window grid the full backward map, the passive scalar,
    // the vorticity, the distribution function and psi sampled at the window points.
    // Statistics use the spacing of the n x n grid over the whole domain, the reference's
    // zoom variable's own grid.
    if (vlasov_) return kOk;
    bool synced = false;
    for (size_t iz = 0; iz < s.save_zoom.size(); ++iz) {
        auto& r = s.save_zoom[iz];
        if (r.grid <= 0 || r.rep <= 0 || !instant_fires(r.is_instant, r.time_start, r.time_end, r.time_step, t_now, dt_now, dt))
            continue;
        const int n = r.grid;
        int rc;
        if ((rc = reserve_sample_buffers(n))) return rc;
        if (!synced && mixed_) {
            if ((rc = sync_fp64_views())) return rc;   // psi level 0 as FP64 planes
            synced = true;
        }
        const Grid gstat = make_grid(n, n, s.domain_bounds);
        const std::string ns = std::to_string(n), zs = "_Zoom_" + std::to_string(iz + 1), var = r.var;
        const bool all = has(var, "All"), dbg = s.verbose >= 4;
        const std::string tname = std::abs(t_now - kTMax) < 1 ? "final" : to_str3(t_now);
        if (dbg) append_f64(run_dir(s) + "/Monitoring_data/Debug_globals/Time_s_" + ns + zs + ".data", &t_now, 1);
        double wx = r.width_x / 2.0, wy = r.width_y / 2.0;
        double *X = smp_[0], *Y = smp_[1], *V = smp_[2];
        for (int rep = 0; rep < r.rep; ++rep) {
            const double b[4] = {r.pos_x - wx, r.pos_x + wx, r.pos_y - wy, r.pos_y + wy};
            const Grid gz = make_grid(n, n, b);
            const std::string rs = zs + "_rep_" + std::to_string(rep);
            const std::string sub = "/Zoom_data/Time_" + tname + "/Zoom_" + std::to_string(iz + 1) + "_rep_" + std::to_string(rep);
            if (!dbg) {
                make_dir(run_dir(s) + "/Zoom_data/Time_" + tname);
                make_dir(run_dir(s) + sub);
            }
            auto out = [&](const std::string& name, const double* v) {
                return dbg ? debug_globals(name + "_" + ns + rs, v, gz.N, true, gstat) : write_field(sub, name + "_" + ns, v, gz.N);
            };
            if (s.forward_map && (has(var, "Map_f") || has(var, "Chi_f") || all || !s.particles_forwarded.empty())) {
                // forward part (cmm-simulation-host.cu:1087-1136): the forwarded particles are
                // written only for sets named with PartF_<ii>, as P<ii - 1>
                CMM_LAUNCH(1, launch_compose_fwd(gc, gz, ChiX_f, ChiY_f, stack_f, n_maps_f_, X, Y, stream));
                if (has(var, "Map_f") || has(var, "Chi_f") || all)
                    if ((rc = out("Map_ChiX_f", X)) || (rc = out("Map_ChiY_f", Y))) return rc;
                if ((rc = write_forwarded(b, sub, true, var))) return rc;
            }
            if (mixed_) {
                SepDrift drift;
                CMM_LAUNCH(1, launch_compose_pos_m(gc, gz, mapm_, stackm_, n_maps_, X, Y, stream,
                                                   sep_drift(drift, map_tau_)));
            } else {
                CMM_LAUNCH(1, launch_compose_pos(gc, gz, ChiX, ChiY, stack, n_maps_, X, Y, stream));
            }
            if (has(var, "Map_b") || has(var, "Chi_b") || all)
                if ((rc = out("Map_ChiX", X)) || (rc = out("Map_ChiY", Y))) return rc;
            InitSource src{};
            src.params = d_params_;
            src.rand_table = d_rand_;
            src.discrete = wdisc;
            src.gd = gd;
            if (has(var, "Scalar") || has(var, "Theta") || all) {
                scalar_source(src);
                CMM_LAUNCH(1, launch_eval_init(X, Y, gz.N, src, V, stream));
                if ((rc = out("Scalar_Theta", V))) return rc;
            }
            src.ic_num = s.initial_condition_num;
            if (has(var, "Vorticity") || has(var, "W") || all) {
                src.kind = s.initial_discrete ? 3 : 0;
                CMM_LAUNCH(1, launch_eval_init(X, Y, gz.N, src, V, stream));
                if ((rc = out("Vorticity_W", V))) return rc;
            }
            if (has(var, "Dist") || has(var, "F") || all) {
                // var 2 of k_h_sample_from_init: the distribution-function formula with this run's IC number
                src.kind = s.initial_discrete ? 3 : 2;
                CMM_LAUNCH(1, launch_eval_init(X, Y, gz.N, src, V, stream));
                if ((rc = out("Distribution", V))) return rc;
            }
            if (has(var, "Stream") || has(var, "Psi") || all) {
                InitSource ps{};
                ps.kind = 3;
                ps.discrete = psi[0];
                ps.gd = gp;
                CMM_LAUNCH(1, launch_eval_grid(gz, ps, V, stream));
                if ((rc = out("Stream_function_Psi", V))) return rc;
            }
            wx *= r.rep_fac;
            wy *= r.rep_fac;
        }
        if (s.verbose >= 3) log_.push("Processed zoom data " + std::to_string(iz + 1) + " on grid " + ns);
    }
    return kOk;
}

int EulerSim::debug_globals(const std::string& name, const double* v, long long n, bool grid_form, const Grid& g)
{
    CMM_LAUNCH(2, launch_stats(v, n, 1, red_, d_scal_ + 8, stream));
    CMM_CUDA(cudaMemcpyAsync(h_scal_ + 8, d_scal_ + 8, sizeof(double) * 4, cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    double m[4] = {h_scal_[8], h_scal_[9], 0, 0};
    if (grid_form) { m[2] = g.hy * g.hx * h_scal_[10]; m[3] = g.hy * g.hx * h_scal_[11]; }
    else { m[2] = h_scal_[10] / (double)n; m[3] = h_scal_[11] / (double)n; }
    std::string base = run_dir(s) + "/Monitoring_data/Debug_globals/" + name;
    const char* suf[4] = {"_Min", "_Max", "_Avg", "_L2"};
    for (int i = 0; i < 4; ++i) append_f64(base + suf[i] + ".data", &m[i], 1);
    return kOk;
}

int EulerSim::write_field(const std::string& sub, const std::string& name, const double* v, long long n)
{
    std::vector<double> h((size_t)n);
    CMM_CUDA(cudaMemcpyAsync(h.data(), v, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    if (!write_f64(run_dir(s) + sub + "/" + name + ".data", h.data(), (size_t)n)) { err = "cannot write " + name; return kErrIO; }
    return kOk;
}

int EulerSim::write_time_step(double t_now, double dt_now)
{
    // writeTimeStep (src/ui/cmm-io.cu:295-437)
    std::string var;
    bool fire = false;
    for (auto& r : s.save_computational)
        if (instant_fires(r.is_instant, r.time_start, r.time_end, r.time_step, t_now, dt_now, dt)) { fire = true; var += r.var; }
    if (!fire) return kOk;
    if (int rc0 = ensure_vort()) return rc0;
    int rs = sync_fp64_views();
    if (rs) return rs;
    std::string tname = std::abs(t_now - kTMax) < 1 ? "final" : to_str3(t_now);
    bool all = has(var, "All");
    bool dbg = s.verbose >= 4;
    std::string sub = "/Time_data/Time_" + tname;
    bool any = has(var, "Vorticity") || has(var, "W") || has(var, "Stream") || has(var, "Psi") || has(var, "Map") ||
               has(var, "Chi") || has(var, "Velocity") || has(var, "U") || has(var, "Dist") || has(var, "F") || all;
    std::string dbg_time = run_dir(s) + "/Monitoring_data/Debug_globals/Time_s.data";
    if (any) {
        make_dir(run_dir(s) + sub);
        if (dbg) append_f64(dbg_time, &t_now, 1);
    }
    int rc;
    auto var2d = [&](const std::string& name, const double* v, const Grid& g) {
        return dbg ? debug_globals(name, v, g.N, true, g) : write_field(sub, name, v, g.N);
    };
    auto arr = [&](const std::string& sub2, const std::string& name, const double* v, long long n) {
        return dbg ? debug_globals(name, v, n, false, gc) : write_field(sub2, name, v, n);
    };
    if (has(var, "Vorticity") || has(var, "W") || all) if ((rc = var2d("Vorticity_W_coarse", vort, gc))) return rc;
    if (has(var, "Dist") || has(var, "F") || all) if ((rc = var2d("Distribution_coarse", vort, gc))) return rc;
    if (has(var, "Stream") || has(var, "Psi") || all) if ((rc = var2d("Stream_function_Psi_psi", psi[0], gp))) return rc;
    if (has(var, "Stream_H") || has(var, "Psi_H") || all)
        if ((rc = arr(sub, "Stream_function_Psi_H_psi", psi[0], 4 * gp.N))) return rc;
    if (has(var, "Velocity") || has(var, "U") || all) {
        if ((rc = var2d("Velocity_UX_psi", psi[0] + gp.N, gp))) return rc;
        if ((rc = var2d("Velocity_UY_psi", psi[0] + 2 * gp.N, gp))) return rc;
    }
    if (has(var, "Map_b") || has(var, "Chi_b") || all) {
        if ((rc = var2d("Map_ChiX_coarse", ChiX, gc))) return rc;
        if ((rc = var2d("Map_ChiY_coarse", ChiY, gc))) return rc;
    }
    if (has(var, "Map_H") || has(var, "Chi_H") || all) {
        if ((rc = arr(sub, "Map_ChiX_H_coarse", ChiX, 4 * gc.N))) return rc;
        if ((rc = arr(sub, "Map_ChiY_H_coarse", ChiY, 4 * gc.N))) return rc;
    }
    if (s.forward_map && (has(var, "Map_f") || has(var, "Chi_f") || all)) {
        if ((rc = var2d("Map_ChiX_f_coarse", ChiX_f, gc))) return rc;
        if ((rc = var2d("Map_ChiY_f_coarse", ChiY_f, gc))) return rc;
    }
    if (s.forward_map && (has(var, "Map_f_H") || has(var, "Chi_f_H") || all)) {
        if ((rc = arr(sub, "Map_ChiX_f_H_coarse", ChiX_f, 4 * gc.N))) return rc;
        if ((rc = arr(sub, "Map_ChiY_f_H_coarse", ChiY_f, 4 * gc.N))) return rc;
    }
    std::string psub = "/Particle_data/Time_" + tname;
    if (has(var, "PartA_") || all) {
        make_dir(run_dir(s) + psub);
        if (!any && dbg) append_f64(dbg_time, &t_now, 1);
    }
    for (size_t i = 0; i < s.particles_advected.size(); ++i) {
        auto& p = s.particles_advected[i];
        std::string id = two((int)i + 1);
        if (has(var, ("PartA_" + id).c_str()) || all)
            if ((rc = arr(psub, "Particles_advected_pos_P" + id, parts[i], 2ll * p.num))) return rc;
        if (has(var, ("PartA_Vel_" + id).c_str()) || all) {
            // inertial sets: their velocity state; tracers: (psi_x, psi_y) sampled there (cmm-io.cu:580-600)
            if (p.tau != 0) {
                if ((rc = arr(psub, "Particles_advected_vel_U" + id, vels[i], 2ll * p.num))) return rc;
            } else {
                CMM_LAUNCH(1, launch_sample_points_dxdy(gp, psi[0], parts[i], real_buf_, p.num, stream));
                if ((rc = arr(psub, "Particles_advected_vel_U" + id, real_buf_, 2ll * p.num))) return rc;
            }
        }
    }
    return kOk;
}

int EulerSim::diagnostics(double* energy, double* enstrophy, double* palinstrophy, double* wmax)
{
    // Compute_Energy_H, Compute_Enstrophy, Compute_Palinstrophy, w max
    // (src/numerical/cmm-mesure.cu:30-89, cmm-simulation-host.cu:668-673)
    if (int rc0 = ensure_vort()) return rc0;
    if (mixed_) CMM_LAUNCH(2, launch_energy_m(psim_[0], gp.N, red_, d_scal_ + 1, stream));
    else CMM_LAUNCH(2, launch_sumsq(psi[0] + gp.N, 2 * gp.N, red_, d_scal_ + 1, stream));
    CMM_LAUNCH(2, launch_sumsq(vort, gc.N, red_, d_scal_ + 2, stream));
    CMM_FFT(fft_d2z(pc_, vort, spec_, stream));
    CMM_LAUNCH(1, launch_spec_grad(spec_, gc, spec4_, stream));
    CMM_FFT(fft_z2d(pc_, spec4_, real_buf_, 1, stream));
    CMM_LAUNCH(2, launch_sumsq(real_buf_, gc.N, red_, d_scal_ + 3, stream));
    CMM_FFT(fft_z2d(pc_, spec4_ + gc.Nfft, real_buf_, 1, stream));
    CMM_LAUNCH(2, launch_sumsq(real_buf_, gc.N, red_, d_scal_ + 4, stream));
    CMM_LAUNCH(2, launch_stats(vort, gc.N, 1, red_, d_scal_ + 8, stream));
    CMM_CUDA(cudaMemcpyAsync(h_scal_, d_scal_, sizeof(double) * 12, cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    *energy = 0.5 * gp.hx * gp.hy * h_scal_[1];
    *enstrophy = 0.5 * gc.hx * gc.hy * h_scal_[2];
    *palinstrophy = 0.5 * gc.hx * gc.hy * h_scal_[3] + 0.5 * gc.hx * gc.hy * h_scal_[4];
    double w_max = std::max(0.0, h_scal_[9]), w_min = std::min(0.0, h_scal_[8]);
    *wmax = std::max(w_max, -w_min);
    return kOk;
}

int EulerSim::conservation(double t_now, double dt_now)
{
    // compute_conservation_targets (src/simulation/cmm-simulation-host.cu:615-698)
    bool fire = false;
    for (auto& r : s.save_computational)
        if (r.conv && instant_fires(r.is_instant, r.time_start, r.time_end, r.time_step, t_now, dt_now, dt)) fire = true;
    if (!fire) return kOk;
    std::string dir = run_dir(s) + "/Monitoring_data/Mesure/";
    if (vlasov_) {
        double v[9];
        int rv = vlasov_mesure(v);
        if (rv) return rv;
        append_f64(dir + "Time_s.data", &t_now, 1);
        const char* names[9] = {"Etot", "Ekin", "Epot", "Mass", "Momentum", "Emode1", "Emode2", "Emode3", "Emode4"};
        for (int k = 0; k < 9; ++k) append_f64(dir + names[k] + ".data", &v[k], 1);
        if (s.verbose >= 3)
            log_.push("Computed coarse Cons : Etot = " + to_str_prec(v[0], 8) + " \t Momenta = " + to_str_prec(v[4], 8) +
                      " \t Ekin = " + to_str_prec(v[1], 8) + " \t Epot = " + to_str_prec(v[2], 8) +
                      " \t Mass = " + to_str_prec(v[3], 8));
        return kOk;
    }
    double m[4];
    int rc = diagnostics(&m[0], &m[1], &m[2], &m[3]);
    if (rc) return rc;
    append_f64(dir + "Time_s.data", &t_now, 1);
    append_f64(dir + "Energy.data", &m[0], 1);
    append_f64(dir + "Enstrophy.data", &m[1], 1);
    append_f64(dir + "Palinstrophy.data", &m[2], 1);
    append_f64(dir + "Max_vorticity.data", &m[3], 1);
    if (s.verbose >= 3)
        log_.push("Computed coarse Cons : Energ = " + to_str_prec(m[0], 8) + " \t Enstr = " + to_str_prec(m[1], 8) +
                  " \t Palinstr = " + to_str_prec(m[2], 8) + " \t Wmax = " + to_str_prec(m[3], 8));
    return kOk;
}

// ---------------------------------------------------------------- fields
size_t EulerSim::field_bytes(const std::string& n) const
{
    if (n == "Map_ChiX_H_coarse" || n == "Map_ChiY_H_coarse") return sizeof(double) * 4 * gc.N;
    if (n == "Stream_function_Psi_H_psi") return sizeof(double) * 4 * gp.N;
    if (n == "Stream_function_Psi_H_psi_all") return sizeof(double) * 4 * gp.N * L;
    if (n == "Vorticity_W_coarse" || n == "Distribution_coarse") return sizeof(double) * gc.N;
    if (n == "Vorticity_W_fine_H") return sizeof(double) * 4 * gf.N;
    if (n == "Map_stack") return sizeof(double) * 8 * gc.N * n_maps_;
    if (n == "Init_random_table") return sizeof(double) * kInitTable;
    if (s.forward_map && (n == "Map_ChiX_f_H_coarse" || n == "Map_ChiY_f_H_coarse")) return sizeof(double) * 4 * gc.N;
    for (size_t i = 0; i < s.particles_forwarded.size() && s.forward_map; ++i)
        if (n == "Particles_forwarded_pos_P" + two((int)i + 1)) return sizeof(double) * 2 * s.particles_forwarded[i].num;
    for (size_t i = 0; i < s.particles_advected.size(); ++i) {
        std::string id = two((int)i + 1);
        if (n == "Particles_advected_pos_P" + id || n == "Particles_advected_vel_U" + id)
            return sizeof(double) * 2 * s.particles_advected[i].num;
    }
    return 0;
}

int EulerSim::get_field(const std::string& n, void* dst, size_t bytes)
{
    if (!initialised_) { err = "get_field before init"; return kErrState; }
    int rs = sync_fp64_views();
    if (rs) return rs;
    size_t need = field_bytes(n);
    if (need == 0 && n != "Map_stack") { err = "unknown field " + n; return kErrNotFound; }
    if (bytes != need) { err = "field " + n + " needs " + std::to_string(need) + " bytes"; return kErrParam; }
    char* d = static_cast<char*>(dst);
    auto cp = [&](const void* src, size_t b) { return check(cudaMemcpyAsync(d, src, b, cudaMemcpyDeviceToHost, stream), "get_field"); };
    int rc = kOk;
    if (n == "Map_ChiX_H_coarse") rc = cp(ChiX, bytes);
    else if (n == "Map_ChiY_H_coarse") rc = cp(ChiY, bytes);
    else if (n == "Stream_function_Psi_H_psi") rc = cp(psi[0], bytes);
    else if (n == "Stream_function_Psi_H_psi_all") {
        size_t lb = sizeof(double) * 4 * gp.N;
        for (int l = 0; l < L && !rc; ++l) { rc = check(cudaMemcpyAsync(d + l * lb, psi[l], lb, cudaMemcpyDeviceToHost, stream), "get_field"); }
    }
    else if (n == "Vorticity_W_coarse" || n == "Distribution_coarse") rc = ensure_vort() ? kErrCuda : cp(vort, bytes);
    else if (n == "Vorticity_W_fine_H") rc = cp(wfine, bytes);
    else if (n == "Init_random_table") rc = cp(d_rand_, bytes);
    else if (n == "Map_ChiX_f_H_coarse") rc = cp(ChiX_f, bytes);
    else if (n == "Map_ChiY_f_H_coarse") rc = cp(ChiY_f, bytes);
    else if (n.rfind("Particles_forwarded_pos_P", 0) == 0) {
        // positions now, mapped on the whole domain
        rc = forwarded_positions(s.domain_bounds, fpos_);
        size_t off = 0;
        for (size_t i = 0; i < s.particles_forwarded.size() && !rc; ++i) {
            if (n == "Particles_forwarded_pos_P" + two((int)i + 1)) rc = cp(fpos_ + off, bytes);
            off += 2 * (size_t)std::max(s.particles_forwarded[i].num, 0);
        }
    }
    else if (n == "Map_stack" && !mixed_) rc = bytes ? cp(stack, bytes) : kOk;
    else if (n == "Map_stack") {
        // FP32 displacement maps -> the reference's planar X | Y layout, one map at a time
        size_t mb = sizeof(double) * 4 * gc.N;
        for (int m = 0; m < n_maps_ && !rc; ++m) {
            SepDrift drift;
            rc = check(launch_map_to_planes(stackm_ + 2 * (size_t)m * gc.N, gc, ChiX_new, ChiY_new, stream,
                                            sep_drift(drift, m < (int)stack_tau_.size() ? stack_tau_[(size_t)m] : 0.0)),
                       "map_to_planes");
            if (!rc) rc = check(cudaMemcpyAsync(d + 2 * m * mb, ChiX_new, mb, cudaMemcpyDeviceToHost, stream), "get_field");
            if (!rc) rc = check(cudaMemcpyAsync(d + (2 * m + 1) * mb, ChiY_new, mb, cudaMemcpyDeviceToHost, stream), "get_field");
        }
    }
    else {
        for (size_t i = 0; i < s.particles_advected.size(); ++i) {
            std::string id = two((int)i + 1);
            if (n == "Particles_advected_pos_P" + id) rc = cp(parts[i], bytes);
            else if (n == "Particles_advected_vel_U" + id && s.particles_advected[i].tau != 0) rc = cp(vels[i], bytes);
            else if (n == "Particles_advected_vel_U" + id) {
                rc = check(launch_sample_points_dxdy(gp, psi[0], parts[i], real_buf_, s.particles_advected[i].num, stream), "dxdy");
                if (!rc) rc = cp(real_buf_, bytes);
            }
        }
    }
    if (rc) return rc;
    CMM_CUDA(cudaStreamSynchronize(stream));
    return kOk;
}

int EulerSim::get_scalar(const std::string& n, double* out)
{
    if (n == "dt") { *out = dt; return kOk; }
    if (n == "lagrange_order") { *out = L; return kOk; }
    if (n == "stack_capacity") { *out = max_maps; return kOk; }
    if (!initialised_) { err = "get_scalar before init"; return kErrState; }
    if (n == "time") { *out = time(); return kOk; }
    if (n == "e_inc") { *out = e_inc_; return kOk; }
    if (n == "map_counter") { *out = n_maps_; return kOk; }
    if (n == "e_inc_forward") { *out = e_inc_f_; return kOk; }
    if (n == "e_invertibility") { *out = e_inv_; return kOk; }
    if (n == "map_gap") { *out = (loop_ctr_ - 1) - old_ctr_; return kOk; }
    if (n == "loop_ctr") { *out = loop_ctr_; return kOk; }
    if (n == "graph_launches") { *out = (double)graph_launches_; return kOk; }
    if (n == "learned_steps") { *out = (double)learned_steps_; return kOk; }
    if (n == "cheap_steps") { *out = (double)cheap_steps_; return kOk; }
    if (n == "learned_cheaper") { *out = (double)learned_cheaper_; return kOk; }
    if (n == "exact_steps") { *out = (double)exact_steps_; return kOk; }
    if (n == "learned_checks") { *out = (double)learned_checks_; return kOk; }
    if (n == "learned_failures") { *out = (double)learned_fails_; return kOk; }
    if (n == "learned_last_err") { *out = learned_last_err_; return kOk; }
    if (n == "learned_max_err") { *out = learned_max_err_; return kOk; }
    if (n == "kernel_launches") { *out = (double)kernel_launches; return kOk; }
    if (n == "fft_calls") { *out = (double)fft_calls; return kOk; }
    for (int p = 0; p < kNumPhases; ++p) {
        std::string base = std::string("prof_") + phase_name(p);
        if (n == base + "_ms") { *out = prof_ms[p]; return kOk; }
        if (n == base + "_count") { *out = (double)prof_count[p]; return kOk; }
    }
    if (vlasov_) {
        const char* names[9] = {"etot", "ekin", "epot", "mass", "momentum", "emode1", "emode2", "emode3", "emode4"};
        for (int k = 0; k < 9; ++k)
            if (n == names[k]) {
                double v[9];
                int rv = vlasov_mesure(v);
                if (rv) return rv;
                *out = v[k];
                return kOk;
            }
    }
    double m[4];
    if (n == "energy" || n == "enstrophy" || n == "palinstrophy" || n == "max_vorticity") {
        int rc = diagnostics(&m[0], &m[1], &m[2], &m[3]);
        if (rc) return rc;
        *out = n == "energy" ? m[0] : n == "enstrophy" ? m[1] : n == "palinstrophy" ? m[2] : m[3];
        return kOk;
    }
    err = "unknown scalar " + n;
    return kErrNotFound;
}

}  // namespace cmm
