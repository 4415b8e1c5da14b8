// sim.hpp -- the 2D Euler CMM simulation context on one GPU (plain FP64 and
// mixed-precision forms).
//
// Owns every device buffer; all work is ordered on one CUDA stream.  The only
// host synchronisation per loop iteration is the 8-byte read of the
// incompressibility error that decides the remap (the reference also blocks
// there, src/simulation/cmm-simulation-host.cu:48-49).
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <string>
#include <vector>

#include "io.hpp"
#include "kernels.hpp"
#include "mixed.hpp"
#include "settings.hpp"
#include "vlasov.hpp"

namespace cmm {

// status codes shared with the C-ABI
enum Status { kOk = 0, kErrParam = -1, kErrIO = -2, kErrCuda = -3, kErrSaturated = -4, kErrState = -5,
              kErrUnsupported = -6, kErrNotFound = -7, kErrTimeout = -8 };

struct EnsMember;
namespace lrn { class Upsampler; }

class EulerSim {
public:
    explicit EulerSim(const Settings& s);
    ~EulerSim();

    int set_stream(cudaStream_t s);
    int set_initial_discrete(const double* host, size_t n);
    int init();
    // one loop iteration; returns 0, 1 (final time reached, nothing done),
    // kErrSaturated (loop stopped after this iteration) or an error
    int step_once();
    int finish();       // final save + log line
    bool done() const;

    // ensemble step pieces (csrc/ensemble.cpp): the work of step_once for a mixed-form Euler
    // member whose advection, incompressibility check, psi solve and coarse sample run in
    // batched launches over the whole ensemble.  ens_begin: time step, Lagrange
    // coefficients, the advection descriptor and any precombination (returns 1 when the
    // member is done); ens_middle: the map swap, a remap when the checked E_inc asks for
    // one, the psi rotation and the psi-solve descriptor; ens_end: particles, saves and
    // counters.  ens_bind gives the member its slots in the ensemble's class buffers.
    int ens_check(std::string* why) const;
    void ens_bind(float* sample_out, const float2* spec_v, float2* spec4, const float* planes, unsigned long long* einc);
    int ens_begin(EnsMember& e);
    // remap != nullptr (a member of the fused-path work arrays, ens_fused_bind): a remap is
    // described in *remap for the ensemble's batched remap launch instead of run here
    int ens_middle(double e_inc, EnsMember& e, EnsMember* remap = nullptr);
    int ens_end();
    // the single-launch iteration (launch_ens_fused): the remap decision, the remap and the
    // psi solve run on the device after ens_begin.  ens_fused_check: what that path needs
    // beyond ens_check; ens_fused_bind: the member's size class and work arrays;
    // ens_fused_prepare (after ens_begin): stack room, the psi rotation and the rest of the
    // descriptor; ens_fused_finish (after the launch): the map swap and the bookkeeping of
    // the remap the device decided (remapped), then ens_end as usual.
    int ens_fused_check(std::string* why) const;
    void ens_fused_bind(int cls, float* real, float2* w1, float2* w2);
    int ens_fused_prepare(EnsMember& e);
    int ens_fused_finish(double e_inc, bool remapped);
    void remap_fields(EnsMember& e, bool can);

    // learned psi (precision=mixed, Euler; csrc/sim_learned.cpp).  With an upsampler attached,
    // every `every`-th step runs the exact vorticity-grid evaluation and judges the learned
    // psi (cheap vorticity plus the network's sub-grid vorticity on the psi grid, predicted
    // from omega and its gradient on the map grid) and the cheap psi (omega sampled on the
    // map grid) against it; the next every - 1 steps use the network if its relative
    // L-infinity difference is within `tol` and below the cheap one's, else the cheap psi if
    // that is within `tol`, else the exact evaluation.  null detaches.  learned_collect appends the current
    // state's training pair (map-grid fields, the sub-grid vorticity on the psi grid); learned_evaluate gives the
    // relative L-infinity and L2 differences of the cheap psi, the learned psi and the psi of
    // omega sampled exactly on the psi grid from the current exact psi level
    // (out = {cheap Linf, cheap L2, learned Linf, learned L2, psi-grid Linf, psi-grid L2}).
    int attach_upsampler(lrn::Upsampler* u, int every, double tol);
    int learned_collect(lrn::Upsampler& u);
    int learned_evaluate(lrn::Upsampler& u, double* out6);

    int get_field(const std::string& name, void* dst, size_t bytes);
    size_t field_bytes(const std::string& name) const;
    int get_scalar(const std::string& name, double* out);

    Settings s;
    std::string err;

    // grids
    Grid gc, gf, gp, gv, gd;
    double dt = 0;
    int L = 1;
    int max_maps = 0;

    // monitoring state
    double time() const { return t_vec_.empty() ? 0.0 : t_vec_[loop_ctr_ + L - 1]; }
    int loop_ctr() const { return loop_ctr_; }
    int map_count() const { return n_maps_; }
    double last_e_inc() const { return e_inc_; }

    // device state (reference planar layouts)
    double* ChiX = nullptr; double* ChiY = nullptr;
    double* ChiX_new = nullptr; double* ChiY_new = nullptr;
    double* psi[kMaxLagrange] = {nullptr, nullptr, nullptr, nullptr};
    double* vort = nullptr;        // coarse vorticity
    double* wfine = nullptr;       // fine vorticity Hermite (4 planes)
    double* wdisc = nullptr;       // discrete initial vorticity Hermite (4 planes)
    double* stack = nullptr;       // n maps, 8*Nc doubles each
    std::vector<double*> parts;    // particle positions per set
    std::vector<double*> vels;     // inertial velocity state per set (tau != 0; null for tracers)
    // forward map (forward_map = 1): active map, its stack (n maps like stack), forwarded
    // particles' initial positions and the stack index each forwarded set starts from
    double* ChiX_f = nullptr; double* ChiY_f = nullptr;
    double* stack_f = nullptr;
    std::vector<double*> fparts_;
    std::vector<int> init_map_;
    double e_inc_f_ = 0, e_inv_ = 0;
    int n_maps_f_ = 0;             // forward sub-maps (one per remap; a restart may load fewer)
    double* fpos_ = nullptr;       // forwarded particle positions of a save (all sets)
    cudaStream_t stream = nullptr;

    // diagnostics (reference Mesure)
    int diagnostics(double* energy, double* enstrophy, double* palinstrophy, double* wmax);

    // per-phase CUDA-event timers (off by default) and launch counters
    enum Phase { kPhAdvect = 0, kPhIncomp, kPhRemap, kPhPsi, kPhCoarse, kPhParticles, kPhSave, kNumPhases };
    static const char* phase_name(int p);
    void set_profiling(bool on);
    double prof_ms[kNumPhases] = {0};
    long long prof_count[kNumPhases] = {0};
    long long kernel_launches = 0;    // launches of this library's kernels
    long long fft_calls = 0;          // 2D / 1D transform calls (csrc/fft.hpp)

private:
    int alloc();
    void release();
    int translate_ic();
    int evaluate_stream();
    int vort_spectrum();
    void predict_combinations();
    int psi_planes(float2* spec4, float* out);
    int coarse_vort();
    int ensure_vort();           // sample the coarse vorticity if a step left it stale
    void scalar_source(InitSource& src) const;
    bool vort_stale_ = false;
    int advect(const double* t, const double* dtv, int loop_ctr, int ti_num, int l_order);
    int advect_m(const double* t, const double* dtv, int loop_ctr, int ti_num, int l_order);
    int reset_map();
    void swap_levels(int a, int b);
    int incomp(double* out);
    int init_particles();
    int init_positions(double* dst, int num, unsigned long long seed, int init_num, const double* param,
                       const std::string& init_name);
    // forward map (forward_map = 1, plain FP64 form): advection, checks and forced remaps of one
    // step, and the forwarded particles' positions on a frame (apply_map_stack_points, direction 1)
    int forward_step(int lcl, bool* forced_remap);
    int forwarded_positions(const double* frame, double* out);
    int init_inertial_velocity(size_t i);   // v = u(x) of psi level 0, or 0 (init_vel)
    int advect_particles(int lcl);
    int push_stack();
    int reserve_stack(int n);          // device stack capacity for n sub-maps
    // MapStack folder (writeMapStack / writeParticlesState / readMapStack, cmm-io.cu:611-688,
    // cmm-simulation-host.cu:1256-1302): map_num >= 0 a stacked sub-map, -1 the active map
    int write_map_stack(int map_num, bool forward = false);
    int write_particles_state();
    int restart_from_map_stack();      // the restart branch of init (cmm-euler2d.cu:634-685)
    int sample_outputs(double t_now, double dt_now);   // sampled outputs on user grids
    int vlasov_sample_outputs(double t_now, double dt_now);   // their Vlasov-Poisson form
    int zoom_outputs(double t_now, double dt_now);     // zoom windows (compute_zoom)
    int reserve_sample_buffers(int n);                 // smp_ / smp_c_ for an n x n grid
    // forwarded particles mapped on a frame, raw files under sub for the sets var names
    int write_forwarded(const double* frame, const std::string& sub, bool zoom, const std::string& var);
    int evaluate_potential();          // Vlasov-Poisson psi from the distribution function
    int vlasov_setup_h();              // the periodification h(v), once per run
    int vlasov_mesure(double* out9);   // Etot, Ekin, Epot, Mass, Momentum, Emode1..4
    int save_functions(double t_now, double dt_now);
    int write_time_step(double t_now, double dt_now);
    int conservation(double t_now, double dt_now);
    int debug_globals(const std::string& name, const double* v, long long n, bool grid_form, const Grid& g);
    int write_field(const std::string& sub, const std::string& name, const double* v, long long n);
    int write_monitors();
    int check(cudaError_t e, const char* what);
    double compute_next_timestep(double t) const;
    void rotate_psi(int n);
    void unrotate_psi(int n);
    cudaEvent_t einc_ev_ = nullptr;    // E_inc's readback (speculative psi evaluation)
    // the readback runs on a side stream forked after the check (fork_ev_) and joined at the
    // end of the step's front (join_ev_), so the psi solve's kernels follow the check directly
    cudaStream_t side_ = nullptr;
    cudaEvent_t fork_ev_ = nullptr, join_ev_ = nullptr;
    double* d_einc2_ = nullptr;   // the check's two result slots (zero when taken), used alternately
    int einc_slot_ = 0;
    cudaGraphExec_t step_graph_ = nullptr;   // the captured front of a mixed Euler step
    bool use_graphs_ = true;
    long long graph_launches_ = 0;
    double wall() const;

    void ph_begin(int p);
    void ph_end(int p);
    void ph_collect();
    int sync_fp64_views();   // mixed form: refresh the FP64 reference-layout copies

    // mixed form (precision=mixed): FP32 displacement maps and FP32 Hermite nodes
    bool mixed_ = false;
    // learned psi state
    int learned_check() const;
    int load_upsampler();     // psi_upsampler=<file>: an owned network read from the file
    int learned_setup();
    void learned_release();
    int cheap_fields();
    int learned_planes(lrn::Upsampler& u, float* out);
    int learned_stream();
    int cheap_planes(float* out);
    int diff_stats(const float* a, long long sa, const float* e, long long se, long long n, double* host4);
    lrn::Upsampler* ups_ = nullptr;
    lrn::Upsampler* ups_owned_ = nullptr;
    int learned_every_ = 8;
    double learned_tol_ = 1e-4;
    int learned_level_ = 2;            // 0 network, 1 cheap psi, 2 exact until the next judged step
    long long learned_steps_ = 0, cheap_steps_ = 0, exact_steps_ = 0, learned_checks_ = 0, learned_fails_ = 0,
              learned_cheaper_ = 0;
    double learned_last_err_ = 0, learned_max_err_ = 0;
    float *lc_omega_ = nullptr, *lc_planes_ = nullptr, *l_delta_ = nullptr, *l_planes_ = nullptr;
    float2 *lc_spec_ = nullptr, *lc_spec4_ = nullptr, *l_dspec_ = nullptr;
    fft::Plan2D fc_;           // FP32 transforms of the map grid (learned psi)
    double* d_stats_ = nullptr;
    bool in_step_ = false;

    // ensemble members keep their per-step Monitoring_data records (Time_s,
    // Error_incompressibility, Map_gaps, Map_counter) here and append them in blocks
    enum { kMonTimeS, kMonEinc, kMonEincF, kMonEinv, kMonGap, kMonCounter, kMonTimeC, kMonSeries };
    std::vector<double> mon_buf_[kMonSeries];
public:
    void flush_monitor();
private:
    // ensemble binding
    float* ens_sample_ = nullptr;
    const float2* ens_spec_v_ = nullptr;
    float2* ens_spec4_ = nullptr;
    const float* ens_planes_ = nullptr;
    unsigned long long* ens_einc_ = nullptr;
    int ens_cls_ = 0;
    float* ens_real_ = nullptr;
    float2* ens_w1_ = nullptr;
    float2* ens_w2_ = nullptr;
    int ens_lcl_ = 0;
    double ens_dt_ = 0, ens_gap_ = 0, ens_counter_ = 0;
    bool ens_saturated_ = false;
    // tracer storage order: sets of at least kReorderMin tracers are sorted by 4 x 4 psi-cell
    // bucket every kReorderEvery steps; tperm_[i][j] = original index of stored tracer j
    static constexpr int kReorderMin = 4096, kReorderEvery = 32;
    std::vector<int*> tperm_;
    TracerScratch tscratch_;
    float4* mapm_ = nullptr;         // 2*Nc float4 (current map)
    float4* mapm_new_ = nullptr;
    float4* psim_[kMaxLagrange] = {nullptr, nullptr, nullptr, nullptr};
    float4* psiA_ = nullptr;         // Lagrange combinations of the psi levels
    float4* psiB_ = nullptr;
    float4* psiP_ = nullptr;         // tracers' t_{n+1/2} combination
    // combinations written by the psi solve's last pass (three levels): valid for the
    // coefficients below; the next advection and this step's tracers check them bitwise
    int psi_lcl_ = -1;
    bool fused_ = false;
    double fusedL1_[kMaxLagrange] = {0, 0, 0, 0}, fusedL12_[kMaxLagrange] = {0, 0, 0, 0},
           fusedLp_[kMaxLagrange] = {0, 0, 0, 0};
    float4* wfm_ = nullptr;          // fine vorticity nodes
    float4* wdiscm_ = nullptr;       // discrete initial vorticity nodes (FP32 Hermite)
    float4* stackm_ = nullptr;       // n maps, 2*Nc float4 each
    // Vlasov mixed form: the maps are stored in the free-streaming frame (SepDrift), which needs
    // each map's age: the active map's, and every stacked map's (host and device copies)
    double map_tau_ = 0.0;
    double2* drift_rows_ = nullptr;  // SepDrift's per-row table (built once from h)
    std::vector<double> stack_tau_;
    double* d_stack_tau_ = nullptr;
    int stack_tau_cap_ = 0;
    const SepDrift* sep_drift(SepDrift& d, double tau) const;   // null unless the Vlasov mixed form
    int upload_stack_taus();
    std::vector<unsigned long long*> partfix_;   // tracer positions, 64-bit fixed point (x, y interleaved)
    std::vector<float2*> velm_;                  // inertial velocity state (FP32), null for tracer sets

    // sampled outputs: buffers and plans of the largest sample grid seen so far
    int smp_n_ = 0, smp_plan_n_ = 0;
    FftPlans ps_;
    double* smp_[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};   // X, Y, scalar, W, psi, work
    double2* smp_c_[2] = {nullptr, nullptr};

    // Vlasov-Poisson (simulation_type cmm_vlasov_poisson_1d)
    bool vlasov_ = false;
    VlasovPlans vp_;
    VlasovPlans vps_;          // 1D plans of the Vlasov sample grid's length
    int vsmp_plan_n_ = 0;
    double* phi_lv_[kMaxLagrange] = {nullptr, nullptr, nullptr, nullptr};   // per psi level: phi (NX), phi' (NX)
    double* vl_h_ = nullptr;         // h(v) (NY), h'(v) (NY) on the psi grid
    double* vl_rho_ = nullptr;       // rho - 1 on the vort grid's x-nodes
    double* vl_part_ = nullptr;      // v-integral partial sums
    double2* vl_c_[3] = {nullptr, nullptr, nullptr};   // 1D spectra
    double2* vtab_[4] = {nullptr, nullptr, nullptr, nullptr};  // mixed form: tables A, B, 0 (x) and h (v)
    float* realf_ = nullptr;         // FP32 real scratch (4 planes of the largest grid)
    float2* specf_ = nullptr;        // FP32 complex scratch
    float2* spec4f_ = nullptr;       // 4 FP32 spectra
    fft::Plan2D fv_, fp_, ff_;   // FP32 transforms of the vort, psi and fine grids (mixed form)
    int vcols_ = 0;              // columns kx <= freq_cut_psi the psi solve keeps
    bool psi_fused_ = false;     // the psi solve runs on the kept-column kernels of psi_solve.cuh
    void* psw1_ = nullptr;       // their work arrays (kept columns of omega's and psi's spectra)
    void* psw2_ = nullptr;
    bool prof_ = false;
    cudaEvent_t ev_[kNumPhases][2] = {};
    bool ev_live_[kNumPhases] = {};
    bool own_stream_ = false;
    bool initialised_ = false, finished_ = false, continue_ = true;
    double* real_buf_ = nullptr;     // real scratch (largest grid)
    double2* spec_ = nullptr;        // complex scratch (largest grid)
    double2* spec4_ = nullptr;       // 4 complex spectra (largest grid)
    double* red_ = nullptr;          // reduction partials
    double* d_scal_ = nullptr;       // 8 device scalars
    double* h_scal_ = nullptr;       // pinned mirror
    double* d_params_ = nullptr;     // 10 initial params
    double* d_rand_ = nullptr;       // 1000 random numbers (gaussian_blobs)
    int stack_cap_ = 0;
    FftPlans pf_, pv_, pp_, pc_, pd_;
    std::vector<double> host_discrete_;
    std::vector<double> t_vec_, dt_vec_;
    int loop_ctr_ = 0, old_ctr_ = 0, n_maps_ = 0;
    double e_inc_ = 0;
    Logger log_;
    std::chrono::steady_clock::time_point begin_;
};

}  // namespace cmm
