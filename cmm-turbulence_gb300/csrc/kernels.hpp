// kernels.hpp -- host launchers of the sm_103a CMM kernels (FP64 plain form).
// Every launcher is stream-ordered and returns the launch status.
#pragma once
#include <cuda_runtime.h>

#include "cmm_common.cuh"
#include "fft.hpp"

namespace cmm {

constexpr int kMaxLagrange = 4;
constexpr int kMaxFoot = 12;

// Map advection (advect_using_stream_hermite + k_advect_using_stream_hermite,
// Cuda-CMM/src/simulation/cmm-simulation-host.cu:64-104,
// src/simulation/cmm-simulation-kernel.cu:207-298), backward direction.
struct AdvectArgs {
    Grid gm, gp;
    const double* ChiX;
    const double* ChiY;
    double* outX;
    double* outY;
    const double* psi[kMaxLagrange];     // psi[l]: Hermite level l (l=0 newest)
    double L1[kMaxLagrange], L12[kMaxLagrange];
    double coef[4][kMaxFoot];            // c1, cx, cy, cxy footpoint weights
    double dt, ep;
    int time_integration_num;            // 10 EulerExp, 21 RK2 (Heun), 20 AB2, 30 RK3, 40 RK4, 31 RK3Mod, 41 RK4Mod
    int l_order;                         // Lagrange levels used (1..4)
    int nfoot;                           // 4, 8 or 12 footpoints
    int direction;                       // -1 backward map (default), 1 forward map
};

void map_update_coefficients(int order_num, double ep, double coef[4][kMaxFoot], int* nfoot);

cudaError_t launch_init_map(double* X, double* Y, const Grid& g, cudaStream_t s);
cudaError_t launch_advect(const AdvectArgs& a, cudaStream_t s);
// max |x - X_b(X_f(x))| over the half-shifted nodes of gc -> *d_result (forward map check)
cudaError_t launch_invert(const Grid& gc, const Grid& gm, const double* Xb, const double* Yb, const double* Xf,
                          const double* Yf, double* d_result, cudaStream_t s);
// max |1 - det grad X| over the half-shifted check grid -> *d_result (double);
// d_result is reset by the launcher
cudaError_t launch_incomp(const Grid& gcheck, const Grid& gmap, const double* X, const double* Y,
                          double* d_result, cudaStream_t s);

// Initial-condition selector for sampling omega_0 (k_h_sample_from_init,
// src/simulation/cmm-simulation-kernel.cu:342-373).
// random tables of the analytic initial conditions: kRandTable uniform(-1, 1) values of
// mt19937_64 seed 0 (gaussian_blobs, cmm-euler2d.cu:347-352) followed by the
// 2 * kGaussBlobs^2 cuRAND offsets of turbulence_gaussienne (init_tables.cu)
constexpr int kRandTable = 1000;
constexpr int kGaussBlobs = 7;
constexpr int kInitTable = kRandTable + 2 * kGaussBlobs * kGaussBlobs;
cudaError_t launch_gaussienne_offsets(double* out, cudaStream_t s);

struct InitSource {
    int kind;                 // 0 analytic vorticity, 1 analytic passive scalar, 2 Vlasov distribution, 3 discrete Hermite
    int ic_num;               // analytic initial-condition number
    const double* discrete;   // Hermite planes of the discrete initial field
    Grid gd;                  // its grid
    const double* params;     // 10 initial_params (device)
    const double* rand_table; // kInitTable values (device): gaussian_blobs, turbulence_gaussienne
};

// omega_0( X_0( ... X_{n-1}( X_cur(x) ) ) ) on the target grid, fused over a
// device-resident stack (translate_initial_condition_through_map_stack,
// src/simulation/cmm-simulation-host.cu:112-128,299-327).
// stack holds n maps, map i = [X planes (4N) | Y planes (4N)] at stack + i*8N.
cudaError_t launch_compose_sample(const Grid& gm, const Grid& gt, const double* X, const double* Y,
                                  const double* stack, int n_maps, const InitSource& src, double* out,
                                  cudaStream_t s);

// omega(x) = W_fine_H( X(x) ) on the output grid (k_apply_map_and_sample_from_hermite,
// src/simulation/cmm-simulation-kernel.cu:402-461); out has row stride `ld`.
cudaError_t launch_sample_vort(const Grid& gm, const Grid& gout, const Grid& gf, const double* X,
                               const double* Y, const double* Wf, int molly, double* out, long long ld,
                               cudaStream_t s);

// the psi solve (evaluate_stream_hermite, cmm-simulation-host.cu:333-375) on the library's
// FFT: omega through the map on gv (into the scratch omega, gv.N doubles), its kept modes,
// the four psi Hermite planes on gp, in four launches (psi_solve.cuh); runs when
// psi_solve_fits, which also gives the complex values the work arrays w1, w2 need
bool psi_solve_fits(const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv, const fft::Plan2D& pp,
                    long long* w1_values, long long* w2_values);
void psi_solve_prepare();
cudaError_t launch_psi_solve(const Grid& gm, const Grid& gv, const Grid& gf, const double* X, const double* Y,
                             const double* Wf, int molly, const Grid& gp, double freq, const fft::Plan2D& pv,
                             const fft::Plan2D& pp, double* omega, double2* w1, double2* w2, double* psi_out,
                             cudaStream_t s);

// tracer and inertial particles (Particle_advect / Particle_advect_inertia,
// src/numerical/cmm-particles.cu:119-551); psi[0] is t_{n+1}, psi[1] t_n, psi[2] t_{n-1}
struct ParticleArgs {
    Grid gp;
    double* pos;
    double* vel;                // inertial velocity state (tau != 0), else unused
    int num;
    const double* psi[kMaxLagrange];
    double Lp12[kMaxLagrange];
    double dt;
    double tau;                 // 0: fluid tracers
    int time_integration_num;   // 10, 20, 30, 40, 31, 41
    int l_order;
};
cudaError_t launch_particles(const ParticleArgs& a, cudaStream_t s);
// v = u(x) of psi level psi0 (Particle_advect_inertia_init, cmm-particles.cu:50-60)
cudaError_t launch_particle_vel_init(const double* pos, int num, const double* psi0, const Grid& gp, double* vel,
                                     cudaStream_t s);
// U(0,1) -> frame and wrap (k_rescale, cmm-particles.cu:30-46)
cudaError_t launch_particle_rescale(double* pos, int num, const double* p4, const Grid& g, cudaStream_t s);
// circle / uniform grid / sine-sheet layouts (mode 2, 3, 4)
cudaError_t launch_particle_layout(double* pos, int num, int mode, const double* p4, const Grid& g, cudaStream_t s);
// psi_x, psi_y at particle positions (k_h_sample_points_dxdy, cmm-simulation-kernel.cu:138-155)
cudaError_t launch_sample_points_dxdy(const Grid& gp, const double* psi, const double* pos, double* out, int num,
                                      cudaStream_t s);

// ---------------------------------------------------------------- spectral
// FP64 2D transforms of one grid (the reference's D2Z / Z2D plans, cmm-grid2d.cu:123-131)
// on the library's own FFT (csrc/fft.hpp) plus fused spectral operators (src/numerical/cmm-fft.cu)
struct FftPlans {
    fft::Plan2D p;
    Grid g;
    bool ok = false;
};
bool make_plans(FftPlans& p, const Grid& g, cudaStream_t s);
void destroy_plans(FftPlans& p);
// real -> half spectrum (unnormalised); batch half spectra -> real planes (unnormalised;
// the input is overwritten)
cudaError_t fft_d2z(const FftPlans& p, const double* in, double2* out, cudaStream_t s);
cudaError_t fft_z2d(const FftPlans& p, double2* in, double* out, int batch, cudaStream_t s);

// normalised spectrum -> 4 spectra [F, dx F, dy F, dxdy F] (fourier_hermite prep)
cudaError_t launch_spec_hermite(const double2* F, const Grid& g, double2* out4, cudaStream_t s);
// vort spectrum (raw D2Z) -> psi-grid 4 spectra: normalise, grid move, circular cut,
// inverse Laplacian, derivatives (evaluate_stream_hermite, cmm-simulation-host.cu:333-375)
cudaError_t launch_spec_psi(const double2* Fv, const Grid& gv, const Grid& gp, double freq, double2* out4,
                            cudaStream_t s);
// raw D2Z spectrum -> normalised (dx F, dy F) for the palinstrophy (cmm-mesure.cu:77-89)
cudaError_t launch_spec_grad(const double2* F, const Grid& g, double2* out2, cudaStream_t s);

// ---------------------------------------------------------------- sampled outputs
// positions of the nodes of gt through the current map and n_maps stacked maps (wrapped)
cudaError_t launch_compose_pos(const Grid& gm, const Grid& gt, const double* X, const double* Y, const double* stack,
                               int n_maps, double* px, double* py, cudaStream_t s);
// nodes of gt through the forward stack (oldest first) and then the active forward map
cudaError_t launch_compose_fwd(const Grid& gm, const Grid& gt, const double* X, const double* Y, const double* stack,
                               int n_maps, double* px, double* py, cudaStream_t s);
// num points (x, y interleaved) through one map; NaN for points not strictly inside the
// frame (x_min, x_max, y_min, y_max)
cudaError_t launch_map_points(const Grid& gm, const double* frame, const double* X, const double* Y, const double* in,
                              double* out, int num, cudaStream_t s);
// an initial field at n positions (src.kind 0 vorticity, 1 scalar, 2 distribution, 3 discrete)
// the Hermite field src.discrete (on src.gd) at the nodes of g
cudaError_t launch_eval_grid(const Grid& g, const InitSource& src, double* out, cudaStream_t s);
cudaError_t launch_eval_init(const double* px, const double* py, long long n, const InitSource& src, double* out,
                             cudaStream_t s);
// normalised spectral operator on a D2Z half spectrum: 0 Laplacian, 1 d/dx, 2 d/dy, 3 inverse Laplacian
cudaError_t launch_spec_op(const double2* in, const Grid& g, int op, double2* out, cudaStream_t s);

// ---------------------------------------------------------------- reductions
// min, max, max(0,max), sum over n values at stride `stride` (Debug_globals);
// result -> d_out[4]; partial scratch of kReduceBlocks*4 doubles
constexpr int kReduceBlocks = 304;
cudaError_t launch_stats(const double* v, long long n, long long stride, double* d_scratch, double* d_out,
                         cudaStream_t s);
// sum of squares of n values (energy, enstrophy) -> d_out[0]
cudaError_t launch_sumsq(const double* v, long long n, double* d_scratch, double* d_out, cudaStream_t s);

}  // namespace cmm
