/*
 * cmm_oracle.h -- CPU restatement (plain C99 + OpenMP, FP64) of the
 * characteristic-mapping-method time step of Arcadia197/cmm-turbulence.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * CUDA product in cmm-turbulence_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference legs may load it.  The
 * product never links, loads or falls back to it.
 *
 * Every routine restates the reference's arithmetic in the reference's
 * memory layout (planar Hermite planes [f, f_x, f_y, f_xy], row-major
 * iY*NX+iX) and cites the reference file:line it follows.  Paths are
 * relative to the reference project's Cuda-CMM/ directory.
 *
 * Parity pin: the reference's own golden Debug_globals / Mesure /
 * Monitoring_data files (tests/euler2D_init_fields, tests/euler2D_one_step,
 * tests/euler2D_11b_4nodes_reference_remapping) are reproduced by this
 * oracle; see tests/test_oracle_golden.py.  The reference's FFT is cuFFT
 * (closed); this oracle uses its own mixed-radix FFT (og_fft.c), so FFT
 * rounding differs at the 1e-16 level.
 */
#ifndef CMM_ORACLE_H
#define CMM_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Grid metadata: src/grid/cmm-grid2d.h:25-39, ctor src/grid/cmm-grid2d.cu:20-52. */
typedef struct {
    int NX, NY, NX_fft;
    long N, Nfft;
    double hx, hy;
    double bounds[4];
} og_grid;

void og_grid_fill(og_grid* g, int NX, int NY, const double* bounds);

/* ---------------- Hermite helpers (src/numerical/cmm-hermite.cu) ---------------- */
double og_hermite_interpolate_2D(const double* H, double x, double y, const og_grid* g);
double og_hermite_interpolate_dx_2D(const double* H, double x, double y, const og_grid* g);
double og_hermite_interpolate_dy_2D(const double* H, double x, double y, const og_grid* g);
void og_hermite_interpolate_grad_2D(const double* H, const double* x, double* u, const og_grid* g, int n_l);
void og_diffeo_interpolate_2D(const double* Hx, const double* Hy, double x, double y,
                              double* x2, double* y2, const og_grid* g);
double og_diffeo_grad_2D(const double* Hx, const double* Hy, double x, double y, const og_grid* g);

/* ---------------- time stepping (src/numerical/cmm-timestep.cu) ---------------- */
double og_get_L_coefficient(const double* t, double t_next, int loop_ctr, int i_point, int l_order);

/* ---------------- kernels restated as loops ---------------- */
/* k_init_diffeo: src/simulation/cmm-simulation-kernel.cu:27-41 */
void og_init_diffeo(double* ChiX, double* ChiY, const og_grid* g);
/* advect_using_stream_hermite + k_advect_using_stream_hermite (direction -1):
 * src/simulation/cmm-simulation-host.cu:64-104, src/simulation/cmm-simulation-kernel.cu:207-298.
 * L1/L12 are the Lagrange coefficients, c1/cx/cy/cxy the footpoint weights. */
void og_advect_map(const double* ChiX, const double* ChiY, double* ChiX_new, double* ChiY_new,
                   const double* psi, const og_grid* gmap, const og_grid* gpsi,
                   double dt, double ep, int time_integration_num, int map_update_order_num,
                   int l_order, const double* L1, const double* L12,
                   const double* c1, const double* cx, const double* cy, const double* cxy);
/* footpoint weights: src/simulation/cmm-simulation-host.cu:76-90 */
void og_map_update_coefficients(int map_update_order_num, double ep,
                                double* c1, double* cx, double* cy, double* cxy);
/* incompressibility_check: src/simulation/cmm-simulation-host.cu:44-50 +
 * k_incompressibility_check src/simulation/cmm-simulation-kernel.cu:159-173 */
double og_incompressibility_check(const og_grid* gcheck, const og_grid* gmap,
                                  const double* ChiX, const double* ChiY);
/* k_h_sample_map_compact / k_apply_map_compact: src/simulation/cmm-simulation-kernel.cu:302-340 */
void og_sample_map_compact(const double* ChiX, const double* ChiY, double* x_y,
                           const og_grid* gmap, const og_grid* g);
void og_apply_map_compact(const double* ChiX, const double* ChiY, double* x_y,
                          const og_grid* gmap, const og_grid* g);
/* stack composition + initial-condition sampling on gt (stack: n maps of [X|Y] planes) */
void og_compose_sample(const double* ChiX, const double* ChiY, const double* stack, int n, const og_grid* gm,
                       const og_grid* gt, int ic_num, const double* discrete, const og_grid* gd, double* out);
/* d_init_vorticity "4_nodes": src/simulation/cmm-init.cu:45-52 */
double og_init_vorticity(double x, double y, int ic_num);
/* initial_params (10) and the random tables (1000 uniform(-1,1) then 98 turbulence_gaussienne
 * offsets) that the analytic initial conditions read; NULL leaves one unchanged */
void og_set_init_data(const double* params10, const double* table1098);
/* k_apply_map_and_sample_from_hermite: src/simulation/cmm-simulation-kernel.cu:402-461 */
void og_apply_map_and_sample_from_hermite(const double* ChiX, const double* ChiY, double* fs,
                                          const double* H, const og_grid* gmap, const og_grid* gvort,
                                          const og_grid* gfine, int molly_stencil, int padd_inline_fft);

/* ---------------- spectral (src/numerical/cmm-fft.cu) ---------------- */
/* complex arrays are interleaved (re, im) doubles, length 2*Nfft */
void og_fft_d2z(const og_grid* g, const double* in, double* out_c);
void og_fft_z2d(const og_grid* g, const double* in_c, double* out);
void og_normalize_h(double* F, const og_grid* g);
void og_fft_grid_move(const double* in_c, double* out_c, const og_grid* gout, const og_grid* gin);
void og_fft_cut_off_scale_h(double* W, const og_grid* g, double freq);
void og_fft_iLap_h(const double* in_c, double* out_c, const og_grid* g);
void og_fft_dx_h(const double* in_c, double* out_c, const og_grid* g);
void og_fft_dy_h(const double* in_c, double* out_c, const og_grid* g);
/* fourier_hermite: src/numerical/cmm-fft.cu:398-429; out has 4*N doubles */
void og_fourier_hermite(const og_grid* g, const double* in_c, double* out4);

/* ---------------- the Euler-2D driver (src/simulation/cmm-euler2d.cu) ---------------- */
typedef struct {
    int num;                      /* particles in the set */
    double tau;                   /* 0: fluid tracers; otherwise inertial particles */
    int time_integration_num;     /* 10, 20, 30, 40, 31, 41 */
    double init_time;
    int init_vel;                 /* inertial: start at the fluid velocity (1) or at rest (0) */
} og_particle_set;

typedef struct {
    int num;                      /* forwarded particles in the set */
    double init_time;             /* the set is mapped forward from this time on */
} og_fwd_set;

typedef struct {
    int grid_coarse, grid_fine, grid_psi, grid_vort;
    double bounds[4];
    double dt;
    int time_integration_num;     /* map advection scheme (30 = RK3) */
    int lagrange_order;           /* after particle / override adjustment */
    int lagrange_init_higher_order;
    int map_update_order_num;     /* 0 = 2nd, 1 = 4th, 2 = 6th */
    double map_epsilon;
    double incomp_threshold;
    int skip_remapping;
    int molly_stencil;
    double freq_cut_psi;
    int initial_condition_num;    /* 0 = 4_nodes */
    int initial_discrete;
    int initial_discrete_grid;
    int max_maps;                 /* stack capacity (cpu_map_num) */
    int n_particle_sets;
    og_particle_set psets[8];
    int simulation_type_num;      /* 0 = cmm_euler_2d, 2 = cmm_vlasov_poisson_1d */
    int forward_map;              /* advect a forward map beside the backward one */
    int n_fwd_sets;               /* forwarded particle sets */
    og_fwd_set fsets[8];
} og_settings;

typedef struct og_state og_state;

og_state* og_create(const og_settings* s);
void og_destroy(og_state* st);
/* discrete IC values (NxN row-major) -- Hermite form is built internally
 * (src/simulation/cmm-euler2d.cu:325-344) */
int og_set_discrete_initial(og_state* st, const double* values);
/* particle initial positions (interleaved x,y) for set i */
int og_set_particles(og_state* st, int i_set, const double* pos);
/* Particle_advect_inertia (src/numerical/cmm-particles.cu:280-551) and its initialisation (:50-60) */
void og_particle_advect_inertia(int num, double dt, double* pos, double* vel, const double* psi, const og_grid* g,
                                double tau, int ti, int l_order, const double* Lp12);
void og_particle_inertia_init(int num, const double* pos, double* vel, const double* psi, const og_grid* g);
/* initial state + Lagrange history (src/simulation/cmm-euler2d.cu:495-619,
 * src/simulation/cmm-vlasov1d.cu:516-656); -1 if the Vlasov potential rejects the grids */
int og_init(og_state* st);
/* one loop iteration (src/simulation/cmm-euler2d.cu:750-897, cmm-vlasov1d.cu:782-960);
 * dt_now from the caller (compute_next_timestep). Returns 0 ok, 1 stack saturated
 * (loop stops), 2 Vlasov incompressibility blow-up (cmm-vlasov1d.cu:838-840). */
int og_step(og_state* st, double dt_now, double* e_inc, int* remapped);
/* in place of og_init: restart from a stored map stack (n sub-maps, each 4*Nc X planes in
 * stackX and 4*Nc Y planes in stackY), the stored active map and psi levels 1..L-1
 * (src/simulation/cmm-simulation-host.cu:1256-1302, src/simulation/cmm-euler2d.cu:634-715) */
int og_restart(og_state* st, double restart_time, int n_maps, const double* stackX, const double* stackY,
               const double* chix, const double* chiy, const double* psi_prev);
const double* og_stack_x(const og_state* st);     /* n_maps x 4*Nc */
/* forward map (forward_map = 1): the active forward map, the last step's forward
 * incompressibility and invertibility errors, the forwarded particles' initial positions,
 * and the forward composition on an n x n frame (bounds4; the map through the forward
 * stack oldest first, then the active map) with the forwarded particles mapped from their
 * start map on (NaN outside the frame): apply_map_stack / apply_map_stack_points with
 * direction 1, src/simulation/cmm-simulation-host.cu:130-152, 160-292 */
const double* og_chix_f(const og_state* st);
const double* og_chiy_f(const og_state* st);
void og_forward_monitors(const og_state* st, double* einc_f, double* einv);
int og_set_forwarded_particles(og_state* st, int i_set, const double* pos);
void og_forward_sample(const og_state* st, int n, const double* bounds4, double* map_xy, double* parts);
/* k_invertibility_check (src/simulation/cmm-simulation-kernel.cu:177-198): max over the
 * half-shifted check grid of |x - X_b(X_f(x))| */
double og_invertibility_check(const og_grid* gcheck, const og_grid* gb, const double* Xb, const double* Yb,
                              const og_grid* gf, const double* Xf, const double* Yf);
const double* og_stack_y(const og_state* st);

/* state access (reference layouts) */
double og_time(const og_state* st);
int og_map_count(const og_state* st);
int og_loop_ctr(const og_state* st);
int og_old_ctr(const og_state* st);
const double* og_chix(const og_state* st);        /* 4*Nc */
const double* og_chiy(const og_state* st);
const double* og_psi(const og_state* st);         /* L*4*Npsi, level 0 first */
const double* og_vort_coarse(const og_state* st); /* Nc */
const double* og_vort_fine(const og_state* st);   /* 4*Nf */
const double* og_particles(const og_state* st, int i_set);
double* og_particle_vel(og_state* st, int i_set);  /* inertial velocity state (2*num) */
const og_grid* og_grid_of(const og_state* st, int which); /* 0 coarse,1 fine,2 psi,3 vort */

/* diagnostics: src/numerical/cmm-mesure.cu:30-89, cmm-simulation-host.cu:668-680 */
double og_energy_H(const og_state* st);
double og_enstrophy(const og_state* st);
double og_palinstrophy(const og_state* st);
double og_max_vorticity(const og_state* st);
/* debug globals (src/numerical/cmm-mesure.cu:217-249): grid form uses hx*hy, raw form /N */
void og_stats_grid(const double* v, const og_grid* g, double* out4);
void og_stats_raw(const double* v, long n, double* out4);
/* ---------------- Vlasov-Poisson (og_vlasov.c) ---------------- */
/* d_init_distirbution_function: src/simulation/cmm-init.cu:457-493 */
double og_init_distribution(double x, double v, int ic_num);
/* integral_v with its output aliasing row 0 of f: cmm-simulation-kernel.cu:570-586 */
void og_integral_v(const double* f, double* rho, int nx, int ny, double hy);
/* h(v) of compute_periodification_function on grid g (NY values): cmm-simulation-host.cu:478-494,534-571 */
void og_periodification(const og_grid* g, double* h);
/* evaluate_potential_from_density_hermite: cmm-simulation-host.cu:385-415; -1 if unsupported grids */
int og_vlasov_potential(const double* ChiX, const double* ChiY, const double* f_fine, const og_grid* gmap,
                        const og_grid* gvort, const og_grid* gfine, const og_grid* gpsi, int molly, double* psi_out);
/* out[9] = {Etot, Ekin, Epot, Mass, Momentum, Emode1..4}: cmm-simulation-host.cu:639-664 */
void og_vlasov_mesure(const double* f_coarse, const og_grid* gc, const double* psi, const og_grid* gp, double* out);
void og_vlasov_state_mesure(const og_state* st, double* out);
/* stack composition + sampling of initial field var_num (0 vorticity, 2 distribution function) */
void og_compose_sample_var(const double* ChiX, const double* ChiY, const double* stack, int n, const og_grid* gm,
                           const og_grid* gt, int var_num, int ic_num, const double* discrete, const og_grid* gd,
                           double* out);

/* ---------------- sampled outputs (og_sample.c) ---------------- */
/* d_init_scalar: src/simulation/cmm-init.cu:253-298 */
double og_init_scalar(double x, double y, int scalar_num);
typedef struct {
    const og_grid* gc;              /* map grid */
    const double *ChiX, *ChiY;      /* current map */
    const double *stackX, *stackY;  /* n_maps stacked maps, 4*Nc each */
    int n_maps;
    const double* discrete;         /* Hermite discrete initial vorticity or NULL */
    const og_grid* gd;
    int ic_num;
    const double* psi;              /* psi level 0 (4*Np), for the zoom's psi samples */
    const og_grid* gp;
} og_state_view;
/* sample_compute_and_write, backward part (cmm-simulation-host.cu:706-893) on grid gs:
 * out = 10 planes of gs->N: map X, map Y, scalar, W, Laplacian W, dW/dx, dW/dy, psi,
 * dpsi/dx (Velocity_UX), dpsi/dy (Velocity_UY); mes = {Energy, Enstrophy,
 * Palinstrophy, Max_vorticity, Scalar_integral} with the reference's quirks */
void og_sample_fields(const og_state_view* st, const og_grid* gs, int scalar_num, double* out, double* mes);
void og_state_sample(const og_state* st, int n_sample, int scalar_num, double* out, double* mes);
/* compute_zoom, backward part (cmm-simulation-host.cu:1039-1201) on an n x n window grid with
 * bounds4 = (x_min, x_max, y_min, y_max): out = 6 planes of n*n: map X, map Y, scalar,
 * vorticity, distribution function, psi level 0 at the window points */
void og_zoom_fields(const og_state_view* st, int n, const double* bounds4, int scalar_num, double* out);
/* Vlasov sampled outputs on gs: 4 planes (map x, map y, distribution, stream) and
 * {Etot, Ekin, Epot, Mass, Momentum, Emode1..4} */
void og_vlasov_sample_fields(const og_state_view* st, const og_grid* gs, double* out, double* mes);
void og_state_vlasov_sample(const og_state* st, int n_sample, double* out, double* mes);
void og_state_zoom(const og_state* st, int n, const double* bounds4, int scalar_num, double* out);

/* ψ_x, ψ_y at particle positions (k_h_sample_points_dxdy, cmm-simulation-kernel.cu:138-155) */
void og_sample_points_dxdy(const og_state* st, const double* pos, double* out, int num);

/* particle advection on an explicit ψ history (src/numerical/cmm-particles.cu:119-276) */
void og_particle_advect(int num, double dt, double* pos, const double* psi, const og_grid* g,
                        int time_integration_num, int l_order, const double* Lp12);

/* ---- learned psi upsampler (og_learned.c): FP64 network, optional BF16 rounding emulation */
double og_bf16_round(double v);
void og_conv3x3(const double* x, int B, int H, int W, int cin, const double* w, const double* bias, int cout,
                const double* mask, const double* res, int relu, double* out);
void og_conv3x3_t(const double* dy, int B, int H, int W, int cin, const double* w, int cout, const double* mask,
                  const double* res, double* dx);
void og_conv3x3_dw(const double* x, const double* dy, int B, int H, int W, int cin, int cout, double* dw, double* db);
double og_upsampler_loss_grad(const double* params, int nb, int C, const double* s_in, double s_out,
                              const float* inputs, const float* targets, int B, int h, int w, int emulate_bf16, int cut,
                              double* grad);
double og_upsampler_loss_grad_sq(const double* params, int nb, int C, const double* s_in, double s_out,
                                 const float* inputs, const float* targets, int B, int h, int w, int emu, int cut,
                                 double* grad, double* dy_sq);

#ifdef __cplusplus
}
#endif
#endif
