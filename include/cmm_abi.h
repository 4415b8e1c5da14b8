/*
 * cmm_abi.h -- C-ABI of the GB300 (sm_103a) characteristic-mapping-method
 * time-step library, libcmm_gb300.so.
 *
 * Two levels:
 *  1. Context API: a drop-in for the reference drivers cuda_euler_2d
 *     (Cuda-CMM/src/simulation/cmm-euler2d.cu:45-1099) and cuda_vlasov_1d
 *     (src/simulation/cmm-vlasov1d.cu:48-1148, simulation_type
 *     cmm_vlasov_poisson_1d), configured exactly like
 *     the reference executable (src/main2d.cpp:66-105): presets, then every
 *     param_file=F argument, then COMMAND=VALUE arguments.  It writes the
 *     reference's output tree (data/<sim_name>_<ic>_C<c>_F<f>_t<1/dt>_T<T>/).
 *  2. Kernel API on caller-owned device buffers in the reference's planar
 *     Hermite layout ([f, f_x, f_y, f_xy] planes of N doubles, row-major
 *     iY*NX+iX), each a drop-in for one host function of
 *     src/simulation/cmm-simulation-host.h:23-77.
 *
 * Conventions: every function returns 0 on success or a negative CMM_ERR_*
 * code; nothing calls exit().  cmm_last_error() describes the last failure of
 * the calling thread.  All GPU work is ordered on the context stream (or on
 * the stream argument of the kernel API); one context per host thread.
 * No torch or CUDA runtime types appear in these signatures: streams are
 * passed as void* (a cudaStream_t, NULL = legacy default stream).
 */
#ifndef CMM_ABI_H
#define CMM_ABI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CMM_OK 0
#define CMM_ERR_PARAM (-1)      /* bad setting / argument (reference: error() -> exit) */
#define CMM_ERR_IO (-2)         /* unreadable input file, unwritable output */
#define CMM_ERR_CUDA (-3)       /* CUDA / cuRAND failure (reference: exit(0)) */
#define CMM_ERR_SATURATED (-4)  /* map stack full; loop stopped (reference: "Stack Saturated") */
#define CMM_ERR_STATE (-5)      /* call out of order (e.g. step before init) */
#define CMM_ERR_UNSUPPORTED (-6)/* option of the reference not built in this library */
#define CMM_ERR_NOT_FOUND (-7)  /* unknown field / scalar name */
#define CMM_ERR_TIMEOUT (-8)    /* a bounded device wait gave up (grid barrier of a batched ensemble iteration) */

typedef struct cmm_ctx cmm_ctx;

/* text of the last error of the calling thread ("" if none) */
const char* cmm_last_error(void);
/* library version string */
const char* cmm_version(void);

/* ---------------------------------------------------------------- context API */

/* Parse settings like main() (src/main2d.cpp:73-89) and create a context.
 * No GPU work happens here.  Replaces: SettingsCMM(argc,args) +
 * load_param_file (src/ui/cmm-param.cu:149-229) + applyCommands
 * (src/ui/settings.cu:334-343). */
int cmm_create(int argc, const char* const* argv, cmm_ctx** out);

/* Use this CUDA stream (cudaStream_t as void*) for all work of the context;
 * must precede cmm_init.  Default: a stream owned by the context. */
int cmm_set_stream(cmm_ctx* ctx, void* stream);

/* Provide the discrete initial vorticity (n = initial_discrete_grid^2 values,
 * row-major, host memory) instead of reading initial_discrete_location.
 * Must precede cmm_init.  Replaces readTransferFromBinaryFile at
 * src/simulation/cmm-euler2d.cu:329. */
int cmm_set_initial_discrete(cmm_ctx* ctx, const double* host_values, size_t n);

/* Allocate, build the initial state and the Lagrange velocity history, write
 * the t=0 outputs.  Replaces cmm-euler2d.cu:129-737. */
int cmm_init(cmm_ctx* ctx);

/* Advance n loop iterations (each: map advection, incompressibility check,
 * remap, psi solve, coarse vorticity, particles, saves, monitors).  Returns
 * CMM_ERR_SATURATED when the map stack filled (the loop has stopped), and 1
 * when the final time was reached before n iterations.  Replaces one pass of
 * the loop at cmm-euler2d.cu:750-960. */
int cmm_step(cmm_ctx* ctx, int n);

/* Run to the final time and write the final outputs ("Finished simulation").
 * Replaces cmm-euler2d.cu:750-1099. */
int cmm_run(cmm_ctx* ctx);

/* Copy a field to host memory, in the reference's layout.  Names follow the
 * reference's output files: "Map_ChiX_H_coarse", "Map_ChiY_H_coarse" (4*Nc),
 * "Stream_function_Psi_H_psi" (4*Npsi, newest level), "Stream_function_Psi_H_psi_all"
 * (L*4*Npsi), "Vorticity_W_coarse" (Nc; for Vlasov-Poisson the distribution,
 * also as "Distribution_coarse"), "Vorticity_W_fine_H" (4*Nf), "Map_stack"
 * (n_maps * 8*Nc, oldest first),
 * "Particles_advected_pos_PNN" (2*num), "Particles_advected_vel_UNN" (2*num: the
 * velocity state of an inertial set, (psi_x, psi_y) at the particles of a tracer set),
 * "Init_random_table" (1098: the 1000 uniform(-1,1) values of gaussian_blobs, then the
 * 98 cuRAND blob offsets of turbulence_gaussienne).
 * bytes must equal the field size. */
int cmm_get_field(cmm_ctx* ctx, const char* name, void* host_dst, size_t bytes);
/* Size in bytes of a field (0 if unknown). */
size_t cmm_field_bytes(cmm_ctx* ctx, const char* name);

/* Scalars: "time", "dt", "e_inc", "map_counter", "map_gap", "loop_ctr",
 * "lagrange_order", "stack_capacity"; Euler: "energy", "enstrophy",
 * "palinstrophy", "max_vorticity" (src/numerical/cmm-mesure.cu:30-89);
 * Vlasov-Poisson: "etot", "ekin", "epot", "mass", "momentum", "emode1".."emode4"
 * (src/numerical/cmm-mesure.cu:97-202).  Diagnostics are computed on request. */
int cmm_get_scalar(cmm_ctx* ctx, const char* name, double* out);

/* Time each loop phase with CUDA events on the context stream (adds one
 * stream synchronisation per iteration while on).  Totals are read back as
 * scalars "prof_<phase>_ms" / "prof_<phase>_count" for the phases advect,
 * incomp, remap, psi, coarse, particles, save; "kernel_launches" and
 * "fft_calls" count this library's kernel launches and 2D / 1D transform calls.
 * The reference has no counterpart (it only logs wall-clock C-Time,
 * src/simulation/cmm-euler2d.cu:940-959). */
int cmm_set_profiling(cmm_ctx* ctx, int on);

/* Resolved settings as the reference's param-file text (cmm-param.cu:39-146)
 * into buf (NUL-terminated, truncated to cap); returns the full length.
 * Works without a GPU. */
int cmm_settings_text(cmm_ctx* ctx, char* buf, size_t cap);
/* Derived name of the output folder (cmm-euler2d.cu:81-83); works without a GPU. */
int cmm_file_name(cmm_ctx* ctx, char* buf, size_t cap);

int cmm_destroy(cmm_ctx* ctx);

/* ---------------------------------------------------------------- kernel API */

/* Periodic grid: NX x NY nodes on [bounds[0],bounds[1]) x [bounds[2],bounds[3]),
 * spacing (bounds[1]-bounds[0])/NX.  Mirrors TCudaGrid2D
 * (src/grid/cmm-grid2d.h:25-39). */
typedef struct {
    int NX, NY;
    double bounds[4];
} cmm_grid;

/* Backward map advection by GALS footpoints.  Replaces
 * advect_using_stream_hermite (src/simulation/cmm-simulation-host.cu:64-104)
 * for direction -1.  psi_levels: l_order device pointers to Hermite levels
 * (level 0 newest).  L1/L12: Lagrange coefficients for t_{n+1} and
 * t_{n+1/2} (get_L_coefficient, src/numerical/cmm-timestep.cu:474-484).
 * time_integration_num: 10 EulerExp, 21 RK2, 30 RK3; map_update_order_num:
 * 0 2nd, 1 4th, 2 6th.  Writes the new map to chix_out / chiy_out. */
int cmm_advect_map(const cmm_grid* grid_map, const cmm_grid* grid_psi, const double* chix, const double* chiy,
                   double* chix_out, double* chiy_out, const double* const* psi_levels, int l_order,
                   const double* L1, const double* L12, double dt, double map_epsilon, int time_integration_num,
                   int map_update_order_num, void* stream);

/* max |1 - det grad X| at half-shifted points of grid_check -> *d_result
 * (one double in device memory).  Replaces incompressibility_check
 * (src/simulation/cmm-simulation-host.cu:44-50). */
int cmm_incomp_max(const cmm_grid* grid_check, const cmm_grid* grid_map, const double* chix, const double* chiy,
                   double* d_result, void* stream);

/* omega_0(X_0(...X_{n-1}(X_cur(x)))) on grid_target.  stack: n_maps maps
 * contiguous in device memory, map i = [X planes | Y planes] at stack + i*8*Nc
 * (i = 0 oldest).  ic_num: analytic initial-condition number (settings name table);
 * when discrete != NULL the Hermite discrete field on grid_discrete is
 * sampled instead.  Replaces apply_map_stack + k_h_sample_from_init
 * (src/simulation/cmm-simulation-host.cu:112-128,299-316). */
int cmm_compose_stack(const cmm_grid* grid_map, const cmm_grid* grid_target, const double* chix,
                      const double* chiy, const double* stack, int n_maps, int ic_num,
                      const double* discrete, const cmm_grid* grid_discrete, double* out, void* stream);

/* As cmm_compose_stack for the initial field selected by var_num, the
 * reference's last argument of translate_initial_condition_through_map_stack
 * (cmm-simulation-host.cu:299-327; k_h_sample_from_init,
 * cmm-simulation-kernel.cu:342-373): 0 vorticity, 1 passive scalar,
 * 2 Vlasov distribution function (ic_num 0 landau_damping, 1 two_stream,
 * 2 nonlin_landau_damping). */
int cmm_compose_stack_var(const cmm_grid* grid_map, const cmm_grid* grid_target, const double* chix,
                          const double* chiy, const double* stack, int n_maps, int var_num, int ic_num,
                          const double* discrete, const cmm_grid* grid_discrete, double* out, void* stream);

/* omega(x) = W_fine(X(x)) on grid_out (molly_stencil 0, 4 or 8).  Replaces
 * k_apply_map_and_sample_from_hermite (src/simulation/cmm-simulation-kernel.cu:402-461). */
int cmm_sample_vort(const cmm_grid* grid_map, const cmm_grid* grid_out, const cmm_grid* grid_fine,
                    const double* chix, const double* chiy, const double* w_fine, int molly_stencil, double* out,
                    void* stream);

/* Poisson / Hermite solve: vorticity samples on grid_vort -> Hermite stream
 * function (4 planes) on grid_psi.  Replaces the FFT part of
 * evaluate_stream_hermite (src/simulation/cmm-simulation-host.cu:349-374).
 * Plans and workspace live in the opaque handle. */
typedef struct cmm_poisson cmm_poisson;
int cmm_poisson_create(const cmm_grid* grid_vort, const cmm_grid* grid_psi, double freq_cut_psi, void* stream,
                       cmm_poisson** out);
int cmm_poisson_hermite(cmm_poisson* p, const double* vort, double* psi_out);
int cmm_poisson_destroy(cmm_poisson* p);

/* ---------------------------------------------------------------- transforms
 * The library's own 2D real FFT on sm_103a (no cuFFT): replaces the cuFFT D2Z / Z2D plans
 * the reference builds per grid (src/grid/cmm-grid2d.cu:123-131) and their cufftExecD2Z /
 * cufftExecZ2D calls (src/numerical/cmm-fft.cu:398-429, src/simulation/cmm-simulation-host.cu:
 * 299-375).  ny rows of nx real values <-> ny rows of nx/2+1 complex values (interleaved re,
 * im), unnormalised, cuFFT's sign conventions; `batch` items back to back; precision 0 =
 * FP64, 1 = FP32.  C2R ignores the imaginary parts of the kx = 0 and kx = nx/2 columns after
 * the column transform and may overwrite its input, as cuFFT's C2R does.  Shapes: nx even,
 * nx/2 and ny at most 8192 (FP64 columns longer than 4096 and lengths with prime factors
 * 5..13 run slower), every prime factor at most 13 (else CMM_ERR_PARAM).  Stream-ordered;
 * the transforms allocate nothing. */
typedef struct cmm_fft cmm_fft;
int cmm_fft_create(int nx, int ny, int precision, void* stream, cmm_fft** out);
int cmm_fft_r2c(cmm_fft* f, const void* in, void* out, int batch);
int cmm_fft_c2r(cmm_fft* f, void* in, void* out, int batch);
int cmm_fft_destroy(cmm_fft* f);

/* Vlasov-Poisson potential.  Replaces evaluate_potential_from_density_hermite
 * (src/simulation/cmm-simulation-host.cu:385-471,534-571): f = f_fine_H o X on
 * grid_vort, rho = h_v sum_v f - 1, phi from the 1D Poisson solve on the x
 * axis, psi = phi(x) - h(v) with h the periodification of the velocity, and
 * psi's Hermite planes [psi, psi_x, psi_y, psi_xy] on grid_psi (4*Npsi
 * doubles).  grid_vort may not be finer than grid_psi and grid_psi must be
 * square (the reference's restrictions, CMM_ERR_PARAM).  h is built at
 * creation (it depends on the grid only). */
typedef struct cmm_vlasov cmm_vlasov;
int cmm_vlasov_create(const cmm_grid* grid_vort, const cmm_grid* grid_psi, void* stream, cmm_vlasov** out);
int cmm_vlasov_potential(cmm_vlasov* p, const cmm_grid* grid_map, const cmm_grid* grid_fine, const double* chix,
                         const double* chiy, const double* f_fine_H, int molly_stencil, double* psi_out);
/* Vlasov conservation targets (cmm-simulation-host.cu:639-664, cmm-mesure.cu:97-202):
 * out9 = {Etot, Ekin, Epot, Mass, Momentum, |E_1|..|E_4|} from the coarse
 * distribution f_coarse (grid_coarse) and psi (grid_psi).  Synchronises the stream. */
int cmm_vlasov_diagnostics(cmm_vlasov* p, const cmm_grid* grid_coarse, const double* f_coarse, const double* psi,
                           double* out9);
int cmm_vlasov_destroy(cmm_vlasov* p);

/* Tracer particles (tau = 0).  Replaces particles_advect / Particle_advect
 * (src/numerical/cmm-particles.cu:63-87,119-276).  pos: 2*num interleaved
 * (x, y) in device memory; psi_levels[0] = t_{n+1}, [1] = t_n, ... */
int cmm_particles_advect(const cmm_grid* grid_psi, double* pos, int num, const double* const* psi_levels,
                         int l_order, const double* Lp12, double dt, int time_integration_num, void* stream);

/* Energy (psi Hermite), enstrophy (coarse omega) and max |omega| -> host out[3].
 * Replaces Compute_Energy_H / Compute_Enstrophy / the w_max reduction
 * (src/numerical/cmm-mesure.cu:30-57, cmm-simulation-host.cu:668-673).
 * Synchronises the stream. */
int cmm_diagnostics(const cmm_grid* grid_psi, const double* psi, const cmm_grid* grid_coarse, const double* vort,
                    double* out3, void* stream);

/* Same results as cmm_diagnostics (to rounding: the partial sums are grouped
 * differently) without allocating device memory: no counterpart in the
 * reference.  For callers that may not allocate, e.g. a host that reserves
 * all device memory up front or a loop that cannot take cudaFree's implicit
 * device-wide synchronisation.  The reduction scratch is a fixed array
 * inside the library (about 393 KB per GPU, resident while the library is
 * loaded), so 2*NX*NY of grid_psi and NX*NY of grid_coarse may each be at
 * most 4194304 (2048^2 coarse, 1448^2 psi); larger grids -> CMM_ERR_PARAM.
 * The first call on each device looks up the array's address (set-up, with
 * that device current) and keeps it for the life of the process; later calls
 * only launch.  A cudaDeviceReset ends that address's validity: a process that
 * resets the device must not call this entry point afterwards.  Nothing in the
 * scratch has to start at zero.  Calls that overlap -- other streams or host
 * threads -- race on the one array: serialise them.  Synchronises the stream. */
int cmm_diagnostics_noalloc(const cmm_grid* grid_psi, const double* psi, const cmm_grid* grid_coarse,
                            const double* vort, double* out3, void* stream);

/* ---------------------------------------------------------------- ensembles
 * Many mixed-form 2D Euler runs of uneven sizes advanced together: one iteration
 * advances every member by one of its own time steps.  By default the whole iteration of
 * every member -- advection, incompressibility check, remap decision and remap (composition
 * through the stack, fine-grid transforms), psi solve and coarse sample -- runs in one
 * cooperative launch of persistent blocks fed by device work queues, with its shape (resident
 * blocks, tiles per task) picked by an autotuner on the first iterations and the iteration
 * replayed from a CUDA graph.  Where a member does not allow that (see cmm_ensemble_fused_info)
 * the iteration runs as two batched phases with the remaps on the host between them.  Each
 * member is configured like cmm_create (argc[i] strings of argv, members one after another)
 * and must be precision=mixed, 2D Euler, three Lagrange levels, EulerExp / RK2 / RK3 maps.
 * The reference has no ensemble driver; this is new API. */
typedef struct cmm_ensemble cmm_ensemble;
int cmm_ensemble_create(int n_members, const int* argc, const char* const* argv, void* stream, cmm_ensemble** out);
int cmm_ensemble_set_initial_discrete(cmm_ensemble* e, int member, const double* values, size_t n);
/* 0: plain launches every iteration; 1 (default): CUDA graphs after the first iteration */
int cmm_ensemble_set_graphs(cmm_ensemble* e, int on);
int cmm_ensemble_init(cmm_ensemble* e);
/* n iterations; 1 when every member has reached its final time */
int cmm_ensemble_step(cmm_ensemble* e, int n);
int cmm_ensemble_run(cmm_ensemble* e);
int cmm_ensemble_get_scalar(cmm_ensemble* e, int member, const char* name, double* out);
int cmm_ensemble_get_field(cmm_ensemble* e, int member, const char* name, void* host_dst, size_t bytes);
size_t cmm_ensemble_field_bytes(cmm_ensemble* e, int member, const char* name);
/* out6 = {member time steps, iterations, batched launches, members, advection grid, sample grid} */
int cmm_ensemble_stats(cmm_ensemble* e, long long* out6);
/* before cmm_ensemble_init, the iteration form: 0 the two-phase iteration with the remaps on the
 * host, 1 the single launch, 2 (default) the autotuner's choice between the single launch in each
 * of its shapes and the two-phase iteration with the remaps in one batched launch.  1 and 2 fall
 * back to 0 where a member does not allow the single launch (cmm_ensemble_fused_info). */
int cmm_ensemble_set_fused(cmm_ensemble* e, int mode);
/* polls (about 64 ns apart) after which a grid barrier of the single launch gives up: the
 * launch ends, cmm_ensemble_step returns CMM_ERR_TIMEOUT and the ensemble refuses further
 * steps (its members' states are partial); the CUDA context stays usable.  Default 2^24. */
int cmm_ensemble_set_wait_limit(cmm_ensemble* e, long long polls);
/* out6 = {single launch available (1) or not (0), in use (1: the single launch, 0: the two-phase
 * iteration), the shape in use: register budget (resident blocks per SM the launch is compiled
 * for: 4 -> 64 registers, 6 -> 40; 0 the two-phase iteration), blocks, tiles per task, waves of
 * the last single launch}; why (if not NULL, why_cap bytes) receives the reason it is unavailable */
int cmm_ensemble_fused_info(cmm_ensemble* e, long long* out6, char* why, size_t why_cap);
/* the autotuner's table, up to cap entries of {register budget (0: the two-phase iteration with
 * batched remaps), blocks, tiles per task, median iteration wall ns}; returns the number of
 * entries (0 until tuning has finished) */
int cmm_ensemble_tuning(cmm_ensemble* e, long long* out4, int cap);
/* profiling of the single-launch iteration (after cmm_ensemble_init; on = 1 zeroes the counters).
 * cmm_ensemble_profile fills out56: [0..10] block cycles per stage (precombine, advect, check,
 * compose, fine rows, fine columns, fine inverse rows, sample, psi rows, psi columns, psi inverse
 * rows), [16..26] tasks per stage, [32] block cycles waiting in grid barriers, [40..55] nanoseconds
 * per wave, each summed over the iterations since profiling was switched on */
int cmm_ensemble_set_profiling(cmm_ensemble* e, int on);
int cmm_ensemble_profile(cmm_ensemble* e, unsigned long long* out56);
int cmm_ensemble_destroy(cmm_ensemble* e);

/* ---------------------------------------------------------------- learned psi
 * A residual network of 3x3 periodic convolutions (BF16 tensor-core kernels, FP32
 * accumulation) that predicts, on the psi grid (2h x 2w, the 2 x 2 sub-pixels of each map
 * cell), the vorticity the map-grid samples miss (omega sampled through the map on the psi
 * grid minus the spectral interpolation of the map-grid samples) from fields of the map
 * grid (h x w, w a multiple of 128): the cheap psi (from omega sampled on the map grid) with
 * psi_x, psi_y, psi_xy, and omega with omega_x, omega_y (through the map's Jacobian).  The
 * learned psi is the method's spectral solve of the cheap vorticity plus the prediction.  Trained on the GPU on pairs collected from running simulations
 * (precision=mixed, psi grid = 2 x map grid).  The reference has no learned part; this is
 * new API.  With cmm_attach_upsampler (or psi_upsampler=<file> in the settings) every
 * exact_every-th step of a simulation runs the exact evaluation and judges the learned psi
 * and the cheap psi against it (relative L-infinity difference); the following
 * exact_every - 1 steps use the network if it is within tol and closer than the cheap psi,
 * else the cheap psi if that is within tol, else the exact evaluation.  Scalars of the
 * context: learned_steps, cheap_steps, exact_steps, learned_checks, learned_cheaper (checks
 * where the cheap psi was chosen), learned_failures (checks where neither met tol),
 * learned_last_err, learned_max_err (of the learned psi at the checks). */
typedef struct cmm_upsampler cmm_upsampler;
/* blocks residual blocks of two convolutions of `channels` (= 32) channels; weights drawn
 * from mt19937_64(seed) */
int cmm_upsampler_create(int blocks, int channels, unsigned long long seed, void* stream, cmm_upsampler** out);
int cmm_upsampler_destroy(cmm_upsampler* u);
long long cmm_upsampler_num_params(const cmm_upsampler* u);
/* FP32 parameters, layer by layer: W[9][cin][cout] (tap = 3 (dy + 1) + dx + 1), b[cout];
 * layers: head (16 -> C, input channels 7..15 unused), per block two (C -> C), tail
 * (C -> 16, output channels 4..15 unused) */
int cmm_upsampler_get_params(const cmm_upsampler* u, float* out, long long n);
int cmm_upsampler_set_params(cmm_upsampler* u, const float* in, long long n);
/* gradient of the last cmm_upsampler_loss_grad, same layout */
int cmm_upsampler_get_grads(const cmm_upsampler* u, float* out, long long n);
/* input channel scales (7) and target scale: the network sees inputs / s_in and predicts
 * target / s_out; set from the training pairs' RMS by the first cmm_upsampler_train */
int cmm_upsampler_set_scales(cmm_upsampler* u, const double* s_in7, double s_out);
int cmm_upsampler_get_scales(const cmm_upsampler* u, double* s_in7, double* s_out);
/* one training pair from the context's current state (its last psi must be exact) */
int cmm_upsampler_collect(cmm_upsampler* u, cmm_ctx* c);
int cmm_upsampler_dataset_size(const cmm_upsampler* u);
/* drop every collected pair (their device buffers are freed, after the work queued on the
 * device), so that training can stream pairs: collect a chunk, train on it, clear, collect
 * the next */
int cmm_upsampler_clear_dataset(cmm_upsampler* u);
/* iters Adam steps (lr) on batches of `batch` pairs drawn with mt19937_64(seed); mean loss
 * of the last min(iters, 16) steps and the device seconds of the call */
int cmm_upsampler_train(cmm_upsampler* u, int iters, int batch, double lr, unsigned long long seed, double* loss,
                        double* seconds);
/* loss and its gradient for B host samples: inputs[B][7][h][w] (psi, psi_x, psi_y, psi_xy,
 * omega, omega_x, omega_y), targets[B][2h][2w] (the sub-grid vorticity).  cut = 0: mean
 * squared error of the scaled prediction; cut > 0: the training loss, the relative
 * psi-space error sum w |FFT(pred - target)|^2 / sum w |FFT(target)|^2 with w = 1/|k|^4 on
 * 0 < |k| <= cut (integer wavenumbers of the 2h x 2w grid) */
int cmm_upsampler_loss_grad(cmm_upsampler* u, const float* inputs, const float* targets, int B, int h, int w, int cut,
                            double* loss);
/* the predicted sub-grid vorticity on the psi grid (fine[2h][2w]) for host inputs[7][h][w] */
int cmm_upsampler_infer(cmm_upsampler* u, const float* inputs, int h, int w, float* fine);
/* relative differences from the context's exact psi level of the cheap psi, the learned psi
 * and the psi of omega sampled exactly on the psi grid (the best a network can reach):
 * out6 = {cheap Linf, cheap L2, learned Linf, learned L2, psi-grid Linf, psi-grid L2} */
int cmm_upsampler_evaluate(cmm_upsampler* u, cmm_ctx* c, double* out6);
/* device milliseconds of one inference on an h x w map grid (mean of iters after 2 warm-ups) */
int cmm_upsampler_time_infer(cmm_upsampler* u, int h, int w, int iters, double* ms);
int cmm_upsampler_save(const cmm_upsampler* u, const char* path);
int cmm_upsampler_load(cmm_upsampler* u, const char* path);
/* attach (NULL detaches) after cmm_init; the upsampler must outlive the attachment */
int cmm_attach_upsampler(cmm_ctx* c, cmm_upsampler* u, int exact_every, double tol);

/* one periodic 3x3 convolution on host buffers (the network's kernel):
 * out = [relu](conv(x, w) + bias) [* (mask > 0)] [+ res]; x[B*H][W][cin] BF16 bits,
 * w[9][cin][cout] BF16 bits, bias[cout] or NULL, mask / res [B*H][W][cout] BF16 bits or
 * NULL; out_f32 and/or out_bf16 [B*H][W][cout]; cin, cout in {16, 32}; W a multiple of 128 */
int cmm_conv3x3(const unsigned short* x, const unsigned short* w, const float* bias, const unsigned short* mask,
                const unsigned short* res, int relu, int B, int H, int W, int cin, int cout, float* out_f32,
                unsigned short* out_bf16);
/* its weight and bias gradients for the output gradient dy[B*H][W][cout]:
 * dw[9][cin][cout] = sum_p x[p + tap offset][ci] dy[p][co], db[cout] = sum_p dy[p][co] */
int cmm_conv3x3_weight_grad(const unsigned short* x, const unsigned short* dy, int B, int H, int W, int cin, int cout,
                            float* dw, float* db);

#ifdef __cplusplus
}
#endif
#endif
