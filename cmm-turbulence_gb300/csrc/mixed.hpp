// mixed.hpp -- launchers of the mixed-precision form (FP32 displacement maps,
// FP32 Hermite stream function / fine vorticity, FP64 composition, FP64
// determinant deviation and FP64 diagnostic sums).
#pragma once
#include <cuda_runtime.h>

#include "kernels.hpp"

namespace cmm {

// Map node layout: two float4 per node,
//   a = (dX, dY, dX_x, dY_x), b = (dX_y, dY_y, dX_xy, dY_xy),  d = X - x, dX_x = X_x - 1, dY_y = Y_y - 1.
struct AdvectMArgs {
    Grid gm, gp;
    const float4* map;      // 2*Nc float4
    float4* out;            // 2*Nc float4
    const float4* psiA;     // k1 field: sum_l L1[l] psi_l
    const float4* psiB;     // k2 field of RK3: sum_l L12[l] psi_l
    const float4* psi0;     // newest level
    const float4* psi1;     // level 1 (Adams-Bashforth 2, RK3Mod)
    // separable stream function (Vlasov-Poisson): FP64 1D tables (f(i+1) - f(i), f'(i)) of
    // the x-part of each combination and of h(v); tv != nullptr selects them (and FP64
    // characteristics, coef64 / dt64 / ep64) over the nodes
    const double2* tA;
    const double2* tB;
    const double2* t0;
    const double2* tv;
    double coef64[4][kMaxFoot];
    double dt64, ep64;
    double tau64;               // separable psi: the map's age (time since its identity), see SepDrift
    const double2* drows;       // separable psi: SepDrift's per-row table
    float coef[4][kMaxFoot];
    float dt, ep;
    int time_integration_num;   // 10, 21, 20, 30, 40, 31, 41
    int nfoot;
    int rp;                     // psi cells per map cell (Npsi / Nmap, integer)
    int nx_log2;                // log2 of the map grid's NX when a power of two, else -1
};

// The Vlasov-Poisson mixed form stores its maps in the free-streaming frame: a map of age tau
// (the time since it was the identity) is X = x + tau Phi(v) + d'(x, v), Y = v + d_v(x, v), where
// Phi is the map grid's cubic Hermite interpolant of h' (u_x = -h'(v): free streaming; h the
// velocity part of the separable psi) with node values h'(v_j) and slopes h''(v_j) (the mean of
// the two sides at a node of h's table, as the GALS stencil's symmetric differences see it), and
// only d' sits in the FP32 nodes.  Free streaming moves X by |v| tau, tens of length units
// between remaps; d' holds what the electric field adds, so FP32 keeps it to 1e-7 of a small
// number.  Because the drift is the map grid's own interpolant of its node data, X is exactly
// the Hermite map of node data d' + (tau h'(v_j), 0, tau h''(v_j), 0) -- the map the plain form
// would hold -- and every reader adds the drift in FP64 from the per-row table.
struct SepDrift {
    const double2* rows;        // (h'(v_j), h''(v_j)) for each map-grid row j
    Grid gm;                    // the map grid
    double tau;                 // the active map's age
    const double* taus;         // the stacked maps' ages (compositions; null elsewhere)
};
// the per-row table of SepDrift from h's table tv (T[i] = (h(i+1) - h(i), h'(i)) on gp's v axis)
cudaError_t launch_drift_rows(const double2* tv, const Grid& gp, const Grid& gm, double2* rows, cudaStream_t s);

cudaError_t launch_init_map_m(float4* map, const Grid& g, cudaStream_t s);
// outA = sum_l cA[l] levels[l], outB likewise (outB may be null)
cudaError_t launch_precombine(float4* const* levels, int L, const double* cA, const double* cB, long long n,
                              float4* outA, float4* outB, cudaStream_t s);
// psi solve's last pass for 3 Lagrange levels: new level nodes (out0) from 4 FP32 planes and the
// combinations c1, c2, c3 of the levels (new, l1, l2) -> o1, o2, o3 (same arithmetic as launch_precombine)
cudaError_t launch_psi_nodes3(const float* planes, long long n, const float4* l1, const float4* l2, const double* c1,
                              const double* c2, const double* c3, float4* out0, float4* o1, float4* o2, float4* o3,
                              cudaStream_t s);
cudaError_t launch_advect_m(const AdvectMArgs& a, cudaStream_t s);
// the psi solve on the library's FFT (psi_solve.cuh): omega through the map on gv (into the
// scratch omega, gv.N floats), its kept modes, the psi nodes on gp and, with c1 != nullptr,
// the three Lagrange combinations of launch_psi_nodes3, in four launches; runs when
// psi_solve_m_fits (vort grid an integer multiple of the map grid, shapes the kernels
// hold), which also gives the complex values the work arrays w1, w2 need
bool psi_solve_m_fits(const Grid& gm, const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv,
                      const fft::Plan2D& pp, long long* w1_values, long long* w2_values);
void psi_solve_m_prepare();
cudaError_t launch_psi_solve_m(const Grid& gm, const Grid& gv, const Grid& gf, const float4* map, const float4* W,
                               const Grid& gp, double freq, const fft::Plan2D& pv, const fft::Plan2D& pp, float* omega,
                               float2* w1, float2* w2, float4* out0, const float4* l1, const float4* l2,
                               const double* c1, const double* c2, const double* c3, float4* o1, float4* o2,
                               float4* o3, cudaStream_t s);
// max |det grad X - 1| on the half-shifted check grid with r = Ncheck / Nmap points per cell and axis
// (r * Nmap^2 < 2^31)
cudaError_t launch_incomp_m(const Grid& gm, int r, const float4* map, double* d_result, cudaStream_t s,
                            const SepDrift* drift = nullptr);
// the same check writing d_result, which must be zero on entry, and zeroing d_clear for the
// next check (two slots used alternately: no clearing memset between the map advection and
// the check); launched as a programmatic dependent of the previous kernel
cudaError_t launch_incomp_m_pp(const Grid& gm, int r, const float4* map, double* d_result, double* d_clear,
                               cudaStream_t s);
// omega_0 through current map + n stacked maps (n * 2*Nc float4), 64-bit fixed-point
// positions; a discrete initial field (src.kind 3) is read from its FP32 Hermite nodes disc
// (out_f != nullptr: FP32 output instead of out)
cudaError_t launch_compose_m(const Grid& gm, const Grid& gt, const float4* map, const float4* stack, int n_maps,
                             const InitSource& src, const float4* disc, double* out, cudaStream_t s,
                             float* out_f = nullptr,
                             const SepDrift* drift = nullptr);
// fixed-point constants of launch_compose_m: the target grid's node spacing, the map domain's scale
void fix_constants(const Grid& gm, const Grid& gt, unsigned long long* stx, unsigned long long* sty, float2* scx,
                   float2* scy);
// FP32 Hermite spectra [F, i kx F, i ky F, -kx ky F] of an unnormalised R2C half spectrum
cudaError_t launch_spec_hermite_f(const float2* F, const Grid& g, float2* out4, cudaStream_t s);
// positions of the nodes of gt through the current map and the stack (fixed point), as FP64
cudaError_t launch_compose_pos_m(const Grid& gm, const Grid& gt, const float4* map, const float4* stack, int n_maps,
                                 double* px, double* py, cudaStream_t s, const SepDrift* drift = nullptr);
// W(x + d(x)) on grid go (Ngo multiple of Nmap, Nf multiple of Ngo); out_f or out_d
cudaError_t launch_sample_m(const Grid& gm, const Grid& go, const Grid& gf, const float4* map, const float4* W,
                            float* out_f, double* out_d, cudaStream_t s,
                            const SepDrift* drift = nullptr);
// tracers at 64-bit fixed-point positions P = (x - b0) / W * 2^64 (interleaved x, y)
// (tA, tB, t0, tv: separable tables as in AdvectMArgs, used when tv != nullptr)
// psiA = level t_n, psiB = the t_{n+1/2} combination, psi0 = t_{n+1}, psiC = t_{n-1} (RK3Mod);
// tau != 0: inertial particles with FP32 velocity state vel; tv != nullptr: separable psi tables
cudaError_t launch_particles_m(const Grid& gp, unsigned long long* pos, int num, const float4* psiA,
                               const float4* psiB, const float4* psi0, double dt, int ti, cudaStream_t s,
                               const double2* tA = nullptr, const double2* tB = nullptr,
                               const double2* t0 = nullptr, const double2* tv = nullptr,
                               const float4* psiC = nullptr, float2* vel = nullptr, double tau = 0.0);
cudaError_t launch_particle_vel_init_m(const Grid& gp, const unsigned long long* pos, int num, const float4* psi0,
                                       float2* vel, cudaStream_t s);
cudaError_t launch_vel_to_f64(const float2* v, int num, double* out, cudaStream_t s, const int* perm = nullptr);
cudaError_t launch_vel_from_f64(const double* v, int num, float2* out, cudaStream_t s);
cudaError_t launch_pos_to_fix(const double* pos, int num, const Grid& g, unsigned long long* out, cudaStream_t s);
cudaError_t launch_fix_to_pos(const unsigned long long* in, int num, const Grid& g, double* pos, cudaStream_t s,
                              const int* perm = nullptr);
// tracer storage order (counting sort by bucket of 4 x 4 psi cells; perm = original index of
// each stored tracer; the FP64 views above write through perm)
struct TracerScratch {
    unsigned long long* pos = nullptr;   // 2 x cap
    float2* vel = nullptr;               // cap
    int *perm = nullptr, *key = nullptr, *rank = nullptr;   // cap each
    int* count = nullptr;                // nb_cap
    int cap = 0, nb_cap = 0;
};
cudaError_t launch_tracer_reorder(const Grid& gp, unsigned long long* pos, float2* vel, int* perm, int num,
                                  TracerScratch& t, cudaStream_t s);
cudaError_t launch_iota(int* p, int num, cudaStream_t s);
// learned psi: the psi solve of (omega sampled on the map grid gc, spectrum Fc, interpolated
// spectrally) + (vorticity correction on the psi grid, spectrum D); cut off and
// differentiated like launch_spec_psi_f
cudaError_t launch_spec_psi_learned(const float2* Fc, const Grid& gc, const float2* D, const Grid& gp, double freq,
                                    float2* out4, cudaStream_t s);
// the map-grid spectrum Fc placed in the psi grid's spectrum (normalised by 1/gc.N): its
// inverse transform on the psi grid is the spectral interpolation of the map-grid samples
cudaError_t launch_spec_pad(const float2* Fc, const Grid& gc, const Grid& gp, float2* out, cudaStream_t s);
// omega, omega_x, omega_y at the map-grid nodes (3 planes of gm.N floats)
cudaError_t launch_sample_grad_m(const Grid& gm, const Grid& gf, const float4* map, const float4* W, float* out3,
                                 cudaStream_t s);
cudaError_t launch_spec_psi_f(const float2* Fv, const Grid& gv, const Grid& gp, double freq, float2* out4,
                              cudaStream_t s);
// 4 planes (float or double) -> float4 nodes
cudaError_t launch_planes_to_float4(const float* planes, const double* planes_d, long long n, float4* out,
                                    cudaStream_t s);
cudaError_t launch_float4_to_planes(const float4* in, long long n, double* planes, cudaStream_t s);
cudaError_t launch_map_to_planes(const float4* map, const Grid& g, double* X, double* Y, cudaStream_t s,
                                 const SepDrift* drift = nullptr);
cudaError_t launch_planes_to_map(const double* X, const double* Y, const Grid& g, float4* map, cudaStream_t s);
// sum psi_x^2 + psi_y^2 (FP64 accumulation) -> out[0]
cudaError_t launch_energy_m(const float4* psi, long long n, double* scratch, double* out, cudaStream_t s);

// ---------------------------------------------------------------- ensembles
// Lagrange coefficients of three psi levels for three combinations
struct Combo3 { float c[3][3]; };

// one member of an ensemble step, as the batched kernels see it (csrc/ensemble.cpp fills it)
struct EnsMember {
    AdvectMArgs adv;                 // advection of the member's map (gm, gp, map, out, combinations, ...)
    int active;                      // 0: the member's tiles do nothing
    int r_check;                     // check points per map cell and axis (fine / map)
    float ir_check;
    int fused;                       // the nodes pass also writes the three Lagrange combinations
    unsigned long long* einc;        // the member's incompressibility result (FP64 bits)
    Grid gv, gf;                     // vort and fine grids
    const float4* wfm;               // fine vorticity nodes
    float* sample_out;               // omega on the vort grid (R2C input, class buffer slot)
    const float2* spec_v;            // its half spectrum (class buffer slot)
    float2* spec4;                   // the four psi spectra (C2R input, class buffer slot)
    const float* planes;             // the four psi planes (C2R output, class buffer slot)
    float freq, inv_nv;              // psi cut-off frequency, 1 / N of the vort grid
    float4* psi_new;                 // the new psi level's nodes
    const float4* lv1n;              // levels 1 and 2 after the rotation (fused combinations)
    const float4* lv2n;
    float4* o1;
    float4* o2;
    float4* o3;
    Combo3 cm;
    double* vort;                    // coarse vorticity
    int precombine;                  // combine lv0..lv2 into pa (ca) and pb (cb) before the advection
    const float4* lv0;
    const float4* lv1;
    const float4* lv2;
    float4* pa;
    float4* pb;
    float ca[3], cb[3];
    // the single-launch iteration (launch_ens_fused)
    int cls;                         // the member's size class (index into the EnsClass array)
    int can_remap;                   // remapping on and room on the stack
    double threshold;                // incomp_threshold
    int n_maps;                      // maps on the stack
    float inv_nf;                    // 1 / N of the fine grid (FP32)
    const float4* stack;             // the stack (n_maps maps of 2 Nc float4)
    float4* push_slot;               // where the advected map goes at a remap
    InitSource src;                  // omega_0 (analytic, or the discrete field's nodes disc)
    const float4* disc;
    unsigned long long stx, sty;     // fixed-point spacing of the fine grid
    float2 scx, scy;                 // fixed-point scale of the domain
    float* real;                     // omega_0 on the fine grid at a remap, then omega on the vort grid
    float2* w1;                      // row spectra (fine grid at a remap, then the psi solve's kept columns)
    float2* w2;                      // the four Hermite spectra (fine grid, then psi grid)
    float4* wfm_out;                 // the fine vorticity nodes a remap writes (= wfm)
};

// the transforms of one size class of the single-launch iteration (group shapes for
// 256-thread blocks, 4 values per thread)
struct EnsClass {
    fft::RadixPlan v_rx, v_ry, p_rx, p_ry, f_rx, f_ry;   // vort, psi, fine grids: rows (n/2), columns
    const float2* v_twx;             // row tables (pass twiddles, then W^k for k <= n)
    const float2* v_twy;             // column tables
    const float2* p_twx;
    const float2* p_twy;
    const float2* f_twx;
    const float2* f_twy;
    long long ld, f_ld;              // row strides of the work arrays: psi solve, fine grid
    int kv, ncols;                   // psi solve: vort-row bins kept, psi columns kept
    int C_p, C_f;                    // columns per group of the column passes (psi, fine)
    int nb_prow, nb_pinv, nb_frow, nb_finv;   // rows per group of the row passes
    int pow2;                        // every length a power of two (else 2^a 3^b)
    int pad_;
};

constexpr int kEnsFusedThreads = 256;
constexpr int kEnsFusedMaxMembers = 512;
constexpr int kEnsFusedMaxWaves = 16;

// state one launch shares between its blocks (zeroed before the launch): the grid barrier,
// one work-queue counter per wave, the members' check results and remap flags
struct EnsShared {
    unsigned int count;              // barrier arrivals
    int status;                      // 0, or 1 + the wave after which a barrier gave up waiting
    int waves;                       // waves the launch ran
    int pad_;
    unsigned int queue[kEnsFusedMaxWaves];
};

struct EnsFusedArgs {
    const EnsMember* mem;
    const EnsClass* cls;
    int M;
    int g;                           // 256-thread tiles per task of the elementwise stages
    int lpn_log2;                    // advection lanes per node (log2)
    int tab_values, work_values;     // dynamic shared memory: tables, then work (float2 units)
    long long wait_limit;            // polls before a grid barrier gives up
    EnsShared* sh;
    unsigned long long* einc;        // M check results (FP64 bits), zeroed before the launch
    int* remapped;                   // M flags, written by the launch
    unsigned long long* prof;        // null, or kProfValues counters the launch adds to (profiling)
    int remaps_only;                 // 1: only the remap stages of the members whose descriptors are active
    int pad_;
};

// profiling counters of the single launch: block cycles and tasks per stage (11 stages),
// block cycles in grid barriers, nanoseconds of each wave (block 0's clock)
enum { kProfStage = 0, kProfTasks = 16, kProfBarrier = 32, kProfWave = 40, kProfValues = 40 + kEnsFusedMaxWaves };

// shared-memory values (float2 units) the tables and the work of one class need
void ens_fused_smem_values(const EnsClass& c, const Grid& gv, const Grid& gp, const Grid& gf, int* tab, int* work);
// every member's whole step (precombination, advection, check, remap decision and remap, psi
// solve, coarse vorticity) in one cooperative launch of `blocks` blocks; TI in {10, 21, 30}; minb
// in {4, 6}: the register budget is that of minb resident blocks per SM (64 or 40 registers)
cudaError_t launch_ens_fused(int TI, int minb, const EnsFusedArgs& a, int blocks, cudaStream_t s);
// resident blocks per SM of the launch of that register budget (0: it cannot run)
int ens_fused_blocks_per_sm(int TI, int minb, const EnsFusedArgs& a);

enum { kEnsAdvect = 0, kEnsIncomp, kEnsSampleVort, kEnsSampleCoarse, kEnsSpec, kEnsNodes, kEnsPrecombine, kEnsKinds };
// one batched launch of kernel kind over the work list cum (M members, cum[M] tiles) with
// blocks persistent blocks; TI / lpn_log2 for the advection
cudaError_t launch_ens(int kind, int TI, const EnsMember* mem, const int* cum, int M, int blocks, int lpn_log2,
                       cudaStream_t s);

}  // namespace cmm

