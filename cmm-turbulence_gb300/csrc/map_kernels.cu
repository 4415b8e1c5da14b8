// map_kernels.cu -- FP64 kernels of the CMM map: identity, GALS advection,
// incompressibility check, stack composition with initial-condition sampling,
// and sampling of the fine vorticity through the current map.
#include <cuda_runtime.h>

#include "init_conditions.cuh"
#include "kernels.hpp"
#include "psi_solve.cuh"

namespace cmm {

// ---------------------------------------------------------------------------
// identity map (k_init_diffeo, src/simulation/cmm-simulation-kernel.cu:27-41)
// ---------------------------------------------------------------------------
__global__ void k_init_map(double* __restrict__ X, double* __restrict__ Y, Grid g)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    int iX = (int)(i % g.NX), iY = (int)(i / g.NX);
    X[i] = g.b0 + iX * g.hx;
    Y[i] = g.b2 + iY * g.hy;
    X[g.N + i] = 1.0; Y[2 * g.N + i] = 1.0;
    X[2 * g.N + i] = 0.0; Y[g.N + i] = 0.0; X[3 * g.N + i] = 0.0; Y[3 * g.N + i] = 0.0;
}

cudaError_t launch_init_map(double* X, double* Y, const Grid& g, cudaStream_t s)
{
    int threads = 256;
    long long blocks = (g.N + threads - 1) / threads;
    k_init_map<<<(unsigned)blocks, threads, 0, s>>>(X, Y, g);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// GALS footpoint weights (src/simulation/cmm-simulation-host.cu:76-90)
// ---------------------------------------------------------------------------
void map_update_coefficients(int order_num, double ep, double coef[4][kMaxFoot], int* nfoot)
{
    double hc[3] = {0, 0, 0};
    switch (order_num) {
        case 2: hc[0] = 3.0 / 8.0; hc[1] = -3.0 / 20.0; hc[2] = 1.0 / 40.0; break;
        case 1: hc[0] = 1.0 / 3.0; hc[1] = -1.0 / 12.0; break;
        default: hc[0] = 1.0 / 4.0; break;
    }
    int n = 4 + 4 * (order_num < 0 ? 0 : order_num > 2 ? 2 : order_num);
    for (int k = 0; k < kMaxFoot; ++k) {
        int r = k / 4;
        double sx = 1 - 2 * ((k / 2) % 2), sy = 1 - 2 * (((k + 1) / 2) % 2), sxy = 1 - 2 * (k % 2);
        bool on = k < n;
        coef[0][k] = on ? hc[r] : 0.0;
        coef[1][k] = on ? hc[r] * sx / ep / double(r + 1) : 0.0;
        coef[2][k] = on ? hc[r] * sy / ep / double(r + 1) : 0.0;
        coef[3][k] = on ? hc[r] * sxy / ep / ep / double(r + 1) / double(r + 1) : 0.0;
    }
    *nfoot = n;
}

// ---------------------------------------------------------------------------
// backward characteristic integrators on the Hermite stream function
// (src/numerical/cmm-timestep.cu: :35-45 euler_exp_b, :66-81 RK2_heun_b,
//  :112-135 adam_bashford_2_pc_b, :175-207 RK3_classical_b, :260-307 RK4_classical_b,
//  :348-374 RK3_optimized_b, :428-466 RK4_optimized_b).  u = (psi_y, -psi_x); psi level 0
// is t_n, level 1 t_{n-1}; L1 / L12 extrapolate the levels to t_{n+1} / t_{n+1/2}.
// ---------------------------------------------------------------------------
template <int L>
__device__ __forceinline__ void vel_comb(const AdvectArgs& a, const double* c, double x, double y, double& kx, double& ky)
{
    double ux[L], uy[L];
    velocity_levels<L>(a.psi, a.gp, x, y, ux, uy);
    kx = c[0] * ux[0];
    ky = c[0] * uy[0];
#pragma unroll
    for (int l = 1; l < L; ++l) { kx = fma(c[l], ux[l], kx); ky = fma(c[l], uy[l], ky); }
}

__device__ __forceinline__ void vel_level(const AdvectArgs& a, int l, double x, double y, double& ux, double& uy)
{
    const double* lv[1] = {a.psi[l]};
    double u1[1], v1[1];
    velocity_levels<1>(lv, a.gp, x, y, u1, v1);
    ux = u1[0];
    uy = v1[0];
}

template <int L, int TI>
__device__ __forceinline__ void integrate_back(const AdvectArgs& a, double x, double y, double& xo, double& yo)
{
    const double dt = a.dt;
    if (TI == 20) {
        // second-order Adams-Bashforth, ten fixed-point sweeps on levels 0 and 1
        double px = x, py = y, ox = x, oy = y, u2x, u2y, ux, uy;
        for (int it = 0; it < 10; ++it) {
            vel_level(a, 1, px, py, u2x, u2y);
            px = ox - dt * u2x;
            py = oy - dt * u2y;
            vel_level(a, 1, px, py, u2x, u2y);
            vel_level(a, 0, ox, oy, ux, uy);
            ox = x - dt * (1.5 * ux - 0.5 * u2x);
            oy = y - dt * (1.5 * uy - 0.5 * u2y);
        }
        xo = ox;
        yo = oy;
        return;
    }
    double k1x, k1y;
    vel_comb<L>(a, a.L1, x, y, k1x, k1y);
    if (TI == 10) {
        xo = x - dt * k1x;
        yo = y - dt * k1y;
    } else if (TI == 21) {
        double k2x, k2y;
        vel_level(a, 0, x - dt * k1x, y - dt * k1y, k2x, k2y);
        xo = x - dt * (k1x + k2x) / 2;
        yo = y - dt * (k1y + k2y) / 2;
    } else if (TI == 30) {
        double k2x, k2y, k3x, k3y;
        vel_comb<L>(a, a.L12, x - dt * k1x / 2.0, y - dt * k1y / 2.0, k2x, k2y);
        vel_level(a, 0, x + dt * k1x - 2 * dt * k2x, y + dt * k1y - 2 * dt * k2y, k3x, k3y);
        xo = x - dt * (k1x + 4 * k2x + k3x) / 6.0;
        yo = y - dt * (k1y + 4 * k2y + k3y) / 6.0;
    } else if (TI == 40) {
        double k2x, k2y, k3x, k3y, k4x, k4y;
        vel_comb<L>(a, a.L12, x - dt * k1x / 2.0, y - dt * k1y / 2.0, k2x, k2y);
        vel_comb<L>(a, a.L12, x - dt * k2x / 2.0, y - dt * k2y / 2.0, k3x, k3y);
        vel_level(a, 0, x - dt * k3x, y - dt * k3y, k4x, k4y);
        xo = x - dt * (k1x + 2 * k2x + 2 * k3x + k4x) / 6.0;
        yo = y - dt * (k1y + 2 * k2y + 2 * k3y + k4y) / 6.0;
    } else if (TI == 31) {
        double k2x, k2y, k3x, k3y;
        vel_level(a, 0, x - dt * k1x, y - dt * k1y, k2x, k2y);
        vel_level(a, 1, x + 2 * dt * (-2 * k1x + k2x), y + 2 * dt * (-2 * k1y + k2y), k3x, k3y);
        xo = x - dt * (5 * k1x + 8 * k2x - k3x) / 12.0;
        yo = y - dt * (5 * k1y + 8 * k2y - k3y) / 12.0;
    } else {   // 41
        double k2x, k2y, k3x, k3y, k4x, k4y;
        vel_level(a, 0, x - dt * k1x, y - dt * k1y, k2x, k2y);
        vel_comb<L>(a, a.L12, x - dt * (3 * k1x + k2x) / 8.0, y - dt * (3 * k1y + k2y) / 8.0, k3x, k3y);
        vel_level(a, 0, x + dt * (k2x - 4 * k3x) / 3.0, y + dt * (k2y - 4 * k3y) / 3.0, k4x, k4y);
        xo = x - dt * (2 * k1x - k2x + 8 * k3x + 3 * k4x) / 12.0;
        yo = y - dt * (2 * k1y - k2y + 8 * k3y + 3 * k4y) / 12.0;
    }
}

// forward integrators for the forward map (src/numerical/cmm-timestep.cu: :26-31
// euler_exp, :48-64 RK2_heun, :84-110 adam_bashford_2_pc, :144-173 RK3_classical,
// :216-258 RK4_classical, :314-339 RK3_optimized, :385-420 RK4_optimized): from the
// footpoint's current position forward over dt.  Kept as the reference has them:
// RK4_classical's first half-step velocity is the t_{n+1} extrapolation and its last
// stage the t_{n+1/2} one, and RK4_optimized is the backward scheme.
template <int L, int TI>
__device__ __forceinline__ void integrate_fwd(const AdvectArgs& a, double x, double y, double& xo, double& yo)
{
    const double dt = a.dt;
    if (TI == 41) { integrate_back<L, 41>(a, x, y, xo, yo); return; }
    if (TI == 20) {
        double px = x, py = y, ox = x, oy = y, u2x, u2y, ux, uy;
        for (int it = 0; it < 10; ++it) {
            vel_level(a, 1, px, py, u2x, u2y);
            px = ox + dt * u2x;
            py = oy + dt * u2y;
            vel_level(a, 1, px, py, u2x, u2y);
            vel_level(a, 0, ox, oy, ux, uy);
            ox = x + dt * (1.5 * ux - 0.5 * u2x);
            oy = y + dt * (1.5 * uy - 0.5 * u2y);
        }
        xo = ox;
        yo = oy;
        return;
    }
    double k1x, k1y;
    vel_level(a, 0, x, y, k1x, k1y);
    if (TI == 10) {
        xo = x + dt * k1x;
        yo = y + dt * k1y;
    } else if (TI == 21) {
        double k2x, k2y;
        vel_comb<L>(a, a.L1, x + dt * k1x, y + dt * k1y, k2x, k2y);
        xo = x + dt * (k1x + k2x) / 2;
        yo = y + dt * (k1y + k2y) / 2;
    } else if (TI == 30) {
        double k2x, k2y, k3x, k3y;
        vel_comb<L>(a, a.L12, x + dt * k1x / 2.0, y + dt * k1y / 2.0, k2x, k2y);
        vel_comb<L>(a, a.L1, x - dt * k1x + 2 * dt * k2x, y - dt * k1y + 2 * dt * k2y, k3x, k3y);
        xo = x + dt * (k1x + 4 * k2x + k3x) / 6.0;
        yo = y + dt * (k1y + 4 * k2y + k3y) / 6.0;
    } else if (TI == 40) {
        double k2x, k2y, k3x, k3y, k4x, k4y;
        vel_comb<L>(a, a.L1, x + dt * k1x / 2.0, y + dt * k1y / 2.0, k2x, k2y);
        vel_comb<L>(a, a.L12, x + dt * k2x / 2.0, y + dt * k2y / 2.0, k3x, k3y);
        vel_comb<L>(a, a.L12, x + dt * k3x, y + dt * k3y, k4x, k4y);
        xo = x + dt * (k1x + 2 * k2x + 2 * k3x + k4x) / 6.0;
        yo = y + dt * (k1y + 2 * k2y + 2 * k3y + k4y) / 6.0;
    } else {   // 31
        double k2x, k2y, k3x, k3y;
        vel_level(a, 1, x - dt * k1x, y - dt * k1y, k2x, k2y);
        vel_level(a, 2, x - dt * (8 * k1x + 2 * k2x) / 5.0, y - dt * (8 * k1y + 2 * k2y) / 5.0, k3x, k3y);
        xo = x + dt * (23 * k1x - 16 * k2x + 5 * k3x) / 12.0;
        yo = y + dt * (23 * k1y - 16 * k2y + 5 * k3y) / 12.0;
    }
}

// One lane per (node, footpoint); LPN lanes per node (power of two >= nfoot).
// Lanes 0..7 of each group combine the footpoints into the 8 output planes
// [X, X_x, X_y, X_xy, Y, Y_x, Y_y, Y_xy] with the same sequential
// multiply-add order as the reference's accumulation (:280-289).
template <int L, int TI, bool FWD>
__global__ void __launch_bounds__(256) k_advect(const AdvectArgs a, int lpn_log2)
{
    __shared__ double sc[4][kMaxFoot];
    if (threadIdx.x < 4 * kMaxFoot) sc[threadIdx.x / kMaxFoot][threadIdx.x % kMaxFoot] =
        a.coef[threadIdx.x / kMaxFoot][threadIdx.x % kMaxFoot];
    __syncthreads();

    const int lpn = 1 << lpn_log2;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long node = t >> lpn_log2;
    int k = (int)(t & (lpn - 1));
    bool live = node < a.gm.N;
    long long nd = live ? node : 0;
    int iX = (int)(nd % a.gm.NX), iY = (int)(nd / a.gm.NX);

    double xf = 0.0, yf = 0.0;
    if (live && k < a.nfoot) {
        double r = (double)((k >> 2) + 1) * a.ep;
        double x = a.gm.b0 + iX * a.gm.hx + r * (1 - 2 * ((k >> 1) & 1));
        double y = a.gm.b2 + iY * a.gm.hy + r * (1 - 2 * (((k + 1) >> 1) & 1));
        if (FWD) {
            // forward map: the footpoint's image under the map, carried forward over dt
            double mx, my;
            map_value(a.ChiX, a.ChiY, a.gm, x, y, mx, my);
            integrate_fwd<L, TI>(a, mx, my, xf, yf);
        } else {
            // backward map: the footpoint carried back over dt, then looked up in the map
            double xb, yb;
            integrate_back<L, TI>(a, x, y, xb, yb);
            map_value(a.ChiX, a.ChiY, a.gm, xb, yb, xf, yf);
        }
    }
    // gather the footpoints of this node in every lane of the group
    const int comp = (k >> 2) & 1, plane = k & 3;
    double acc = 0.0;
    for (int kk = 0; kk < a.nfoot; ++kk) {
        double vx = __shfl_sync(0xffffffffu, xf, kk, lpn);
        double vy = __shfl_sync(0xffffffffu, yf, kk, lpn);
        acc = fma(comp ? vy : vx, sc[plane][kk], acc);
    }
    if (live && k < 8) {
        double* out = comp ? a.outY : a.outX;
        out[plane * a.gm.N + node] = acc;
    }
}

cudaError_t launch_advect(const AdvectArgs& a, cudaStream_t s)
{
    int lpn_log2 = a.nfoot <= 4 ? 3 : a.nfoot <= 8 ? 3 : 4;   // >= 8 lanes so lanes 0..7 can store
    int lpn = 1 << lpn_log2;
    long long total = a.gm.N * lpn;
    int threads = 256;
    unsigned blocks = (unsigned)((total + threads - 1) / threads);
#define CMM_ADV(LL, TT)                                                          \
    do {                                                                          \
        if (a.direction == 1) k_advect<LL, TT, true><<<blocks, threads, 0, s>>>(a, lpn_log2);   \
        else k_advect<LL, TT, false><<<blocks, threads, 0, s>>>(a, lpn_log2);     \
    } while (0)
    switch (a.time_integration_num * 10 + a.l_order) {
        case 101: CMM_ADV(1, 10); break;
        case 102: CMM_ADV(2, 10); break;
        case 103: CMM_ADV(3, 10); break;
        case 104: CMM_ADV(4, 10); break;
        case 211: CMM_ADV(1, 21); break;
        case 212: CMM_ADV(2, 21); break;
        case 213: CMM_ADV(3, 21); break;
        case 214: CMM_ADV(4, 21); break;
        case 301: CMM_ADV(1, 30); break;
        case 302: CMM_ADV(2, 30); break;
        case 303: CMM_ADV(3, 30); break;
        case 304: CMM_ADV(4, 30); break;
        case 202: CMM_ADV(2, 20); break;
        case 203: CMM_ADV(3, 20); break;
        case 204: CMM_ADV(4, 20); break;
        case 404: CMM_ADV(4, 40); break;
        case 313: CMM_ADV(3, 31); break;
        case 314: CMM_ADV(4, 31); break;
        case 414: CMM_ADV(4, 41); break;
        default: return cudaErrorInvalidValue;
    }
#undef CMM_ADV
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// incompressibility: max |1 - det grad X| over the check grid, points shifted
// by half a check cell (k_incompressibility_check + thrust max,
// src/simulation/cmm-simulation-kernel.cu:159-173, cmm-simulation-host.cu:44-50)
// fused with a warp-shuffle max and one atomic per block.  |1-det| >= 0, so
// the IEEE bit pattern orders like the value and atomicMax on it is exact.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_incomp(Grid gc, Grid gm, const double* __restrict__ X,
                                                const double* __restrict__ Y, unsigned long long* result)
{
    __shared__ unsigned long long wmax[8];
    unsigned long long best = 0ull;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < gc.N;
         i += (long long)gridDim.x * blockDim.x) {
        int iX = (int)(i % gc.NX), iY = (int)(i / gc.NX);
        double x = gm.b0 + iX * gc.hx + 0.5 * gc.hx;
        double y = gm.b2 + iY * gc.hy + 0.5 * gc.hy;
        double d = fabs(1.0 - map_det(X, Y, gm, x, y));
        unsigned long long b = (unsigned long long)__double_as_longlong(d);
        best = b > best ? b : best;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long v = __shfl_xor_sync(0xffffffffu, best, o);
        best = v > best ? v : best;
    }
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = wmax[w] > m ? wmax[w] : m;
        atomicMax(result, m);
    }
}

// max over the half-shifted check grid of |x - X_b(X_f(x))| (k_invertibility_check,
// src/simulation/cmm-simulation-kernel.cu:177-198), fused with its reduction
__global__ void __launch_bounds__(256) k_invert(Grid gc, Grid gm, const double* __restrict__ Xb,
                                                const double* __restrict__ Yb, const double* __restrict__ Xf,
                                                const double* __restrict__ Yf, unsigned long long* result)
{
    __shared__ unsigned long long wmax[8];
    unsigned long long best = 0ull;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < gc.N;
         i += (long long)gridDim.x * blockDim.x) {
        int iX = (int)(i % gc.NX), iY = (int)(i / gc.NX);
        double x = gc.b0 + iX * gc.hx + 0.5 * gc.hx;
        double y = gc.b2 + iY * gc.hy + 0.5 * gc.hy;
        double a, b, c, d;
        map_value(Xf, Yf, gm, x, y, a, b);
        map_value(Xb, Yb, gm, a, b, c, d);
        double e = hypot(x - c, y - d);
        unsigned long long v = (unsigned long long)__double_as_longlong(e);
        best = v > best ? v : best;
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long v = __shfl_xor_sync(0xffffffffu, best, o);
        best = v > best ? v : best;
    }
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = wmax[w] > m ? wmax[w] : m;
        atomicMax(result, m);
    }
}

cudaError_t launch_invert(const Grid& gc, const Grid& gm, const double* Xb, const double* Yb, const double* Xf,
                          const double* Yf, double* d_result, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(d_result, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    long long need = (gc.N + 255) / 256;
    unsigned blocks = (unsigned)(need < 152 * 16 ? need : 152 * 16);
    k_invert<<<blocks, 256, 0, s>>>(gc, gm, Xb, Yb, Xf, Yf, reinterpret_cast<unsigned long long*>(d_result));
    return cudaGetLastError();
}

cudaError_t launch_incomp(const Grid& gc, const Grid& gm, const double* X, const double* Y, double* d_result,
                          cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(d_result, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    int threads = 256;
    long long need = (gc.N + threads - 1) / threads;
    unsigned blocks = (unsigned)(need < 152 * 16 ? need : 152 * 16);
    k_incomp<<<blocks, threads, 0, s>>>(gc, gm, X, Y, reinterpret_cast<unsigned long long*>(d_result));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// stack composition + initial-condition sampling, fused: every target point
// chases its footpoint through the current map and all stacked maps in
// registers, instead of one launch and one HBM round trip of (x, y) per map.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_compose_sample(Grid gm, Grid gt, const double* __restrict__ X,
                                                        const double* __restrict__ Y,
                                                        const double* __restrict__ stack, int n_maps,
                                                        InitSource src, double* __restrict__ out)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= gt.N) return;
    int iX = (int)(i % gt.NX), iY = (int)(i / gt.NX);
    double x = gt.b0 + iX * gt.hx, y = gt.b2 + iY * gt.hy;
    double xo, yo;
    map_value(X, Y, gm, x, y, xo, yo);
    x = wrap(xo, gm.b0, gm.Wx);
    y = wrap(yo, gm.b2, gm.Wy);
    for (int m = n_maps - 1; m >= 0; --m) {
        const double* MX = stack + (long long)m * 8 * gm.N;
        map_value(MX, MX + 4 * gm.N, gm, x, y, xo, yo);
        x = wrap(xo, gm.b0, gm.Wx);
        y = wrap(yo, gm.b2, gm.Wy);
    }
    double v;
    if (src.kind == 3) v = interp_value(src.discrete, src.gd, x, y);
    else v = init_field(src.kind, x, y, src.ic_num, src.params, src.rand_table);
    out[i] = v;
}

cudaError_t launch_compose_sample(const Grid& gm, const Grid& gt, const double* X, const double* Y,
                                  const double* stack, int n_maps, const InitSource& src, double* out,
                                  cudaStream_t s)
{
    int threads = 256;
    unsigned blocks = (unsigned)((gt.N + threads - 1) / threads);
    k_compose_sample<<<blocks, threads, 0, s>>>(gm, gt, X, Y, stack, n_maps, src, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// vorticity through the current map (k_apply_map_and_sample_from_hermite)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double sample_vort_point(const Grid& gm, const Grid& go, const Grid& gf,
                                                   const double* __restrict__ X, const double* __restrict__ Y,
                                                   const double* __restrict__ Wf, int molly, int iX, int iY)
{
    double x = gm.b0 + iX * go.hx, y = gm.b2 + iY * go.hy;
    double x2, y2, v;
    if (molly == 4) {
        // reference stencil; its x offset term evaluates to zero (operator
        // precedence of `i>>1+1`), kept for identical results
        map_value(X, Y, gm, x, y, x2, y2);
        v = interp_value(Wf, gf, x2, y2) / 3.0;
        for (int m = 0; m < 4; ++m) {
            double xs = x + go.hx / 2.0 * ((m >> 2) & 1) * (-1 + 2 * (m & 1));
            double ys = y + go.hy / 2.0 * ((m >> 1) & 1) * (-1 + 2 * (m & 1));
            map_value(X, Y, gm, xs, ys, x2, y2);
            v += interp_value(Wf, gf, x2, y2) / 6.0;
        }
    } else if (molly == 8) {
        v = 0.0;
        for (int m = 0; m < 9; ++m) {
            double xs = x + go.hx * (-1 + m % 3) / 2.0;
            double ys = y + go.hy * (-1 + m / 3) / 2.0;
            map_value(X, Y, gm, xs, ys, x2, y2);
            // reference weights ((1 + m%3) & 1) * ((1 + m/3) & 1), kept for identical results
            v += ((1 + (m % 3)) & 1) * ((1 + (m / 3)) & 1) * interp_value(Wf, gf, x2, y2) / 16.0;
        }
    } else {
        map_value(X, Y, gm, x, y, x2, y2);
        v = interp_value(Wf, gf, x2, y2);
    }
    return v;
}

__global__ void __launch_bounds__(256) k_sample_vort(Grid gm, Grid go, Grid gf, const double* __restrict__ X,
                                                     const double* __restrict__ Y, const double* __restrict__ Wf,
                                                     int molly, double* __restrict__ out, long long ld)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= go.N) return;
    int iX = (int)(i % go.NX), iY = (int)(i / go.NX);
    out[(long long)iY * ld + iX] = sample_vort_point(gm, go, gf, X, Y, Wf, molly, iX, iY);
}

cudaError_t launch_sample_vort(const Grid& gm, const Grid& go, const Grid& gf, const double* X, const double* Y,
                               const double* Wf, int molly, double* out, long long ld, cudaStream_t s)
{
    int threads = 256;
    unsigned blocks = (unsigned)((go.N + threads - 1) / threads);
    k_sample_vort<<<blocks, threads, 0, s>>>(gm, go, gf, X, Y, Wf, molly, out, ld);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// the psi solve of the plain form on the library's FFT (psi_solve.cuh): omega through
// the map on the vorticity grid (k_sample_vort), the kept modes, the four psi planes
// ---------------------------------------------------------------------------
struct PlanesEpi {
    int nx;
    long long n;
    double* out;
    __device__ __forceinline__ void store(int iX, int iY, double f, double fx, double fy, double fxy) const
    {
        const long long i = (long long)iY * nx + iX;
        out[i] = f;
        out[n + i] = fx;
        out[2 * n + i] = fy;
        out[3 * n + i] = fxy;
    }
};

bool psi_solve_fits(const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv, const fft::Plan2D& pp,
                    long long* w1_values, long long* w2_values)
{
    const psi::Layout L = psi::make_layout<double>(gv, gp, freq, pv, pp);
    if (!L.ok) return false;
    if (w1_values) *w1_values = L.w1_values;
    if (w2_values) *w2_values = L.w2_values;
    return true;
}

void psi_solve_prepare()
{
    psi::prepare<double, PlanesEpi>();
}

cudaError_t launch_psi_solve(const Grid& gm, const Grid& gv, const Grid& gf, const double* X, const double* Y,
                             const double* Wf, int molly, const Grid& gp, double freq, const fft::Plan2D& pv,
                             const fft::Plan2D& pp, double* omega, double2* w1, double2* w2, double* psi_out,
                             cudaStream_t s)
{
    const psi::Layout L = psi::make_layout<double>(gv, gp, freq, pv, pp);
    if (!L.ok) return cudaErrorInvalidValue;
    cudaError_t e = launch_sample_vort(gm, gv, gf, X, Y, Wf, molly, omega, gv.NX, s);
    if (e != cudaSuccess) return e;
    PlanesEpi epi{gp.NX, gp.N, psi_out};
    return psi::launch<double>(L, gv, gp, freq, pv, pp, omega, w1, w2, epi, s);
}

}  // namespace cmm
