// mixed_kernels.cu -- the mixed-precision form of the CMM step (sm_103a).
//
// Maps are stored and interpolated as FP32 displacements d = X - x (periodic,
// so the reference's wrap jumps vanish), node-interleaved:
//   MapNode = {a = (dX, dY, dX_x, dY_x), b = (dX_y, dY_y, dX_xy, dY_xy)}   (32 B)
// with dX_x = X_x - 1, dY_y = Y_y - 1.  The stream function and the fine
// vorticity are FP32 Hermite nodes (f, f_x, f_y, f_xy) in one float4.
// Positions are reconstructed without FP32 cancellation: GALS footpoints are
// integer node + FP32 offset, corner values are taken relative to the node
// (map) or to a cell corner (velocity), so the 1/eps and 1/eps^2 GALS stencil
// only amplifies rounding of small quantities.  FP64 is kept in the remap-time
// composition (positions accumulated in FP64 through the whole stack), in the
// Jacobian-determinant deviation, and in the diagnostics' sums.
#include <cuda_runtime.h>

#include "init_conditions.cuh"
#include "mixed.hpp"

namespace cmm {

// ---------------------------------------------------------------------------
// FP32 Hermite helpers
// ---------------------------------------------------------------------------
struct W4f { float w0, w1, w2, w3; };

__device__ __forceinline__ W4f value_weights_f(float t, float h)
{
    float s = 1.0f - t, t2 = t * t, s2 = s * s;
    W4f w;
    w.w0 = s2 * fmaf(2.0f, t, 1.0f);
    w.w1 = t2 * fmaf(-2.0f, t, 3.0f);
    w.w2 = (t * s2) * h;
    w.w3 = -(s * t2) * h;
    return w;
}

__device__ __forceinline__ W4f slope_weights_f(float t, float ih)
{
    float s = 1.0f - t, st6 = 6.0f * s * t * ih;
    W4f w;
    w.w0 = -st6;
    w.w1 = st6;
    w.w2 = s * fmaf(3.0f, s, -2.0f);
    w.w3 = t * fmaf(3.0f, t, -2.0f);
    return w;
}

struct CellF {
    int i00, i10, i01, i11;
    float tx, ty;
};

__device__ __forceinline__ int wrap_index(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

// cell of the point (bx*h + ox, by*h + oy): integer base cell + FP32 offset
__device__ __forceinline__ CellF locate_rel(const Grid& g, int bx, int by, float ox, float oy)
{
    float qx = ox * (float)g.ihx, qy = oy * (float)g.ihy;
    float fx = floorf(qx), fy = floorf(qy);
    CellF c;
    c.tx = qx - fx;
    c.ty = qy - fy;
    int ix0 = wrap_index(bx + (int)fx, g.NX), iy0 = wrap_index(by + (int)fy, g.NY);
    int ix1 = ix0 + 1 == g.NX ? 0 : ix0 + 1, iy1 = iy0 + 1 == g.NY ? 0 : iy0 + 1;
    c.i00 = iy0 * g.NX + ix0; c.i10 = iy0 * g.NX + ix1;
    c.i01 = iy1 * g.NX + ix0; c.i11 = iy1 * g.NX + ix1;
    return c;
}

// cell of an absolute FP64 position; the fraction is rounded to FP32 once
__device__ __forceinline__ CellF locate_abs(const Grid& g, double x, double y)
{
    double qx = (x - g.b0) * g.ihx, qy = (y - g.b2) * g.ihy;
    double fx = floor(qx), fy = floor(qy);
    CellF c;
    c.tx = (float)(qx - fx);
    c.ty = (float)(qy - fy);
    int ix0 = wrap_index((int)fx, g.NX), iy0 = wrap_index((int)fy, g.NY);
    int ix1 = ix0 + 1 == g.NX ? 0 : ix0 + 1, iy1 = iy0 + 1 == g.NY ? 0 : iy0 + 1;
    c.i00 = iy0 * g.NX + ix0; c.i10 = iy0 * g.NX + ix1;
    c.i01 = iy1 * g.NX + ix0; c.i11 = iy1 * g.NX + ix1;
    return c;
}

// one Hermite component at 4 corners: (f, f_x, f_y, f_xy) per corner
struct Q4 { float4 c00, c10, c01, c11; };

__device__ __forceinline__ void xrow_f(const W4f& w, const float4& a, const float4& b, float& s, float& t)
{
    s = fmaf(w.w3, b.y, fmaf(w.w2, a.y, fmaf(w.w1, b.x, w.w0 * a.x)));
    t = fmaf(w.w3, b.w, fmaf(w.w2, a.w, fmaf(w.w1, b.z, w.w0 * a.z)));
}

__device__ __forceinline__ float ycomb_f(const W4f& w, float s0, float s1, float t0, float t1)
{
    return fmaf(w.w3, t1, fmaf(w.w2, t0, fmaf(w.w1, s1, w.w0 * s0)));
}

__device__ __forceinline__ float herm_value_f(const Q4& q, const W4f& wx, const W4f& wy)
{
    float s0, t0, s1, t1;
    xrow_f(wx, q.c00, q.c10, s0, t0);
    xrow_f(wx, q.c01, q.c11, s1, t1);
    return ycomb_f(wy, s0, s1, t0, t1);
}

__device__ __forceinline__ void herm_grad_f(const Q4& q, const W4f& wx, const W4f& wy, const W4f& dx, const W4f& dy,
                                            float& gx, float& gy)
{
    float s0, t0, s1, t1, ds0, dt0, ds1, dt1;
    xrow_f(wx, q.c00, q.c10, s0, t0);
    xrow_f(wx, q.c01, q.c11, s1, t1);
    xrow_f(dx, q.c00, q.c10, ds0, dt0);
    xrow_f(dx, q.c01, q.c11, ds1, dt1);
    gx = ycomb_f(wy, ds0, ds1, dt0, dt1);
    gy = ycomb_f(dy, s0, s1, t0, t1);
}

// velocity (psi_y, -psi_x) of an FP32 Hermite stream function at a cell; the
// value plane is taken relative to the cell's first corner (slope weights sum
// to zero), so psi's magnitude does not cost precision in its gradient
__device__ __forceinline__ void velocity_f(const float4* __restrict__ P, const Grid& g, const CellF& c,
                                           float& ux, float& uy)
{
    Q4 q;
    q.c00 = __ldg(P + c.i00); q.c10 = __ldg(P + c.i10); q.c01 = __ldg(P + c.i01); q.c11 = __ldg(P + c.i11);
    float ref = q.c00.x;
    q.c00.x = 0.0f; q.c10.x -= ref; q.c01.x -= ref; q.c11.x -= ref;
    W4f wx = value_weights_f(c.tx, (float)g.hx), wy = value_weights_f(c.ty, (float)g.hy);
    W4f dx = slope_weights_f(c.tx, (float)g.ihx), dy = slope_weights_f(c.ty, (float)g.ihy);
    float gx, gy;
    herm_grad_f(q, wx, wy, dx, dy, gx, gy);
    ux = gy;
    uy = -gx;
}

// map displacement at a cell, X and Y components, corner values minus (rx, ry)
__device__ __forceinline__ void map_disp_f(const float4* __restrict__ M, const Grid& g, const CellF& c, float rx,
                                           float ry, float& dxo, float& dyo)
{
    float4 a00 = __ldg(M + 2 * c.i00), b00 = __ldg(M + 2 * c.i00 + 1);
    float4 a10 = __ldg(M + 2 * c.i10), b10 = __ldg(M + 2 * c.i10 + 1);
    float4 a01 = __ldg(M + 2 * c.i01), b01 = __ldg(M + 2 * c.i01 + 1);
    float4 a11 = __ldg(M + 2 * c.i11), b11 = __ldg(M + 2 * c.i11 + 1);
    W4f wx = value_weights_f(c.tx, (float)g.hx), wy = value_weights_f(c.ty, (float)g.hy);
    Q4 q;
    q.c00 = make_float4(a00.x - rx, a00.z, b00.x, b00.z);
    q.c10 = make_float4(a10.x - rx, a10.z, b10.x, b10.z);
    q.c01 = make_float4(a01.x - rx, a01.z, b01.x, b01.z);
    q.c11 = make_float4(a11.x - rx, a11.z, b11.x, b11.z);
    dxo = herm_value_f(q, wx, wy);
    q.c00 = make_float4(a00.y - ry, a00.w, b00.y, b00.w);
    q.c10 = make_float4(a10.y - ry, a10.w, b10.y, b10.w);
    q.c01 = make_float4(a01.y - ry, a01.w, b01.y, b01.w);
    q.c11 = make_float4(a11.y - ry, a11.w, b11.y, b11.w);
    dyo = herm_value_f(q, wx, wy);
}

// ---------------------------------------------------------------------------
// identity map and Lagrange pre-combination
// ---------------------------------------------------------------------------
cudaError_t launch_init_map_m(float4* map, const Grid& g, cudaStream_t s)
{
    return cudaMemsetAsync(map, 0, sizeof(float4) * 2 * (size_t)g.N, s);
}

__global__ void k_precombine(const float4* __restrict__ p0, const float4* __restrict__ p1,
                             const float4* __restrict__ p2, const float4* __restrict__ p3, long long n, int L,
                             float4 cA, float4 cB, float4* __restrict__ outA, float4* __restrict__ outB)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ca[4] = {cA.x, cA.y, cA.z, cA.w}, cb[4] = {cB.x, cB.y, cB.z, cB.w};
    const float4* lv[4] = {p0, p1, p2, p3};
    float4 a = make_float4(0, 0, 0, 0), b = make_float4(0, 0, 0, 0);
    for (int l = 0; l < L; ++l) {
        float4 v = __ldg(lv[l] + i);
        a.x = fmaf(ca[l], v.x, a.x); a.y = fmaf(ca[l], v.y, a.y); a.z = fmaf(ca[l], v.z, a.z); a.w = fmaf(ca[l], v.w, a.w);
        if (outB) { b.x = fmaf(cb[l], v.x, b.x); b.y = fmaf(cb[l], v.y, b.y); b.z = fmaf(cb[l], v.z, b.z); b.w = fmaf(cb[l], v.w, b.w); }
    }
    outA[i] = a;
    if (outB) outB[i] = b;
}

cudaError_t launch_precombine(float4* const* levels, int L, const double* cA, const double* cB, long long n,
                              float4* outA, float4* outB, cudaStream_t s)
{
    float4 a = make_float4(0, 0, 0, 0), b = make_float4(0, 0, 0, 0);
    float* pa = &a.x;
    float* pb = &b.x;
    for (int l = 0; l < L && l < 4; ++l) { pa[l] = (float)cA[l]; if (cB) pb[l] = (float)cB[l]; }
    const float4* lv[4] = {levels[0], L > 1 ? levels[1] : levels[0], L > 2 ? levels[2] : levels[0],
                           L > 3 ? levels[3] : levels[0]};
    k_precombine<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(lv[0], lv[1], lv[2], lv[3], n, L, a, b, outA, outB);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// GALS map advection in displacement form.  One lane per (node, footpoint),
// 8 (or 16) lanes per node.  For footpoint k at node offset e_k:
//   Delta_k = RK displacement of the backward characteristic,
//   g_k     = [d(x_f) - d(node)] - Delta_k          (x_f = node + e_k - Delta_k)
// new map:  d = d(node) + sum c1 g,  d_x = sum cx g,  d_y = sum cy g,  d_xy = sum cxy g
// (the identity parts sum c1 e = 0, sum cx e_x = 1, ... are applied exactly).
// ---------------------------------------------------------------------------
template <int TI>
__global__ void __launch_bounds__(256) k_advect_m(const AdvectMArgs a, int lpn_log2)
{
    __shared__ float sc[4][kMaxFoot];
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
    float4 n0 = __ldg(a.map + 2 * nd);     // (dX, dY, dX_x, dY_x) at the node
    float gX = 0.0f, gY = 0.0f;
    if (live && k < a.nfoot) {
        float r = (float)((k >> 2) + 1) * a.ep;
        float ex = r * (float)(1 - 2 * ((k >> 1) & 1));
        float ey = r * (float)(1 - 2 * (((k + 1) >> 1) & 1));
        const int bx = iX * a.rp, by = iY * a.rp;
        const float dt = a.dt;
        float k1x, k1y, Dx, Dy;
        velocity_f(a.psiA, a.gp, locate_rel(a.gp, bx, by, ex, ey), k1x, k1y);
        if (TI == 10) {
            Dx = dt * k1x;
            Dy = dt * k1y;
        } else if (TI == 21) {
            float k2x, k2y;
            velocity_f(a.psi0, a.gp, locate_rel(a.gp, bx, by, ex - dt * k1x, ey - dt * k1y), k2x, k2y);
            Dx = dt * (k1x + k2x) * 0.5f;
            Dy = dt * (k1y + k2y) * 0.5f;
        } else {
            float k2x, k2y, k3x, k3y;
            velocity_f(a.psiB, a.gp, locate_rel(a.gp, bx, by, ex - 0.5f * dt * k1x, ey - 0.5f * dt * k1y), k2x, k2y);
            velocity_f(a.psi0, a.gp,
                       locate_rel(a.gp, bx, by, ex + dt * k1x - 2.0f * dt * k2x, ey + dt * k1y - 2.0f * dt * k2y), k3x, k3y);
            Dx = dt * (k1x + 4.0f * k2x + k3x) * (1.0f / 6.0f);
            Dy = dt * (k1y + 4.0f * k2y + k3y) * (1.0f / 6.0f);
        }
        float fx = ex - Dx, fy = ey - Dy;
        float mx, my;
        map_disp_f(a.map, a.gm, locate_rel(a.gm, iX, iY, fx, fy), n0.x, n0.y, mx, my);
        gX = mx - Dx;
        gY = my - Dy;
    }
    const int comp = k & 1, plane = (k >> 1) & 3;
    float acc = 0.0f;
    for (int kk = 0; kk < a.nfoot; ++kk) {
        float vx = __shfl_sync(0xffffffffu, gX, kk, lpn);
        float vy = __shfl_sync(0xffffffffu, gY, kk, lpn);
        acc = fmaf(comp ? vy : vx, sc[plane][kk], acc);
    }
    if (live && k < 8) {
        if (plane == 0) acc += comp ? n0.y : n0.x;
        reinterpret_cast<float*>(a.out)[8 * node + k] = acc;
    }
}

cudaError_t launch_advect_m(const AdvectMArgs& a, cudaStream_t s)
{
    int lpn_log2 = a.nfoot <= 8 ? 3 : 4;
    long long total = a.gm.N << lpn_log2;
    unsigned blocks = (unsigned)((total + 255) / 256);
    switch (a.time_integration_num) {
        case 10: k_advect_m<10><<<blocks, 256, 0, s>>>(a, lpn_log2); break;
        case 21: k_advect_m<21><<<blocks, 256, 0, s>>>(a, lpn_log2); break;
        case 30: k_advect_m<30><<<blocks, 256, 0, s>>>(a, lpn_log2); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// incompressibility: one thread per (coarse cell, check row).  The slopes of
// the displacement are interpolated in FP32; the deviation of the Jacobian
// determinant  det - 1 = a + b + a*b - c*e  (a = dX_x, b = dY_y, c = dX_y,
// e = dY_x) is formed and maximised in FP64.  Check points are the fine grid
// shifted by half a fine cell (k_incompressibility_check), r = Nf / Nc per cell.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_incomp_m(Grid gm, int r, const float4* __restrict__ M,
                                                  unsigned long long* result)
{
    __shared__ unsigned long long wmax[8];
    unsigned long long best = 0ull;
    long long total = gm.N * r;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        int sub_y = (int)(i % r);
        long long cell = i / r;
        int cx = (int)(cell % gm.NX), cy = (int)(cell / gm.NX);
        int cx1 = cx + 1 == gm.NX ? 0 : cx + 1, cy1 = cy + 1 == gm.NY ? 0 : cy + 1;
        long long i00 = (long long)cy * gm.NX + cx, i10 = (long long)cy * gm.NX + cx1;
        long long i01 = (long long)cy1 * gm.NX + cx, i11 = (long long)cy1 * gm.NX + cx1;
        float4 a00 = __ldg(M + 2 * i00), b00 = __ldg(M + 2 * i00 + 1);
        float4 a10 = __ldg(M + 2 * i10), b10 = __ldg(M + 2 * i10 + 1);
        float4 a01 = __ldg(M + 2 * i01), b01 = __ldg(M + 2 * i01 + 1);
        float4 a11 = __ldg(M + 2 * i11), b11 = __ldg(M + 2 * i11 + 1);
        // value planes relative to corner 00: slope weights sum to zero, so the
        // gradient is unchanged and FP32 keeps the precision of the differences
        Q4 qX, qY;
        qX.c00 = make_float4(0.0f, a00.z, b00.x, b00.z); qY.c00 = make_float4(0.0f, a00.w, b00.y, b00.w);
        qX.c10 = make_float4(a10.x - a00.x, a10.z, b10.x, b10.z); qY.c10 = make_float4(a10.y - a00.y, a10.w, b10.y, b10.w);
        qX.c01 = make_float4(a01.x - a00.x, a01.z, b01.x, b01.z); qY.c01 = make_float4(a01.y - a00.y, a01.w, b01.y, b01.w);
        qX.c11 = make_float4(a11.x - a00.x, a11.z, b11.x, b11.z); qY.c11 = make_float4(a11.y - a00.y, a11.w, b11.y, b11.w);
        float ty = ((float)sub_y + 0.5f) / (float)r;
        W4f wy = value_weights_f(ty, (float)gm.hy), dy = slope_weights_f(ty, (float)gm.ihy);
        for (int sx = 0; sx < r; ++sx) {
            float tx = ((float)sx + 0.5f) / (float)r;
            W4f wx = value_weights_f(tx, (float)gm.hx), dx = slope_weights_f(tx, (float)gm.ihx);
            float Xx, Xy, Yx, Yy;
            herm_grad_f(qX, wx, wy, dx, dy, Xx, Xy);
            herm_grad_f(qY, wx, wy, dx, dy, Yx, Yy);
            double A = Xx, B = Yy, Cc = Xy, E = Yx;
            double dev = fabs(A + B + A * B - Cc * E);
            unsigned long long bits = (unsigned long long)__double_as_longlong(dev);
            best = bits > best ? bits : best;
        }
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

cudaError_t launch_incomp_m(const Grid& gm, int r, const float4* map, double* d_result, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(d_result, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    long long total = gm.N * r;
    long long need = (total + 255) / 256;
    unsigned blocks = (unsigned)(need < 152 * 8 ? need : 152 * 8);
    k_incomp_m<<<blocks, 256, 0, s>>>(gm, r, map, reinterpret_cast<unsigned long long*>(d_result));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// remap-time composition with FP64 positions: every target point is chased
// through the current map and all stacked maps (x <- x + d(x)); the FP32
// displacement is added to the FP64 position once per map
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_compose_m(Grid gm, Grid gt, const float4* __restrict__ map,
                                                   const float4* __restrict__ stack, int n_maps, InitSource src,
                                                   double* __restrict__ out)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= gt.N) return;
    int iX = (int)(i % gt.NX), iY = (int)(i / gt.NX);
    double x = gt.b0 + iX * gt.hx, y = gt.b2 + iY * gt.hy;
    float dx, dy;
    map_disp_f(map, gm, locate_abs(gm, x, y), 0.0f, 0.0f, dx, dy);
    x += (double)dx;
    y += (double)dy;
    for (int m = n_maps - 1; m >= 0; --m) {
        map_disp_f(stack + 2 * (long long)m * gm.N, gm, locate_abs(gm, x, y), 0.0f, 0.0f, dx, dy);
        x += (double)dx;
        y += (double)dy;
    }
    x = wrap(x, gm.b0, gm.Wx);
    y = wrap(y, gm.b2, gm.Wy);
    double v;
    if (src.kind == 3) v = interp_value(src.discrete, src.gd, x, y);
    else if (src.kind == 1) v = init_scalar(x, y, src.ic_num);
    else v = init_vorticity(x, y, src.ic_num, src.params, src.rand_table);
    out[i] = v;
}

cudaError_t launch_compose_m(const Grid& gm, const Grid& gt, const float4* map, const float4* stack, int n_maps,
                             const InitSource& src, double* out, cudaStream_t s)
{
    k_compose_m<<<(unsigned)((gt.N + 255) / 256), 256, 0, s>>>(gm, gt, map, stack, n_maps, src, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// omega(x) = W(x + d(x)) on an output grid whose spacing divides the map's and
// the fine grid's (integer ratios): positions are integer node + FP32 offset
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_sample_m(Grid gm, Grid go, Grid gf, int ro, int rf,
                                                  const float4* __restrict__ map, const float4* __restrict__ W,
                                                  T* __restrict__ out)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= go.N) return;
    int iX = (int)(i % go.NX), iY = (int)(i / go.NX);
    // position on the map grid: node (iX / ro) + fraction (iX % ro) / ro
    int mx = iX / ro, my = iY / ro;
    float ox = (float)(iX - mx * ro) * (float)go.hx, oy = (float)(iY - my * ro) * (float)go.hy;
    float dx, dy;
    map_disp_f(map, gm, locate_rel(gm, mx, my, ox, oy), 0.0f, 0.0f, dx, dy);
    // on the fine grid the output point is node iX * rf
    CellF c = locate_rel(gf, iX * rf, iY * rf, dx, dy);
    Q4 q;
    q.c00 = __ldg(W + c.i00); q.c10 = __ldg(W + c.i10); q.c01 = __ldg(W + c.i01); q.c11 = __ldg(W + c.i11);
    float v = herm_value_f(q, value_weights_f(c.tx, (float)gf.hx), value_weights_f(c.ty, (float)gf.hy));
    out[i] = (T)v;
}

cudaError_t launch_sample_m(const Grid& gm, const Grid& go, const Grid& gf, const float4* map, const float4* W,
                            float* out_f, double* out_d, cudaStream_t s)
{
    int ro = go.NX / gm.NX, rf = gf.NX / go.NX;
    unsigned blocks = (unsigned)((go.N + 255) / 256);
    if (out_f) k_sample_m<float><<<blocks, 256, 0, s>>>(gm, go, gf, ro, rf, map, W, out_f);
    else k_sample_m<double><<<blocks, 256, 0, s>>>(gm, go, gf, ro, rf, map, W, out_d);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// tracers: FP64 positions, FP32 velocities (psiA = level 1 = t_n, psiB =
// Lagrange t_{n+1/2} combination, psi0 = t_{n+1})
// ---------------------------------------------------------------------------
template <int TI>
__global__ void __launch_bounds__(256) k_particles_m(Grid gp, double* pos, int num, const float4* __restrict__ psiA,
                                                     const float4* __restrict__ psiB, const float4* __restrict__ psi0,
                                                     double dt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    double px = pos[2 * i], py = pos[2 * i + 1];
    float k1x, k1y;
    velocity_f(psiA, gp, locate_abs(gp, px, py), k1x, k1y);
    if (TI == 10) {
        px += dt * k1x;
        py += dt * k1y;
    } else if (TI == 20) {
        float k2x, k2y;
        velocity_f(psi0, gp, locate_abs(gp, px + dt * k1x, py + dt * k1y), k2x, k2y);
        px += dt * (double)(k1x + k2x) * 0.5;
        py += dt * (double)(k1y + k2y) * 0.5;
    } else {
        float k2x, k2y, k3x, k3y;
        velocity_f(psiB, gp, locate_abs(gp, px + 0.5 * dt * k1x, py + 0.5 * dt * k1y), k2x, k2y);
        velocity_f(psi0, gp, locate_abs(gp, px - dt * k1x + 2.0 * dt * k2x, py - dt * k1y + 2.0 * dt * k2y), k3x, k3y);
        px += dt * (double)(k1x + 4.0f * k2x + k3x) / 6.0;
        py += dt * (double)(k1y + 4.0f * k2y + k3y) / 6.0;
    }
    pos[2 * i] = wrap(px, gp.b0, gp.Wx);
    pos[2 * i + 1] = wrap(py, gp.b2, gp.Wy);
}

cudaError_t launch_particles_m(const Grid& gp, double* pos, int num, const float4* psiA, const float4* psiB,
                               const float4* psi0, double dt, int ti, cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    unsigned blocks = (unsigned)((num + 255) / 256);
    if (ti == 10) k_particles_m<10><<<blocks, 256, 0, s>>>(gp, pos, num, psiA, psiB, psi0, dt);
    else if (ti == 20) k_particles_m<20><<<blocks, 256, 0, s>>>(gp, pos, num, psiA, psiB, psi0, dt);
    else if (ti == 30) k_particles_m<30><<<blocks, 256, 0, s>>>(gp, pos, num, psiA, psiB, psi0, dt);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP32 spectral step of the psi solve and layout conversions
// ---------------------------------------------------------------------------
__global__ void k_spec_psi_f(const float2* __restrict__ Fv, Grid gv, Grid gp, float freq, float2* __restrict__ out4)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= gp.Nfft) return;
    int iXc = (int)(i % gp.NX_fft), iYc = (int)(i / gp.NX_fft);
    float2 P = make_float2(0.f, 0.f);
    bool outside = (iXc + (iXc > gp.NX / 2.0) * (gp.NX - 2 * iXc) > gv.NX / 2.0) ||
                   (iYc + (iYc > gp.NY / 2.0) * (gp.NY - 2 * iYc) > gv.NY / 2.0);
    if (!outside) {
        int iXs = iXc + (iXc > gp.NX / 2.0) * (gv.NX - gp.NX);
        int iYs = iYc + (iYc > gp.NY / 2.0) * (gv.NY - gp.NY);
        float2 f = Fv[(long long)iYs * gv.NX_fft + iXs];
        float inv = (float)(1.0 / (double)gv.N);
        P = make_float2(f.x * inv, f.y * inv);
    }
    int fX = iXc + (iXc > gp.NX / 2.0) * (gp.NX - 2 * iXc);
    int fY = iYc + (iYc > gp.NY / 2.0) * (gp.NY - 2 * iYc);
    if ((float)(fX * fX + fY * fY) > freq * freq || i == 0) P = make_float2(0.f, 0.f);
    float kx = (float)(gp.kfx * (iXc - (iXc > gp.NX / 2) * gp.NX));
    float ky = (float)(gp.kfy * (iYc - (iYc > gp.NY / 2) * gp.NY));
    if (iXc == 0 && iYc == 0) P = make_float2(0.f, 0.f);
    else {
        float ik2 = 1.0f / (kx * kx + ky * ky);
        P = make_float2(-P.x * ik2, -P.y * ik2);
    }
    float2 Py = make_float2(-P.y * ky, P.x * ky);
    out4[i] = P;
    out4[gp.Nfft + i] = make_float2(-P.y * kx, P.x * kx);
    out4[2 * gp.Nfft + i] = Py;
    out4[3 * gp.Nfft + i] = make_float2(-Py.y * kx, Py.x * kx);
}

cudaError_t launch_spec_psi_f(const float2* Fv, const Grid& gv, const Grid& gp, double freq, float2* out4, cudaStream_t s)
{
    k_spec_psi_f<<<(unsigned)((gp.Nfft + 255) / 256), 256, 0, s>>>(Fv, gv, gp, (float)freq, out4);
    return cudaGetLastError();
}

template <typename T>
__global__ void k_planes_to_float4(const T* __restrict__ planes, long long n, float4* __restrict__ out)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = make_float4((float)planes[i], (float)planes[n + i], (float)planes[2 * n + i], (float)planes[3 * n + i]);
}

cudaError_t launch_planes_to_float4(const float* planes, const double* planes_d, long long n, float4* out,
                                    cudaStream_t s)
{
    unsigned blocks = (unsigned)((n + 255) / 256);
    if (planes) k_planes_to_float4<float><<<blocks, 256, 0, s>>>(planes, n, out);
    else k_planes_to_float4<double><<<blocks, 256, 0, s>>>(planes_d, n, out);
    return cudaGetLastError();
}

__global__ void k_float4_to_planes(const float4* __restrict__ in, long long n, double* __restrict__ planes)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = in[i];
    planes[i] = v.x; planes[n + i] = v.y; planes[2 * n + i] = v.z; planes[3 * n + i] = v.w;
}

cudaError_t launch_float4_to_planes(const float4* in, long long n, double* planes, cudaStream_t s)
{
    k_float4_to_planes<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, n, planes);
    return cudaGetLastError();
}

// displacement map -> reference planar map X, Y (X = x + dX, X_x = 1 + dX_x, ...)
__global__ void k_map_to_planes(const float4* __restrict__ M, Grid g, double* __restrict__ X, double* __restrict__ Y)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    int iX = (int)(i % g.NX), iY = (int)(i / g.NX);
    float4 a = M[2 * i], b = M[2 * i + 1];
    X[i] = g.b0 + iX * g.hx + (double)a.x;
    Y[i] = g.b2 + iY * g.hy + (double)a.y;
    X[g.N + i] = 1.0 + (double)a.z; Y[g.N + i] = (double)a.w;
    X[2 * g.N + i] = (double)b.x; Y[2 * g.N + i] = 1.0 + (double)b.y;
    X[3 * g.N + i] = (double)b.z; Y[3 * g.N + i] = (double)b.w;
}

cudaError_t launch_map_to_planes(const float4* map, const Grid& g, double* X, double* Y, cudaStream_t s)
{
    k_map_to_planes<<<(unsigned)((g.N + 255) / 256), 256, 0, s>>>(map, g, X, Y);
    return cudaGetLastError();
}

// sum of psi_x^2 + psi_y^2 over an FP32 Hermite level, accumulated in FP64 (energy)
__global__ void __launch_bounds__(256) k_energy_partial(const float4* __restrict__ P, long long n, double* part)
{
    __shared__ double s[256];
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 v = P[i];
        acc = fma((double)v.y, (double)v.y, acc);
        acc = fma((double)v.z, (double)v.z, acc);
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void k_energy_final(const double* part, int nb, double* out)
{
    __shared__ double s[256];
    double acc = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += part[b];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = s[0];
}

cudaError_t launch_energy_m(const float4* psi, long long n, double* scratch, double* out, cudaStream_t s)
{
    long long need = (n + 255) / 256;
    int nb = (int)(need < kReduceBlocks ? (need > 0 ? need : 1) : kReduceBlocks);
    k_energy_partial<<<nb, 256, 0, s>>>(psi, n, scratch);
    k_energy_final<<<1, 256, 0, s>>>(scratch, nb, out);
    return cudaGetLastError();
}

}  // namespace cmm
