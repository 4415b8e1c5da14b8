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
// composition (positions accumulated in FP64 through the whole stack) and in
// the diagnostics' sums; the Jacobian-determinant deviation is formed exactly
// from FP32 slopes with error-free transformations (FP64-accurate), and tracer
// positions are 64-bit fixed point.  No per-step kernel issues FP64
// instructions: GB300 runs them at about 1/64 of the FP32 rate.
#include <cuda_runtime.h>

#include "init_conditions.cuh"
#include "mixed.hpp"
#include "pdl.cuh"
#include "psi_solve.cuh"

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
    if ((unsigned)i < (unsigned)n) return i;   // the common case: no integer division
    int r = i % n;
    return r < 0 ? r + n : r;
}

// cell of the point (bx + qx, by + qy) in cell units: integer base cell + FP32 offset
struct CellXY {
    int ix0, iy0, ix1, iy1;
    float tx, ty;
};

__device__ __forceinline__ CellXY locate_q_xy(const Grid& g, int bx, int by, float qx, float qy)
{
    float fx = floorf(qx), fy = floorf(qy);
    CellXY c;
    c.tx = qx - fx;
    c.ty = qy - fy;
    c.ix0 = wrap_index(bx + (int)fx, g.NX);
    c.iy0 = wrap_index(by + (int)fy, g.NY);
    c.ix1 = c.ix0 + 1 == g.NX ? 0 : c.ix0 + 1;
    c.iy1 = c.iy0 + 1 == g.NY ? 0 : c.iy0 + 1;
    return c;
}

__device__ __forceinline__ CellF locate_q(const Grid& g, int bx, int by, float qx, float qy)
{
    CellXY q = locate_q_xy(g, bx, by, qx, qy);
    CellF c;
    c.tx = q.tx;
    c.ty = q.ty;
    c.i00 = q.iy0 * g.NX + q.ix0; c.i10 = q.iy0 * g.NX + q.ix1;
    c.i01 = q.iy1 * g.NX + q.ix0; c.i11 = q.iy1 * g.NX + q.ix1;
    return c;
}

// cell of the point (bx*h + ox, by*h + oy): integer base cell + FP32 offset in length units
__device__ __forceinline__ CellF locate_rel(const Grid& g, int bx, int by, float ox, float oy)
{
    return locate_q(g, bx, by, ox * g.ihxf, oy * g.ihyf);
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
__device__ __forceinline__ void velocity_q(Q4 q, const Grid& g, float tx, float ty, float& ux, float& uy)
{
    float ref = q.c00.x;
    q.c00.x = 0.0f; q.c10.x -= ref; q.c01.x -= ref; q.c11.x -= ref;
    W4f wx = value_weights_f(tx, g.hxf), wy = value_weights_f(ty, g.hyf);
    W4f dx = slope_weights_f(tx, g.ihxf), dy = slope_weights_f(ty, g.ihyf);
    float gx, gy;
    herm_grad_f(q, wx, wy, dx, dy, gx, gy);
    ux = gy;
    uy = -gx;
}

__device__ __forceinline__ void velocity_f(const float4* __restrict__ P, const Grid& g, const CellF& c,
                                           float& ux, float& uy)
{
    Q4 q;
    q.c00 = __ldg(P + c.i00); q.c10 = __ldg(P + c.i10); q.c01 = __ldg(P + c.i01); q.c11 = __ldg(P + c.i11);
    velocity_q(q, g, c.tx, c.ty, ux, uy);
}

// map displacement from the four corner nodes (a, b float4 pairs), X and Y components,
// corner values minus (rx, ry)
__device__ __forceinline__ void map_disp_q(const float4& a00, const float4& b00, const float4& a10, const float4& b10,
                                           const float4& a01, const float4& b01, const float4& a11, const float4& b11,
                                           const Grid& g, float tx, float ty, float rx, float ry, float& dxo, float& dyo)
{
    W4f wx = value_weights_f(tx, g.hxf), wy = value_weights_f(ty, g.hyf);
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

// map displacement at a cell, X and Y components, corner values minus (rx, ry)
__device__ __forceinline__ void map_disp_f(const float4* __restrict__ M, const Grid& g, const CellF& c, float rx,
                                           float ry, float& dxo, float& dyo)
{
    float4 a00 = __ldg(M + 2 * c.i00), b00 = __ldg(M + 2 * c.i00 + 1);
    float4 a10 = __ldg(M + 2 * c.i10), b10 = __ldg(M + 2 * c.i10 + 1);
    float4 a01 = __ldg(M + 2 * c.i01), b01 = __ldg(M + 2 * c.i01 + 1);
    float4 a11 = __ldg(M + 2 * c.i11), b11 = __ldg(M + 2 * c.i11 + 1);
    map_disp_q(a00, b00, a10, b10, a01, b01, a11, b11, g, c.tx, c.ty, rx, ry, dxo, dyo);
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

// the psi solve's last pass for three Lagrange levels: the new level's four FP32
// planes -> its nodes, and in the same pass three combinations of the levels
// (new, 1, 2), accumulated in the order of k_precombine so the results are identical

__device__ __forceinline__ float4 combo(const float* c, const float4& v0, const float4& v1, const float4& v2)
{
    float4 a = make_float4(0, 0, 0, 0);
    a.x = fmaf(c[0], v0.x, a.x); a.y = fmaf(c[0], v0.y, a.y); a.z = fmaf(c[0], v0.z, a.z); a.w = fmaf(c[0], v0.w, a.w);
    a.x = fmaf(c[1], v1.x, a.x); a.y = fmaf(c[1], v1.y, a.y); a.z = fmaf(c[1], v1.z, a.z); a.w = fmaf(c[1], v1.w, a.w);
    a.x = fmaf(c[2], v2.x, a.x); a.y = fmaf(c[2], v2.y, a.y); a.z = fmaf(c[2], v2.z, a.z); a.w = fmaf(c[2], v2.w, a.w);
    return a;
}

__global__ void __launch_bounds__(256) k_psi_nodes3(const float* __restrict__ planes, long long n,
                                                    const float4* __restrict__ l1, const float4* __restrict__ l2,
                                                    Combo3 cm, float4* __restrict__ out0, float4* __restrict__ o1,
                                                    float4* __restrict__ o2, float4* __restrict__ o3)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v0 = make_float4(planes[i], planes[n + i], planes[2 * n + i], planes[3 * n + i]);
    const float4 v1 = __ldg(l1 + i), v2 = __ldg(l2 + i);
    out0[i] = v0;
    o1[i] = combo(cm.c[0], v0, v1, v2);
    o2[i] = combo(cm.c[1], v0, v1, v2);
    o3[i] = combo(cm.c[2], v0, v1, v2);
}

cudaError_t launch_psi_nodes3(const float* planes, long long n, const float4* l1, const float4* l2, const double* c1,
                              const double* c2, const double* c3, float4* out0, float4* o1, float4* o2, float4* o3,
                              cudaStream_t s)
{
    Combo3 cm;
    for (int l = 0; l < 3; ++l) { cm.c[0][l] = (float)c1[l]; cm.c[1][l] = (float)c2[l]; cm.c[2][l] = (float)c3[l]; }
    k_psi_nodes3<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(planes, n, l1, l2, cm, out0, o1, o2, o3);
    return cudaGetLastError();
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
// one 256-lane tile of the advection: global lane t of the map a (the footpoint weights
// already in shared memory, sc); shared by the single-map and the ensemble launches
template <int TI>
__device__ __forceinline__ void advect_m_tile(const AdvectMArgs& a, int lpn_log2, long long t,
                                              const float (&sc)[4][kMaxFoot])
{
    const int lpn = 1 << lpn_log2;
    long long node = t >> lpn_log2;
    int k = (int)(t & (lpn - 1));
    bool live = node < a.gm.N;
    const int nd = live ? (int)node : 0;
    const int iY = a.nx_log2 >= 0 ? nd >> a.nx_log2 : nd / a.gm.NX, iX = nd - iY * a.gm.NX;
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
        } else if (TI == 30) {
            float k2x, k2y, k3x, k3y;
            velocity_f(a.psiB, a.gp, locate_rel(a.gp, bx, by, ex - 0.5f * dt * k1x, ey - 0.5f * dt * k1y), k2x, k2y);
            velocity_f(a.psi0, a.gp,
                       locate_rel(a.gp, bx, by, ex + dt * k1x - 2.0f * dt * k2x, ey + dt * k1y - 2.0f * dt * k2y), k3x, k3y);
            Dx = dt * (k1x + 4.0f * k2x + k3x) * (1.0f / 6.0f);
            Dy = dt * (k1y + 4.0f * k2y + k3y) * (1.0f / 6.0f);
        } else if (TI == 20) {
            // Adams-Bashforth 2, ten fixed-point sweeps on levels 0 and 1 (adam_bashford_2_pc_b)
            float px = ex, py = ey, ox = ex, oy = ey, u2x, u2y, ux, uy;
            for (int it = 0; it < 10; ++it) {
                velocity_f(a.psi1, a.gp, locate_rel(a.gp, bx, by, px, py), u2x, u2y);
                px = ox - dt * u2x;
                py = oy - dt * u2y;
                velocity_f(a.psi1, a.gp, locate_rel(a.gp, bx, by, px, py), u2x, u2y);
                velocity_f(a.psi0, a.gp, locate_rel(a.gp, bx, by, ox, oy), ux, uy);
                ox = ex - dt * (1.5f * ux - 0.5f * u2x);
                oy = ey - dt * (1.5f * uy - 0.5f * u2y);
            }
            Dx = ex - ox;
            Dy = ey - oy;
        } else if (TI == 40) {
            float k2x, k2y, k3x, k3y, k4x, k4y;
            velocity_f(a.psiB, a.gp, locate_rel(a.gp, bx, by, ex - 0.5f * dt * k1x, ey - 0.5f * dt * k1y), k2x, k2y);
            velocity_f(a.psiB, a.gp, locate_rel(a.gp, bx, by, ex - 0.5f * dt * k2x, ey - 0.5f * dt * k2y), k3x, k3y);
            velocity_f(a.psi0, a.gp, locate_rel(a.gp, bx, by, ex - dt * k3x, ey - dt * k3y), k4x, k4y);
            Dx = dt * (k1x + 2.0f * k2x + 2.0f * k3x + k4x) * (1.0f / 6.0f);
            Dy = dt * (k1y + 2.0f * k2y + 2.0f * k3y + k4y) * (1.0f / 6.0f);
        } else if (TI == 31) {
            float k2x, k2y, k3x, k3y;
            velocity_f(a.psi0, a.gp, locate_rel(a.gp, bx, by, ex - dt * k1x, ey - dt * k1y), k2x, k2y);
            velocity_f(a.psi1, a.gp,
                       locate_rel(a.gp, bx, by, ex + 2.0f * dt * fmaf(-2.0f, k1x, k2x), ey + 2.0f * dt * fmaf(-2.0f, k1y, k2y)),
                       k3x, k3y);
            Dx = dt * (5.0f * k1x + 8.0f * k2x - k3x) * (1.0f / 12.0f);
            Dy = dt * (5.0f * k1y + 8.0f * k2y - k3y) * (1.0f / 12.0f);
        } else {   // 41
            float k2x, k2y, k3x, k3y, k4x, k4y;
            velocity_f(a.psi0, a.gp, locate_rel(a.gp, bx, by, ex - dt * k1x, ey - dt * k1y), k2x, k2y);
            velocity_f(a.psiB, a.gp,
                       locate_rel(a.gp, bx, by, ex - 0.125f * dt * fmaf(3.0f, k1x, k2x), ey - 0.125f * dt * fmaf(3.0f, k1y, k2y)),
                       k3x, k3y);
            velocity_f(a.psi0, a.gp,
                       locate_rel(a.gp, bx, by, ex + dt * (1.0f / 3.0f) * fmaf(-4.0f, k3x, k2x),
                                  ey + dt * (1.0f / 3.0f) * fmaf(-4.0f, k3y, k2y)),
                       k4x, k4y);
            Dx = dt * (2.0f * k1x - k2x + 8.0f * k3x + 3.0f * k4x) * (1.0f / 12.0f);
            Dy = dt * (2.0f * k1y - k2y + 8.0f * k3y + 3.0f * k4y) * (1.0f / 12.0f);
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

template <int TI>
__global__ void __launch_bounds__(256) k_advect_m(const AdvectMArgs a, int lpn_log2)
{
    __shared__ float sc[4][kMaxFoot];
    pdl_launch();
    if (threadIdx.x < 4 * kMaxFoot) sc[threadIdx.x / kMaxFoot][threadIdx.x % kMaxFoot] =
        a.coef[threadIdx.x / kMaxFoot][threadIdx.x % kMaxFoot];
    __syncthreads();
    pdl_wait();
    advect_m_tile<TI>(a, lpn_log2, blockIdx.x * (long long)blockDim.x + threadIdx.x, sc);
}

// ---------------------------------------------------------------------------
// separable stream function psi = F(x) - h(v) (the Vlasov-Poisson potential):
// characteristics in FP64.  The velocity u = (psi_y, -psi_x) = (-h'(v),
// -F'(x)) is a pair of 1D cubic Hermite derivatives from FP64 tables
// T[i] = (f(i+1) - f(i), f'(i)).  Vlasov characteristics move up to |v| dt
// per step (0.2 at dt = 1/32), 60x the Euler displacement of the 2048^2
// workload; FP32 velocities and offsets would put their rounding (~1e-7 of
// the displacement) through the 1/eps^2 GALS stencil into the map's cross
// derivative at the 1e-2 level, so footpoints, RK stages, the map
// interpolation and the stencil sums are FP64 here, over the FP32 map nodes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void locate64(int b, double q, int n, int& i0, int& i1, double& t)
{
    double fl = floor(q);
    t = q - fl;
    i0 = wrap_index(b + (int)fl, n);
    i1 = i0 + 1 == n ? 0 : i0 + 1;
}

__device__ __forceinline__ double sep_slope64(const double2* __restrict__ T, int i0, int i1, double t, double ih)
{
    double s = 1.0 - t;
    double2 a0 = __ldg(T + i0);
    double s1 = __ldg(&T[i1].y);
    return fma(6.0 * s * t * ih, a0.x, fma(s * fma(3.0, s, -2.0), a0.y, t * fma(3.0, t, -2.0) * s1));
}

__device__ __forceinline__ void velocity_sep64(const double2* __restrict__ TX, const double2* __restrict__ TV,
                                               const Grid& g, int bx, int by, double qx, double qy, double& ux,
                                               double& uy)
{
    int x0, x1, y0, y1;
    double tx, ty;
    locate64(bx, qx, g.NX, x0, x1, tx);
    locate64(by, qy, g.NY, y0, y1, ty);
    uy = -sep_slope64(TX, x0, x1, tx, g.ihx);
    ux = -sep_slope64(TV, y0, y1, ty, g.ihy);
}

// h'(v) and h''(v) (FP64) of the separable psi's velocity part from its 1D table (on gp's v
// axis): the slope of the table's cubic Hermite piece (sep_slope64) and that slope's derivative
__device__ __forceinline__ void sep_h12(const double2* __restrict__ tv, const Grid& gp, double v, double& h1, double& h2)
{
    int i0, i1;
    double t;
    locate64(0, (v - gp.b2) * gp.ihy, gp.NY, i0, i1, t);
    const double ih = gp.ihy, s = 1.0 - t;
    const double2 a0 = __ldg(tv + i0);
    const double s1 = __ldg(&tv[i1].y);
    h1 = fma(6.0 * s * t * ih, a0.x, fma(s * fma(3.0, s, -2.0), a0.y, t * fma(3.0, t, -2.0) * s1));
    h2 = ih * fma(6.0 * (1.0 - 2.0 * t) * ih, a0.x, fma(6.0 * t - 4.0, a0.y, (6.0 * t - 2.0) * s1));
}

// SepDrift's per-row table: h' at each map row and h'' as the mean of its two sides
__global__ void k_drift_rows(const double2* __restrict__ tv, Grid gp, Grid gm, double2* __restrict__ rows)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= gm.NY) return;
    const double v = gm.b2 + j * gm.hy, e = 1e-9 * gp.hy;
    double h1, h2l, h2r, g;
    sep_h12(tv, gp, v, h1, g);
    sep_h12(tv, gp, v - e, g, h2l);
    sep_h12(tv, gp, v + e, g, h2r);
    rows[j] = make_double2(h1, 0.5 * (h2l + h2r));
}

cudaError_t launch_drift_rows(const double2* tv, const Grid& gp, const Grid& gm, double2* rows, cudaStream_t s)
{
    k_drift_rows<<<(gm.NY + 127) / 128, 128, 0, s>>>(tv, gp, gm, rows);
    return cudaGetLastError();
}

// Phi(v) of SepDrift: the map rows' cubic Hermite interpolant of h' (FP64)
__device__ __forceinline__ double drift_phi(const double2* __restrict__ rows, const Grid& gm, double v)
{
    int j0, j1;
    double t;
    locate64(0, (v - gm.b2) * gm.ihy, gm.NY, j0, j1, t);
    const double2 r0 = __ldg(rows + j0), r1 = __ldg(rows + j1);
    const W4 w = value_weights(t, gm.hy);
    return fma(w.w3, r1.y, fma(w.w2, r0.y, fma(w.w1, r1.x, w.w0 * r0.x)));
}

// FP64 interpolation of the FP32 displacement nodes, values taken relative to (rx, ry)
__device__ __forceinline__ void map_disp64(const float4* __restrict__ M, const Grid& g, int bx, int by, double qx,
                                           double qy, double rx, double ry, double& dxo, double& dyo)
{
    int x0, x1, y0, y1;
    double tx, ty;
    locate64(bx, qx, g.NX, x0, x1, tx);
    locate64(by, qy, g.NY, y0, y1, ty);
    const int i00 = y0 * g.NX + x0, i10 = y0 * g.NX + x1, i01 = y1 * g.NX + x0, i11 = y1 * g.NX + x1;
    float4 a00 = __ldg(M + 2 * i00), b00 = __ldg(M + 2 * i00 + 1);
    float4 a10 = __ldg(M + 2 * i10), b10 = __ldg(M + 2 * i10 + 1);
    float4 a01 = __ldg(M + 2 * i01), b01 = __ldg(M + 2 * i01 + 1);
    float4 a11 = __ldg(M + 2 * i11), b11 = __ldg(M + 2 * i11 + 1);
    W4 wx = value_weights(tx, g.hx), wy = value_weights(ty, g.hy);
    double s0, t0, s1, t1;
    xrow(wx, a00.x - rx, a10.x - rx, a00.z, a10.z, b00.x, b10.x, b00.z, b10.z, s0, t0);
    xrow(wx, a01.x - rx, a11.x - rx, a01.z, a11.z, b01.x, b11.x, b01.z, b11.z, s1, t1);
    dxo = ycombine(wy, s0, s1, t0, t1);
    xrow(wx, a00.y - ry, a10.y - ry, a00.w, a10.w, b00.y, b10.y, b00.w, b10.w, s0, t0);
    xrow(wx, a01.y - ry, a11.y - ry, a01.w, a11.w, b01.y, b11.y, b01.w, b11.w, s1, t1);
    dyo = ycombine(wy, s0, s1, t0, t1);
}

template <int TI>
__global__ void __launch_bounds__(256) k_advect_sep(const AdvectMArgs a, int lpn_log2)
{
    __shared__ double sc[4][kMaxFoot];
    if (threadIdx.x < 4 * kMaxFoot) sc[threadIdx.x / kMaxFoot][threadIdx.x % kMaxFoot] =
        a.coef64[threadIdx.x / kMaxFoot][threadIdx.x % kMaxFoot];
    __syncthreads();
    const int lpn = 1 << lpn_log2;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long node = t >> lpn_log2;
    int k = (int)(t & (lpn - 1));
    bool live = node < a.gm.N;
    const int nd = live ? (int)node : 0;
    const int iY = nd / a.gm.NX, iX = nd - iY * a.gm.NX;
    float4 n0 = __ldg(a.map + 2 * nd);     // (dX, dY, dX_x, dY_x) at the node
    double gX = 0.0, gY = 0.0;
    if (live && k < a.nfoot) {
        const double r = (double)((k >> 2) + 1) * a.ep64;
        const double ex = r * (double)(1 - 2 * ((k >> 1) & 1));
        const double ey = r * (double)(1 - 2 * (((k + 1) >> 1) & 1));
        const int bx = iX * a.rp, by = iY * a.rp;
        const double dt = a.dt64, ihx = a.gp.ihx, ihy = a.gp.ihy;
        double k1x, k1y, Dx, Dy;
        velocity_sep64(a.tA, a.tv, a.gp, bx, by, ex * ihx, ey * ihy, k1x, k1y);
        if (TI == 10) {
            Dx = dt * k1x;
            Dy = dt * k1y;
        } else if (TI == 21) {
            double k2x, k2y;
            velocity_sep64(a.t0, a.tv, a.gp, bx, by, (ex - dt * k1x) * ihx, (ey - dt * k1y) * ihy, k2x, k2y);
            Dx = dt * (k1x + k2x) * 0.5;
            Dy = dt * (k1y + k2y) * 0.5;
        } else {
            double k2x, k2y, k3x, k3y;
            velocity_sep64(a.tB, a.tv, a.gp, bx, by, (ex - 0.5 * dt * k1x) * ihx, (ey - 0.5 * dt * k1y) * ihy, k2x, k2y);
            velocity_sep64(a.t0, a.tv, a.gp, bx, by, (ex + dt * k1x - 2.0 * dt * k2x) * ihx,
                           (ey + dt * k1y - 2.0 * dt * k2y) * ihy, k3x, k3y);
            Dx = dt * (k1x + 4.0 * k2x + k3x) / 6.0;
            Dy = dt * (k1y + 4.0 * k2y + k3y) / 6.0;
        }
        double mx, my;
        map_disp64(a.map, a.gm, iX, iY, (ex - Dx) * a.gm.ihx, (ey - Dy) * a.gm.ihy, n0.x, n0.y, mx, my);
        // free-streaming frame (SepDrift): X = x + tau Phi(v) + d'.  At the stencil point y = node +
        // e_k the new map is X_old at its footpoint x_f = y - D, so d'_new(y) = d'_old(x_f) - D_x +
        // tau (Phi(v_f) - Phi(v_y)) - dt Phi(v_y): free streaming alone (D_x = -dt h'(v_y), v_f =
        // v_y) leaves d' unchanged up to Phi - h'
        const double vy = a.gm.b2 + iY * a.gm.hy + ey;
        const double sy = drift_phi(a.drows, a.gm, vy), sf = drift_phi(a.drows, a.gm, vy - Dy);
        gX = mx - Dx + fma(a.tau64, sf - sy, -dt * sy);
        gY = my - Dy;
    }
    const int comp = k & 1, plane = (k >> 1) & 3;
    double acc = 0.0;
    for (int kk = 0; kk < a.nfoot; ++kk) {
        double vx = __shfl_sync(0xffffffffu, gX, kk, lpn);
        double vy = __shfl_sync(0xffffffffu, gY, kk, lpn);
        acc = fma(comp ? vy : vx, sc[plane][kk], acc);
    }
    if (live && k < 8) {
        if (plane == 0) acc += comp ? (double)n0.y : (double)n0.x;
        reinterpret_cast<float*>(a.out)[8 * node + k] = (float)acc;
    }
}

cudaError_t launch_advect_m(const AdvectMArgs& a, cudaStream_t s)
{
    int lpn_log2 = a.nfoot <= 8 ? 3 : 4;
    long long total = a.gm.N << lpn_log2;
    unsigned blocks = (unsigned)((total + 255) / 256);
    if (a.tv) {
        switch (a.time_integration_num) {
            case 10: k_advect_sep<10><<<blocks, 256, 0, s>>>(a, lpn_log2); break;
            case 21: k_advect_sep<21><<<blocks, 256, 0, s>>>(a, lpn_log2); break;
            case 30: k_advect_sep<30><<<blocks, 256, 0, s>>>(a, lpn_log2); break;
            default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    cudaError_t e;
    switch (a.time_integration_num) {
        case 10: e = launch_pdl(k_advect_m<10>, blocks, 256, 0, s, a, lpn_log2); break;
        case 21: e = launch_pdl(k_advect_m<21>, blocks, 256, 0, s, a, lpn_log2); break;
        case 30: e = launch_pdl(k_advect_m<30>, blocks, 256, 0, s, a, lpn_log2); break;
        case 20: e = launch_pdl(k_advect_m<20>, blocks, 256, 0, s, a, lpn_log2); break;
        case 40: e = launch_pdl(k_advect_m<40>, blocks, 256, 0, s, a, lpn_log2); break;
        case 31: e = launch_pdl(k_advect_m<31>, blocks, 256, 0, s, a, lpn_log2); break;
        case 41: e = launch_pdl(k_advect_m<41>, blocks, 256, 0, s, a, lpn_log2); break;
        default: return cudaErrorInvalidValue;
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

// ---------------------------------------------------------------------------
// incompressibility: one thread per (coarse cell, check row).  The slopes of
// the displacement are interpolated in FP32; the deviation of the Jacobian
// determinant  det - 1 = a + b + a*b - c*e  (a = dX_x, b = dY_y, c = dX_y,
// e = dY_x) is formed exactly from them with error-free transformations
// (TwoSum, FMA TwoProduct) and kept as a normalised FP32 pair hi + lo, which
// is as accurate as an FP64 evaluation (~1e-14 of |a|+|b|+|ab|+|ce|) but
// needs no FP64 instruction.  Check points are the fine grid shifted by half
// a fine cell (k_incompressibility_check), r = Nf / Nc per cell.
// ---------------------------------------------------------------------------
struct F2 { float hi, lo; };

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ F2 abs_det_deviation(float a, float b, float c, float e)
{
    float s, es, t, et, u, eu;
    two_sum(a, b, s, es);
    float p = __fmul_rn(a, b), ep = fmaf(a, b, -p);
    float q = __fmul_rn(c, e), eq = fmaf(c, e, -q);
    two_sum(p, -q, t, et);
    two_sum(s, t, u, eu);
    float lo = __fadd_rn(__fadd_rn(__fadd_rn(es, et), __fsub_rn(ep, eq)), eu);
    F2 r;
    r.hi = __fadd_rn(u, lo);
    r.lo = __fsub_rn(lo, __fsub_rn(r.hi, u));
    if (r.hi < 0.0f || (r.hi == 0.0f && r.lo < 0.0f)) { r.hi = -r.hi; r.lo = -r.lo; }
    return r;
}

__device__ __forceinline__ bool f2_greater(const F2& x, const F2& y)
{
    return x.hi > y.hi || (x.hi == y.hi && x.lo > y.lo);
}

// y-contraction of one Hermite column pair of a map component at fixed ty:
// at each of the cell's two x-columns j, V_j = value, S_j = x-slope (both at
// ty), DV_j / DS_j = their y-derivatives.  Corner value planes are taken
// relative to f00 (slope weights sum to zero; values follow by adding f00).
struct YCol { float V0, V1, S0, S1, DV0, DV1, DS0, DS1; };

__device__ __forceinline__ YCol ycontract(float f00, float f10, float f01, float f11, float x00, float x10, float x01,
                                          float x11, float y00, float y10, float y01, float y11, float z00, float z10,
                                          float z01, float z11, const W4f& wy, const W4f& dy)
{
    // corners: (x0,y0) = 00, (x1,y0) = 10, (x0,y1) = 01, (x1,y1) = 11; x = f_x, y = f_y, z = f_xy
    YCol c;
    c.V0 = fmaf(wy.w3, y01, fmaf(wy.w2, y00, fmaf(wy.w1, f01, wy.w0 * f00)));
    c.V1 = fmaf(wy.w3, y11, fmaf(wy.w2, y10, fmaf(wy.w1, f11, wy.w0 * f10)));
    c.S0 = fmaf(wy.w3, z01, fmaf(wy.w2, z00, fmaf(wy.w1, x01, wy.w0 * x00)));
    c.S1 = fmaf(wy.w3, z11, fmaf(wy.w2, z10, fmaf(wy.w1, x11, wy.w0 * x10)));
    c.DV0 = fmaf(dy.w3, y01, fmaf(dy.w2, y00, fmaf(dy.w1, f01, dy.w0 * f00)));
    c.DV1 = fmaf(dy.w3, y11, fmaf(dy.w2, y10, fmaf(dy.w1, f11, dy.w0 * f10)));
    c.DS0 = fmaf(dy.w3, z01, fmaf(dy.w2, z00, fmaf(dy.w1, x01, dy.w0 * x00)));
    c.DS1 = fmaf(dy.w3, z11, fmaf(dy.w2, z10, fmaf(dy.w1, x11, dy.w0 * x10)));
    return c;
}

// gradient at tx from a y-contracted column pair (wx: value weights, dx: slope weights at tx)
__device__ __forceinline__ void ycol_grad(const YCol& c, const W4f& wx, const W4f& dx, float& gx, float& gy)
{
    gx = fmaf(dx.w3, c.S1, fmaf(dx.w2, c.S0, fmaf(dx.w1, c.V1, dx.w0 * c.V0)));
    gy = fmaf(wx.w3, c.DS1, fmaf(wx.w2, c.DS0, fmaf(wx.w1, c.DV1, wx.w0 * c.DV0)));
}

constexpr int kMaxCheckRatio = 32;   // check points per map cell and axis

// x-weights of the r check columns of a map cell (shared by the threads of a block)
__device__ __forceinline__ void incomp_tables(const Grid& gm, int r, float ir, W4f* sw, W4f* sd)
{
    if ((int)threadIdx.x < r) {
        float tx = ((float)threadIdx.x + 0.5f) * ir;
        sw[threadIdx.x] = value_weights_f(tx, gm.hxf);
        sd[threadIdx.x] = slope_weights_f(tx, gm.ihxf);
    }
}

// check item i (map cell, row of check points in it): the largest deviation over its r points;
// R > 0 a compile-time r, nx_log2 >= 0 a power-of-two map width (shifts for the index split)
template <int R = 0>
__device__ __forceinline__ void incomp_item(const Grid& gm, int r_rt, float ir, const float4* __restrict__ M, int i,
                                            const W4f* sw, const W4f* sd, F2& best, int nx_log2 = -1,
                                            const SepDrift* drift = nullptr)
{
        const int r = R > 0 ? R : r_rt;
        int cell = i / r, sub_y = i - cell * r;
        int cy = nx_log2 >= 0 ? cell >> nx_log2 : cell / gm.NX, cx = cell - cy * gm.NX;
        int cx1 = cx + 1 == gm.NX ? 0 : cx + 1, cy1 = cy + 1 == gm.NY ? 0 : cy + 1;
        int i00 = cy * gm.NX + cx, i10 = cy * gm.NX + cx1;
        int i01 = cy1 * gm.NX + cx, i11 = cy1 * gm.NX + cx1;
        float4 a00 = __ldg(M + 2 * i00), b00 = __ldg(M + 2 * i00 + 1);
        float4 a10 = __ldg(M + 2 * i10), b10 = __ldg(M + 2 * i10 + 1);
        float4 a01 = __ldg(M + 2 * i01), b01 = __ldg(M + 2 * i01 + 1);
        float4 a11 = __ldg(M + 2 * i11), b11 = __ldg(M + 2 * i11 + 1);
        float drow = 0.0f;   // free-streaming frame: the drift's value difference between the cell's rows
        if (drift) {
            // X as the map grid represents it: node data d' + (tau h'(v_j), 0, tau h''(v_j), 0)
            const double2 r0 = __ldg(drift->rows + cy), r1 = __ldg(drift->rows + cy1);
            const float s0 = (float)(r0.y * drift->tau), s1 = (float)(r1.y * drift->tau);
            drow = (float)((r1.x - r0.x) * drift->tau);
            b00.x += s0; b10.x += s0; b01.x += s1; b11.x += s1;
        }
        float ty = ((float)sub_y + 0.5f) * ir;
        W4f wy = value_weights_f(ty, gm.hyf), dy = slope_weights_f(ty, gm.ihyf);
        // X: f = a.x, f_x = a.z, f_y = b.x, f_xy = b.z;  Y: f = a.y, f_x = a.w, f_y = b.y, f_xy = b.w
        YCol cX = ycontract(0.0f, a10.x - a00.x, a01.x - a00.x + drow, a11.x - a00.x + drow, a00.z, a10.z, a01.z,
                            a11.z, b00.x, b10.x, b01.x, b11.x, b00.z, b10.z, b01.z, b11.z, wy, dy);
        YCol cY = ycontract(0.0f, a10.y - a00.y, a01.y - a00.y, a11.y - a00.y, a00.w, a10.w, a01.w, a11.w,
                            b00.y, b10.y, b01.y, b11.y, b00.w, b10.w, b01.w, b11.w, wy, dy);
        for (int sx = 0; sx < r; ++sx) {
            float Xx, Xy, Yx, Yy;
            ycol_grad(cX, sw[sx], sd[sx], Xx, Xy);
            ycol_grad(cY, sw[sx], sd[sx], Yx, Yy);
            F2 dev = abs_det_deviation(Xx, Yy, Xy, Yx);
            if (f2_greater(dev, best)) best = dev;
        }
}

// block maximum of best (an exact FP32 pair), one atomicMax of its FP64 value into result
__device__ __forceinline__ void incomp_block_max(F2 best, F2* wmax, unsigned long long* result)
{
    for (int o = 16; o > 0; o >>= 1) {
        F2 v;
        v.hi = __shfl_xor_sync(0xffffffffu, best.hi, o);
        v.lo = __shfl_xor_sync(0xffffffffu, best.lo, o);
        if (f2_greater(v, best)) best = v;
    }
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (f2_greater(wmax[w], best)) best = wmax[w];
        double dev = (double)best.hi + (double)best.lo;   // non-negative: its bits order like its value
        atomicMax(result, (unsigned long long)__double_as_longlong(dev));
    }
}

// clear (optional): a second result slot zeroed for the next check
template <int R>
__global__ void __launch_bounds__(256) k_incomp_m(Grid gm, int r, float ir, const float4* __restrict__ M,
                                                  unsigned long long* result, int nx_log2,
                                                  unsigned long long* clear = nullptr)
{
    __shared__ W4f sw[kMaxCheckRatio], sd[kMaxCheckRatio];
    __shared__ F2 wmax[8];
    pdl_launch();
    incomp_tables(gm, r, ir, sw, sd);
    __syncthreads();
    pdl_wait();
    if (clear && blockIdx.x == 0 && threadIdx.x == 0) *clear = 0ull;
    F2 best = {0.0f, 0.0f};
    const int total = (int)gm.N * r;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
        incomp_item<R>(gm, r, ir, M, i, sw, sd, best, nx_log2);
    incomp_block_max(best, wmax, result);
}

// the same for a map in the free-streaming frame (SepDrift)
__global__ void __launch_bounds__(256) k_incomp_m_drift(Grid gm, int r, float ir, const float4* __restrict__ M,
                                                        unsigned long long* result, int nx_log2, SepDrift drift)
{
    __shared__ W4f sw[kMaxCheckRatio], sd[kMaxCheckRatio];
    __shared__ F2 wmax[8];
    incomp_tables(gm, r, ir, sw, sd);
    __syncthreads();
    F2 best = {0.0f, 0.0f};
    const int total = (int)gm.N * r;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
        incomp_item<0>(gm, r, ir, M, i, sw, sd, best, nx_log2, &drift);
    incomp_block_max(best, wmax, result);
}

cudaError_t launch_incomp_m_pp(const Grid& gm, int r, const float4* map, double* d_result, double* d_clear,
                               cudaStream_t s)
{
    if (r <= 0 || r > kMaxCheckRatio || gm.N * r > 0x7fffffffLL || d_result == d_clear) return cudaErrorInvalidValue;
    const long long need = (gm.N * r + 255) / 256;
    const int nx_log2 = (gm.NX & (gm.NX - 1)) == 0 ? __builtin_ctz((unsigned)gm.NX) : -1;
    unsigned long long* res = reinterpret_cast<unsigned long long*>(d_result);
    unsigned long long* clr = reinterpret_cast<unsigned long long*>(d_clear);
    const float ir = 1.0f / (float)r;
    // one resident wave of blocks over the grid-strided items: no tail wave
    auto go = [&](auto kernel) {
        const int blocks = fft::resident_grid(reinterpret_cast<const void*>(kernel), 256, 0, need);
        return launch_pdl(kernel, (unsigned)blocks, 256, 0, s, gm, r, ir, map, res, nx_log2, clr);
    };
    switch (r) {
        case 2: return go(k_incomp_m<2>);
        case 4: return go(k_incomp_m<4>);
        case 8: return go(k_incomp_m<8>);
        default: return go(k_incomp_m<0>);
    }
}

cudaError_t launch_incomp_m(const Grid& gm, int r, const float4* map, double* d_result, cudaStream_t s,
                            const SepDrift* drift)
{
    if (r <= 0 || r > kMaxCheckRatio || gm.N * r > 0x7fffffffLL) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(d_result, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    long long total = gm.N * r;
    long long need = (total + 255) / 256;
    unsigned blocks = (unsigned)(need < 152 * 8 ? need : 152 * 8);
    const int nx_log2 = (gm.NX & (gm.NX - 1)) == 0 ? __builtin_ctz((unsigned)gm.NX) : -1;
    unsigned long long* res = reinterpret_cast<unsigned long long*>(d_result);
    const float ir = 1.0f / (float)r;
    if (drift) {
        k_incomp_m_drift<<<blocks, 256, 0, s>>>(gm, r, ir, map, res, nx_log2, *drift);
        return cudaGetLastError();
    }
    switch (r) {
        case 2: k_incomp_m<2><<<blocks, 256, 0, s>>>(gm, r, ir, map, res, nx_log2); break;
        case 4: k_incomp_m<4><<<blocks, 256, 0, s>>>(gm, r, ir, map, res, nx_log2); break;
        case 8: k_incomp_m<8><<<blocks, 256, 0, s>>>(gm, r, ir, map, res, nx_log2); break;
        default: k_incomp_m<0><<<blocks, 256, 0, s>>>(gm, r, ir, map, res, nx_log2); break;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 64-bit fixed-point positions: a coordinate is P = (x - b0) / W * 2^64
// (mod 2^64), so the periodic wrap is unsigned overflow, the cell and its
// fraction are integer operations (cell = hi64(P * N), fraction = top bits of
// lo64(P * N)), and a displacement D (FP32, length units) is added as the
// exact fixed-point number nearest D * 2^64 / W, the scale 2^32 / W carried
// as an FP32 pair.  Positions accumulate with 2^-64 resolution (finer than
// FP64's 2^-53 relative) and no FP64 instruction.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long fix_increment(float d, float2 sc)
{
    float sh = __fmul_rn(d, sc.x);
    float sl = __fadd_rn(fmaf(d, sc.x, -sh), __fmul_rn(d, sc.y));   // d * 2^32 / W = sh + sl
    float n = rintf(sh);
    float r = __fadd_rn(__fsub_rn(sh, n), sl);                       // |r| <= 0.5 + 2^-20
    unsigned long long hi = (unsigned long long)(long long)__float2int_rn(n);   // saturates beyond W / 2
    unsigned long long lo = (unsigned long long)(long long)__float2int_rn(r * 2147483648.0f);
    return (hi << 32) + (lo << 1);
}

// FP64 coordinate -> 64-bit fixed point of the periodic domain [b, b + W)
__device__ __forceinline__ unsigned long long fix_from(double x, double b, double W)
{
    double t = (x - b) / W;
    t -= floor(t);
    const double v = t * 18446744073709551616.0;
    return v >= 18446744073709551616.0 ? 0ull : __double2ull_rn(v);
}

// the drift tau Phi(v) of a map in the free-streaming frame (SepDrift) at fixed-point v = Py, as a
// fixed-point x increment (FP64: the drift is tens of domain lengths' worth of free streaming)
__device__ __forceinline__ unsigned long long fix_drift(const SepDrift& d, const Grid& gm, unsigned long long Py,
                                                        double tau)
{
    const double phi = drift_phi(d.rows, d.gm, gm.b2 + __ull2double_rn(Py) * (gm.Wy * 5.42101086242752217e-20));
    return fix_from(phi * tau, 0.0, gm.Wx);
}

__device__ __forceinline__ void fix_cell(unsigned long long P, int n, int& cell, float& frac)
{
    cell = (int)__umul64hi(P, (unsigned long long)n);
    frac = (float)(unsigned)((P * (unsigned long long)n) >> 40) * 5.9604644775390625e-8f;   // 24 bits * 2^-24
}

static float2 fix_scale(double W)
{
    double c = 4294967296.0 / W;
    float hi = (float)c;
    return make_float2(hi, (float)(c - (double)hi));
}

// floor(2^64 / n): the fixed-point spacing of an n-point grid
static unsigned long long fix_step(int n)
{
    if (n <= 1) return 0ull;
    if ((n & (n - 1)) == 0) {
        int l = 0;
        while ((1 << l) < n) ++l;
        return 1ull << (64 - l);
    }
    return ~0ull / (unsigned long long)n;
}

void fix_constants(const Grid& gm, const Grid& gt, unsigned long long* stx, unsigned long long* sty, float2* scx,
                   float2* scy)
{
    *stx = fix_step(gt.NX);
    *sty = fix_step(gt.NY);
    *scx = fix_scale(gm.Wx);
    *scy = fix_scale(gm.Wy);
}

// ---------------------------------------------------------------------------
// remap-time composition: every target node is chased through the current
// map and all stacked maps (x <- x + d(x)) at 64-bit fixed-point positions;
// omega_0 is then evaluated there (a discrete initial field from its FP32
// Hermite nodes, an analytic one with its FP64 formula).  Target, map and
// discrete grids span the same domain.
// ---------------------------------------------------------------------------
// omega_0 at target node (iX, iY) (fixed-point spacing stx, sty)
// the fixed-point position of a target node through the current map and the stack (drift: the
// maps are in the free-streaming frame, drift->tau the current map's age, drift->taus the stack's)
__device__ __forceinline__ void compose_chase(const Grid& gm, float2 scx, float2 scy, const float4* __restrict__ map,
                                              const float4* __restrict__ stack, int n_maps, unsigned long long& Px,
                                              unsigned long long& Py, const SepDrift* drift)
{
    int cx, cy;
    float tx, ty, dx, dy;
    fix_cell(Px, gm.NX, cx, tx);
    fix_cell(Py, gm.NY, cy, ty);
    map_disp_f(map, gm, locate_q(gm, cx, cy, tx, ty), 0.0f, 0.0f, dx, dy);
    if (drift) Px += fix_drift(*drift, gm, Py, drift->tau);
    Px += fix_increment(dx, scx);
    Py += fix_increment(dy, scy);
    for (int m = n_maps - 1; m >= 0; --m) {
        fix_cell(Px, gm.NX, cx, tx);
        fix_cell(Py, gm.NY, cy, ty);
        map_disp_f(stack + 2 * (long long)m * gm.N, gm, locate_q(gm, cx, cy, tx, ty), 0.0f, 0.0f, dx, dy);
        if (drift) Px += fix_drift(*drift, gm, Py, __ldg(drift->taus + m));
        Px += fix_increment(dx, scx);
        Py += fix_increment(dy, scy);
    }
}

__device__ __forceinline__ double compose_value(const Grid& gm, unsigned long long stx, unsigned long long sty,
                                                float2 scx, float2 scy, const float4* __restrict__ map,
                                                const float4* __restrict__ stack, int n_maps, const InitSource& src,
                                                const float4* __restrict__ disc, int iX, int iY,
                                                const SepDrift* drift = nullptr)
{
    unsigned long long Px = (unsigned long long)iX * stx, Py = (unsigned long long)iY * sty;
    compose_chase(gm, scx, scy, map, stack, n_maps, Px, Py, drift);
    int cx, cy;
    float tx, ty;
    double v;
    if (src.kind == 3) {
        fix_cell(Px, src.gd.NX, cx, tx);
        fix_cell(Py, src.gd.NY, cy, ty);
        CellF c = locate_q(src.gd, cx, cy, tx, ty);
        Q4 q;
        q.c00 = __ldg(disc + c.i00); q.c10 = __ldg(disc + c.i10); q.c01 = __ldg(disc + c.i01); q.c11 = __ldg(disc + c.i11);
        v = herm_value_f(q, value_weights_f(c.tx, src.gd.hxf), value_weights_f(c.ty, src.gd.hyf));
    } else {
        double x = gm.b0 + __ull2double_rn(Px) * (gm.Wx * 5.42101086242752217e-20);
        double y = gm.b2 + __ull2double_rn(Py) * (gm.Wy * 5.42101086242752217e-20);
        v = init_field(src.kind, x, y, src.ic_num, src.params, src.rand_table);
    }
    return v;
}

template <typename T>
__global__ void __launch_bounds__(256) k_compose_m(Grid gm, Grid gt, unsigned long long stx, unsigned long long sty,
                                                   float2 scx, float2 scy, const float4* __restrict__ map,
                                                   const float4* __restrict__ stack, int n_maps, InitSource src,
                                                   const float4* __restrict__ disc, T* __restrict__ out)
{
    const int iX = blockIdx.x * blockDim.x + threadIdx.x, iY = blockIdx.y;
    if (iX >= gt.NX) return;
    out[(long long)iY * gt.NX + iX] = (T)compose_value(gm, stx, sty, scx, scy, map, stack, n_maps, src, disc, iX, iY);
}

// maps in the free-streaming frame (the Vlasov-Poisson mixed form)
__global__ void __launch_bounds__(256) k_compose_m_drift(Grid gm, Grid gt, unsigned long long stx,
                                                         unsigned long long sty, float2 scx, float2 scy,
                                                         const float4* __restrict__ map,
                                                         const float4* __restrict__ stack, int n_maps, InitSource src,
                                                         const float4* __restrict__ disc, double* __restrict__ out,
                                                         SepDrift drift)
{
    const int iX = blockIdx.x * blockDim.x + threadIdx.x, iY = blockIdx.y;
    if (iX >= gt.NX) return;
    out[(long long)iY * gt.NX + iX] = compose_value(gm, stx, sty, scx, scy, map, stack, n_maps, src, disc, iX, iY,
                                                    &drift);
}

cudaError_t launch_compose_m(const Grid& gm, const Grid& gt, const float4* map, const float4* stack, int n_maps,
                             const InitSource& src, const float4* disc, double* out, cudaStream_t s, float* out_f,
                             const SepDrift* drift)
{
    if (gt.b0 != gm.b0 || gt.b2 != gm.b2 || gt.Wx != gm.Wx || gt.Wy != gm.Wy || gt.NY > 65535) return cudaErrorInvalidValue;
    if (src.kind == 3 && (!disc || src.gd.b0 != gm.b0 || src.gd.b2 != gm.b2 || src.gd.Wx != gm.Wx || src.gd.Wy != gm.Wy))
        return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((gt.NX + 255) / 256), (unsigned)gt.NY);
    if (drift) {
        if (out_f || (n_maps > 0 && !drift->taus)) return cudaErrorInvalidValue;
        k_compose_m_drift<<<blocks, 256, 0, s>>>(gm, gt, fix_step(gt.NX), fix_step(gt.NY), fix_scale(gm.Wx),
                                                 fix_scale(gm.Wy), map, stack, n_maps, src, disc, out, *drift);
    } else if (out_f)
        k_compose_m<float><<<blocks, 256, 0, s>>>(gm, gt, fix_step(gt.NX), fix_step(gt.NY), fix_scale(gm.Wx),
                                                  fix_scale(gm.Wy), map, stack, n_maps, src, disc, out_f);
    else
        k_compose_m<double><<<blocks, 256, 0, s>>>(gm, gt, fix_step(gt.NX), fix_step(gt.NY), fix_scale(gm.Wx),
                                                   fix_scale(gm.Wy), map, stack, n_maps, src, disc, out);
    return cudaGetLastError();
}

// normalised half spectrum -> the four Hermite spectra [F, i kx F, i ky F, -kx ky F]
// (fourier_hermite, src/numerical/cmm-fft.cu:398-429) in FP32
__global__ void k_spec_hermite_f(const float2* __restrict__ F, Grid g, float inv_n, float2* __restrict__ out4)
{
    const int iX = blockIdx.x * blockDim.x + threadIdx.x, iY = blockIdx.y;
    if (iX >= g.NX_fft) return;
    const long long i = (long long)iY * g.NX_fft + iX;
    float2 P = F[i];
    P.x *= inv_n;
    P.y *= inv_n;
    const float kx = g.kfxf * (float)(2 * iX > g.NX ? iX - g.NX : iX);
    const float ky = g.kfyf * (float)(2 * iY > g.NY ? iY - g.NY : iY);
    const float2 Py = make_float2(-P.y * ky, P.x * ky);
    out4[i] = P;
    out4[g.Nfft + i] = make_float2(-P.y * kx, P.x * kx);
    out4[2 * g.Nfft + i] = Py;
    out4[3 * g.Nfft + i] = make_float2(-Py.y * kx, Py.x * kx);
}

cudaError_t launch_spec_hermite_f(const float2* F, const Grid& g, float2* out4, cudaStream_t s)
{
    if (g.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((g.NX_fft + 255) / 256), (unsigned)g.NY);
    k_spec_hermite_f<<<blocks, 256, 0, s>>>(F, g, (float)(1.0 / (double)g.N), out4);
    return cudaGetLastError();
}


// positions of the nodes of gt through the current map and the stack, at
// fixed-point precision, returned as FP64 coordinates in [b0, b0 + W).  gt spans
// the map's domain (node i at i * stx exactly) or, with window set, any frame (its
// nodes converted from FP64 coordinates)
__global__ void __launch_bounds__(256) k_compose_pos_m(Grid gm, Grid gt, unsigned long long stx, unsigned long long sty,
                                                       float2 scx, float2 scy, const float4* __restrict__ map,
                                                       const float4* __restrict__ stack, int n_maps,
                                                       double* __restrict__ px, double* __restrict__ py, bool window,
                                                       SepDrift drift)
{
    const int iX = blockIdx.x * blockDim.x + threadIdx.x, iY = blockIdx.y;
    if (iX >= gt.NX) return;
    unsigned long long Px = (unsigned long long)iX * stx, Py = (unsigned long long)iY * sty;
    if (window) {
        Px = fix_from(gt.b0 + iX * gt.hx, gm.b0, gm.Wx);
        Py = fix_from(gt.b2 + iY * gt.hy, gm.b2, gm.Wy);
    }
    compose_chase(gm, scx, scy, map, stack, n_maps, Px, Py, drift.rows ? &drift : nullptr);
    const long long i = (long long)iY * gt.NX + iX;
    px[i] = gm.b0 + __ull2double_rn(Px) * (gm.Wx * 5.42101086242752217e-20);
    py[i] = gm.b2 + __ull2double_rn(Py) * (gm.Wy * 5.42101086242752217e-20);
}

cudaError_t launch_compose_pos_m(const Grid& gm, const Grid& gt, const float4* map, const float4* stack, int n_maps,
                                 double* px, double* py, cudaStream_t s, const SepDrift* drift)
{
    if (gt.NY > 65535) return cudaErrorInvalidValue;
    const bool window = gt.b0 != gm.b0 || gt.b2 != gm.b2 || gt.Wx != gm.Wx || gt.Wy != gm.Wy;
    dim3 blocks((unsigned)((gt.NX + 255) / 256), (unsigned)gt.NY);
    if (drift && n_maps > 0 && !drift->taus) return cudaErrorInvalidValue;
    SepDrift d{};
    if (drift) d = *drift;
    k_compose_pos_m<<<blocks, 256, 0, s>>>(gm, gt, fix_step(gt.NX), fix_step(gt.NY), fix_scale(gm.Wx), fix_scale(gm.Wy),
                                           map, stack, n_maps, px, py, window, d);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// omega(x) = W(x + d(x)) on an output grid whose spacing divides the map's and
// the fine grid's (integer ratios ro = No / Nm, rf = Nf / No).  One thread per
// (map cell, output row): the cell's map corners are loaded and contracted in
// y once, then the ro output points of the cell in that row are evaluated
// (x-weights from a table); positions are integer node + FP32 offset.
// ---------------------------------------------------------------------------
// map column mx, output row iY of the sample (x-weights of the ro output columns in swx)
// omega = W(X(x)) at output point (iX, iY) of grid go (ro output points per map cell in x and
// y).  One thread per output point: the lanes of a warp sample consecutive points, so their
// fine-grid gathers land on consecutive nodes (one 128-byte line per 8 lanes) instead of
// nodes ro apart; the map cell's y-contraction is recomputed by each of its ro points.
// ZM: the map is the identity (its nodes are taken as zero, not read)
template <typename T, int RO = 0, bool ZM = false>
__device__ __forceinline__ void sample_m_point(const Grid& gm, const Grid& go, const Grid& gf, int ro_rt, int rf,
                                               float iro, const float4* __restrict__ map, const float4* __restrict__ W,
                                               T* __restrict__ out, int iX, int iY, const W4f* swx)
{
    if (iX >= go.NX) return;
    const int ro = RO > 0 ? RO : ro_rt;   // RO > 0: a compile-time ratio, the divisions become shifts
    const int mx = iX / ro, k = iX - mx * ro;
    const int my = iY / ro, sy = iY - my * ro;
    const int mx1 = mx + 1 == gm.NX ? 0 : mx + 1, my1 = my + 1 == gm.NY ? 0 : my + 1;
    const int i00 = my * gm.NX + mx, i10 = my * gm.NX + mx1, i01 = my1 * gm.NX + mx, i11 = my1 * gm.NX + mx1;
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 a00 = ZM ? z4 : __ldg(map + 2 * i00), b00 = ZM ? z4 : __ldg(map + 2 * i00 + 1);
    float4 a10 = ZM ? z4 : __ldg(map + 2 * i10), b10 = ZM ? z4 : __ldg(map + 2 * i10 + 1);
    float4 a01 = ZM ? z4 : __ldg(map + 2 * i01), b01 = ZM ? z4 : __ldg(map + 2 * i01 + 1);
    float4 a11 = ZM ? z4 : __ldg(map + 2 * i11), b11 = ZM ? z4 : __ldg(map + 2 * i11 + 1);
    const W4f wy = value_weights_f((float)sy * iro, gm.hyf);
    // y-contracted value (V) and x-slope (S) of each component at the two x-columns
    const float VX0 = fmaf(wy.w3, b01.x, fmaf(wy.w2, b00.x, fmaf(wy.w1, a01.x, wy.w0 * a00.x)));
    const float VX1 = fmaf(wy.w3, b11.x, fmaf(wy.w2, b10.x, fmaf(wy.w1, a11.x, wy.w0 * a10.x)));
    const float SX0 = fmaf(wy.w3, b01.z, fmaf(wy.w2, b00.z, fmaf(wy.w1, a01.z, wy.w0 * a00.z)));
    const float SX1 = fmaf(wy.w3, b11.z, fmaf(wy.w2, b10.z, fmaf(wy.w1, a11.z, wy.w0 * a10.z)));
    const float VY0 = fmaf(wy.w3, b01.y, fmaf(wy.w2, b00.y, fmaf(wy.w1, a01.y, wy.w0 * a00.y)));
    const float VY1 = fmaf(wy.w3, b11.y, fmaf(wy.w2, b10.y, fmaf(wy.w1, a11.y, wy.w0 * a10.y)));
    const float SY0 = fmaf(wy.w3, b01.w, fmaf(wy.w2, b00.w, fmaf(wy.w1, a01.w, wy.w0 * a00.w)));
    const float SY1 = fmaf(wy.w3, b11.w, fmaf(wy.w2, b10.w, fmaf(wy.w1, a11.w, wy.w0 * a10.w)));
    const W4f w = swx[k];
    const float dx = fmaf(w.w3, SX1, fmaf(w.w2, SX0, fmaf(w.w1, VX1, w.w0 * VX0)));
    const float dy = fmaf(w.w3, SY1, fmaf(w.w2, SY0, fmaf(w.w1, VY1, w.w0 * VY0)));
    // on the fine grid the output point is node iX * rf
    const CellF c = locate_rel(gf, iX * rf, iY * rf, dx, dy);
    Q4 q;
    q.c00 = __ldg(W + c.i00); q.c10 = __ldg(W + c.i10); q.c01 = __ldg(W + c.i01); q.c11 = __ldg(W + c.i11);
    out[(long long)iY * go.NX + iX] = (T)herm_value_f(q, value_weights_f(c.tx, gf.hxf), value_weights_f(c.ty, gf.hyf));
}

template <typename T, int RO>
__global__ void __launch_bounds__(256) k_sample_m(Grid gm, Grid go, Grid gf, int ro, int rf, float iro,
                                                  const float4* __restrict__ map, const float4* __restrict__ W,
                                                  T* __restrict__ out)
{
    __shared__ W4f swx[kMaxCheckRatio];
    if ((int)threadIdx.x < ro) swx[threadIdx.x] = value_weights_f((float)threadIdx.x * iro, gm.hxf);
    __syncthreads();
    sample_m_point<T, RO>(gm, go, gf, ro, rf, iro, map, W, out, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y,
                          swx);
}

// ro = 4.  The four lanes of a map cell (one quad of the warp: 256-thread blocks, go.NX a
// multiple of 4) share the cell's y-contraction: lane k loads one component of the cell's four
// nodes (X, X_x, Y, Y_x by k: 8 scalar loads), contracts it in y (the fmaf chains of
// sample_m_point, so the values are identical) and the quad exchanges the results.  A thread
// takes the four points of vorticity column iX0 in map-cell row my (vorticity rows 4 my ..
// 4 my + 3), so the 8 map loads of the cell serve four points.  Lanes with iX0 >= go.NX still
// take part in the quad exchange and write nothing.  ZM: the map is the identity (zero
// displacement).
template <bool ZM, typename T>
__device__ __forceinline__ void sample_m4_rows(const Grid& gm, const Grid& go, const Grid& gf, int rf,
                                               const float4* __restrict__ map, const float4* __restrict__ W,
                                               int iX0, int my, T* __restrict__ out)
{
    const bool live = iX0 < go.NX;
    const int iX = live ? iX0 : go.NX - 1;
    const int mx = iX >> 2, k = iX & 3;
    const int mx1 = mx + 1 == gm.NX ? 0 : mx + 1, my1 = my + 1 == gm.NY ? 0 : my + 1;
    const int i00 = my * gm.NX + mx, i10 = my * gm.NX + mx1, i01 = my1 * gm.NX + mx, i11 = my1 * gm.NX + mx1;
    const int comp = k == 0 ? 0 : (k == 1 ? 2 : (k == 2 ? 1 : 3));
    const float* m = reinterpret_cast<const float*>(map);
    const float a00 = ZM ? 0.0f : __ldg(m + 8ll * i00 + comp), b00 = ZM ? 0.0f : __ldg(m + 8ll * i00 + 4 + comp);
    const float a10 = ZM ? 0.0f : __ldg(m + 8ll * i10 + comp), b10 = ZM ? 0.0f : __ldg(m + 8ll * i10 + 4 + comp);
    const float a01 = ZM ? 0.0f : __ldg(m + 8ll * i01 + comp), b01 = ZM ? 0.0f : __ldg(m + 8ll * i01 + 4 + comp);
    const float a11 = ZM ? 0.0f : __ldg(m + 8ll * i11 + comp), b11 = ZM ? 0.0f : __ldg(m + 8ll * i11 + 4 + comp);
    const W4f w = value_weights_f((float)k * 0.25f, gm.hxf);   // sub-point k of the cell at k / 4
    const unsigned full = 0xffffffffu;
#pragma unroll 2
    for (int sy = 0; sy < 4; ++sy) {
        const W4f wy = value_weights_f((float)sy * 0.25f, gm.hyf);
        const float C0 = fmaf(wy.w3, b01, fmaf(wy.w2, b00, fmaf(wy.w1, a01, wy.w0 * a00)));
        const float C1 = fmaf(wy.w3, b11, fmaf(wy.w2, b10, fmaf(wy.w1, a11, wy.w0 * a10)));
        const float VX0 = __shfl_sync(full, C0, 0, 4), VX1 = __shfl_sync(full, C1, 0, 4);
        const float SX0 = __shfl_sync(full, C0, 1, 4), SX1 = __shfl_sync(full, C1, 1, 4);
        const float VY0 = __shfl_sync(full, C0, 2, 4), VY1 = __shfl_sync(full, C1, 2, 4);
        const float SY0 = __shfl_sync(full, C0, 3, 4), SY1 = __shfl_sync(full, C1, 3, 4);
        if (live) {
            const int iY = 4 * my + sy;
            const float dx = fmaf(w.w3, SX1, fmaf(w.w2, SX0, fmaf(w.w1, VX1, w.w0 * VX0)));
            const float dy = fmaf(w.w3, SY1, fmaf(w.w2, SY0, fmaf(w.w1, VY1, w.w0 * VY0)));
            const CellF c = locate_rel(gf, iX * rf, iY * rf, dx, dy);
            Q4 q;
            q.c00 = __ldg(W + c.i00); q.c10 = __ldg(W + c.i10); q.c01 = __ldg(W + c.i01); q.c11 = __ldg(W + c.i11);
            out[(long long)iY * go.NX + iX] =
                (T)herm_value_f(q, value_weights_f(c.tx, gf.hxf), value_weights_f(c.ty, gf.hyf));
        }
    }
}

// the kernel: one thread per vorticity column and map-cell row
template <typename T>
__global__ void __launch_bounds__(256) k_sample_m4(Grid gm, Grid go, Grid gf, int rf, const float4* __restrict__ map,
                                                   const float4* __restrict__ W, T* __restrict__ out)
{
    pdl_launch();
    pdl_wait();
    sample_m4_rows<false>(gm, go, gf, rf, map, W, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y, out);
}

// omega = W(X(x)) for a map in the free-streaming frame (SepDrift): the map's FP32 displacement
// d' is contracted as in sample_m_point, the drift tau Phi(v) of the point's row is added in FP64
// and the fine-grid cell is located in FP64 (the drift is tens of cells)
template <typename T>
__global__ void __launch_bounds__(256) k_sample_m_drift(Grid gm, Grid go, Grid gf, int ro, int rf, float iro,
                                                        const float4* __restrict__ map, const float4* __restrict__ W,
                                                        T* __restrict__ out, SepDrift drift)
{
    __shared__ W4f swx[kMaxCheckRatio];
    __shared__ double sdrift;
    const int iY = blockIdx.y;
    if ((int)threadIdx.x < ro) swx[threadIdx.x] = value_weights_f((float)threadIdx.x * iro, gm.hxf);
    if (threadIdx.x == 0) sdrift = drift_phi(drift.rows, drift.gm, go.b2 + iY * go.hy) * drift.tau;
    __syncthreads();
    const int iX = blockIdx.x * blockDim.x + threadIdx.x;
    if (iX >= go.NX) return;
    const int mx = iX / ro, k = iX - mx * ro;
    const int my = iY / ro, sy = iY - my * ro;
    const int mx1 = mx + 1 == gm.NX ? 0 : mx + 1, my1 = my + 1 == gm.NY ? 0 : my + 1;
    const int i00 = my * gm.NX + mx, i10 = my * gm.NX + mx1, i01 = my1 * gm.NX + mx, i11 = my1 * gm.NX + mx1;
    float4 a00 = __ldg(map + 2 * i00), b00 = __ldg(map + 2 * i00 + 1);
    float4 a10 = __ldg(map + 2 * i10), b10 = __ldg(map + 2 * i10 + 1);
    float4 a01 = __ldg(map + 2 * i01), b01 = __ldg(map + 2 * i01 + 1);
    float4 a11 = __ldg(map + 2 * i11), b11 = __ldg(map + 2 * i11 + 1);
    const W4f wy = value_weights_f((float)sy * iro, gm.hyf);
    const float VX0 = fmaf(wy.w3, b01.x, fmaf(wy.w2, b00.x, fmaf(wy.w1, a01.x, wy.w0 * a00.x)));
    const float VX1 = fmaf(wy.w3, b11.x, fmaf(wy.w2, b10.x, fmaf(wy.w1, a11.x, wy.w0 * a10.x)));
    const float SX0 = fmaf(wy.w3, b01.z, fmaf(wy.w2, b00.z, fmaf(wy.w1, a01.z, wy.w0 * a00.z)));
    const float SX1 = fmaf(wy.w3, b11.z, fmaf(wy.w2, b10.z, fmaf(wy.w1, a11.z, wy.w0 * a10.z)));
    const float VY0 = fmaf(wy.w3, b01.y, fmaf(wy.w2, b00.y, fmaf(wy.w1, a01.y, wy.w0 * a00.y)));
    const float VY1 = fmaf(wy.w3, b11.y, fmaf(wy.w2, b10.y, fmaf(wy.w1, a11.y, wy.w0 * a10.y)));
    const float SY0 = fmaf(wy.w3, b01.w, fmaf(wy.w2, b00.w, fmaf(wy.w1, a01.w, wy.w0 * a00.w)));
    const float SY1 = fmaf(wy.w3, b11.w, fmaf(wy.w2, b10.w, fmaf(wy.w1, a11.w, wy.w0 * a10.w)));
    const W4f w = swx[k];
    const float dx = fmaf(w.w3, SX1, fmaf(w.w2, SX0, fmaf(w.w1, VX1, w.w0 * VX0)));
    const float dy = fmaf(w.w3, SY1, fmaf(w.w2, SY0, fmaf(w.w1, VY1, w.w0 * VY0)));
    // the fine-grid cell of node (iX rf, iY rf) + (dx + drift, dy), located in FP64
    const double qx = (double)(iX * rf) + ((double)dx + sdrift) * gf.ihx;
    const double qy = (double)(iY * rf) + (double)dy * gf.ihy;
    const double fx = floor(qx), fy = floor(qy);
    CellF c;
    c.tx = (float)(qx - fx);
    c.ty = (float)(qy - fy);
    const int ix0 = wrap_index((int)fx, gf.NX), iy0 = wrap_index((int)fy, gf.NY);
    const int ix1 = ix0 + 1 == gf.NX ? 0 : ix0 + 1, iy1 = iy0 + 1 == gf.NY ? 0 : iy0 + 1;
    c.i00 = iy0 * gf.NX + ix0; c.i10 = iy0 * gf.NX + ix1;
    c.i01 = iy1 * gf.NX + ix0; c.i11 = iy1 * gf.NX + ix1;
    Q4 q;
    q.c00 = __ldg(W + c.i00); q.c10 = __ldg(W + c.i10); q.c01 = __ldg(W + c.i01); q.c11 = __ldg(W + c.i11);
    out[(long long)iY * go.NX + iX] = (T)herm_value_f(q, value_weights_f(c.tx, gf.hxf), value_weights_f(c.ty, gf.hyf));
}

template <typename T>
void sample_m_dispatch(dim3 blocks, cudaStream_t s, const Grid& gm, const Grid& go, const Grid& gf, int ro, int rf,
                       float iro, const float4* map, const float4* W, T* out)
{
    switch (ro) {
        case 1: k_sample_m<T, 1><<<blocks, 256, 0, s>>>(gm, go, gf, ro, rf, iro, map, W, out); break;
        case 2: k_sample_m<T, 2><<<blocks, 256, 0, s>>>(gm, go, gf, ro, rf, iro, map, W, out); break;
        case 4: launch_pdl(k_sample_m4<T>, dim3(blocks.x, blocks.y / 4), 256, 0, s, gm, go, gf, rf, map, W, out); break;
        case 8: k_sample_m<T, 8><<<blocks, 256, 0, s>>>(gm, go, gf, ro, rf, iro, map, W, out); break;
        default: k_sample_m<T, 0><<<blocks, 256, 0, s>>>(gm, go, gf, ro, rf, iro, map, W, out); break;
    }
}

cudaError_t launch_sample_m(const Grid& gm, const Grid& go, const Grid& gf, const float4* map, const float4* W,
                            float* out_f, double* out_d, cudaStream_t s, const SepDrift* drift)
{
    int ro = go.NX / gm.NX, rf = gf.NX / go.NX;
    if (ro < 1 || ro > kMaxCheckRatio || ro * gm.NX != go.NX || ro * gm.NY != go.NY || go.NY > 65535)
        return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((go.NX + 255) / 256), (unsigned)go.NY);
    float iro = 1.0f / (float)ro;
    if (drift) {
        if (out_f) k_sample_m_drift<float><<<blocks, 256, 0, s>>>(gm, go, gf, ro, rf, iro, map, W, out_f, *drift);
        else k_sample_m_drift<double><<<blocks, 256, 0, s>>>(gm, go, gf, ro, rf, iro, map, W, out_d, *drift);
        return cudaGetLastError();
    }
    if (out_f) sample_m_dispatch<float>(blocks, s, gm, go, gf, ro, rf, iro, map, W, out_f);
    else sample_m_dispatch<double>(blocks, s, gm, go, gf, ro, rf, iro, map, W, out_d);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// particles at 64-bit fixed-point positions (see fix_increment): the stage
// positions are FP32 offsets from the start cell, velocities are FP32.  Levels:
// l1 = t_n, l0 = t_{n+1}, l2 = t_{n-1}, half = the Lagrange t_{n+1/2} combination;
// stages as Particle_advect / Particle_advect_inertia
// (src/numerical/cmm-particles.cu:119-276, 280-551).
// ---------------------------------------------------------------------------
struct SepTables { const double2* tA; const double2* tB; const double2* t0; const double2* tv; };

struct PartM {
    Grid gp;
    ulonglong2* pos;
    float2* vel;           // inertial velocity state
    int num;
    const float4* l1;
    const float4* l0;
    const float4* l2;
    const float4* half;
    float dt, tau;
    float2 scx, scy;
};

enum { kLvN = 1, kLvN1 = 0, kLvNm1 = 2, kLvHalf = 3 };

struct StageVel {
    const PartM& a;
    int bx, by;
    float tx, ty;
    // velocity of level `which` at the start position displaced by (dx, dy)
    __device__ __forceinline__ void operator()(int which, float dx, float dy, float& ux, float& uy) const
    {
        const float4* f = which == kLvN ? a.l1 : which == kLvN1 ? a.l0 : which == kLvNm1 ? a.l2 : a.half;
        velocity_f(f, a.gp, locate_q(a.gp, bx, by, fmaf(dx, a.gp.ihxf, tx), fmaf(dy, a.gp.ihyf, ty)), ux, uy);
    }
};

template <int TI>
__device__ __forceinline__ void tracer_step_m(const StageVel& V, float dt, float& Dx, float& Dy)
{
    float k1x, k1y, k2x, k2y, k3x, k3y, k4x, k4y;
    V(kLvN, 0.0f, 0.0f, k1x, k1y);
    if (TI == 10) {
        Dx = dt * k1x;
        Dy = dt * k1y;
    } else if (TI == 20) {
        V(kLvN1, dt * k1x, dt * k1y, k2x, k2y);
        Dx = dt * (k1x + k2x) * 0.5f;
        Dy = dt * (k1y + k2y) * 0.5f;
    } else if (TI == 30) {
        V(kLvHalf, 0.5f * dt * k1x, 0.5f * dt * k1y, k2x, k2y);
        V(kLvN1, dt * fmaf(2.0f, k2x, -k1x), dt * fmaf(2.0f, k2y, -k1y), k3x, k3y);
        Dx = dt * (k1x + 4.0f * k2x + k3x) * (1.0f / 6.0f);
        Dy = dt * (k1y + 4.0f * k2y + k3y) * (1.0f / 6.0f);
    } else if (TI == 40) {
        V(kLvHalf, 0.5f * dt * k1x, 0.5f * dt * k1y, k2x, k2y);
        V(kLvHalf, 0.5f * dt * k2x, 0.5f * dt * k2y, k3x, k3y);
        V(kLvN1, dt * k3x, dt * k3y, k4x, k4y);
        Dx = dt * (k1x + 2.0f * k2x + 2.0f * k3x + k4x) * (1.0f / 6.0f);
        Dy = dt * (k1y + 2.0f * k2y + 2.0f * k3y + k4y) * (1.0f / 6.0f);
    } else if (TI == 31) {
        V(kLvN1, dt * k1x, dt * k1y, k2x, k2y);
        V(kLvNm1, dt * fmaf(-2.0f, k2x, k1x), dt * fmaf(-2.0f, k2y, k1y), k3x, k3y);
        Dx = dt * (8.0f * k1x + 5.0f * k2x - k3x) * (1.0f / 12.0f);
        Dy = dt * (8.0f * k1y + 5.0f * k2y - k3y) * (1.0f / 12.0f);
    } else {   // 41
        V(kLvN1, dt * k1x, dt * k1y, k2x, k2y);
        V(kLvHalf, dt * 0.125f * fmaf(3.0f, k1x, k2x), dt * 0.125f * fmaf(3.0f, k1y, k2y), k3x, k3y);
        V(kLvN1, dt * (1.0f / 3.0f) * fmaf(4.0f, k3x, -k2x), dt * (1.0f / 3.0f) * fmaf(4.0f, k3y, -k2y), k4x, k4y);
        Dx = dt * (2.0f * k1x - k2x + 8.0f * k3x + 3.0f * k4x) * (1.0f / 12.0f);
        Dy = dt * (2.0f * k1y - k2y + 8.0f * k3y + 3.0f * k4y) * (1.0f / 12.0f);
    }
}

// inertial: stage s has a position rate xs (a velocity) and an acceleration
// as = -(xs - u) / tau; D is the position change, dv the velocity change
template <int TI>
__device__ __forceinline__ void inertial_step_m(const StageVel& V, float dt, float tau, float vx, float vy, float& Dx,
                                                float& Dy, float& dvx, float& dvy)
{
    const float it = 1.0f / tau;
    float ux, uy;
    V(kLvN, 0.0f, 0.0f, ux, uy);
    const float a1x = (ux - vx) * it, a1y = (uy - vy) * it;
    if (TI == 10) {
        Dx = dt * vx; Dy = dt * vy;
        dvx = dt * a1x; dvy = dt * a1y;
    } else if (TI == 20) {
        const float x2x = fmaf(dt, a1x, vx), x2y = fmaf(dt, a1y, vy);
        V(kLvN1, dt * vx, dt * vy, ux, uy);
        const float a2x = (ux - x2x) * it, a2y = (uy - x2y) * it;
        Dx = 0.5f * dt * (vx + x2x); Dy = 0.5f * dt * (vy + x2y);
        dvx = 0.5f * dt * (a1x + a2x); dvy = 0.5f * dt * (a1y + a2y);
    } else if (TI == 30) {
        const float x2x = fmaf(0.5f * dt, a1x, vx), x2y = fmaf(0.5f * dt, a1y, vy);
        V(kLvHalf, 0.5f * dt * vx, 0.5f * dt * vy, ux, uy);
        const float a2x = (ux - x2x) * it, a2y = (uy - x2y) * it;
        const float x3x = fmaf(dt, fmaf(2.0f, a2x, -a1x), vx), x3y = fmaf(dt, fmaf(2.0f, a2y, -a1y), vy);
        V(kLvN1, dt * fmaf(2.0f, x2x, -vx), dt * fmaf(2.0f, x2y, -vy), ux, uy);
        const float a3x = (ux - x3x) * it, a3y = (uy - x3y) * it;
        Dx = dt * (1.0f / 6.0f) * (vx + 4.0f * x2x + x3x); Dy = dt * (1.0f / 6.0f) * (vy + 4.0f * x2y + x3y);
        dvx = dt * (1.0f / 6.0f) * (a1x + 4.0f * a2x + a3x); dvy = dt * (1.0f / 6.0f) * (a1y + 4.0f * a2y + a3y);
    } else if (TI == 40) {
        const float x2x = fmaf(0.5f * dt, a1x, vx), x2y = fmaf(0.5f * dt, a1y, vy);
        V(kLvHalf, 0.5f * dt * vx, 0.5f * dt * vy, ux, uy);
        const float a2x = (ux - x2x) * it, a2y = (uy - x2y) * it;
        const float x3x = fmaf(0.5f * dt, a2x, vx), x3y = fmaf(0.5f * dt, a2y, vy);
        V(kLvHalf, 0.5f * dt * x2x, 0.5f * dt * x2y, ux, uy);
        const float a3x = (ux - x3x) * it, a3y = (uy - x3y) * it;
        const float x4x = fmaf(dt, a3x, vx), x4y = fmaf(dt, a3y, vy);
        V(kLvN1, dt * x3x, dt * x3y, ux, uy);
        const float a4x = (ux - x4x) * it, a4y = (uy - x4y) * it;
        Dx = dt * (1.0f / 6.0f) * (vx + 2.0f * x2x + 2.0f * x3x + x4x);
        Dy = dt * (1.0f / 6.0f) * (vy + 2.0f * x2y + 2.0f * x3y + x4y);
        dvx = dt * (1.0f / 6.0f) * (a1x + 2.0f * a2x + 2.0f * a3x + a4x);
        dvy = dt * (1.0f / 6.0f) * (a1y + 2.0f * a2y + 2.0f * a3y + a4y);
    } else if (TI == 31) {
        const float x2x = fmaf(dt, a1x, vx), x2y = fmaf(dt, a1y, vy);
        V(kLvN1, dt * vx, dt * vy, ux, uy);
        const float a2x = (ux - x2x) * it, a2y = (uy - x2y) * it;
        const float x3x = fmaf(dt, fmaf(-2.0f, a2x, a1x), vx), x3y = fmaf(dt, fmaf(-2.0f, a2y, a1y), vy);
        V(kLvNm1, dt * fmaf(-2.0f, x2x, vx), dt * fmaf(-2.0f, x2y, vy), ux, uy);
        const float a3x = (ux - x3x) * it, a3y = (uy - x3y) * it;
        Dx = dt * (1.0f / 12.0f) * (8.0f * vx + 5.0f * x2x - x3x);
        Dy = dt * (1.0f / 12.0f) * (8.0f * vy + 5.0f * x2y - x3y);
        dvx = dt * (1.0f / 12.0f) * (8.0f * a1x + 5.0f * a2x - a3x);
        dvy = dt * (1.0f / 12.0f) * (8.0f * a1y + 5.0f * a2y - a3y);
    } else {   // 41
        const float x2x = fmaf(dt, a1x, vx), x2y = fmaf(dt, a1y, vy);
        V(kLvN1, dt * vx, dt * vy, ux, uy);
        const float a2x = (ux - x2x) * it, a2y = (uy - x2y) * it;
        const float x3x = fmaf(0.125f * dt, fmaf(3.0f, a1x, a2x), vx), x3y = fmaf(0.125f * dt, fmaf(3.0f, a1y, a2y), vy);
        V(kLvHalf, 0.125f * dt * fmaf(3.0f, vx, x2x), 0.125f * dt * fmaf(3.0f, vy, x2y), ux, uy);
        const float a3x = (ux - x3x) * it, a3y = (uy - x3y) * it;
        const float x4x = fmaf(dt * (1.0f / 3.0f), fmaf(4.0f, a3x, -a2x), vx);
        const float x4y = fmaf(dt * (1.0f / 3.0f), fmaf(4.0f, a3y, -a2y), vy);
        V(kLvN1, dt * (1.0f / 3.0f) * fmaf(4.0f, x3x, -x2x), dt * (1.0f / 3.0f) * fmaf(4.0f, x3y, -x2y), ux, uy);
        const float a4x = (ux - x4x) * it, a4y = (uy - x4y) * it;
        Dx = dt * (1.0f / 12.0f) * (2.0f * vx - x2x + 8.0f * x3x + 3.0f * x4x);
        Dy = dt * (1.0f / 12.0f) * (2.0f * vy - x2y + 8.0f * x3y + 3.0f * x4y);
        dvx = dt * (1.0f / 12.0f) * (2.0f * a1x - a2x + 8.0f * a3x + 3.0f * a4x);
        dvy = dt * (1.0f / 12.0f) * (2.0f * a1y - a2y + 8.0f * a3y + 3.0f * a4y);
    }
}

template <int TI, bool INERT>
__global__ void __launch_bounds__(256) k_particles_m(const PartM a)
{
    pdl_launch();
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.num) return;
    ulonglong2 P = a.pos[i];
    StageVel V{a, 0, 0, 0.0f, 0.0f};
    fix_cell(P.x, a.gp.NX, V.bx, V.tx);
    fix_cell(P.y, a.gp.NY, V.by, V.ty);
    float Dx, Dy;
    if (INERT) {
        float2 v = a.vel[i];
        float dvx, dvy;
        inertial_step_m<TI>(V, a.dt, a.tau, v.x, v.y, Dx, Dy, dvx, dvy);
        a.vel[i] = make_float2(v.x + dvx, v.y + dvy);
    } else {
        tracer_step_m<TI>(V, a.dt, Dx, Dy);
    }
    P.x += fix_increment(Dx, a.scx);
    P.y += fix_increment(Dy, a.scy);
    a.pos[i] = P;
}

// v = u of a level at the particles (Particle_advect_inertia_init, cmm-particles.cu:50-60)
__global__ void k_particle_vel_init_m(const PartM a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.num) return;
    ulonglong2 P = a.pos[i];
    StageVel V{a, 0, 0, 0.0f, 0.0f};
    fix_cell(P.x, a.gp.NX, V.bx, V.tx);
    fix_cell(P.y, a.gp.NY, V.by, V.ty);
    float ux, uy;
    V(kLvN1, 0.0f, 0.0f, ux, uy);
    a.vel[i] = make_float2(ux, uy);
}

// tracers in a separable stream function: FP64 stages from the 1D tables
template <int TI>
__global__ void __launch_bounds__(256) k_particles_sep(Grid gp, ulonglong2* __restrict__ pos, int num, SepTables tb,
                                                       double dt, float2 scx, float2 scy)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    ulonglong2 P = pos[i];
    int bx, by;
    float txf, tyf;
    fix_cell(P.x, gp.NX, bx, txf);
    fix_cell(P.y, gp.NY, by, tyf);
    const double tx = txf, ty = tyf;
    double k1x, k1y, Dx, Dy;
    velocity_sep64(tb.tA, tb.tv, gp, bx, by, tx, ty, k1x, k1y);
    if (TI == 10) {
        Dx = dt * k1x;
        Dy = dt * k1y;
    } else if (TI == 20) {
        double k2x, k2y;
        velocity_sep64(tb.t0, tb.tv, gp, bx, by, tx + dt * k1x * gp.ihx, ty + dt * k1y * gp.ihy, k2x, k2y);
        Dx = dt * (k1x + k2x) * 0.5;
        Dy = dt * (k1y + k2y) * 0.5;
    } else {
        double k2x, k2y, k3x, k3y;
        velocity_sep64(tb.tB, tb.tv, gp, bx, by, tx + 0.5 * dt * k1x * gp.ihx, ty + 0.5 * dt * k1y * gp.ihy, k2x, k2y);
        velocity_sep64(tb.t0, tb.tv, gp, bx, by, tx + dt * (2.0 * k2x - k1x) * gp.ihx,
                       ty + dt * (2.0 * k2y - k1y) * gp.ihy, k3x, k3y);
        Dx = dt * (k1x + 4.0 * k2x + k3x) / 6.0;
        Dy = dt * (k1y + 4.0 * k2y + k3y) / 6.0;
    }
    P.x += fix_increment((float)Dx, scx);
    P.y += fix_increment((float)Dy, scy);
    pos[i] = P;
}

cudaError_t launch_particles_m(const Grid& gp, unsigned long long* pos, int num, const float4* psiA,
                               const float4* psiB, const float4* psi0, double dt, int ti, cudaStream_t s,
                               const double2* tA, const double2* tB, const double2* t0, const double2* tv,
                               const float4* psiC, float2* vel, double tau)
{
    if (num <= 0) return cudaSuccess;
    unsigned blocks = (unsigned)((num + 255) / 256);
    ulonglong2* P = reinterpret_cast<ulonglong2*>(pos);
    float2 sx = fix_scale(gp.Wx), sy = fix_scale(gp.Wy);
    if (tv) {
        if (tau != 0) return cudaErrorInvalidValue;
        SepTables tb{tA, tB, t0, tv};
        if (ti == 10) k_particles_sep<10><<<blocks, 256, 0, s>>>(gp, P, num, tb, dt, sx, sy);
        else if (ti == 20) k_particles_sep<20><<<blocks, 256, 0, s>>>(gp, P, num, tb, dt, sx, sy);
        else if (ti == 30) k_particles_sep<30><<<blocks, 256, 0, s>>>(gp, P, num, tb, dt, sx, sy);
        else return cudaErrorInvalidValue;
        return cudaGetLastError();
    }
    const bool inert = tau != 0;
    if ((inert && !vel) || (ti == 31 && !psiC)) return cudaErrorInvalidValue;
    PartM a{gp, P, vel, num, psiA, psi0, psiC, psiB, (float)dt, (float)tau, sx, sy};
#define CMM_PM(TT)                                                         \
    do {                                                                   \
        if (inert) launch_pdl(k_particles_m<TT, true>, blocks, 256, 0, s, a);  \
        else launch_pdl(k_particles_m<TT, false>, blocks, 256, 0, s, a);       \
    } while (0)
    switch (ti) {
        case 10: CMM_PM(10); break;
        case 20: CMM_PM(20); break;
        case 30: CMM_PM(30); break;
        case 40: CMM_PM(40); break;
        case 31: CMM_PM(31); break;
        case 41: CMM_PM(41); break;
        default: return cudaErrorInvalidValue;
    }
#undef CMM_PM
    return cudaGetLastError();
}

cudaError_t launch_particle_vel_init_m(const Grid& gp, const unsigned long long* pos, int num, const float4* psi0,
                                       float2* vel, cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    PartM a{gp, reinterpret_cast<ulonglong2*>(const_cast<unsigned long long*>(pos)), vel, num, nullptr, psi0,
            nullptr, nullptr, 0.0f, 0.0f, make_float2(0, 0), make_float2(0, 0)};
    k_particle_vel_init_m<<<(unsigned)((num + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

__global__ void k_vel_convert(const float2* __restrict__ vf, double* __restrict__ vd, const double* __restrict__ vin,
                              float2* __restrict__ vout, int num, const int* __restrict__ perm)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    if (vf) {
        const float2 v = vf[i];
        const long long o = perm ? perm[i] : i;
        vd[2 * o] = v.x;
        vd[2 * o + 1] = v.y;
    } else vout[i] = make_float2((float)vin[2 * i], (float)vin[2 * i + 1]);
}

cudaError_t launch_vel_to_f64(const float2* v, int num, double* out, cudaStream_t s, const int* perm)
{
    if (num <= 0) return cudaSuccess;
    k_vel_convert<<<(num + 255) / 256, 256, 0, s>>>(v, out, nullptr, nullptr, num, perm);
    return cudaGetLastError();
}

cudaError_t launch_vel_from_f64(const double* v, int num, float2* out, cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    k_vel_convert<<<(num + 255) / 256, 256, 0, s>>>(nullptr, nullptr, v, out, num, nullptr);
    return cudaGetLastError();
}

// FP64 positions (reference layout, interleaved x, y) <-> fixed point
__global__ void k_pos_to_fix(const double* __restrict__ pos, long long n2, Grid g, unsigned long long* __restrict__ out)
{
    long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= n2) return;
    const bool y = j & 1;
    double t = (pos[j] - (y ? g.b2 : g.b0)) / (y ? g.Wy : g.Wx);
    t -= floor(t);
    double v = t * 18446744073709551616.0;
    out[j] = v >= 18446744073709551616.0 ? 0ull : __double2ull_rn(v);
}

__global__ void k_fix_to_pos(const unsigned long long* __restrict__ in, long long n2, Grid g, double* __restrict__ pos,
                             const int* __restrict__ perm)
{
    long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= n2) return;
    const bool y = j & 1;
    const long long o = perm ? 2ll * perm[j >> 1] + (j & 1) : j;
    pos[o] = (y ? g.b2 : g.b0) + __ull2double_rn(in[j]) * ((y ? g.Wy : g.Wx) * 5.42101086242752217e-20);
}

cudaError_t launch_pos_to_fix(const double* pos, int num, const Grid& g, unsigned long long* out, cudaStream_t s)
{
    long long n2 = 2LL * num;
    if (n2 <= 0) return cudaSuccess;
    k_pos_to_fix<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(pos, n2, g, out);
    return cudaGetLastError();
}

cudaError_t launch_fix_to_pos(const unsigned long long* in, int num, const Grid& g, double* pos, cudaStream_t s,
                              const int* perm)
{
    long long n2 = 2LL * num;
    if (n2 <= 0) return cudaSuccess;
    k_fix_to_pos<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(in, n2, g, pos, perm);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// tracer storage order: a counting sort by bucket of 4 x 4 psi cells, so a warp's tracers
// gather psi nodes from one neighbourhood.  Each tracer's arithmetic does not depend on the
// order; perm[i] is the original index of stored tracer i (the FP64 views write through it).
// ---------------------------------------------------------------------------
__global__ void k_bucket_count(const unsigned long long* __restrict__ pos, int num, int nx, int ny, int nbx,
                               int* __restrict__ key, int* __restrict__ rank, int* __restrict__ count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    const int cx = (int)__umul64hi(pos[2 * i], (unsigned long long)nx);
    const int cy = (int)__umul64hi(pos[2 * i + 1], (unsigned long long)ny);
    const int b = (cy >> 2) * nbx + (cx >> 2);
    key[i] = b;
    rank[i] = atomicAdd(count + b, 1);
}

// exclusive scan of count[0..nb) in place, one block of 1024 threads
__global__ void __launch_bounds__(1024) k_bucket_scan(int* __restrict__ count, int nb)
{
    __shared__ int part[1024];
    const int per = (nb + 1023) / 1024;
    const int b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
    int s = 0;
    for (int b = b0; b < b1; ++b) s += count[b];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = part[threadIdx.x] - s;   // exclusive prefix of this thread's range
    for (int b = b0; b < b1; ++b) {
        const int c = count[b];
        count[b] = run;
        run += c;
    }
}

__global__ void k_bucket_scatter(const unsigned long long* __restrict__ pos, const float2* __restrict__ vel,
                                 const int* __restrict__ perm, const int* __restrict__ key, const int* __restrict__ rank,
                                 const int* __restrict__ start, int num, unsigned long long* __restrict__ pos2,
                                 float2* __restrict__ vel2, int* __restrict__ perm2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    const int j = start[key[i]] + rank[i];
    pos2[2 * j] = pos[2 * i];
    pos2[2 * j + 1] = pos[2 * i + 1];
    perm2[j] = perm[i];
    if (vel) vel2[j] = vel[i];
}

cudaError_t launch_tracer_reorder(const Grid& gp, unsigned long long* pos, float2* vel, int* perm, int num,
                                  TracerScratch& t, cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    const int nbx = (gp.NX + 3) / 4, nby = (gp.NY + 3) / 4, nb = nbx * nby;
    if (num > t.cap || nb > t.nb_cap) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(t.count, 0, sizeof(int) * (size_t)nb, s);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)((num + 255) / 256);
    k_bucket_count<<<blocks, 256, 0, s>>>(pos, num, gp.NX, gp.NY, nbx, t.key, t.rank, t.count);
    k_bucket_scan<<<1, 1024, 0, s>>>(t.count, nb);
    k_bucket_scatter<<<blocks, 256, 0, s>>>(pos, vel, perm, t.key, t.rank, t.count, num, t.pos, t.vel, t.perm);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(pos, t.pos, sizeof(unsigned long long) * 2 * (size_t)num, cudaMemcpyDeviceToDevice, s)))
        return e;
    if ((e = cudaMemcpyAsync(perm, t.perm, sizeof(int) * (size_t)num, cudaMemcpyDeviceToDevice, s))) return e;
    if (vel && (e = cudaMemcpyAsync(vel, t.vel, sizeof(float2) * (size_t)num, cudaMemcpyDeviceToDevice, s))) return e;
    return cudaSuccess;
}

__global__ void k_iota(int* __restrict__ p, int num)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < num) p[i] = i;
}

cudaError_t launch_iota(int* p, int num, cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    k_iota<<<(unsigned)((num + 255) / 256), 256, 0, s>>>(p, num);
    return cudaGetLastError();
}

// omega and its gradient at the map-grid nodes: omega = W(X(x)) and, with J the map's
// Jacobian at the node (identity plus the displacement's stored derivatives),
// grad omega = J^T grad W(X(x)); three planes of gm.N values
__global__ void __launch_bounds__(256) k_sample_grad_m(Grid gm, Grid gf, int rf, const float4* __restrict__ map,
                                                      const float4* __restrict__ W, float* __restrict__ out3)
{
    const int mx = blockIdx.x * blockDim.x + threadIdx.x, my = blockIdx.y;
    if (mx >= gm.NX) return;
    const long long i = (long long)my * gm.NX + mx;
    const float4 a = __ldg(map + 2 * i), b = __ldg(map + 2 * i + 1);   // (X, Y, X_x, Y_x), (X_y, Y_y, X_xy, Y_xy)
    const CellF c = locate_rel(gf, mx * rf, my * rf, a.x, a.y);
    Q4 q;
    q.c00 = __ldg(W + c.i00); q.c10 = __ldg(W + c.i10); q.c01 = __ldg(W + c.i01); q.c11 = __ldg(W + c.i11);
    const W4f wx = value_weights_f(c.tx, gf.hxf), wy = value_weights_f(c.ty, gf.hyf);
    const W4f dx = slope_weights_f(c.tx, gf.ihxf), dy = slope_weights_f(c.ty, gf.ihyf);
    float gx, gy;
    herm_grad_f(q, wx, wy, dx, dy, gx, gy);
    out3[i] = herm_value_f(q, wx, wy);
    out3[gm.N + i] = gx * (1.0f + a.z) + gy * a.w;
    out3[2 * gm.N + i] = gx * b.x + gy * (1.0f + b.y);
}

cudaError_t launch_sample_grad_m(const Grid& gm, const Grid& gf, const float4* map, const float4* W, float* out3,
                                 cudaStream_t s)
{
    const int rf = gf.NX / gm.NX;
    if (rf < 1 || rf * gm.NX != gf.NX || rf * gm.NY != gf.NY || gm.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((gm.NX + 255) / 256), (unsigned)gm.NY);
    k_sample_grad_m<<<blocks, 256, 0, s>>>(gm, gf, rf, map, W, out3);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP32 spectral step of the psi solve and layout conversions
// ---------------------------------------------------------------------------
// (integer forms of the reference's "index > N/2.0" tests: 2*index > N)
__device__ __forceinline__ void spec_psi_item(const float2* __restrict__ Fv, const Grid& gv, const Grid& gp, float freq,
                                              float inv_nv, float2* __restrict__ out4, int iXc, int iYc)
{
    if (iXc >= gp.NX_fft) return;
    const long long i = (long long)iYc * gp.NX_fft + iXc;
    const bool hx = 2 * iXc > gp.NX, hy = 2 * iYc > gp.NY;
    const int fX = hx ? gp.NX - iXc : iXc, fY = hy ? gp.NY - iYc : iYc;   // |frequency| on the psi grid
    float2 P = make_float2(0.f, 0.f);
    if (!(2 * fX > gv.NX || 2 * fY > gv.NY)) {
        int iXs = iXc + (hx ? gv.NX - gp.NX : 0);
        int iYs = iYc + (hy ? gv.NY - gp.NY : 0);
        float2 f = Fv[(long long)iYs * gv.NX_fft + iXs];
        P = make_float2(f.x * inv_nv, f.y * inv_nv);
    }
    if ((float)(fX * fX + fY * fY) > freq * freq || i == 0) P = make_float2(0.f, 0.f);
    float kx = gp.kfxf * (float)(hx ? iXc - gp.NX : iXc);
    float ky = gp.kfyf * (float)(hy ? iYc - gp.NY : iYc);
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

__global__ void k_spec_psi_f(const float2* __restrict__ Fv, Grid gv, Grid gp, float freq, float inv_nv,
                             float2* __restrict__ out4)
{
    spec_psi_item(Fv, gv, gp, freq, inv_nv, out4, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

cudaError_t launch_spec_psi_f(const float2* Fv, const Grid& gv, const Grid& gp, double freq, float2* out4, cudaStream_t s)
{
    if (gp.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((gp.NX_fft + 255) / 256), (unsigned)gp.NY);
    k_spec_psi_f<<<blocks, 256, 0, s>>>(Fv, gv, gp, (float)freq, (float)(1.0 / (double)gv.N), out4);
    return cudaGetLastError();
}

__device__ __forceinline__ float2 padded_mode(const float2* __restrict__ Fc, const Grid& gc, const Grid& gp, int iXc,
                                              int iYc, float inv_nc)
{
    const bool hx = 2 * iXc > gp.NX, hy = 2 * iYc > gp.NY;
    const int fX = hx ? gp.NX - iXc : iXc, fY = hy ? gp.NY - iYc : iYc;
    if (2 * fX > gc.NX || 2 * fY > gc.NY) return make_float2(0.f, 0.f);
    const int iXs = iXc + (hx ? gc.NX - gp.NX : 0);
    const int iYs = iYc + (hy ? gc.NY - gp.NY : 0);
    const float2 f = Fc[(long long)iYs * gc.NX_fft + iXs];
    return make_float2(f.x * inv_nc, f.y * inv_nc);
}

__global__ void k_spec_psi_learned(const float2* __restrict__ Fc, Grid gc, const float2* __restrict__ D, Grid gp,
                                   float freq, float inv_nc, float inv_np, float2* __restrict__ out4)
{
    const int iXc = blockIdx.x * blockDim.x + threadIdx.x, iYc = blockIdx.y;
    if (iXc >= gp.NX_fft) return;
    const long long i = (long long)iYc * gp.NX_fft + iXc;
    const bool hx = 2 * iXc > gp.NX, hy = 2 * iYc > gp.NY;
    const int fX = hx ? gp.NX - iXc : iXc, fY = hy ? gp.NY - iYc : iYc;
    const float kx = gp.kfxf * (float)(hx ? iXc - gp.NX : iXc);
    const float ky = gp.kfyf * (float)(hy ? iYc - gp.NY : iYc);
    float2 P = make_float2(0.f, 0.f);
    if (!(iXc == 0 && iYc == 0) && !((float)(fX * fX + fY * fY) > freq * freq)) {
        const float2 w = padded_mode(Fc, gc, gp, iXc, iYc, inv_nc);
        const float2 d = D[i];
        const float ik2 = 1.0f / (kx * kx + ky * ky);
        P = make_float2(-(w.x + d.x * inv_np) * ik2, -(w.y + d.y * inv_np) * ik2);
    }
    const float2 Py = make_float2(-P.y * ky, P.x * ky);
    out4[i] = P;
    out4[gp.Nfft + i] = make_float2(-P.y * kx, P.x * kx);
    out4[2 * gp.Nfft + i] = Py;
    out4[3 * gp.Nfft + i] = make_float2(-Py.y * kx, Py.x * kx);
}

cudaError_t launch_spec_psi_learned(const float2* Fc, const Grid& gc, const float2* D, const Grid& gp, double freq,
                                    float2* out4, cudaStream_t s)
{
    if (gp.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((gp.NX_fft + 255) / 256), (unsigned)gp.NY);
    k_spec_psi_learned<<<blocks, 256, 0, s>>>(Fc, gc, D, gp, (float)freq, (float)(1.0 / (double)gc.N),
                                              (float)(1.0 / (double)gp.N), out4);
    return cudaGetLastError();
}

__global__ void k_spec_pad(const float2* __restrict__ Fc, Grid gc, Grid gp, float inv_nc, float2* __restrict__ out)
{
    const int iXc = blockIdx.x * blockDim.x + threadIdx.x, iYc = blockIdx.y;
    if (iXc >= gp.NX_fft) return;
    out[(long long)iYc * gp.NX_fft + iXc] = padded_mode(Fc, gc, gp, iXc, iYc, inv_nc);
}

cudaError_t launch_spec_pad(const float2* Fc, const Grid& gc, const Grid& gp, float2* out, cudaStream_t s)
{
    if (gp.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((gp.NX_fft + 255) / 256), (unsigned)gp.NY);
    k_spec_pad<<<blocks, 256, 0, s>>>(Fc, gc, gp, (float)(1.0 / (double)gc.N), out);
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

// displacement map -> reference planar map X, Y (X = x + dX, X_x = 1 + dX_x, ...); a map in the
// free-streaming frame (drift.rows) adds its drift's node data tau h'(v), tau h''(v) to X, X_y
__global__ void k_map_to_planes(const float4* __restrict__ M, Grid g, double* __restrict__ X, double* __restrict__ Y,
                                SepDrift drift)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    int iX = (int)(i % g.NX), iY = (int)(i / g.NX);
    float4 a = M[2 * i], b = M[2 * i + 1];
    double h1 = 0.0, h2 = 0.0;
    if (drift.rows) {
        const double2 r = drift.rows[iY];   // the drift's node data on this row
        h1 = r.x * drift.tau;
        h2 = r.y * drift.tau;
    }
    X[i] = g.b0 + iX * g.hx + (double)a.x + h1;
    Y[i] = g.b2 + iY * g.hy + (double)a.y;
    X[g.N + i] = 1.0 + (double)a.z; Y[g.N + i] = (double)a.w;
    X[2 * g.N + i] = (double)b.x + h2; Y[2 * g.N + i] = 1.0 + (double)b.y;
    X[3 * g.N + i] = (double)b.z; Y[3 * g.N + i] = (double)b.w;
}

cudaError_t launch_map_to_planes(const float4* map, const Grid& g, double* X, double* Y, cudaStream_t s,
                                 const SepDrift* drift)
{
    SepDrift d{};
    if (drift) d = *drift;
    k_map_to_planes<<<(unsigned)((g.N + 255) / 256), 256, 0, s>>>(map, g, X, Y, d);
    return cudaGetLastError();
}

// reference planar map X, Y -> displacement map (a stored map read back at a restart)
__global__ void k_planes_to_map(const double* __restrict__ X, const double* __restrict__ Y, Grid g, float4* __restrict__ M)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    int iX = (int)(i % g.NX), iY = (int)(i / g.NX);
    M[2 * i] = make_float4((float)(X[i] - (g.b0 + iX * g.hx)), (float)(Y[i] - (g.b2 + iY * g.hy)),
                           (float)(X[g.N + i] - 1.0), (float)Y[g.N + i]);
    M[2 * i + 1] = make_float4((float)X[2 * g.N + i], (float)(Y[2 * g.N + i] - 1.0), (float)X[3 * g.N + i],
                               (float)Y[3 * g.N + i]);
}

cudaError_t launch_planes_to_map(const double* X, const double* Y, const Grid& g, float4* map, cudaStream_t s)
{
    k_planes_to_map<<<(unsigned)((g.N + 255) / 256), 256, 0, s>>>(X, Y, g, map);
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

// ===========================================================================
// Ensembles: every member's step kernels in one launch.  A launch covers a work
// list of 256-thread tiles, member m owning tiles [cum[m], cum[m+1]); blocks walk
// the list with a grid stride, so the grid size is a tuning choice, not a
// function of the work.  Each tile runs the same device body as the single-member
// kernel on that member's descriptor (copied to shared memory), so a member of an
// ensemble computes exactly what it computes alone.
// ===========================================================================
namespace {

__device__ __forceinline__ int ens_member_of(const int* __restrict__ cum, int M, int tile)
{
    int lo = 0, hi = M - 1;
    while (lo < hi) {   // last m with cum[m] <= tile
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(cum + mid) <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// copy a descriptor into shared memory, 4 bytes per thread
template <typename T>
__device__ __forceinline__ void ens_load(T& dst, const T* src)
{
    static_assert(sizeof(T) % 4 == 0, "descriptor size");
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(&dst);
    for (int k = threadIdx.x; k < (int)(sizeof(T) / 4); k += blockDim.x) d[k] = __ldg(s + k);
}

}  // namespace

template <int TI>
__global__ void __launch_bounds__(256) k_ens_advect(const EnsMember* __restrict__ mem, const int* __restrict__ cum, int M,
                                                    int lpn_log2)
{
    __shared__ float sc[4][kMaxFoot];
    __shared__ AdvectMArgs sa;
    const int total = __ldg(cum + M);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int m = ens_member_of(cum, M, tile);
        if (!mem[m].active) continue;   // the same member for every thread of the block
        ens_load(sa, &mem[m].adv);
        __syncthreads();
        if (threadIdx.x < 4 * kMaxFoot) sc[threadIdx.x / kMaxFoot][threadIdx.x % kMaxFoot] =
            sa.coef[threadIdx.x / kMaxFoot][threadIdx.x % kMaxFoot];
        __syncthreads();
        advect_m_tile<TI>(sa, lpn_log2, (long long)(tile - __ldg(cum + m)) * 256 + threadIdx.x, sc);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_ens_incomp(const EnsMember* __restrict__ mem, const int* __restrict__ cum, int M)
{
    __shared__ W4f sw[kMaxCheckRatio], sd[kMaxCheckRatio];
    __shared__ F2 wmax[8];
    const int total = __ldg(cum + M);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int m = ens_member_of(cum, M, tile);
        const EnsMember& e = mem[m];
        if (!e.active) continue;   // block-uniform
        const Grid gm = e.adv.gm;
        const int r = e.r_check;
        const float ir = e.ir_check;
        incomp_tables(gm, r, ir, sw, sd);
        __syncthreads();
        F2 best = {0.0f, 0.0f};
        const int i = (tile - __ldg(cum + m)) * 256 + threadIdx.x;
        if (i < (int)gm.N * r) incomp_item(gm, r, ir, e.adv.out, i, sw, sd, best);   // the advected map
        incomp_block_max(best, wmax, e.einc);
        __syncthreads();
    }
}

// omega through the map on the vort grid (which = 0, into the class buffer) or on the
// coarse grid (which = 1, FP64 into the member's coarse vorticity); items are (row, column)
// pairs of map columns, flattened
__global__ void __launch_bounds__(256) k_ens_sample(const EnsMember* __restrict__ mem, const int* __restrict__ cum, int M,
                                                    int which)
{
    __shared__ W4f swx[kMaxCheckRatio];
    const int total = __ldg(cum + M);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int m = ens_member_of(cum, M, tile);
        const EnsMember& e = mem[m];
        if (!e.active) continue;   // block-uniform
        const Grid gm = e.adv.gm, gf = e.gf;
        const Grid go = which == 0 ? e.gv : gm;
        const int ro = go.NX / gm.NX, rf = gf.NX / go.NX;
        const float iro = 1.0f / (float)ro;
        if ((int)threadIdx.x < ro) swx[threadIdx.x] = value_weights_f((float)threadIdx.x * iro, gm.hxf);
        __syncthreads();
        const int i = (tile - __ldg(cum + m)) * 256 + threadIdx.x;
        if (i < go.NX * go.NY) {
            const int iY = i / go.NX, iX = i - iY * go.NX;
            if (which == 0) sample_m_point<float>(gm, go, gf, ro, rf, iro, e.adv.map, e.wfm, e.sample_out, iX, iY, swx);
            else sample_m_point<double>(gm, go, gf, ro, rf, iro, e.adv.map, e.wfm, e.vort, iX, iY, swx);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_ens_spec(const EnsMember* __restrict__ mem, const int* __restrict__ cum, int M)
{
    const int total = __ldg(cum + M);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int m = ens_member_of(cum, M, tile);
        const EnsMember& e = mem[m];
        if (!e.active) continue;
        const Grid gp = e.adv.gp;
        const int i = (tile - __ldg(cum + m)) * 256 + threadIdx.x;
        if (i < gp.NX_fft * gp.NY)
            spec_psi_item(e.spec_v, e.gv, gp, e.freq, e.inv_nv, e.spec4, i % gp.NX_fft, i / gp.NX_fft);
    }
}

// the new psi level's nodes (and, fused, the three Lagrange combinations), or a
// precombination of the levels (which = 1) before an advection that found no fused fields
__global__ void __launch_bounds__(256) k_ens_nodes(const EnsMember* __restrict__ mem, const int* __restrict__ cum, int M,
                                                   int which)
{
    const int total = __ldg(cum + M);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int m = ens_member_of(cum, M, tile);
        const EnsMember& e = mem[m];
        const long long n = e.adv.gp.N;
        const long long i = (long long)(tile - __ldg(cum + m)) * 256 + threadIdx.x;
        if (!e.active || i >= n) continue;
        if (which == 1) {
            if (!e.precombine) continue;
            const float4 v0 = __ldg(e.lv0 + i), v1 = __ldg(e.lv1 + i), v2 = __ldg(e.lv2 + i);
            e.pa[i] = combo(e.ca, v0, v1, v2);
            if (e.pb) e.pb[i] = combo(e.cb, v0, v1, v2);
            continue;
        }
        const float* pl = e.planes;
        const float4 v0 = make_float4(pl[i], pl[n + i], pl[2 * n + i], pl[3 * n + i]);
        e.psi_new[i] = v0;
        if (!e.fused) continue;
        const float4 v1 = __ldg(e.lv1n + i), v2 = __ldg(e.lv2n + i);
        e.o1[i] = combo(e.cm.c[0], v0, v1, v2);
        e.o2[i] = combo(e.cm.c[1], v0, v1, v2);
        e.o3[i] = combo(e.cm.c[2], v0, v1, v2);
    }
}

cudaError_t launch_ens(int kind, int TI, const EnsMember* mem, const int* cum, int M, int blocks, int lpn_log2,
                       cudaStream_t s)
{
    if (blocks <= 0) return cudaSuccess;
    switch (kind) {
        case kEnsAdvect:
            switch (TI) {
                case 10: k_ens_advect<10><<<blocks, 256, 0, s>>>(mem, cum, M, lpn_log2); break;
                case 21: k_ens_advect<21><<<blocks, 256, 0, s>>>(mem, cum, M, lpn_log2); break;
                case 30: k_ens_advect<30><<<blocks, 256, 0, s>>>(mem, cum, M, lpn_log2); break;
                default: return cudaErrorInvalidValue;
            }
            break;
        case kEnsIncomp: k_ens_incomp<<<blocks, 256, 0, s>>>(mem, cum, M); break;
        case kEnsSampleVort: k_ens_sample<<<blocks, 256, 0, s>>>(mem, cum, M, 0); break;
        case kEnsSampleCoarse: k_ens_sample<<<blocks, 256, 0, s>>>(mem, cum, M, 1); break;
        case kEnsSpec: k_ens_spec<<<blocks, 256, 0, s>>>(mem, cum, M); break;
        case kEnsNodes: k_ens_nodes<<<blocks, 256, 0, s>>>(mem, cum, M, 0); break;
        case kEnsPrecombine: k_ens_nodes<<<blocks, 256, 0, s>>>(mem, cum, M, 1); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// the psi solve of the mixed form on the library's FFT (psi_solve.cuh): omega through
// the map on the vorticity grid (launch_sample_m), the kept modes, the four psi planes
// as FP32 nodes and, in the same pass, the Lagrange combinations of k_psi_nodes3
// ---------------------------------------------------------------------------
struct NodesEpi {
    int nx;
    float4* out0;
    const float4* l1;
    const float4* l2;
    float4* o1;
    float4* o2;
    float4* o3;
    Combo3 cm;
    int fused;
    __device__ __forceinline__ void store(int iX, int iY, float f, float fx, float fy, float fxy) const
    {
        const long long i = (long long)iY * nx + iX;
        const float4 v0 = make_float4(f, fx, fy, fxy);
        out0[i] = v0;
        if (fused) {
            const float4 v1 = __ldg(l1 + i), v2 = __ldg(l2 + i);
            o1[i] = combo(cm.c[0], v0, v1, v2);
            o2[i] = combo(cm.c[1], v0, v1, v2);
            o3[i] = combo(cm.c[2], v0, v1, v2);
        }
    }
};

bool psi_solve_m_fits(const Grid& gm, const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv,
                      const fft::Plan2D& pp, long long* w1_values, long long* w2_values)
{
    const int ro = gv.NX / gm.NX;
    if (ro < 1 || ro > kMaxCheckRatio || ro * gm.NX != gv.NX || ro * gm.NY != gv.NY || gv.NY > 65535) return false;
    const psi::Layout L = psi::make_layout<float>(gv, gp, freq, pv, pp);
    if (!L.ok) return false;
    if (w1_values) *w1_values = L.w1_values;
    if (w2_values) *w2_values = L.w2_values;
    return true;
}

void psi_solve_m_prepare()
{
    psi::prepare<float, NodesEpi>();
}

cudaError_t launch_psi_solve_m(const Grid& gm, const Grid& gv, const Grid& gf, const float4* map, const float4* W,
                               const Grid& gp, double freq, const fft::Plan2D& pv, const fft::Plan2D& pp, float* omega,
                               float2* w1, float2* w2, float4* out0, const float4* l1, const float4* l2,
                               const double* c1, const double* c2, const double* c3, float4* o1, float4* o2,
                               float4* o3, cudaStream_t s)
{
    if (!psi_solve_m_fits(gm, gv, gp, freq, pv, pp, nullptr, nullptr)) return cudaErrorInvalidValue;
    const psi::Layout L = psi::make_layout<float>(gv, gp, freq, pv, pp);
    cudaError_t e = launch_sample_m(gm, gv, gf, map, W, omega, nullptr, s);
    if (e != cudaSuccess) return e;
    NodesEpi epi;
    epi.nx = gp.NX;
    epi.out0 = out0;
    epi.fused = c1 != nullptr;
    epi.l1 = l1; epi.l2 = l2; epi.o1 = o1; epi.o2 = o2; epi.o3 = o3;
    for (int l = 0; l < 3; ++l) {
        epi.cm.c[0][l] = c1 ? (float)c1[l] : 0.f;
        epi.cm.c[1][l] = c2 ? (float)c2[l] : 0.f;
        epi.cm.c[2][l] = c3 ? (float)c3[l] : 0.f;
    }
    return psi::launch<float>(L, gv, gp, freq, pv, pp, omega, w1, w2, epi, s);
}

}  // namespace cmm

#include "ens_fused.cuh"
