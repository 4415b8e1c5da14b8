// cmm_common.cuh -- grid descriptor and FP64 bicubic-Hermite device helpers
// shared by the CMM kernels (sm_103a).
//
// Data layout (reference-compatible "planar Hermite"): a Hermite field on an
// NX x NY periodic grid is 4 consecutive planes [f, f_x, f_y, f_xy] of N
// doubles, row-major index iY*NX+iX.  A backward map is two such fields
// (X and Y components).  This is the layout of the reference's CmmVar2D
// buffers (Cuda-CMM/src/grid/cmm-grid2d.cu:96-121, src/numerical/cmm-fft.cu:
// 418-429), kept so the kernel-level C-ABI can take the reference's own
// device buffers.
//
// The interpolants evaluate the same bicubic Hermite polynomial as the
// reference (src/numerical/cmm-hermite.cu:239-271 basis, :30-86 contraction)
// but in a separable order that needs fewer FP64 instructions: GB300 issues
// FP64 at about 1/64 of its FP32 rate, so every DFMA counts.  Divisions by the grid
// spacing are replaced by multiplications with its reciprocal.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cmm {

constexpr double kTwoPi = 6.283185307179586476925286766559005768394338798750211641949889184615632812572417997256069650684234136;

// Periodic grid descriptor, passed by value to kernels.
struct Grid {
    int NX, NY, NX_fft;
    long long N, Nfft;
    double hx, hy;        // spacing (bounds[1]-bounds[0]) / NX
    double ihx, ihy;      // 1/hx, 1/hy
    double b0, b1, b2, b3;  // domain bounds x0, x1, y0, y1
    double Lx, Ly;        // NX*hx, NY*hy: jump of a periodic map across the domain
    double Wx, Wy;        // bounds[1]-bounds[0], bounds[3]-bounds[2]: wrap length
    double kfx, kfy;      // 2*pi/(hx*NX), 2*pi/(hy*NY): spectral wavenumber factor
    // FP32 copies for the mixed-precision kernels: converting a double in a
    // kernel is an FP64-pipe instruction, which GB300 issues at 1/64 rate
    float hxf, hyf, ihxf, ihyf, kfxf, kfyf;
};

inline Grid make_grid(int NX, int NY, const double* bounds)
{
    Grid g;
    g.NX = NX; g.NY = NY;
    g.NX_fft = NX / 2 + 1;
    g.N = (long long)NX * NY;
    g.Nfft = (long long)g.NX_fft * NY;
    // same spacing formula as the reference grid (cmm-grid2d.cu:26-27)
    g.hx = (bounds[1] - bounds[0]) / (double)(float)NX;
    g.hy = (bounds[3] - bounds[2]) / (double)(float)NY;
    g.ihx = 1.0 / g.hx; g.ihy = 1.0 / g.hy;
    g.b0 = bounds[0]; g.b1 = bounds[1]; g.b2 = bounds[2]; g.b3 = bounds[3];
    g.Lx = NX * g.hx; g.Ly = NY * g.hy;
    g.Wx = bounds[1] - bounds[0]; g.Wy = bounds[3] - bounds[2];
    g.kfx = kTwoPi / (g.hx * NX); g.kfy = kTwoPi / (g.hy * NY);
    g.hxf = (float)g.hx; g.hyf = (float)g.hy; g.ihxf = (float)g.ihx; g.ihyf = (float)g.ihy;
    g.kfxf = (float)g.kfx; g.kfyf = (float)g.kfy;
    return g;
}

#ifdef __CUDACC__
// ---------------------------------------------------------------------------
// cell location
// ---------------------------------------------------------------------------
struct Cell {
    int i00, i10, i01, i11;   // linear indices of corners (x0,y0),(x1,y0),(x0,y1),(x1,y1)
    int wx0, wx1, wy0, wy1;   // periodic wrap counts of the corner columns / rows
    double tx, ty;            // fractional position in the cell
};

__device__ __forceinline__ int floor_div(int a, int n)
{
    return a >= 0 ? a / n : -((-a + n - 1) / n);
}

__device__ __forceinline__ Cell locate(const Grid& g, double x, double y)
{
    Cell c;
    double fx = (x - g.b0) * g.ihx;
    double fy = (y - g.b2) * g.ihy;
    double flx = floor(fx), fly = floor(fy);
    c.tx = fx - flx; c.ty = fy - fly;
    int ix0 = (int)flx, iy0 = (int)fly;
    int ix1 = ix0 + 1, iy1 = iy0 + 1;
    c.wx0 = floor_div(ix0, g.NX); c.wx1 = floor_div(ix1, g.NX);
    c.wy0 = floor_div(iy0, g.NY); c.wy1 = floor_div(iy1, g.NY);
    ix0 -= c.wx0 * g.NX; ix1 -= c.wx1 * g.NX;
    iy0 -= c.wy0 * g.NY; iy1 -= c.wy1 * g.NY;
    c.i00 = iy0 * g.NX + ix0; c.i10 = iy0 * g.NX + ix1;
    c.i01 = iy1 * g.NX + ix0; c.i11 = iy1 * g.NX + ix1;
    return c;
}

// ---------------------------------------------------------------------------
// 1D cubic Hermite weights on [0,1] at fraction t (s = 1-t):
//   value  weights  v0 = s^2(1+2t), v1 = t^2(3-2t)           (node values)
//                   v2 = t s^2 * h, v3 = -s t^2 * h          (node slopes, times h)
//   slope  weights  d0 = -6ts/h, d1 = 6ts/h, d2 = s(3s-2), d3 = t(3t-2)
// The slope weights already include the 1/h of d/dx, the value weights the h
// that converts stored slopes to per-cell units (cmm-hermite.cu:40-41, 350).
// ---------------------------------------------------------------------------
struct W4 { double w0, w1, w2, w3; };

__device__ __forceinline__ W4 value_weights(double t, double h)
{
    double s = 1.0 - t;
    double t2 = t * t, s2 = s * s;
    W4 w;
    w.w0 = s2 * fma(2.0, t, 1.0);
    w.w1 = t2 * fma(-2.0, t, 3.0);
    w.w2 = (t * s2) * h;
    w.w3 = -(s * t2) * h;
    return w;
}

__device__ __forceinline__ W4 slope_weights(double t, double ih)
{
    double s = 1.0 - t;
    double st6 = 6.0 * s * t * ih;
    W4 w;
    w.w0 = -st6;
    w.w1 = st6;
    w.w2 = s * fma(3.0, s, -2.0);
    w.w3 = t * fma(3.0, t, -2.0);
    return w;
}

// Corner data of one Hermite field at a cell: planes f, fx, fy, fxy at the
// four corners, with an optional periodic jump added to the value plane.
struct Corners {
    double f00, f10, f01, f11;
    double x00, x10, x01, x11;   // f_x
    double y00, y10, y01, y11;   // f_y
    double z00, z10, z01, z11;   // f_xy
};

__device__ __forceinline__ Corners load_corners(const double* __restrict__ H, long long N, const Cell& c)
{
    Corners q;
    q.f00 = __ldg(H + c.i00); q.f10 = __ldg(H + c.i10); q.f01 = __ldg(H + c.i01); q.f11 = __ldg(H + c.i11);
    const double* Hx = H + N;
    q.x00 = __ldg(Hx + c.i00); q.x10 = __ldg(Hx + c.i10); q.x01 = __ldg(Hx + c.i01); q.x11 = __ldg(Hx + c.i11);
    const double* Hy = H + 2 * N;
    q.y00 = __ldg(Hy + c.i00); q.y10 = __ldg(Hy + c.i10); q.y01 = __ldg(Hy + c.i01); q.y11 = __ldg(Hy + c.i11);
    const double* Hz = H + 3 * N;
    q.z00 = __ldg(Hz + c.i00); q.z10 = __ldg(Hz + c.i10); q.z01 = __ldg(Hz + c.i01); q.z11 = __ldg(Hz + c.i11);
    return q;
}

// x-contraction of one row of corners: returns (value part, y-slope part)
__device__ __forceinline__ void xrow(const W4& wx, double fa, double fb, double xa, double xb,
                                     double ya, double yb, double za, double zb, double& s, double& t)
{
    s = fma(wx.w3, xb, fma(wx.w2, xa, fma(wx.w1, fb, wx.w0 * fa)));
    t = fma(wx.w3, zb, fma(wx.w2, za, fma(wx.w1, yb, wx.w0 * ya)));
}

__device__ __forceinline__ double ycombine(const W4& wy, double s0, double s1, double t0, double t1)
{
    return fma(wy.w3, t1, fma(wy.w2, t0, fma(wy.w1, s1, wy.w0 * s0)));
}

// value of the Hermite interpolant
__device__ __forceinline__ double hermite_value(const Corners& q, const W4& wx, const W4& wy)
{
    double s0, t0, s1, t1;
    xrow(wx, q.f00, q.f10, q.x00, q.x10, q.y00, q.y10, q.z00, q.z10, s0, t0);
    xrow(wx, q.f01, q.f11, q.x01, q.x11, q.y01, q.y11, q.z01, q.z11, s1, t1);
    return ycombine(wy, s0, s1, t0, t1);
}

// gradient (d/dx, d/dy) of the Hermite interpolant
__device__ __forceinline__ void hermite_grad(const Corners& q, const W4& wx, const W4& wy,
                                             const W4& dx, const W4& dy, double& gx, double& gy)
{
    double s0, t0, s1, t1, ds0, dt0, ds1, dt1;
    xrow(wx, q.f00, q.f10, q.x00, q.x10, q.y00, q.y10, q.z00, q.z10, s0, t0);
    xrow(wx, q.f01, q.f11, q.x01, q.x11, q.y01, q.y11, q.z01, q.z11, s1, t1);
    xrow(dx, q.f00, q.f10, q.x00, q.x10, q.y00, q.y10, q.z00, q.z10, ds0, dt0);
    xrow(dx, q.f01, q.f11, q.x01, q.x11, q.y01, q.y11, q.z01, q.z11, ds1, dt1);
    gx = ycombine(wy, ds0, ds1, dt0, dt1);
    gy = ycombine(dy, s0, s1, t0, t1);
}

// Hermite value at (x, y)
__device__ __forceinline__ double interp_value(const double* __restrict__ H, const Grid& g, double x, double y)
{
    Cell c = locate(g, x, y);
    Corners q = load_corners(H, g.N, c);
    return hermite_value(q, value_weights(c.tx, g.hx), value_weights(c.ty, g.hy));
}

// velocity u = (psi_y, -psi_x) of one stream-function level at (x, y)
// (device_hermite_interpolate_grad_2D, cmm-hermite.cu:396-420)
template <int NL>
__device__ __forceinline__ void velocity_levels(const double* const* __restrict__ psi, const Grid& g,
                                                double x, double y, double* ux, double* uy)
{
    Cell c = locate(g, x, y);
    W4 wx = value_weights(c.tx, g.hx), wy = value_weights(c.ty, g.hy);
    W4 dx = slope_weights(c.tx, g.ihx), dy = slope_weights(c.ty, g.ihy);
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        Corners q = load_corners(psi[l], g.N, c);
        double gx, gy;
        hermite_grad(q, wx, wy, dx, dy, gx, gy);
        ux[l] = gy;
        uy[l] = -gx;
    }
}

// periodic map evaluation with jump (device_diffeo_interpolate_2D, cmm-hermite.cu:446-460)
__device__ __forceinline__ void map_value(const double* __restrict__ MX, const double* __restrict__ MY,
                                          const Grid& g, double x, double y, double& xo, double& yo)
{
    Cell c = locate(g, x, y);
    W4 wx = value_weights(c.tx, g.hx), wy = value_weights(c.ty, g.hy);
    Corners q = load_corners(MX, g.N, c);
    q.f00 = fma((double)c.wx0, g.Lx, q.f00); q.f10 = fma((double)c.wx1, g.Lx, q.f10);
    q.f01 = fma((double)c.wx0, g.Lx, q.f01); q.f11 = fma((double)c.wx1, g.Lx, q.f11);
    xo = hermite_value(q, wx, wy);
    q = load_corners(MY, g.N, c);
    q.f00 = fma((double)c.wy0, g.Ly, q.f00); q.f10 = fma((double)c.wy0, g.Ly, q.f10);
    q.f01 = fma((double)c.wy1, g.Ly, q.f01); q.f11 = fma((double)c.wy1, g.Ly, q.f11);
    yo = hermite_value(q, wx, wy);
}

// Jacobian determinant of a periodic map (device_diffeo_grad_2D, cmm-hermite.cu:479-503)
__device__ __forceinline__ double map_det(const double* __restrict__ MX, const double* __restrict__ MY,
                                          const Grid& g, double x, double y)
{
    Cell c = locate(g, x, y);
    W4 wx = value_weights(c.tx, g.hx), wy = value_weights(c.ty, g.hy);
    W4 dx = slope_weights(c.tx, g.ihx), dy = slope_weights(c.ty, g.ihy);
    Corners q = load_corners(MX, g.N, c);
    q.f00 = fma((double)c.wx0, g.Lx, q.f00); q.f10 = fma((double)c.wx1, g.Lx, q.f10);
    q.f01 = fma((double)c.wx0, g.Lx, q.f01); q.f11 = fma((double)c.wx1, g.Lx, q.f11);
    double Xx, Xy;
    hermite_grad(q, wx, wy, dx, dy, Xx, Xy);
    q = load_corners(MY, g.N, c);
    q.f00 = fma((double)c.wy0, g.Ly, q.f00); q.f10 = fma((double)c.wy0, g.Ly, q.f10);
    q.f01 = fma((double)c.wy1, g.Ly, q.f01); q.f11 = fma((double)c.wy1, g.Ly, q.f11);
    double Yx, Yy;
    hermite_grad(q, wx, wy, dx, dy, Yx, Yy);
    return Xx * Yy - Xy * Yx;
}

// wrap a coordinate into [b, b+W) (cmm-simulation-kernel.cu:318-319)
__device__ __forceinline__ double wrap(double v, double b, double W)
{
    return v - floor((v - b) / W) * W;
}
#endif  // __CUDACC__

}  // namespace cmm
