// sample_kernels.cu -- sampled outputs on a user grid (sm_103a): the full
// backward map of every sample node through the current map and the
// device-resident stack, initial fields at those positions, and spectral
// operators on the sample grid (sample_compute_and_write,
// src/simulation/cmm-simulation-host.cu:706-893).
#include <cuda_runtime.h>

#include "init_conditions.cuh"
#include "kernels.hpp"

namespace cmm {

// positions X(x), Y(x) of the nodes of gt through the current map and the
// stack (newest first), wrapped into the domain after each map like
// k_h_sample_map_compact / k_apply_map_compact (cmm-simulation-kernel.cu:302-340)
__global__ void __launch_bounds__(256) k_compose_pos(Grid gm, Grid gt, const double* __restrict__ X,
                                                     const double* __restrict__ Y, const double* __restrict__ stack,
                                                     int n_maps, double* __restrict__ px, double* __restrict__ py)
{
    const int iX = blockIdx.x * blockDim.x + threadIdx.x, iY = blockIdx.y;
    if (iX >= gt.NX) return;
    const long long i = (long long)iY * gt.NX + iX;
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
    px[i] = x;
    py[i] = y;
}

cudaError_t launch_compose_pos(const Grid& gm, const Grid& gt, const double* X, const double* Y, const double* stack,
                               int n_maps, double* px, double* py, cudaStream_t s)
{
    if (gt.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((gt.NX + 255) / 256), (unsigned)gt.NY);
    k_compose_pos<<<blocks, 256, 0, s>>>(gm, gt, X, Y, stack, n_maps, px, py);
    return cudaGetLastError();
}

// forward composition (apply_map_stack, direction 1, cmm-simulation-host.cu:130-152): the nodes
// of gt through the forward stack oldest first, then the active forward map, wrapped after each
__global__ void __launch_bounds__(256) k_compose_fwd(Grid gm, Grid gt, const double* __restrict__ X,
                                                     const double* __restrict__ Y, const double* __restrict__ stack,
                                                     int n_maps, double* __restrict__ px, double* __restrict__ py)
{
    const int iX = blockIdx.x * blockDim.x + threadIdx.x, iY = blockIdx.y;
    if (iX >= gt.NX) return;
    double x = gt.b0 + iX * gt.hx, y = gt.b2 + iY * gt.hy, xo, yo;
    for (int m = 0; m <= n_maps; ++m) {
        const double* MX = m < n_maps ? stack + (long long)m * 8 * gm.N : X;
        const double* MY = m < n_maps ? MX + 4 * gm.N : Y;
        map_value(MX, MY, gm, x, y, xo, yo);
        x = wrap(xo, gm.b0, gm.Wx);
        y = wrap(yo, gm.b2, gm.Wy);
    }
    const long long i = (long long)iY * gt.NX + iX;
    px[i] = x;
    py[i] = y;
}

cudaError_t launch_compose_fwd(const Grid& gm, const Grid& gt, const double* X, const double* Y, const double* stack,
                               int n_maps, double* px, double* py, cudaStream_t s)
{
    if (gt.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((gt.NX + 255) / 256), (unsigned)gt.NY);
    k_compose_fwd<<<blocks, 256, 0, s>>>(gm, gt, X, Y, stack, n_maps, px, py);
    return cudaGetLastError();
}

// points through one map (k_h_sample_points_map, cmm-simulation-kernel.cu:97-118): a point
// strictly inside the frame is mapped and wrapped by the domain width (floor(x / L) L, the
// reference's wrap), any other point becomes NaN; in and out may alias
__global__ void k_map_points(Grid gm, double f0, double f1, double f2, double f3, const double* __restrict__ X,
                             const double* __restrict__ Y, const double* in, double* out, int num)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    const double x = in[2 * i], y = in[2 * i + 1];
    if (x > f0 && x < f1 && y > f2 && y < f3) {
        double a, b;
        map_value(X, Y, gm, x, y, a, b);
        out[2 * i] = a - floor(a / gm.Wx) * gm.Wx;
        out[2 * i + 1] = b - floor(b / gm.Wy) * gm.Wy;
    } else {
        out[2 * i] = out[2 * i + 1] = __longlong_as_double(0x7ff8000000000000ll);
    }
}

cudaError_t launch_map_points(const Grid& gm, const double* frame, const double* X, const double* Y, const double* in,
                              double* out, int num, cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    k_map_points<<<(num + 255) / 256, 256, 0, s>>>(gm, frame[0], frame[1], frame[2], frame[3], X, Y, in, out, num);
    return cudaGetLastError();
}

// an initial field (analytic kind 0/1/2, or the discrete Hermite field, kind 3) at given positions
__global__ void __launch_bounds__(256) k_eval_init(const double* __restrict__ px, const double* __restrict__ py,
                                                   long long n, InitSource src, double* __restrict__ out)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = px[i], y = py[i];
    out[i] = src.kind == 3 ? interp_value(src.discrete, src.gd, x, y)
                           : init_field(src.kind, x, y, src.ic_num, src.params, src.rand_table);
}

cudaError_t launch_eval_init(const double* px, const double* py, long long n, const InitSource& src, double* out,
                             cudaStream_t s)
{
    k_eval_init<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(px, py, n, src, out);
    return cudaGetLastError();
}

// a Hermite field (src.discrete on src.gd) at the nodes of grid g (k_h_sample,
// src/simulation/cmm-simulation-kernel.cu:122-135)
__global__ void __launch_bounds__(256) k_eval_grid(Grid g, InitSource src, double* __restrict__ out)
{
    const int iX = blockIdx.x * blockDim.x + threadIdx.x, iY = blockIdx.y;
    if (iX >= g.NX) return;
    out[(long long)iY * g.NX + iX] = interp_value(src.discrete, src.gd, g.b0 + iX * g.hx, g.b2 + iY * g.hy);
}

cudaError_t launch_eval_grid(const Grid& g, const InitSource& src, double* out, cudaStream_t s)
{
    if (g.NY > 65535 || !src.discrete) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((g.NX + 255) / 256), (unsigned)g.NY);
    k_eval_grid<<<blocks, 256, 0, s>>>(g, src, out);
    return cudaGetLastError();
}

// normalised spectral operator on a D2Z half spectrum: 0 Laplacian (k_fft_lap_h),
// 1 d/dx, 2 d/dy (k_fft_dx_h, k_fft_dy_h), 3 inverse Laplacian (k_fft_iLap_h);
// cmm-fft.cu:27-78,147-187,326-339
__global__ void k_spec_op(const double2* __restrict__ in, Grid g, int op, double2* __restrict__ out)
{
    const int iX = blockIdx.x * blockDim.x + threadIdx.x, iY = blockIdx.y;
    if (iX >= g.NX_fft) return;
    const long long i = (long long)iY * g.NX_fft + iX;
    double2 v = in[i];
    v.x /= (double)g.N;
    v.y /= (double)g.N;
    const double kx = g.kfx * (iX - (iX > g.NX / 2) * g.NX);
    const double ky = g.kfy * (iY - (iY > g.NY / 2) * g.NY);
    double2 r;
    if (op == 1) r = make_double2(-v.y * kx, v.x * kx);
    else if (op == 2) r = make_double2(-v.y * ky, v.x * ky);
    else if (iX == 0 && iY == 0) r = make_double2(0.0, 0.0);
    else {
        const double k2 = kx * kx + ky * ky;
        r = op == 0 ? make_double2(-v.x * k2, -v.y * k2) : make_double2(-v.x / k2, -v.y / k2);
    }
    out[i] = r;
}

cudaError_t launch_spec_op(const double2* in, const Grid& g, int op, double2* out, cudaStream_t s)
{
    if (g.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((g.NX_fft + 255) / 256), (unsigned)g.NY);
    k_spec_op<<<blocks, 256, 0, s>>>(in, g, op, out);
    return cudaGetLastError();
}

}  // namespace cmm
