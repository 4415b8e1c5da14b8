// aux_kernels.cu -- tracer particles, spectral operators of the Poisson /
// Hermite solve, and deterministic reductions (FP64, sm_103a).
#include <cuda_runtime.h>

#include "kernels.hpp"

namespace cmm {

// ---------------------------------------------------------------------------
// tracer and inertial particles (Particle_advect, src/numerical/cmm-particles.cu:119-276;
// Particle_advect_inertia, :280-551).  psi[0] holds t_{n+1}, psi[1] t_n, psi[2] t_{n-1};
// Lp12 combines the L levels to t_{n+1/2}.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void part_level(const ParticleArgs& a, int l, double x, double y, double& ux, double& uy)
{
    const double* lv[1] = {a.psi[l]};
    double u1[1], v1[1];
    velocity_levels<1>(lv, a.gp, x, y, u1, v1);
    ux = u1[0];
    uy = v1[0];
}

template <int L>
__device__ __forceinline__ void part_half(const ParticleArgs& a, double x, double y, double& kx, double& ky)
{
    double ux[L], uy[L];
    velocity_levels<L>(a.psi, a.gp, x, y, ux, uy);
    kx = a.Lp12[0] * ux[0];
    ky = a.Lp12[0] * uy[0];
#pragma unroll
    for (int l = 1; l < L; ++l) { kx = fma(a.Lp12[l], ux[l], kx); ky = fma(a.Lp12[l], uy[l], ky); }
}

template <int L, int TI>
__global__ void __launch_bounds__(256) k_particles(const ParticleArgs a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.num) return;
    double px = a.pos[2 * i], py = a.pos[2 * i + 1];
    const double dt = a.dt;
    double k1x, k1y, k2x, k2y, k3x, k3y, k4x, k4y;
    part_level(a, 1, px, py, k1x, k1y);
    if (TI == 10) {
        px += dt * k1x;
        py += dt * k1y;
    } else if (TI == 20) {
        part_level(a, 0, px + dt * k1x, py + dt * k1y, k2x, k2y);
        px += dt * (k1x + k2x) / 2;
        py += dt * (k1y + k2y) / 2;
    } else if (TI == 30) {
        part_half<L>(a, px + dt * k1x / 2.0, py + dt * k1y / 2.0, k2x, k2y);
        part_level(a, 0, px - dt * k1x + 2 * dt * k2x, py - dt * k1y + 2 * dt * k2y, k3x, k3y);
        px += dt * (k1x + 4 * k2x + k3x) / 6.0;
        py += dt * (k1y + 4 * k2y + k3y) / 6.0;
    } else if (TI == 40) {
        part_half<L>(a, px + dt * k1x / 2.0, py + dt * k1y / 2.0, k2x, k2y);
        part_half<L>(a, px + dt * k2x / 2.0, py + dt * k2y / 2.0, k3x, k3y);
        part_level(a, 0, px + dt * k3x, py + dt * k3y, k4x, k4y);
        px += dt * (k1x + 2 * k2x + 2 * k3x + k4x) / 6.0;
        py += dt * (k1y + 2 * k2y + 2 * k3y + k4y) / 6.0;
    } else if (TI == 31) {
        part_level(a, 0, px + dt * k1x, py + dt * k1y, k2x, k2y);
        part_level(a, 2, px + dt * (k1x - 2 * k2x), py + dt * (k1y - 2 * k2y), k3x, k3y);
        px += dt * (8 * k1x + 5 * k2x - k3x) / 12.0;
        py += dt * (8 * k1y + 5 * k2y - k3y) / 12.0;
    } else {   // 41
        part_level(a, 0, px + dt * k1x, py + dt * k1y, k2x, k2y);
        part_half<L>(a, px + dt / 8.0 * (3 * k1x + k2x), py + dt / 8.0 * (3 * k1y + k2y), k3x, k3y);
        part_level(a, 0, px + dt / 3.0 * (-k2x + 4 * k3x), py + dt / 3.0 * (-k2y + 4 * k3y), k4x, k4y);
        px += dt * (2 * k1x - k2x + 8 * k3x + 3 * k4x) / 12.0;
        py += dt * (2 * k1y - k2y + 8 * k3y + 3 * k4y) / 12.0;
    }
    a.pos[2 * i] = wrap(px, a.gp.b0, a.gp.Wx);
    a.pos[2 * i + 1] = wrap(py, a.gp.b2, a.gp.Wy);
}

// inertial particles: dx/dt = v, dv/dt = -(v - u(x, t)) / tau.  Each stage s has a position
// increment xs (a velocity) and an acceleration as = -(vs - u(x + ..., t_s)) / tau.
template <int L, int TI>
__global__ void __launch_bounds__(256) k_particles_inertia(const ParticleArgs a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.num) return;
    const double px = a.pos[2 * i], py = a.pos[2 * i + 1];
    const double vx = a.vel[2 * i], vy = a.vel[2 * i + 1];
    const double dt = a.dt, tau = a.tau;
    double ux, uy, nx, ny, nvx, nvy;
    auto acc = [&](double sx, double sy, double& ax, double& ay) { ax = -(sx - ux) / tau; ay = -(sy - uy) / tau; };
    part_level(a, 1, px, py, ux, uy);
    double a1x, a1y;
    acc(vx, vy, a1x, a1y);
    if (TI == 10) {
        nx = px + dt * vx;
        ny = py + dt * vy;
        nvx = vx - dt * (vx - ux) / tau;
        nvy = vy - dt * (vy - uy) / tau;
    } else if (TI == 20) {
        const double x2x = vx + dt * a1x, x2y = vy + dt * a1y;
        double a2x, a2y;
        part_level(a, 0, px + dt * vx, py + dt * vy, ux, uy);
        acc(x2x, x2y, a2x, a2y);
        nx = px + dt / 2.0 * (vx + x2x);
        ny = py + dt / 2.0 * (vy + x2y);
        nvx = vx + dt / 2.0 * (a1x + a2x);
        nvy = vy + dt / 2.0 * (a1y + a2y);
    } else if (TI == 30) {
        const double x2x = vx + dt / 2.0 * a1x, x2y = vy + dt / 2.0 * a1y;
        double a2x, a2y, a3x, a3y;
        part_half<L>(a, px + dt / 2.0 * vx, py + dt / 2.0 * vy, ux, uy);
        acc(x2x, x2y, a2x, a2y);
        const double x3x = vx + dt * (-a1x + 2 * a2x), x3y = vy + dt * (-a1y + 2 * a2y);
        part_level(a, 0, px + dt * (-vx + 2 * x2x), py + dt * (-vy + 2 * x2y), ux, uy);
        acc(x3x, x3y, a3x, a3y);
        nx = px + dt / 6.0 * (vx + 4 * x2x + x3x);
        ny = py + dt / 6.0 * (vy + 4 * x2y + x3y);
        nvx = vx + dt / 6.0 * (a1x + 4 * a2x + a3x);
        nvy = vy + dt / 6.0 * (a1y + 4 * a2y + a3y);
    } else if (TI == 40) {
        const double x2x = vx + dt / 2.0 * a1x, x2y = vy + dt / 2.0 * a1y;
        double a2x, a2y, a3x, a3y, a4x, a4y;
        part_half<L>(a, px + dt / 2.0 * vx, py + dt / 2.0 * vy, ux, uy);
        acc(x2x, x2y, a2x, a2y);
        const double x3x = vx + dt / 2.0 * a2x, x3y = vy + dt / 2.0 * a2y;
        part_half<L>(a, px + dt / 2.0 * x2x, py + dt / 2.0 * x2y, ux, uy);
        acc(x3x, x3y, a3x, a3y);
        const double x4x = vx + dt * a3x, x4y = vy + dt * a3y;
        part_level(a, 0, px + dt * x3x, py + dt * x3y, ux, uy);
        acc(x4x, x4y, a4x, a4y);
        nx = px + dt / 6.0 * (vx + 2 * x2x + 2 * x3x + x4x);
        ny = py + dt / 6.0 * (vy + 2 * x2y + 2 * x3y + x4y);
        nvx = vx + dt / 6.0 * (a1x + 2 * a2x + 2 * a3x + a4x);
        nvy = vy + dt / 6.0 * (a1y + 2 * a2y + 2 * a3y + a4y);
    } else if (TI == 31) {
        const double x2x = vx + dt * a1x, x2y = vy + dt * a1y;
        double a2x, a2y, a3x, a3y;
        part_level(a, 0, px + dt * vx, py + dt * vy, ux, uy);
        acc(x2x, x2y, a2x, a2y);
        const double x3x = vx + dt * (a1x - 2 * a2x), x3y = vy + dt * (a1y - 2 * a2y);
        part_level(a, 2, px + dt * (vx - 2 * x2x), py + dt * (vy - 2 * x2y), ux, uy);
        acc(x3x, x3y, a3x, a3y);
        nx = px + dt / 12.0 * (8 * vx + 5 * x2x - x3x);
        ny = py + dt / 12.0 * (8 * vy + 5 * x2y - x3y);
        nvx = vx + dt / 12.0 * (8 * a1x + 5 * a2x - a3x);
        nvy = vy + dt / 12.0 * (8 * a1y + 5 * a2y - a3y);
    } else {   // 41
        const double x2x = vx + dt * a1x, x2y = vy + dt * a1y;
        double a2x, a2y, a3x, a3y, a4x, a4y;
        part_level(a, 0, px + dt * vx, py + dt * vy, ux, uy);
        acc(x2x, x2y, a2x, a2y);
        const double x3x = vx + dt / 8.0 * (3 * a1x + a2x), x3y = vy + dt / 8.0 * (3 * a1y + a2y);
        part_half<L>(a, px + dt / 8.0 * (3 * vx + x2x), py + dt / 8.0 * (3 * vy + x2y), ux, uy);
        acc(x3x, x3y, a3x, a3y);
        const double x4x = vx + dt / 3.0 * (-a2x + 4 * a3x), x4y = vy + dt / 3.0 * (-a2y + 4 * a3y);
        part_level(a, 0, px + dt / 3.0 * (-x2x + 4 * x3x), py + dt / 3.0 * (-x2y + 4 * x3y), ux, uy);
        acc(x4x, x4y, a4x, a4y);
        nx = px + dt / 12.0 * (2 * vx - x2x + 8 * x3x + 3 * x4x);
        ny = py + dt / 12.0 * (2 * vy - x2y + 8 * x3y + 3 * x4y);
        nvx = vx + dt / 12.0 * (2 * a1x - a2x + 8 * a3x + 3 * a4x);
        nvy = vy + dt / 12.0 * (2 * a1y - a2y + 8 * a3y + 3 * a4y);
    }
    a.pos[2 * i] = wrap(nx, a.gp.b0, a.gp.Wx);
    a.pos[2 * i + 1] = wrap(ny, a.gp.b2, a.gp.Wy);
    a.vel[2 * i] = nvx;
    a.vel[2 * i + 1] = nvy;
}

cudaError_t launch_particles(const ParticleArgs& a, cudaStream_t s)
{
    if (a.num <= 0) return cudaSuccess;
    const int threads = 256;
    const unsigned blocks = (unsigned)((a.num + threads - 1) / threads);
    const bool inert = a.tau != 0;
    if (inert && !a.vel) return cudaErrorInvalidValue;
#define CMM_PART(LL, TT)                                                                    \
    do {                                                                                    \
        if (inert) k_particles_inertia<LL, TT><<<blocks, threads, 0, s>>>(a);               \
        else k_particles<LL, TT><<<blocks, threads, 0, s>>>(a);                             \
    } while (0)
    // level 1 (t_n) is read by every scheme, level 2 by RK3Mod; the half-step
    // combination uses all L levels
    switch (a.time_integration_num * 10 + a.l_order) {
        case 101: case 102: case 103: case 104: CMM_PART(1, 10); break;
        case 202: case 203: case 204: CMM_PART(1, 20); break;
        case 303: CMM_PART(3, 30); break;
        case 304: CMM_PART(4, 30); break;
        case 404: CMM_PART(4, 40); break;
        case 313: case 314: CMM_PART(1, 31); break;
        case 414: CMM_PART(4, 41); break;
        default: return cudaErrorInvalidValue;
    }
#undef CMM_PART
    return cudaGetLastError();
}

__global__ void k_particle_vel_init(const double* __restrict__ pos, int num, const double* __restrict__ psi0, Grid g,
                                    double* __restrict__ vel)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    const double* lv[1] = {psi0};
    double ux[1], uy[1];
    velocity_levels<1>(lv, g, pos[2 * i], pos[2 * i + 1], ux, uy);
    vel[2 * i] = ux[0];
    vel[2 * i + 1] = uy[0];
}

cudaError_t launch_particle_vel_init(const double* pos, int num, const double* psi0, const Grid& gp, double* vel,
                                     cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    k_particle_vel_init<<<(num + 255) / 256, 256, 0, s>>>(pos, num, psi0, gp, vel);
    return cudaGetLastError();
}

__global__ void k_particle_rescale(double* pos, int num, double p0, double p1, double p2, double p3, Grid g)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    double x = p0 + p2 * (pos[2 * i] - 0.5);
    double y = p1 + p3 * (pos[2 * i + 1] - 0.5);
    pos[2 * i] = wrap(x, g.b0, g.Wx);
    pos[2 * i + 1] = wrap(y, g.b2, g.Wy);
}

cudaError_t launch_particle_rescale(double* pos, int num, const double* p4, const Grid& g, cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    k_particle_rescale<<<(num + 255) / 256, 256, 0, s>>>(pos, num, p4[0], p4[1], p4[2], p4[3], g);
    return cudaGetLastError();
}

// deterministic particle layouts (k_part_init_circle / _uniform_grid / _sine_sheets,
// src/simulation/cmm-init.cu:394-451): mode 2 circle, 3 uniform grid, 4 sine sheet
__global__ void k_particle_layout(double* pos, int num, int mode, double p0, double p1, double p2, double p3, Grid g)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    double x, y;
    if (mode == 2) {
        x = p0 + p2 * cos(i / (double)num * kTwoPi);
        y = p1 + p3 * sin(i / (double)num * kTwoPi);
    } else if (mode == 3) {
        int len = (int)ceil(sqrt((double)num));
        x = p0 + p2 * (-1 + 2 * (i % len) / (double)len);
        y = p1 + p3 * (-1 + 2 * (i / len) / (double)len);
    } else {
        x = i / (double)num * kTwoPi + p0;
        y = sin(i / (double)num * kTwoPi) / 2.0 + p1;
    }
    pos[2 * i] = wrap(x, g.b0, g.Wx);
    pos[2 * i + 1] = wrap(y, g.b2, g.Wy);
}

cudaError_t launch_particle_layout(double* pos, int num, int mode, const double* p4, const Grid& g, cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    k_particle_layout<<<(num + 255) / 256, 256, 0, s>>>(pos, num, mode, p4[0], p4[1], p4[2], p4[3], g);
    return cudaGetLastError();
}

__global__ void k_sample_points_dxdy(Grid gp, const double* __restrict__ psi, const double* __restrict__ pos,
                                     double* __restrict__ out, int num)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num) return;
    double x = pos[2 * i], y = pos[2 * i + 1];
    if (x > gp.b0 && x < gp.b1 && y > gp.b2 && y < gp.b3) {
        Cell c = locate(gp, x, y);
        Corners q = load_corners(psi, gp.N, c);
        double gx, gy;
        hermite_grad(q, value_weights(c.tx, gp.hx), value_weights(c.ty, gp.hy), slope_weights(c.tx, gp.ihx),
                     slope_weights(c.ty, gp.ihy), gx, gy);
        out[2 * i] = gx;
        out[2 * i + 1] = gy;
    } else {
        out[2 * i] = out[2 * i + 1] = __longlong_as_double(0x7ff8000000000000ll);
    }
}

cudaError_t launch_sample_points_dxdy(const Grid& gp, const double* psi, const double* pos, double* out, int num,
                                      cudaStream_t s)
{
    if (num <= 0) return cudaSuccess;
    k_sample_points_dxdy<<<(num + 255) / 256, 256, 0, s>>>(gp, psi, pos, out, num);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// spectral operators on D2Z half spectra [NY][NX/2+1]
// (src/numerical/cmm-fft.cu:55-78 iLap, :147-187 dx/dy, :267-286 cut-off,
//  :294-323 grid move, :326-339 normalise, :398-429 fourier_hermite)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void hermite_spectra(double2 P, double kx, double ky, long long idx, long long nf,
                                                double2* __restrict__ out4)
{
    double2 Px = make_double2(-P.y * kx, P.x * kx);
    double2 Py = make_double2(-P.y * ky, P.x * ky);
    double2 Pxy = make_double2(-Py.y * kx, Py.x * kx);
    out4[idx] = P;
    out4[nf + idx] = Px;
    out4[2 * nf + idx] = Py;
    out4[3 * nf + idx] = Pxy;
}

__global__ void k_spec_hermite(const double2* __restrict__ F, Grid g, double2* __restrict__ out4)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g.Nfft) return;
    int iX = (int)(i % g.NX_fft), iY = (int)(i / g.NX_fft);
    double2 f = F[i];
    double2 P = make_double2(f.x / (double)g.N, f.y / (double)g.N);
    double kx = g.kfx * (iX - (iX > g.NX / 2) * g.NX);
    double ky = g.kfy * (iY - (iY > g.NY / 2) * g.NY);
    hermite_spectra(P, kx, ky, i, g.Nfft, out4);
}

cudaError_t launch_spec_hermite(const double2* F, const Grid& g, double2* out4, cudaStream_t s)
{
    k_spec_hermite<<<(unsigned)((g.Nfft + 255) / 256), 256, 0, s>>>(F, g, out4);
    return cudaGetLastError();
}

__global__ void k_spec_psi(const double2* __restrict__ Fv, Grid gv, Grid gp, double freq, double2* __restrict__ out4)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= gp.Nfft) return;
    int iXc = (int)(i % gp.NX_fft), iYc = (int)(i / gp.NX_fft);
    double2 P = make_double2(0.0, 0.0);
    // grid move (zero pad or truncate) from the vorticity grid spectrum
    bool outside = (iXc + (iXc > gp.NX / 2.0) * (gp.NX - 2 * iXc) > gv.NX / 2.0) ||
                   (iYc + (iYc > gp.NY / 2.0) * (gp.NY - 2 * iYc) > gv.NY / 2.0);
    if (!outside) {
        int iXs = iXc + (iXc > gp.NX / 2.0) * (gv.NX - gp.NX);
        int iYs = iYc + (iYc > gp.NY / 2.0) * (gv.NY - gp.NY);
        double2 f = Fv[(long long)iYs * gv.NX_fft + iXs];
        P = make_double2(f.x / (double)gv.N, f.y / (double)gv.N);
    }
    // circular low-pass, also removes the mean mode
    int fX = iXc + (iXc > gp.NX / 2.0) * (gp.NX - 2 * iXc);
    int fY = iYc + (iYc > gp.NY / 2.0) * (gp.NY - 2 * iYc);
    if ((double)(fX * fX + fY * fY) > freq * freq || i == 0) P = make_double2(0.0, 0.0);
    double kx = gp.kfx * (iXc - (iXc > gp.NX / 2) * gp.NX);
    double ky = gp.kfy * (iYc - (iYc > gp.NY / 2) * gp.NY);
    // inverse Laplacian
    if (iXc == 0 && iYc == 0) P = make_double2(0.0, 0.0);
    else {
        double k2 = kx * kx + ky * ky;
        P = make_double2(-P.x / k2, -P.y / k2);
    }
    hermite_spectra(P, kx, ky, i, gp.Nfft, out4);
}

cudaError_t launch_spec_psi(const double2* Fv, const Grid& gv, const Grid& gp, double freq, double2* out4,
                            cudaStream_t s)
{
    k_spec_psi<<<(unsigned)((gp.Nfft + 255) / 256), 256, 0, s>>>(Fv, gv, gp, freq, out4);
    return cudaGetLastError();
}

__global__ void k_spec_grad(const double2* __restrict__ F, Grid g, double2* __restrict__ out2)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g.Nfft) return;
    int iX = (int)(i % g.NX_fft), iY = (int)(i / g.NX_fft);
    double2 f = F[i];
    double2 P = make_double2(f.x / (double)g.N, f.y / (double)g.N);
    double kx = g.kfx * (iX - (iX > g.NX / 2) * g.NX);
    double ky = g.kfy * (iY - (iY > g.NY / 2) * g.NY);
    out2[i] = make_double2(-P.y * kx, P.x * kx);
    out2[g.Nfft + i] = make_double2(-P.y * ky, P.x * ky);
}

cudaError_t launch_spec_grad(const double2* F, const Grid& g, double2* out2, cudaStream_t s)
{
    k_spec_grad<<<(unsigned)((g.Nfft + 255) / 256), 256, 0, s>>>(F, g, out2);
    return cudaGetLastError();
}

bool make_plans(FftPlans& p, const Grid& g, cudaStream_t s)
{
    p.g = g;
    p.ok = fft::plan_create(p.p, g.NX, g.NY, true, s) == 0;
    return p.ok;
}

void destroy_plans(FftPlans& p)
{
    fft::plan_destroy(p.p);
    p.ok = false;
}

cudaError_t fft_d2z(const FftPlans& p, const double* in, double2* out, cudaStream_t s)
{
    return fft::r2c(p.p, in, out, 1, s);
}

cudaError_t fft_z2d(const FftPlans& p, double2* in, double* out, int batch, cudaStream_t s)
{
    return fft::c2r(p.p, in, out, batch, s);
}

// ---------------------------------------------------------------------------
// deterministic two-pass reductions (fixed grid, fixed order)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_stats_partial(const double* __restrict__ v, long long n, long long stride,
                                                       double* __restrict__ part)
{
    __shared__ double smin[256], smax[256], ssum[256];
    double mn = __longlong_as_double(0x7ff0000000000000ll), mx = -mn, sm = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double x = v[i * stride];
        mn = fmin(mn, x);
        mx = fmax(mx, x);
        sm += x;
    }
    smin[threadIdx.x] = mn; smax[threadIdx.x] = mx; ssum[threadIdx.x] = sm;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
            ssum[threadIdx.x] += ssum[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = smin[0];
        part[3 * blockIdx.x + 1] = smax[0];
        part[3 * blockIdx.x + 2] = ssum[0];
    }
}

__global__ void k_stats_final(const double* __restrict__ part, int nb, double* __restrict__ out)
{
    __shared__ double smin[256], smax[256], ssum[256];
    double mn = __longlong_as_double(0x7ff0000000000000ll), mx = -mn, sm = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        mn = fmin(mn, part[3 * b]);
        mx = fmax(mx, part[3 * b + 1]);
        sm += part[3 * b + 2];
    }
    smin[threadIdx.x] = mn; smax[threadIdx.x] = mx; ssum[threadIdx.x] = sm;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
            ssum[threadIdx.x] += ssum[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = smin[0];
        out[1] = smax[0];
        out[2] = fmax(0.0, smax[0]);
        out[3] = ssum[0];
    }
}

cudaError_t launch_stats(const double* v, long long n, long long stride, double* d_scratch, double* d_out,
                         cudaStream_t s)
{
    long long need = (n + 255) / 256;
    int nb = (int)(need < kReduceBlocks ? (need > 0 ? need : 1) : kReduceBlocks);
    k_stats_partial<<<nb, 256, 0, s>>>(v, n, stride, d_scratch);
    k_stats_final<<<1, 256, 0, s>>>(d_scratch, nb, d_out);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) k_sumsq_partial(const double* __restrict__ v, long long n,
                                                       double* __restrict__ part)
{
    __shared__ double ssum[256];
    double sm = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        sm = fma(v[i], v[i], sm);
    ssum[threadIdx.x] = sm;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) ssum[threadIdx.x] += ssum[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = ssum[0];
}

__global__ void k_sum_final(const double* __restrict__ part, int nb, double* __restrict__ out)
{
    __shared__ double ssum[256];
    double sm = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) sm += part[b];
    ssum[threadIdx.x] = sm;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) ssum[threadIdx.x] += ssum[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = ssum[0];
}

cudaError_t launch_sumsq(const double* v, long long n, double* d_scratch, double* d_out, cudaStream_t s)
{
    long long need = (n + 255) / 256;
    int nb = (int)(need < kReduceBlocks ? (need > 0 ? need : 1) : kReduceBlocks);
    k_sumsq_partial<<<nb, 256, 0, s>>>(v, n, d_scratch);
    k_sum_final<<<1, 256, 0, s>>>(d_scratch, nb, d_out);
    return cudaGetLastError();
}

}  // namespace cmm
