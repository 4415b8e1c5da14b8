// vlasov_kernels.cu -- Vlasov-Poisson potential and diagnostics (sm_103a).
//
// The v-integral is a column sum over the vort grid done in row chunks (one
// coalesced pass, partial sums reduced in a fixed order); the Poisson solve
// and the periodification h(v) are 1D spectra; the Hermite planes of the
// separable psi are written directly (see vlasov.hpp).
#include <cuda_runtime.h>

#include "vlasov.hpp"

namespace cmm {

bool make_vlasov_plans(VlasovPlans& p, const Grid& gv, const Grid& gp, cudaStream_t s)
{
    return fft::plan_create_rows(p.v, gv.NX, true, s) == 0 && fft::plan_create_rows(p.p, gp.NX, true, s) == 0;
}

void destroy_vlasov_plans(VlasovPlans& p)
{
    fft::plan_destroy(p.v);
    fft::plan_destroy(p.p);
}

cudaError_t fft_d2z_1d(const fft::Plan2D& p, const double* in, double2* out, cudaStream_t s)
{
    return fft::rows_r2c(p, in, p.nx, p.nx, out, p.nx / 2 + 1, p.nx / 2 + 1, 1, 1, p.nx / 2 + 1, s);
}

cudaError_t fft_z2d_1d(const fft::Plan2D& p, const double2* in, double* out, cudaStream_t s)
{
    return fft::rows_c2r(p, in, p.nx / 2 + 1, p.nx / 2 + 1, p.nx / 2 + 1, out, p.nx, p.nx, 1, 1, s);
}

// ---------------------------------------------------------------- v-integral
template <typename T>
__global__ void __launch_bounds__(256) k_vlasov_rho_partial(const T* __restrict__ f, int nx, int ny,
                                                            double* __restrict__ partial)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (ix >= nx) return;
    const int y0 = c * kVlasovRowChunk, y1 = min(ny, y0 + kVlasovRowChunk);
    double acc = 0.0;
    for (int iy = y0; iy < y1; ++iy) acc += (double)f[(long long)iy * nx + ix];
    partial[(long long)c * nx + ix] = acc;
}

template <typename T>
__global__ void k_vlasov_rho_final(const T* __restrict__ f, const double* __restrict__ partial, int nx, int nchunks,
                                   double hy, double* __restrict__ rho)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    if (ix >= nx) return;
    double acc = (double)f[ix];   // row 0 once more: the reference's output aliases it
    for (int c = 0; c < nchunks; ++c) acc += partial[(long long)c * nx + ix];
    acc *= hy;
    rho[ix] = acc + -1.0;
}

cudaError_t launch_vlasov_rho(const double* fd, const float* ff, const Grid& gv, double* partial, double* rho,
                              cudaStream_t s)
{
    const int nchunks = (gv.NY + kVlasovRowChunk - 1) / kVlasovRowChunk;
    dim3 blocks((unsigned)((gv.NX + 255) / 256), (unsigned)nchunks);
    unsigned b1 = (unsigned)((gv.NX + 255) / 256);
    if (fd) {
        k_vlasov_rho_partial<double><<<blocks, 256, 0, s>>>(fd, gv.NX, gv.NY, partial);
        k_vlasov_rho_final<double><<<b1, 256, 0, s>>>(fd, partial, gv.NX, nchunks, gv.hy, rho);
    } else {
        k_vlasov_rho_partial<float><<<blocks, 256, 0, s>>>(ff, gv.NX, gv.NY, partial);
        k_vlasov_rho_final<float><<<b1, 256, 0, s>>>(ff, partial, gv.NX, nchunks, gv.hy, rho);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- 1D spectra
// derivative spectrum i k F; the Nyquist bin of a real signal's derivative is
// dropped by a complex-to-real transform, so it is written as zero
__device__ __forceinline__ double2 ik_times(double2 v, double k, bool nyquist)
{
    return nyquist ? make_double2(0.0, 0.0) : make_double2(-v.y * k, v.x * k);
}

__global__ void k_vlasov_phi_spec(const double2* __restrict__ rho_hat, Grid gv, Grid gp, double2* __restrict__ phi_hat,
                                  double2* __restrict__ dphi_hat)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= gp.NX_fft) return;
    double2 v = make_double2(0.0, 0.0);
    if (i > 0 && 2 * i <= gv.NX) {   // modes beyond the vort grid's half spectrum are zero padding
        double2 r = rho_hat[i];
        r.x /= (double)gv.NX;
        r.y /= (double)gv.NX;
        double kx = gv.kfx * i, k2 = kx * kx;
        v = make_double2(r.x / k2, r.y / k2);
    }
    phi_hat[i] = v;
    dphi_hat[i] = ik_times(v, gp.kfx * i, 2 * i == gp.NX);
}

cudaError_t launch_vlasov_phi_spec(const double2* rho_hat, const Grid& gv, const Grid& gp, double2* phi_hat,
                                   double2* dphi_hat, cudaStream_t s)
{
    k_vlasov_phi_spec<<<(unsigned)((gp.NX_fft + 255) / 256), 256, 0, s>>>(rho_hat, gv, gp, phi_hat, dphi_hat);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(1024) k_vlasov_bump(Grid gp, double* __restrict__ sigma)
{
    __shared__ double red[1024];
    const int n = gp.NY;
    const double PI = kTwoPi / 2, Lv = gp.b3 - gp.b2, a = 0.4, b = 0.1;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double v = gp.b2 + i * gp.hy;
        double sg = 0.5 - 0.5 * tanh(2 * PI * (fabs(v) - a * Lv) / (b * Lv));
        sigma[i] = sg;
        acc += sg;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double mean = red[0] / (double)n;
    __syncthreads();
    double mx = -1e300;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double sg = sigma[i] - mean;
        sigma[i] = sg;
        mx = fmax(mx, sg);
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    const double max_v = red[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) sigma[i] = sigma[i] / max_v;
}

cudaError_t launch_vlasov_bump(const Grid& gp, double* sigma, cudaStream_t s)
{
    k_vlasov_bump<<<1, 1024, 0, s>>>(gp, sigma);
    return cudaGetLastError();
}

__global__ void k_vlasov_h_spec(const double2* __restrict__ sig_hat, Grid gp, double2* __restrict__ h_hat,
                                double2* __restrict__ dh_hat)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nfft = gp.NY / 2 + 1;
    if (i >= nfft) return;
    double2 v = make_double2(0.0, 0.0);
    if (i > 0) {
        double2 r = sig_hat[i];
        r.x /= (double)gp.NY;
        r.y /= (double)gp.NY;
        double ky = gp.kfy * i, k2 = ky * ky;
        v = make_double2(r.x / k2, r.y / k2);
    }
    h_hat[i] = v;
    dh_hat[i] = ik_times(v, gp.kfy * i, 2 * i == gp.NY);
}

cudaError_t launch_vlasov_h_spec(const double2* sig_hat, const Grid& gp, double2* h_hat, double2* dh_hat,
                                 cudaStream_t s)
{
    k_vlasov_h_spec<<<(unsigned)((gp.NY / 2 + 1 + 255) / 256), 256, 0, s>>>(sig_hat, gp, h_hat, dh_hat);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- psi planes
__global__ void k_vlasov_assemble(const double* __restrict__ phi, const double* __restrict__ dphi,
                                  const double* __restrict__ h, const double* __restrict__ dh, Grid gp,
                                  double* __restrict__ psi4)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y;
    if (ix >= gp.NX) return;
    const long long i = (long long)iy * gp.NX + ix;
    psi4[i] = phi[ix] - h[iy];
    psi4[gp.N + i] = dphi[ix];
    psi4[2 * gp.N + i] = -dh[iy];
    psi4[3 * gp.N + i] = 0.0;
}

cudaError_t launch_vlasov_assemble(const double* phi, const double* dphi, const double* h, const double* dh,
                                   const Grid& gp, double* psi4, cudaStream_t s)
{
    if (gp.NY > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)((gp.NX + 255) / 256), (unsigned)gp.NY);
    k_vlasov_assemble<<<blocks, 256, 0, s>>>(phi, dphi, h, dh, gp, psi4);
    return cudaGetLastError();
}

// phi, phi' of a separable psi's Hermite planes (a psi level read back at a restart):
// row 0 of psi + h(v_0) and row 0 of psi_x
__global__ void k_vlasov_phi_from_psi(const double* __restrict__ psi4, const double* __restrict__ h, Grid gp,
                                      double* __restrict__ phi)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    if (ix >= gp.NX) return;
    phi[ix] = psi4[ix] + h[0];
    phi[gp.NX + ix] = psi4[gp.N + ix];
}

cudaError_t launch_vlasov_phi_from_psi(const double* psi4, const double* h, const Grid& gp, double* phi, cudaStream_t s)
{
    k_vlasov_phi_from_psi<<<(unsigned)((gp.NX + 255) / 256), 256, 0, s>>>(psi4, h, gp, phi);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- diagnostics
__global__ void __launch_bounds__(256) k_vlasov_moments_partial(const double* __restrict__ f, Grid gc,
                                                                double* __restrict__ partial)
{
    __shared__ double s0[256], s1[256], s2[256];
    double a0 = 0, a1 = 0, a2 = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < gc.N; i += (long long)gridDim.x * blockDim.x) {
        const int iy = (int)(i / gc.NX);
        const double v = gc.b2 + iy * gc.hy, fv = f[i];
        a0 += fv;
        a1 += v * fv;
        a2 += v * v * fv;
    }
    s0[threadIdx.x] = a0; s1[threadIdx.x] = a1; s2[threadIdx.x] = a2;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s0[threadIdx.x] += s0[threadIdx.x + o];
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[3 * blockIdx.x] = s0[0];
        partial[3 * blockIdx.x + 1] = s1[0];
        partial[3 * blockIdx.x + 2] = s2[0];
    }
}

__global__ void k_vlasov_moments_final(const double* __restrict__ partial, int nb, double* __restrict__ out3)
{
    __shared__ double s[3][256];
    double a[3] = {0, 0, 0};
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        for (int k = 0; k < 3; ++k) a[k] += partial[3 * b + k];
    for (int k = 0; k < 3; ++k) s[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int k = 0; k < 3; ++k) s[k][threadIdx.x] += s[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) for (int k = 0; k < 3; ++k) out3[k] = s[k][0];
}

cudaError_t launch_vlasov_moments(const double* f, const Grid& gc, double* partial, double* out3, cudaStream_t s)
{
    long long need = (gc.N + 255) / 256;
    int nb = (int)(need < kReduceBlocks ? (need > 0 ? need : 1) : kReduceBlocks);
    k_vlasov_moments_partial<<<nb, 256, 0, s>>>(f, gc, partial);
    k_vlasov_moments_final<<<1, 256, 0, s>>>(partial, nb, out3);
    return cudaGetLastError();
}

struct LevelPtrs { const double* p[kMaxLagrange]; double c[kMaxLagrange]; };

__global__ void k_vlasov_table(LevelPtrs lv, int n_levels, int n, double2* __restrict__ table)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int i1 = i + 1 == n ? 0 : i + 1;
    double d = 0.0, sl = 0.0;
    for (int l = 0; l < n_levels; ++l) {
        d += lv.c[l] * (lv.p[l][i1] - lv.p[l][i]);
        sl += lv.c[l] * lv.p[l][n + i];
    }
    table[i] = make_double2(d, sl);
}

cudaError_t launch_vlasov_table(const double* const* levels, const double* coef, int n_levels, int n, double2* table,
                                cudaStream_t s)
{
    if (n_levels < 1 || n_levels > kMaxLagrange) return cudaErrorInvalidValue;
    LevelPtrs lv{};
    for (int l = 0; l < n_levels; ++l) { lv.p[l] = levels[l]; lv.c[l] = coef[l]; }
    k_vlasov_table<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(lv, n_levels, n, table);
    return cudaGetLastError();
}

__global__ void k_vlasov_modes(const double2* __restrict__ spec, int n, int nfft, double* __restrict__ out4)
{
    if (threadIdx.x >= 4) return;
    int k = (int)threadIdx.x + 1 < nfft ? (int)threadIdx.x + 1 : nfft - 1;
    double2 v = spec[k];
    double re = v.x / (double)n, im = v.y / (double)n;
    out4[threadIdx.x] = sqrt(re * re + im * im);
}

cudaError_t launch_vlasov_modes(const double2* spec, int n, int nfft, double* out4, cudaStream_t s)
{
    k_vlasov_modes<<<1, 32, 0, s>>>(spec, n, nfft, out4);
    return cudaGetLastError();
}

}  // namespace cmm
