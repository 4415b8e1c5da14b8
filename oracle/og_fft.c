/*
 * og_fft.c -- FP64 2D real FFTs and the spectral operators of the ψ solve.
 *
 * TEST INFRASTRUCTURE ONLY (parity oracle; see cmm_oracle.h).
 *
 * The reference calls cuFFT (D2Z / Z2D plans of src/grid/cmm-grid2d.cu:123-131).
 * cuFFT is a closed library, so this file computes the same mathematical
 * transforms with a textbook mixed-radix (2, 3, 5, generic) decimation-in-time
 * Cooley-Tukey FFT:
 *   D2Z:  X[ky][kx] = sum_{y,x} f[y][x] exp(-2 pi i (kx x/NX + ky y/NY)),  kx <= NX/2
 *   Z2D:  f[y][x]  = sum_{ky,kx} X[ky][kx] exp(+2 pi i (...)) over the Hermitian
 *         extension, unnormalised; imaginary parts of the kx = 0 and kx = NX/2
 *         columns are ignored in the final real-axis transform (C2R convention).
 * The spectral point-wise operators restate src/numerical/cmm-fft.cu:28-78,
 * 147-187, 267-339 and fourier_hermite :398-429.
 */
#include "cmm_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OG_TWO_PI 6.283185307179586476925286766559005768394338798750211641949889184615632812572417997256069650684234136

/* recursive mixed-radix complex DFT, out-of-place, stride-aware.
 * sign = -1 forward, +1 inverse.  n = length, in[k*stride]. */
static void fft_rec(const double* in, double* out, long n, long stride, int sign, const double* tw, long tw_n)
{
    if (n == 1) { out[0] = in[0]; out[1] = in[1]; return; }
    long p = 0;
    if (n % 4 == 0) p = 4; else if (n % 2 == 0) p = 2; else if (n % 3 == 0) p = 3; else if (n % 5 == 0) p = 5;
    else p = n;  /* generic prime: direct DFT */
    long m = n / p;
    if (p == n) {
        for (long k = 0; k < n; ++k) {
            double sr = 0, si = 0;
            for (long j = 0; j < n; ++j) {
                long idx = ((k * j) % n) * (tw_n / n);
                double c = tw[2 * idx], s = sign * tw[2 * idx + 1];
                double ar = in[2 * j * stride], ai = in[2 * j * stride + 1];
                sr += ar * c - ai * s; si += ar * s + ai * c;
            }
            out[2 * k] = sr; out[2 * k + 1] = si;
        }
        return;
    }
    /* sub-transforms of the p decimated sequences */
    for (long r = 0; r < p; ++r)
        fft_rec(in + 2 * r * stride, out + 2 * r * m, m, stride * p, sign, tw, tw_n);
    /* butterflies */
    double tmp[2 * 5], res[2 * 5];
    for (long k = 0; k < m; ++k) {
        for (long r = 0; r < p; ++r) {
            long idx = (r * k) * (tw_n / n);
            double c = tw[2 * idx], s = sign * tw[2 * idx + 1];
            double ar = out[2 * (r * m + k)], ai = out[2 * (r * m + k) + 1];
            tmp[2 * r] = ar * c - ai * s; tmp[2 * r + 1] = ar * s + ai * c;
        }
        for (long q = 0; q < p; ++q) {
            double sr = 0, si = 0;
            for (long r = 0; r < p; ++r) {
                long idx = ((q * r) % p) * (tw_n / p);
                double c = tw[2 * idx], s = sign * tw[2 * idx + 1];
                sr += tmp[2 * r] * c - tmp[2 * r + 1] * s;
                si += tmp[2 * r] * s + tmp[2 * r + 1] * c;
            }
            res[2 * q] = sr; res[2 * q + 1] = si;
        }
        for (long q = 0; q < p; ++q) {
            out[2 * (q * m + k)] = res[2 * q];
            out[2 * (q * m + k) + 1] = res[2 * q + 1];
        }
    }
}

/* twiddles exp(-2 pi i k / n): tw[2k] = cos, tw[2k+1] = -sin (sign applied later) */
static double* make_twiddles(long n)
{
    double* tw = (double*)malloc(sizeof(double) * 2 * n);
    for (long k = 0; k < n; ++k) {
        double a = OG_TWO_PI * (double)k / (double)n;
        tw[2 * k] = cos(a); tw[2 * k + 1] = -sin(a);
    }
    return tw;
}

static void fft_1d(const double* in, double* out, long n, int sign, const double* tw)
{
    /* sign convention: tw holds exp(-i...), fft_rec multiplies the sin part by sign... */
    /* forward (sign=-1) wants exp(-i a) = cos - i sin -> s = -sin = tw[1]; passing sign=+1
     * to fft_rec keeps tw as is; inverse flips.  */
    fft_rec(in, out, n, 1, sign == -1 ? 1 : -1, tw, n);
}

/* 2D D2Z of a real NY x NX row-major field -> NY x (NX/2+1) complex */
void og_fft_d2z(const og_grid* g, const double* in, double* out_c)
{
    int NX = g->NX, NY = g->NY, NXf = g->NX_fft;
    double* twx = make_twiddles(NX);
    double* twy = make_twiddles(NY);
    /* rows */
    #pragma omp parallel
    {
        double* a = (double*)malloc(sizeof(double) * 2 * (NX > NY ? NX : NY));
        double* b = (double*)malloc(sizeof(double) * 2 * (NX > NY ? NX : NY));
        #pragma omp for schedule(static)
        for (int iy = 0; iy < NY; ++iy) {
            for (int ix = 0; ix < NX; ++ix) { a[2 * ix] = in[(long)iy * NX + ix]; a[2 * ix + 1] = 0.0; }
            fft_1d(a, b, NX, -1, twx);
            memcpy(out_c + 2L * iy * NXf, b, sizeof(double) * 2 * NXf);
        }
        #pragma omp for schedule(static)
        for (int kx = 0; kx < NXf; ++kx) {
            for (int iy = 0; iy < NY; ++iy) {
                a[2 * iy] = out_c[2L * (iy * (long)NXf + kx)];
                a[2 * iy + 1] = out_c[2L * (iy * (long)NXf + kx) + 1];
            }
            fft_1d(a, b, NY, -1, twy);
            for (int iy = 0; iy < NY; ++iy) {
                out_c[2L * (iy * (long)NXf + kx)] = b[2 * iy];
                out_c[2L * (iy * (long)NXf + kx) + 1] = b[2 * iy + 1];
            }
        }
        free(a); free(b);
    }
    free(twx); free(twy);
}

/* 2D Z2D: NY x (NX/2+1) complex -> NY x NX real (unnormalised) */
void og_fft_z2d(const og_grid* g, const double* in_c, double* out)
{
    int NX = g->NX, NY = g->NY, NXf = g->NX_fft;
    double* twx = make_twiddles(NX);
    double* twy = make_twiddles(NY);
    double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)NXf * NY);
    #pragma omp parallel
    {
        int nmax = NX > NY ? NX : NY;
        double* a = (double*)malloc(sizeof(double) * 2 * nmax);
        double* b = (double*)malloc(sizeof(double) * 2 * nmax);
        #pragma omp for schedule(static)
        for (int kx = 0; kx < NXf; ++kx) {
            for (int iy = 0; iy < NY; ++iy) {
                a[2 * iy] = in_c[2L * (iy * (long)NXf + kx)];
                a[2 * iy + 1] = in_c[2L * (iy * (long)NXf + kx) + 1];
            }
            fft_1d(a, b, NY, +1, twy);
            for (int iy = 0; iy < NY; ++iy) {
                tmp[2L * (iy * (long)NXf + kx)] = b[2 * iy];
                tmp[2L * (iy * (long)NXf + kx) + 1] = b[2 * iy + 1];
            }
        }
        #pragma omp for schedule(static)
        for (int iy = 0; iy < NY; ++iy) {
            const double* row = tmp + 2L * iy * NXf;
            for (int k = 0; k < NX; ++k) {
                double re, im;
                if (k < NXf) { re = row[2 * k]; im = row[2 * k + 1]; }
                else { re = row[2 * (NX - k)]; im = -row[2 * (NX - k) + 1]; }
                if (k == 0 || (NX % 2 == 0 && k == NX / 2)) im = 0.0;
                a[2 * k] = re; a[2 * k + 1] = im;
            }
            fft_1d(a, b, NX, +1, twx);
            for (int ix = 0; ix < NX; ++ix) out[(long)iy * NX + ix] = b[2 * ix];
        }
        free(a); free(b);
    }
    free(tmp); free(twx); free(twy);
}

/* k_normalize_h: cmm-fft.cu:326-339 */
void og_normalize_h(double* F, const og_grid* g)
{
    long n = g->Nfft;
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) { F[2 * i] /= (double)g->N; F[2 * i + 1] /= (double)g->N; }
}

/* k_fft_grid_move: cmm-fft.cu:294-323 (spectral zero-pad / truncate) */
void og_fft_grid_move(const double* in_c, double* out_c, const og_grid* gout, const og_grid* gin)
{
    #pragma omp parallel for schedule(static)
    for (int iYc = 0; iYc < gout->NY; ++iYc) {
        for (int iXc = 0; iXc < gout->NX_fft; ++iXc) {
            long Inc = (long)iYc * gout->NX_fft + iXc;
            if ((iXc + (iXc > gout->NX / 2.0) * (gout->NX - 2 * iXc) > gin->NX / 2.0) ||
                (iYc + (iYc > gout->NY / 2.0) * (gout->NY - 2 * iYc) > gin->NY / 2.0)) {
                out_c[2 * Inc] = out_c[2 * Inc + 1] = 0;
            } else {
                int iXs = iXc + (iXc > gout->NX / 2.0) * (gin->NX - gout->NX);
                int iYs = iYc + (iYc > gout->NY / 2.0) * (gin->NY - gout->NY);
                long Ins = (long)iYs * gin->NX_fft + iXs;
                out_c[2 * Inc] = in_c[2 * Ins];
                out_c[2 * Inc + 1] = in_c[2 * Ins + 1];
            }
        }
    }
}

/* k_fft_cut_off_scale_h: cmm-fft.cu:267-286 */
void og_fft_cut_off_scale_h(double* W, const og_grid* g, double freq)
{
    int NXf = (int)(g->NX / 2.0 + 1);
    #pragma omp parallel for schedule(static)
    for (int iY0 = 0; iY0 < g->NY; ++iY0) {
        for (int iX0 = 0; iX0 < NXf; ++iX0) {
            long In = (long)iY0 * NXf + iX0;
            int iX = iX0 + (iX0 > g->NX / 2.0) * (g->NX - 2 * iX0);
            int iY = iY0 + (iY0 > g->NY / 2.0) * (g->NY - 2 * iY0);
            if ((iX * iX + iY * iY) > freq * freq || In == 0) { W[2 * In] = 0; W[2 * In + 1] = 0; }
        }
    }
}

static inline double kx_of(const og_grid* g, int iX)
{
    return OG_TWO_PI / (g->hx * g->NX) * (iX - (iX > g->NX / 2) * g->NX);
}
static inline double ky_of(const og_grid* g, int iY)
{
    return OG_TWO_PI / (g->hy * g->NY) * (iY - (iY > g->NY / 2) * g->NY);
}

/* k_fft_iLap_h: cmm-fft.cu:55-78 */
void og_fft_iLap_h(const double* in_c, double* out_c, const og_grid* g)
{
    #pragma omp parallel for schedule(static)
    for (int iY = 0; iY < g->NY; ++iY) {
        for (int iX = 0; iX < g->NX_fft; ++iX) {
            long In = (long)iY * g->NX_fft + iX;
            if (iX == 0 && iY == 0) { out_c[0] = out_c[1] = 0; continue; }
            double kx = kx_of(g, iX), ky = ky_of(g, iY);
            double k2 = kx * kx + ky * ky;
            double re = in_c[2 * In], im = in_c[2 * In + 1];
            out_c[2 * In] = -re / k2;
            out_c[2 * In + 1] = -im / k2;
        }
    }
}

/* k_fft_dx_h: cmm-fft.cu:147-165 */
void og_fft_dx_h(const double* in_c, double* out_c, const og_grid* g)
{
    #pragma omp parallel for schedule(static)
    for (int iY = 0; iY < g->NY; ++iY) {
        for (int iX = 0; iX < g->NX_fft; ++iX) {
            long In = (long)iY * g->NX_fft + iX;
            double kx = kx_of(g, iX);
            double re = in_c[2 * In], im = in_c[2 * In + 1];
            out_c[2 * In] = -im * kx;
            out_c[2 * In + 1] = re * kx;
        }
    }
}

/* k_fft_dy_h: cmm-fft.cu:169-187 */
void og_fft_dy_h(const double* in_c, double* out_c, const og_grid* g)
{
    #pragma omp parallel for schedule(static)
    for (int iY = 0; iY < g->NY; ++iY) {
        double ky = ky_of(g, iY);
        for (int iX = 0; iX < g->NX_fft; ++iX) {
            long In = (long)iY * g->NX_fft + iX;
            double re = in_c[2 * In], im = in_c[2 * In + 1];
            out_c[2 * In] = -im * ky;
            out_c[2 * In + 1] = re * ky;
        }
    }
}

/* fourier_hermite: cmm-fft.cu:398-429 -> out4 = [f, f_x, f_y, f_xy] planes */
void og_fourier_hermite(const og_grid* g, const double* in_c, double* out4)
{
    long N = g->N, Nfft = g->Nfft;
    double* t1 = (double*)malloc(sizeof(double) * 2 * Nfft);
    double* t2 = (double*)malloc(sizeof(double) * 2 * Nfft);
    og_fft_dy_h(in_c, t1, g);          /* dy */
    og_fft_dx_h(t1, t2, g);            /* dx dy */
    og_fft_z2d(g, t2, out4 + 3 * N);
    og_fft_z2d(g, t1, out4 + 2 * N);
    og_fft_dx_h(in_c, t1, g);          /* dx */
    og_fft_z2d(g, t1, out4 + 1 * N);
    og_fft_z2d(g, in_c, out4);
    free(t1); free(t2);
}
