/*
 * og_sample.c -- CPU restatement of the sampled outputs of the reference
 * (sample_compute_and_write, src/simulation/cmm-simulation-host.cu:706-893,
 * backward-map part).  TEST INFRASTRUCTURE ONLY (see cmm_oracle.h).
 *
 * On a sample grid gs: the full backward map (current map, then the stacked
 * maps newest to oldest, wrapped after each), the passive scalar and the
 * vorticity evaluated there (k_h_sample_from_init), and from the vorticity by
 * spectral operators its Laplacian, gradient, stream function (inverse
 * Laplacian without cut-off) and the velocity (the reference stores
 * d psi/dx as Velocity_UX and d psi/dy as Velocity_UY); the conservation
 * values on gs with two quirks kept: "Max_vorticity" is max(w_max, -w_max)
 * because both extremes are taken with Compute_max (:807-809), and
 * "Scalar_integral" is hx hy max(0, max theta) because Compute_avg reduces with
 * thrust::maximum (src/numerical/cmm-mesure.cu:226-229).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cmm_oracle.h"

#define OG_PI_S 3.141592653589793238462643383279502884197169399375105820974944592307816406286
#define OG_TWO_PI_S 6.283185307179586476925286766559005768394338798750211641949889184615632812572417997256069650684234136

/* d_init_scalar: src/simulation/cmm-init.cu:253-298 */
double og_init_scalar(double x, double y, int scalar_num)
{
    switch (scalar_num) {
        case 0: { /* rectangle */
            x -= floor(x / OG_TWO_PI_S) * OG_TWO_PI_S;
            y -= floor(y / OG_TWO_PI_S) * OG_TWO_PI_S;
            double cx = OG_PI_S, cy = OG_PI_S / 2.0, wx = 2 * OG_PI_S, wy = OG_PI_S;
            return (x > cx - wx / 2.0 && x < cx + wx / 2.0 && y > cy - wy / 2.0 && y < cy + wy / 2.0) ? 1.0 : 0.0;
        }
        case 1: { /* gaussian */
            double mx = OG_PI_S, my = OG_PI_S, vx = OG_PI_S / 4.0, vy = OG_PI_S / 4.0;
            return 1.0 / (OG_TWO_PI_S * vx * vy) *
                   exp(-((x - mx) * (x - mx) / (2 * vx * vx) + (y - my) * (y - my) / (2 * vy * vy)));
        }
        case 2: { /* circular_ring */
            double r = OG_PI_S / 2.0, rw = r / 8.0, s1 = 10.0, s2 = 10.0;
            double q = (x - OG_PI_S) * (x - OG_PI_S) + (y - OG_PI_S) * (y - OG_PI_S);
            return (tanh(s1 * (q - (r + rw) * (r + rw))) - tanh(s2 * (q - (r - rw) * (r - rw)))) / 2.0;
        }
        default: return 0.0;
    }
}

/* k_fft_lap_h (cmm-fft.cu:27-51): -k^2 F, mode 0 -> 0 */
static void fft_lap_h(double* c, const og_grid* g)
{
    for (int iY = 0; iY < g->NY; ++iY)
        for (int iX = 0; iX < g->NX_fft; ++iX) {
            long In = (long)iY * g->NX_fft + iX;
            if (iX == 0 && iY == 0) { c[0] = c[1] = 0.0; continue; }
            double kx = OG_TWO_PI_S / (g->hx * g->NX) * (iX - (iX > g->NX / 2) * g->NX);
            double ky = OG_TWO_PI_S / (g->hy * g->NY) * (iY - (iY > g->NY / 2) * g->NY);
            double k2 = kx * kx + ky * ky;
            c[2 * In] = -c[2 * In] * k2;
            c[2 * In + 1] = -c[2 * In + 1] * k2;
        }
}

/* D2Z, normalise, spectral operator op (0 lap, 1 dx, 2 dy, 3 iLap), Z2D */
static void spectral(const og_grid* g, const double* in, double* out, int op)
{
    double* c = (double*)malloc(sizeof(double) * 2 * g->Nfft);
    double* d = (double*)malloc(sizeof(double) * 2 * g->Nfft);
    og_fft_d2z(g, in, c);
    og_normalize_h(c, g);
    switch (op) {
        case 0: fft_lap_h(c, g); memcpy(d, c, sizeof(double) * 2 * g->Nfft); break;
        case 1: og_fft_dx_h(c, d, g); break;
        case 2: og_fft_dy_h(c, d, g); break;
        default: og_fft_iLap_h(c, d, g); break;
    }
    og_fft_z2d(g, d, out);
    free(c); free(d);
}

static double sumsq(const double* v, long n)
{
    double a = 0;
    for (long i = 0; i < n; ++i) a += v[i] * v[i];
    return a;
}

void og_sample_fields(const og_state_view* st, const og_grid* gs, int scalar_num, double* out, double* mes)
{
    const og_grid* gm = st->gc;
    long N = gs->N;
    double* xy = (double*)malloc(sizeof(double) * 2 * N);
    og_sample_map_compact(st->ChiX, st->ChiY, xy, gm, gs);
    for (int i = st->n_maps - 1; i >= 0; i--)
        og_apply_map_compact(st->stackX + 4 * gm->N * (size_t)i, st->stackY + 4 * gm->N * (size_t)i, xy, gm, gs);
    double *mapx = out, *mapy = out + N, *theta = out + 2 * N, *w = out + 3 * N, *lap = out + 4 * N, *gx = out + 5 * N,
           *gy = out + 6 * N, *psi = out + 7 * N, *ux = out + 8 * N, *uy = out + 9 * N;
    for (long i = 0; i < N; ++i) {
        mapx[i] = xy[2 * i];
        mapy[i] = xy[2 * i + 1];
        theta[i] = og_init_scalar(xy[2 * i], xy[2 * i + 1], scalar_num);
        w[i] = st->discrete ? og_hermite_interpolate_2D(st->discrete, xy[2 * i], xy[2 * i + 1], st->gd)
                            : og_init_vorticity(xy[2 * i], xy[2 * i + 1], st->ic_num);
    }
    free(xy);
    spectral(gs, w, lap, 0);
    spectral(gs, w, gx, 1);
    spectral(gs, w, gy, 2);
    spectral(gs, w, psi, 3);
    spectral(gs, psi, ux, 1);
    spectral(gs, psi, uy, 2);
    double hh = gs->hx * gs->hy;
    double wmax = w[0], tmax = 0.0;
    for (long i = 0; i < N; ++i) { if (w[i] > wmax) wmax = w[i]; if (theta[i] > tmax) tmax = theta[i]; }
    mes[0] = 0.5 * hh * sumsq(ux, N) + 0.5 * hh * sumsq(uy, N);   /* Energy */
    mes[1] = 0.5 * hh * sumsq(w, N);                               /* Enstrophy */
    mes[2] = 0.5 * hh * sumsq(gx, N) + 0.5 * hh * sumsq(gy, N);   /* Palinstrophy */
    mes[3] = wmax > -wmax ? wmax : -wmax;                          /* Max_vorticity */
    mes[4] = hh * tmax;                                            /* Scalar_integral */
}

/* compute_zoom, backward-map part (src/simulation/cmm-simulation-host.cu:1039-1201): on the
 * n x n window grid with bounds (x_min, x_max, y_min, y_max) -- points x_min + i h, h the
 * window width over n -- the full backward map through the stack, the passive scalar, the
 * vorticity and the distribution function (the Vlasov formula with the run's initial-condition
 * number, as k_h_sample_from_init with var 2 does) there, and psi level 0 interpolated at the
 * window points themselves (k_h_sample).  out: 6 planes of n*n. */
void og_zoom_fields(const og_state_view* st, int n, const double* bounds4, int scalar_num, double* out)
{
    og_grid gz;
    og_grid_fill(&gz, n, n, bounds4);
    const og_grid* gm = st->gc;
    long N = gz.N;
    double* xy = (double*)malloc(sizeof(double) * 2 * N);
    og_sample_map_compact(st->ChiX, st->ChiY, xy, gm, &gz);
    for (int i = st->n_maps - 1; i >= 0; i--)
        og_apply_map_compact(st->stackX + 4 * gm->N * (size_t)i, st->stackY + 4 * gm->N * (size_t)i, xy, gm, &gz);
    double *mapx = out, *mapy = out + N, *theta = out + 2 * N, *w = out + 3 * N, *f = out + 4 * N, *psi = out + 5 * N;
    for (long i = 0; i < N; ++i) {
        double x = xy[2 * i], y = xy[2 * i + 1];
        mapx[i] = x;
        mapy[i] = y;
        theta[i] = og_init_scalar(x, y, scalar_num);
        w[i] = st->discrete ? og_hermite_interpolate_2D(st->discrete, x, y, st->gd) : og_init_vorticity(x, y, st->ic_num);
        f[i] = st->discrete ? og_hermite_interpolate_2D(st->discrete, x, y, st->gd) : og_init_distribution(x, y, st->ic_num);
        long iX = i % gz.NX, iY = i / gz.NX;
        psi[i] = og_hermite_interpolate_2D(st->psi, gz.bounds[0] + iX * gz.hx, gz.bounds[2] + iY * gz.hy, st->gp);
    }
    free(xy);
}

/* sample_compute_and_write_vlasov, backward-map part (src/simulation/cmm-simulation-host.cu:898-1030)
 * on the n x n sample grid gs: the full backward map through the stack, the distribution
 * function there (k_h_sample_from_init with var 2: the Vlasov formula of the run's
 * initial-condition number, or the discrete initial field), and from it
 *   Ekin = hx hy / 2 sum f v^2, Momentum = hx hy sum f v, Mass = hx hy sum f
 * (cmm-mesure.cu:97-183, v = bounds[2] + iY hy), the field e = d phi / dx of calc_phi on
 * the sample grid itself (integral_v, solve_1D_laplace, k_fft_dx_h_1D with the Nyquist
 * mode kept, a 1D Z2D of length n: cmm-simulation-host.cu:436-471) and
 * Epot = hx / 2 sum e^2; the four mode amplitudes come from the run's psi (Compute_kth_Mode
 * on psi_x row 0).  The reference writes its sample buffer as Stream_function_Psi after
 * those in-place steps: e in its first n entries, the distribution from entry N / 8 on
 * (a copy of N bytes of the spectrum sits before it, left-over scratch past the
 * spectrum); here the entries between are 0.
 * out: 4 planes of N (map x, map y, distribution, stream); mes = {Etot, Ekin, Epot, Mass,
 * Momentum, Emode1..4}. */
void og_vlasov_sample_fields(const og_state_view* st, const og_grid* gs, double* out, double* mes)
{
    const og_grid* gm = st->gc;
    long N = gs->N;
    int n = gs->NX;
    double* xy = (double*)malloc(sizeof(double) * 2 * N);
    og_sample_map_compact(st->ChiX, st->ChiY, xy, gm, gs);
    for (int i = st->n_maps - 1; i >= 0; i--)
        og_apply_map_compact(st->stackX + 4 * gm->N * (size_t)i, st->stackY + 4 * gm->N * (size_t)i, xy, gm, gs);
    double *mapx = out, *mapy = out + N, *f = out + 2 * N, *stream = out + 3 * N;
    for (long i = 0; i < N; ++i) {
        double x = xy[2 * i], y = xy[2 * i + 1];
        mapx[i] = x;
        mapy[i] = y;
        f[i] = st->discrete ? og_hermite_interpolate_2D(st->discrete, x, y, st->gd) : og_init_distribution(x, y, st->ic_num);
    }
    free(xy);
    double ekin = 0, mom = 0, mass = 0;
    for (int iY = 0; iY < gs->NY; ++iY) {
        double v = gs->bounds[2] + iY * gs->hy;
        for (int iX = 0; iX < n; ++iX) {
            double fv = f[(long)iY * n + iX];
            ekin += v * v * fv;
            mom += v * fv;
            mass += fv;
        }
    }
    double hh = gs->hx * gs->hy;
    double* rho = (double*)malloc(sizeof(double) * n);
    og_integral_v(f, rho, n, gs->NY, gs->hy);
    og_grid g1;
    og_grid_fill(&g1, n, 1, gs->bounds);
    double* c = (double*)malloc(sizeof(double) * 2 * g1.NX_fft);
    double* d = (double*)malloc(sizeof(double) * 2 * g1.NX_fft);
    og_fft_d2z(&g1, rho, c);
    d[0] = d[1] = 0.0;
    for (int i = 1; i < g1.NX_fft; ++i) {
        double kx = OG_TWO_PI_S / (gs->hx * n) * (i - (i > n / 2) * n);
        double re = c[2 * i] / (double)n / (kx * kx), im = c[2 * i + 1] / (double)n / (kx * kx);
        d[2 * i] = -im * kx;     /* k_fft_dx_h_1D: i kx */
        d[2 * i + 1] = re * kx;
    }
    memset(stream, 0, sizeof(double) * N);
    og_fft_z2d(&g1, d, stream);
    double epot = 0;
    for (int i = 0; i < n; ++i) epot += stream[i] * stream[i];
    long tail = N / 8 > n + 2 ? N / 8 : n + 2;
    for (long i = tail; i < N; ++i) stream[i] = f[i];
    free(rho); free(c); free(d);
    double vm[9];
    og_vlasov_mesure(f, gs, st->psi, st->gp, vm);
    mes[1] = 0.5 * hh * ekin;
    mes[2] = 0.5 * gs->hx * epot;
    mes[0] = mes[1] + mes[2];
    mes[3] = hh * mass;
    mes[4] = hh * mom;
    for (int k = 0; k < 4; ++k) mes[5 + k] = vm[5 + k];
}
