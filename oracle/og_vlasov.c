/*
 * og_vlasov.c -- CPU restatement of the Vlasov-Poisson pieces of the
 * reference (1D1V, x periodic, v the second coordinate).  TEST
 * INFRASTRUCTURE ONLY (see cmm_oracle.h).
 *
 * The potential follows evaluate_potential_from_density_hermite
 * (src/simulation/cmm-simulation-host.cu:385-415) step by step, including its
 * 2D FFT of the assembled psi and two of its quirks: the v-integral's output
 * row aliases row 0 of the sampled distribution, so that row is counted
 * twice (integral_v, src/simulation/cmm-simulation-kernel.cu:570-586, called
 * with f_in.Dev_var == Dev_Temp_C1, cmm-vlasov1d.cu:328 and
 * cmm-simulation-host.cu:391-393,443), and the 1D "inverse Laplacians"
 * divide by +k^2 (src/numerical/cmm-fft.cu:81-124).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cmm_oracle.h"

#define OG_PI 3.141592653589793238462643383279502884197169399375105820974944592307816406286
#define OG_TWO_PI_V 6.283185307179586476925286766559005768394338798750211641949889184615632812572417997256069650684234136

/* d_init_distirbution_function: src/simulation/cmm-init.cu:457-493 */
double og_init_distribution(double x, double v, int ic)
{
    switch (ic) {
        case 0: { /* landau_damping */
            double k = 0.5, eps = 5 * 1e-2;
            return (1 + eps * cos(k * x)) * exp(-(v) * (v) * 0.5) / sqrt(2 * OG_PI);
        }
        case 1: { /* two_stream */
            double v0 = 3, k = 0.2, eps = 5 * 1e-2;
            return 1 / (2 * sqrt(2 * OG_PI)) * (1 + eps * cos(k * x)) *
                   (exp(-(v - v0) * (v - v0) * 0.5) + exp(-(v + v0) * (v + v0) * 0.5));
        }
        case 2: { /* nonlin_landau_damping */
            double k = 0.5, eps = 0.5;
            return (1 + eps * cos(k * x)) * exp(-(v) * (v) * 0.5) / sqrt(2 * OG_PI);
        }
        default: return 0;
    }
}

/* integral_v (cmm-simulation-kernel.cu:570-586) with the output aliasing row 0 */
void og_integral_v(const double* f, double* rho, int nx, int ny, double hy)
{
    for (int ix = 0; ix < nx; ++ix) {
        double acc = f[ix];
        for (int iy = 0; iy < ny; ++iy) acc += f[(long)iy * nx + ix];
        acc *= hy;
        rho[ix] = acc + -1.0;
    }
}

static og_grid row_grid(int n, const double* bounds)
{
    og_grid g;
    og_grid_fill(&g, n, 1, bounds);
    return g;
}

/* solve_1D_laplace (cmm-simulation-host.cu:417-432): 1D D2Z over x, /NX
 * (k_normalize_1D_hx), /kx^2 with the zero mode zeroed (k_fft_iLap_hx_1D) */
static void solve_1d_laplace(const double* rhs, double* out_c, const og_grid* g)
{
    og_grid g1 = row_grid(g->NX, g->bounds);
    double* tmp = (double*)malloc(sizeof(double) * 2 * g1.NX_fft);
    og_fft_d2z(&g1, rhs, tmp);
    for (int i = 0; i < g1.NX_fft; ++i) { tmp[2 * i] /= (double)g->NX; tmp[2 * i + 1] /= (double)g->NX; }
    out_c[0] = out_c[1] = 0.0;
    for (int i = 1; i < g1.NX_fft; ++i) {
        double kx = OG_TWO_PI_V / (g->hx * g->NX) * (i - (i > g->NX / 2) * g->NX);
        double k2 = kx * kx;
        out_c[2 * i] = tmp[2 * i] / k2;
        out_c[2 * i + 1] = tmp[2 * i + 1] / k2;
    }
    free(tmp);
}

/* compute_bump_function + compute_periodification_function
 * (cmm-simulation-host.cu:478-494,534-571) on the psi grid; h has NY values */
void og_periodification(const og_grid* g, double* h)
{
    int n = g->NY;
    double* sigma = (double*)malloc(sizeof(double) * n);
    double Lv = g->bounds[3] - g->bounds[2], a = 0.4, b = 0.1;
    for (int iY = 0; iY < n; ++iY) {
        double v = g->bounds[2] + iY * g->hy;
        sigma[iY] = 0.5 - 0.5 * tanh(2 * OG_PI * (fabs(v) - a * Lv) / (b * Lv));
    }
    double mean = 0.0;
    for (int i = 0; i < n; ++i) mean += sigma[i];
    mean /= (double)n;
    for (int i = 0; i < n; ++i) sigma[i] = sigma[i] - mean;
    double max_v = sigma[0];
    for (int i = 1; i < n; ++i) if (sigma[i] > max_v) max_v = sigma[i];
    for (int i = 0; i < n; ++i) sigma[i] = sigma[i] / max_v;
    /* 1D D2Z of length NX (== NY), /NY, /ky^2, Z2D */
    og_grid g1 = row_grid(g->NX, g->bounds);
    double* c = (double*)malloc(sizeof(double) * 2 * g1.NX_fft);
    double* d = (double*)malloc(sizeof(double) * 2 * g1.NX_fft);
    og_fft_d2z(&g1, sigma, c);
    for (int i = 0; i < g1.NX_fft; ++i) { c[2 * i] /= (double)g->NY; c[2 * i + 1] /= (double)g->NY; }
    d[0] = d[1] = 0.0;
    for (int i = 1; i < g1.NX_fft; ++i) {
        double ky = OG_TWO_PI_V / (g->hy * g->NY) * (i - (i > g->NY / 2) * g->NY);
        double k2 = ky * ky;
        d[2 * i] = c[2 * i] / k2;
        d[2 * i + 1] = c[2 * i + 1] / k2;
    }
    og_fft_z2d(&g1, d, h);
    free(sigma); free(c); free(d);
}

/* evaluate_potential_from_density_hermite (cmm-simulation-host.cu:385-415):
 * f on the vort grid -> rho -> phi (1D) -> psi = phi(x) - h(v) -> 2D FFT
 * Hermite into psi_out (4 planes on gp).  Returns -1 when the vort grid is
 * finer than the psi grid (calc_phi's error, :457-460) or NX != NY on gp. */
int og_vlasov_potential(const double* ChiX, const double* ChiY, const double* f_fine, const og_grid* gm,
                        const og_grid* gv, const og_grid* gf, const og_grid* gp, int molly, double* psi_out)
{
    if (gv->NX > gp->NX || gv->NY > gp->NY) return -1;
    if (gp->NX != gp->NY) return -1;
    double* fs = (double*)malloc(sizeof(double) * gv->N);
    og_apply_map_and_sample_from_hermite(ChiX, ChiY, fs, f_fine, gm, gv, gf, molly, 0);
    double* rho = (double*)malloc(sizeof(double) * gv->NX);
    og_integral_v(fs, rho, gv->NX, gv->NY, gv->hy);
    free(fs);
    og_grid gv1 = row_grid(gv->NX, gv->bounds), gp1 = row_grid(gp->NX, gp->bounds);
    double* phic = (double*)malloc(sizeof(double) * 2 * gp1.NX_fft);
    double* lap = (double*)malloc(sizeof(double) * 2 * gv1.NX_fft);
    solve_1d_laplace(rho, lap, gv);
    free(rho);
    double* phi = (double*)malloc(sizeof(double) * gp->NX);
    if (gv->NX < gp->NX) {
        /* zero_padding_1D (cmm-fft.cu:367-391) */
        for (int iXc = 0; iXc < gp1.NX_fft; ++iXc) {
            if (iXc + (iXc > gp->NX / 2.0) * (gp->NX - 2 * iXc) > gv->NX / 2.0) {
                phic[2 * iXc] = phic[2 * iXc + 1] = 0.0;
            } else {
                int iXs = iXc + (iXc > gp->NX / 2.0) * (gv->NX - gp->NX);
                phic[2 * iXc] = lap[2 * iXs];
                phic[2 * iXc + 1] = lap[2 * iXs + 1];
            }
        }
        og_fft_z2d(&gp1, phic, phi);
    } else {
        og_fft_z2d(&gv1, lap, phi);
    }
    free(lap); free(phic);
    double* h = (double*)malloc(sizeof(double) * gp->NY);
    og_periodification(gp, h);
    /* k_assemble_psi_periodified (cmm-simulation-kernel.cu:504-512) */
    double* psi = (double*)malloc(sizeof(double) * gp->N);
    for (int iY = 0; iY < gp->NY; ++iY)
        for (int iX = 0; iX < gp->NX; ++iX) psi[(long)iY * gp->NX + iX] = phi[iX] - h[iY];
    free(phi); free(h);
    double* c = (double*)malloc(sizeof(double) * 2 * gp->Nfft);
    og_fft_d2z(gp, psi, c);
    og_normalize_h(c, gp);
    og_fourier_hermite(gp, c, psi_out);
    free(c); free(psi);
    return 0;
}

/* Vlasov conservation targets (cmm-simulation-host.cu:639-664, cmm-mesure.cu:97-202)
 * on the coarse distribution f (grid gc) and psi level 0 (grid gp):
 * out = {Etot, Ekin, Epot, Mass, Momentum, Emode1..4} */
void og_vlasov_mesure(const double* f, const og_grid* gc, const double* psi, const og_grid* gp, double* out)
{
    double ekin = 0, mass = 0, mom = 0;
    for (int iY = 0; iY < gc->NY; ++iY) {
        double v = gc->bounds[2] + iY * gc->hy;
        for (int iX = 0; iX < gc->NX; ++iX) {
            double fv = f[(long)iY * gc->NX + iX];
            ekin += v * v * fv;
            mass += fv;
            mom += v * fv;
        }
    }
    ekin = 0.5 * gc->hy * gc->hx * ekin;
    mass = gc->hy * gc->hx * mass;
    mom = gc->hy * gc->hx * mom;
    const double* px = psi + gp->N;   /* psi_x, first row = -E(x) */
    double epot = 0;
    for (int iX = 0; iX < gp->NX; ++iX) epot += px[iX] * px[iX];
    epot = 0.5 * gp->hx * epot;
    out[0] = ekin + epot; out[1] = ekin; out[2] = epot; out[3] = mass; out[4] = mom;
    /* Compute_kth_Mode: 1D D2Z of the first row of psi_x, /NX, |F_k| for k = 1..4 */
    og_grid g1 = row_grid(gp->NX, gp->bounds);
    double* c = (double*)malloc(sizeof(double) * 2 * g1.NX_fft);
    og_fft_d2z(&g1, px, c);
    for (int i = 0; i < 4; ++i) {
        int k = i + 1 < g1.NX_fft ? i + 1 : g1.NX_fft - 1;
        double re = c[2 * k] / (double)gp->NX, im = c[2 * k + 1] / (double)gp->NX;
        out[5 + i] = sqrt(re * re + im * im);
    }
    free(c);
}
