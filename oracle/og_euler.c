/*
 * og_euler.c -- the 2D Euler CMM loop restated on the CPU (FP64, OpenMP).
 *
 * TEST INFRASTRUCTURE ONLY (parity oracle; see cmm_oracle.h).
 *
 * Follows src/simulation/cmm-simulation-kernel.cu (kernels as loops),
 * src/simulation/cmm-simulation-host.cu (host orchestration),
 * src/numerical/cmm-timestep.cu (backward integrators),
 * src/numerical/cmm-particles.cu (tracer advection),
 * src/numerical/cmm-mesure.cu (diagnostics) and the driver
 * src/simulation/cmm-euler2d.cu:495-897.
 */
#include "cmm_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OG_TWO_PI 6.283185307179586476925286766559005768394338798750211641949889184615632812572417997256069650684234136

/* ------------------------------------------------------------------ */
/* backward integrators: src/numerical/cmm-timestep.cu                 */
/* ------------------------------------------------------------------ */
typedef struct { const double* L1; const double* L12; } og_lcoef;

/* euler_exp_b: cmm-timestep.cu:35-45 */
static void euler_exp_b(const double* psi, const double* x_in, double* x_out, const og_grid* g,
                        double dt, int l_order, const og_lcoef* lc)
{
    double u[8];
    og_hermite_interpolate_grad_2D(psi, x_in, u, g, l_order);
    double k0 = lc->L1[0] * u[0], k1 = lc->L1[0] * u[1];
    for (int i_l = 1; i_l < l_order; i_l++) { k0 += lc->L1[i_l] * u[i_l * 2]; k1 += lc->L1[i_l] * u[i_l * 2 + 1]; }
    x_out[0] = x_in[0] - dt * k0;
    x_out[1] = x_in[1] - dt * k1;
}

/* RK2_heun_b: cmm-timestep.cu:66-81 */
static void rk2_heun_b(const double* psi, const double* x_in, double* x_out, const og_grid* g,
                       double dt, int l_order, const og_lcoef* lc)
{
    double u[8];
    og_hermite_interpolate_grad_2D(psi, x_in, u, g, l_order);
    double k1[2] = {lc->L1[0] * u[0], lc->L1[0] * u[1]};
    for (int i_l = 1; i_l < l_order; i_l++) { k1[0] += lc->L1[i_l] * u[i_l * 2]; k1[1] += lc->L1[i_l] * u[i_l * 2 + 1]; }
    double k2[2] = {x_in[0] - dt * k1[0], x_in[1] - dt * k1[1]};
    og_hermite_interpolate_grad_2D(psi, k2, u, g, 1);
    x_out[0] = x_in[0] - dt * (k1[0] + u[0]) / 2;
    x_out[1] = x_in[1] - dt * (k1[1] + u[1]) / 2;
}

/* RK3_classical_b: cmm-timestep.cu:175-207 */
static void rk3_classical_b(const double* psi, const double* x_in, double* x_out, const og_grid* g,
                            double dt, int l_order, const og_lcoef* lc)
{
    double u[8], k[6];
    og_hermite_interpolate_grad_2D(psi, x_in, u, g, l_order);
    k[0] = lc->L1[0] * u[0]; k[1] = lc->L1[0] * u[1];
    for (int i_l = 1; i_l < l_order; i_l++) { k[0] += lc->L1[i_l] * u[i_l * 2]; k[1] += lc->L1[i_l] * u[i_l * 2 + 1]; }
    k[2] = x_in[0] - dt * k[0] / 2.0; k[3] = x_in[1] - dt * k[1] / 2.0;
    og_hermite_interpolate_grad_2D(psi, k + 2, u, g, l_order);
    k[2] = lc->L12[0] * u[0]; k[3] = lc->L12[0] * u[1];
    for (int i_l = 1; i_l < l_order; i_l++) { k[2] += lc->L12[i_l] * u[i_l * 2]; k[3] += lc->L12[i_l] * u[i_l * 2 + 1]; }
    k[4] = x_in[0] + dt * k[0] - 2 * dt * k[2]; k[5] = x_in[1] + dt * k[1] - 2 * dt * k[3];
    og_hermite_interpolate_grad_2D(psi, k + 4, k + 4, g, 1);
    x_out[0] = x_in[0] - dt * (k[0] + 4 * k[2] + k[4]) / 6.0;
    x_out[1] = x_in[1] - dt * (k[1] + 4 * k[3] + k[5]) / 6.0;
}

/* velocity u = (psi_y, -psi_x) of psi level lv at x */
static void vel_level(const double* psi, int lv, const double* x, double* u, const og_grid* g)
{
    og_hermite_interpolate_grad_2D(psi + 4 * g->N * (long)lv, x, u, g, 1);
}

/* sum_l c[l] u_l(x) over l_order levels, accumulated from level 0 upwards */
static void vel_comb(const double* psi, const double* c, int l_order, const double* x, double* k, const og_grid* g)
{
    double u[8];
    og_hermite_interpolate_grad_2D(psi, x, u, g, l_order);
    k[0] = c[0] * u[0]; k[1] = c[0] * u[1];
    for (int i_l = 1; i_l < l_order; i_l++) { k[0] += c[i_l] * u[i_l * 2]; k[1] += c[i_l] * u[i_l * 2 + 1]; }
}

/* adam_bashford_2_pc_b: cmm-timestep.cu:112-135 -- ten fixed-point sweeps on levels 0 and 1 */
static void ab2_pc_b(const double* psi, const double* x_in, double* x_out, const og_grid* g, double dt)
{
    double u[2], u2[2], xf_p[2] = {x_in[0], x_in[1]};
    x_out[0] = x_in[0]; x_out[1] = x_in[1];
    for (int ctr = 0; ctr < 10; ctr++) {
        vel_level(psi, 1, xf_p, u2, g);
        xf_p[0] = x_out[0] - dt * u2[0]; xf_p[1] = x_out[1] - dt * u2[1];
        vel_level(psi, 1, xf_p, u2, g);
        vel_level(psi, 0, x_out, u, g);
        x_out[0] = x_in[0] - dt * (1.5 * u[0] - 0.5 * u2[0]);
        x_out[1] = x_in[1] - dt * (1.5 * u[1] - 0.5 * u2[1]);
    }
}

/* RK4_classical_b: cmm-timestep.cu:260-307 */
static void rk4_classical_b(const double* psi, const double* x_in, double* x_out, const og_grid* g,
                            double dt, int l_order, const og_lcoef* lc)
{
    double k1[2], k2[2], k3[2], k4[2], y[2];
    vel_comb(psi, lc->L1, l_order, x_in, k1, g);
    y[0] = x_in[0] - dt * k1[0] / 2.0; y[1] = x_in[1] - dt * k1[1] / 2.0;
    vel_comb(psi, lc->L12, l_order, y, k2, g);
    y[0] = x_in[0] - dt * k2[0] / 2.0; y[1] = x_in[1] - dt * k2[1] / 2.0;
    vel_comb(psi, lc->L12, l_order, y, k3, g);
    y[0] = x_in[0] - dt * k3[0]; y[1] = x_in[1] - dt * k3[1];
    vel_level(psi, 0, y, k4, g);
    x_out[0] = x_in[0] - dt * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0]) / 6.0;
    x_out[1] = x_in[1] - dt * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1]) / 6.0;
}

/* RK3_optimized_b: cmm-timestep.cu:348-374 */
static void rk3_optimized_b(const double* psi, const double* x_in, double* x_out, const og_grid* g,
                            double dt, int l_order, const og_lcoef* lc)
{
    double k1[2], k2[2], k3[2], y[2];
    vel_comb(psi, lc->L1, l_order, x_in, k1, g);
    y[0] = x_in[0] - dt * k1[0]; y[1] = x_in[1] - dt * k1[1];
    vel_level(psi, 0, y, k2, g);
    y[0] = x_in[0] + 2 * dt * (-2 * k1[0] + k2[0]); y[1] = x_in[1] + 2 * dt * (-2 * k1[1] + k2[1]);
    vel_level(psi, 1, y, k3, g);
    x_out[0] = x_in[0] - dt * (5 * k1[0] + 8 * k2[0] - k3[0]) / 12.0;
    x_out[1] = x_in[1] - dt * (5 * k1[1] + 8 * k2[1] - k3[1]) / 12.0;
}

/* RK4_optimized_b: cmm-timestep.cu:428-466 */
static void rk4_optimized_b(const double* psi, const double* x_in, double* x_out, const og_grid* g,
                            double dt, int l_order, const og_lcoef* lc)
{
    double k1[2], k2[2], k3[2], k4[2], y[2];
    vel_comb(psi, lc->L1, l_order, x_in, k1, g);
    y[0] = x_in[0] - dt * k1[0]; y[1] = x_in[1] - dt * k1[1];
    vel_level(psi, 0, y, k2, g);
    y[0] = x_in[0] - dt * (3 * k1[0] + k2[0]) / 8.0; y[1] = x_in[1] - dt * (3 * k1[1] + k2[1]) / 8.0;
    vel_comb(psi, lc->L12, l_order, y, k3, g);
    y[0] = x_in[0] + dt * (k2[0] - 4 * k3[0]) / 3.0; y[1] = x_in[1] + dt * (k2[1] - 4 * k3[1]) / 3.0;
    vel_level(psi, 0, y, k4, g);
    x_out[0] = x_in[0] - dt * (2 * k1[0] - k2[0] + 8 * k3[0] + 3 * k4[0]) / 12.0;
    x_out[1] = x_in[1] - dt * (2 * k1[1] - k2[1] + 8 * k3[1] + 3 * k4[1]) / 12.0;
}

/* forward integrators (forward map), src/numerical/cmm-timestep.cu: psi level 0 is t_n,
 * level 1 t_{n-1}, level 2 t_{n-2}; L1 / L12 extrapolate to t_{n+1} / t_{n+1/2}.  Two of
 * them are kept exactly as the reference has them: RK4_classical takes its first
 * half-step velocity from L1 and its last stage from L12, and RK4_optimized is the
 * backward scheme (it integrates with -dt). */
static void euler_exp_f(const double* psi, const double* x_in, double* x_out, const og_grid* g, double dt)
{   /* :26-31 */
    double u[2];
    vel_level(psi, 0, x_in, u, g);
    x_out[0] = x_in[0] + dt * u[0];
    x_out[1] = x_in[1] + dt * u[1];
}

static void rk2_heun_f(const double* psi, const double* x_in, double* x_out, const og_grid* g, double dt, int l_order,
                       const og_lcoef* lc)
{   /* :48-64 */
    double k1[2], k2[2], y[2];
    vel_level(psi, 0, x_in, k1, g);
    y[0] = x_in[0] + dt * k1[0]; y[1] = x_in[1] + dt * k1[1];
    vel_comb(psi, lc->L1, l_order, y, k2, g);
    x_out[0] = x_in[0] + dt * (k1[0] + k2[0]) / 2;
    x_out[1] = x_in[1] + dt * (k1[1] + k2[1]) / 2;
}

static void ab2_pc_f(const double* psi, const double* x_in, double* x_out, const og_grid* g, double dt)
{   /* :84-110 */
    double u[2], u2[2], xf_p[2] = {x_in[0], x_in[1]}, o[2] = {x_in[0], x_in[1]};
    for (int ctr = 0; ctr < 10; ctr++) {
        vel_level(psi, 1, xf_p, u2, g);
        xf_p[0] = o[0] + dt * u2[0]; xf_p[1] = o[1] + dt * u2[1];
        vel_level(psi, 1, xf_p, u2, g);
        vel_level(psi, 0, o, u, g);
        o[0] = x_in[0] + dt * (1.5 * u[0] - 0.5 * u2[0]);
        o[1] = x_in[1] + dt * (1.5 * u[1] - 0.5 * u2[1]);
    }
    x_out[0] = o[0]; x_out[1] = o[1];
}

static void rk3_classical_f(const double* psi, const double* x_in, double* x_out, const og_grid* g, double dt,
                            int l_order, const og_lcoef* lc)
{   /* :144-173 */
    double k1[2], k2[2], k3[2], y[2];
    vel_level(psi, 0, x_in, k1, g);
    y[0] = x_in[0] + dt * k1[0] / 2.0; y[1] = x_in[1] + dt * k1[1] / 2.0;
    vel_comb(psi, lc->L12, l_order, y, k2, g);
    y[0] = x_in[0] - dt * k1[0] + 2 * dt * k2[0]; y[1] = x_in[1] - dt * k1[1] + 2 * dt * k2[1];
    vel_comb(psi, lc->L1, l_order, y, k3, g);
    x_out[0] = x_in[0] + dt * (k1[0] + 4 * k2[0] + k3[0]) / 6.0;
    x_out[1] = x_in[1] + dt * (k1[1] + 4 * k2[1] + k3[1]) / 6.0;
}

static void rk4_classical_f(const double* psi, const double* x_in, double* x_out, const og_grid* g, double dt,
                            int l_order, const og_lcoef* lc)
{   /* :216-258 */
    double k1[2], k2[2], k3[2], k4[2], y[2];
    vel_level(psi, 0, x_in, k1, g);
    y[0] = x_in[0] + dt * k1[0] / 2.0; y[1] = x_in[1] + dt * k1[1] / 2.0;
    vel_comb(psi, lc->L1, l_order, y, k2, g);
    y[0] = x_in[0] + dt * k2[0] / 2.0; y[1] = x_in[1] + dt * k2[1] / 2.0;
    vel_comb(psi, lc->L12, l_order, y, k3, g);
    y[0] = x_in[0] + dt * k3[0]; y[1] = x_in[1] + dt * k3[1];
    vel_comb(psi, lc->L12, l_order, y, k4, g);
    x_out[0] = x_in[0] + dt * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0]) / 6.0;
    x_out[1] = x_in[1] + dt * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1]) / 6.0;
}

static void rk3_optimized_f(const double* psi, const double* x_in, double* x_out, const og_grid* g, double dt)
{   /* :314-339 */
    double k1[2], k2[2], k3[2], y[2];
    vel_level(psi, 0, x_in, k1, g);
    y[0] = x_in[0] - dt * k1[0]; y[1] = x_in[1] - dt * k1[1];
    vel_level(psi, 1, y, k2, g);
    y[0] = x_in[0] - dt * (8 * k1[0] + 2 * k2[0]) / 5.0; y[1] = x_in[1] - dt * (8 * k1[1] + 2 * k2[1]) / 5.0;
    vel_level(psi, 2, y, k3, g);
    x_out[0] = x_in[0] + dt * (23 * k1[0] - 16 * k2[0] + 5 * k3[0]) / 12.0;
    x_out[1] = x_in[1] + dt * (23 * k1[1] - 16 * k2[1] + 5 * k3[1]) / 12.0;
}

/* ------------------------------------------------------------------ */
/* kernels restated as loops                                           */
/* ------------------------------------------------------------------ */
void og_init_diffeo(double* ChiX, double* ChiY, const og_grid* g)
{
    long N = g->N;
    #pragma omp parallel for schedule(static)
    for (int iY = 0; iY < g->NY; ++iY)
        for (int iX = 0; iX < g->NX; ++iX) {
            long In = (long)iY * g->NX + iX;
            ChiX[In] = g->bounds[0] + iX * g->hx; ChiY[In] = g->bounds[2] + iY * g->hy;
            ChiX[1 * N + In] = ChiY[2 * N + In] = 1;
            ChiX[2 * N + In] = ChiY[1 * N + In] = ChiX[3 * N + In] = ChiY[3 * N + In] = 0;
        }
}

void og_map_update_coefficients(int order_num, double ep, double* c1, double* cx, double* cy, double* cxy)
{
    double h_c[3] = {0, 0, 0};
    switch (order_num) {
        case 2: h_c[0] = +3.0 / 8.0; h_c[1] = -3.0 / 20.0; h_c[2] = +1.0 / 40.0; break;
        case 1: h_c[0] = +1.0 / 3.0; h_c[1] = -1.0 / 12.0; break;
        case 0: h_c[0] = +1.0 / 4.0; break;
    }
    for (int i = 0; i < 4 + 4 * order_num; ++i) {
        c1[i] = h_c[i / 4];
        cx[i] = h_c[i / 4] * (1 - 2 * ((i / 2) % 2)) / ep / (double)(i / 4 + 1);
        cy[i] = h_c[i / 4] * (1 - 2 * (((i + 1) / 2) % 2)) / ep / (double)(i / 4 + 1);
        cxy[i] = h_c[i / 4] * (1 - 2 * (i % 2)) / ep / ep / (double)(i / 4 + 1) / (double)(i / 4 + 1);
    }
}

static void advect_map_dir(const double* ChiX, const double* ChiY, double* ChiX_new, double* ChiY_new,
                           const double* psi, const og_grid* gm, const og_grid* gp,
                           double dt, double ep, int ti_num, int order_num, int l_order,
                           const double* L1, const double* L12,
                           const double* c1, const double* cx, const double* cy, const double* cxy, int direction);

void og_advect_map(const double* ChiX, const double* ChiY, double* ChiX_new, double* ChiY_new,
                   const double* psi, const og_grid* gm, const og_grid* gp,
                   double dt, double ep, int ti_num, int order_num, int l_order,
                   const double* L1, const double* L12,
                   const double* c1, const double* cx, const double* cy, const double* cxy)
{
    advect_map_dir(ChiX, ChiY, ChiX_new, ChiY_new, psi, gm, gp, dt, ep, ti_num, order_num, l_order, L1, L12,
                   c1, cx, cy, cxy, -1);
}

/* k_advect_using_stream_hermite (src/simulation/cmm-simulation-kernel.cu:207-298): direction -1
 * integrates each footpoint back in time and looks it up in the map; direction 1 (forward
 * map) looks the footpoint up in the map first and integrates it forward */
static void advect_map_dir(const double* ChiX, const double* ChiY, double* ChiX_new, double* ChiY_new,
                           const double* psi, const og_grid* gm, const og_grid* gp,
                           double dt, double ep, int ti_num, int order_num, int l_order,
                           const double* L1, const double* L12,
                           const double* c1, const double* cx, const double* cy, const double* cxy, int direction)
{
    og_lcoef lc = {L1, L12};
    long N = gm->N;
    int nfoot = order_num * 4 + 4;
    #pragma omp parallel for schedule(static)
    for (int iY = 0; iY < gm->NY; ++iY) {
        for (int iX = 0; iX < gm->NX; ++iX) {
            long In = (long)iY * gm->NX + iX;
            double x_ep[2], x_f[2];
            double fx[4] = {0, 0, 0, 0}, fy[4] = {0, 0, 0, 0};
            for (int k = 0; k < nfoot; k++) {
                x_ep[0] = gm->bounds[0] + iX * gm->hx + ((k >> 2) + 1) * ep * (1 - 2 * ((k >> 1) & 1));
                x_ep[1] = gm->bounds[2] + iY * gm->hy + ((k >> 2) + 1) * ep * (1 - 2 * (((k + 1) >> 1) & 1));
                if (direction == -1) {
                    switch (ti_num) {
                        case 10: euler_exp_b(psi, x_ep, x_f, gp, dt, l_order, &lc); break;
                        case 21: rk2_heun_b(psi, x_ep, x_f, gp, dt, l_order, &lc); break;
                        case 30: rk3_classical_b(psi, x_ep, x_f, gp, dt, l_order, &lc); break;
                        case 20: ab2_pc_b(psi, x_ep, x_f, gp, dt); break;
                        case 40: rk4_classical_b(psi, x_ep, x_f, gp, dt, l_order, &lc); break;
                        case 31: rk3_optimized_b(psi, x_ep, x_f, gp, dt, l_order, &lc); break;
                        case 41: rk4_optimized_b(psi, x_ep, x_f, gp, dt, l_order, &lc); break;
                        default: x_f[0] = x_f[1] = 0;
                    }
                    og_diffeo_interpolate_2D(ChiX, ChiY, x_f[0], x_f[1], &x_f[0], &x_f[1], gm);
                } else {
                    double y[2];
                    og_diffeo_interpolate_2D(ChiX, ChiY, x_ep[0], x_ep[1], &y[0], &y[1], gm);
                    switch (ti_num) {
                        case 10: euler_exp_f(psi, y, x_f, gp, dt); break;
                        case 20: ab2_pc_f(psi, y, x_f, gp, dt); break;
                        case 21: rk2_heun_f(psi, y, x_f, gp, dt, l_order, &lc); break;
                        case 30: rk3_classical_f(psi, y, x_f, gp, dt, l_order, &lc); break;
                        case 40: rk4_classical_f(psi, y, x_f, gp, dt, l_order, &lc); break;
                        case 31: rk3_optimized_f(psi, y, x_f, gp, dt); break;
                        case 41: rk4_optimized_b(psi, y, x_f, gp, dt, l_order, &lc); break;
                        default: x_f[0] = x_f[1] = 0;
                    }
                }
                fx[0] += x_f[0] * c1[k];  fy[0] += x_f[1] * c1[k];
                fx[1] += x_f[0] * cx[k];  fy[1] += x_f[1] * cx[k];
                fx[2] += x_f[0] * cy[k];  fy[2] += x_f[1] * cy[k];
                fx[3] += x_f[0] * cxy[k]; fy[3] += x_f[1] * cxy[k];
            }
            for (int p = 0; p < 4; ++p) { ChiX_new[p * N + In] = fx[p]; ChiY_new[p * N + In] = fy[p]; }
        }
    }
}

double og_incompressibility_check(const og_grid* gc, const og_grid* gm, const double* ChiX, const double* ChiY)
{
    double mx = 0.0;
    #pragma omp parallel for schedule(static) reduction(max:mx)
    for (int iY = 0; iY < gc->NY; ++iY)
        for (int iX = 0; iX < gc->NX; ++iX) {
            double x = gm->bounds[0] + iX * gc->hx + 0.5 * gc->hx;
            double y = gm->bounds[2] + iY * gc->hy + 0.5 * gc->hy;
            double d = fabs(1 - og_diffeo_grad_2D(ChiX, ChiY, x, y, gm));
            if (d > mx) mx = d;
        }
    return mx;
}

void og_sample_map_compact(const double* ChiX, const double* ChiY, double* x_y, const og_grid* gm, const og_grid* g)
{
    double LX = gm->bounds[1] - gm->bounds[0], LY = gm->bounds[3] - gm->bounds[2];
    #pragma omp parallel for schedule(static)
    for (int iY = 0; iY < g->NY; ++iY)
        for (int iX = 0; iX < g->NX; ++iX) {
            long In = (long)iY * g->NX + iX;
            double x = g->bounds[0] + iX * g->hx, y = g->bounds[2] + iY * g->hy;
            og_diffeo_interpolate_2D(ChiX, ChiY, x, y, &x, &y, gm);
            x_y[2 * In] = x - floor((x - gm->bounds[0]) / LX) * LX;
            x_y[2 * In + 1] = y - floor((y - gm->bounds[2]) / LY) * LY;
        }
}

void og_apply_map_compact(const double* ChiX, const double* ChiY, double* x_y, const og_grid* gm, const og_grid* g)
{
    double LX = gm->bounds[1] - gm->bounds[0], LY = gm->bounds[3] - gm->bounds[2];
    #pragma omp parallel for schedule(static)
    for (long In = 0; In < g->N; ++In) {
        double p0, p1;
        og_diffeo_interpolate_2D(ChiX, ChiY, x_y[2 * In], x_y[2 * In + 1], &p0, &p1, gm);
        x_y[2 * In] = p0 - floor((p0 - gm->bounds[0]) / LX) * LX;
        x_y[2 * In + 1] = p1 - floor((p1 - gm->bounds[2]) / LY) * LY;
    }
}

/* inputs of the analytic initial conditions that are not formulas: initial_params, the
 * 1000 uniform(-1, 1) values of mt19937_64 seed 0 (cmm-euler2d.cu:347-352) and the 98
 * cuRAND blob offsets of turbulence_gaussienne (cmm-init.cu:148-160), given by the caller */
static double og_params[10];
static double og_rand[1000 + 98];

void og_set_init_data(const double* params10, const double* table1098)
{
    if (params10) memcpy(og_params, params10, sizeof(og_params));
    if (table1098) memcpy(og_rand, table1098, sizeof(og_rand));
}

/* d_init_vorticity: src/simulation/cmm-init.cu:30-241 */
double og_init_vorticity(double x, double y, int ic)
{
    const double PI = OG_TWO_PI / 2, TP = OG_TWO_PI;
    switch (ic) {
        case 0: /* 4_nodes :45-52 */
            x -= floor(x / TP) * TP;
            y -= floor(y / TP) * TP;
            return cos(x) + cos(y) + 0.6 * cos(2 * x) + 0.2 * cos(3 * x);
        case 1: { /* quadropole :53-70, 5 x 5 periodic images */
            double r = 0;
            for (int iy = -2; iy <= 2; iy++)
                for (int ix = -2; ix <= 2; ix++) {
                    double dx = x - PI / 2 + ix * 2 * PI, dy = y - PI / 2 + iy * 2 * PI, s = 0.5;
                    double B = 0.6258473 / (s * s * s * s) * (dx * dy) * (dx * dx + dy * dy - 6 * s * s);
                    r += B * exp(-(dx * dx + dy * dy) / (2 * s * s));
                }
            return r;
        }
        case 2: { /* one_vortex :71-77 */
            double sg = TP * 0.125;
            return 1.0 / (TP * sg * sg) * exp(-((x - PI) * (x - PI) + (y - PI) * (y - PI)) / (2 * sg * sg));
        }
        case 3: case 4: { /* two_votices :78-89, three_vortices :90-109 (3 x 3 images) */
            double r = 0, LX = PI / 2, LY = PI / (2.0 * sqrt(2.0));
            for (int iy = -1; iy <= 1; iy++)
                for (int ix = -1; ix <= 1; ix++) {
                    double a = x + TP * ix, b = y + TP * iy, c = b + TP * iy;
                    double env = sin(0.5 * a) * sin(0.5 * a) * sin(0.5 * c) * sin(0.5 * c), e;
                    if (ic == 3)
                        e = exp(-((a - PI) * (a - PI) + (b - 0.33 * TP) * (b - 0.33 * TP)) * 5) +
                            exp(-((a - PI) * (a - PI) + (b - 0.67 * TP) * (b - 0.67 * TP)) * 5);
                    else
                        e = exp(-((a - PI - LX) * (a - PI - LX) + (b - PI) * (b - PI)) * 5) +
                            exp(-((a - PI + LX) * (a - PI + LX) + (b - PI) * (b - PI)) * 5) -
                            exp(-((a - PI + LX) * (a - PI + LX) + (b - PI - LY) * (b - PI - LY)) * 5);
                    r += env * e;
                }
            return r;
        }
        case 5: /* single_shear_layer :110-117 */
            return (1 + 0.01 * cos(2 * x)) * exp(-50.0 * (y - PI) * (y - PI));
        case 6: { /* tanh_shear_layer :118-129 */
            double d = 14 * 2 / TP, q = exp(-d * (y - PI)) + exp(d * (y - PI));
            return 5.0 * (1 + 0.01 * cos(2 * x)) * 4 / q / q;
        }
        case 7: { /* turbulence_gaussienne :130-171 */
            x -= floor(x / TP) * TP;
            y -= floor(y / TP) * TP;
            const int NB = 8;
            double sg = 0.2, den = 2 * sg * sg, amp = 1 / (TP * sg * sg), r = 0;
            for (int mx = 0; mx < NB; mx++)
                for (int my = 0; my < NB; my++) {
                    double ex = x - mx * TP / (NB - 1), ey = y - my * TP / (NB - 1);
                    r += amp * exp(-(ex * ex / den + ey * ey / den));
                }
            for (int mx = 0; mx < NB - 1; mx++)
                for (int my = 0; my < NB - 1; my++) {
                    double ex = x - (2 * mx + 1) * TP / (2 * (NB - 1)) + og_rand[1000 + mx * (NB - 1) + my];
                    double ey = y - (2 * my + 1) * TP / (2 * (NB - 1)) + og_rand[1049 + mx * (NB - 1) + my];
                    r -= amp * exp(-(ex * ex / den + ey * ey / den));
                }
            return r - 0.008857380480028442;
        }
        case 8: { /* gaussian_blobs :172-203, alternating signs, 2-cell border of images */
            x -= floor(x / TP) * TP;
            y -= floor(y / TP) * TP;
            const int NB = 10, border = 2;
            double sg = TP * 0.01, off = TP * 0.005, r = 0;
            int dir = 1;
            for (int mx = -border; mx < 2 * NB + border; mx++) {
                for (int my = -border; my < 2 * NB + border; my++) {
                    int bn = (int)((mx - floor(mx / (double)(NB * 2)) * NB * 2) + (my - floor(my / (double)(NB * 2)) * NB * 2) * NB * 2);
                    double ex = x - (mx + 0.5) * TP / (2 * NB) + og_rand[bn] * off;
                    double ey = y - (my + 0.5) * TP / (2 * NB) + og_rand[bn + NB * NB * 4] * off;
                    r += dir / (TP * sg * sg) * exp(-(ex * ex + ey * ey) / (2 * sg * sg));
                    dir = -dir;
                }
                dir = -dir;
            }
            return r;
        }
        case 9: { /* shielded_vortex :207-219 */
            double nu = 2e-1, xr = PI - x, yr = PI - y;
            return 1 / (2 * nu * nu * nu) * (4 * nu - xr * xr - yr * yr) * exp(-(xr * xr + yr * yr) / (4 * nu));
        }
        case 10: /* two_cosine :220-226 */
            x -= floor(x / TP) * TP;
            y -= floor(y / TP) * TP;
            return cos(x) * cos(y);
        case 11: { /* vortex_sheets :228-234, delta = 1 / sqrt(initial_params[0]) */
            double d = 1 / sqrt(og_params[0]), q = y - PI - sin(x) / 2.0;
            return exp(-q * q / (2 * d * d)) / sqrt(2 * PI) / d;
        }
        default: return 0.0;
    }
}

void og_apply_map_and_sample_from_hermite(const double* ChiX, const double* ChiY, double* fs, const double* H,
                                          const og_grid* gm, const og_grid* gv, const og_grid* gf,
                                          int molly, int padd)
{
    #pragma omp parallel for schedule(static)
    for (int iY = 0; iY < gv->NY; ++iY)
        for (int iX = 0; iX < gv->NX; ++iX) {
            long In = padd ? (long)iY * gv->NX_fft * 2 + iX : (long)iY * gv->NX + iX;
            double x = gm->bounds[0] + iX * gv->hx, y = gm->bounds[2] + iY * gv->hy;
            double x2, y2;
            if (molly == 4) {
                og_diffeo_interpolate_2D(ChiX, ChiY, x, y, &x2, &y2, gm);
                double moll = og_hermite_interpolate_2D(H, x2, y2, gf) / 3.0;
                for (int i = 0; i < 4; i++) {
                    /* reference precedence: (i>>1+1) == i>>2 */
                    x2 = x + gv->hx / 2.0 * ((i >> (1 + 1)) & 1) * (-1 + 2 * (i & 1));
                    y2 = y + gv->hy / 2.0 * ((i >> 1) & 1) * (-1 + 2 * (i & 1));
                    og_diffeo_interpolate_2D(ChiX, ChiY, x2, y2, &x2, &y2, gm);
                    moll += og_hermite_interpolate_2D(H, x2, y2, gf) / 6.0;
                }
                fs[In] = moll;
            } else if (molly == 8) {
                double moll = 0;
                for (int i = 0; i < 9; i++) {
                    x2 = x + gv->hx * (-1 + i % 3) / 2.0;
                    y2 = y + gv->hy * (-1 + i / 3) / 2.0;
                    og_diffeo_interpolate_2D(ChiX, ChiY, x2, y2, &x2, &y2, gm);
                    /* reference precedence: (1 + (i%3)) & 1 ... */
                    moll += ((1 + (i % 3)) & 1) * ((1 + (i / 3)) & 1) * og_hermite_interpolate_2D(H, x2, y2, gf) / 16.0;
                }
                fs[In] = moll;
            } else {
                og_diffeo_interpolate_2D(ChiX, ChiY, x, y, &x, &y, gm);
                fs[In] = og_hermite_interpolate_2D(H, x, y, gf);
            }
        }
}

/* Particle_advect: src/numerical/cmm-particles.cu:119-276 (fluid tracers) */
void og_particle_advect(int num, double dt, double* pos, const double* psi, const og_grid* g,
                        int ti, int l_order, const double* Lp12)
{
    long N = g->N;
    double LX = g->bounds[1] - g->bounds[0], LY = g->bounds[3] - g->bounds[2];
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < num; ++i) {
        double p[2] = {pos[2 * i], pos[2 * i + 1]};
        switch (ti) {
            case 10: {
                double u[2];
                og_hermite_interpolate_grad_2D(psi + 4 * N, p, u, g, 1);
                p[0] += dt * u[0]; p[1] += dt * u[1];
                break;
            }
            case 20: {
                double k[4];
                og_hermite_interpolate_grad_2D(psi + 4 * N, p, k, g, 1);
                k[2] = p[0] + dt * k[0]; k[3] = p[1] + dt * k[1];
                og_hermite_interpolate_grad_2D(psi, k + 2, k + 2, g, 1);
                p[0] += dt * (k[0] + k[2]) / 2; p[1] += dt * (k[1] + k[3]) / 2;
                break;
            }
            case 30: {
                double u[8], k[6];
                og_hermite_interpolate_grad_2D(psi + 4 * N, p, k, g, 1);
                k[2] = p[0] + dt * k[0] / 2.0; k[3] = p[1] + dt * k[1] / 2.0;
                og_hermite_interpolate_grad_2D(psi, k + 2, u, g, l_order);
                k[2] = Lp12[0] * u[0]; k[3] = Lp12[0] * u[1];
                for (int i_l = 1; i_l < l_order; i_l++) { k[2] += Lp12[i_l] * u[i_l * 2]; k[3] += Lp12[i_l] * u[i_l * 2 + 1]; }
                k[4] = p[0] - dt * k[0] + 2 * dt * k[2]; k[5] = p[1] - dt * k[1] + 2 * dt * k[3];
                og_hermite_interpolate_grad_2D(psi, k + 4, k + 4, g, 1);
                p[0] += dt * (k[0] + 4 * k[2] + k[4]) / 6.0;
                p[1] += dt * (k[1] + 4 * k[3] + k[5]) / 6.0;
                break;
            }
            case 40: {   /* :206-240 */
                double k1[2], k2[2], k3[2], k4[2], y[2];
                vel_level(psi, 1, p, k1, g);
                y[0] = p[0] + dt * k1[0] / 2.0; y[1] = p[1] + dt * k1[1] / 2.0;
                vel_comb(psi, Lp12, l_order, y, k2, g);
                y[0] = p[0] + dt * k2[0] / 2.0; y[1] = p[1] + dt * k2[1] / 2.0;
                vel_comb(psi, Lp12, l_order, y, k3, g);
                y[0] = p[0] + dt * k3[0]; y[1] = p[1] + dt * k3[1];
                vel_level(psi, 0, y, k4, g);
                p[0] += dt * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0]) / 6.0;
                p[1] += dt * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1]) / 6.0;
                break;
            }
            case 31: {   /* :242-262 */
                double k1[2], k2[2], k3[2], y[2];
                vel_level(psi, 1, p, k1, g);
                y[0] = p[0] + dt * k1[0]; y[1] = p[1] + dt * k1[1];
                vel_level(psi, 0, y, k2, g);
                y[0] = p[0] + dt * (k1[0] - 2 * k2[0]); y[1] = p[1] + dt * (k1[1] - 2 * k2[1]);
                vel_level(psi, 2, y, k3, g);
                p[0] += dt * (8 * k1[0] + 5 * k2[0] - k3[0]) / 12.0;
                p[1] += dt * (8 * k1[1] + 5 * k2[1] - k3[1]) / 12.0;
                break;
            }
            case 41: {   /* :263-293 */
                double k1[2], k2[2], k3[2], k4[2], y[2];
                vel_level(psi, 1, p, k1, g);
                y[0] = p[0] + dt * k1[0]; y[1] = p[1] + dt * k1[1];
                vel_level(psi, 0, y, k2, g);
                y[0] = p[0] + dt / 8.0 * (3 * k1[0] + k2[0]); y[1] = p[1] + dt / 8.0 * (3 * k1[1] + k2[1]);
                vel_comb(psi, Lp12, l_order, y, k3, g);
                y[0] = p[0] + dt / 3.0 * (-k2[0] + 4 * k3[0]); y[1] = p[1] + dt / 3.0 * (-k2[1] + 4 * k3[1]);
                vel_level(psi, 0, y, k4, g);
                p[0] += dt * (2 * k1[0] - k2[0] + 8 * k3[0] + 3 * k4[0]) / 12.0;
                p[1] += dt * (2 * k1[1] - k2[1] + 8 * k3[1] + 3 * k4[1]) / 12.0;
                break;
            }
            default: p[0] = p[1] = 0; break;
        }
        pos[2 * i] = p[0] - floor((p[0] - g->bounds[0]) / LX) * LX;
        pos[2 * i + 1] = p[1] - floor((p[1] - g->bounds[2]) / LY) * LY;
    }
}

/* Particle_advect_inertia: src/numerical/cmm-particles.cu:280-551.  State (x, v); the
 * particle relaxes to the fluid velocity u with time constant tau:
 *   dx/dt = v,  dv/dt = -(v - u(x, t)) / tau
 * u(t_n) is psi level 1, u(t_{n+1}) level 0, u(t_{n-1}) level 2 and u(t_{n+1/2}) the Lp12
 * combination, as for the tracers. */
void og_particle_advect_inertia(int num, double dt, double* pos, double* vel, const double* psi, const og_grid* g,
                                double tau, int ti, int l_order, const double* Lp12)
{
    double LX = g->bounds[1] - g->bounds[0], LY = g->bounds[3] - g->bounds[2];
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < num; ++i) {
        double p[2] = {pos[2 * i], pos[2 * i + 1]};
        double v[2] = {vel[2 * i], vel[2 * i + 1]};
        double u[2], y[2];
        switch (ti) {
            case 10: {   /* :300-317 */
                vel_level(psi, 1, p, u, g);
                p[0] += dt * v[0]; p[1] += dt * v[1];
                vel[2 * i] -= dt * (v[0] - u[0]) / tau;
                vel[2 * i + 1] -= dt * (v[1] - u[1]) / tau;
                break;
            }
            case 20: {   /* :318-348 */
                vel_level(psi, 1, p, u, g);
                double a1[2] = {-(v[0] - u[0]) / tau, -(v[1] - u[1]) / tau};
                double x2[2] = {v[0] + dt * a1[0], v[1] + dt * a1[1]};
                y[0] = p[0] + dt * v[0]; y[1] = p[1] + dt * v[1];
                vel_level(psi, 0, y, u, g);
                double a2[2] = {-(x2[0] - u[0]) / tau, -(x2[1] - u[1]) / tau};
                p[0] += dt / 2.0 * (v[0] + x2[0]); p[1] += dt / 2.0 * (v[1] + x2[1]);
                vel[2 * i] += dt / 2.0 * (a1[0] + a2[0]);
                vel[2 * i + 1] += dt / 2.0 * (a1[1] + a2[1]);
                break;
            }
            case 30: {   /* :349-397 */
                vel_level(psi, 1, p, u, g);
                double a1[2] = {-(v[0] - u[0]) / tau, -(v[1] - u[1]) / tau};
                double x2[2] = {v[0] + dt / 2.0 * a1[0], v[1] + dt / 2.0 * a1[1]};
                y[0] = p[0] + dt / 2.0 * v[0]; y[1] = p[1] + dt / 2.0 * v[1];
                vel_comb(psi, Lp12, l_order, y, u, g);
                double a2[2] = {-(x2[0] - u[0]) / tau, -(x2[1] - u[1]) / tau};
                double x3[2] = {v[0] + dt * (-a1[0] + 2 * a2[0]), v[1] + dt * (-a1[1] + 2 * a2[1])};
                y[0] = p[0] + dt * (-v[0] + 2 * x2[0]); y[1] = p[1] + dt * (-v[1] + 2 * x2[1]);
                vel_level(psi, 0, y, u, g);
                double a3[2] = {-(x3[0] - u[0]) / tau, -(x3[1] - u[1]) / tau};
                p[0] += dt / 6.0 * (v[0] + 4 * x2[0] + x3[0]); p[1] += dt / 6.0 * (v[1] + 4 * x2[1] + x3[1]);
                vel[2 * i] += dt / 6.0 * (a1[0] + 4 * a2[0] + a3[0]);
                vel[2 * i + 1] += dt / 6.0 * (a1[1] + 4 * a2[1] + a3[1]);
                break;
            }
            case 40: {   /* :398-462 */
                vel_level(psi, 1, p, u, g);
                double a1[2] = {-(v[0] - u[0]) / tau, -(v[1] - u[1]) / tau};
                double x2[2] = {v[0] + dt / 2.0 * a1[0], v[1] + dt / 2.0 * a1[1]};
                y[0] = p[0] + dt / 2.0 * v[0]; y[1] = p[1] + dt / 2.0 * v[1];
                vel_comb(psi, Lp12, l_order, y, u, g);
                double a2[2] = {-(x2[0] - u[0]) / tau, -(x2[1] - u[1]) / tau};
                double x3[2] = {v[0] + dt / 2.0 * a2[0], v[1] + dt / 2.0 * a2[1]};
                y[0] = p[0] + dt / 2.0 * x2[0]; y[1] = p[1] + dt / 2.0 * x2[1];
                vel_comb(psi, Lp12, l_order, y, u, g);
                double a3[2] = {-(x3[0] - u[0]) / tau, -(x3[1] - u[1]) / tau};
                double x4[2] = {v[0] + dt * a3[0], v[1] + dt * a3[1]};
                y[0] = p[0] + dt * x3[0]; y[1] = p[1] + dt * x3[1];
                vel_level(psi, 0, y, u, g);
                double a4[2] = {-(x4[0] - u[0]) / tau, -(x4[1] - u[1]) / tau};
                p[0] += dt / 6.0 * (v[0] + 2 * x2[0] + 2 * x3[0] + x4[0]);
                p[1] += dt / 6.0 * (v[1] + 2 * x2[1] + 2 * x3[1] + x4[1]);
                vel[2 * i] += dt / 6.0 * (a1[0] + 2 * a2[0] + 2 * a3[0] + a4[0]);
                vel[2 * i + 1] += dt / 6.0 * (a1[1] + 2 * a2[1] + 2 * a3[1] + a4[1]);
                break;
            }
            case 31: {   /* :463-497 */
                vel_level(psi, 1, p, u, g);
                double a1[2] = {-(v[0] - u[0]) / tau, -(v[1] - u[1]) / tau};
                double x2[2] = {v[0] + dt * a1[0], v[1] + dt * a1[1]};
                y[0] = p[0] + dt * v[0]; y[1] = p[1] + dt * v[1];
                vel_level(psi, 0, y, u, g);
                double a2[2] = {-(x2[0] - u[0]) / tau, -(x2[1] - u[1]) / tau};
                double x3[2] = {v[0] + dt * (a1[0] - 2 * a2[0]), v[1] + dt * (a1[1] - 2 * a2[1])};
                y[0] = p[0] + dt * (v[0] - 2 * x2[0]); y[1] = p[1] + dt * (v[1] - 2 * x2[1]);
                vel_level(psi, 2, y, u, g);
                double a3[2] = {-(x3[0] - u[0]) / tau, -(x3[1] - u[1]) / tau};
                p[0] += dt / 12.0 * (8 * v[0] + 5 * x2[0] - x3[0]); p[1] += dt / 12.0 * (8 * v[1] + 5 * x2[1] - x3[1]);
                vel[2 * i] += dt / 12.0 * (8 * a1[0] + 5 * a2[0] - a3[0]);
                vel[2 * i + 1] += dt / 12.0 * (8 * a1[1] + 5 * a2[1] - a3[1]);
                break;
            }
            case 41: {   /* :498-545 */
                vel_level(psi, 1, p, u, g);
                double a1[2] = {-(v[0] - u[0]) / tau, -(v[1] - u[1]) / tau};
                double x2[2] = {v[0] + dt * a1[0], v[1] + dt * a1[1]};
                y[0] = p[0] + dt * v[0]; y[1] = p[1] + dt * v[1];
                vel_level(psi, 0, y, u, g);
                double a2[2] = {-(x2[0] - u[0]) / tau, -(x2[1] - u[1]) / tau};
                double x3[2] = {v[0] + dt / 8.0 * (3 * a1[0] + a2[0]), v[1] + dt / 8.0 * (3 * a1[1] + a2[1])};
                y[0] = p[0] + dt / 8.0 * (3 * v[0] + x2[0]); y[1] = p[1] + dt / 8.0 * (3 * v[1] + x2[1]);
                vel_comb(psi, Lp12, l_order, y, u, g);
                double a3[2] = {-(x3[0] - u[0]) / tau, -(x3[1] - u[1]) / tau};
                double x4[2] = {v[0] + dt / 3.0 * (-a2[0] + 4 * a3[0]), v[1] + dt / 3.0 * (-a2[1] + 4 * a3[1])};
                y[0] = p[0] + dt / 3.0 * (-x2[0] + 4 * x3[0]); y[1] = p[1] + dt / 3.0 * (-x2[1] + 4 * x3[1]);
                vel_level(psi, 0, y, u, g);
                double a4[2] = {-(x4[0] - u[0]) / tau, -(x4[1] - u[1]) / tau};
                p[0] += dt / 12.0 * (2 * v[0] - x2[0] + 8 * x3[0] + 3 * x4[0]);
                p[1] += dt / 12.0 * (2 * v[1] - x2[1] + 8 * x3[1] + 3 * x4[1]);
                vel[2 * i] += dt / 12.0 * (2 * a1[0] - a2[0] + 8 * a3[0] + 3 * a4[0]);
                vel[2 * i + 1] += dt / 12.0 * (2 * a1[1] - a2[1] + 8 * a3[1] + 3 * a4[1]);
                break;
            }
            default: p[0] = p[1] = 0; vel[2 * i] = vel[2 * i + 1] = 0; break;
        }
        pos[2 * i] = p[0] - floor((p[0] - g->bounds[0]) / LX) * LX;
        pos[2 * i + 1] = p[1] - floor((p[1] - g->bounds[2]) / LY) * LY;
    }
}

/* Particle_advect_inertia_init: cmm-particles.cu:50-60 -- v = u of psi level 0 at x */
void og_particle_inertia_init(int num, const double* pos, double* vel, const double* psi, const og_grid* g)
{
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < num; ++i) vel_level(psi, 0, pos + 2 * i, vel + 2 * i, g);
}

/* ------------------------------------------------------------------ */
/* driver state                                                        */
/* ------------------------------------------------------------------ */
struct og_state {
    og_settings s;
    og_grid gc, gf, gp, gv, gd;
    double *ChiX, *ChiY, *ChiX_new, *ChiY_new;
    double* psi;            /* L levels x 4 planes x Np */
    double* vort;           /* coarse */
    double* vort_fine;      /* 4 planes x Nf */
    double* vort_disc;      /* 4 planes x Nd (discrete IC Hermite) */
    double *stackX, *stackY; int n_maps;
    double* xy;             /* 2*Nf */
    double* cbuf1; double* cbuf2; double* rbuf;
    double* parts[8];
    double* vels[8];        /* inertial velocity state per set */
    /* forward map: active map, its stack, the forwarded particles' initial positions and
     * the stack index each forwarded set starts from (init_map), last step's monitors */
    double *ChiX_f, *ChiY_f, *stackX_f, *stackY_f;
    double* fparts[8];
    int init_map[8];
    double einc_f, einv;
    double* t_vec; double* dt_vec; int t_cap;
    int loop_ctr, old_ctr;
};

static void* xmalloc(size_t n) { void* p = malloc(n ? n : 1); if (p) memset(p, 0, n ? n : 1); return p; }

og_state* og_create(const og_settings* s)
{
    og_state* st = (og_state*)xmalloc(sizeof(og_state));
    st->s = *s;
    og_grid_fill(&st->gc, s->grid_coarse, s->grid_coarse, s->bounds);
    og_grid_fill(&st->gf, s->grid_fine, s->grid_fine, s->bounds);
    og_grid_fill(&st->gp, s->grid_psi, s->grid_psi, s->bounds);
    og_grid_fill(&st->gv, s->grid_vort, s->grid_vort, s->bounds);
    og_grid_fill(&st->gd, s->initial_discrete ? s->initial_discrete_grid : 1,
                 s->initial_discrete ? s->initial_discrete_grid : 1, s->bounds);
    long Nc = st->gc.N, Nf = st->gf.N, Np = st->gp.N;
    st->ChiX = (double*)xmalloc(sizeof(double) * 4 * Nc);
    st->ChiY = (double*)xmalloc(sizeof(double) * 4 * Nc);
    st->ChiX_new = (double*)xmalloc(sizeof(double) * 4 * Nc);
    st->ChiY_new = (double*)xmalloc(sizeof(double) * 4 * Nc);
    int L = s->lagrange_order < 1 ? 1 : s->lagrange_order;
    st->psi = (double*)xmalloc(sizeof(double) * 4 * Np * L);
    st->vort = (double*)xmalloc(sizeof(double) * Nc);
    st->vort_fine = (double*)xmalloc(sizeof(double) * 4 * Nf);
    st->vort_disc = (double*)xmalloc(sizeof(double) * 4 * st->gd.N);
    st->stackX = (double*)xmalloc(sizeof(double) * 4 * Nc * (size_t)(s->max_maps > 0 ? s->max_maps : 1));
    st->stackY = (double*)xmalloc(sizeof(double) * 4 * Nc * (size_t)(s->max_maps > 0 ? s->max_maps : 1));
    st->xy = (double*)xmalloc(sizeof(double) * 2 * Nf);
    long cmax = st->gf.Nfft;
    if (st->gv.Nfft > cmax) cmax = st->gv.Nfft;
    if (st->gp.Nfft > cmax) cmax = st->gp.Nfft;
    if (st->gd.Nfft > cmax) cmax = st->gd.Nfft;
    if (st->gc.Nfft > cmax) cmax = st->gc.Nfft;
    st->cbuf1 = (double*)xmalloc(sizeof(double) * 2 * cmax);
    st->cbuf2 = (double*)xmalloc(sizeof(double) * 2 * cmax);
    long rmax = st->gf.N > st->gv.N ? st->gf.N : st->gv.N;
    if (st->gc.N > rmax) rmax = st->gc.N;
    st->rbuf = (double*)xmalloc(sizeof(double) * rmax);
    for (int i = 0; i < s->n_particle_sets; ++i) {
        st->parts[i] = (double*)xmalloc(sizeof(double) * 2 * (size_t)s->psets[i].num);
        st->vels[i] = (double*)xmalloc(sizeof(double) * 2 * (size_t)s->psets[i].num);
    }
    if (s->forward_map) {
        st->ChiX_f = (double*)xmalloc(sizeof(double) * 4 * Nc);
        st->ChiY_f = (double*)xmalloc(sizeof(double) * 4 * Nc);
        st->stackX_f = (double*)xmalloc(sizeof(double) * 4 * Nc * (size_t)(s->max_maps > 0 ? s->max_maps : 1));
        st->stackY_f = (double*)xmalloc(sizeof(double) * 4 * Nc * (size_t)(s->max_maps > 0 ? s->max_maps : 1));
        for (int i = 0; i < s->n_fwd_sets; ++i)
            st->fparts[i] = (double*)xmalloc(sizeof(double) * 2 * (size_t)(s->fsets[i].num > 0 ? s->fsets[i].num : 1));
    }
    st->t_cap = 1 << 16;
    st->t_vec = (double*)xmalloc(sizeof(double) * st->t_cap);
    st->dt_vec = (double*)xmalloc(sizeof(double) * st->t_cap);
    return st;
}

void og_destroy(og_state* st)
{
    if (!st) return;
    free(st->ChiX); free(st->ChiY); free(st->ChiX_new); free(st->ChiY_new);
    free(st->psi); free(st->vort); free(st->vort_fine); free(st->vort_disc);
    free(st->stackX); free(st->stackY); free(st->xy);
    free(st->cbuf1); free(st->cbuf2); free(st->rbuf);
    for (int i = 0; i < st->s.n_particle_sets; ++i) { free(st->parts[i]); free(st->vels[i]); }
    free(st->ChiX_f); free(st->ChiY_f); free(st->stackX_f); free(st->stackY_f);
    for (int i = 0; i < st->s.n_fwd_sets; ++i) free(st->fparts[i]);
    free(st->t_vec); free(st->dt_vec);
    free(st);
}

int og_set_discrete_initial(og_state* st, const double* values)
{
    /* src/simulation/cmm-euler2d.cu:325-344: D2Z, normalise, fourier_hermite */
    og_grid* g = &st->gd;
    og_fft_d2z(g, values, st->cbuf1);
    og_normalize_h(st->cbuf1, g);
    og_fourier_hermite(g, st->cbuf1, st->vort_disc);
    return 0;
}

int og_set_particles(og_state* st, int i, const double* pos)
{
    if (i < 0 || i >= st->s.n_particle_sets) return -1;
    memcpy(st->parts[i], pos, sizeof(double) * 2 * (size_t)st->s.psets[i].num);
    return 0;
}

/* apply_map_stack (direction -1) + k_h_sample_from_init: cmm-simulation-host.cu:112-128,
 * cmm-simulation-kernel.cu:342-373; stack = n maps of [X planes | Y planes] */
void og_compose_sample_var(const double* ChiX, const double* ChiY, const double* stack, int n, const og_grid* gm,
                           const og_grid* gt, int var_num, int ic_num, const double* discrete, const og_grid* gd,
                           double* out)
{
    double* xy = (double*)xmalloc(sizeof(double) * 2 * gt->N);
    og_sample_map_compact(ChiX, ChiY, xy, gm, gt);
    for (int i = n - 1; i >= 0; i--)
        og_apply_map_compact(stack + 8 * gm->N * (size_t)i, stack + 8 * gm->N * (size_t)i + 4 * gm->N, xy, gm, gt);
    #pragma omp parallel for schedule(static)
    for (long In = 0; In < gt->N; ++In)
        out[In] = discrete ? og_hermite_interpolate_2D(discrete, xy[2 * In], xy[2 * In + 1], gd)
                  : var_num == 2 ? og_init_distribution(xy[2 * In], xy[2 * In + 1], ic_num)
                                 : og_init_vorticity(xy[2 * In], xy[2 * In + 1], ic_num);
    free(xy);
}

void og_compose_sample(const double* ChiX, const double* ChiY, const double* stack, int n, const og_grid* gm,
                       const og_grid* gt, int ic_num, const double* discrete, const og_grid* gd, double* out)
{
    og_compose_sample_var(ChiX, ChiY, stack, n, gm, gt, 0, ic_num, discrete, gd, out);
}

/* translate_initial_condition_through_map_stack: cmm-simulation-host.cu:299-327 */
static void translate_ic(og_state* st)
{
    og_grid* gf = &st->gf; long Nc = st->gc.N;
    og_sample_map_compact(st->ChiX, st->ChiY, st->xy, &st->gc, gf);
    for (int i = st->n_maps - 1; i >= 0; i--)
        og_apply_map_compact(st->stackX + 4 * Nc * (size_t)i, st->stackY + 4 * Nc * (size_t)i, st->xy, &st->gc, gf);
    /* k_h_sample_from_init: cmm-simulation-kernel.cu:342-373 */
    #pragma omp parallel for schedule(static)
    for (long In = 0; In < gf->N; ++In) {
        if (!st->s.initial_discrete && st->s.simulation_type_num == 2)   /* ID_DIST_FUNC, cmm-vlasov1d.cu:538 */
            st->rbuf[In] = og_init_distribution(st->xy[2 * In], st->xy[2 * In + 1], st->s.initial_condition_num);
        else if (!st->s.initial_discrete)
            st->rbuf[In] = og_init_vorticity(st->xy[2 * In], st->xy[2 * In + 1], st->s.initial_condition_num);
        else
            st->rbuf[In] = og_hermite_interpolate_2D(st->vort_disc, st->xy[2 * In], st->xy[2 * In + 1], &st->gd);
    }
    og_fft_d2z(gf, st->rbuf, st->cbuf1);
    og_normalize_h(st->cbuf1, gf);
    og_fourier_hermite(gf, st->cbuf1, st->vort_fine);
}

/* evaluate_stream_hermite: cmm-simulation-host.cu:333-375 (Euler) or
 * evaluate_potential_from_density_hermite (Vlasov, og_vlasov.c) */
static int evaluate_stream(og_state* st)
{
    og_grid* gv = &st->gv; og_grid* gp = &st->gp;
    if (st->s.simulation_type_num == 2)
        return og_vlasov_potential(st->ChiX, st->ChiY, st->vort_fine, &st->gc, gv, &st->gf, gp,
                                   st->s.molly_stencil, st->psi);
    double* fs = (double*)xmalloc(sizeof(double) * gv->N);
    og_apply_map_and_sample_from_hermite(st->ChiX, st->ChiY, fs, st->vort_fine, &st->gc, gv, &st->gf,
                                         st->s.molly_stencil, 0);
    og_fft_d2z(gv, fs, st->cbuf1);
    free(fs);
    og_normalize_h(st->cbuf1, gv);
    if (gv->NX != gp->NX || gv->NY != gp->NY) og_fft_grid_move(st->cbuf1, st->cbuf2, gp, gv);
    else memcpy(st->cbuf2, st->cbuf1, sizeof(double) * 2 * gv->Nfft);
    og_fft_cut_off_scale_h(st->cbuf2, gp, st->s.freq_cut_psi);
    og_fft_iLap_h(st->cbuf2, st->cbuf1, gp);
    og_fourier_hermite(gp, st->cbuf1, st->psi);
    return 0;
}

static void coarse_vort(og_state* st)
{
    og_apply_map_and_sample_from_hermite(st->ChiX, st->ChiY, st->vort, st->vort_fine, &st->gc, &st->gc,
                                         &st->gf, 0, 0);
}

/* advect_using_stream_hermite (direction -1): cmm-simulation-host.cu:64-104 */
static void advect(og_state* st, const double* t, const double* dt, int loop_ctr, int ti_num, int l_order)
{
    double L1[4] = {0, 0, 0, 0}, L12[4] = {0, 0, 0, 0};
    int lcl = loop_ctr + l_order - 1;
    for (int i = 0; i < l_order; ++i) {
        L1[i] = og_get_L_coefficient(t, t[lcl + 1], lcl, i, l_order);
        L12[i] = og_get_L_coefficient(t, t[lcl] + dt[lcl + 1] / 2.0, lcl, i, l_order);
    }
    double c1[12], cx[12], cy[12], cxy[12];
    og_map_update_coefficients(st->s.map_update_order_num, st->s.map_epsilon, c1, cx, cy, cxy);
    og_advect_map(st->ChiX, st->ChiY, st->ChiX_new, st->ChiY_new, st->psi, &st->gc, &st->gp,
                  dt[lcl + 1], st->s.map_epsilon, ti_num, st->s.map_update_order_num, l_order,
                  L1, L12, c1, cx, cy, cxy);
    double* tx = st->ChiX; st->ChiX = st->ChiX_new; st->ChiX_new = tx;
    double* ty = st->ChiY; st->ChiY = st->ChiY_new; st->ChiY_new = ty;
}

/* the forward map's step: advect_using_stream_hermite with direction 1 (cmm-euler2d.cu:780-786) */
static void advect_forward(og_state* st, const double* t, const double* dt, int loop_ctr, int ti_num, int l_order)
{
    double L1[4] = {0, 0, 0, 0}, L12[4] = {0, 0, 0, 0};
    int lcl = loop_ctr + l_order - 1;
    for (int i = 0; i < l_order; ++i) {
        L1[i] = og_get_L_coefficient(t, t[lcl + 1], lcl, i, l_order);
        L12[i] = og_get_L_coefficient(t, t[lcl] + dt[lcl + 1] / 2.0, lcl, i, l_order);
    }
    double c1[12], cx[12], cy[12], cxy[12];
    og_map_update_coefficients(st->s.map_update_order_num, st->s.map_epsilon, c1, cx, cy, cxy);
    advect_map_dir(st->ChiX_f, st->ChiY_f, st->ChiX_new, st->ChiY_new, st->psi, &st->gc, &st->gp, dt[lcl + 1],
                   st->s.map_epsilon, ti_num, st->s.map_update_order_num, l_order, L1, L12, c1, cx, cy, cxy, 1);
    double* tx = st->ChiX_f; st->ChiX_f = st->ChiX_new; st->ChiX_new = tx;
    double* ty = st->ChiY_f; st->ChiY_f = st->ChiY_new; st->ChiY_new = ty;
}

/* k_swap_h over whole Hermite levels: cmm-simulation-kernel.cu:62-74 */
static void swap_levels(og_state* st, int a, int b)
{
    long n = 4 * st->gp.N;
    double* pa = st->psi + n * a; double* pb = st->psi + n * b;
    for (long i = 0; i < n; ++i) { double t = pa[i]; pa[i] = pb[i]; pb[i] = t; }
}

int og_init(og_state* st)
{
    og_settings* s = &st->s;
    long Np4 = 4 * st->gp.N;
    og_init_diffeo(st->ChiX, st->ChiY, &st->gc);
    if (s->forward_map) og_init_diffeo(st->ChiX_f, st->ChiY_f, &st->gc);
    for (int i = 0; i < 8; ++i) st->init_map[i] = 0;
    st->n_maps = 0;
    translate_ic(st);
    if (evaluate_stream(st)) return -1;
    coarse_vort(st);
    /* Lagrange history initialisation: src/simulation/cmm-euler2d.cu:520-619 */
    int Lo = s->lagrange_order;
    if (Lo > 1) {
        double dt = s->dt;
        double dt_now = dt * pow(-1, Lo);
        double t_init[5] = {0, dt_now, 2 * dt_now, 3 * dt_now, 4 * dt_now};
        double dt_init[5] = {dt_now, dt_now, dt_now, dt_now, dt_now};
        for (int i_order = 1; i_order <= Lo; i_order++) {
            if (!s->lagrange_init_higher_order && i_order != Lo) {
                for (int i = 0; i < 5; i++) { dt_init[i] = -dt_init[i]; t_init[i] = -t_init[i]; }
                continue;
            }
            int ti_num, l_now;
            if (s->lagrange_init_higher_order) {
                switch (i_order) {
                    case 1: ti_num = 10; break;
                    case 2: ti_num = 21; break;
                    case 3: ti_num = 30; break;
                    default: ti_num = 40; break;
                }
                l_now = i_order;
            } else { ti_num = 10; l_now = 1; }
            int n_steps = i_order - (i_order == Lo);
            for (int i_step = 1; i_step <= n_steps; i_step++) {
                advect(st, t_init, dt_init, 0, ti_num, l_now);
                for (int i_l = 1; i_l <= n_steps; i_l++)
                    memcpy(st->psi + Np4 * (n_steps - i_l + 1), st->psi + Np4 * (n_steps - i_l), sizeof(double) * Np4);
                if (evaluate_stream(st)) return -1;
            }
            for (int i = 0; i < 5; i++) { dt_init[i] = -dt_init[i]; t_init[i] = -t_init[i]; }
            swap_levels(st, 0, n_steps);
            if (n_steps >= 3) swap_levels(st, 1, 2);
            og_init_diffeo(st->ChiX, st->ChiY, &st->gc);
        }
        og_init_diffeo(st->ChiX, st->ChiY, &st->gc);
    }
    /* inertial particles start at the fluid velocity or at rest (cmm-euler2d.cu:620-632) */
    for (int i_p = 0; i_p < s->n_particle_sets; ++i_p) {
        og_particle_set* ps = &s->psets[i_p];
        if (ps->tau == 0) continue;
        if (ps->init_vel) og_particle_inertia_init(ps->num, st->parts[i_p], st->vels[i_p], st->psi, &st->gp);
        else memset(st->vels[i_p], 0, sizeof(double) * 2 * (size_t)ps->num);
    }
    for (int i = 0; i < Lo; i++) { st->t_vec[i] = 0 - (Lo - 1 - i) * s->dt; st->dt_vec[i] = s->dt; }
    st->loop_ctr = 0; st->old_ctr = 0;
    return 0;
}

/* Restart from a stored map stack instead of og_init: readMapStack
 * (src/simulation/cmm-simulation-host.cu:1256-1302) and the restart branch of the driver
 * (src/simulation/cmm-euler2d.cu:634-685, clock :711-715).  The n stored sub-maps become the
 * stack and the initial condition is translated through them with the identity as the active
 * map; then the stored active map and psi levels 1..L-1 are put in place, psi level 0 and the
 * coarse vorticity are computed from them, and the clock starts at restart_time.  Particle
 * positions are set beforehand with og_set_particles.  Returns -1 when n exceeds the stack. */
int og_restart(og_state* st, double restart_time, int n_maps, const double* stackX, const double* stackY,
               const double* chix, const double* chiy, const double* psi_prev)
{
    og_settings* s = &st->s;
    long Nc4 = 4 * st->gc.N, Np4 = 4 * st->gp.N;
    int Lo = s->lagrange_order;
    if (n_maps < 0 || n_maps > s->max_maps) return -1;
    if (n_maps > 0) {
        memcpy(st->stackX, stackX, sizeof(double) * Nc4 * (size_t)n_maps);
        memcpy(st->stackY, stackY, sizeof(double) * Nc4 * (size_t)n_maps);
    }
    st->n_maps = n_maps;
    og_init_diffeo(st->ChiX, st->ChiY, &st->gc);
    translate_ic(st);
    memcpy(st->ChiX, chix, sizeof(double) * Nc4);
    memcpy(st->ChiY, chiy, sizeof(double) * Nc4);
    for (int l = 1; l < Lo; ++l) memcpy(st->psi + Np4 * l, psi_prev + Np4 * (l - 1), sizeof(double) * Np4);
    if (evaluate_stream(st)) return -1;
    coarse_vort(st);
    for (int i = 0; i < Lo; i++) { st->t_vec[i] = restart_time - (Lo - 1 - i) * s->dt; st->dt_vec[i] = s->dt; }
    st->loop_ctr = 0; st->old_ctr = 0;
    return 0;
}

const double* og_stack_x(const og_state* st) { return st->stackX; }
const double* og_stack_y(const og_state* st) { return st->stackY; }

int og_step(og_state* st, double dt_now, double* e_inc, int* remapped)
{
    og_settings* s = &st->s;
    int Lo = s->lagrange_order;
    int lcl = st->loop_ctr + Lo - 1;
    if (lcl + 2 >= st->t_cap) return -1;
    st->t_vec[lcl + 1] = st->t_vec[lcl] + dt_now;
    st->dt_vec[lcl + 1] = dt_now;
    advect(st, st->t_vec, st->dt_vec, st->loop_ctr, s->time_integration_num, Lo);
    if (s->forward_map) advect_forward(st, st->t_vec, st->dt_vec, st->loop_ctr, s->time_integration_num, Lo);
    double einc = og_incompressibility_check(&st->gf, &st->gc, st->ChiX, st->ChiY);
    *e_inc = einc; *remapped = 0;
    if (s->simulation_type_num == 2 && (einc <= 0 || einc > 1e15)) return 2;
    /* forward map: invertibility and incompressibility on the coarse grid, and a forced remap
     * in the step that reaches a forwarded set's start time (cmm-euler2d.cu:795-811) */
    int forwarded_init = 0;
    if (s->forward_map) {
        st->einv = og_invertibility_check(&st->gc, &st->gc, st->ChiX, st->ChiY, &st->gc, st->ChiX_f, st->ChiY_f);
        st->einc_f = og_incompressibility_check(&st->gc, &st->gc, st->ChiX_f, st->ChiY_f);
        for (int i_p = 0; i_p < s->n_fwd_sets; ++i_p) {
            double d = st->t_vec[lcl + 1] - s->fsets[i_p].init_time + s->dt * 1e-5;
            if (d < st->dt_vec[lcl + 1] && d >= 0) {
                forwarded_init = 1;
                st->init_map[i_p] = st->n_maps + 1;
            }
        }
    }
    int saturated = 0;
    if ((einc > s->incomp_threshold && !s->skip_remapping) || forwarded_init) {
        if (st->n_maps >= s->max_maps) saturated = 1;
        else {
            st->old_ctr = st->loop_ctr;
            translate_ic(st);
            long Nc4 = 4 * st->gc.N;
            memcpy(st->stackX + Nc4 * (size_t)st->n_maps, st->ChiX, sizeof(double) * Nc4);
            memcpy(st->stackY + Nc4 * (size_t)st->n_maps, st->ChiY, sizeof(double) * Nc4);
            if (s->forward_map) {
                memcpy(st->stackX_f + Nc4 * (size_t)st->n_maps, st->ChiX_f, sizeof(double) * Nc4);
                memcpy(st->stackY_f + Nc4 * (size_t)st->n_maps, st->ChiY_f, sizeof(double) * Nc4);
                og_init_diffeo(st->ChiX_f, st->ChiY_f, &st->gc);
            }
            st->n_maps++;
            og_init_diffeo(st->ChiX, st->ChiY, &st->gc);
            *remapped = 1;
        }
    }
    long Np4 = 4 * st->gp.N;
    for (int i_l = 1; i_l < Lo; i_l++)
        memcpy(st->psi + Np4 * (Lo - i_l), st->psi + Np4 * (Lo - i_l - 1), sizeof(double) * Np4);
    if (evaluate_stream(st)) return 2;
    coarse_vort(st);
    /* particles_advect: cmm-particles.cu:63-87 */
    double Lp12[4] = {0, 0, 0, 0};
    for (int i = 0; i < Lo; ++i)
        Lp12[i] = og_get_L_coefficient(st->t_vec, st->t_vec[lcl] + st->dt_vec[lcl + 1] / 2.0, lcl + 1, i, Lo);
    for (int i_p = 0; i_p < s->n_particle_sets; ++i_p) {
        og_particle_set* ps = &s->psets[i_p];
        if (!(st->t_vec[lcl + 1] + 1e-5 * st->dt_vec[lcl + 1] >= ps->init_time)) continue;
        if (ps->tau == 0)
            og_particle_advect(ps->num, st->dt_vec[lcl + 1], st->parts[i_p], st->psi, &st->gp,
                               ps->time_integration_num, Lo, Lp12);
        else
            og_particle_advect_inertia(ps->num, st->dt_vec[lcl + 1], st->parts[i_p], st->vels[i_p], st->psi,
                                       &st->gp, ps->tau, ps->time_integration_num, Lo, Lp12);
    }
    /* a set whose start time was crossed in this step restarts its inertial velocity
     * (cmm-euler2d.cu:883-895) */
    for (int i_p = 0; i_p < s->n_particle_sets; ++i_p) {
        og_particle_set* ps = &s->psets[i_p];
        if (ps->tau == 0) continue;
        if (st->t_vec[lcl] - ps->init_time + s->dt * 1e-5 < 0 && st->t_vec[lcl + 1] - ps->init_time + s->dt * 1e-5 > 0) {
            if (ps->init_vel) og_particle_inertia_init(ps->num, st->parts[i_p], st->vels[i_p], st->psi, &st->gp);
            else memset(st->vels[i_p], 0, sizeof(double) * 2 * (size_t)ps->num);
        }
    }
    st->loop_ctr++;
    return saturated;
}

double og_time(const og_state* st) { return st->t_vec[st->loop_ctr + st->s.lagrange_order - 1]; }
int og_map_count(const og_state* st) { return st->n_maps; }
int og_loop_ctr(const og_state* st) { return st->loop_ctr; }
int og_old_ctr(const og_state* st) { return st->old_ctr; }
const double* og_chix(const og_state* st) { return st->ChiX; }
const double* og_chiy(const og_state* st) { return st->ChiY; }
const double* og_psi(const og_state* st) { return st->psi; }
const double* og_vort_coarse(const og_state* st) { return st->vort; }
const double* og_vort_fine(const og_state* st) { return st->vort_fine; }
const double* og_particles(const og_state* st, int i) { return st->parts[i]; }
double* og_particle_vel(og_state* st, int i) { return st->vels[i]; }
const og_grid* og_grid_of(const og_state* st, int which)
{
    switch (which) { case 0: return &st->gc; case 1: return &st->gf; case 2: return &st->gp; default: return &st->gv; }
}

/* ------------------------------------------------------------------ */
/* diagnostics: src/numerical/cmm-mesure.cu                            */
/* ------------------------------------------------------------------ */
double og_energy_H(const og_state* st)
{
    /* Compute_Energy_H: cmm-mesure.cu:30-35, planes 1 and 2 of ψ level 0 */
    const og_grid* g = &st->gp; double s = 0;
    #pragma omp parallel for reduction(+:s) schedule(static)
    for (long i = g->N; i < 3 * g->N; ++i) s += st->psi[i] * st->psi[i];
    return 0.5 * g->hx * g->hy * s;
}
double og_enstrophy(const og_state* st)
{
    /* Compute_Enstrophy: cmm-mesure.cu:52-57 */
    const og_grid* g = &st->gc; double s = 0;
    #pragma omp parallel for reduction(+:s) schedule(static)
    for (long i = 0; i < g->N; ++i) s += st->vort[i] * st->vort[i];
    return 0.5 * g->hx * g->hy * s;
}
double og_palinstrophy(const og_state* st)
{
    /* Compute_Palinstrophy: cmm-mesure.cu:77-89 via grad_x / grad_y (cmm-fft.cu:462-474) */
    const og_grid* g = &st->gc; double pal = 0;
    double* c = (double*)xmalloc(sizeof(double) * 2 * g->Nfft);
    double* c2 = (double*)xmalloc(sizeof(double) * 2 * g->Nfft);
    double* r = (double*)xmalloc(sizeof(double) * g->N);
    for (int dir = 0; dir < 2; ++dir) {
        og_fft_d2z(g, st->vort, c);
        og_normalize_h(c, g);
        if (dir == 0) og_fft_dx_h(c, c2, g); else og_fft_dy_h(c, c2, g);
        og_fft_z2d(g, c2, r);
        double s = 0;
        for (long i = 0; i < g->N; ++i) s += r[i] * r[i];
        pal += 0.5 * g->hx * g->hy * s;
    }
    free(c); free(c2); free(r);
    return pal;
}
double og_max_vorticity(const og_state* st)
{
    /* cmm-simulation-host.cu:668-673: thrust reduce with init 0 */
    const og_grid* g = &st->gc; double mx = 0.0, mn = 0.0;
    for (long i = 0; i < g->N; ++i) { if (st->vort[i] > mx) mx = st->vort[i]; if (st->vort[i] < mn) mn = st->vort[i]; }
    return mx > -mn ? mx : -mn;
}

void og_stats_grid(const double* v, const og_grid* g, double* out)
{
    /* Compute_min/max/avg/L2 grid form: cmm-mesure.cu:217-232 */
    double mn = v[0], mx = v[0], s = 0;
    for (long i = 0; i < g->N; ++i) { if (v[i] < mn) mn = v[i]; if (v[i] > mx) mx = v[i]; s += v[i]; }
    double mx0 = 0.0; for (long i = 0; i < g->N; ++i) if (v[i] > mx0) mx0 = v[i];
    out[0] = mn; out[1] = mx; out[2] = g->hy * g->hx * mx0; out[3] = g->hy * g->hx * s;
}
void og_stats_raw(const double* v, long n, double* out)
{
    /* raw-array form: cmm-mesure.cu:234-249 */
    double mn = v[0], mx = v[0], s = 0, mx0 = 0.0;
    for (long i = 0; i < n; ++i) { if (v[i] < mn) mn = v[i]; if (v[i] > mx) mx = v[i]; s += v[i]; if (v[i] > mx0) mx0 = v[i]; }
    out[0] = mn; out[1] = mx; out[2] = mx0 / (double)n; out[3] = s / (double)n;
}

void og_sample_points_dxdy(const og_state* st, const double* pos, double* out, int num)
{
    const og_grid* g = &st->gp;
    for (int i = 0; i < num; ++i) {
        double x = pos[2 * i], y = pos[2 * i + 1];
        if (x > g->bounds[0] && x < g->bounds[1] && y > g->bounds[2] && y < g->bounds[3]) {
            out[2 * i] = og_hermite_interpolate_dx_2D(st->psi, x, y, g);
            out[2 * i + 1] = og_hermite_interpolate_dy_2D(st->psi, x, y, g);
        } else out[2 * i] = out[2 * i + 1] = NAN;
    }
}

void og_vlasov_state_mesure(const og_state* st, double* out)
{
    og_vlasov_mesure(st->vort, &st->gc, st->psi, &st->gp, out);
}

static og_state_view state_view(const og_state* st)
{
    og_state_view v;
    v.gc = &st->gc;
    v.ChiX = st->ChiX; v.ChiY = st->ChiY;
    v.stackX = st->stackX; v.stackY = st->stackY;
    v.n_maps = st->n_maps;
    v.discrete = st->s.initial_discrete ? st->vort_disc : NULL;
    v.gd = &st->gd;
    v.ic_num = st->s.initial_condition_num;
    v.psi = st->psi;
    v.gp = &st->gp;
    return v;
}

void og_state_sample(const og_state* st, int n_sample, int scalar_num, double* out, double* mes)
{
    og_grid gs;
    og_grid_fill(&gs, n_sample, n_sample, st->gc.bounds);
    og_state_view v = state_view(st);
    og_sample_fields(&v, &gs, scalar_num, out, mes);
}

void og_state_vlasov_sample(const og_state* st, int n_sample, double* out, double* mes)
{
    og_grid gs;
    og_grid_fill(&gs, n_sample, n_sample, st->gc.bounds);
    og_state_view v = state_view(st);
    og_vlasov_sample_fields(&v, &gs, out, mes);
}

void og_state_zoom(const og_state* st, int n, const double* bounds4, int scalar_num, double* out)
{
    og_state_view v = state_view(st);
    og_zoom_fields(&v, n, bounds4, scalar_num, out);
}

/* ------------------------------------------------------------------ */
/* forward map outputs                                                 */

double og_invertibility_check(const og_grid* gc, const og_grid* gb, const double* Xb, const double* Yb,
                              const og_grid* gfw, const double* Xf, const double* Yf)
{
    double m = 0.0;
    #pragma omp parallel for reduction(max : m) schedule(static)
    for (long In = 0; In < gc->N; ++In) {
        long iX = In % gc->NX, iY = In / gc->NX;
        double x = gc->bounds[0] + iX * gc->hx + 0.5 * gc->hx, y = gc->bounds[2] + iY * gc->hy + 0.5 * gc->hy;
        double a, b;
        og_diffeo_interpolate_2D(Xf, Yf, x, y, &a, &b, gfw);
        og_diffeo_interpolate_2D(Xb, Yb, a, b, &a, &b, gb);
        double d = hypot(x - a, y - b);
        if (d > m) m = d;
    }
    return m;
}

const double* og_chix_f(const og_state* st) { return st->ChiX_f; }
const double* og_chiy_f(const og_state* st) { return st->ChiY_f; }
void og_forward_monitors(const og_state* st, double* einc_f, double* einv) { *einc_f = st->einc_f; *einv = st->einv; }

int og_set_forwarded_particles(og_state* st, int i, const double* pos)
{
    if (!st->s.forward_map || i < 0 || i >= st->s.n_fwd_sets) return -1;
    memcpy(st->fparts[i], pos, sizeof(double) * 2 * (size_t)st->s.fsets[i].num);
    return 0;
}

/* k_h_sample_points_map (cmm-simulation-kernel.cu:97-118): a point strictly inside the frame
 * goes through the map and is wrapped to the domain; any other point becomes NaN */
static void map_points(const double* X, const double* Y, const og_grid* gm, const og_grid* frame, const double* in,
                       double* out, int num)
{
    double LX = gm->bounds[1] - gm->bounds[0], LY = gm->bounds[3] - gm->bounds[2];
    for (int i = 0; i < num; ++i) {
        double x = in[2 * i], y = in[2 * i + 1];
        if (x > frame->bounds[0] && x < frame->bounds[1] && y > frame->bounds[2] && y < frame->bounds[3]) {
            double a, b;
            og_diffeo_interpolate_2D(X, Y, x, y, &a, &b, gm);
            out[2 * i] = a - floor(a / LX) * LX;
            out[2 * i + 1] = b - floor(b / LY) * LY;
        } else {
            out[2 * i] = out[2 * i + 1] = NAN;
        }
    }
}

void og_forward_sample(const og_state* st, int n, const double* bounds4, double* map_xy, double* parts)
{
    og_grid gz;
    og_grid_fill(&gz, n, n, bounds4);
    const og_grid* gm = &st->gc;
    const og_settings* s = &st->s;
    long Nc4 = 4 * gm->N;
    int nm = st->n_maps;
    /* the frame's nodes: forward stack oldest first, then the active forward map */
    if (nm > 0) {
        og_sample_map_compact(st->stackX_f, st->stackY_f, map_xy, gm, &gz);
        for (int i = 1; i < nm; ++i) og_apply_map_compact(st->stackX_f + Nc4 * i, st->stackY_f + Nc4 * i, map_xy, gm, &gz);
        og_apply_map_compact(st->ChiX_f, st->ChiY_f, map_xy, gm, &gz);
    } else {
        og_sample_map_compact(st->ChiX_f, st->ChiY_f, map_xy, gm, &gz);
    }
    if (!parts) return;
    /* forwarded particles, each set from its start map on (apply_map_stack_points, direction 1) */
    double* p = parts;
    for (int i_p = 0; i_p < s->n_fwd_sets; ++i_p) {
        int num = s->fsets[i_p].num, im = st->init_map[i_p];
        double t0 = s->fsets[i_p].init_time;
        const double* in = st->fparts[i_p];
        if (nm > 0) {
            if (t0 == 0) map_points(st->stackX_f, st->stackY_f, gm, &gz, in, p, num);
            else memcpy(p, in, sizeof(double) * 2 * (size_t)num);
            for (int i = 1; i < nm; ++i)
                if ((i >= im && t0 != 0) || t0 == 0)
                    map_points(st->stackX_f + Nc4 * i, st->stackY_f + Nc4 * i, gm, &gz, p, p, num);
            if ((im != 0 && t0 != 0) || t0 == 0) map_points(st->ChiX_f, st->ChiY_f, gm, &gz, p, p, num);
        } else {
            map_points(st->ChiX_f, st->ChiY_f, gm, &gz, in, p, num);
        }
        p += 2 * (size_t)num;
    }
}
