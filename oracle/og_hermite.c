/*
 * og_hermite.c -- bicubic Hermite interpolation and backward/forward
 * characteristic integrators, restated on the CPU in FP64.
 *
 * TEST INFRASTRUCTURE ONLY (parity oracle; see cmm_oracle.h).
 *
 * Follows src/numerical/cmm-hermite.h:22-30 (basis), cmm-hermite.cu:30-45,
 * 67-86 (contraction order), :151-208 (index / wrap), :239-271 (1D weights),
 * :302-309 (tensor matrix), :323-503 (interpolants), and
 * src/numerical/cmm-timestep.cu:28-207,474-484 (integrators, Lagrange).
 */
#include "cmm_oracle.h"
#include <math.h>

/* cubic Hermite basis, "functions 3 and 4" of cmm-hermite.h:27-30 */
#define H_f3_3(x)  ((3 - 2*(x)) * (x)*(x))
#define H_f3x_3(x) ((6 - 6*(x)) * (x))
#define H_f4_3(x)  (((x) - 1) * (x)*(x))
#define H_f4x_3(x) ((3*(x) - 2) * (x))

void og_grid_fill(og_grid* g, int NX, int NY, const double* bounds)
{
    /* src/grid/cmm-grid2d.cu:58-82 (fill_grid) */
    g->NX = NX;
    g->NY = NY;
    g->NX_fft = (int)(NX / 2.0 + 1);
    g->hx = (bounds[1] - bounds[0]) / (float)NX;
    g->hy = (bounds[3] - bounds[2]) / (float)NY;
    for (int i = 0; i < 4; ++i) g->bounds[i] = bounds[i];
    g->N = (long)NX * NY;
    g->Nfft = (long)g->NX_fft * NY;
}

/* device_init_ind: cmm-hermite.cu:151-166 */
static void init_ind(int* I, double* dxy, double x, double y, const og_grid* g)
{
    int Ix0 = (int)floor((x - g->bounds[0]) / g->hx);
    int Iy0 = (int)floor((y - g->bounds[2]) / g->hy);
    int Ix1 = Ix0 + 1, Iy1 = Iy0 + 1;
    dxy[0] = (x - g->bounds[0]) / g->hx - Ix0;
    dxy[1] = (y - g->bounds[2]) / g->hy - Iy0;
    Ix0 -= (Ix0 / g->NX - (Ix0 < 0)) * g->NX; Iy0 -= (Iy0 / g->NY - (Iy0 < 0)) * g->NY;
    Ix1 -= (Ix1 / g->NX - (Ix1 < 0)) * g->NX; Iy1 -= (Iy1 / g->NY - (Iy1 < 0)) * g->NY;
    I[0] = Iy0 * g->NX + Ix0; I[1] = Iy0 * g->NX + Ix1;
    I[2] = Iy1 * g->NX + Ix0; I[3] = Iy1 * g->NX + Ix1;
}

/* device_init_ind_diff: cmm-hermite.cu:190-208 */
static void init_ind_diff(int* I, int* I_w, double* dxy, double x, double y, const og_grid* g)
{
    int Ix0 = (int)floor((x - g->bounds[0]) / g->hx);
    int Iy0 = (int)floor((y - g->bounds[2]) / g->hy);
    int Ix1 = Ix0 + 1, Iy1 = Iy0 + 1;
    dxy[0] = (x - g->bounds[0]) / g->hx - Ix0;
    dxy[1] = (y - g->bounds[2]) / g->hy - Iy0;
    I_w[0] = Ix0 / g->NX - (Ix0 < 0); I_w[1] = Iy0 / g->NY - (Iy0 < 0);
    I_w[2] = Ix1 / g->NX - (Ix1 < 0); I_w[3] = Iy1 / g->NY - (Iy1 < 0);
    Ix0 -= I_w[0] * g->NX; Iy0 -= I_w[1] * g->NY; Ix1 -= I_w[2] * g->NX; Iy1 -= I_w[3] * g->NY;
    I[0] = Iy0 * g->NX + Ix0; I[1] = Iy0 * g->NX + Ix1;
    I[2] = Iy1 * g->NX + Ix0; I[3] = Iy1 * g->NX + Ix1;
}

/* device_build_b / _bx / _by: cmm-hermite.cu:239-271 */
static void build_b(double* bX, double* bY, double dx, double dy)
{
    bX[0] = H_f3_3(1 - dx); bX[1] = H_f3_3(dx); bX[2] = -H_f4_3(1 - dx); bX[3] = H_f4_3(dx);
    bY[0] = H_f3_3(1 - dy); bY[1] = H_f3_3(dy); bY[2] = -H_f4_3(1 - dy); bY[3] = H_f4_3(dy);
}
static void build_bx(double* bX, double* bY, double dx, double dy)
{
    bX[0] = -H_f3x_3(1 - dx); bX[1] = H_f3x_3(dx); bX[2] = H_f4x_3(1 - dx); bX[3] = H_f4x_3(dx);
    bY[0] = H_f3_3(1 - dy);   bY[1] = H_f3_3(dy);  bY[2] = -H_f4_3(1 - dy); bY[3] = H_f4_3(dy);
}
static void build_by(double* bX, double* bY, double dx, double dy)
{
    bX[0] = H_f3_3(1 - dx);   bX[1] = H_f3_3(dx);  bX[2] = -H_f4_3(1 - dx); bX[3] = H_f4_3(dx);
    bY[0] = -H_f3x_3(1 - dy); bY[1] = H_f3x_3(dy); bY[2] = H_f4x_3(1 - dy); bY[3] = H_f4x_3(dy);
}
/* device_build_b_mat: cmm-hermite.cu:302-309 */
static void build_b_mat(double b[4][4], const double* bX, const double* bY)
{
    for (int i_x = 0; i_x < 4; ++i_x)
        for (int i_y = 0; i_y < 4; ++i_y) b[i_x][i_y] = bX[i_y] * bY[i_x];
}

/* device_hermite_mult_2D, matrix form: cmm-hermite.cu:30-45 */
static double mult_2D_mat(const double* H, double b[4][4], const int* I, long N, double hx, double hy)
{
    double h_out = 0.0;
    for (int i_ord = 0; i_ord < 4; ++i_ord) {
        double h_temp = 0.0;
        int ox = 2 * ((i_ord >> 1) & 1), oy = 2 * (i_ord & 1);
        for (int i_p = 0; i_p < 4; ++i_p)
            h_temp += b[((i_p >> 1) & 1) + ox][(i_p & 1) + oy] * H[i_ord * N + I[i_p]];
        if ((i_ord & 1) == 1) h_temp *= hx;
        if (((i_ord >> 1) & 1) == 1) h_temp *= hy;
        h_out += h_temp;
    }
    return h_out;
}
/* device_hermite_mult_2D, vector form: cmm-hermite.cu:113-128 */
static double mult_2D_vec(const double* H, const double* bX, const double* bY, const int* I,
                          long N, double hx, double hy)
{
    double h_out = 0.0;
    for (int i_ord = 0; i_ord < 4; ++i_ord) {
        double h_temp = 0.0;
        int ox = 2 * ((i_ord >> 1) & 1), oy = 2 * (i_ord & 1);
        for (int i_p = 0; i_p < 4; ++i_p)
            h_temp += bY[((i_p >> 1) & 1) + ox] * bX[(i_p & 1) + oy] * H[i_ord * N + I[i_p]];
        if ((i_ord & 1) == 1) h_temp *= hx;
        if (((i_ord >> 1) & 1) == 1) h_temp *= hy;
        h_out += h_temp;
    }
    return h_out;
}
/* device_hermite_mult_2D_warp: cmm-hermite.cu:66-86 */
static double mult_2D_warp(const double* H, double b[4][4], const int* I, const int* I_w, double L,
                           long N, double hx, double hy)
{
    double h_out = 0.0;
    for (int i_ord = 0; i_ord < 4; ++i_ord) {
        double h_temp = 0.0;
        int ox = 2 * ((i_ord >> 1) & 1), oy = 2 * (i_ord & 1);
        for (int i_p = 0; i_p < 4; ++i_p) {
            if (i_ord == 0)
                h_temp += b[((i_p >> 1) & 1) + ox][(i_p & 1) + oy] * (H[I[i_p]] + I_w[i_p] * L);
            else
                h_temp += b[((i_p >> 1) & 1) + ox][(i_p & 1) + oy] * H[i_ord * N + I[i_p]];
        }
        if ((i_ord & 1) == 1) h_temp *= hx;
        if (((i_ord >> 1) & 1) == 1) h_temp *= hy;
        h_out += h_temp;
    }
    return h_out;
}

/* cmm-hermite.cu:323-331 */
double og_hermite_interpolate_2D(const double* H, double x, double y, const og_grid* g)
{
    int I[4]; double dxy[2], bX[4], bY[4];
    init_ind(I, dxy, x, y, g);
    build_b(bX, bY, dxy[0], dxy[1]);
    return mult_2D_vec(H, bX, bY, I, g->N, g->hx, g->hy);
}
/* cmm-hermite.cu:343-351 */
double og_hermite_interpolate_dx_2D(const double* H, double x, double y, const og_grid* g)
{
    int I[4]; double dxy[2], bX[4], bY[4];
    init_ind(I, dxy, x, y, g);
    build_bx(bX, bY, dxy[0], dxy[1]);
    return mult_2D_vec(H, bX, bY, I, g->N, g->hx, g->hy) / g->hx;
}
/* cmm-hermite.cu:363-371 */
double og_hermite_interpolate_dy_2D(const double* H, double x, double y, const og_grid* g)
{
    int I[4]; double dxy[2], bX[4], bY[4];
    init_ind(I, dxy, x, y, g);
    build_by(bX, bY, dxy[0], dxy[1]);
    return mult_2D_vec(H, bX, bY, I, g->N, g->hx, g->hy) / g->hy;
}

/* device_hermite_interpolate_grad_2D: cmm-hermite.cu:396-420.
 * u[2l] = psi_y, u[2l+1] = -psi_x at level l; x and u may alias. */
void og_hermite_interpolate_grad_2D(const double* H, const double* x, double* u, const og_grid* g, int n_l)
{
    int I[4]; double dxy[2];
    init_ind(I, dxy, x[0], x[1], g);
    for (int i_xy = 0; i_xy <= 1; ++i_xy) {
        double bX[4], bY[4], b[4][4];
        if (i_xy == 0) build_bx(bX, bY, dxy[0], dxy[1]);
        else build_by(bX, bY, dxy[0], dxy[1]);
        build_b_mat(b, bX, bY);
        if (i_xy == 0) {
            for (int i_l = 0; i_l < n_l; i_l++)
                u[2 * i_l + 1] = -mult_2D_mat(H + 4 * g->N * i_l, b, I, g->N, g->hx, g->hy) / g->hx;
        } else {
            for (int i_l = 0; i_l < n_l; i_l++)
                u[2 * i_l] = mult_2D_mat(H + 4 * g->N * i_l, b, I, g->N, g->hx, g->hy) / g->hy;
        }
    }
}

/* device_diffeo_interpolate_2D: cmm-hermite.cu:446-460 */
void og_diffeo_interpolate_2D(const double* Hx, const double* Hy, double x, double y,
                              double* x2, double* y2, const og_grid* g)
{
    int I[4], I_w[4]; double dxy[2];
    init_ind_diff(I, I_w, dxy, x, y, g);
    double L0 = g->NX * g->hx, L1 = g->NY * g->hy;
    double bX[4], bY[4], b[4][4];
    build_b(bX, bY, dxy[0], dxy[1]);
    build_b_mat(b, bX, bY);
    int I_w_n[4] = {I_w[0], I_w[2], I_w[0], I_w[2]};
    double xo = mult_2D_warp(Hx, b, I, I_w_n, L0, g->N, g->hx, g->hy);
    I_w_n[0] = I_w[1]; I_w_n[1] = I_w[1]; I_w_n[2] = I_w[3]; I_w_n[3] = I_w[3];
    double yo = mult_2D_warp(Hy, b, I, I_w_n, L1, g->N, g->hx, g->hy);
    *x2 = xo; *y2 = yo;
}

/* device_diffeo_grad_2D: cmm-hermite.cu:479-503 */
double og_diffeo_grad_2D(const double* Hx, const double* Hy, double x, double y, const og_grid* g)
{
    int I[4], I_w[4]; double dxy[2];
    init_ind_diff(I, I_w, dxy, x, y, g);
    double L0 = g->NX * g->hx, L1 = g->NY * g->hy;
    double Xx = 0, Xy = 0, Yx = 0, Yy = 0;
    for (int i_xy = 0; i_xy <= 1; ++i_xy) {
        double bX[4], bY[4], b[4][4];
        if (i_xy == 0) build_bx(bX, bY, dxy[0], dxy[1]);
        else build_by(bX, bY, dxy[0], dxy[1]);
        build_b_mat(b, bX, bY);
        int I_w_n[4] = {I_w[0], I_w[2], I_w[0], I_w[2]};
        double x_der = mult_2D_warp(Hx, b, I, I_w_n, L0, g->N, g->hx, g->hy) / g->hx;
        I_w_n[0] = I_w[1]; I_w_n[1] = I_w[1]; I_w_n[2] = I_w[3]; I_w_n[3] = I_w[3];
        double y_der = mult_2D_warp(Hy, b, I, I_w_n, L1, g->N, g->hx, g->hy) / g->hy;
        if (i_xy == 0) { Xx = x_der; Yx = y_der; }
        else { Xy = x_der; Yy = y_der; }
    }
    return Xx * Yy - Xy * Yx;
}

/* get_L_coefficient: cmm-timestep.cu:474-484 */
double og_get_L_coefficient(const double* t, double t_next, int loop_ctr, int i_point, int l_order)
{
    double coeff = 1;
    for (int i_p = 0; i_p < l_order; ++i_p)
        if (i_p != i_point)
            coeff *= (t_next - t[loop_ctr - i_p]) / (t[loop_ctr - i_point] - t[loop_ctr - i_p]);
    return coeff;
}
