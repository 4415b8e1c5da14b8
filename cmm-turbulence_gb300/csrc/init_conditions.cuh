// init_conditions.cuh -- analytic initial vorticity, passive-scalar and
// Vlasov distribution fields sampled by the remap-time composition kernels (header-only so every
// translation unit that composes maps can inline them).
#pragma once
#include "cmm_common.cuh"

namespace cmm {

// ---------------------------------------------------------------------------
// analytic initial conditions (d_init_vorticity / d_init_scalar,
// src/simulation/cmm-init.cu:30-241, 253-298)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double init_vorticity(double x, double y, int ic, const double* __restrict__ prm,
                                 const double* __restrict__ rnd)
{
    const double PI = kTwoPi / 2;
    switch (ic) {
        case 0: {  // 4_nodes
            x -= floor(x / kTwoPi) * kTwoPi;
            y -= floor(y / kTwoPi) * kTwoPi;
            return cos(x) + cos(y) + 0.6 * cos(2 * x) + 0.2 * cos(3 * x);
        }
        case 1: {  // quadropole
            double r = 0;
            for (int iy = -2; iy <= 2; iy++)
                for (int ix = -2; ix <= 2; ix++) {
                    double dx = x - PI / 2 + ix * 2 * PI, dy = y - PI / 2 + iy * 2 * PI;
                    double A = 0.6258473, s = 0.5;
                    double B = A / (s * s * s * s) * (dx * dy) * (dx * dx + dy * dy - 6 * s * s);
                    double D = (dx * dx + dy * dy) / (2 * s * s);
                    r += B * exp(-D);
                }
            return r;
        }
        case 2: {  // one_vortex
            double sig = kTwoPi * 0.125;
            return 1.0 / (kTwoPi * sig * sig) * exp(-((x - PI) * (x - PI) + (y - PI) * (y - PI)) / (2 * sig * sig));
        }
        case 3: case 4: {  // two_votices / three_vortices
            double r = 0, LX = PI / 2, LY = PI / (2.0 * sqrt(2.0));
            for (int iy = -1; iy <= 1; iy++)
                for (int ix = -1; ix <= 1; ix++) {
                    double xs = x + kTwoPi * ix, ys = y + kTwoPi * iy;
                    double env = sin(0.5 * xs) * sin(0.5 * xs) * sin(0.5 * (ys + kTwoPi * iy)) * sin(0.5 * (ys + kTwoPi * iy));
                    double e;
                    if (ic == 3)
                        e = exp(-((xs - PI) * (xs - PI) + (ys - 0.33 * kTwoPi) * (ys - 0.33 * kTwoPi)) * 5) +
                            exp(-((xs - PI) * (xs - PI) + (ys - 0.67 * kTwoPi) * (ys - 0.67 * kTwoPi)) * 5);
                    else
                        e = exp(-((xs - PI - LX) * (xs - PI - LX) + (ys - PI) * (ys - PI)) * 5) +
                            exp(-((xs - PI + LX) * (xs - PI + LX) + (ys - PI) * (ys - PI)) * 5) -
                            exp(-((xs - PI + LX) * (xs - PI + LX) + (ys - PI - LY) * (ys - PI - LY)) * 5);
                    r += env * e;
                }
            return r;
        }
        case 5:  // single_shear_layer
            return (1 + 0.01 * cos(2 * x)) * exp(-50.0 * (y - PI) * (y - PI));
        case 6: {  // tanh_shear_layer
            double freq = 2, d = 14 * freq / kTwoPi;
            double c = exp(-d * (y - PI)) + exp(d * (y - PI));
            return 5.0 * (1 + 0.01 * cos(freq * x)) * 4 / c / c;
        }
        case 7: {  // turbulence_gaussienne: 8 x 8 positive blobs on the corners, 7 x 7 negative ones
                   // between them, offset by the cuRAND table after the 1000 uniform values
            x -= floor(x / kTwoPi) * kTwoPi;
            y -= floor(y / kTwoPi) * kTwoPi;
            const int NB = 8;
            const double sig = 0.2, amp = 1 / (kTwoPi * sig * sig), den = 2 * sig * sig;
            double r = 0;
            for (int mx = 0; mx < NB; mx++)
                for (int my = 0; my < NB; my++) {
                    const double ex = x - mx * kTwoPi / (NB - 1), ey = y - my * kTwoPi / (NB - 1);
                    r += amp * exp(-(ex * ex / den + ey * ey / den));
                }
            const double* off = rnd + 1000;
            for (int mx = 0; mx < NB - 1; mx++)
                for (int my = 0; my < NB - 1; my++) {
                    const double ex = x - (2 * mx + 1) * kTwoPi / (2 * (NB - 1)) + off[mx * (NB - 1) + my];
                    const double ey = y - (2 * my + 1) * kTwoPi / (2 * (NB - 1)) + off[49 + mx * (NB - 1) + my];
                    r -= amp * exp(-(ex * ex / den + ey * ey / den));
                }
            return r - 0.008857380480028442;   // the reference's mean correction
        }
        case 8: {  // gaussian_blobs (random offsets from a host-drawn table)
            x -= floor(x / kTwoPi) * kTwoPi;
            y -= floor(y / kTwoPi) * kTwoPi;
            const int NB = 10, border = 2;
            double sig = kTwoPi * 0.01, off = kTwoPi * 0.005, r = 0;
            int dir = 1;
            for (int mx = -border; mx < 2 * NB + border; mx++) {
                for (int my = -border; my < 2 * NB + border; my++) {
                    int bn = (int)((mx - floor(mx / (double)(NB * 2)) * NB * 2) +
                                   (my - floor(my / (double)(NB * 2)) * NB * 2) * NB * 2);
                    double ex = x - (mx + 0.5) * kTwoPi / (2 * NB) + rnd[bn] * off;
                    double ey = y - (my + 0.5) * kTwoPi / (2 * NB) + rnd[bn + NB * NB * 4] * off;
                    r += dir / (kTwoPi * sig * sig) * exp(-(ex * ex + ey * ey) / (2 * sig * sig));
                    dir = -dir;
                }
                dir = -dir;
            }
            return r;
        }
        case 9: {  // shielded_vortex
            double nu = 2e-1, xr = PI - x, yr = PI - y;
            return 1 / (2 * nu * nu * nu) * (4 * nu - xr * xr - yr * yr) * exp(-(xr * xr + yr * yr) / (4 * nu));
        }
        case 10: {  // two_cosine
            x -= floor(x / kTwoPi) * kTwoPi;
            y -= floor(y / kTwoPi) * kTwoPi;
            return cos(x) * cos(y);
        }
        case 11: {  // vortex_sheets
            double d = 1 / sqrt(prm[0]);
            double q = y - PI - sin(x) / 2.0;
            return exp(-q * q / (2 * d * d)) / sqrt(2 * PI) / d;
        }
        default: return 0.0;
    }
}

__device__ __forceinline__ double init_scalar(double x, double y, int sn)
{
    const double PI = kTwoPi / 2;
    switch (sn) {
        case 0: {  // rectangle
            x -= floor(x / kTwoPi) * kTwoPi;
            y -= floor(y / kTwoPi) * kTwoPi;
            return (x > PI - PI && x < PI + PI && y > PI / 2.0 - PI / 2.0 && y < PI / 2.0 + PI / 2.0) ? 1.0 : 0.0;
        }
        case 1: {  // gaussian
            double v = PI / 4.0;
            return 1.0 / (kTwoPi * v * v) * exp(-((x - PI) * (x - PI) / (2 * v * v) + (y - PI) * (y - PI) / (2 * v * v)));
        }
        case 2: {  // circular_ring
            double r = PI / 2.0, w = r / 8.0, q = (x - PI) * (x - PI) + (y - PI) * (y - PI);
            return (tanh(10.0 * (q - (r + w) * (r + w))) - tanh(10.0 * (q - (r - w) * (r - w)))) / 2.0;
        }
        default: return 0.0;
    }
}

// initial distribution function of the Vlasov-Poisson system
// (d_init_distirbution_function, src/simulation/cmm-init.cu:457-493): x is
// the periodic space coordinate, v the velocity
__device__ __forceinline__ double init_distribution(double x, double v, int ic)
{
    const double PI = kTwoPi / 2;
    switch (ic) {
        case 0: {  // landau_damping
            const double k = 0.5, eps = 5 * 1e-2;
            return (1 + eps * cos(k * x)) * exp(-(v) * (v) * 0.5) / sqrt(2 * PI);
        }
        case 1: {  // two_stream
            const double v0 = 3, k = 0.2, eps = 5 * 1e-2;
            return 1 / (2 * sqrt(2 * PI)) * (1 + eps * cos(k * x)) *
                   (exp(-(v - v0) * (v - v0) * 0.5) + exp(-(v + v0) * (v + v0) * 0.5));
        }
        case 2: {  // nonlin_landau_damping
            const double k = 0.5, eps = 0.5;
            return (1 + eps * cos(k * x)) * exp(-(v) * (v) * 0.5) / sqrt(2 * PI);
        }
        default: return 0.0;
    }
}

// value of an initial field at (x, y) by source kind (0 vorticity, 1 passive
// scalar, 2 distribution function; kind 3, a discrete field, is interpolated
// by the caller)
__device__ __forceinline__ double init_field(int kind, double x, double y, int ic, const double* __restrict__ prm,
                                             const double* __restrict__ rnd)
{
    if (kind == 1) return init_scalar(x, y, ic);
    if (kind == 2) return init_distribution(x, y, ic);
    return init_vorticity(x, y, ic, prm, rnd);
}

}  // namespace cmm
