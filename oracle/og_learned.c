/* og_learned.c -- CPU oracle of the learned psi upsampler (TEST INFRASTRUCTURE ONLY).
 *
 * The reference has no learned part; this file is the FP64 statement of the network the
 * product trains (periodic 3x3 convolutions, residual blocks, sub-pixel output, mean
 * squared error) and of its gradients, used to check the product's tensor-core forward,
 * input-gradient and weight-gradient kernels.  With emulate_bf16 != 0 every tensor the
 * product stores in BF16 (weights, network input, activations, output gradient and the
 * propagated gradients) is rounded to BF16 at the same point, so the remaining difference
 * is the product's FP32 accumulation order; with emulate_bf16 == 0 the whole computation is
 * FP64 (the tests check those gradients against finite differences).
 *
 * Layouts (as the product): activations [rows = B*H][W][C]; W[tap][cin][cout] with
 * tap = 3 dy + dx for offsets (dy - 1, dx - 1); parameters layer by layer (W then b):
 * head 16 -> C (input channels 7..15 zero; inputs psi, psi_x, psi_y, psi_xy, omega,
 * omega_x, omega_y), per block two C -> C, tail C -> 16 (output
 * channels 0..3 = sub-pixels (0,0), (0,1), (1,0), (1,1) of the 2x finer grid).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "cmm_oracle.h"

double og_bf16_round(double v)
{
    float f = (float)v;
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) {
        u += 0x7fffu + ((u >> 16) & 1u); /* round to nearest, ties to even */
    }
    u &= 0xffff0000u;
    memcpy(&f, &u, 4);
    return (double)f;
}

static int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

void og_conv3x3(const double* x, int B, int H, int W, int cin, const double* w, const double* bias, int cout,
                const double* mask, const double* res, int relu, double* out)
{
    const long rows = (long)B * H;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; ++r) {
        const int img = (int)(r / H), y = (int)(r % H);
        double acc[64];
        for (int xx = 0; xx < W; ++xx) {
            for (int co = 0; co < cout; ++co) acc[co] = bias ? bias[co] : 0.0;
            for (int dy = 0; dy < 3; ++dy) {
                const long rr = (long)img * H + wrapi(y + dy - 1, H);
                for (int dx = 0; dx < 3; ++dx) {
                    const double* xp = x + (rr * W + wrapi(xx + dx - 1, W)) * cin;
                    const double* wp = w + (long)(dy * 3 + dx) * cin * cout;
                    for (int ci = 0; ci < cin; ++ci) {
                        const double v = xp[ci];
                        if (v == 0.0) continue;
                        for (int co = 0; co < cout; ++co) acc[co] += v * wp[ci * cout + co];
                    }
                }
            }
            const long p = r * W + xx;
            for (int co = 0; co < cout; ++co) {
                double v = acc[co];
                if (relu && v < 0) v = 0;
                if (mask && !(mask[p * cout + co] > 0)) v = 0;
                if (res) v += res[p * cout + co];
                out[p * cout + co] = v;
            }
        }
    }
}

/* input gradient: dx[p][ci] = sum_tap sum_co dy[p - offset(tap)][co] w[tap][ci][co],
 * then * (mask > 0) and + res (both cin channels) */
void og_conv3x3_t(const double* dy, int B, int H, int W, int cin, const double* w, int cout, const double* mask,
                  const double* res, double* dx)
{
    const long rows = (long)B * H;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; ++r) {
        const int img = (int)(r / H), y = (int)(r % H);
        double acc[64];
        for (int xx = 0; xx < W; ++xx) {
            for (int ci = 0; ci < cin; ++ci) acc[ci] = 0.0;
            for (int ty = 0; ty < 3; ++ty) {
                const long rr = (long)img * H + wrapi(y - (ty - 1), H);
                for (int tx = 0; tx < 3; ++tx) {
                    const double* gp = dy + (rr * W + wrapi(xx - (tx - 1), W)) * cout;
                    const double* wp = w + (long)(ty * 3 + tx) * cin * cout;
                    for (int ci = 0; ci < cin; ++ci) {
                        double s = 0;
                        for (int co = 0; co < cout; ++co) s += gp[co] * wp[ci * cout + co];
                        acc[ci] += s;
                    }
                }
            }
            const long p = r * W + xx;
            for (int ci = 0; ci < cin; ++ci) {
                double v = acc[ci];
                if (mask && !(mask[p * cin + ci] > 0)) v = 0;
                if (res) v += res[p * cin + ci];
                dx[p * cin + ci] = v;
            }
        }
    }
}

void og_conv3x3_dw(const double* x, const double* dy, int B, int H, int W, int cin, int cout, double* dw, double* db)
{
    const long rows = (long)B * H;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < 9 * cin; ++k) {
        const int tap = k / cin, ci = k % cin, ty = tap / 3, tx = tap % 3;
        double acc[64];
        for (int co = 0; co < cout; ++co) acc[co] = 0.0;
        for (long r = 0; r < rows; ++r) {
            const int img = (int)(r / H), y = (int)(r % H);
            const long rr = (long)img * H + wrapi(y + ty - 1, H);
            for (int xx = 0; xx < W; ++xx) {
                const double v = x[(rr * W + wrapi(xx + tx - 1, W)) * cin + ci];
                if (v == 0.0) continue;
                const double* gp = dy + (r * W + xx) * cout;
                for (int co = 0; co < cout; ++co) acc[co] += v * gp[co];
            }
        }
        for (int co = 0; co < cout; ++co) dw[((long)tap * cin + ci) * cout + co] = acc[co];
    }
    for (int co = 0; co < cout; ++co) {
        double s = 0;
        for (long p = 0; p < rows * W; ++p) s += dy[p * cout + co];
        db[co] = s;
    }
}

/* full 2D DFT of a real H x W field (unnormalised, exp(-i k x)) */
static void dft2(const double* in, int H, int W, double* re, double* im)
{
    double* tr = (double*)malloc(sizeof(double) * H * W);
    double* ti = (double*)malloc(sizeof(double) * H * W);
    const double tp = 6.283185307179586;
    for (int y = 0; y < H; ++y)
        for (int kx = 0; kx < W; ++kx) {
            double a = 0, b = 0;
            for (int x = 0; x < W; ++x) {
                const double ph = -tp * (double)((long)kx * x % W) / W;
                a += in[(long)y * W + x] * cos(ph);
                b += in[(long)y * W + x] * sin(ph);
            }
            tr[(long)y * W + kx] = a;
            ti[(long)y * W + kx] = b;
        }
    for (int ky = 0; ky < H; ++ky)
        for (int kx = 0; kx < W; ++kx) {
            double a = 0, b = 0;
            for (int y = 0; y < H; ++y) {
                const double ph = -tp * (double)((long)ky * y % H) / H;
                const double c = cos(ph), s = sin(ph);
                a += tr[(long)y * W + kx] * c - ti[(long)y * W + kx] * s;
                b += tr[(long)y * W + kx] * s + ti[(long)y * W + kx] * c;
            }
            re[(long)ky * W + kx] = a;
            im[(long)ky * W + kx] = b;
        }
    free(tr);
    free(ti);
}

/* real part of the unnormalised inverse DFT (exp(+i k x)) */
static void idft2_real(const double* re, const double* im, int H, int W, double* out)
{
    double* tr = (double*)malloc(sizeof(double) * H * W);
    double* ti = (double*)malloc(sizeof(double) * H * W);
    const double tp = 6.283185307179586;
    for (int y = 0; y < H; ++y)
        for (int kx = 0; kx < W; ++kx) {
            double a = 0, b = 0;
            for (int ky = 0; ky < H; ++ky) {
                const double ph = tp * (double)((long)ky * y % H) / H;
                const double c = cos(ph), s = sin(ph);
                a += re[(long)ky * W + kx] * c - im[(long)ky * W + kx] * s;
                b += re[(long)ky * W + kx] * s + im[(long)ky * W + kx] * c;
            }
            tr[(long)y * W + kx] = a;
            ti[(long)y * W + kx] = b;
        }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            double a = 0;
            for (int kx = 0; kx < W; ++kx) {
                const double ph = tp * (double)((long)kx * x % W) / W;
                a += tr[(long)y * W + kx] * cos(ph) - ti[(long)y * W + kx] * sin(ph);
            }
            out[(long)y * W + x] = a;
        }
    free(tr);
    free(ti);
}

static double spec_weight(int ky, int kx, int H, int W, int cut)
{
    const int a = 2 * kx >= W ? kx - W : kx, b = 2 * ky >= H ? ky - H : ky;
    const double k2 = (double)a * a + (double)b * b;
    return (k2 > 0 && k2 <= (double)cut * cut) ? 1.0 / (k2 * k2) : 0.0;
}

static void round_all(double* v, long n, int emu)
{
    if (!emu) return;
    for (long i = 0; i < n; ++i) v[i] = og_bf16_round(v[i]);
}

/* sum over pixels of dy^2 per output channel (the scale of a bias gradient's rounding noise) */
static void sq_cols(const double* dy, long n, int cout, double* out)
{
    if (!out) return;
    for (int co = 0; co < cout; ++co) {
        double s = 0;
        for (long p = 0; p < n; ++p) s += dy[p * cout + co] * dy[p * cout + co];
        out[co] = s;
    }
}

double og_upsampler_loss_grad(const double* params, int nb, int C, const double* s_in, double s_out,
                              const float* inputs, const float* targets, int B, int h, int w, int emu, int cut,
                              double* grad)
{
    return og_upsampler_loss_grad_sq(params, nb, C, s_in, s_out, inputs, targets, B, h, w, emu, cut, grad, NULL);
}

/* as og_upsampler_loss_grad; dy_sq (NULL or the size of params): at each layer's bias slots, the
 * sum over pixels of the squared output gradient of that channel */
double og_upsampler_loss_grad_sq(const double* params, int nb, int C, const double* s_in, double s_out,
                                 const float* inputs, const float* targets, int B, int h, int w, int emu, int cut,
                                 double* grad, double* dy_sq)
{
    const int n_layers = 2 * nb + 2;
    long woff[130], boff[130];
    int lin[130], lout[130];
    long off = 0;
    for (int l = 0; l < n_layers; ++l) {
        lin[l] = l == 0 ? 16 : C;
        lout[l] = l == n_layers - 1 ? 16 : C;
        woff[l] = off;
        off += 9L * lin[l] * lout[l];
        boff[l] = off;
        off += lout[l];
    }
    const long npar = off;
    double* wq = (double*)malloc(sizeof(double) * npar);
    memcpy(wq, params, sizeof(double) * npar);
    for (int l = 0; l < n_layers; ++l) round_all(wq + woff[l], 9L * lin[l] * lout[l], emu); /* biases stay FP32 */
    const long hw = (long)h * w, n = (long)B * hw;
    double* x0 = (double*)calloc((size_t)n * 16, sizeof(double));
    for (int b = 0; b < B; ++b)
        for (long p = 0; p < hw; ++p)
            for (int c = 0; c < 7; ++c) {
                const float v = inputs[((long)b * 7 + c) * hw + p];
                double q = emu ? (double)(v / (float)s_in[c]) : (double)v / s_in[c];
                x0[((long)b * hw + p) * 16 + c] = emu ? og_bf16_round(q) : q;
            }
    double** a = (double**)malloc(sizeof(double*) * (nb + 1));
    double** hb = (double**)malloc(sizeof(double*) * (nb > 0 ? nb : 1));
    for (int i = 0; i <= nb; ++i) a[i] = (double*)malloc(sizeof(double) * n * C);
    for (int i = 0; i < nb; ++i) hb[i] = (double*)malloc(sizeof(double) * n * C);
    double* out = (double*)malloc(sizeof(double) * n * 16);
    og_conv3x3(x0, B, h, w, 16, wq + woff[0], params + boff[0], C, NULL, NULL, 0, a[0]);
    round_all(a[0], n * C, emu);
    for (int i = 0; i < nb; ++i) {
        const int l1 = 1 + 2 * i, l2 = 2 + 2 * i;
        og_conv3x3(a[i], B, h, w, C, wq + woff[l1], params + boff[l1], C, NULL, NULL, 1, hb[i]);
        round_all(hb[i], n * C, emu);
        og_conv3x3(hb[i], B, h, w, C, wq + woff[l2], params + boff[l2], C, NULL, a[i], 0, a[i + 1]);
        round_all(a[i + 1], n * C, emu);
    }
    const int lt = n_layers - 1;
    og_conv3x3(a[nb], B, h, w, C, wq + woff[lt], params + boff[lt], 16, NULL, NULL, 0, out);
    if (emu)
        for (long i = 0; i < n * 16; ++i) out[i] = (double)(float)out[i];
    /* loss and its gradient */
    double* dout = (double*)calloc((size_t)n * 16, sizeof(double));
    const double inv_n = 1.0 / (4.0 * (double)n);
    const float inv_out_f = (float)(1.0 / s_out), inv_n_f = (float)inv_n;
    double loss = 0;
    for (int b = 0; b < B; ++b)
        for (long p = 0; p < hw; ++p) {
            const long y = p / w, x = p % w;
            for (int k = 0; k < 4; ++k) {
                const float tv = targets[(long)b * 4 * hw + (2 * y + k / 2) * 2L * w + 2 * x + k % 2];
                const long q = ((long)b * hw + p) * 16 + k;
                if (emu) {
                    const float d = (float)out[q] - tv * inv_out_f;
                    loss += (double)d * (double)d;
                    dout[q] = og_bf16_round((double)(2.f * d * inv_n_f));
                } else {
                    const double d = out[q] - (double)tv / s_out;
                    loss += d * d;
                    dout[q] = 2.0 * d * inv_n;
                }
            }
        }
    loss *= inv_n;
    if (cut > 0) {
        /* psi-space loss: the mean over samples of num_b / den_b over the full spectra of
         * r = pred - target and of the target on the 2h x 2w grid, w = 1/|k|^4 on
         * 0 < |k| <= cut; gradient 2 IDFT(w R_b) / (B den_b) */
        const int H2 = 2 * h, W2 = 2 * w;
        const long m2 = (long)H2 * W2;
        double *r = (double*)malloc(sizeof(double) * m2), *t = (double*)malloc(sizeof(double) * m2);
        double *rr = (double*)malloc(sizeof(double) * m2), *ri = (double*)malloc(sizeof(double) * m2);
        double *tr = (double*)malloc(sizeof(double) * m2), *ti = (double*)malloc(sizeof(double) * m2);
        double *g = (double*)malloc(sizeof(double) * m2);
        double* num = (double*)calloc((size_t)B, sizeof(double));
        double* den = (double*)calloc((size_t)B, sizeof(double));
        double** spec = (double**)malloc(sizeof(double*) * 2 * B);
        for (int b = 0; b < B; ++b) {
            for (long p = 0; p < hw; ++p) {
                const long y = p / w, x = p % w;
                for (int k = 0; k < 4; ++k) {
                    const long q = (2 * y + k / 2) * W2 + 2 * x + k % 2;
                    const float tv = targets[(long)b * 4 * hw + q];
                    const double tt = emu ? (double)(tv * inv_out_f) : (double)tv / s_out;
                    const double pv = out[((long)b * hw + p) * 16 + k];
                    r[q] = emu ? (double)((float)pv - (float)tt) : pv - tt;
                    t[q] = tt;
                }
            }
            dft2(r, H2, W2, rr, ri);
            dft2(t, H2, W2, tr, ti);
            spec[2 * b] = (double*)malloc(sizeof(double) * m2);
            spec[2 * b + 1] = (double*)malloc(sizeof(double) * m2);
            for (int ky = 0; ky < H2; ++ky)
                for (int kx = 0; kx < W2; ++kx) {
                    const long q = (long)ky * W2 + kx;
                    const double wk = spec_weight(ky, kx, H2, W2, cut);
                    num[b] += wk * (rr[q] * rr[q] + ri[q] * ri[q]);
                    den[b] += wk * (tr[q] * tr[q] + ti[q] * ti[q]);
                    spec[2 * b][q] = wk * rr[q];
                    spec[2 * b + 1][q] = wk * ri[q];
                }
        }
        for (int b = 0; b < B; ++b) {
            idft2_real(spec[2 * b], spec[2 * b + 1], H2, W2, g);
            for (long p = 0; p < hw; ++p) {
                const long y = p / w, x = p % w;
                for (int k = 0; k < 4; ++k) {
                    const double v = den[b] > 0 ? g[(2 * y + k / 2) * W2 + 2 * x + k % 2] * 2.0 / (B * den[b]) : 0.0;
                    dout[((long)b * hw + p) * 16 + k] = emu ? og_bf16_round(v) : v;
                }
            }
            free(spec[2 * b]);
            free(spec[2 * b + 1]);
        }
        free(spec);
        free(r); free(t); free(rr); free(ri); free(tr); free(ti); free(g);
        loss = 0;
        for (int b = 0; b < B; ++b) loss += den[b] > 0 ? num[b] / den[b] : 0.0;
        loss /= B;
        free(num);
        free(den);
    }
    /* backward */
    double* da = (double*)malloc(sizeof(double) * n * C);
    double* da2 = (double*)malloc(sizeof(double) * n * C);
    double* dh = (double*)malloc(sizeof(double) * n * C);
    og_conv3x3_dw(a[nb], dout, B, h, w, C, 16, grad + woff[lt], grad + boff[lt]);
    sq_cols(dout, n, 16, dy_sq ? dy_sq + boff[lt] : NULL);
    og_conv3x3_t(dout, B, h, w, C, wq + woff[lt], 16, NULL, NULL, da);
    round_all(da, n * C, emu);
    for (int i = nb - 1; i >= 0; --i) {
        const int l1 = 1 + 2 * i, l2 = 2 + 2 * i;
        og_conv3x3_dw(hb[i], da, B, h, w, C, C, grad + woff[l2], grad + boff[l2]);
        sq_cols(da, n, C, dy_sq ? dy_sq + boff[l2] : NULL);
        og_conv3x3_t(da, B, h, w, C, wq + woff[l2], C, hb[i], NULL, dh);
        round_all(dh, n * C, emu);
        og_conv3x3_dw(a[i], dh, B, h, w, C, C, grad + woff[l1], grad + boff[l1]);
        sq_cols(dh, n, C, dy_sq ? dy_sq + boff[l1] : NULL);
        og_conv3x3_t(dh, B, h, w, C, wq + woff[l1], C, NULL, da, da2);
        round_all(da2, n * C, emu);
        double* t = da;
        da = da2;
        da2 = t;
    }
    og_conv3x3_dw(x0, da, B, h, w, 16, C, grad + woff[0], grad + boff[0]);
    sq_cols(da, n, C, dy_sq ? dy_sq + boff[0] : NULL);
    for (int i = 0; i <= nb; ++i) free(a[i]);
    for (int i = 0; i < nb; ++i) free(hb[i]);
    free(a);
    free(hb);
    free(out);
    free(dout);
    free(da);
    free(da2);
    free(dh);
    free(x0);
    free(wq);
    return loss;
}
