// fft.cuh -- the library's own FFT engine (sm_103a): mixed-radix Stockham
// transforms in shared memory, executed by one thread block over a batch of
// transforms, and the device pieces of the real <-> half-spectrum transforms.
//
// The reference computes every transform of the psi solve and of the remap with
// cuFFT (D2Z / Z2D plans, Cuda-CMM/src/grid/cmm-grid2d.cu:123-131; called from
// src/simulation/cmm-simulation-host.cu:299-375 and src/numerical/cmm-fft.cu:398-429).
// Here they are hand-written so that the passes around them (sampling, spectral
// operators, Hermite node writes) can be fused into the same kernels.
//
// Conventions (those of cuFFT and of the CPU oracle):
//   forward   X[k] = sum_j x[j] exp(-2 pi i jk/n)      (unnormalised)
//   inverse   x[j] = sum_k X[k] exp(+2 pi i jk/n)      (unnormalised)
//   R2C of N reals keeps k = 0..N/2; C2R reads k = 0..N/2 and ignores the
//   imaginary parts of k = 0 and k = N/2 (the Hermitian extension of the half
//   spectrum with those two bins taken as real).
//
// Algorithm.  A length-n complex transform, n = R_1 R_2 ... R_m with radices
// 2, 3, 4, 5, 7, 8, 11, 13, runs m Stockham (self-sorting) passes.  Pass with
// radix R after a span p (product of the previous radices): butterfly
// i in [0, n/R), k = i mod p, inputs a_r = x[i + r n/R] twiddled by
// w^(r k n/(pR)) (w = exp(-2 pi i/n)), an R-point DFT, outputs
// y[(i - k) R + k + r p].  Every pass reads its inputs into registers, the
// block synchronises, and the outputs are written back in place (one buffer
// of n values per transform in shared memory).  Twiddles come from per-pass
// tables (RadixPlan::toff) laid out so that the butterflies of a warp read
// consecutive entries, computed on the host in extended precision and copied
// into shared memory once per block (the kernels are persistent: a block
// transforms group after group).
//
// Real transforms of even length N pack x into the complex length-N/2
// sequence z[m] = x[2m] + i x[2m+1]:
//   R2C  X[k] = 1/2 [(Z_k + conj Z_{n-k}) - i W^k (Z_k - conj Z_{n-k})],  W = exp(-2 pi i/N)
//   C2R  Z_k = (X_k + conj X_{n-k}) + i W^-k (X_k - conj X_{n-k}),  z = inverse(Z),
//        x[2m] = Re z_m, x[2m+1] = Im z_m.
// (the standard even/odd split of a real DFT).
#pragma once
#include <cuda_runtime.h>

namespace cmm {
namespace fft {

constexpr int kMaxPasses = 24;

// radices of one transform length, in pass order; for power-of-two lengths the log2 of
// n / R and of the span p before each pass (index arithmetic by shifts).  The twiddles of
// pass q sit at toff[q] of the plan's table: entry k (R - 1) + r - 1 holds w^(r k n/(pR))
// (w = exp(-2 pi i / n), k < p, 1 <= r < R), so a warp's butterflies read consecutive
// entries; a generic radix appends its R roots of unity.  tlen: the table's length.
struct RadixPlan {
    int n;                      // complex length
    int np;                     // number of passes
    unsigned char r[kMaxPasses];
    unsigned char lnr[kMaxPasses], lp[kMaxPasses];
    int toff[kMaxPasses];
    int tlen;
};

#ifdef __CUDACC__
template <typename T> struct Cx;
template <> struct Cx<float> { using V = float2; };
template <> struct Cx<double> { using V = double2; };

__device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }

template <typename V> __device__ __forceinline__ V cadd(const V& a, const V& b) { return mk(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(const V& a, const V& b) { return mk(a.x - b.x, a.y - b.y); }
template <typename V> __device__ __forceinline__ V cmul(const V& a, const V& b)
{
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename V> __device__ __forceinline__ V cconj(const V& a) { return mk(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <typename V> __device__ __forceinline__ V rot(const V& a, bool inv) { return inv ? mk(-a.y, a.x) : mk(a.y, -a.x); }

// shared-memory padding: one spare slot every 32 (8-byte) or 8 (16-byte) values
// keeps the strided butterfly writes of the first passes off a single bank
template <typename V> __device__ __forceinline__ int pad(int i);
template <> __device__ __forceinline__ int pad<float2>(int i) { return i + (i >> 5); }
template <> __device__ __forceinline__ int pad<double2>(int i) { return i + (i >> 3); }
template <typename V> __host__ __device__ constexpr int padded_len(int n) { return sizeof(V) == 8 ? n + (n >> 5) + 1 : n + (n >> 3) + 1; }

// ---------------------------------------------------------------- R-point DFTs (in registers)
template <typename V> __device__ __forceinline__ void dft2(V* a)
{
    V t = a[1];
    a[1] = csub(a[0], t);
    a[0] = cadd(a[0], t);
}

template <typename V> __device__ __forceinline__ void dft4(V* a, bool inv)
{
    V s0 = cadd(a[0], a[2]), d0 = csub(a[0], a[2]);
    V s1 = cadd(a[1], a[3]), d1 = rot(csub(a[1], a[3]), inv);
    a[0] = cadd(s0, s1);
    a[2] = csub(s0, s1);
    a[1] = cadd(d0, d1);
    a[3] = csub(d0, d1);
}

template <typename V> __device__ __forceinline__ void dft8(V* a, bool inv)
{
    using T = decltype(a[0].x);
    const T h = (T)0.70710678118654752440084436210484903928;
    V e[4] = {a[0], a[2], a[4], a[6]}, o[4] = {a[1], a[3], a[5], a[7]};
    dft4(e, inv);
    dft4(o, inv);
    // o[k] *= exp(-+ 2 pi i k / 8)
    V o1 = o[1], o3 = o[3];
    if (!inv) {
        o[1] = mk(h * (o1.x + o1.y), h * (o1.y - o1.x));
        o[3] = mk(h * (o3.y - o3.x), -h * (o3.x + o3.y));
    } else {
        o[1] = mk(h * (o1.x - o1.y), h * (o1.x + o1.y));
        o[3] = mk(-h * (o3.x + o3.y), h * (o3.x - o3.y));
    }
    o[2] = rot(o[2], inv);
    for (int k = 0; k < 4; ++k) {
        a[k] = cadd(e[k], o[k]);
        a[k + 4] = csub(e[k], o[k]);
    }
}

template <typename V> __device__ __forceinline__ void dft3(V* a, bool inv)
{
    using T = decltype(a[0].x);
    const T c = (T)-0.5, s = inv ? (T)0.86602540378443864676372317075293618347 : (T)-0.86602540378443864676372317075293618347;
    V t1 = cadd(a[1], a[2]), t2 = csub(a[1], a[2]);
    V m1 = mk(a[0].x + c * t1.x, a[0].y + c * t1.y);
    V m2 = mk(-s * t2.y, s * t2.x);   // i s t2
    a[0] = cadd(a[0], t1);
    a[1] = cadd(m1, m2);
    a[2] = csub(m1, m2);
}

// any small R: direct DFT with the R roots of unity of the pass table
template <int R, typename V>
__device__ __forceinline__ void dft_generic(V* a, bool inv, const V* roots)
{
    V out[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
        V s = a[0];
#pragma unroll
        for (int r = 1; r < R; ++r) {
            V w = roots[(q * r) % R];
            if (inv) w = cconj(w);
            s = cadd(s, cmul(a[r], w));
        }
        out[q] = s;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) a[q] = out[q];
}

// ---------------------------------------------------------------- one Stockham pass
// nb transforms of length n at s[pad(b n + i)]; VPT = values per thread the block was
// sized for (nb n <= VPT blockDim.x); POW2: n, R and p are powers of two (lnr = log2(n/R),
// lp = log2(p)); ptw: this pass's twiddles (shared memory, or global for the longest lengths)
template <int R, int VPT, bool POW2, typename V>
__device__ __forceinline__ void pass(V* s, int nb, int n, int p, int lnr, int lp, const V* ptw, bool inv)
{
    constexpr int B = (VPT + R - 1) / R;
    const int nR = n / R;
    const int total = nb * nR;
    V v[B][R];
    int dst[B];
#pragma unroll
    for (int j = 0; j < B; ++j) {
        const int t = threadIdx.x + j * blockDim.x;
        dst[j] = -1;
        if (t < total) {
            const int b = POW2 ? t >> lnr : t / nR;
            const int i = t - b * nR;
            const int k = POW2 ? i & ((1 << lp) - 1) : i % p;
            const int base = b * n;
#pragma unroll
            for (int r = 0; r < R; ++r) v[j][r] = s[pad<V>(base + i + r * nR)];
            if (k != 0) {
                const V* tk = ptw + k * (R - 1);
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    V w = tk[r - 1];
                    if (inv) w = cconj(w);
                    v[j][r] = cmul(v[j][r], w);
                }
            }
            if (R == 2) dft2(v[j]);
            else if (R == 4) dft4(v[j], inv);
            else if (R == 8) dft8(v[j], inv);
            else if (R == 3) dft3(v[j], inv);
            else dft_generic<R>(v[j], inv, ptw + p * (R - 1));
            dst[j] = base + (i - k) * R + k;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < B; ++j) {
        if (dst[j] >= 0) {
#pragma unroll
            for (int r = 0; r < R; ++r) s[pad<V>(dst[j] + r * p)] = v[j][r];
        }
    }
    __syncthreads();
}

// radix families: a kernel instantiated for a family carries only those radices' passes,
// so the common power-of-two (and 3 * 2^k) lengths run without the register pressure of
// the large generic radices
enum Family { kPow2 = 0, kPow2x3 = 1, kAny = 2 };

inline int family_of(const RadixPlan& P)
{
    int f = kPow2;
    for (int q = 0; q < P.np; ++q) {
        if (P.r[q] == 3 && f < kPow2x3) f = kPow2x3;
        if (P.r[q] > 4 && P.r[q] != 8) f = kAny;
    }
    return f;
}

// all passes of nb length-n transforms held in shared memory (in place); every thread
// of the block takes part.  tw: the plan's table (RadixPlan::toff).
template <int VPT, int FAM, typename V>
__device__ __forceinline__ void block_fft(V* s, int nb, const RadixPlan& P, const V* tw, bool inv)
{
    constexpr bool P2 = FAM == kPow2;
    int p = 1;
    for (int q = 0; q < P.np; ++q) {
        const int R = P.r[q], lnr = P.lnr[q], lp = P.lp[q];
        const V* ptw = tw + P.toff[q];
        if (R == 8) pass<8, VPT, P2>(s, nb, P.n, p, lnr, lp, ptw, inv);
        else if (R == 4) pass<4, VPT, P2>(s, nb, P.n, p, lnr, lp, ptw, inv);
        else if (R == 2) pass<2, VPT, P2>(s, nb, P.n, p, lnr, lp, ptw, inv);
        else if (FAM >= kPow2x3 && R == 3) pass<3, VPT, false>(s, nb, P.n, p, lnr, lp, ptw, inv);
        else if (FAM == kAny) {
            if (R == 5) pass<5, VPT, false>(s, nb, P.n, p, lnr, lp, ptw, inv);
            else if (R == 7) pass<7, VPT, false>(s, nb, P.n, p, lnr, lp, ptw, inv);
            else if (R == 11) pass<11, VPT, false>(s, nb, P.n, p, lnr, lp, ptw, inv);
            else pass<13, VPT, false>(s, nb, P.n, p, lnr, lp, ptw, inv);
        }
        p *= R;
    }
}

// ---------------------------------------------------------------- ping-pong passes
// The same Stockham pass from `in` to a second buffer `out`: no thread overwrites what
// another still has to read, so a pass needs one barrier (after its writes) instead of two,
// and each butterfly is stored as soon as it is computed (its values leave the registers).
// Results are identical to pass().
template <int R, int VPT, bool POW2, typename V>
__device__ __forceinline__ void pass_pp(const V* in, V* out, int nb, int n, int p, int lnr, int lp, const V* ptw,
                                        bool inv)
{
    constexpr int B = (VPT + R - 1) / R;
    const int nR = n / R;
    const int total = nb * nR;
#pragma unroll
    for (int j = 0; j < B; ++j) {
        const int t = threadIdx.x + j * blockDim.x;
        if (t < total) {
            const int b = POW2 ? t >> lnr : t / nR;
            const int i = t - b * nR;
            const int k = POW2 ? i & ((1 << lp) - 1) : i % p;
            const int base = b * n;
            V v[R];
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = in[pad<V>(base + i + r * nR)];
            if (k != 0) {
                const V* tk = ptw + k * (R - 1);
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    V w = tk[r - 1];
                    if (inv) w = cconj(w);
                    v[r] = cmul(v[r], w);
                }
            }
            if (R == 2) dft2(v);
            else if (R == 4) dft4(v, inv);
            else if (R == 8) dft8(v, inv);
            else if (R == 3) dft3(v, inv);
            else dft_generic<R>(v, inv, ptw + p * (R - 1));
            const int dst = base + (i - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) out[pad<V>(dst + r * p)] = v[r];
        }
    }
    __syncthreads();
}

// block_fft with a second buffer: the transforms start in `a`, `b` is scratch; returns the
// buffer that holds the results (a after an even number of passes, b after an odd one).
// The caller synchronises after filling `a`; the last pass ends with a barrier.
template <int VPT, int FAM, typename V>
__device__ __forceinline__ V* block_fft_pp(V* a, V* b, int nb, const RadixPlan& P, const V* tw, bool inv)
{
    constexpr bool P2 = FAM == kPow2;
    int p = 1;
    V* src = a;
    V* dst = b;
    for (int q = 0; q < P.np; ++q) {
        const int R = P.r[q], lnr = P.lnr[q], lp = P.lp[q];
        const V* ptw = tw + P.toff[q];
        if (R == 8) pass_pp<8, VPT, P2>(src, dst, nb, P.n, p, lnr, lp, ptw, inv);
        else if (R == 4) pass_pp<4, VPT, P2>(src, dst, nb, P.n, p, lnr, lp, ptw, inv);
        else if (R == 2) pass_pp<2, VPT, P2>(src, dst, nb, P.n, p, lnr, lp, ptw, inv);
        else if (FAM >= kPow2x3 && R == 3) pass_pp<3, VPT, false>(src, dst, nb, P.n, p, lnr, lp, ptw, inv);
        else if (FAM == kAny) {
            if (R == 5) pass_pp<5, VPT, false>(src, dst, nb, P.n, p, lnr, lp, ptw, inv);
            else if (R == 7) pass_pp<7, VPT, false>(src, dst, nb, P.n, p, lnr, lp, ptw, inv);
            else if (R == 11) pass_pp<11, VPT, false>(src, dst, nb, P.n, p, lnr, lp, ptw, inv);
            else pass_pp<13, VPT, false>(src, dst, nb, P.n, p, lnr, lp, ptw, inv);
        }
        p *= R;
        V* t = src;
        src = dst;
        dst = t;
    }
    return src;
}

// ---------------------------------------------------------------- compile-time plans
// The radix sequence, spans and table offsets of make_radix_plan for a length 2^a 3^b known
// at compile time (8s, then a 4, or 4 4 in place of a trailing 8 2, or a 2; then 3s).
namespace sp {
constexpr int radix(int n, int q)
{
    int rs[kMaxPasses] = {};
    int c = 0, m = n;
    while (m % 8 == 0) { rs[c++] = 8; m /= 8; }
    if (m % 4 == 0) { rs[c++] = 4; m /= 4; }
    if (m % 2 == 0) {
        if (c > 0 && rs[c - 1] == 8) { rs[c - 1] = 4; rs[c++] = 4; }
        else rs[c++] = 2;
        m /= 2;
    }
    while (m % 3 == 0) { rs[c++] = 3; m /= 3; }
    return q < c ? rs[q] : 1;
}
// n = 2^a 3^b >= 2
constexpr bool supported(int n)
{
    if (n < 2) return false;
    int m = n;
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    return m == 1;
}
constexpr int gcd(int a, int b) { return b == 0 ? a : gcd(b, a % b); }
constexpr int npass(int n) { int c = 0; while (radix(n, c) > 1) ++c; return c; }
constexpr int span(int n, int q) { int s = 1; for (int i = 0; i < q; ++i) s *= radix(n, i); return s; }
constexpr int toff(int n, int q) { int o = 0; for (int i = 0; i < q; ++i) o += span(n, i) * (radix(n, i) - 1); return o; }
constexpr int tlen(int n) { return toff(n, npass(n)); }
constexpr bool pow2(int n) { return n >= 2 && (n & (n - 1)) == 0; }
// true when (x + c) >> S = (x >> S) + (c >> S) for every first index x and offset c of the
// butterflies of pass q of length n (see padc), over enough transforms b to cycle b n mod 2^S
constexpr bool pad_linear(int n, int q, int S)
{
    const int R = radix(n, q), P = span(n, q), nR = n / R;
    const int nbt = (1 << S) / gcd(n, 1 << S) + 1;   // b n mod 2^S repeats with this period
    for (int t = 0; t < nbt * nR; ++t) {
        const int b = t / nR, i = t % nR, k = i % P;
        const int x0 = b * n + i, d0 = b * n + (i - k) * R + k;
        for (int r = 0; r < R; ++r) {
            if (((x0 + r * nR) >> S) != (x0 >> S) + ((r * nR) >> S)) return false;
            if (((d0 + r * P) >> S) != (d0 >> S) + ((r * P) >> S)) return false;
        }
    }
    return true;
}
// true when the runtime plan P has the passes, spans and table offsets of the compile-time
// plan of length n (the static kernels read P's tables with sp:: offsets)
inline bool matches(int n, const RadixPlan& P)
{
    if (P.n != n || P.np != npass(n) || P.tlen != tlen(n)) return false;
    for (int q = 0; q < P.np; ++q)
        if (P.r[q] != radix(n, q) || P.toff[q] != toff(n, q)) return false;
    return true;
}
}  // namespace sp

template <typename V> struct PadShift;
template <> struct PadShift<float2> { static constexpr int value = 5; };
template <> struct PadShift<double2> { static constexpr int value = 3; };

// Offsets inside a pass.  pad(x) = x + (x >> S) is not linear, but for the accesses of one
// butterfly of a power-of-two pass it is: a butterfly reads x0 + r n/R and writes
// d0 + r p (r < R), where x0 = b n + i (i < n/R) and d0 = b n + (i - k) R + k (k < p).  With
// L = 2^S: a stride (n/R or p) of at least L makes every offset a multiple of L; a smaller
// stride divides L, the offsets' low S bits are multiples of it, and the low S bits of x0
// (d0) leave room for them below L.  Either way no carry crosses bit S, (x0 + c) >> S =
// (x0 >> S) + (c >> S) and pad(x0 + c) = pad(x0) + padc(c): one address register per
// butterfly and an immediate per value.  sp::pad_linear checks this at compile time for each
// pass (it holds for every power-of-two pass); a pass where it fails (lengths with a factor
// 3) computes the padded index of each value.
template <typename V> __host__ __device__ constexpr int padc(int c) { return c + (c >> PadShift<V>::value); }

// The butterfly of pass Q of the length-N plan whose first input is x0 = b N + i (k = i mod
// p): reads the R inputs (from `in`, unpadded when UIN), twiddles, transforms; d0: the first
// output index.  LIN (sp::pad_linear): the padded offsets are immediates.  The k = 0
// twiddles (exactly 1) are applied like the others: values equal those of the plan-driven
// passes up to the sign of zeros.  GT: the table is in global memory (read through the L1
// cache), else in shared memory.
template <int N, int Q, bool INV, bool GT, bool UIN, typename V>
__device__ __forceinline__ void sbutterfly(const V* __restrict__ in, int t, const V* tw, V* v, int& d0)
{
    constexpr int R = sp::radix(N, Q), P = sp::span(N, Q), nR = N / R;
    constexpr bool LIN = sp::pad_linear(N, Q, PadShift<V>::value);
    const int b = t / nR, i = t % nR, k = i % P;
    const int x0 = b * N + i;
    d0 = b * N + (i - k) * R + k;
    if (UIN) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = in[x0 + r * nR];
    } else if (LIN) {
        const V* src = in + pad<V>(x0);
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[padc<V>(r * nR)];
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = in[pad<V>(x0 + r * nR)];
    }
    if (P > 1) {
        const V* tk = tw + sp::toff(N, Q) + k * (R - 1);
#pragma unroll
        for (int r = 1; r < R; ++r) {
            V w = GT ? __ldg(tk + r - 1) : tk[r - 1];
            if (INV) w = cconj(w);
            v[r] = cmul(v[r], w);
        }
    }
    if (R == 2) dft2(v);
    else if (R == 4) dft4(v, INV);
    else if (R == 8) dft8(v, INV);
    else dft3(v, INV);
}

// the R outputs of a butterfly from d0
template <int N, int Q, typename V>
__device__ __forceinline__ void sstore(V* __restrict__ out, int d0, const V* v)
{
    constexpr int R = sp::radix(N, Q), P = sp::span(N, Q);
    if (sp::pad_linear(N, Q, PadShift<V>::value)) {
        V* dst = out + pad<V>(d0);
#pragma unroll
        for (int r = 0; r < R; ++r) dst[padc<V>(r * P)] = v[r];
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r) out[pad<V>(d0 + r * P)] = v[r];
    }
}

// pass Q of the length-N plan from `in` to `out` (ping-pong, one barrier), nb transforms,
// VPT values per thread of the block (nb N <= VPT blockDim.x).  Every index is a constant
// shift, mask or division.  UIN: `in` holds the transforms unpadded (x at in[b n + i]): the
// first pass may read a buffer filled by 16-byte copies (its reads, consecutive i per warp,
// need no padding).
template <int N, int Q, int VPT, bool INV, bool GT, bool UIN = false, typename V>
__device__ __forceinline__ void spass(const V* __restrict__ in, V* __restrict__ out, int nb, const V* tw)
{
    constexpr int R = sp::radix(N, Q), nR = N / R, B = (VPT + R - 1) / R;
    static_assert(sp::supported(N), "static passes are for lengths 2^a 3^b");
    const int total = nb * nR;
#pragma unroll
    for (int j = 0; j < B; ++j) {
        const int t = threadIdx.x + j * blockDim.x;
        if (t < total) {
            V v[R];
            int d0;
            sbutterfly<N, Q, INV, GT, UIN>(in, t, tw, v, d0);
            sstore<N, Q>(out, d0, v);
        }
    }
    __syncthreads();
}

// every pass of nb length-N transforms (N = 2^a 3^b) between a and b (both of
// padded_len(nb N) values); returns the buffer holding the results.  UIN0: a holds the
// input unpadded.  The caller synchronises after filling a.
template <int N, int VPT, bool INV, bool GT, bool UIN0 = false, int Q = 0, typename V>
__device__ __forceinline__ V* block_fft_s(V* a, V* b, int nb, const V* tw)
{
    if constexpr (Q == sp::npass(N)) {
        return a;
    } else {
        spass<N, Q, VPT, INV, GT, UIN0 && Q == 0>(a, b, nb, tw);
        return block_fft_s<N, VPT, INV, GT, false, Q + 1>(b, a, nb, tw);
    }
}

// the twiddle table (len entries) into shared memory
template <typename V>
__device__ __forceinline__ void load_table(V* dst, const V* __restrict__ src, int len)
{
    for (int t = threadIdx.x; t < len; t += blockDim.x) dst[t] = __ldg(src + t);
}

// ---------------------------------------------------------------- real packing
// R2C output bin k (0 <= k <= n) of the real length-2n sequence whose packed transform
// Z (length n, padded at s + off) sits in shared memory; W^k = tw[k] (the row plan's
// table of W^k, k <= n, after its pass twiddles)
template <typename V>
__device__ __forceinline__ V r2c_bin(const V* s, int off, int n, int k, const V* tw)
{
    using T = decltype(s[0].x);
    const V zk = s[pad<V>(off + (k == n ? 0 : k))];
    const V zc = cconj(s[pad<V>(off + (k == 0 ? 0 : n - k))]);
    const V sum = cadd(zk, zc), dif = csub(zk, zc);
    const V w = tw[k];
    const V t = cmul(w, dif);            // W^k (Z_k - conj Z_{n-k})
    return mk((T)0.5 * (sum.x + t.y), (T)0.5 * (sum.y - t.x));   // 1/2 (sum - i t)
}

// C2R packed input Z_k (0 <= k < n) from the half-spectrum bins X_k and X_{n-k} (with
// the imaginary parts of X_0 and X_n already dropped); W^-k = conj(tw[k])
template <typename V>
__device__ __forceinline__ V c2r_pack(const V& xk, const V& xnk, int k, const V* tw)
{
    const V b = cconj(xnk);
    const V sum = cadd(xk, b), dif = csub(xk, b);
    const V t = cmul(cconj(tw[k]), dif);   // W^-k (X_k - conj X_{n-k})
    return mk(sum.x - t.y, sum.y + t.x);          // sum + i t
}
#endif  // __CUDACC__

}  // namespace fft
}  // namespace cmm
