// psi_solve.cuh -- the psi solve of one time step on the library's FFT engine
// (fft.cuh), templated on the precision (FP64 plain form, FP32 mixed form).
//
// Reference: evaluate_stream_hermite (Cuda-CMM/src/simulation/cmm-simulation-host.cu:
// 333-375): omega sampled through the map on the vorticity grid
// (k_apply_map_and_sample_from_hermite), D2Z, k_normalize_h, k_fft_grid_move to the psi
// grid, k_fft_cut_off_scale_h, k_fft_iLap_h (src/numerical/cmm-fft.cu:55-78,267-339), and
// fourier_hermite (:398-429: the spectra of psi, d/dx, d/dy, d2/dxdy and four Z2D).
//
// Here the sampled vorticity (its own full-occupancy kernel) goes through three passes:
//   rows   (fft::rows_r2c)   the row R2C of every vorticity row, writing only the columns
//                            kx the cut-off and the psi grid keep;
//   cols   (k_psi_cols)      per (group of C kept columns, Hermite plane): the columns'
//                            forward transform over the vorticity grid, the spectral steps
//                            (normalise, grid move, circular cut-off, inverse Laplacian,
//                            the plane's derivative multiplier) and the inverse column
//                            transform over the psi grid;
//   inverse rows (k_psi_rows_inv)  per few psi rows: the row C2R of the four planes
//                            (missing columns are zero) and an epilogue that writes the
//                            Hermite nodes (and, in the mixed form, the Lagrange
//                            combinations of the next step).
// Between them only the kept columns travel through global memory: at the metric's
// sizes (vorticity 2048^2, psi 1024^2, cut-off 128) 2048 x 129 and 4 x 1024 x 129
// complex values instead of the full half spectra.  The kernels are persistent (a block
// copies its twiddle tables into shared memory once, then takes group after group) and
// sized for occupancy: FP32 8 values per thread within 64 registers.
#pragma once
#include <algorithm>
#include <cmath>

#include "cmm_common.cuh"
#include "fft.hpp"
#include "pdl.cuh"

namespace cmm {
namespace psi {

// block shapes: values per thread (VPT, a template argument of the kernels) and the launch
// bound (one block per SM at the bound gives 65536 / MAXT registers): FP32 4 values per
// thread (8 for the longest lengths) within 64 registers, FP64 8 values within 128 (an FP64
// radix-8 butterfly and its inputs)
template <typename T> struct Shape;
template <> struct Shape<float> { static constexpr int VPT = 4, VPT_LONG = 8, MAXT = 1024; };
template <> struct Shape<double> { static constexpr int VPT = 8, VPT_LONG = 8, MAXT = 512; };
constexpr int kBlockValues = 2048;   // values per group the launchers aim for

struct ColsArgs {
    const void* w1;          // vorticity-grid row spectra: NYv rows, columns 0..kv-1, row stride ld1
    void* w2;                // the four psi-grid spectra: 4 x NYp rows, columns 0..ncols-1, row stride ld2
    long long ld1, ld2;
    int kv, ncols;
    int C;                   // columns per group
    Grid gv, gp;
    double freq;
    fft::RadixPlan Pv, Pp;   // column lengths NYv, NYp
    const void* twv;         // the NYv column plan's pass twiddles
    const void* twp;         // the NYp column plan's pass twiddles
};

// psi spectrum of plane q (0: psi, 1: d/dx, 2: d/dy, 3: d2/dxdy) at psi-grid column iXc, row
// iYc from the forward-transformed vorticity column F (row iYs of the vort grid); the
// FP64 form restates k_spec_psi (reference operation order), the FP32 form k_spec_psi_f
template <typename V>
__device__ __forceinline__ V plane_mode(const V* s, int off, int q, int iXc, int iYc, const Grid& gv, const Grid& gp,
                                        double freq);

template <>
__device__ __forceinline__ double2 plane_mode<double2>(const double2* s, int off, int q, int iXc, int iYc,
                                                       const Grid& gv, const Grid& gp, double freq)
{
    double2 P = make_double2(0.0, 0.0);
    const bool hx = iXc > gp.NX / 2.0, hy = iYc > gp.NY / 2.0;
    const int fX = iXc + hx * (gp.NX - 2 * iXc), fY = iYc + hy * (gp.NY - 2 * iYc);
    if (!(fX > gv.NX / 2.0 || fY > gv.NY / 2.0)) {
        const int iYs = iYc + hy * (gv.NY - gp.NY);
        const double2 f = s[fft::pad<double2>(off + iYs)];
        P = make_double2(f.x / (double)gv.N, f.y / (double)gv.N);
    }
    if ((double)(fX * fX + fY * fY) > freq * freq || (iXc == 0 && iYc == 0)) P = make_double2(0.0, 0.0);
    const double kx = gp.kfx * (iXc - (iXc > gp.NX / 2) * gp.NX);
    const double ky = gp.kfy * (iYc - (iYc > gp.NY / 2) * gp.NY);
    if (iXc == 0 && iYc == 0) P = make_double2(0.0, 0.0);
    else {
        const double k2 = kx * kx + ky * ky;
        P = make_double2(-P.x / k2, -P.y / k2);
    }
    if (q == 0) return P;
    if (q == 1) return make_double2(-P.y * kx, P.x * kx);
    const double2 Py = make_double2(-P.y * ky, P.x * ky);
    return q == 2 ? Py : make_double2(-Py.y * kx, Py.x * kx);
}

// FP32 form with 1 / N_v and the cut-off already rounded to float, in two parts: the mode
// -F/(N_v k^2) of psi-grid column iXc, row iYc shared by the four planes (zero outside the
// vorticity grid's spectrum, beyond the cut-off and at k = 0, where no division is done) and
// the plane's derivative multiplier
__device__ __forceinline__ float2 plane_base_f(const float2* s, int off, int iXc, int iYc, const Grid& gv,
                                               const Grid& gp, float freq, float inv_nv, float& kx, float& ky)
{
    const bool hx = 2 * iXc > gp.NX, hy = 2 * iYc > gp.NY;
    const int fX = hx ? gp.NX - iXc : iXc, fY = hy ? gp.NY - iYc : iYc;
    kx = gp.kfxf * (float)(hx ? iXc - gp.NX : iXc);
    ky = gp.kfyf * (float)(hy ? iYc - gp.NY : iYc);
    if (2 * fX > gv.NX || 2 * fY > gv.NY || (float)(fX * fX + fY * fY) > freq * freq || (iXc == 0 && iYc == 0))
        return make_float2(0.f, 0.f);
    const int iYs = iYc + (hy ? gv.NY - gp.NY : 0);
    const float2 f = s[fft::pad<float2>(off + iYs)];
    const float ik2 = 1.0f / (kx * kx + ky * ky);
    return make_float2(-(f.x * inv_nv) * ik2, -(f.y * inv_nv) * ik2);
}

__device__ __forceinline__ float2 plane_mul_f(float2 P, int q, float kx, float ky)
{
    if (q == 0) return P;
    if (q == 1) return make_float2(-P.y * kx, P.x * kx);
    const float2 Py = make_float2(-P.y * ky, P.x * ky);
    return q == 2 ? Py : make_float2(-Py.y * kx, Py.x * kx);
}

__device__ __forceinline__ float2 plane_mode_f(const float2* s, int off, int q, int iXc, int iYc, const Grid& gv,
                                               const Grid& gp, float freq, float inv_nv)
{
    float kx, ky;
    const float2 P = plane_base_f(s, off, iXc, iYc, gv, gp, freq, inv_nv, kx, ky);
    return plane_mul_f(P, q, kx, ky);
}

template <>
__device__ __forceinline__ float2 plane_mode<float2>(const float2* s, int off, int q, int iXc, int iYc, const Grid& gv,
                                                     const Grid& gp, double freqd)
{
    return plane_mode_f(s, off, q, iXc, iYc, gv, gp, (float)freqd, (float)(1.0 / (double)gv.N));
}

// FP32: the transforms run through scratch buffers (fft::block_fft_pp, one barrier per pass)
template <typename T> struct UsePP { static constexpr bool value = sizeof(T) == 4; };

// groups (C kept columns, plane q) grid-strided; dynamic shared memory: padded(C NYv) +
// padded(C NYp) values (twice for FP32: the scratch buffers) + the two column plans' tables
template <typename T, int FAM, int VPT>
__global__ void __launch_bounds__(Shape<T>::MAXT, 1) k_psi_cols(ColsArgs a)
{
    using V = typename fft::Cx<T>::V;
    constexpr bool PP = UsePP<T>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nv = a.gv.NY, np = a.gp.NY, C = a.C;
    V* A = reinterpret_cast<V*>(smem_raw);
    V* B = A + fft::padded_len<V>(C * nv);
    V* A2 = B + fft::padded_len<V>(C * np);                 // scratch (PP)
    V* B2 = A2 + (PP ? fft::padded_len<V>(C * nv) : 0);
    V* tv = B2 + (PP ? fft::padded_len<V>(C * np) : 0);
    V* tp = tv + a.Pv.tlen;
    fft::load_table(tv, reinterpret_cast<const V*>(a.twv), a.Pv.tlen);
    fft::load_table(tp, reinterpret_cast<const V*>(a.twp), a.Pp.tlen);
    const V* w1 = reinterpret_cast<const V*>(a.w1);
    const int gx = (a.ncols + C - 1) / C;
    for (int grp = blockIdx.x; grp < 4 * gx; grp += gridDim.x) {
        const int q = grp / gx, col0 = (grp - q * gx) * C;
        __syncthreads();   // tables in place, the previous group's outputs read
        for (int e = threadIdx.x; e < C * nv; e += blockDim.x) {
            const int c = e % C, r = e / C, col = col0 + c;
            A[fft::pad<V>(c * nv + r)] = col < a.kv ? w1[r * a.ld1 + col] : fft::mk((T)0, (T)0);
        }
        __syncthreads();
        const V* FA = A;
        if (PP) FA = fft::block_fft_pp<VPT, FAM>(A, A2, C, a.Pv, tv, false);
        else fft::block_fft<VPT, FAM>(A, C, a.Pv, tv, false);
        for (int e = threadIdx.x; e < C * np; e += blockDim.x) {
            const int c = e / np, r = e - c * np;
            B[fft::pad<V>(e)] = plane_mode<V>(FA, c * nv, q, col0 + c, r, a.gv, a.gp, a.freq);
        }
        __syncthreads();
        const V* FB = B;
        if (PP) FB = fft::block_fft_pp<VPT, FAM>(B, B2, C, a.Pp, tp, true);
        else fft::block_fft<VPT, FAM>(B, C, a.Pp, tp, true);
        V* w2 = reinterpret_cast<V*>(a.w2) + (long long)q * np * a.ld2;
        for (int e = threadIdx.x; e < C * np; e += blockDim.x) {
            const int c = e % C, r = e / C, col = col0 + c;
            if (col < a.ncols) w2[r * a.ld2 + col] = FB[fft::pad<V>(c * np + r)];
        }
    }
}

// ---------------------------------------------------------------- inverse rows
struct RowsInvArgs {
    const void* w2;          // 4 planes of NYp rows, columns 0..kin-1, row stride ld2
    long long ld2;
    int kin;
    int nx, ny;              // psi grid
    int nb;                  // rows per group
    fft::RadixPlan P;        // packed length nx/2
    const void* tw;          // the row plan's pass twiddles, then W^k for k <= nx/2
};

// Epi::store(iX, iY, f, fx, fy, fxy): the four Hermite planes' values at psi node (iX, iY);
// groups of nb rows grid-strided; dynamic shared memory: padded(4 nb nx/2) values (twice for
// FP32: the scratch buffer) + the row plan's table
template <typename T, int FAM, int VPT, class Epi>
__global__ void __launch_bounds__(Shape<T>::MAXT, 1) k_psi_rows_inv(RowsInvArgs a, Epi epi)
{
    using V = typename fft::Cx<T>::V;
    constexpr bool PP = UsePP<T>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = a.nx / 2;
    V* s = reinterpret_cast<V*>(smem_raw);
    V* s2 = s + fft::padded_len<V>(4 * a.nb * n);          // scratch (PP)
    V* tw = s2 + (PP ? fft::padded_len<V>(4 * a.nb * n) : 0);
    fft::load_table(tw, reinterpret_cast<const V*>(a.tw), a.P.tlen + n + 1);
    const V* post = tw + a.P.tlen;
    const V zero = fft::mk((T)0, (T)0);
    const V* w2 = reinterpret_cast<const V*>(a.w2);
    for (int row0 = blockIdx.x * a.nb; row0 < a.ny; row0 += gridDim.x * a.nb) {
        const int nb = min(a.nb, a.ny - row0);
        __syncthreads();
        // transform t = 4 b + q: plane q of row row0 + b
        for (int t = 0; t < 4 * nb; ++t) {
            const int b = t >> 2, q = t & 3;
            const V* src = w2 + ((long long)q * a.ny + row0 + b) * a.ld2;
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                V xk = k < a.kin ? src[k] : zero;
                V xn = n - k < a.kin ? src[n - k] : zero;
                if (k == 0) { xk.y = (T)0; xn.y = (T)0; }
                s[fft::pad<V>(t * n + k)] = fft::c2r_pack(xk, xn, k, post);
            }
        }
        __syncthreads();
        const V* res = s;
        if (PP) res = fft::block_fft_pp<VPT, FAM>(s, s2, 4 * nb, a.P, tw, true);
        else fft::block_fft<VPT, FAM>(s, 4 * nb, a.P, tw, true);
        const T* sr = reinterpret_cast<const T*>(res);
        for (int b = 0; b < nb; ++b) {
            for (int iX = threadIdx.x; iX < a.nx; iX += blockDim.x) {
                const int base = 4 * b * n + (iX >> 1), c = iX & 1;
                epi.store(iX, row0 + b, sr[2 * fft::pad<V>(base) + c], sr[2 * fft::pad<V>(base + n) + c],
                          sr[2 * fft::pad<V>(base + 2 * n) + c], sr[2 * fft::pad<V>(base + 3 * n) + c]);
            }
        }
    }
}

// ---------------------------------------------------------------- static FP32 kernels
// The same two passes for power-of-two lengths known at compile time (fft::block_fft_s:
// every index a constant shift or mask), kStaticThreads threads, launched as programmatic
// dependents (each loads its tables, then waits for the previous kernel).  GT: the twiddle
// tables are read from global memory through L1 (shared memory holds only the data), else
// they are staged in shared memory.
constexpr int kStaticThreads = 256;

// groups (kept column, block of PQ planes), the column's PQ plane groups adjacent; the
// forward column transform (length NV) once per group, the PQ inverse transforms (length
// NP) as one batch.  The row spectra arrive column-major (fft::rows_r2c_t: bin col of row r
// at w1[col ld1 + r]), so a column is one contiguous read.  Shared memory: padded(NV) twice,
// padded(PQ NP) twice (and the tables).
template <int NV, int NP, int PQ, bool GT>
__host__ __device__ constexpr size_t cols_s_smem()
{
    return sizeof(float2) * (2 * (size_t)fft::padded_len<float2>(NV) + 2 * (size_t)fft::padded_len<float2>(PQ * NP) +
                             (GT ? 0 : (size_t)fft::sp::tlen(NV) + (size_t)fft::sp::tlen(NP)));
}

template <int NV, int NP, int PQ, bool GT>
__global__ void __launch_bounds__(kStaticThreads, 3) k_psi_cols_s(ColsArgs a)
{
    using V = float2;
    constexpr int VF = (NV + kStaticThreads - 1) / kStaticThreads, VI = (PQ * NP + kStaticThreads - 1) / kStaticThreads;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* A = reinterpret_cast<V*>(smem_raw);
    V* A2 = A + fft::padded_len<V>(NV);
    V* B = A2 + fft::padded_len<V>(NV);
    V* B2 = B + fft::padded_len<V>(PQ * NP);
    const V* tv = reinterpret_cast<const V*>(a.twv);
    const V* tp = reinterpret_cast<const V*>(a.twp);
    // the tables and each group's column arrive by 8-byte cp.async: their latencies overlap
    auto copy8 = [](V* dst, const V* src) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(src));
    };
    if (!GT) {
        V* stv = B2 + fft::padded_len<V>(PQ * NP);
        V* stp = stv + fft::sp::tlen(NV);
        for (int i = threadIdx.x; i < fft::sp::tlen(NV); i += kStaticThreads) copy8(stv + i, tv + i);
        for (int i = threadIdx.x; i < fft::sp::tlen(NP); i += kStaticThreads) copy8(stp + i, tp + i);
        tv = stv;
        tp = stp;
    }
    pdl_launch();
    pdl_wait();   // the row spectra come from the previous kernel
    const V* w1 = reinterpret_cast<const V*>(a.w1);
    const float freq = (float)a.freq, inv_nv = (float)(1.0 / (double)a.gv.N);
    constexpr int nq = 4 / PQ;
    for (int grp = blockIdx.x; grp < nq * a.ncols; grp += gridDim.x) {
        const int col = grp / nq, q0 = (grp - col * nq) * PQ;
        __syncthreads();   // the previous group's outputs are read
        for (int r = threadIdx.x; r < NV; r += kStaticThreads) {
            if (col < a.kv) copy8(A + fft::pad<V>(r), w1 + col * a.ld1 + r);
            else A[fft::pad<V>(r)] = fft::mk(0.f, 0.f);
        }
        asm volatile("cp.async.commit_group;");
        asm volatile("cp.async.wait_group 0;");
        __syncthreads();
        const V* FA = fft::block_fft_s<NV, VF, false, GT>(A, A2, 1, tv);
        // each row's mode once, then the PQ planes' multipliers
        for (int r = threadIdx.x; r < NP; r += kStaticThreads) {
            float kx, ky;
            const V P = plane_base_f(FA, 0, col, r, a.gv, a.gp, freq, inv_nv, kx, ky);
#pragma unroll
            for (int qq = 0; qq < PQ; ++qq) B[fft::pad<V>(qq * NP + r)] = plane_mul_f(P, q0 + qq, kx, ky);
        }
        __syncthreads();
        const V* FB = fft::block_fft_s<NP, VI, true, GT>(B, B2, PQ, tp);
        V* w2 = reinterpret_cast<V*>(a.w2) + (long long)q0 * NP * a.ld2 + col;
        for (int e = threadIdx.x; e < PQ * NP; e += kStaticThreads) w2[e * a.ld2] = FB[fft::pad<V>(e)];
    }
}

// groups of NBR psi rows (the four planes of each as one batch of 4 NBR transforms of the
// packed length N = nx / 2).  Shared memory: padded(4 NBR N) twice (and the table).
template <int N, int NBR, bool GT>
__host__ __device__ constexpr size_t rows_inv_s_smem()
{
    return sizeof(float2) * (2 * (size_t)fft::padded_len<float2>(4 * NBR * N) + (GT ? 0 : (size_t)fft::sp::tlen(N) + N + 1));
}

template <int N, int NBR, bool GT, class Epi>
__global__ void __launch_bounds__(kStaticThreads, 4) k_psi_rows_inv_s(RowsInvArgs a, Epi epi)
{
    using V = float2;
    constexpr int VPT = (4 * NBR * N + kStaticThreads - 1) / kStaticThreads;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* s = reinterpret_cast<V*>(smem_raw);
    V* s2 = s + fft::padded_len<V>(4 * NBR * N);
    const V* tw = reinterpret_cast<const V*>(a.tw);
    if (!GT) {
        V* stw = s2 + fft::padded_len<V>(4 * NBR * N);
        fft::load_table(stw, tw, fft::sp::tlen(N) + N + 1);
        tw = stw;
    }
    pdl_launch();
    pdl_wait();   // the column spectra come from the previous kernel
    const V* post = tw + fft::sp::tlen(N);
    const V zero = fft::mk(0.f, 0.f);
    const V* w2 = reinterpret_cast<const V*>(a.w2);
    const int kin = a.kin;   // at most N + 1: the 4 NBR rows' bins fit s2
    static_assert(4 * NBR * (N + 1) <= fft::padded_len<float2>(4 * NBR * N), "kept bins do not fit the scratch buffer");
    for (int row0 = blockIdx.x * NBR; row0 < a.ny; row0 += gridDim.x * NBR) {
        const int nb = min(NBR, a.ny - row0);
        __syncthreads();   // the previous group's results (in s or s2) are read
        // transform t = 4 b + q: plane q of row row0 + b.  Its kin kept bins go to s2 by 8-byte
        // cp.async (one round trip for all of them; s2 is the transform's scratch, free until
        // then), and the packing reads them there
        for (int t = 0; t < 4 * nb; ++t) {
            const V* src = w2 + ((long long)(t & 3) * a.ny + row0 + (t >> 2)) * a.ld2;
            for (int k = threadIdx.x; k < kin; k += kStaticThreads) {
                const unsigned sa = (unsigned)__cvta_generic_to_shared(s2 + t * kin + k);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(src + k));
            }
        }
        asm volatile("cp.async.commit_group;");
        asm volatile("cp.async.wait_group 0;");
        __syncthreads();
        for (int e = threadIdx.x; e < 4 * nb * N; e += kStaticThreads) {
            const int t = e / N, k = e % N;
            const V* sb = s2 + t * kin;
            V xk = k < kin ? sb[k] : zero;
            V xn = N - k < kin ? sb[N - k] : zero;
            if (k == 0) { xk.y = 0.f; xn.y = 0.f; }
            s[fft::pad<V>(e)] = fft::c2r_pack(xk, xn, k, post);
        }
        __syncthreads();
        const float* sr = reinterpret_cast<const float*>(fft::block_fft_s<N, VPT, true, GT>(s, s2, 4 * nb, tw));
        for (int e = threadIdx.x; e < nb * 2 * N; e += kStaticThreads) {
            const int b = e / (2 * N), iX = e % (2 * N);
            const int base = 4 * b * N + (iX >> 1), c = iX & 1;
            epi.store(iX, row0 + b, sr[2 * fft::pad<V>(base) + c], sr[2 * fft::pad<V>(base + N) + c],
                      sr[2 * fft::pad<V>(base + 2 * N) + c], sr[2 * fft::pad<V>(base + 3 * N) + c]);
        }
    }
}

// (vorticity column length, psi column length = psi row length) with a static kernel set,
// and the shape those kernels run (chosen by timing at the metric's sizes): planes per
// column group, rows per inverse-row group, tables in global memory (false: staged in
// shared memory)
#define CMM_PSI_STATIC(X) X(512, 256) X(1024, 512) X(2048, 1024) X(4096, 2048)
constexpr int kStaticPQ = 2, kStaticNBR = 1;
constexpr bool kStaticGT = false;

}  // namespace psi
}  // namespace cmm

namespace cmm {
namespace psi {

// ---------------------------------------------------------------- host side
// the shape of one solve on these kernels, or ok = false when the sizes need the 2D path
struct Layout {
    bool ok = false;
    int fam = 0;
    int ncols = 0;           // psi-grid columns kept: 0 .. min(NXp/2, freq)
    int kv = 0;              // vorticity-row bins written: 0 .. min(NXv/2, ncols - 1)
    long long ld = 0;        // row stride of both intermediate arrays (complex values)
    int nb_inv = 0, C = 0;   // psi rows per inverse-row group, columns per column group
    int vpt = 0;             // values per thread of both kernels
    bool stat = false;       // FP32 power-of-two sizes with a static kernel set (CMM_PSI_STATIC)
    size_t smem_cols = 0, smem_inv = 0;
    long long w1_values = 0, w2_values = 0;   // complex values of the intermediate arrays
};

template <typename T>
Layout make_layout(const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv, const fft::Plan2D& pp)
{
    using V = typename fft::Cx<T>::V;
    Layout L;
    if (!pv.ok() || !pp.ok() || gv.NX % 2 || gp.NX % 2 || pv.nx != gv.NX || pv.ny != gv.NY || pp.nx != gp.NX ||
        pp.ny != gp.NY)
        return L;
    L.fam = std::max(std::max(fft::family_of(pv.rx), fft::family_of(pv.ry)),
                     std::max(fft::family_of(pp.rx), fft::family_of(pp.ry)));
    if (L.fam == fft::kAny) return L;
    const int fc = freq >= (double)(1 << 30) ? (1 << 30) : (freq < 0 ? -1 : (int)std::floor(freq));
    L.ncols = std::min(gp.NX / 2, fc) + 1;
    if (L.ncols < 1) return L;
    L.kv = std::min(gv.NX / 2, L.ncols - 1) + 1;
    L.ld = (L.ncols + 3) / 4 * 4;
    const int np = gp.NX / 2;
    const int need = std::max(4 * np, std::max(gv.NY, gp.NY));   // values of the largest group
    L.vpt = need <= Shape<T>::VPT * Shape<T>::MAXT ? Shape<T>::VPT : Shape<T>::VPT_LONG;
    if (need > L.vpt * Shape<T>::MAXT) return L;
    L.nb_inv = std::max(1, kBlockValues / (4 * np));
    L.C = 1;
    while (2 * L.C * std::max(gv.NY, gp.NY) <= kBlockValues && L.C < 4) L.C *= 2;
    const size_t pp2 = UsePP<T>::value ? 2 : 1;   // FP32: ping-pong scratch buffers
    L.smem_inv = sizeof(V) * (pp2 * (size_t)fft::padded_len<V>(4 * L.nb_inv * np) + (size_t)pp.rx.tlen + (size_t)np + 1);
    L.smem_cols = sizeof(V) * (pp2 * ((size_t)fft::padded_len<V>(L.C * gv.NY) + (size_t)fft::padded_len<V>(L.C * gp.NY)) +
                               (size_t)pv.ry.tlen + (size_t)pp.ry.tlen);
    if (L.smem_cols > 200 * 1024 || L.smem_inv > 200 * 1024) return L;
    L.w1_values = (long long)gv.NY * L.ld;
    L.w2_values = 4ll * gp.NY * L.ld;
    L.ok = true;
    if (sizeof(T) == 4 && gp.NX == gp.NY) {
#define X(NV, NP)                                                                                       \
        if (gv.NY == NV && gp.NY == NP && fft::sp::matches(NV, pv.ry) && fft::sp::matches(NP, pp.ry) &&   \
            fft::sp::matches(NP / 2, pp.rx) && fft::rows_r2c_t_supported(pv)) {                         \
            L.stat = true;                                                                              \
            L.smem_cols = cols_s_smem<NV, NP, kStaticPQ, kStaticGT>();                                  \
            L.smem_inv = rows_inv_s_smem<NP / 2, kStaticNBR, kStaticGT>();                              \
        }
        CMM_PSI_STATIC(X)
#undef X
    }
    return L;
}

template <typename T, int FAM, int VPT, class Epi>
void set_smem_limits()
{
    cudaFuncSetAttribute(k_psi_cols<T, FAM, VPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_psi_rows_inv<T, FAM, VPT, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

// raise the kernels' shared-memory limits (before any stream capture)
template <typename T, class Epi>
void prepare()
{
    set_smem_limits<T, fft::kPow2, Shape<T>::VPT, Epi>();
    set_smem_limits<T, fft::kPow2x3, Shape<T>::VPT, Epi>();
    set_smem_limits<T, fft::kPow2, Shape<T>::VPT_LONG, Epi>();
    set_smem_limits<T, fft::kPow2x3, Shape<T>::VPT_LONG, Epi>();
    if (sizeof(T) == 4) {
#define X(NV, NP)                                                                                       \
        cudaFuncSetAttribute(k_psi_cols_s<NV, NP, kStaticPQ, kStaticGT>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             200 * 1024);                                                               \
        cudaFuncSetAttribute(k_psi_rows_inv_s<NP / 2, kStaticNBR, kStaticGT, Epi>,                       \
                             cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        CMM_PSI_STATIC(X)
#undef X
    }
}

// the static column and inverse-row kernels (FP32, L.stat) of one shape
template <int NV, int NP, int PQ, int NBR, bool GT, class Epi>
cudaError_t launch_static(const ColsArgs& c, const RowsInvArgs& v, const Epi& epi, cudaStream_t s)
{
    constexpr size_t smc = cols_s_smem<NV, NP, PQ, GT>(), smi = rows_inv_s_smem<NP / 2, NBR, GT>();
    const void* fc = reinterpret_cast<const void*>(k_psi_cols_s<NV, NP, PQ, GT>);
    cudaError_t e = launch_pdl(k_psi_cols_s<NV, NP, PQ, GT>,
                               fft::resident_grid(fc, kStaticThreads, smc, (4 / PQ) * (long long)c.ncols), kStaticThreads,
                               smc, s, c);
    if (e != cudaSuccess) return e;
    const void* fi = reinterpret_cast<const void*>(k_psi_rows_inv_s<NP / 2, NBR, GT, Epi>);
    return launch_pdl(k_psi_rows_inv_s<NP / 2, NBR, GT, Epi>,
                      fft::resident_grid(fi, kStaticThreads, smi, (v.ny + NBR - 1) / NBR), kStaticThreads, smi, s, v, epi);
}

inline int threads_for(int values, int vpt)
{
    int t = (values + vpt - 1) / vpt;
    t = (t + 31) / 32 * 32;
    return t < 32 ? 32 : t;
}

template <typename T, int FAM, int VPT, class Epi>
cudaError_t launch_fam(const Layout& L, const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv,
                       const fft::Plan2D& pp, const void* omega, void* w1, void* w2, const Epi& epi, cudaStream_t s)
{
    // static kernels: the kept bins column-major (kv columns of NY values: within w1_values)
    cudaError_t e = L.stat ? fft::rows_r2c_t(pv, omega, gv.NX, w1, gv.NY, gv.NY, L.kv, s)
                           : fft::rows_r2c(pv, omega, gv.NX, gv.N, w1, L.ld, L.w1_values, gv.NY, 1, L.kv, s);
    if (e != cudaSuccess) return e;
    ColsArgs c;
    c.w1 = w1; c.w2 = w2; c.ld1 = L.stat ? gv.NY : L.ld; c.ld2 = L.ld; c.kv = L.kv; c.ncols = L.ncols; c.C = L.C;
    c.gv = gv; c.gp = gp; c.freq = freq; c.Pv = pv.ry; c.Pp = pp.ry; c.twv = pv.twy; c.twp = pp.twy;
    if (L.stat) {
        RowsInvArgs v;
        v.w2 = w2; v.ld2 = L.ld; v.kin = L.ncols; v.nx = gp.NX; v.ny = gp.NY; v.nb = kStaticNBR; v.P = pp.rx;
        v.tw = pp.twx;
#define X(NV, NP)                                                                                       \
        if (gv.NY == NV && gp.NY == NP) return launch_static<NV, NP, kStaticPQ, kStaticNBR, kStaticGT>(c, v, epi, s);
        CMM_PSI_STATIC(X)
#undef X
        return cudaErrorInvalidValue;
    }
    const int tc = threads_for(L.C * std::max(gv.NY, gp.NY), VPT);
    const long long gc = 4ll * ((L.ncols + L.C - 1) / L.C);
    k_psi_cols<T, FAM, VPT><<<fft::resident_grid(reinterpret_cast<const void*>(k_psi_cols<T, FAM, VPT>), tc, L.smem_cols,
                                                 gc), tc, L.smem_cols, s>>>(c);
    RowsInvArgs v;
    v.w2 = w2; v.ld2 = L.ld; v.kin = L.ncols; v.nx = gp.NX; v.ny = gp.NY; v.nb = L.nb_inv; v.P = pp.rx; v.tw = pp.twx;
    const int ti = threads_for(4 * L.nb_inv * (gp.NX / 2), VPT);
    const long long gi = (gp.NY + L.nb_inv - 1) / L.nb_inv;
    k_psi_rows_inv<T, FAM, VPT, Epi><<<fft::resident_grid(reinterpret_cast<const void*>(k_psi_rows_inv<T, FAM, VPT, Epi>),
                                                          ti, L.smem_inv, gi), ti, L.smem_inv, s>>>(v, epi);
    return cudaGetLastError();
}

// the three transform passes of one psi solve from the sampled vorticity omega (gv rows,
// FP32 or FP64); w1, w2 hold L.w1_values, L.w2_values complex values
template <typename T, class Epi>
cudaError_t launch(const Layout& L, const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv,
                   const fft::Plan2D& pp, const void* omega, void* w1, void* w2, const Epi& epi, cudaStream_t s)
{
    if (!L.ok) return cudaErrorInvalidValue;
    constexpr int A = Shape<T>::VPT, B = Shape<T>::VPT_LONG;
    if (L.fam == fft::kPow2)
        return L.vpt == A ? launch_fam<T, fft::kPow2, A>(L, gv, gp, freq, pv, pp, omega, w1, w2, epi, s)
                          : launch_fam<T, fft::kPow2, B>(L, gv, gp, freq, pv, pp, omega, w1, w2, epi, s);
    return L.vpt == A ? launch_fam<T, fft::kPow2x3, A>(L, gv, gp, freq, pv, pp, omega, w1, w2, epi, s)
                      : launch_fam<T, fft::kPow2x3, B>(L, gv, gp, freq, pv, pp, omega, w1, w2, epi, s);
}

}  // namespace psi
}  // namespace cmm
