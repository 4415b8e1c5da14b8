// psi_solve.cuh -- the psi solve of one time step as three fused kernels on the
// library's FFT engine (fft.cuh), templated on the precision (FP64 plain form,
// FP32 mixed form).
//
// Reference: evaluate_stream_hermite (Cuda-CMM/src/simulation/cmm-simulation-host.cu:
// 333-375): omega sampled through the map on the vorticity grid
// (k_apply_map_and_sample_from_hermite), D2Z, k_normalize_h, k_fft_grid_move to the psi
// grid, k_fft_cut_off_scale_h, k_fft_iLap_h (src/numerical/cmm-fft.cu:55-78,267-339), and
// fourier_hermite (:398-429: the spectra of psi, d/dx, d/dy, d2/dxdy and four Z2D).
//
// Here:
//   rows   (k_psi_rows)   one block per few vorticity-grid rows samples omega for the
//                         whole row straight into shared memory, transforms the row and
//                         writes only the columns kx the cut-off and the psi grid keep;
//   cols   (k_psi_cols)   one block per (group of C kept columns, Hermite plane): the
//                         column's forward transform over the vorticity grid, the
//                         spectral steps (normalise, grid move, circular cut-off, inverse
//                         Laplacian, the plane's derivative multiplier) and the inverse
//                         column transform over the psi grid;
//   inverse rows (k_psi_rows_inv)  one block per few psi rows: the row C2R of the four
//                         planes (missing columns are zero) and an epilogue that writes
//                         the Hermite nodes (and, in the mixed form, the Lagrange
//                         combinations of the next step).
// Between them only the kept columns travel through global memory: at the metric's
// sizes (vorticity 2048^2, psi 1024^2, cut-off 128) 2048 x 129 and 4 x 1024 x 129
// complex values instead of the full half spectra.
#pragma once
#include <algorithm>
#include <cmath>

#include "cmm_common.cuh"
#include "fft.hpp"

namespace cmm {
namespace psi {

// block shapes: values per thread (VPT) and threads.  FP64 blocks hold 8 values per
// thread (an FP64 radix-8 butterfly with its inputs fits the 128 registers of a 512-thread
// block); FP32 blocks 16.  Every block holds up to 4096 complex values.
template <typename T> struct Shape;
template <> struct Shape<float> { static constexpr int VPT = 16, ROWT = 256, COLC = 4; };
template <> struct Shape<double> { static constexpr int VPT = 8, ROWT = 512, COLC = 2; };
constexpr int kColThreads = 512;
constexpr int kMaxValues = 4096;   // complex values a block transforms at once

struct ColsArgs {
    const void* w1;          // vorticity-grid row spectra: NYv rows, columns 0..kv-1, row stride ld1
    void* w2;                // the four psi-grid spectra: 4 x NYp rows, columns 0..ncols-1, row stride ld2
    long long ld1, ld2;
    int kv, ncols;
    int C;                   // columns per block (32-byte row segments where they fit)
    Grid gv, gp;
    double freq;
    fft::RadixPlan Pv, Pp;   // column lengths NYv, NYp
    const void* twv;         // NYv entries exp(-2 pi i t / NYv)
    const void* twp;         // NYp entries
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

template <>
__device__ __forceinline__ float2 plane_mode<float2>(const float2* s, int off, int q, int iXc, int iYc, const Grid& gv,
                                                     const Grid& gp, double freqd)
{
    const float freq = (float)freqd, inv_nv = (float)(1.0 / (double)gv.N);
    const bool hx = 2 * iXc > gp.NX, hy = 2 * iYc > gp.NY;
    const int fX = hx ? gp.NX - iXc : iXc, fY = hy ? gp.NY - iYc : iYc;
    float2 P = make_float2(0.f, 0.f);
    if (!(2 * fX > gv.NX || 2 * fY > gv.NY)) {
        const int iYs = iYc + (hy ? gv.NY - gp.NY : 0);
        const float2 f = s[fft::pad<float2>(off + iYs)];
        P = make_float2(f.x * inv_nv, f.y * inv_nv);
    }
    if ((float)(fX * fX + fY * fY) > freq * freq || (iXc == 0 && iYc == 0)) P = make_float2(0.f, 0.f);
    const float kx = gp.kfxf * (float)(hx ? iXc - gp.NX : iXc);
    const float ky = gp.kfyf * (float)(hy ? iYc - gp.NY : iYc);
    if (iXc == 0 && iYc == 0) P = make_float2(0.f, 0.f);
    else {
        const float ik2 = 1.0f / (kx * kx + ky * ky);
        P = make_float2(-P.x * ik2, -P.y * ik2);
    }
    if (q == 0) return P;
    if (q == 1) return make_float2(-P.y * kx, P.x * kx);
    const float2 Py = make_float2(-P.y * ky, P.x * ky);
    return q == 2 ? Py : make_float2(-Py.y * kx, Py.x * kx);
}

// grid (ceil(ncols / C), 4 planes); dynamic shared memory: padded(C NYv) + padded(C NYp) values
template <typename T, int FAM>
__global__ void __launch_bounds__(kColThreads, 1) k_psi_cols(ColsArgs a)
{
    using V = typename fft::Cx<T>::V;
    constexpr int VPT = Shape<T>::VPT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nv = a.gv.NY, np = a.gp.NY, C = a.C;
    V* A = reinterpret_cast<V*>(smem_raw);
    V* B = A + fft::padded_len<V>(C * nv);
    const int col0 = blockIdx.x * C, q = blockIdx.y;
    const V* w1 = reinterpret_cast<const V*>(a.w1);
    for (int e = threadIdx.x; e < C * nv; e += blockDim.x) {
        const int c = e % C, r = e / C, col = col0 + c;
        A[fft::pad<V>(c * nv + r)] = col < a.kv ? w1[r * a.ld1 + col] : fft::mk((T)0, (T)0);
    }
    __syncthreads();
    fft::block_fft<VPT, FAM>(A, C, a.Pv, reinterpret_cast<const V*>(a.twv), 1, false);
    for (int e = threadIdx.x; e < C * np; e += blockDim.x) {
        const int c = e / np, r = e - c * np;
        B[fft::pad<V>(e)] = plane_mode<V>(A, c * nv, q, col0 + c, r, a.gv, a.gp, a.freq);
    }
    __syncthreads();
    fft::block_fft<VPT, FAM>(B, C, a.Pp, reinterpret_cast<const V*>(a.twp), 1, true);
    V* w2 = reinterpret_cast<V*>(a.w2) + (long long)q * np * a.ld2;
    for (int e = threadIdx.x; e < C * np; e += blockDim.x) {
        const int c = e % C, r = e / C, col = col0 + c;
        if (col < a.ncols) w2[r * a.ld2 + col] = B[fft::pad<V>(c * np + r)];
    }
}

// ---------------------------------------------------------------- forward rows
struct RowsArgs {
    void* w1;                // output: row stride ld1, columns 0..kv-1
    long long ld1;
    int kv;
    int nx, ny;              // vorticity grid
    int nb;                  // rows per block
    fft::RadixPlan P;        // packed length nx/2
    const void* tw;          // nx entries
};

// Src::value(iX, iY, live) -> T: omega at vort node (iX, iY); every thread of a warp calls it
// together (samplers may exchange values between lanes); `live` false for padding lanes
template <typename T, int FAM, class Src>
__global__ void __launch_bounds__(Shape<T>::ROWT, 1) k_psi_rows(RowsArgs a, Src src)
{
    using V = typename fft::Cx<T>::V;
    constexpr int VPT = Shape<T>::VPT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* s = reinterpret_cast<V*>(smem_raw);
    T* sr = reinterpret_cast<T*>(smem_raw);
    const int n = a.nx / 2;
    const int row0 = blockIdx.x * a.nb;
    const int nb = min(a.nb, a.ny - row0);
    const int total = nb * a.nx;
    const int iters = (a.nb * a.nx + blockDim.x - 1) / blockDim.x;
    for (int j = 0; j < iters; ++j) {
        const int e = threadIdx.x + j * blockDim.x;
        const bool live = e < total;
        const int ee = live ? e : total - 1;
        const int b = ee / a.nx, iX = ee - b * a.nx;
        const T v = src.value(iX, row0 + b, live);
        if (live) {
            const int m = b * n + (iX >> 1);
            sr[2 * fft::pad<V>(m) + (iX & 1)] = v;
        }
    }
    __syncthreads();
    fft::block_fft<VPT, FAM>(s, nb, a.P, reinterpret_cast<const V*>(a.tw), 2, false);
    V* w1 = reinterpret_cast<V*>(a.w1);
    for (int e = threadIdx.x; e < nb * a.kv; e += blockDim.x) {
        const int b = e / a.kv, k = e - b * a.kv;
        w1[(row0 + b) * a.ld1 + k] = fft::r2c_bin(s, b * n, n, k, reinterpret_cast<const V*>(a.tw));
    }
}

// ---------------------------------------------------------------- inverse rows
struct RowsInvArgs {
    const void* w2;          // 4 planes of NYp rows, columns 0..kin-1, row stride ld2
    long long ld2;
    int kin;
    int nx, ny;              // psi grid
    int nb;                  // rows per block
    fft::RadixPlan P;        // packed length nx/2
    const void* tw;          // nx entries
};

// Epi::store(iX, iY, f, fx, fy, fxy): the four Hermite planes' values at psi node (iX, iY)
template <typename T, int FAM, class Epi>
__global__ void __launch_bounds__(Shape<T>::ROWT, 1) k_psi_rows_inv(RowsInvArgs a, Epi epi)
{
    using V = typename fft::Cx<T>::V;
    constexpr int VPT = Shape<T>::VPT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* s = reinterpret_cast<V*>(smem_raw);
    const T* sr = reinterpret_cast<const T*>(smem_raw);
    const V* tw = reinterpret_cast<const V*>(a.tw);
    const int n = a.nx / 2;
    const int row0 = blockIdx.x * a.nb;
    const int nb = min(a.nb, a.ny - row0);
    const V zero = fft::mk((T)0, (T)0);
    const V* w2 = reinterpret_cast<const V*>(a.w2);
    // transform t = 4 b + q: plane q of row row0 + b
    for (int e = threadIdx.x; e < 4 * nb * n; e += blockDim.x) {
        const int t = e / n, k = e - t * n, b = t >> 2, q = t & 3;
        const V* src = w2 + ((long long)q * a.ny + row0 + b) * a.ld2;
        V xk = k < a.kin ? src[k] : zero;
        V xn = n - k < a.kin ? src[n - k] : zero;
        if (k == 0) { xk.y = (T)0; xn.y = (T)0; }
        s[fft::pad<V>(e)] = fft::c2r_pack(xk, xn, k, tw);
    }
    __syncthreads();
    fft::block_fft<VPT, FAM>(s, 4 * nb, a.P, tw, 2, true);
    for (int e = threadIdx.x; e < nb * a.nx; e += blockDim.x) {
        const int b = e / a.nx, iX = e - b * a.nx;
        const int base = 4 * b * n + (iX >> 1), c = iX & 1;
        epi.store(iX, row0 + b, sr[2 * fft::pad<V>(base) + c], sr[2 * fft::pad<V>(base + n) + c],
                  sr[2 * fft::pad<V>(base + 2 * n) + c], sr[2 * fft::pad<V>(base + 3 * n) + c]);
    }
}

}  // namespace psi
}  // namespace cmm

namespace cmm {
namespace psi {

// ---------------------------------------------------------------- host side
// the shape of one fused solve, or ok = false when the sizes need the unfused path
struct Layout {
    bool ok = false;
    int fam = 0;
    int ncols = 0;           // psi-grid columns kept: 0 .. min(NXp/2, freq)
    int kv = 0;              // vorticity-row bins written: 0 .. min(NXv/2, ncols - 1)
    long long ld = 0;        // row stride of both intermediate arrays (complex values)
    int nb_rows = 0, nb_inv = 0, C = 0;
    size_t smem_rows = 0, smem_cols = 0, smem_inv = 0;
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
    const int cap = Shape<T>::VPT * Shape<T>::ROWT;   // values one row block transforms
    const int nv = gv.NX / 2, np = gp.NX / 2;
    if (nv > cap || 4 * np > cap) return L;
    L.nb_rows = std::max(1, std::min(kMaxValues, cap) / nv);
    L.nb_inv = std::max(1, std::min(kMaxValues, cap) / (4 * np));
    L.C = Shape<T>::COLC;
    const int ccap = Shape<T>::VPT * kColThreads;
    auto col_smem = [&](int C) {
        return sizeof(V) * ((size_t)fft::padded_len<V>(C * gv.NY) + (size_t)fft::padded_len<V>(C * gp.NY));
    };
    while (L.C > 1 && (L.C * std::max(gv.NY, gp.NY) > ccap || col_smem(L.C) > 200 * 1024)) L.C /= 2;
    if (L.C * std::max(gv.NY, gp.NY) > ccap || col_smem(L.C) > 200 * 1024) return L;
    L.smem_rows = sizeof(V) * (size_t)fft::padded_len<V>(L.nb_rows * nv);
    L.smem_inv = sizeof(V) * (size_t)fft::padded_len<V>(4 * L.nb_inv * np);
    L.smem_cols = col_smem(L.C);
    L.w1_values = (long long)gv.NY * L.ld;
    L.w2_values = 4ll * gp.NY * L.ld;
    L.ok = true;
    return L;
}

template <typename T, int FAM, class Src, class Epi>
void set_smem_limits()
{
    cudaFuncSetAttribute(k_psi_rows<T, FAM, Src>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_psi_cols<T, FAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_psi_rows_inv<T, FAM, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

// raise the kernels' shared-memory limits (before any stream capture)
template <typename T, class Src, class Epi>
void prepare()
{
    set_smem_limits<T, fft::kPow2, Src, Epi>();
    set_smem_limits<T, fft::kPow2x3, Src, Epi>();
}

template <typename T, int FAM, class Src, class Epi>
cudaError_t launch_fam(const Layout& L, const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv,
                       const fft::Plan2D& pp, void* w1, void* w2, const Src& src, const Epi& epi, cudaStream_t s)
{
    RowsArgs r;
    r.w1 = w1; r.ld1 = L.ld; r.kv = L.kv; r.nx = gv.NX; r.ny = gv.NY; r.nb = L.nb_rows; r.P = pv.rx; r.tw = pv.twx;
    k_psi_rows<T, FAM, Src><<<(unsigned)((gv.NY + L.nb_rows - 1) / L.nb_rows), Shape<T>::ROWT, L.smem_rows, s>>>(r, src);
    ColsArgs c;
    c.w1 = w1; c.w2 = w2; c.ld1 = L.ld; c.ld2 = L.ld; c.kv = L.kv; c.ncols = L.ncols; c.C = L.C;
    c.gv = gv; c.gp = gp; c.freq = freq; c.Pv = pv.ry; c.Pp = pp.ry; c.twv = pv.twy; c.twp = pp.twy;
    k_psi_cols<T, FAM><<<dim3((unsigned)((L.ncols + L.C - 1) / L.C), 4), kColThreads, L.smem_cols, s>>>(c);
    RowsInvArgs v;
    v.w2 = w2; v.ld2 = L.ld; v.kin = L.ncols; v.nx = gp.NX; v.ny = gp.NY; v.nb = L.nb_inv; v.P = pp.rx; v.tw = pp.twx;
    k_psi_rows_inv<T, FAM, Epi><<<(unsigned)((gp.NY + L.nb_inv - 1) / L.nb_inv), Shape<T>::ROWT, L.smem_inv, s>>>(v, epi);
    return cudaGetLastError();
}

// the three kernels of one psi solve (3 launches); w1, w2 hold L.w1_values, L.w2_values
template <typename T, class Src, class Epi>
cudaError_t launch(const Layout& L, const Grid& gv, const Grid& gp, double freq, const fft::Plan2D& pv,
                   const fft::Plan2D& pp, void* w1, void* w2, const Src& src, const Epi& epi, cudaStream_t s)
{
    if (!L.ok) return cudaErrorInvalidValue;
    if (L.fam == fft::kPow2) return launch_fam<T, fft::kPow2>(L, gv, gp, freq, pv, pp, w1, w2, src, epi, s);
    return launch_fam<T, fft::kPow2x3>(L, gv, gp, freq, pv, pp, w1, w2, src, epi, s);
}

}  // namespace psi
}  // namespace cmm
