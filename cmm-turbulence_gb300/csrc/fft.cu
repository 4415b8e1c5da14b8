// fft.cu -- batched real / complex transforms on the library's own Stockham engine
// (fft.cuh): the row pass (R2C or C2R of whole rows, a few rows per block) and the
// column pass (in-place complex transforms of C adjacent columns per block).  Every
// kernel is persistent: a block copies its twiddle table into shared memory once and
// then transforms group after group (rows or column groups) with a grid stride.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "fft.hpp"
#include "pdl.cuh"

namespace cmm {
namespace fft {

namespace {

// Block shapes: VPT values per thread, at most MAXT threads (launch bound with one block
// per SM, so up to 65536 / MAXT registers).  FP32 power-of-two (and 3 * 2^k) lengths run
// 4 values per thread (8 beyond 4096 values) within 64 registers: short passes, several
// blocks per SM; FP64 blocks hold 8 values per thread within 128 registers (a radix-8
// butterfly and its inputs), 16 beyond 4096 values; lengths with larger prime factors
// run 256 threads (registers for the generic butterflies).
struct Shape { int vpt, maxt; };
constexpr int kBlockValues = 2048;      // values per block the launchers aim for
constexpr int kMaxSmem = 227 * 1024;    // dynamic shared memory the kernels may request (sm_103a opt-in maximum)

struct RowsArgs {
    const void* in;
    void* out;
    long long ild, idist, old, odist;   // in elements of the input / output type
    int rows_per_item, rows_total;
    int kio;                            // R2C: bins written; C2R: bins read (the rest zero)
    int nb;                             // rows per group
    int tout;                           // R2C (static kernel): bin k of row r at out[k old + r]
    RadixPlan P;                        // packed complex length nx/2
    const void* tw;                     // P.tlen pass twiddles, then W^k for k <= nx/2
};

struct ColsArgs {
    void* data;
    long long ld, bdist;                // complex elements
    int ncols, C, lc;                   // columns, columns per group (a power of two), log2 C
    int batch;
    int inv;
    RadixPlan P;                        // length ny
    const void* tw;                     // P.tlen pass twiddles
};

// the nb rows of the group at row0 (row0 < rows_total) into shared memory with cp.async
// (global -> shared, no register round trip), one commit group
template <typename T, typename V>
__device__ __forceinline__ void rows_prefetch(const RowsArgs& a, V* dst, int row0)
{
    const int n = a.P.n, nb = min(a.nb, a.rows_total - row0);
    for (int b = 0; b < nb; ++b) {
        const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
        const V* src = reinterpret_cast<const V*>(reinterpret_cast<const T*>(a.in) + item * a.idist + r * a.ild);
        for (int m = threadIdx.x; m < n; m += blockDim.x) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + pad<V>(b * n + m));
            asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(sa), "l"(src + m), "n"(sizeof(V)));
        }
    }
}

// GTW: the twiddle table is read from global memory (too large to stage next to the data).
// Otherwise two data buffers: while a group is transformed, the next group's rows arrive
// by cp.async.
// FP32 rows transform through a scratch buffer (block_fft_pp: one barrier per pass)
template <typename T> struct RowsPP { static constexpr bool value = std::is_same<T, float>::value; };

template <typename T, int FAM, int VPT, int MAXT, bool GTW>
__global__ void __launch_bounds__(MAXT, 1) k_rows_r2c(RowsArgs a)
{
    using V = typename Cx<T>::V;
    constexpr bool DB = !GTW, PP = RowsPP<T>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = a.P.n;
    V* cur = reinterpret_cast<V*>(smem_raw);
    V* nxt = cur + (DB ? padded_len<V>(a.nb * n) : 0);
    V* tmp = nxt + padded_len<V>(a.nb * n);   // ping-pong scratch (PP)
    V* stw = tmp + (PP ? padded_len<V>(a.nb * n) : 0);
    if (!GTW) load_table(stw, reinterpret_cast<const V*>(a.tw), a.P.tlen + n + 1);
    const V* tw = GTW ? reinterpret_cast<const V*>(a.tw) : stw;
    const V* post = tw + a.P.tlen;
    const int stride = gridDim.x * a.nb;
    if (DB) {
        if (blockIdx.x * a.nb < a.rows_total) rows_prefetch<T>(a, cur, blockIdx.x * a.nb);
        asm volatile("cp.async.commit_group;");
    }
    for (int row0 = blockIdx.x * a.nb; row0 < a.rows_total; row0 += stride) {
        const int nb = min(a.nb, a.rows_total - row0);
        __syncthreads();   // the previous group's bins are read: its buffer may be refilled
        if (DB) {
            if (row0 + stride < a.rows_total) rows_prefetch<T>(a, nxt, row0 + stride);
            asm volatile("cp.async.commit_group;");
            asm volatile("cp.async.wait_group 1;");   // this group's rows have landed
        } else {
            for (int b = 0; b < nb; ++b) {
                const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
                const V* src = reinterpret_cast<const V*>(reinterpret_cast<const T*>(a.in) + item * a.idist + r * a.ild);
                for (int m = threadIdx.x; m < n; m += blockDim.x) cur[pad<V>(b * n + m)] = src[m];
            }
        }
        __syncthreads();
        const V* res = cur;
        if (PP) res = block_fft_pp<VPT, FAM>(cur, tmp, nb, a.P, tw, false);
        else block_fft<VPT, FAM>(cur, nb, a.P, tw, false);
        for (int b = 0; b < nb; ++b) {
            const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
            V* dst = reinterpret_cast<V*>(a.out) + item * a.odist + r * a.old;
            for (int k = threadIdx.x; k < a.kio; k += blockDim.x) dst[k] = r2c_bin(res, b * n, n, k, post);
        }
        if (DB) {
            V* t = cur;
            cur = nxt;
            nxt = t;
        }
    }
    if (DB) asm volatile("cp.async.wait_group 0;");
}

// FP32 rows of a compile-time power-of-two packed length N (block_fft_s: constant index
// arithmetic), kStaticThreads threads of kStaticVPT values, nb = kStaticThreads kStaticVPT / N
// rows per group.  The rows arrive unpadded by 16-byte cp.async.cg (past L1, into the
// second of two row buffers while the first is transformed) and the first pass reads them
// so; GT: the twiddle tables are read from global memory through L1, else staged in
// shared memory.  Needs 16-byte aligned rows.
constexpr int kStaticThreads = 256, kStaticVPT = 8;

template <int N>
__device__ __forceinline__ void rows_prefetch_s(const RowsArgs& a, float2* dst, int row0)
{
    const int nb = min(a.nb, a.rows_total - row0);
    for (int b = 0; b < nb; ++b) {
        const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
        const float* src = reinterpret_cast<const float*>(a.in) + item * a.idist + r * a.ild;
        for (int m = threadIdx.x; m < N / 2; m += kStaticThreads) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + b * N + 2 * m);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(src + 4 * m));
        }
    }
}

template <int N, bool GT>
__global__ void __launch_bounds__(kStaticThreads, GT ? 4 : 3) k_rows_r2c_s(RowsArgs a)
{
    using V = float2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int len = (padded_len<V>(a.nb * N) + 1) & ~1;   // even: the buffers stay 16-byte aligned
    V* cur = reinterpret_cast<V*>(smem_raw);
    V* nxt = cur + len;
    V* tmp = nxt + len;
    const V* tw = reinterpret_cast<const V*>(a.tw);
    if (!GT) {
        V* stw = tmp + len;
        load_table(stw, tw, sp::tlen(N) + N + 1);
        tw = stw;
    }
    const V* post = tw + sp::tlen(N);
    const int stride = gridDim.x * a.nb;
    pdl_launch();
    pdl_wait();   // the rows come from the previous kernel
    if (blockIdx.x * a.nb < a.rows_total) rows_prefetch_s<N>(a, cur, blockIdx.x * a.nb);
    asm volatile("cp.async.commit_group;");
    for (int row0 = blockIdx.x * a.nb; row0 < a.rows_total; row0 += stride) {
        const int nb = min(a.nb, a.rows_total - row0);
        __syncthreads();   // the previous group's bins are read: its buffers may be refilled
        if (row0 + stride < a.rows_total) rows_prefetch_s<N>(a, nxt, row0 + stride);
        asm volatile("cp.async.commit_group;");
        asm volatile("cp.async.wait_group 1;");
        __syncthreads();
        const V* res = block_fft_s<N, kStaticVPT, false, GT, true>(cur, tmp, nb, tw);
        if (a.tout) {
            // column-major bins (one item): rows row0 + b and row0 + b + 1 of bin k are adjacent,
            // one 16-byte store per pair
            V* out = reinterpret_cast<V*>(a.out);
            for (int b = 0; b + 1 < nb; b += 2)
                for (int k = threadIdx.x; k < a.kio; k += kStaticThreads) {
                    const V u = r2c_bin(res, b * N, N, k, post), w = r2c_bin(res, (b + 1) * N, N, k, post);
                    *reinterpret_cast<float4*>(out + k * a.old + row0 + b) = make_float4(u.x, u.y, w.x, w.y);
                }
            if (nb & 1)
                for (int k = threadIdx.x; k < a.kio; k += kStaticThreads)
                    out[k * a.old + row0 + nb - 1] = r2c_bin(res, (nb - 1) * N, N, k, post);
        } else {
            for (int b = 0; b < nb; ++b) {
                const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
                V* dst = reinterpret_cast<V*>(a.out) + item * a.odist + r * a.old;
                for (int k = threadIdx.x; k < a.kio; k += kStaticThreads) dst[k] = r2c_bin(res, b * N, N, k, post);
            }
        }
        V* t = cur;
        cur = nxt;
        nxt = t;
    }
    asm volatile("cp.async.wait_group 0;");
}

// packed lengths with a static kernel
#define CMM_FFT_STATIC_ROWS(X) X(128) X(256) X(512) X(1024) X(2048)
constexpr bool kStaticGT = false;   // tables staged in shared memory
// table length of the power-of-two plan of length n (host side of sp::tlen)
inline int sp_tlen_pow2(int n)
{
#define X(N) if (n == N) return sp::tlen(N);
    CMM_FFT_STATIC_ROWS(X)
#undef X
    return 0;
}

template <typename T, int FAM, int VPT, int MAXT, bool GTW>
__global__ void __launch_bounds__(MAXT, 1) k_rows_c2r(RowsArgs a)
{
    using V = typename Cx<T>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = a.P.n;
    V* s = reinterpret_cast<V*>(smem_raw);
    V* stw = s + padded_len<V>(a.nb * n);
    if (!GTW) load_table(stw, reinterpret_cast<const V*>(a.tw), a.P.tlen + n + 1);
    const V* tw = GTW ? reinterpret_cast<const V*>(a.tw) : stw;
    const V* post = tw + a.P.tlen;
    const V zero = mk((T)0, (T)0);
    for (int row0 = blockIdx.x * a.nb; row0 < a.rows_total; row0 += gridDim.x * a.nb) {
        const int nb = min(a.nb, a.rows_total - row0);
        __syncthreads();
        for (int b = 0; b < nb; ++b) {
            const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
            const V* src = reinterpret_cast<const V*>(a.in) + item * a.idist + r * a.ild;
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                V xk = k < a.kio ? src[k] : zero;
                V xn = n - k < a.kio ? src[n - k] : zero;
                if (k == 0) { xk.y = (T)0; xn.y = (T)0; }
                s[pad<V>(b * n + k)] = c2r_pack(xk, xn, k, post);
            }
        }
        __syncthreads();
        block_fft<VPT, FAM>(s, nb, a.P, tw, true);
        for (int b = 0; b < nb; ++b) {
            const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
            V* dst = reinterpret_cast<V*>(reinterpret_cast<T*>(a.out) + item * a.odist + r * a.old);
            for (int m = threadIdx.x; m < n; m += blockDim.x) dst[m] = s[pad<V>(b * n + m)];
        }
    }
}

// groups of C adjacent columns of every batch item, grid-strided
template <typename T, int FAM, int VPT, int MAXT, bool GTW>
__global__ void __launch_bounds__(MAXT, 1) k_cols(ColsArgs a)
{
    using V = typename Cx<T>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = a.P.n, C = a.C, lc = a.lc;
    V* s = reinterpret_cast<V*>(smem_raw);
    V* stw = s + padded_len<V>(C * n);
    if (!GTW) load_table(stw, reinterpret_cast<const V*>(a.tw), a.P.tlen);
    const V* tw = GTW ? reinterpret_cast<const V*>(a.tw) : stw;
    const int gx = (a.ncols + C - 1) / C;
    for (int grp = blockIdx.x; grp < gx * a.batch; grp += gridDim.x) {
        const int item = grp / gx, col0 = (grp - item * gx) * C;
        const int cn = min(C, a.ncols - col0);
        V* base = reinterpret_cast<V*>(a.data) + item * a.bdist + col0;
        __syncthreads();
        for (int e = threadIdx.x; e < C * n; e += blockDim.x) {
            const int c = e & (C - 1), r = e >> lc;
            s[pad<V>(c * n + r)] = c < cn ? base[r * a.ld + c] : mk((T)0, (T)0);
        }
        __syncthreads();
        block_fft<VPT, FAM>(s, C, a.P, tw, a.inv != 0);
        for (int e = threadIdx.x; e < C * n; e += blockDim.x) {
            const int c = e & (C - 1), r = e >> lc;
            if (c < cn) base[r * a.ld + c] = s[pad<V>(c * n + r)];
        }
    }
}

Shape shape_for(bool dbl, int fam, int values)
{
    if (fam == kAny) return values <= 16 * 256 ? Shape{16, 256} : Shape{32, 256};
    if (!dbl) return values <= 4 * 1024 ? Shape{4, 1024} : Shape{8, 1024};
    return values <= 8 * 512 ? Shape{8, 512} : Shape{16, 512};
}

int threads_for(int values, const Shape& sh)
{
    int t = (values + sh.vpt - 1) / sh.vpt;
    t = (t + 31) / 32 * 32;
    return t < 32 ? 32 : (t > sh.maxt ? sh.maxt : t);
}

template <typename T>
size_t smem_bytes(int values, int table)
{
    using V = typename Cx<T>::V;
    return sizeof(V) * ((size_t)padded_len<V>(values) + (size_t)table);
}

template <typename T, int FAM, int VPT, int MAXT, bool G>
void configure_one()
{
    cudaFuncSetAttribute(k_rows_r2c<T, FAM, VPT, MAXT, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    cudaFuncSetAttribute(k_rows_c2r<T, FAM, VPT, MAXT, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    cudaFuncSetAttribute(k_cols<T, FAM, VPT, MAXT, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
}

// every (type, family, shape, global table) instantiation the launchers below dispatch to;
// the global-table kernels serve the longest lengths, whose table and data outgrow shared memory
#define CMM_FFT_SHAPES(X)                                                                                  \
    X(float, kPow2, 4, 1024, false) X(float, kPow2x3, 4, 1024, false)                                      \
    X(float, kPow2, 8, 1024, false) X(float, kPow2x3, 8, 1024, false) X(float, kAny, 16, 256, false)        \
    X(float, kAny, 32, 256, false) X(double, kPow2, 8, 512, false) X(double, kPow2, 16, 512, false)         \
    X(double, kPow2x3, 8, 512, false) X(double, kPow2x3, 16, 512, false) X(double, kAny, 16, 256, false)   \
    X(double, kAny, 32, 256, false) X(double, kPow2, 16, 512, true) X(double, kPow2x3, 16, 512, true)       \
    X(double, kAny, 32, 256, true) X(float, kPow2, 8, 1024, true) X(float, kPow2x3, 8, 1024, true)

void configure()
{
#define X(T, F, V, M, G) configure_one<T, F, V, M, G>();
    CMM_FFT_SHAPES(X)
#undef X
#define X(N)                                                                                        \
    cudaFuncSetAttribute(k_rows_r2c_s<N, kStaticGT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    CMM_FFT_STATIC_ROWS(X)
#undef X
}

// shared memory of k_rows_r2c_s<N, GT> with nb rows per group
size_t static_rows_smem(int n, int nb, bool gt)
{
    const size_t len = (size_t)((padded_len<float2>(nb * n) + 1) & ~1);
    return sizeof(float2) * (3 * len + (gt ? 0 : (size_t)sp_tlen_pow2(n) + (size_t)n + 1));
}

// the static FP32 R2C kernel of packed length n (cudaErrorInvalidValue when there is none)
cudaError_t launch_rows_static(int n, long long groups, size_t sm, cudaStream_t s, const RowsArgs& a)
{
#define X(N)                                                                                           \
    if (n == N) {                                                                                      \
        const void* f = reinterpret_cast<const void*>(k_rows_r2c_s<N, kStaticGT>);                     \
        return launch_pdl(k_rows_r2c_s<N, kStaticGT>, resident_grid(f, kStaticThreads, sm, groups), kStaticThreads, \
                          sm, s, a);                                                                   \
    }
    CMM_FFT_STATIC_ROWS(X)
#undef X
    return cudaErrorInvalidValue;
}

bool has_static_rows(int n)
{
#define X(N) if (n == N) return true;
    CMM_FFT_STATIC_ROWS(X)
#undef X
    return false;
}

template <typename T>
bool launch_rows(int fam, const Shape& sh, bool gtw, bool forward, long long groups, int thr, size_t sm, cudaStream_t s,
                 const RowsArgs& a)
{
#define X(TT, F, V, M, G)                                                                               \
    if (std::is_same<T, TT>::value && fam == F && sh.vpt == V && sh.maxt == M && gtw == G) {           \
        if (forward) {                                                                                  \
            const void* f = reinterpret_cast<const void*>(k_rows_r2c<T, F, V, M, G>);                    \
            k_rows_r2c<T, F, V, M, G><<<resident_grid(f, thr, sm, groups), thr, sm, s>>>(a);             \
        } else {                                                                                        \
            const void* f = reinterpret_cast<const void*>(k_rows_c2r<T, F, V, M, G>);                    \
            k_rows_c2r<T, F, V, M, G><<<resident_grid(f, thr, sm, groups), thr, sm, s>>>(a);             \
        }                                                                                               \
        return true;                                                                                    \
    }
    CMM_FFT_SHAPES(X)
#undef X
    return false;
}

template <typename T>
bool launch_cols(int fam, const Shape& sh, bool gtw, long long groups, int thr, size_t sm, cudaStream_t s,
                 const ColsArgs& a)
{
#define X(TT, F, V, M, G)                                                                               \
    if (std::is_same<T, TT>::value && fam == F && sh.vpt == V && sh.maxt == M && gtw == G) {           \
        const void* f = reinterpret_cast<const void*>(k_cols<T, F, V, M, G>);                            \
        k_cols<T, F, V, M, G><<<resident_grid(f, thr, sm, groups), thr, sm, s>>>(a);                     \
        return true;                                                                                    \
    }
    CMM_FFT_SHAPES(X)
#undef X
    return false;
}

// exp(-2 pi i j / n), computed in long double and rounded once
template <typename V, typename T>
V root(long long j, long long n)
{
    const long double two_pi = 6.283185307179586476925286766559005768L;
    const long double a = two_pi * (long double)(j % n) / (long double)n;
    V v;
    v.x = (T)std::cos(a);
    v.y = (T)-std::sin(a);
    return v;
}

// the pass twiddles of plan P (RadixPlan::toff layout), then, for a row plan, W^k =
// exp(-2 pi i k / (2n)) for k <= n (the real packing)
template <typename V, typename T>
void* upload_table(const RadixPlan& P, bool post, cudaStream_t s)
{
    const int n = P.n;
    // (at least one entry: a one-point plan has no passes but still gets a valid table)
    std::vector<V> h(std::max<size_t>(1, (size_t)P.tlen + (post ? (size_t)n + 1 : 0)));
    int span = 1;
    for (int q = 0; q < P.np; ++q) {
        const int R = P.r[q];
        V* t = h.data() + P.toff[q];
        for (int k = 0; k < span; ++k)
            for (int r = 1; r < R; ++r) t[k * (R - 1) + r - 1] = root<V, T>((long long)r * k * (n / (span * R)), n);
        if (R != 2 && R != 3 && R != 4 && R != 8)
            for (int m = 0; m < R; ++m) t[span * (R - 1) + m] = root<V, T>((long long)m * (n / R), n);
        span *= R;
    }
    if (post)
        for (int k = 0; k <= n; ++k) h[(size_t)P.tlen + (size_t)k] = root<V, T>(k, 2ll * n);
    void* d = nullptr;
    if (cudaMalloc(&d, sizeof(V) * h.size()) != cudaSuccess) return nullptr;
    if (cudaMemcpyAsync(d, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

}  // namespace

int resident_grid(const void* func, int threads, size_t smem, long long groups)
{
    static int sms = 0;
    if (sms == 0) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        sms = cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0 ? v : 152;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const long long g = (long long)per_sm * sms;
    return (int)(groups < g ? groups : g);
}

bool make_radix_plan(int n, RadixPlan& p)
{
    p = RadixPlan{};
    p.n = n;
    if (n < 1 || n > kMaxLen) return false;
    int m = n;
    std::vector<int> rs;
    while (m % 8 == 0) { rs.push_back(8); m /= 8; }
    if (m % 4 == 0) { rs.push_back(4); m /= 4; }
    if (m % 2 == 0) {
        // 8 * 2 -> 4 * 4: a radix-2 pass has the most butterflies per thread
        if (!rs.empty() && rs.back() == 8) { rs.back() = 4; rs.push_back(4); }
        else rs.push_back(2);
        m /= 2;
    }
    for (int q : {3, 5, 7, 11, 13})
        while (m % q == 0) { rs.push_back(q); m /= q; }
    if (m != 1 || (int)rs.size() > kMaxPasses) return false;
    p.np = (int)rs.size();
    const bool pow2 = (n & (n - 1)) == 0;
    auto lg = [](int v) { int l = 0; while ((1 << l) < v) ++l; return l; };
    int span = 1, off = 0;
    for (int i = 0; i < p.np; ++i) {
        const int R = rs[(size_t)i];
        p.r[i] = (unsigned char)R;
        p.lnr[i] = (unsigned char)(pow2 ? lg(n / R) : 0);
        p.lp[i] = (unsigned char)(pow2 ? lg(span) : 0);
        p.toff[i] = off;
        off += span * (R - 1) + (R == 2 || R == 3 || R == 4 || R == 8 ? 0 : R);
        span *= R;
    }
    p.tlen = off;
    return true;
}

bool supported_length(int n)
{
    RadixPlan p;
    return make_radix_plan(n, p);
}

int plan_create(Plan2D& p, int nx, int ny, bool dbl, cudaStream_t s)
{
    plan_destroy(p);
    if (nx < 2 || nx % 2 != 0 || ny < 1) return -1;
    Plan2D q;
    q.nx = nx; q.ny = ny; q.dbl = dbl;
    if (!make_radix_plan(nx / 2, q.rx) || !make_radix_plan(ny, q.ry)) return -1;
    configure();
    q.twx = dbl ? upload_table<double2, double>(q.rx, true, s) : upload_table<float2, float>(q.rx, true, s);
    q.twy = dbl ? upload_table<double2, double>(q.ry, false, s) : upload_table<float2, float>(q.ry, false, s);
    if (!q.twx || !q.twy) {
        if (q.twx) cudaFree(q.twx);
        if (q.twy) cudaFree(q.twy);
        return -2;
    }
    p = q;
    return 0;
}

void plan_destroy(Plan2D& p)
{
    if (p.twx) cudaFree(p.twx);
    if (p.twy) cudaFree(p.twy);
    p = Plan2D{};
}

static cudaError_t rows_launch(const Plan2D& p, bool forward, const void* in, long long ild, long long idist, void* out,
                               long long old, long long odist, int rows_per_item, int items, int kio, cudaStream_t s,
                               bool tout = false)
{
    if (!p.ok() || rows_per_item < 1 || items < 1 || kio < 0 || kio > p.nx / 2 + 1) return cudaErrorInvalidValue;
    const int n = p.nx / 2;
    const size_t real_al = p.dbl ? 16 : 8;
    // the real rows are read / written as complex pairs
    const long long rld = forward ? ild : old, rdist = forward ? idist : odist;
    const void* rptr = forward ? in : out;
    if (rld % 2 != 0 || rdist % 2 != 0 || !aligned(rptr, real_al) || !aligned(forward ? out : in, real_al))
        return cudaErrorInvalidValue;
    RowsArgs a;
    a.in = in; a.out = out;
    a.ild = ild; a.idist = idist; a.old = old; a.odist = odist;
    a.rows_per_item = rows_per_item;
    a.rows_total = rows_per_item * items;
    a.kio = kio;
    a.tout = 0;
    const bool stat = forward && !p.dbl && has_static_rows(n) && sp::matches(n, p.rx) && aligned(in, 16) &&
                      ild % 4 == 0 && idist % 4 == 0;
    // column-major output: the static kernel, one item, 16-byte aligned row pairs
    if (tout && (!stat || items != 1 || old % 2 != 0 || old < rows_per_item || !aligned(out, 16)))
        return cudaErrorInvalidValue;
    if (stat) {
        a.tout = tout ? 1 : 0;
        a.nb = kStaticThreads * kStaticVPT / n;
        a.P = p.rx;
        a.tw = p.twx;
        const long long groups = (a.rows_total + a.nb - 1) / a.nb;
        return launch_rows_static(n, groups, static_rows_smem(n, a.nb, kStaticGT), s, a);
    }
    // rows per group: about kBlockValues values, at least one row
    const int fam = family_of(p.rx);
    a.nb = n >= kBlockValues ? 1 : kBlockValues / n;
    if (a.nb > a.rows_total) a.nb = a.rows_total;
    const Shape sh = shape_for(p.dbl, fam, a.nb * n);
    if (a.nb * n > sh.vpt * sh.maxt) return cudaErrorInvalidValue;
    a.P = p.rx;
    a.tw = p.twx;
    const int thr = threads_for(a.nb * n, sh);
    const long long groups = (a.rows_total + a.nb - 1) / a.nb;
    // with its table staged the forward kernel double-buffers its rows (cp.async of the next
    // group); when that does not fit, one buffer and the table in global memory
    // (the FP32 forward kernel adds a ping-pong scratch buffer: block_fft_pp)
    const int tl = p.rx.tlen + n + 1;
    const size_t data = p.dbl ? smem_bytes<double>(a.nb * n, 0) : smem_bytes<float>(a.nb * n, 0);
    const int pp = forward && !p.dbl ? 1 : 0;
    const size_t full = data * (forward ? 2 + pp : 1) + (p.dbl ? sizeof(double2) : sizeof(float2)) * (size_t)tl;
    const bool gtw = full > (size_t)kMaxSmem;
    const size_t sm = gtw ? data * (1 + pp) : full;
    if (sm > (size_t)kMaxSmem) return cudaErrorInvalidValue;
    const bool ok = p.dbl ? launch_rows<double>(fam, sh, gtw, forward, groups, thr, sm, s, a)
                          : launch_rows<float>(fam, sh, gtw, forward, groups, thr, sm, s, a);
    return ok ? cudaGetLastError() : cudaErrorInvalidValue;
}

cudaError_t rows_r2c(const Plan2D& p, const void* in, long long ild, long long idist, void* out, long long old,
                     long long odist, int rows_per_item, int items, int kout, cudaStream_t s)
{
    return rows_launch(p, true, in, ild, idist, out, old, odist, rows_per_item, items, kout, s);
}

cudaError_t rows_r2c_t(const Plan2D& p, const void* in, long long ild, void* out, long long ocol, int rows, int kout,
                       cudaStream_t s)
{
    return rows_launch(p, true, in, ild, 0, out, ocol, 0, rows, 1, kout, s, true);
}

bool rows_r2c_t_supported(const Plan2D& p)
{
    const int n = p.nx / 2;
    return p.ok() && !p.dbl && has_static_rows(n) && sp::matches(n, p.rx);
}

cudaError_t rows_c2r(const Plan2D& p, const void* in, long long ild, long long idist, int kin, void* out,
                     long long old, long long odist, int rows_per_item, int items, cudaStream_t s)
{
    return rows_launch(p, false, in, ild, idist, out, old, odist, rows_per_item, items, kin, s);
}

cudaError_t cols_c2c(const Plan2D& p, void* data, long long ld, long long bdist, int ncols, int batch, bool inverse,
                     cudaStream_t s)
{
    if (!p.ok() || ncols < 1 || batch < 1) return cudaErrorInvalidValue;
    if (p.ny == 1) return cudaSuccess;
    const int n = p.ny;
    // C adjacent columns per group (32-byte row segments) while a group stays near
    // kBlockValues values
    const int fam = family_of(p.ry);
    int C = p.dbl ? 2 : 4;
    while (C > 1 && C * n > kBlockValues) C /= 2;
    const Shape sh = shape_for(p.dbl, fam, C * n);
    if (C * n > sh.vpt * sh.maxt) return cudaErrorInvalidValue;
    ColsArgs a;
    a.data = data; a.ld = ld; a.bdist = bdist; a.ncols = ncols; a.C = C; a.batch = batch; a.inv = inverse ? 1 : 0;
    a.lc = C == 4 ? 2 : (C == 2 ? 1 : 0);
    a.P = p.ry;
    a.tw = p.twy;
    const long long groups = (long long)((ncols + C - 1) / C) * batch;
    const int thr = threads_for(C * n, sh);
    const size_t full = p.dbl ? smem_bytes<double>(C * n, p.ry.tlen) : smem_bytes<float>(C * n, p.ry.tlen);
    const bool gtw = full > (size_t)kMaxSmem;
    const size_t sm = gtw ? (p.dbl ? smem_bytes<double>(C * n, 0) : smem_bytes<float>(C * n, 0)) : full;
    const bool ok = p.dbl ? launch_cols<double>(fam, sh, gtw, groups, thr, sm, s, a)
                          : launch_cols<float>(fam, sh, gtw, groups, thr, sm, s, a);
    return ok ? cudaGetLastError() : cudaErrorInvalidValue;
}

cudaError_t r2c(const Plan2D& p, const void* in, void* out, int batch, cudaStream_t s, long long idist, long long odist)
{
    const long long nxf = p.nx / 2 + 1;
    if (idist == 0) idist = (long long)p.nx * p.ny;
    if (odist == 0) odist = nxf * p.ny;
    cudaError_t e = rows_r2c(p, in, p.nx, idist, out, nxf, odist, p.ny, batch, (int)nxf, s);
    if (e != cudaSuccess) return e;
    return cols_c2c(p, out, nxf, odist, (int)nxf, batch, false, s);
}

cudaError_t c2r(const Plan2D& p, void* in, void* out, int batch, cudaStream_t s, long long idist, long long odist)
{
    const long long nxf = p.nx / 2 + 1;
    if (idist == 0) idist = nxf * p.ny;
    if (odist == 0) odist = (long long)p.nx * p.ny;
    cudaError_t e = cols_c2c(p, in, nxf, idist, (int)nxf, batch, true, s);
    if (e != cudaSuccess) return e;
    return rows_c2r(p, in, nxf, idist, (int)nxf, out, p.nx, odist, p.ny, batch, s);
}

}  // namespace fft
}  // namespace cmm
