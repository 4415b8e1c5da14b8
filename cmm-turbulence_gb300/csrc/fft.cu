// fft.cu -- batched real / complex transforms on the library's own Stockham engine
// (fft.cuh): the row pass (R2C or C2R of whole rows, one block per few rows) and the
// column pass (in-place complex transforms of C adjacent columns per block).
#include <cmath>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "fft.hpp"

namespace cmm {
namespace fft {

namespace {

// Block shapes: VPT values per thread, at most MAXT threads (launch bound with one block
// per SM, so up to 65536 / MAXT registers).  Power-of-two (and 3 * 2^k) lengths run 512
// threads of 8 (FP64) or 16 (FP32) values, which keeps an FP64 radix-8 butterfly and its
// inputs in registers; FP64 transforms longer than 4096 use 16 values per thread; lengths
// with larger prime factors run 256 threads (registers for the generic butterflies).
struct Shape { int vpt, maxt; };
constexpr int kMaxSmem = 200 * 1024;    // dynamic shared memory the kernels may request

struct RowsArgs {
    const void* in;
    void* out;
    long long ild, idist, old, odist;   // in elements of the input / output type
    int rows_per_item, rows_total;
    int kio;                            // R2C: bins written; C2R: bins read (the rest zero)
    int nb;                             // rows per block
    RadixPlan P;                        // packed complex length nx/2
    const void* tw;                     // nx entries
};

struct ColsArgs {
    void* data;
    long long ld, bdist;                // complex elements
    int ncols, C;                       // columns, columns per block
    int inv;
    RadixPlan P;                        // length ny
    const void* tw;                     // ny entries
};

template <typename T, int FAM, int VPT, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) k_rows_r2c(RowsArgs a)
{
    using V = typename Cx<T>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* s = reinterpret_cast<V*>(smem_raw);
    const V* tw = reinterpret_cast<const V*>(a.tw);
    const int n = a.P.n;
    const int row0 = blockIdx.x * a.nb;
    const int nb = min(a.nb, a.rows_total - row0);
    for (int e = threadIdx.x; e < nb * n; e += blockDim.x) {
        const int b = e / n, m = e - b * n;
        const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
        const T* src = reinterpret_cast<const T*>(a.in) + item * a.idist + r * a.ild;
        s[pad<V>(e)] = reinterpret_cast<const V*>(src)[m];
    }
    __syncthreads();
    block_fft<VPT, FAM>(s, nb, a.P, tw, 2, false);
    for (int e = threadIdx.x; e < nb * a.kio; e += blockDim.x) {
        const int b = e / a.kio, k = e - b * a.kio;
        const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
        V* dst = reinterpret_cast<V*>(a.out) + item * a.odist + r * a.old;
        dst[k] = r2c_bin(s, b * n, n, k, tw);
    }
}

template <typename T, int FAM, int VPT, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) k_rows_c2r(RowsArgs a)
{
    using V = typename Cx<T>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* s = reinterpret_cast<V*>(smem_raw);
    const V* tw = reinterpret_cast<const V*>(a.tw);
    const int n = a.P.n;
    const int row0 = blockIdx.x * a.nb;
    const int nb = min(a.nb, a.rows_total - row0);
    const V zero = mk((T)0, (T)0);
    for (int e = threadIdx.x; e < nb * n; e += blockDim.x) {
        const int b = e / n, k = e - b * n;
        const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
        const V* src = reinterpret_cast<const V*>(a.in) + item * a.idist + r * a.ild;
        V xk = k < a.kio ? src[k] : zero;
        V xn = n - k < a.kio ? src[n - k] : zero;
        if (k == 0) { xk.y = (T)0; xn.y = (T)0; }
        s[pad<V>(e)] = c2r_pack(xk, xn, k, tw);
    }
    __syncthreads();
    block_fft<VPT, FAM>(s, nb, a.P, tw, 2, true);
    for (int e = threadIdx.x; e < nb * n; e += blockDim.x) {
        const int b = e / n, m = e - b * n;
        const int g = row0 + b, item = g / a.rows_per_item, r = g - item * a.rows_per_item;
        T* dst = reinterpret_cast<T*>(a.out) + item * a.odist + r * a.old;
        reinterpret_cast<V*>(dst)[m] = s[pad<V>(e)];
    }
}

template <typename T, int FAM, int VPT, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) k_cols(ColsArgs a)
{
    using V = typename Cx<T>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* s = reinterpret_cast<V*>(smem_raw);
    const int n = a.P.n, C = a.C;
    const int col0 = blockIdx.x * C;
    const int cn = min(C, a.ncols - col0);
    V* base = reinterpret_cast<V*>(a.data) + blockIdx.y * a.bdist + col0;
    for (int e = threadIdx.x; e < C * n; e += blockDim.x) {
        const int c = e % C, r = e / C;
        s[pad<V>(c * n + r)] = c < cn ? base[r * a.ld + c] : mk((T)0, (T)0);
    }
    __syncthreads();
    block_fft<VPT, FAM>(s, C, a.P, reinterpret_cast<const V*>(a.tw), 1, a.inv != 0);
    for (int e = threadIdx.x; e < C * n; e += blockDim.x) {
        const int c = e % C, r = e / C;
        if (c < cn) base[r * a.ld + c] = s[pad<V>(c * n + r)];
    }
}

Shape shape_for(bool dbl, int fam, int values)
{
    if (fam == kAny) return values <= 16 * 256 ? Shape{16, 256} : Shape{32, 256};
    if (!dbl) return Shape{16, 512};
    return values <= 8 * 512 ? Shape{8, 512} : Shape{16, 512};
}

int threads_for(int values, const Shape& sh)
{
    int t = (values + sh.vpt - 1) / sh.vpt;
    t = (t + 31) / 32 * 32;
    return t < 32 ? 32 : (t > sh.maxt ? sh.maxt : t);
}

template <typename T>
size_t smem_bytes(int values)
{
    using V = typename Cx<T>::V;
    return sizeof(V) * (size_t)padded_len<V>(values);
}

template <typename T, int FAM, int VPT, int MAXT>
void configure_one()
{
    cudaFuncSetAttribute(k_rows_r2c<T, FAM, VPT, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    cudaFuncSetAttribute(k_rows_c2r<T, FAM, VPT, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    cudaFuncSetAttribute(k_cols<T, FAM, VPT, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
}

// every (type, family, shape) instantiation the launchers below dispatch to
#define CMM_FFT_SHAPES(X)                                                                                  \
    X(float, kPow2, 16, 512) X(float, kPow2x3, 16, 512) X(float, kAny, 16, 256) X(float, kAny, 32, 256)    \
    X(double, kPow2, 8, 512) X(double, kPow2, 16, 512) X(double, kPow2x3, 8, 512)                         \
    X(double, kPow2x3, 16, 512) X(double, kAny, 16, 256) X(double, kAny, 32, 256)

void configure()
{
#define X(T, F, V, M) configure_one<T, F, V, M>();
    CMM_FFT_SHAPES(X)
#undef X
}

template <typename T>
void launch_rows(int fam, const Shape& sh, bool forward, unsigned blocks, int thr, size_t sm, cudaStream_t s,
                 const RowsArgs& a)
{
#define X(TT, F, V, M)                                                                                  \
    if (std::is_same<T, TT>::value && fam == F && sh.vpt == V && sh.maxt == M) {                       \
        if (forward) k_rows_r2c<T, F, V, M><<<blocks, thr, sm, s>>>(a);                                 \
        else k_rows_c2r<T, F, V, M><<<blocks, thr, sm, s>>>(a);                                         \
        return;                                                                                         \
    }
    CMM_FFT_SHAPES(X)
#undef X
}

template <typename T>
void launch_cols(int fam, const Shape& sh, dim3 grid, int thr, size_t sm, cudaStream_t s, const ColsArgs& a)
{
#define X(TT, F, V, M)                                                                                  \
    if (std::is_same<T, TT>::value && fam == F && sh.vpt == V && sh.maxt == M) {                       \
        k_cols<T, F, V, M><<<grid, thr, sm, s>>>(a);                                                    \
        return;                                                                                         \
    }
    CMM_FFT_SHAPES(X)
#undef X
}

// exp(-2 pi i t / len) for t < len, computed in long double and rounded once
template <typename V, typename T>
std::vector<V> table(int len)
{
    std::vector<V> h((size_t)len);
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int t = 0; t < len; ++t) {
        long double a = two_pi * (long double)t / (long double)len;
        h[(size_t)t].x = (T)std::cos(a);
        h[(size_t)t].y = (T)-std::sin(a);
    }
    return h;
}

template <typename V, typename T>
void* upload_table(int len, cudaStream_t s)
{
    std::vector<V> h = table<V, T>(len);
    void* d = nullptr;
    if (cudaMalloc(&d, sizeof(V) * (size_t)len) != cudaSuccess) return nullptr;
    if (cudaMemcpyAsync(d, h.data(), sizeof(V) * (size_t)len, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

}  // namespace

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
    for (int i = 0; i < p.np; ++i) p.r[i] = (unsigned char)rs[(size_t)i];
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
    q.twx = dbl ? upload_table<double2, double>(nx, s) : upload_table<float2, float>(nx, s);
    q.twy = dbl ? upload_table<double2, double>(ny, s) : upload_table<float2, float>(ny, s);
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
                               long long old, long long odist, int rows_per_item, int items, int kio, cudaStream_t s)
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
    // rows per block: about 4096 values, at least one row
    const int fam = family_of(p.rx);
    a.nb = n >= 4096 ? 1 : 4096 / n;
    if (a.nb > a.rows_total) a.nb = a.rows_total;
    const Shape sh = shape_for(p.dbl, fam, a.nb * n);
    if (a.nb * n > sh.vpt * sh.maxt) return cudaErrorInvalidValue;
    a.P = p.rx;
    a.tw = p.twx;
    const int thr = threads_for(a.nb * n, sh);
    const unsigned blocks = (unsigned)((a.rows_total + a.nb - 1) / a.nb);
    if (p.dbl) launch_rows<double>(fam, sh, forward, blocks, thr, smem_bytes<double>(a.nb * n), s, a);
    else launch_rows<float>(fam, sh, forward, blocks, thr, smem_bytes<float>(a.nb * n), s, a);
    return cudaGetLastError();
}

cudaError_t rows_r2c(const Plan2D& p, const void* in, long long ild, long long idist, void* out, long long old,
                     long long odist, int rows_per_item, int items, int kout, cudaStream_t s)
{
    return rows_launch(p, true, in, ild, idist, out, old, odist, rows_per_item, items, kout, s);
}

cudaError_t rows_c2r(const Plan2D& p, const void* in, long long ild, long long idist, int kin, void* out,
                     long long old, long long odist, int rows_per_item, int items, cudaStream_t s)
{
    return rows_launch(p, false, in, ild, idist, out, old, odist, rows_per_item, items, kin, s);
}

cudaError_t cols_c2c(const Plan2D& p, void* data, long long ld, long long bdist, int ncols, int batch, bool inverse,
                     cudaStream_t s)
{
    if (!p.ok() || ncols < 1 || batch < 1 || batch > 65535) return cudaErrorInvalidValue;
    if (p.ny == 1) return cudaSuccess;
    const int n = p.ny;
    // C adjacent columns per block: 32-byte row segments where shared memory allows
    // C adjacent columns per block: 32-byte row segments where the block can hold them
    const int fam = family_of(p.ry);
    int C = p.dbl ? 2 : 4;
    while (C > 1 && (C * n > 4096 || (p.dbl ? smem_bytes<double>(C * n) : smem_bytes<float>(C * n)) > 100 * 1024))
        C /= 2;
    const Shape sh = shape_for(p.dbl, fam, C * n);
    if (C * n > sh.vpt * sh.maxt) return cudaErrorInvalidValue;
    ColsArgs a;
    a.data = data; a.ld = ld; a.bdist = bdist; a.ncols = ncols; a.C = C; a.inv = inverse ? 1 : 0;
    a.P = p.ry;
    a.tw = p.twy;
    dim3 grid((unsigned)((ncols + C - 1) / C), (unsigned)batch);
    const int thr = threads_for(C * n, sh);
    if (p.dbl) launch_cols<double>(fam, sh, grid, thr, smem_bytes<double>(C * n), s, a);
    else launch_cols<float>(fam, sh, grid, thr, smem_bytes<float>(C * n), s, a);
    return cudaGetLastError();
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
