// learned_kernels.cu -- BF16 tcgen05 convolution kernels of the learned psi upsampler and
// the elementwise steps around them (see learned.hpp for the layouts).
//
// Forward / input-gradient convolution (k_conv3x3<CIN, COUT>): a persistent warp-specialised
// kernel, one CTA per SM, over strips of rows of 128-pixel column segments.  Each source row
// is staged once with cp.async as [channel chunk of 8][pixel 0..129][8 channels]: a K-major
// operand whose 8-pixel core matrices are 128 contiguous bytes, so the tap with column offset
// dx is the same slot addressed dx * 16 bytes further.  One source row meets all three kernel
// rows in the same MMAs (M = 128 pixels, N = 3 COUT (dy, co), K = 16): its accumulator in TMEM
// holds its contribution to three output rows, and the epilogue sums the matching column
// blocks of three consecutive accumulators and fuses bias, ReLU, the ReLU mask of the
// backward pass and the residual add (details at the kernel).
//
// Weight gradient (k_conv3x3_dw<CIN, COUT>): dW[(dy, dx, ci)][co] = sum over pixels of
// x[p + (dy - 1, dx - 1)][ci] dy[p][co], a GEMM with K = pixels.  Each staged input row
// is transposed into three K-major copies shifted by dx (M = (dx, ci), padded to 128),
// the output-gradient row into one of two K-major tiles, and three accumulators (one per dy)
// stay in TMEM across the CTA's whole strip; a row's MMAs run while the next row is staged;
// the per-CTA partials are summed in a fixed order by k_dw_reduce.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "learned.hpp"
#include "tc_sm100.cuh"

namespace cmm {
namespace lrn {

namespace {

constexpr long long kMaxPolls = 1ll << 22;   // ~0.2 s of polling before a wait gives up
constexpr long long kMaxTries = 1ll << 20;   // try_wait rounds (each suspends for at most a few us)

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ int src_row(int r, int d, int H)
{
    const int img = r / H;
    int y = r - img * H + d;
    y = y < 0 ? y + H : (y >= H ? y - H : y);
    return img * H + y;
}

__device__ __forceinline__ uint32_t word_of(const uint4& v, int k)
{
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// in[j] = 8 BF16 values (elements e = 0..7) of row j; out[e] = element e of rows 0..7
__device__ __forceinline__ void transpose8(const uint4 (&in)[8], uint4 (&out)[8])
{
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const uint32_t sel = (e & 1) ? 0x7632u : 0x5410u;
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) w[q] = __byte_perm(word_of(in[2 * q], e >> 1), word_of(in[2 * q + 1], e >> 1), sel);
        out[e] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

__device__ __forceinline__ void unpack8(const uint4& v, float (&f)[8])
{
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float2 t = __bfloat1622float2(h[q]);
        f[2 * q] = t.x;
        f[2 * q + 1] = t.y;
    }
}

__device__ __forceinline__ uint4 pack8(const float* f)
{
    uint4 v;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&v);
#pragma unroll
    for (int q = 0; q < 4; ++q) h[q] = __floats2bfloat162_rn(f[2 * q], f[2 * q + 1]);
    return v;
}

// ---------------------------------------------------------------------------
// forward / input-gradient convolution
// ---------------------------------------------------------------------------
// Warp-specialised persistent kernel, one CTA per SM (it holds the whole tensor memory).
// Work items ("tasks") are strips of at most rows_per_cta rows of one 128-pixel column
// segment inside one image; a strip of n rows reads the n + 2 source rows r0 - 1 .. r0 + n
// (wrapped periodically inside the image).  Each source row k is multiplied once by all
// three kernel rows dy at a time: N = 3 COUT columns (dy, co), so an MMA reads its 4 KB
// pixel tile for 96 output columns rather than 32,
//   D_k[p][dy COUT + co] = sum_{dx, ci} x_k[p + dx - 1][ci] w[dy][dx][ci][co],
// and output row j of the strip is D_j[., 0 : COUT] + D_{j+1}[., COUT : 2 COUT] +
// D_{j+2}[., 2 COUT : 3 COUT].  CTA b takes tasks b, b + grid, ...
//   warp 0      producer: stages each source row into a ring of kConvSlots row slots with
//               cp.async; each lane's copies arrive on the slot's "full" barrier when they
//               land (cp.async.mbarrier.arrive);
//   warp 1      one lane issues a source row's 3 x CIN/16 MMAs into one of kConvAcc TMEM
//               accumulators (after a proxy fence for the staged row), then commits to the
//               row slot's "empty" barrier and the accumulator's "full" barrier;
//   warps 2-9   epilogue, two groups of four warps taking alternate output rows: load the
//               row's ReLU mask and residual, wait for its three accumulators, read their
//               column blocks (warp w owns TMEM lanes 32 (w % 4) ..), arrive on each one's
//               "empty" barrier, and apply bias, ReLU, mask, residual and the stores.  An
//               accumulator is free once all its reader rows arrived: 3 x 128 arrivals, the
//               last reader of a strip-edge source row (fewer than three readers) arriving
//               for the missing ones.
// Every wait is bounded: a wait that runs out ends the kernel's loops and sets *status.
constexpr int kConvSlots = 8;       // staged source rows
constexpr int kConvAcc = 5;         // source-row accumulators in TMEM (3 live + 2 ahead)
constexpr int kConvAccCols = 96;    // 3 COUT columns each (COUT <= 32)
constexpr int kConvTmemCols = 512;
constexpr int kConvGroups = 2;      // epilogue groups
constexpr int kConvThreads = 64 + 128 * kConvGroups;
constexpr int kConvMinSmem = 120 * 1024;   // keeps a second CTA (and its TMEM request) off the SM
static_assert(kConvAcc * kConvAccCols <= kConvTmemCols, "accumulators exceed the TMEM allocation");
static_assert(kConvAcc >= 4, "three live accumulators and one being written");

struct ConvTask {
    int x0, r0, nr;
};

__device__ __forceinline__ int conv_tasks(const ConvArgs& a)
{
    const int per_img = (a.H + a.rows_per_cta - 1) / a.rows_per_cta;
    return (a.W / kTile) * (a.rows / a.H) * per_img;
}

__device__ __forceinline__ ConvTask conv_task(const ConvArgs& a, int t)
{
    const int segs = a.W / kTile;
    const int per_img = (a.H + a.rows_per_cta - 1) / a.rows_per_cta;
    const int strip = t / segs;
    const int img = strip / per_img, k = strip - img * per_img;
    ConvTask c;
    c.x0 = (t - strip * segs) * kTile;
    c.r0 = img * a.H + k * a.rows_per_cta;
    c.nr = min(a.rows_per_cta, a.H - k * a.rows_per_cta);
    return c;
}

// the barrier receives this thread's arrival when all its earlier cp.async copies have landed
// (the arrival counts against the barrier's expected count: no increment)
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar)
{
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar, uint32_t count)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(tc::smem_u32(bar)),
                 "r"(count)
                 : "memory");
}

// arrivals output row j of an n-row strip makes on the accumulator of its source row k
// (k = j .. j + 2): 1, plus, from k's last reader, one for each reader k lacks
__device__ __forceinline__ uint32_t conv_arrivals(int j, int k, int n)
{
    const int lo = k - 2 > 0 ? k - 2 : 0, hi = k < n - 1 ? k : n - 1;
    return j == hi ? 1u + (uint32_t)(3 - (hi - lo + 1)) : 1u;
}

// D (TMEM, 3 COUT columns) = the staged source row times all 9 taps; weights in shared
// memory as [dx][ci / 8][dy][co][8]
template <int CIN, int COUT>
__device__ __forceinline__ void conv_issue(uint32_t d_tmem, uint32_t row, uint32_t wbase)
{
    constexpr int C8 = CIN / 8;
    constexpr uint32_t idesc = tc::idesc_bf16(128, 3 * COUT);
    uint32_t acc = 0;
#pragma unroll
    for (int dx = 0; dx < 3; ++dx)
#pragma unroll
        for (int kk = 0; kk < CIN / 16; ++kk) {
            const uint32_t aaddr = row + ((2 * kk) * kPitch + dx) * 16;
            const uint32_t baddr = wbase + ((dx * C8 + 2 * kk) * 3 * COUT) * 16;
            tc::mma_bf16(d_tmem, tc::desc_kmajor(aaddr, kPitch * 16, 128), tc::desc_kmajor(baddr, 3 * COUT * 16, 128),
                         idesc, acc);
            acc = 1;
        }
}

// a staged row is C8 x kPitch 16-byte chunks ([ci / 8][pixel][8]); lane l copies chunks
// l, l + 32, ...: their byte offsets inside the source row (periodic in x) depend on the
// segment only
template <int CIN>
struct StageMap {
    static constexpr int C8 = CIN / 8;
    static constexpr int kChunks = C8 * kPitch;
    static constexpr int kPer = (kChunks + 31) / 32;
    uint32_t src[kPer];
};

template <int CIN>
__device__ __forceinline__ void stage_map(StageMap<CIN>& m, int W, int x0, int lane)
{
    constexpr int C8 = CIN / 8;
#pragma unroll
    for (int k = 0; k < StageMap<CIN>::kPer; ++k) {
        const int i = lane + 32 * k;
        const int c = i % C8, p = i / C8;
        int x = x0 - 1 + p;
        x = x < 0 ? x + W : (x >= W ? x - W : x);
        m.src[k] = (uint32_t)(x * CIN + c * 8) * 2u;
    }
}

template <int CIN>
__device__ __forceinline__ void conv_stage_warp(unsigned char* dst, const bf16* __restrict__ in, int src, int W,
                                                const StageMap<CIN>& m, int lane)
{
    constexpr int C8 = CIN / 8;
    const unsigned char* row = reinterpret_cast<const unsigned char*>(in + (long long)src * W * CIN);
#pragma unroll
    for (int k = 0; k < StageMap<CIN>::kPer; ++k) {
        const int i = lane + 32 * k;
        if (k + 1 < StageMap<CIN>::kPer || i < StageMap<CIN>::kChunks)
            cp_async16(dst + ((i % C8) * kPitch + i / C8) * 16, row + m.src[k]);
    }
}

// the ReLU mask and residual of one output row at this thread's pixel (zero when absent)
template <int COUT>
__device__ __forceinline__ void conv_extra(const ConvArgs& a, int r, int x0, int q4, int lane, uint4 (&mk)[COUT / 8],
                                           uint4 (&rs)[COUT / 8])
{
    const long long pix = (long long)r * a.W + x0 + q4 * 32 + lane;
#pragma unroll
    for (int q = 0; q < COUT / 8; ++q) {
        mk[q] = a.mask ? reinterpret_cast<const uint4*>(a.mask + pix * COUT)[q] : make_uint4(0, 0, 0, 0);
        rs[q] = a.res ? reinterpret_cast<const uint4*>(a.res + pix * COUT)[q] : make_uint4(0, 0, 0, 0);
    }
}

// epilogue of one output row for the 32 pixels of TMEM lane quarter q4 (v: bias included)
template <int COUT>
__device__ __forceinline__ void conv_store(const ConvArgs& a, float (&v)[COUT], const uint4 (&mk)[COUT / 8],
                                           const uint4 (&rs)[COUT / 8], int r, int x0, int q4, int lane)
{
    const long long pix = (long long)r * a.W + x0 + q4 * 32 + lane;
    if (a.relu) {
#pragma unroll
        for (int j = 0; j < COUT; ++j) v[j] = fmaxf(v[j], 0.f);
    }
    if (a.mask) {
#pragma unroll
        for (int q = 0; q < COUT / 8; ++q) {
            float m[8];
            unpack8(mk[q], m);
#pragma unroll
            for (int e = 0; e < 8; ++e) v[8 * q + e] = m[e] > 0.f ? v[8 * q + e] : 0.f;
        }
    }
    if (a.res) {
#pragma unroll
        for (int q = 0; q < COUT / 8; ++q) {
            float m[8];
            unpack8(rs[q], m);
#pragma unroll
            for (int e = 0; e < 8; ++e) v[8 * q + e] += m[e];
        }
    }
    if (a.out) {
        uint4* op = reinterpret_cast<uint4*>(a.out + pix * COUT);
#pragma unroll
        for (int q = 0; q < COUT / 8; ++q) op[q] = pack8(v + 8 * q);
    }
    if (a.out_f32) {
        float4* op = reinterpret_cast<float4*>(a.out_f32 + pix * COUT);
#pragma unroll
        for (int q = 0; q < COUT / 4; ++q) op[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(kConvThreads, 1) k_conv3x3(ConvArgs a)
{
    constexpr int C8 = CIN / 8;
    constexpr int WB = 9 * C8 * COUT * 16;
    constexpr int SLOT = C8 * kPitch * 16;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t full[kConvSlots], empty[kConvSlots], dfull[kConvAcc], dempty[kConvAcc], done;
    __shared__ uint32_t tslot;
    __shared__ float sbias[COUT];
    unsigned char* sw = sm;
    unsigned char* sr = sm + WB;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ntasks = conv_tasks(a);

    // weights: prepared [dy dx][ci / 8][co][8] -> shared [dx][ci / 8][dy][co][8]
    for (int i = tid; i < WB / 16; i += kConvThreads) {
        const int co = i % COUT, t = i / COUT, dy = t % 3, t2 = t / 3, c8 = t2 % C8, dx = t2 / C8;
        const int gi = ((dy * 3 + dx) * C8 + c8) * COUT + co;
        cp_async16(sw + 16 * i, reinterpret_cast<const unsigned char*>(a.wt) + 16 * (long long)gi);
    }
    if (tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.f;
    if (warp == 1) {
        tc::tmem_alloc(&tslot, kConvTmemCols);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        for (int k = 0; k < kConvSlots; ++k) {
            tc::mbar_init(&full[k], 32);
            tc::mbar_init(&empty[k], 1);
        }
        for (int k = 0; k < kConvAcc; ++k) {
            tc::mbar_init(&dfull[k], 1);
            tc::mbar_init(&dempty[k], 3 * 128);
        }
        tc::mbar_init(&done, 1);
        tc::mbar_fence_init();
    }
    cp_async_wait_all();
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    bool ok = true;

    if (warp == 0) {
        // producer
        uint32_t g = 0;
        StageMap<CIN> map;
        int map_x0 = -1;
        for (int t = blockIdx.x; t < ntasks && ok; t += gridDim.x) {
            const ConvTask c = conv_task(a, t);
            if (c.x0 != map_x0) {
                stage_map<CIN>(map, a.W, c.x0, lane);
                map_x0 = c.x0;
            }
            for (int j = 0; j < c.nr + 2; ++j, ++g) {
                const uint32_t slot = g % kConvSlots, use = g / kConvSlots;
                if (use > 0) ok = tc::mbar_try_wait(&empty[slot], (use - 1) & 1, kMaxTries);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                conv_stage_warp<CIN>(sr + slot * SLOT, a.in, src_row(c.r0, j - 1, a.H), a.W, map, lane);
                cp_async_arrive(&full[slot]);
            }
        }
        cp_async_wait_all();
    } else if (warp == 1) {
        // MMA issue (one lane): one accumulator per source row
        if (lane == 0) {
            const uint32_t wbase = tc::smem_u32(sw), rbase = tc::smem_u32(sr);
            uint32_t g = 0;
            for (int t = blockIdx.x; t < ntasks && ok; t += gridDim.x) {
                const ConvTask c = conv_task(a, t);
                for (int j = 0; j < c.nr + 2; ++j, ++g) {
                    const uint32_t slot = g % kConvSlots, d = g % kConvAcc, use = g / kConvAcc;
                    ok = tc::mbar_try_wait(&full[slot], (g / kConvSlots) & 1, kMaxTries);
                    if (ok && use > 0) ok = tc::mbar_try_wait(&dempty[d], (use - 1) & 1, kMaxTries);
                    if (!ok) break;
                    tc::fence_smem_to_async();   // the staged row (generic proxy) -> the MMAs' operand reads
                    tc::fence_after_sync();
                    conv_issue<CIN, COUT>(tmem + d * kConvAccCols, rbase + slot * SLOT, wbase);
                    tc::mma_commit(&empty[slot]);
                    tc::mma_commit(&dfull[d]);
                }
            }
            // every MMA retired before the tensor memory is released
            tc::mma_commit(&done);
            ok = tc::mbar_try_wait(&done, 0, kMaxTries) && ok;
        }
    } else {
        // epilogue: group e takes the output rows q with q % kConvGroups == e; warps 2.. own TMEM
        // lane quarters (warp % 4)
        const int e = (warp - 2) >> 2, q4 = warp & 3;
        const uint32_t lanes = (uint32_t)(q4 * 32) << 16;
        uint32_t g = 0, q = 0;
        for (int t = blockIdx.x; t < ntasks && ok; t += gridDim.x) {
            const ConvTask c = conv_task(a, t);
            for (int j = 0; j < c.nr; ++j, ++q) {
                if ((int)(q % kConvGroups) != e) continue;
                uint4 mk[COUT / 8], rs[COUT / 8];
                conv_extra<COUT>(a, c.r0 + j, c.x0, q4, lane, mk, rs);
                float v[COUT];
#pragma unroll
                for (int i = 0; i < COUT; ++i) v[i] = sbias[i];
#pragma unroll
                for (int dy = 0; dy < 3; ++dy) {
                    const uint32_t m = g + j + dy, d = m % kConvAcc;
                    ok = __all_sync(0xffffffffu, tc::mbar_try_wait(&dfull[d], (m / kConvAcc) & 1, kMaxTries));
                    if (!ok) break;
                    tc::fence_after_sync();
                    float part[COUT];
                    tc::tmem_ld_cols<COUT>(tmem + lanes + d * kConvAccCols + dy * COUT, part);
#pragma unroll
                    for (int i = 0; i < COUT; ++i) v[i] += part[i];
                }
                if (!ok) break;
                tc::fence_before_sync();
#pragma unroll
                for (int dy = 0; dy < 3; ++dy)
                    mbar_arrive(&dempty[(g + j + dy) % kConvAcc], conv_arrivals(j, j + dy, c.nr));
                conv_store<COUT>(a, v, mk, rs, c.r0 + j, c.x0, q4, lane);
            }
            g += c.nr + 2;
        }
    }
    tc::fence_before_sync();
    if (__syncthreads_or(!ok) && tid == 0 && a.status) atomicExch(a.status, 1);
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, kConvTmemCols);
    }
}

// ---------------------------------------------------------------------------
// weight gradient
// ---------------------------------------------------------------------------
constexpr int kDwThreads = 256;              // staging by all; TMEM read-out by warps 0-3
constexpr int kARows = 129;                  // 128 M rows + 1 pad row per 8-pixel group
constexpr int kASlot = 16 * kARows * 16;     // [pixel group 16][m 129][8 pixels]
template <int COUT>
constexpr int kBTile = 16 * (COUT + 1) * 16;   // [pixel group 16][co + 1][8 pixels]

template <int CIN, int COUT>
__global__ void __launch_bounds__(kDwThreads, 1) k_conv3x3_dw(DwArgs a)
{
    constexpr int C8 = CIN / 8, CO8 = COUT / 8;
    constexpr int BROWS = COUT + 1;
    constexpr uint32_t TCOLS = 3 * COUT <= 64 ? 64 : 128;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tslot;
    __shared__ float red[16 * CO8][8];
    unsigned char* sa = sm;                       // 4 slots
    unsigned char* sb = sm + 4 * kASlot;          // 2 dy tiles [pixel group 16][co + 1][8 pixels]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int segs = a.W / kTile;
    const int seg = blockIdx.x % segs;
    const int r0 = (blockIdx.x / segs) * a.rows_per_cta;
    if (r0 >= a.rows) return;
    const int r1 = min(r0 + a.rows_per_cta, a.rows);
    const int x0 = seg * kTile;

    // zero the rows no input channel fills (m >= 3 CIN, and the pad row) in every slot
    for (int i = tid; i < 4 * 16 * (kARows - 3 * CIN); i += kDwThreads) {
        const int s = i / (16 * (kARows - 3 * CIN)), rem = i % (16 * (kARows - 3 * CIN));
        const int pg = rem / (kARows - 3 * CIN), m = 3 * CIN + rem % (kARows - 3 * CIN);
        *reinterpret_cast<uint4*>(sa + s * kASlot + (pg * kARows + m) * 16) = make_uint4(0, 0, 0, 0);
    }
    if (warp == 0) {
        tc::tmem_alloc(&tslot, TCOLS);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        tc::mbar_fence_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;

    // rows are pipelined: row r's MMAs run while the CTA stages row r + 1 (its new source row
    // goes to the slot those MMAs do not read, its output-gradient tile to the other buffer);
    // MMAs of row k commit to bar[k & 1]
    float dbacc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int tag[4] = {-1, -1, -1, -1};
    int busy[3] = {-1, -1, -1};   // slots the MMAs in flight (previous row) read
    bool ok = true;
    int it = 0;
    auto wait_row = [&](int k) {
        return __all_sync(0xffffffffu, tc::mbar_wait(&bar[k & 1], (uint32_t)(k >> 1) & 1u, kMaxPolls));
    };
    for (int r = r0; r < r1; ++r, ++it) {
        // the output-gradient buffer of this row was last read by row it - 2
        if (it >= 2) ok = ok && wait_row(it - 2);
        int src[3], slot_of[3];
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
            src[dy] = src_row(r, dy - 1, a.H);
            slot_of[dy] = -1;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (tag[k] == src[dy]) slot_of[dy] = k;
        }
        // free slots: not read by the MMAs in flight and not holding a row this row needs; when
        // they are too few (a new image starts), wait for those MMAs first
        int missing = 0, nfree = 0;
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) missing += (slot_of[dy] < 0 && (dy == 0 || src[dy] != src[dy - 1])) ? 1 : 0;
        for (int k = 0; k < 4; ++k) {
            bool used = k == busy[0] || k == busy[1] || k == busy[2];
            for (int e = 0; e < 3; ++e) used = used || k == slot_of[e];
            nfree += used ? 0 : 1;
        }
        if (missing > nfree && it >= 1) {
            ok = ok && wait_row(it - 1);
            busy[0] = busy[1] = busy[2] = -1;
        }
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
            if (slot_of[dy] >= 0) continue;
            int s = -1;
            for (int k = 3; k >= 0; --k) {
                bool used = k == busy[0] || k == busy[1] || k == busy[2];
                for (int e = 0; e < 3; ++e) used = used || k == slot_of[e] || (tag[k] >= 0 && tag[k] == src[e]);
                if (!used) s = k;
            }
            if (s < 0) s = 0;   // unreachable: four slots, at most three rows needed, busy cleared above
            unsigned char* dst = sa + s * kASlot;
            const bf16* row = a.x + (long long)src[dy] * a.W * CIN;
            for (int i2 = tid; i2 < 48 * C8; i2 += kDwThreads) {
                const int pg = i2 % 16, c = (i2 / 16) % C8, dx = i2 / (16 * C8);
                uint4 in[8], out[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    int x = x0 + pg * 8 + j + dx - 1;
                    x = x < 0 ? x + a.W : (x >= a.W ? x - a.W : x);
                    in[j] = __ldg(reinterpret_cast<const uint4*>(row + (long long)x * CIN + c * 8));
                }
                transpose8(in, out);
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    *reinterpret_cast<uint4*>(dst + (pg * kARows + dx * CIN + c * 8 + e) * 16) = out[e];
            }
            tag[s] = src[dy];
#pragma unroll
            for (int e = 0; e < 3; ++e)
                if (src[e] == src[dy]) slot_of[e] = s;
        }
        unsigned char* sbr = sb + (it & 1) * kBTile<COUT>;
        if (tid < 16 * CO8) {
            const int pg = tid % 16, c = tid / 16;
            const bf16* row = a.dy + (long long)r * a.W * COUT;
            uint4 in[8], out[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                in[j] = __ldg(reinterpret_cast<const uint4*>(row + (long long)(x0 + pg * 8 + j) * COUT + c * 8));
                float f[8];
                unpack8(in[j], f);
#pragma unroll
                for (int e = 0; e < 8; ++e) dbacc[e] += f[e];
            }
            transpose8(in, out);
#pragma unroll
            for (int e = 0; e < 8; ++e) *reinterpret_cast<uint4*>(sbr + (pg * BROWS + c * 8 + e) * 16) = out[e];
        }
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        tc::fence_after_sync();
        if (tid == 0) {
            const uint32_t abase = tc::smem_u32(sa), bbase = tc::smem_u32(sbr);
            constexpr uint32_t idesc = tc::idesc_bf16(128, COUT);
#pragma unroll
            for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                for (int ks = 0; ks < 8; ++ks) {
                    const uint32_t aaddr = abase + slot_of[dy] * kASlot + (2 * ks) * kARows * 16;
                    const uint32_t baddr = bbase + (2 * ks) * BROWS * 16;
                    tc::mma_bf16(tmem + (uint32_t)(dy * COUT), tc::desc_kmajor(aaddr, kARows * 16, 128),
                                 tc::desc_kmajor(baddr, BROWS * 16, 128), idesc, (r > r0 || ks > 0) ? 1u : 0u);
                }
            tc::mma_commit(&bar[it & 1]);
        }
        __syncwarp();
#pragma unroll
        for (int e = 0; e < 3; ++e) busy[e] = slot_of[e];
    }
    // the last committed row's MMAs (and, in order, all before them) before the accumulators are
    // read or released, also after a failed wait
    if (it > 0) {
        const bool w = wait_row(it - 1);
        ok = ok && w;
    }
    tc::fence_after_sync();
    if (__syncthreads_or(!ok)) {
        ok = false;
        if (tid == 0 && a.status) atomicExch(a.status, 1);
    }
    // partial gradients of this CTA
    const int m = warp * 32 + lane;
    float* part = a.part + (long long)blockIdx.x * 3 * 128 * COUT;
    if (warp < 4) {
#pragma unroll
        for (int dy = 0; dy < 3; ++dy)
#pragma unroll
            for (int c = 0; c < COUT; c += 16) {
                float t[16];
                tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(dy * COUT + c), t);
                if (ok && m < 3 * CIN) {
                    float4* p = reinterpret_cast<float4*>(part + ((long long)dy * 128 + m) * COUT + c);
#pragma unroll
                    for (int q = 0; q < 4; ++q) p[q] = make_float4(t[4 * q], t[4 * q + 1], t[4 * q + 2], t[4 * q + 3]);
                }
            }
    }
    if (tid < 16 * CO8) {
#pragma unroll
        for (int e = 0; e < 8; ++e) red[tid][e] = dbacc[e];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid < COUT) {
        const int c = tid / 8, e = tid % 8;
        float s = 0.f;
        for (int pg = 0; pg < 16; ++pg) s += red[c * 16 + pg][e];
        a.dbpart[(long long)blockIdx.x * COUT + tid] = s;
    }
    if (warp == 0) tc::tmem_dealloc(tmem, TCOLS);
}

__global__ void k_dw_reduce(int cin, int cout, const float* __restrict__ part, const float* __restrict__ dbpart,
                            int grid, float* __restrict__ dw, float* __restrict__ db)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = 9 * cin * cout;
    if (i < n) {
        const int co = i % cout, ci = (i / cout) % cin, tap = i / (cin * cout);
        const int dy = tap / 3, dx = tap % 3;
        const long long off = ((long long)dy * 128 + dx * cin + ci) * cout + co;
        float s = 0.f;
        for (int b = 0; b < grid; ++b) s += part[(long long)b * 3 * 128 * cout + off];
        dw[i] = s;
    } else if (i < n + cout) {
        const int co = i - n;
        float s = 0.f;
        for (int b = 0; b < grid; ++b) s += dbpart[(long long)b * cout + co];
        db[co] = s;
    }
}

// ---------------------------------------------------------------------------
// weights, optimiser, data
// ---------------------------------------------------------------------------
__global__ void k_prepare_weights(const LayerDesc* __restrict__ layers, int n_layers, const float* __restrict__ p,
                                  bf16* __restrict__ wf, bf16* __restrict__ wb)
{
    const LayerDesc L = layers[blockIdx.y];
    const int n = 9 * L.cin * L.cout;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int co = i % L.cout, ci = (i / L.cout) % L.cin, tap = i / (L.cin * L.cout);
        const bf16 v = __float2bfloat16_rn(p[L.w + i]);
        // forward: [tap][ci / 8][co][ci % 8]
        wf[L.wf + (((long long)tap * (L.cin / 8) + ci / 8) * L.cout + co) * 8 + ci % 8] = v;
        // input gradient: tap' = 8 - tap, input channel co, output channel ci
        wb[L.wb + (((long long)(8 - tap) * (L.cout / 8) + co / 8) * L.cin + ci) * 8 + co % 8] = v;
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void k_assemble(const float* const* __restrict__ planes, const float* const* __restrict__ omega,
                           const float* const* __restrict__ target, int B, int h, int w, const float* __restrict__ s_in,
                           float inv_out, bf16* __restrict__ x0, float* __restrict__ tgt)
{
    const long long hw = (long long)h * w;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)B * hw) return;
    const int b = (int)(i / hw);
    const long long p = i - b * hw;
    float f[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) f[c] = 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c) f[c] = planes[b][c * hw + p] / s_in[c];
#pragma unroll
    for (int c = 0; c < 3; ++c) f[4 + c] = omega[b][c * hw + p] / s_in[4 + c];
    uint4* o = reinterpret_cast<uint4*>(x0 + i * 16);
    o[0] = pack8(f);
    o[1] = pack8(f + 8);
    if (tgt && target && target[b]) {
        const int y = (int)(p / w), x = (int)(p % w);
        const long long W2 = 2ll * w;
        const float* t = target[b];
        float* d = tgt + (long long)b * 4 * hw;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const long long q = (2ll * y + k / 2) * W2 + 2 * x + k % 2;
            d[q] = t[q] * inv_out;
        }
    }
}

__global__ void k_loss(const float* __restrict__ out16, const float* __restrict__ tgt, int B, int h, int w,
                       bf16* __restrict__ dout, double* __restrict__ loss)
{
    __shared__ float red[256];
    const long long hw = (long long)h * w;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const float inv_n = 1.0f / (float)(4.0 * (double)B * (double)hw);
    float acc = 0.f;
    if (i < (long long)B * hw) {
        const int b = (int)(i / hw);
        const long long p = i - b * hw;
        const int y = (int)(p / w), x = (int)(p % w);
        const float* t = tgt + (long long)b * 4 * hw;
        float g[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) g[c] = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float d = out16[i * 16 + k] - t[(2ll * y + k / 2) * 2 * w + 2 * x + k % 2];
            acc += d * d;
            g[k] = 2.f * d * inv_n;
        }
        uint4* o = reinterpret_cast<uint4*>(dout + i * 16);
        o[0] = pack8(g);
        o[1] = pack8(g + 8);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, (double)red[0] * (double)inv_n);
}

__global__ void k_shuffle_out(const float* __restrict__ out16, const float* __restrict__ base, int h, int w,
                              float scale, float* __restrict__ fine)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)h * w) return;
    const int y = (int)(i / w), x = (int)(i % w);
    const float4 v = *reinterpret_cast<const float4*>(out16 + i * 16);
    const float b = base ? base[i] : 0.f;
    float2* r0 = reinterpret_cast<float2*>(fine + (2ll * y) * 2 * w + 2 * x);
    float2* r1 = reinterpret_cast<float2*>(fine + (2ll * y + 1) * 2 * w + 2 * x);
    *r0 = make_float2(fmaf(v.x, scale, b), fmaf(v.y, scale, b));
    *r1 = make_float2(fmaf(v.z, scale, b), fmaf(v.w, scale, b));
}

// spectral loss: r = shuffled prediction - target on the 2h x 2w grid of each sample
__global__ void k_shuffle_resid(const float* __restrict__ out16, const float* __restrict__ tgt, int B, int h, int w,
                                float* __restrict__ r)
{
    const long long hw = (long long)h * w;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)B * hw) return;
    const int b = (int)(i / hw);
    const long long p = i - b * hw;
    const int y = (int)(p / w), x = (int)(p % w);
    const float4 v = *reinterpret_cast<const float4*>(out16 + i * 16);
    const long long q0 = (long long)b * 4 * hw + (2ll * y) * 2 * w + 2 * x, q1 = q0 + 2ll * w;
    r[q0] = v.x - tgt[q0];
    r[q0 + 1] = v.y - tgt[q0 + 1];
    r[q1] = v.z - tgt[q1];
    r[q1 + 1] = v.w - tgt[q1 + 1];
}

// half spectra (R2C layout, B x H2 x (W2/2 + 1)) of the residual and the target: per sample b,
// acc[2b], acc[2b + 1] += {sum w |R|^2, sum w |T|^2} over the full spectrum with w = 1/|k|^4
// on 0 < |k| <= cut, and R *= w in place (the gradient's spectrum).  blockIdx.y = sample.
__global__ void k_spec_loss(float2* __restrict__ R, const float2* __restrict__ T, int H2, int W2, float cut2,
                            double* __restrict__ acc)
{
    __shared__ double red[2][256];
    const int nxf = W2 / 2 + 1;
    const long long n = (long long)H2 * nxf;
    const long long b0 = (long long)blockIdx.y * n;
    double num = 0, den = 0;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const long long i = b0 + j;
        const int kx = (int)(i % nxf);
        const int ky0 = (int)((i / nxf) % H2);
        const int ky = 2 * ky0 > H2 ? ky0 - H2 : ky0;
        const float k2 = (float)(kx * kx + ky * ky);
        const float wk = (k2 > 0.f && k2 <= cut2) ? 1.0f / (k2 * k2) : 0.f;
        const double mult = (kx == 0 || 2 * kx == W2) ? 1.0 : 2.0;
        const float2 r = R[i], t = T[i];
        num += mult * wk * ((double)r.x * r.x + (double)r.y * r.y);
        den += mult * wk * ((double)t.x * t.x + (double)t.y * t.y);
        R[i] = make_float2(r.x * wk, r.y * wk);
    }
    red[0][threadIdx.x] = num;
    red[1][threadIdx.x] = den;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            red[0][threadIdx.x] += red[0][threadIdx.x + s];
            red[1][threadIdx.x] += red[1][threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(acc + 2 * blockIdx.y, red[0][0]);
        atomicAdd(acc + 2 * blockIdx.y + 1, red[1][0]);
    }
}

// gradient of L = (1/B) sum_b num_b / den_b: dL/dpred_b = 2 C2R(w R_b) / (B den_b), packed
// into the tail's 16 channels
__global__ void k_grad_pack(const float* __restrict__ g, const double* __restrict__ acc, int B, int h, int w,
                            bf16* __restrict__ dout)
{
    const long long hw = (long long)h * w;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)B * hw) return;
    const int b = (int)(i / hw);
    const double den = acc[2 * b + 1];
    const float sc = den > 0 ? (float)(2.0 / ((double)B * den)) : 0.f;
    const long long p = i - b * hw;
    const int y = (int)(p / w), x = (int)(p % w);
    const long long q0 = (long long)b * 4 * hw + (2ll * y) * 2 * w + 2 * x, q1 = q0 + 2ll * w;
    float f[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) f[c] = 0.f;
    f[0] = g[q0] * sc;
    f[1] = g[q0 + 1] * sc;
    f[2] = g[q1] * sc;
    f[3] = g[q1 + 1] * sc;
    uint4* o = reinterpret_cast<uint4*>(dout + i * 16);
    o[0] = pack8(f);
    o[1] = pack8(f + 8);
}

__global__ void k_sub(const float* __restrict__ a, const float* __restrict__ b, long long n, float* __restrict__ out)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}

__global__ void k_sumsq_ptrs(const float* const* __restrict__ ptrs, int n, long long offset, long long count,
                             double* __restrict__ out)
{
    __shared__ double red[256];
    double acc = 0.0;
    for (int k = blockIdx.y; k < n; k += gridDim.y) {
        const float* p = ptrs[k] + offset;
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
             i += (long long)gridDim.x * blockDim.x) {
            const double v = p[i];
            acc += v * v;
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(out, red[0]);
}

__global__ void k_diff_stats(const float* __restrict__ a, long long sa, const float* __restrict__ e, long long se,
                             long long n, double* __restrict__ out4)
{
    __shared__ double r[4][256];
    double mx = 0, me = 0, sd = 0, se2 = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double ev = e[i * se], d = (double)a[i * sa] - ev;
        mx = fmax(mx, fabs(d));
        me = fmax(me, fabs(ev));
        sd += d * d;
        se2 += ev * ev;
    }
    r[0][threadIdx.x] = mx;
    r[1][threadIdx.x] = me;
    r[2][threadIdx.x] = sd;
    r[3][threadIdx.x] = se2;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) {
            r[0][threadIdx.x] = fmax(r[0][threadIdx.x], r[0][threadIdx.x + k]);
            r[1][threadIdx.x] = fmax(r[1][threadIdx.x], r[1][threadIdx.x + k]);
            r[2][threadIdx.x] += r[2][threadIdx.x + k];
            r[3][threadIdx.x] += r[3][threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicMax(reinterpret_cast<unsigned long long*>(out4), (unsigned long long)__double_as_longlong(r[0][0]));
        atomicMax(reinterpret_cast<unsigned long long*>(out4 + 1), (unsigned long long)__double_as_longlong(r[1][0]));
        atomicAdd(out4 + 2, r[2][0]);
        atomicAdd(out4 + 3, r[3][0]);
    }
}

template <int CIN, int COUT>
cudaError_t conv_launch(const ConvArgs& a, cudaStream_t s)
{
    constexpr int need = 9 * (CIN / 8) * COUT * 16 + kConvSlots * (CIN / 8) * kPitch * 16;
    constexpr int smem = need > kConvMinSmem ? need : kConvMinSmem;
    static int sms = 0;
    if (!sms) {
        cudaError_t e = cudaFuncSetAttribute(k_conv3x3<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        int dev = 0, n = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        sms = std::max(1, n);
    }
    const long long per_img = (a.H + a.rows_per_cta - 1) / a.rows_per_cta;
    const long long tasks = (long long)(a.W / kTile) * (a.rows / a.H) * per_img;
    const int grid = (int)std::min<long long>(tasks, sms);
    k_conv3x3<CIN, COUT><<<grid, kConvThreads, smem, s>>>(a);
    return cudaGetLastError();
}

template <int CIN, int COUT>
cudaError_t dw_launch(const DwArgs& a, int grid, cudaStream_t s)
{
    constexpr int smem = 4 * kASlot + 2 * kBTile<COUT>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_conv3x3_dw<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_conv3x3_dw<CIN, COUT><<<grid, kDwThreads, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

int conv_rows_per_cta(int rows, int H, int W)
{
    // the persistent grid has one CTA per SM and CTA b takes tasks b, b + SMs, ...: pick the
    // strip height R that minimises the busiest CTA's rows, R ceil(tasks / SMs), counting each
    // strip's two halo rows at a third of a row (staged, but no epilogue); ties go to taller
    // strips (fewer halos)
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                      cudaSuccess || sms < 1)
            sms = 152;
    }
    if (H < 1 || W < kTile || rows < H) return 1;
    const long long groups = (long long)(W / kTile) * (rows / H);
    int best = 1;
    double best_cost = 1e300;
    for (int R = 1; R <= H && R <= 64; ++R) {
        const long long tasks = groups * ((H + R - 1) / R);
        const long long per = (tasks + sms - 1) / sms;
        const double cost = (double)per * (R + 2.0 / 3.0);
        if (cost <= best_cost) {
            best_cost = cost;
            best = R;
        }
    }
    return best;
}

int conv_grid(int rows, int W, int rows_per_cta)
{
    return (W / kTile) * ((rows + rows_per_cta - 1) / rows_per_cta);
}

int dw_rows_per_cta(int rows, int W)
{
    const long long tiles = (long long)rows * (W / kTile);
    return (int)std::max(1ll, (tiles + 151) / 152);
}

static bool conv_args_ok(int W, int rows, int H)
{
    return W > 0 && W % kTile == 0 && H > 0 && rows > 0 && rows % H == 0;
}

cudaError_t launch_conv3x3(int cin, int cout, const ConvArgs& a, cudaStream_t s)
{
    if (!conv_args_ok(a.W, a.rows, a.H) || a.rows_per_cta < 1) return cudaErrorInvalidValue;
    if (cin == 16 && cout == 32) return conv_launch<16, 32>(a, s);
    if (cin == 32 && cout == 32) return conv_launch<32, 32>(a, s);
    if (cin == 32 && cout == 16) return conv_launch<32, 16>(a, s);
    if (cin == 16 && cout == 16) return conv_launch<16, 16>(a, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_conv3x3_dw(int cin, int cout, const DwArgs& a, int grid, cudaStream_t s)
{
    if (!conv_args_ok(a.W, a.rows, a.H) || a.rows_per_cta < 1) return cudaErrorInvalidValue;
    if (grid != (a.W / kTile) * ((a.rows + a.rows_per_cta - 1) / a.rows_per_cta)) return cudaErrorInvalidValue;
    if (cin == 16 && cout == 32) return dw_launch<16, 32>(a, grid, s);
    if (cin == 32 && cout == 32) return dw_launch<32, 32>(a, grid, s);
    if (cin == 32 && cout == 16) return dw_launch<32, 16>(a, grid, s);
    if (cin == 16 && cout == 16) return dw_launch<16, 16>(a, grid, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_dw_reduce(int cin, int cout, const float* part, const float* dbpart, int grid, float* dw, float* db,
                             cudaStream_t s)
{
    const int n = 9 * cin * cout + cout;
    k_dw_reduce<<<(n + 255) / 256, 256, 0, s>>>(cin, cout, part, dbpart, grid, dw, db);
    return cudaGetLastError();
}

cudaError_t launch_prepare_weights(const LayerDesc* d_layers, int n_layers, int max_w, const float* params, bf16* wf,
                                   bf16* wb, cudaStream_t s)
{
    dim3 grid((unsigned)std::max(1, std::min(64, (max_w + 255) / 256)), (unsigned)n_layers);
    k_prepare_weights<<<grid, 256, 0, s>>>(d_layers, n_layers, params, wf, wb);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                        float eps, float c1, float c2, cudaStream_t s)
{
    const int blocks = (int)std::min<long long>(1024, (n + 255) / 256);
    k_adam<<<blocks, 256, 0, s>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_assemble(const float* const* planes, const float* const* omega, const float* const* target, int B,
                            int h, int w, const float* s_in, float inv_out, bf16* x0, float* tgt, cudaStream_t s)
{
    const long long n = (long long)B * h * w;
    k_assemble<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(planes, omega, target, B, h, w, s_in, inv_out, x0, tgt);
    return cudaGetLastError();
}

cudaError_t launch_loss(const float* out16, const float* tgt, int B, int h, int w, bf16* dout, double* loss,
                        cudaStream_t s)
{
    const long long n = (long long)B * h * w;
    k_loss<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out16, tgt, B, h, w, dout, loss);
    return cudaGetLastError();
}

cudaError_t launch_shuffle_out(const float* out16, const float* base, int h, int w, float scale, float* fine,
                               cudaStream_t s)
{
    const long long n = (long long)h * w;
    k_shuffle_out<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out16, base, h, w, scale, fine);
    return cudaGetLastError();
}

cudaError_t launch_shuffle_resid(const float* out16, const float* tgt, int B, int h, int w, float* r, cudaStream_t s)
{
    const long long n = (long long)B * h * w;
    k_shuffle_resid<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out16, tgt, B, h, w, r);
    return cudaGetLastError();
}

cudaError_t launch_spec_loss(float2* R, const float2* T, int B, int H2, int W2, int cut, double* acc, cudaStream_t s)
{
    const long long n = (long long)H2 * (W2 / 2 + 1);
    if (B > 65535) return cudaErrorInvalidValue;
    dim3 blocks((unsigned)std::max(1ll, std::min(256ll, (n + 255) / 256)), (unsigned)B);
    k_spec_loss<<<blocks, 256, 0, s>>>(R, T, H2, W2, (float)cut * (float)cut, acc);
    return cudaGetLastError();
}

cudaError_t launch_grad_pack(const float* g, const double* acc, int B, int h, int w, bf16* dout, cudaStream_t s)
{
    const long long n = (long long)B * h * w;
    k_grad_pack<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, acc, B, h, w, dout);
    return cudaGetLastError();
}

cudaError_t launch_sub(const float* a, const float* b, long long n, float* out, cudaStream_t s)
{
    k_sub<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, n, out);
    return cudaGetLastError();
}

cudaError_t launch_sumsq_ptrs(const float* const* ptrs, int n, long long offset, long long count, double* out,
                              cudaStream_t s)
{
    dim3 grid((unsigned)std::max(1ll, std::min(256ll, (count + 255) / 256)), (unsigned)std::min(n, 64));
    k_sumsq_ptrs<<<grid, 256, 0, s>>>(ptrs, n, offset, count, out);
    return cudaGetLastError();
}

cudaError_t launch_diff_stats(const float* a, long long sa, const float* e, long long se, long long n, double* out4,
                              cudaStream_t s)
{
    const int blocks = (int)std::max(1ll, std::min(1024ll, (n + 255) / 256));
    k_diff_stats<<<blocks, 256, 0, s>>>(a, sa, e, se, n, out4);
    return cudaGetLastError();
}

}  // namespace lrn
}  // namespace cmm
