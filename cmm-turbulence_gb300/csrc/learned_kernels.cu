// learned_kernels.cu -- BF16 tcgen05 convolution kernels of the learned psi upsampler and
// the elementwise steps around them (see learned.hpp for the layouts).
//
// Forward / input-gradient convolution (k_conv3x3<CIN, COUT>): a CTA of 128 threads walks
// a strip of consecutive rows of one 128-pixel column segment.  Each source row it needs
// (the tile's row and its two periodic neighbours) is staged once into one of four row
// slots with cp.async, laid out as [channel chunk of 8][pixel 0..129][8 channels]: a
// K-major operand whose 8-pixel core matrices are 128 contiguous bytes, so the tap with
// column offset dx is the same slot addressed dx * 16 bytes further.  The 9 taps x CIN/16
// MMAs (M = 128 pixels, N = COUT, K = 16) accumulate in TMEM; the epilogue reads one
// pixel's COUT accumulators per thread and fuses bias, ReLU, the ReLU mask of the
// backward pass and the residual add.
//
// Weight gradient (k_conv3x3_dw<CIN, COUT>): dW[(dy, dx, ci)][co] = sum over pixels of
// x[p + (dy - 1, dx - 1)][ci] dy[p][co], a GEMM with K = pixels.  Each staged input row
// is transposed into three K-major copies shifted by dx (M = (dx, ci), padded to 128),
// the output-gradient row into one K-major tile, and three accumulators (one per dy)
// stay in TMEM across the CTA's whole strip; the per-CTA partials are summed in a fixed
// order by k_dw_reduce.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "learned.hpp"
#include "tc_sm100.cuh"

namespace cmm {
namespace lrn {

namespace {

constexpr long long kMaxPolls = 1ll << 22;   // ~0.2 s of polling before a wait gives up

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
// Software pipeline over the CTA's strip of rows: while one thread issues row r's MMAs into
// accumulator r % 2, the CTA stages (cp.async) the source rows row r + 1 still lacks and then
// drains row r - 1's accumulator (the epilogue).  Two mbarriers track the two accumulators;
// a source row's slot is reused only after the MMAs reading it completed.
template <int CIN, int COUT>
__device__ __forceinline__ void conv_issue(uint32_t d_tmem, uint32_t rbase, uint32_t wbase, const int (&slot)[3])
{
    constexpr int C8 = CIN / 8;
    constexpr int SLOT = C8 * kPitch * 16;
    constexpr uint32_t idesc = tc::idesc_bf16(128, COUT);
    uint32_t acc = 0;
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
        for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int kk = 0; kk < CIN / 16; ++kk) {
                const uint32_t aaddr = rbase + slot[dy] * SLOT + ((2 * kk) * kPitch + dx) * 16;
                const uint32_t baddr = wbase + ((dy * 3 + dx) * C8 + 2 * kk) * COUT * 16;
                tc::mma_bf16(d_tmem, tc::desc_kmajor(aaddr, kPitch * 16, 128), tc::desc_kmajor(baddr, COUT * 16, 128),
                             idesc, acc);
                acc = 1;
            }
}

template <int CIN>
__device__ __forceinline__ void conv_stage(unsigned char* dst, const bf16* __restrict__ in, int src, int W, int x0)
{
    constexpr int C8 = CIN / 8;
    const bf16* row = in + (long long)src * W * CIN;
    for (int i = threadIdx.x; i < C8 * kPitch; i += 128) {
        const int c = i % C8, p = i / C8;
        int x = x0 - 1 + p;
        x = x < 0 ? x + W : (x >= W ? x - W : x);
        cp_async16(dst + (c * kPitch + p) * 16, row + (long long)x * CIN + c * 8);
    }
}

template <int COUT>
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, uint32_t d_tmem, int r, int x0, const float (&bias)[COUT],
                                              bool store)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float v[COUT];
#pragma unroll
    for (int c = 0; c < COUT; c += 16) {
        float t[16];
        tc::tmem_ld16(d_tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, t);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[c + j] = t[j] + bias[c + j];
    }
    if (!store) return;
    const long long pix = (long long)r * a.W + x0 + warp * 32 + lane;
    if (a.relu) {
#pragma unroll
        for (int j = 0; j < COUT; ++j) v[j] = fmaxf(v[j], 0.f);
    }
    if (a.mask) {
        const uint4* mp = reinterpret_cast<const uint4*>(a.mask + pix * COUT);
#pragma unroll
        for (int q = 0; q < COUT / 8; ++q) {
            float m[8];
            unpack8(mp[q], m);
#pragma unroll
            for (int e = 0; e < 8; ++e) v[8 * q + e] = m[e] > 0.f ? v[8 * q + e] : 0.f;
        }
    }
    if (a.res) {
        const uint4* rp = reinterpret_cast<const uint4*>(a.res + pix * COUT);
#pragma unroll
        for (int q = 0; q < COUT / 8; ++q) {
            float m[8];
            unpack8(rp[q], m);
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

// slots for the source rows of output row r: rows already staged keep their slot; missing
// rows go to slots outside `busy` (the slots MMAs in flight read) and not holding a row r
// needs.  Returns the number of rows it could not place (0 on success).  Uniform over the CTA.
template <int CIN>
__device__ __forceinline__ int conv_place(const ConvArgs& a, int r, int x0, unsigned char* sr, int (&tag)[4],
                                          const int (&busy)[3], int nbusy, int (&slot)[3])
{
    constexpr int SLOT = (CIN / 8) * kPitch * 16;
    int src[3];
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
        src[dy] = src_row(r, dy - 1, a.H);
        slot[dy] = -1;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (tag[k] == src[dy]) slot[dy] = k;
    }
    int unplaced = 0;
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
        if (slot[dy] >= 0) continue;
        int s = -1;
        for (int k = 3; k >= 0; --k) {
            bool used = false;
            for (int e = 0; e < nbusy; ++e) used = used || busy[e] == k;
            for (int e = 0; e < 3; ++e) used = used || slot[e] == k || (tag[k] >= 0 && tag[k] == src[e]);
            if (!used) s = k;
        }
        if (s < 0) {
            ++unplaced;
            continue;
        }
        conv_stage<CIN>(sr + s * SLOT, a.in, src[dy], a.W, x0);
        tag[s] = src[dy];
#pragma unroll
        for (int e = 0; e < 3; ++e)
            if (src[e] == src[dy]) slot[e] = s;
    }
    return unplaced;
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3x3(ConvArgs a)
{
    constexpr int C8 = CIN / 8;
    constexpr int WB = 9 * C8 * COUT * 16;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tslot;
    unsigned char* sw = sm;
    unsigned char* sr = sm + WB;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int segs = a.W / kTile;
    const int seg = blockIdx.x % segs;
    const int r0 = (blockIdx.x / segs) * a.rows_per_cta;
    if (r0 >= a.rows) return;
    const int r1 = min(r0 + a.rows_per_cta, a.rows);
    const int x0 = seg * kTile;

    for (int i = tid; i < WB / 16; i += 128)
        cp_async16(sw + 16 * i, reinterpret_cast<const unsigned char*>(a.wt) + 16 * (long long)i);
    if (warp == 0) {
        tc::tmem_alloc(&tslot, 64);   // two accumulators of 32 columns
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        tc::mbar_fence_init();
    }
    float bias[COUT];
#pragma unroll
    for (int j = 0; j < COUT; ++j) bias[j] = a.bias ? a.bias[j] : 0.f;

    int tag[4] = {-1, -1, -1, -1};
    int cur[3], nxt[3];
    const int none[3] = {-1, -1, -1};
    conv_place<CIN>(a, r0, x0, sr, tag, none, 0, cur);   // four free slots: always places all
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint32_t wbase = tc::smem_u32(sw), rbase = tc::smem_u32(sr);

    bool ok = true;
    int it = 0;
    for (int r = r0; r < r1; ++r, ++it) {
        // this row's source rows (staged in the previous iteration or above) visible to the MMAs
        cp_async_wait_all();
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            conv_issue<CIN, COUT>(tmem + (uint32_t)((it & 1) * 32), rbase, wbase, cur);
            tc::mma_commit(&bar[it & 1]);
        }
        __syncwarp();
        // the previous row's MMAs: their accumulator is drained below, their slots free up
        if (it > 0) ok = ok && tc::mbar_wait(&bar[(it - 1) & 1], ((it - 1) >> 1) & 1, kMaxPolls);
        if (r + 1 < r1) {
            if (conv_place<CIN>(a, r + 1, x0, sr, tag, cur, 3, nxt) > 0) {
                // a new image starts: the rows it needs outnumber the free slots; wait for this
                // row's MMAs, after which only the rows row r + 1 needs are kept
                ok = ok && tc::mbar_wait(&bar[it & 1], (it >> 1) & 1, kMaxPolls);
                conv_place<CIN>(a, r + 1, x0, sr, tag, none, 0, nxt);
            }
        }
        ok = __all_sync(0xffffffffu, ok);
        tc::fence_after_sync();
        if (it > 0) conv_epilogue<COUT>(a, tmem + (uint32_t)(((it - 1) & 1) * 32), r - 1, x0, bias, ok);
        tc::fence_before_sync();
        if (__syncthreads_or(!ok)) break;
#pragma unroll
        for (int d = 0; d < 3; ++d) cur[d] = nxt[d];
    }
    if (ok && it > 0) {
        ok = __all_sync(0xffffffffu, tc::mbar_wait(&bar[(it - 1) & 1], ((it - 1) >> 1) & 1, kMaxPolls));
        tc::fence_after_sync();
        conv_epilogue<COUT>(a, tmem + (uint32_t)(((it - 1) & 1) * 32), r1 - 1, x0, bias, ok);
    }
    cp_async_wait_all();
    tc::fence_before_sync();
    if (__syncthreads_or(!ok) && tid == 0 && a.status) atomicExch(a.status, 1);
    if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// ---------------------------------------------------------------------------
// weight gradient
// ---------------------------------------------------------------------------
constexpr int kARows = 129;                  // 128 M rows + 1 pad row per 8-pixel group
constexpr int kASlot = 16 * kARows * 16;     // [pixel group 16][m 129][8 pixels]

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3x3_dw(DwArgs a)
{
    constexpr int C8 = CIN / 8, CO8 = COUT / 8;
    constexpr int BROWS = COUT + 1;
    constexpr uint32_t TCOLS = 3 * COUT <= 64 ? 64 : 128;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    __shared__ float red[16 * CO8][8];
    unsigned char* sa = sm;                       // 4 slots
    unsigned char* sb = sm + 4 * kASlot;          // dy tile [pixel group 16][co + 1][8 pixels]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int segs = a.W / kTile;
    const int seg = blockIdx.x % segs;
    const int r0 = (blockIdx.x / segs) * a.rows_per_cta;
    if (r0 >= a.rows) return;
    const int r1 = min(r0 + a.rows_per_cta, a.rows);
    const int x0 = seg * kTile;

    // zero the rows no input channel fills (m >= 3 CIN, and the pad row) in every slot
    for (int i = tid; i < 4 * 16 * (kARows - 3 * CIN); i += 128) {
        const int s = i / (16 * (kARows - 3 * CIN)), rem = i % (16 * (kARows - 3 * CIN));
        const int pg = rem / (kARows - 3 * CIN), m = 3 * CIN + rem % (kARows - 3 * CIN);
        *reinterpret_cast<uint4*>(sa + s * kASlot + (pg * kARows + m) * 16) = make_uint4(0, 0, 0, 0);
    }
    if (warp == 0) {
        tc::tmem_alloc(&tslot, TCOLS);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&bar, 1);
        tc::mbar_fence_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;

    float dbacc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int tag[4] = {-1, -1, -1, -1};
    uint32_t phase = 0;
    bool ok = true;
    for (int r = r0; r < r1; ++r) {
        int slot_of[3];
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
            const int src = src_row(r, dy - 1, a.H);
            slot_of[dy] = -1;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (tag[k] == src) slot_of[dy] = k;
        }
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
            if (slot_of[dy] >= 0) continue;
            const int src = src_row(r, dy - 1, a.H);
            int s = 0;
            for (int k = 3; k >= 0; --k)
                if (k != slot_of[0] && k != slot_of[1] && k != slot_of[2]) s = k;
            unsigned char* dst = sa + s * kASlot;
            const bf16* row = a.x + (long long)src * a.W * CIN;
            for (int it = tid; it < 48 * C8; it += 128) {
                const int pg = it % 16, c = (it / 16) % C8, dx = it / (16 * C8);
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
            tag[s] = src;
            slot_of[dy] = s;
        }
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
            for (int e = 0; e < 8; ++e) *reinterpret_cast<uint4*>(sb + (pg * BROWS + c * 8 + e) * 16) = out[e];
        }
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            const uint32_t abase = tc::smem_u32(sa), bbase = tc::smem_u32(sb);
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
            tc::mma_commit(&bar);
        }
        __syncwarp();
        ok = __all_sync(0xffffffffu, tc::mbar_wait(&bar, phase, kMaxPolls));
        phase ^= 1u;
        tc::fence_after_sync();
        tc::fence_before_sync();
        if (__syncthreads_or(!ok)) {
            ok = false;
            if (tid == 0 && a.status) atomicExch(a.status, 1);
            break;
        }
    }
    // partial gradients of this CTA
    const int m = warp * 32 + lane;
    float* part = a.part + (long long)blockIdx.x * 3 * 128 * COUT;
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
    constexpr int smem = 9 * (CIN / 8) * COUT * 16 + 4 * (CIN / 8) * kPitch * 16;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_conv3x3<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int grid = conv_grid(a.rows, a.W, a.rows_per_cta);
    k_conv3x3<CIN, COUT><<<grid, 128, smem, s>>>(a);
    return cudaGetLastError();
}

template <int CIN, int COUT>
cudaError_t dw_launch(const DwArgs& a, int grid, cudaStream_t s)
{
    constexpr int smem = 4 * kASlot + 16 * (COUT + 1) * 16;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_conv3x3_dw<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_conv3x3_dw<CIN, COUT><<<grid, 128, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

int conv_rows_per_cta(int rows, int W)
{
    // about two pipelined CTAs per SM, at least four rows each
    const long long tiles = (long long)rows * (W / kTile);
    const long long target = 152 * 2;
    if (const char* e = getenv("CMM_CONV_ROWS")) return atoi(e);
    return (int)std::max(4ll, (tiles + target - 1) / target);
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
