// ens_fused.cuh -- one ensemble iteration in one cooperative launch (sm_103a).
// Included at the end of mixed_kernels.cu: its stages run that file's device bodies
// (advect_m_tile, incomp_item, compose_value, sample_m4_rows / sample_m_point) and the
// library's FFT pieces (fft.cuh: block_fft, r2c_bin, c2r_pack; psi_solve.cuh: plane_mode),
// so a member of the batched iteration computes what it computes alone.
//
// Schedule.  Member m runs the stages
//     [precombine] advect check [compose rows cols inv-rows] sample rows cols inv-rows
// where the first is there only when its Lagrange coefficients changed and the bracketed
// four only when it remaps; stage w of every member runs in wave w.  Waves are separated by
// grid barriers.  Within a wave the blocks take tasks from the wave's work-queue counter
// (one atomic per task, fetched one task ahead): a task is (member, stage, group), the
// group being g 256-thread tiles of an elementwise stage, one tile of a composition or a few
// rows / columns of a transform stage; the member and stage of every task index follow from
// per-member task counts every block computes for itself at the start of the wave, with the
// long stages' tasks queued first.  Uneven members and stages therefore balance over the grid,
// and a remapping member's composition and fine-grid transforms run beside the other members'
// psi solves.
//
// Remap decision on the device.  After the check's wave each block reads the member's E_inc
// (the exact FP64 value, max-reduced over the check points) and compares it with
// incomp_threshold -- the comparison a single run makes on the host -- and the stack's room.
// Block 0 records the decisions for the host, which only books them afterwards.
// A remapping member's map is reset to the identity in the fine-rows wave; its sample then
// takes the identity without reading the map (no line of the old map can come from a stale
// L1 copy: within the launch every buffer read through the read-only path is written, if at
// all, before its first read).
//
// Barriers.  Thread 0 of a block fences, counts the block in, and polls the count
// (__nanosleep between polls) until every block has arrived -- or until wait_limit polls
// have passed: then it records the wave in the launch's status and the block returns, as
// does every block that sees the status at its next barrier.  The launch is cooperative
// (every block resident), so the limit is only reached when a block has stopped early;
// the host turns the status into CMM_ERR_TIMEOUT.
#pragma once

namespace cmm {
namespace ensf {

constexpr int kT = kEnsFusedThreads;   // threads per block
constexpr int kVPT = 8;                // values per thread of the in-block transforms
constexpr int kBatch = kT * kVPT;      // values one block_fft call holds
constexpr int kCopyChunk = 4 * kT;     // float4 per map copy / reset task

enum Stage : int {
    kStNone = -1,
    kStPre = 0,   // Lagrange precombinations
    kStAdv,       // map advection
    kStInc,       // incompressibility check
    kStCmp,       // remap: omega_0 through the stack on the fine grid, map onto the stack
    kStFrow,      // remap: fine rows (R2C), map reset to the identity
    kStFcol,      // remap: fine columns, Hermite multipliers, inverse columns
    kStFinv,      // remap: fine inverse rows -> fine vorticity nodes
    kStSmp,       // omega on the vort grid, coarse vorticity
    kStProw,      // psi solve: vort rows (kept bins)
    kStPcol,      // psi solve: columns with the spectral step
    kStPinv,      // psi solve: inverse rows -> psi nodes and the Lagrange combinations
};

__device__ __forceinline__ int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

__device__ __forceinline__ bool decide_remap(const EnsMember& e, const unsigned long long* einc, int m)
{
    return e.can_remap && __longlong_as_double((long long)__ldcg(einc + m)) > e.threshold;
}

// stage of member e in wave w (remap: its decision, read only past the check); remaps_only: the
// launch runs the remaps the host decided (four waves)
__device__ __forceinline__ int member_stage(const EnsMember& e, int w, bool remap, bool remaps_only)
{
    if (!e.active) return kStNone;
    if (remaps_only) return remap && w < 4 ? kStCmp + w : kStNone;
    int s = w - (e.precombine ? 1 : 0);
    if (s < 0) return kStPre;
    if (s < 2) return kStAdv + s;
    s -= 2;
    if (remap) {
        if (s < 4) return kStCmp + s;
        s -= 4;
    }
    return s < 4 ? kStSmp + s : kStNone;
}

// split: the wave is short of tasks -- the column stages then take one Hermite plane per task
__device__ __forceinline__ int stage_tasks(const EnsMember& e, const EnsClass& c, int st, int g, int lpn_log2, bool split)
{
    const Grid& gm = e.adv.gm;
    switch (st) {
        case kStPre: return cdiv(cdiv(e.adv.gp.N, kT), g);
        case kStAdv: return cdiv(cdiv(gm.N << lpn_log2, kT), g);
        case kStInc: return cdiv(cdiv(gm.N * e.r_check, kT), g);
        // the long stages: one tile / transform group per task
        case kStCmp: return cdiv(e.gf.N, kT) + cdiv(2 * gm.N, kCopyChunk);
        case kStFrow: return cdiv(e.gf.NY, c.nb_frow) + cdiv(2 * gm.N, kCopyChunk);
        case kStFcol: return (split ? 4 : 1) * cdiv(e.gf.NX / 2 + 1, c.C_f);
        case kStFinv: return cdiv(e.gf.NY, c.nb_finv);
        case kStSmp: return cdiv(cdiv(e.gv.NX == 4 * gm.NX ? e.gv.N / 4 : e.gv.N, kT), g) + cdiv(cdiv(gm.N, kT), g);
        case kStProw: return cdiv(e.gv.NY, c.nb_prow);
        case kStPcol: return (split ? 4 : 1) * cdiv(c.ncols, c.C_p);
        case kStPinv: return cdiv(e.adv.gp.NY, c.nb_pinv);
        default: return 0;
    }
}

// ---------------------------------------------------------------- block-level pieces
// stages whose tasks run long (compositions, transforms): queued first in their wave, so that the
// wave does not end on one of them started last
__device__ __forceinline__ bool heavy_stage(int s) { return s >= kStCmp && s != kStSmp; }

// exclusive prefix sum of v over the block's threads (every thread); *total: the sum
__device__ __forceinline__ int block_scan(int v, int* s_red, int* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_red[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = lane < kT / 32 ? s_red[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kT / 32) s_red[lane] = t;   // inclusive warp totals
    }
    __syncthreads();
    const int ex = (x - v) + (wid > 0 ? s_red[wid - 1] : 0);
    *total = s_red[kT / 32 - 1];
    __syncthreads();   // s_red free again
    return ex;
}

// the members' stages of wave w into st[]; the queue order ord[] (members of heavy stages
// first, each group in member order) and the task prefix sums cum[0..M] over that order for g
// tiles per task of the elementwise stages; returns the wave's task count (every thread)
__device__ int plan_pass(const EnsFusedArgs& a, int w, int g, bool split, signed char* st, int* ord, int* cnt,
                         int* cum, int* s_red)
{
    const int M = a.M;
    const int per = (M + kT - 1) / kT;
    const int m0 = min(M, (int)threadIdx.x * per), m1 = min(M, m0 + per);
    int heavy = 0;
    for (int m = m0; m < m1; ++m) {
        const EnsMember& e = a.mem[m];
        const int pre = e.precombine ? 1 : 0;
        const bool past_check = a.remaps_only || w >= pre + 2;
        const bool remap = e.active && past_check && decide_remap(e, a.einc, m);
        if (blockIdx.x == 0 && !split && e.active && w == (a.remaps_only ? 0 : pre + 2)) a.remapped[m] = remap ? 1 : 0;
        const int sm = member_stage(e, w, remap, a.remaps_only);
        st[m] = (signed char)sm;
        cum[m] = sm == kStNone ? 0 : stage_tasks(e, a.cls[e.cls], sm, g, a.lpn_log2, split);   // counts by member
        heavy += heavy_stage(sm) ? 1 : 0;
    }
    int H, L;
    const int hpos = block_scan(heavy, s_red, &H);
    const int lpos = block_scan((m1 - m0) - heavy, s_red, &L);
    for (int m = m0, h = hpos, l = H + lpos; m < m1; ++m) {
        const int pos = heavy_stage(st[m]) ? h++ : l++;
        ord[pos] = m;
        cnt[pos] = cum[m];
    }
    __syncthreads();
    int local = 0;
    for (int q = m0; q < m1; ++q) local += cnt[q];
    int total;
    int run = block_scan(local, s_red, &total);
    for (int q = m0; q < m1; ++q) {
        run += cnt[q];
        cum[q + 1] = run;
    }
    if (threadIdx.x == 0) cum[0] = 0;
    __syncthreads();
    return total;
}

// the wave's plan (plan_pass); a wave with fewer tasks than blocks (the tail of the remapping
// members' psi solves) is planned again with one tile per task and the column stages split by
// plane.  Block 0 records the remap decisions.  Returns the task count; *g_out, *split_out the
// task shape.
__device__ int plan_wave(const EnsFusedArgs& a, int w, signed char* st, int* ord, int* cnt, int* cum, int* s_red,
                         int* g_out, int* split_out)
{
    int total = plan_pass(a, w, a.g, false, st, ord, cnt, cum, s_red);
    *g_out = a.g;
    *split_out = 0;
    if (total > 0 && total < (int)gridDim.x) {
        total = plan_pass(a, w, 1, true, st, ord, cnt, cum, s_red);
        *g_out = 1;
        *split_out = 1;
    }
    return total;
}

__device__ __forceinline__ int member_of(const int* cum, int M, int task)
{
    int lo = 0, hi = M - 1;
    while (lo < hi) {   // last m with cum[m] <= task
        const int mid = (lo + hi + 1) >> 1;
        if (cum[mid] <= task) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// grid barrier with a bounded wait (see the file comment); false: the launch gave up
__device__ __forceinline__ bool grid_sync(EnsShared* sh, unsigned target, long long limit, int wave, int* s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&sh->count, 1u);
        volatile unsigned* cnt = &sh->count;
        volatile int* status = &sh->status;
        int ok = 1;
        long long polls = 0;
        while (*cnt < target) {
            if (*status != 0) { ok = 0; break; }
            if (++polls > limit) {
                atomicCAS(&sh->status, 0, 1 + wave);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

template <typename V>
__device__ __forceinline__ void fft_run(V* s, int nb, const fft::RadixPlan& P, const V* tw, bool inv, bool pow2)
{
    if (pow2) fft::block_fft<kVPT, fft::kPow2>(s, nb, P, tw, inv);
    else fft::block_fft<kVPT, fft::kPow2x3>(s, nb, P, tw, inv);
}

// the plans and tables of (stage, class) into shared memory, unless they are there already
__device__ __forceinline__ void stage_tables(const EnsClass& c, int st, int ci, fft::RadixPlan* sp, float2* tab,
                                             int* s_key)
{
    const int key = st * kEnsFusedMaxMembers + ci;
    if (*s_key == key) return;
    __syncthreads();   // the previous task's readers are done
    const fft::RadixPlan* p0 = nullptr;
    const fft::RadixPlan* p1 = nullptr;
    const float2* t0 = nullptr;
    const float2* t1 = nullptr;
    int l0 = 0, l1 = 0;
    switch (st) {
        case kStFrow:
        case kStFinv: p0 = &c.f_rx; t0 = c.f_twx; l0 = c.f_rx.tlen + c.f_rx.n + 1; break;
        case kStFcol: p0 = &c.f_ry; t0 = c.f_twy; l0 = c.f_ry.tlen; break;
        case kStProw: p0 = &c.v_rx; t0 = c.v_twx; l0 = c.v_rx.tlen + c.v_rx.n + 1; break;
        case kStPcol: p0 = &c.v_ry; t0 = c.v_twy; l0 = c.v_ry.tlen; p1 = &c.p_ry; t1 = c.p_twy; l1 = c.p_ry.tlen; break;
        default: p0 = &c.p_rx; t0 = c.p_twx; l0 = c.p_rx.tlen + c.p_rx.n + 1; break;   // kStPinv
    }
    if (threadIdx.x == 0) {
        sp[0] = *p0;
        if (p1) sp[1] = *p1;
        *s_key = key;
    }
    fft::load_table(tab, t0, l0);
    if (t1) fft::load_table(tab + l0, t1, l1);
    __syncthreads();
}

// nb rows (row0..) of nx reals at in (row stride nx): R2C, bins 0..kout-1 to out (row stride ld)
__device__ __forceinline__ void rows_fwd(const float* in, int nx, int row0, int nb, const fft::RadixPlan& P,
                                         const float2* tab, float2* s, float2* out, long long ld, int kout, bool pow2)
{
    const int n = nx / 2;
    for (int e = threadIdx.x; e < nb * n; e += kT) {
        const int b = e / n, i = e - b * n;
        s[fft::pad<float2>(e)] = reinterpret_cast<const float2*>(in + (long long)(row0 + b) * nx)[i];
    }
    __syncthreads();
    fft_run(s, nb, P, tab, false, pow2);
    const float2* post = tab + P.tlen;
    for (int e = threadIdx.x; e < nb * kout; e += kT) {
        const int b = e / kout, k = e - b * kout;
        out[(long long)(row0 + b) * ld + k] = fft::r2c_bin(s, b * n, n, k, post);
    }
}

// nb rows (row0..) of the four planes (plane q row r at w2 + (q ny + r) ld, bins 0..kin-1,
// the rest zero): C2R in shared memory.  Transform q nb + b (plane q, row b) sits at
// pad((q nb + b) n) when the four planes fit one block_fft call (joint), else plane q in its own
// buffer of padded(n) values (nb = 1); plane_value reads the results back.
__device__ __forceinline__ bool joint_planes(int nbmax, int n) { return 4 * nbmax * n <= kBatch; }

__device__ __forceinline__ void rows_inv4(const float2* w2, long long ld, int kin, int ny, int nx, int row0, int nb,
                                          int nbmax, const fft::RadixPlan& P, const float2* tab, float2* s, bool pow2)
{
    const int n = nx / 2;
    const bool joint = joint_planes(nbmax, n);
    const int pl = fft::padded_len<float2>(n);
    const float2* post = tab + P.tlen;
    const float2 zero = make_float2(0.0f, 0.0f);
    for (int e = threadIdx.x; e < 4 * nb * n; e += kT) {
        const int t = e / n, k = e - t * n;   // t = q nb + b
        const int q = t / nb, b = t - q * nb;
        const float2* src = w2 + ((long long)q * ny + row0 + b) * ld;
        float2 xk = k < kin ? src[k] : zero;
        float2 xn = n - k < kin ? src[n - k] : zero;
        if (k == 0) { xk.y = 0.0f; xn.y = 0.0f; }
        s[joint ? fft::pad<float2>(e) : q * pl + fft::pad<float2>(k)] = fft::c2r_pack(xk, xn, k, post);
    }
    __syncthreads();
    if (joint) fft_run(s, 4 * nb, P, tab, true, pow2);
    else for (int q = 0; q < 4; ++q) fft_run(s + q * pl, 1, P, tab, true, pow2);
}

__device__ __forceinline__ float plane_value(const float2* s, bool joint, int nb, int q, int b, int n, int iX)
{
    const float* f = reinterpret_cast<const float*>(s);
    const int i = joint ? fft::pad<float2>((q * nb + b) * n + (iX >> 1))
                        : q * fft::padded_len<float2>(n) + fft::pad<float2>(iX >> 1);
    return f[2 * i + (iX & 1)];
}

// the fine grid's Hermite spectrum of plane q from the normalised-to-be column value P
// (k_spec_hermite_f's arithmetic)
__device__ __forceinline__ float2 herm_mode(float2 P, int q, int iX, int iY, const Grid& g, float inv_n)
{
    P.x *= inv_n;
    P.y *= inv_n;
    if (q == 0) return P;
    const float kx = g.kfxf * (float)(2 * iX > g.NX ? iX - g.NX : iX);
    if (q == 1) return make_float2(-P.y * kx, P.x * kx);
    const float ky = g.kfyf * (float)(2 * iY > g.NY ? iY - g.NY : iY);
    const float2 Py = make_float2(-P.y * ky, P.x * ky);
    return q == 2 ? Py : make_float2(-Py.y * kx, Py.x * kx);
}

// ---------------------------------------------------------------- the stages
// Each stage is its own (not inlined) function, so the transforms' unrolled passes of one stage
// do not share a register allocation with every other stage.  They reach the block's shared
// memory through the namespace-scope arrays below (so the compiler addresses it as shared).
struct Smem {
    int cum[kEnsFusedMaxMembers + 1];
    int ord[kEnsFusedMaxMembers];
    int cnt[kEnsFusedMaxMembers];
    signed char stage[kEnsFusedMaxMembers];
    AdvectMArgs adv;
    float sc[4][kMaxFoot];
    W4f w[kMaxCheckRatio], d[kMaxCheckRatio];
    W4f swx[kMaxCheckRatio], swc;
    F2 wmax[kT / 32];
    fft::RadixPlan plan[2];
    int red[kT / 32];
    int task[2];
    int ok;
    int adv_member, inc_member, tab_key, tab_values;
    unsigned long long wave_t0;
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__shared__ Smem g_S;
extern __shared__ __align__(16) float2 g_dyn[];   // tables, then work (g_S.tab_values values in)

__device__ __noinline__ void st_pre(const EnsMember& e, int t, int g)
{
    const int tid = threadIdx.x;
    const long long n = e.adv.gp.N;
    for (int j = 0; j < g; ++j) {
        const long long i = ((long long)t * g + j) * kT + tid;
        if (i >= n) break;
        const float4 v0 = __ldg(e.lv0 + i), v1 = __ldg(e.lv1 + i), v2 = __ldg(e.lv2 + i);
        e.pa[i] = combo(e.ca, v0, v1, v2);
        if (e.pb) e.pb[i] = combo(e.cb, v0, v1, v2);
    }
}

template <int TI>
__device__ __noinline__ void st_adv(const EnsMember& e, int m, int t, int g, int lpn_log2)
{
    const int tid = threadIdx.x;
    if (g_S.adv_member != m) {
        __syncthreads();
        ens_load(g_S.adv, &e.adv);
        __syncthreads();
        if (tid < 4 * kMaxFoot) g_S.sc[tid / kMaxFoot][tid % kMaxFoot] = g_S.adv.coef[tid / kMaxFoot][tid % kMaxFoot];
        if (tid == 0) g_S.adv_member = m;
        __syncthreads();
    }
    const int ntiles = cdiv(e.adv.gm.N << lpn_log2, kT);
    for (int j = 0; j < g; ++j) {
        const int tile = t * g + j;
        if (tile >= ntiles) break;   // block-uniform
        advect_m_tile<TI>(g_S.adv, lpn_log2, (long long)tile * kT + tid, g_S.sc);
    }
}

__device__ __noinline__ void st_inc(const EnsMember& e, int m, int t, int g, unsigned long long* einc)
{
    const int tid = threadIdx.x;
    const Grid& gm = e.adv.gm;
    const int r = e.r_check;
    if (g_S.inc_member != m) {
        __syncthreads();
        incomp_tables(gm, r, e.ir_check, g_S.w, g_S.d);
        if (tid == 0) g_S.inc_member = m;
        __syncthreads();
    }
    F2 best = {0.0f, 0.0f};
    const long long items = gm.N * r;
    for (int j = 0; j < g; ++j) {
        const long long i = ((long long)t * g + j) * kT + tid;
        if (i >= items) break;
        if (r == 4) incomp_item<4>(gm, r, e.ir_check, e.adv.out, (int)i, g_S.w, g_S.d, best, e.adv.nx_log2);
        else incomp_item<0>(gm, r, e.ir_check, e.adv.out, (int)i, g_S.w, g_S.d, best, e.adv.nx_log2);
    }
    incomp_block_max(best, g_S.wmax, einc);
    __syncthreads();   // thread 0 has read g_S.wmax
}

__device__ __noinline__ void st_cmp(const EnsMember& e, int t, int g)
{
    const int tid = threadIdx.x;
    const Grid& gm = e.adv.gm;
    const int nct = cdiv(cdiv(e.gf.N, kT), g);
    if (t < nct) {
        for (int j = 0; j < g; ++j) {
            const long long i = ((long long)t * g + j) * kT + tid;
            if (i >= e.gf.N) break;
            const int iY = (int)(i / e.gf.NX), iX = (int)(i - (long long)iY * e.gf.NX);
            e.real[i] = (float)compose_value(gm, e.stx, e.sty, e.scx, e.scy, e.adv.out, e.stack, e.n_maps, e.src, e.disc,
                                             iX, iY);
        }
    } else {   // the advected map onto the stack
        const long long i0 = (long long)(t - nct) * kCopyChunk;
        for (long long i = i0 + tid; i < i0 + kCopyChunk && i < 2 * gm.N; i += kT) e.push_slot[i] = e.adv.out[i];
    }
}

__device__ __noinline__ void st_frow(const EnsMember& e, const EnsClass& c, int t, int g)
{
    const int tid = threadIdx.x;
    const Grid& gm = e.adv.gm;
    const int groups = cdiv(e.gf.NY, c.nb_frow), ntask = cdiv(groups, g);
    if (t < ntask) {
        stage_tables(c, kStFrow, e.cls, g_S.plan, g_dyn, &g_S.tab_key);
        for (int j = 0; j < g; ++j) {
            const int grp = t * g + j;
            if (grp >= groups) break;
            const int row0 = grp * c.nb_frow;
            __syncthreads();   // the work area's previous readers are done
            rows_fwd(e.real, e.gf.NX, row0, min(c.nb_frow, e.gf.NY - row0), g_S.plan[0], g_dyn, g_dyn + g_S.tab_values,
                     e.w1, c.f_ld, e.gf.NX / 2 + 1, c.pow2);
        }
    } else {   // the map restarts from the identity
        const long long i0 = (long long)(t - ntask) * kCopyChunk;
        float4* out = e.adv.out;
        for (long long i = i0 + tid; i < i0 + kCopyChunk && i < 2 * gm.N; i += kT)
            out[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// C columns: the forward column transform once, then per Hermite plane the multiplier and the
// inverse column transform
__device__ __noinline__ void st_fcol(const EnsMember& e, const EnsClass& c, int t, int g, bool split)
{
    const int tid = threadIdx.x;
    stage_tables(c, kStFcol, e.cls, g_S.plan, g_dyn, &g_S.tab_key);
    const float2* tab = g_dyn;
    const int N = e.gf.NY, ncols = e.gf.NX / 2 + 1, C = c.C_f;
    const int groups = cdiv(ncols, C);
    const int q0 = split ? t / groups : 0, q1 = split ? q0 + 1 : 4;   // the planes of this task
    if (split) t -= q0 * groups;
    const int P = min(4, kBatch / (C * N));                            // planes per inverse call
    float2* A = g_dyn + g_S.tab_values;
    float2* B = A + fft::padded_len<float2>(C * N);
    for (int j = 0; j < g; ++j) {
        const int col0 = (t * g + j) * C;
        if (col0 >= ncols) break;
        __syncthreads();
        for (int x = tid; x < C * N; x += kT) {
            const int cc = x % C, r = x / C, col = col0 + cc;
            A[fft::pad<float2>(cc * N + r)] = col < ncols ? e.w1[(long long)r * c.f_ld + col] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        fft_run(A, C, g_S.plan[0], tab, false, c.pow2);
        for (int qa = q0; qa < q1; qa += P) {
            const int np = min(P, q1 - qa);   // planes in this call
            for (int x = tid; x < np * C * N; x += kT) {
                const int qq = x / (C * N), y = x - qq * C * N, cc = y / N, r = y - cc * N;
                B[fft::pad<float2>(x)] = herm_mode(A[fft::pad<float2>(y)], qa + qq, col0 + cc, r, e.gf, e.inv_nf);
            }
            __syncthreads();
            fft_run(B, np * C, g_S.plan[0], tab, true, c.pow2);
            for (int x = tid; x < np * C * N; x += kT) {
                const int qq = x / (C * N), y = x - qq * C * N, cc = y % C, r = y / C, col = col0 + cc;
                if (col < ncols)
                    e.w2[((long long)(qa + qq) * N + r) * c.f_ld + col] = B[fft::pad<float2>((qq * C + cc) * N + r)];
            }
            __syncthreads();
        }
    }
}

__device__ __noinline__ void st_finv(const EnsMember& e, const EnsClass& c, int t, int g)
{
    const int tid = threadIdx.x;
    stage_tables(c, kStFinv, e.cls, g_S.plan, g_dyn, &g_S.tab_key);
    float2* work = g_dyn + g_S.tab_values;
    const int nx = e.gf.NX, n = nx / 2;
    const bool joint = joint_planes(c.nb_finv, n);
    for (int j = 0; j < g; ++j) {
        const int row0 = (t * g + j) * c.nb_finv;
        if (row0 >= e.gf.NY) break;
        const int nb = min(c.nb_finv, e.gf.NY - row0);
        __syncthreads();
        rows_inv4(e.w2, c.f_ld, n + 1, e.gf.NY, nx, row0, nb, c.nb_finv, g_S.plan[0], g_dyn, work, c.pow2);
        for (int x = tid; x < nb * nx; x += kT) {
            const int b = x / nx, iX = x - b * nx;
            e.wfm_out[(long long)(row0 + b) * nx + iX] =
                make_float4(plane_value(work, joint, nb, 0, b, n, iX), plane_value(work, joint, nb, 1, b, n, iX),
                            plane_value(work, joint, nb, 2, b, n, iX), plane_value(work, joint, nb, 3, b, n, iX));
        }
    }
}

// omega on the vort grid (tasks below the vort tiles) and the coarse vorticity; ident: the
// member remapped, its map is the identity
__device__ __noinline__ void st_smp(const EnsMember& e, int t, int g, bool ident)
{
    const int tid = threadIdx.x;
    const Grid& gm = e.adv.gm;
    const Grid& gv = e.gv;
    const int ro = gv.NX / gm.NX, rf = e.gf.NX / gv.NX, rfc = e.gf.NX / gm.NX;
    // ro = 4: a tile is kT consecutive (map-cell row, vorticity column) pairs, each thread's
    // four points the column's rows in that map-cell row (sample_m4_rows); else kT points
    const long long nq = ro == 4 ? gv.N / 4 : gv.N;
    const int ntv = cdiv(cdiv(nq, kT), g);
    const float iro = 1.0f / (float)ro;
    __syncthreads();   // the previous task's weight tables are read
    if (tid < ro) g_S.swx[tid] = value_weights_f((float)tid * iro, gm.hxf);   // k_ens_sample's tables
    if (tid == 0) g_S.swc = value_weights_f(0.0f * 1.0f, gm.hxf);
    __syncthreads();
    if (t < ntv && ro == 4) {
        for (int j = 0; j < g; ++j) {
            const long long q0 = ((long long)t * g + j) * kT;
            if (q0 >= nq) break;   // block-uniform
            const long long q = q0 + tid;
            const bool live = q < nq;   // the quad of a dead lane is dead too (nq and q0 are multiples of 4)
            const int my = live ? (int)(q / gv.NX) : gm.NY - 1, x = live ? (int)(q - (long long)my * gv.NX) : gv.NX;
            if (ident) sample_m4_rows<true>(gm, gv, e.gf, rf, e.adv.out, e.wfm, x, my, e.real);
            else sample_m4_rows<false>(gm, gv, e.gf, rf, e.adv.out, e.wfm, x, my, e.real);
        }
    } else if (t < ntv) {
        for (int j = 0; j < g; ++j) {
            const long long i0 = ((long long)t * g + j) * kT;
            if (i0 >= gv.N) break;   // block-uniform
            const long long i = i0 + tid;
            const bool live = i < gv.N;
            const int iY = live ? (int)(i / gv.NX) : gv.NY - 1;
            const int iX = live ? (int)(i - (long long)iY * gv.NX) : gv.NX;
            if (ident) {
                sample_m_point<float, 0, true>(gm, gv, e.gf, ro, rf, iro, e.adv.out, e.wfm, e.real, iX, iY, g_S.swx);
            } else {
                sample_m_point<float, 0, false>(gm, gv, e.gf, ro, rf, iro, e.adv.out, e.wfm, e.real, iX, iY, g_S.swx);
            }
        }
    } else {   // coarse vorticity: FP64 copies of the FP32 values (k_ens_sample's arithmetic)
        for (int j = 0; j < g; ++j) {
            const long long i = ((long long)(t - ntv) * g + j) * kT + tid;
            if (i >= gm.N) break;
            const int iY = (int)(i / gm.NX), iX = (int)(i - (long long)iY * gm.NX);
            if (ident) sample_m_point<double, 0, true>(gm, gm, e.gf, 1, rfc, 1.0f, e.adv.out, e.wfm, e.vort, iX, iY, &g_S.swc);
            else sample_m_point<double, 0, false>(gm, gm, e.gf, 1, rfc, 1.0f, e.adv.out, e.wfm, e.vort, iX, iY, &g_S.swc);
        }
    }
}

__device__ __noinline__ void st_prow(const EnsMember& e, const EnsClass& c, int t, int g)
{
    stage_tables(c, kStProw, e.cls, g_S.plan, g_dyn, &g_S.tab_key);
    for (int j = 0; j < g; ++j) {
        const int row0 = (t * g + j) * c.nb_prow;
        if (row0 >= e.gv.NY) break;
        __syncthreads();
        rows_fwd(e.real, e.gv.NX, row0, min(c.nb_prow, e.gv.NY - row0), g_S.plan[0], g_dyn, g_dyn + g_S.tab_values,
                 e.w1, c.ld, c.kv, c.pow2);
    }
}

// C kept columns: the forward column transform over the vort grid once, then per plane the
// spectral step (psi::plane_mode) and the inverse column transform over the psi grid
__device__ __noinline__ void st_pcol(const EnsMember& e, const EnsClass& c, int t, int g, bool split)
{
    const int tid = threadIdx.x;
    stage_tables(c, kStPcol, e.cls, g_S.plan, g_dyn, &g_S.tab_key);
    const Grid& gv = e.gv;
    const Grid& gp = e.adv.gp;
    const int nv = gv.NY, np = gp.NY, C = c.C_p;
    const int groups = cdiv(c.ncols, C);
    const int q0 = split ? t / groups : 0, q1 = split ? q0 + 1 : 4;   // the planes of this task
    if (split) t -= q0 * groups;
    const int P = min(4, kBatch / (C * np));                           // planes per inverse call
    float2* A = g_dyn + g_S.tab_values;
    float2* B = A + fft::padded_len<float2>(C * nv);
    const float2* tv = g_dyn;
    const float2* tp = g_dyn + g_S.plan[0].tlen;
    const float freq = (float)(double)e.freq, inv_nv = (float)(1.0 / (double)gv.N);
    for (int j = 0; j < g; ++j) {
        const int col0 = (t * g + j) * C;
        if (col0 >= c.ncols) break;
        __syncthreads();
        for (int x = tid; x < C * nv; x += kT) {
            const int cc = x % C, r = x / C, col = col0 + cc;
            A[fft::pad<float2>(cc * nv + r)] = col < c.kv ? e.w1[(long long)r * c.ld + col] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        fft_run(A, C, g_S.plan[0], tv, false, c.pow2);
        for (int qa = q0; qa < q1; qa += P) {
            const int nq = min(P, q1 - qa);   // planes in this call
            // each (column, row) mode once, then the call's planes' multipliers
            for (int y = tid; y < C * np; y += kT) {
                const int cc = y / np, r = y - cc * np;
                float kx, ky;
                const float2 M = psi::plane_base_f(A, cc * nv, col0 + cc, r, gv, gp, freq, inv_nv, kx, ky);
                for (int qq = 0; qq < nq; ++qq) B[fft::pad<float2>(qq * C * np + y)] = psi::plane_mul_f(M, qa + qq, kx, ky);
            }
            __syncthreads();
            fft_run(B, nq * C, g_S.plan[1], tp, true, c.pow2);
            for (int x = tid; x < nq * C * np; x += kT) {
                const int qq = x / (C * np), y = x - qq * C * np, cc = y % C, r = y / C, col = col0 + cc;
                if (col < c.ncols)
                    e.w2[((long long)(qa + qq) * np + r) * c.ld + col] = B[fft::pad<float2>((qq * C + cc) * np + r)];
            }
            __syncthreads();
        }
    }
}

__device__ __noinline__ void st_pinv(const EnsMember& e, const EnsClass& c, int t, int g)
{
    const int tid = threadIdx.x;
    stage_tables(c, kStPinv, e.cls, g_S.plan, g_dyn, &g_S.tab_key);
    float2* work = g_dyn + g_S.tab_values;
    const Grid& gp = e.adv.gp;
    const int nx = gp.NX, n = nx / 2;
    const bool joint = joint_planes(c.nb_pinv, n);
    for (int j = 0; j < g; ++j) {
        const int row0 = (t * g + j) * c.nb_pinv;
        if (row0 >= gp.NY) break;
        const int nb = min(c.nb_pinv, gp.NY - row0);
        __syncthreads();
        rows_inv4(e.w2, c.ld, c.ncols, gp.NY, nx, row0, nb, c.nb_pinv, g_S.plan[0], g_dyn, work, c.pow2);
        for (int x = tid; x < nb * nx; x += kT) {
            const int b = x / nx, iX = x - b * nx;
            const long long i = (long long)(row0 + b) * nx + iX;
            const float4 v0 = make_float4(plane_value(work, joint, nb, 0, b, n, iX), plane_value(work, joint, nb, 1, b, n, iX),
                                          plane_value(work, joint, nb, 2, b, n, iX), plane_value(work, joint, nb, 3, b, n, iX));
            e.psi_new[i] = v0;
            if (e.fused) {
                const float4 v1 = __ldg(e.lv1n + i), v2 = __ldg(e.lv2n + i);
                e.o1[i] = combo(e.cm.c[0], v0, v1, v2);
                e.o2[i] = combo(e.cm.c[1], v0, v1, v2);
                e.o3[i] = combo(e.cm.c[2], v0, v1, v2);
            }
        }
    }
}

// ---------------------------------------------------------------- the kernel
template <int TI, int MINB>
__global__ void __launch_bounds__(kT, MINB) k_ens_fused(const EnsFusedArgs a)
{
    const int tid = threadIdx.x;
    if (tid == 0) { g_S.adv_member = -1; g_S.inc_member = -1; g_S.tab_key = -1; g_S.tab_values = a.tab_values; }
    if (a.prof && tid == 0 && blockIdx.x == 0) g_S.wave_t0 = global_ns();
    unsigned arrivals = 0;
    for (int w = 0; w < kEnsFusedMaxWaves; ++w) {
        __syncthreads();
        int g, split;
        const int total = plan_wave(a, w, g_S.stage, g_S.ord, g_S.cnt, g_S.cum, g_S.red, &g, &split);
        if (total == 0) break;
        if (blockIdx.x == 0 && tid == 0) a.sh->waves = w + 1;
        unsigned* queue = &a.sh->queue[w];
        // tasks, each fetched while the previous one runs
        if (tid == 0) g_S.task[0] = (int)atomicAdd(queue, 1u);
        __syncthreads();
        int buf = 0;
        for (int task = g_S.task[0]; task < total;) {
            int next = 0;
            if (tid == 0) next = (int)atomicAdd(queue, 1u);
            const int pos = member_of(g_S.cum, a.M, task);   // place in the queue order
            const int m = g_S.ord[pos];
            const int t = task - g_S.cum[pos];
            const EnsMember& e = a.mem[m];
            const int st = g_S.stage[m];
            long long c0 = 0;
            if (a.prof && tid == 0) c0 = clock64();
            switch (st) {
                case kStPre: st_pre(e, t, g); break;
                case kStAdv: st_adv<TI>(e, m, t, g, a.lpn_log2); break;
                case kStInc: st_inc(e, m, t, g, a.einc + m); break;
                case kStCmp: st_cmp(e, t, 1); break;
                case kStFrow: st_frow(e, a.cls[e.cls], t, 1); break;
                case kStFcol: st_fcol(e, a.cls[e.cls], t, 1, split); break;
                case kStFinv: st_finv(e, a.cls[e.cls], t, 1); break;
                case kStSmp: st_smp(e, t, g, decide_remap(e, a.einc, m)); break;
                case kStProw: st_prow(e, a.cls[e.cls], t, 1); break;
                case kStPcol: st_pcol(e, a.cls[e.cls], t, 1, split); break;
                case kStPinv: st_pinv(e, a.cls[e.cls], t, 1); break;
                default: break;
            }
            if (a.prof && tid == 0) {   // block cycles and tasks per stage
                atomicAdd(a.prof + kProfStage + st, (unsigned long long)(clock64() - c0));
                atomicAdd(a.prof + kProfTasks + st, 1ull);
            }
            // the next task: written to the slot the current one did not use
            if (tid == 0) g_S.task[buf ^ 1] = next;
            __syncthreads();
            buf ^= 1;
            task = g_S.task[buf];
        }
        arrivals += gridDim.x;
        long long b0 = 0;
        if (a.prof && tid == 0) b0 = clock64();
        if (!grid_sync(a.sh, arrivals, a.wait_limit, w, &g_S.ok)) return;
        if (a.prof && tid == 0) {
            atomicAdd(a.prof + kProfBarrier, (unsigned long long)(clock64() - b0));
            if (blockIdx.x == 0) {   // wall time of the wave, barrier included
                const unsigned long long now = global_ns();
                atomicAdd(a.prof + kProfWave + w, now - g_S.wave_t0);
                g_S.wave_t0 = now;
            }
        }
    }
}

}  // namespace ensf

// ---------------------------------------------------------------- host side
void ens_fused_smem_values(const EnsClass& c, const Grid& gv, const Grid& gp, const Grid& gf, int* tab, int* work)
{
    using fft::padded_len;
    const int nf = gf.NX / 2, nv = gv.NX / 2, np = gp.NX / 2;
    int t = c.f_rx.tlen + nf + 1;
    t = std::max(t, c.f_ry.tlen);
    t = std::max(t, c.v_rx.tlen + nv + 1);
    t = std::max(t, c.v_ry.tlen + c.p_ry.tlen);
    t = std::max(t, c.p_rx.tlen + np + 1);
    const int B = ensf::kBatch;
    auto inv_rows = [&](int nb, int n) {   // rows_inv4's layouts
        return 4 * nb * n <= B ? padded_len<float2>(4 * nb * n) : 4 * padded_len<float2>(n);
    };
    const int Pf = std::min(4, B / (c.C_f * gf.NY)), Pp = std::min(4, B / (c.C_p * gp.NY));
    int w = padded_len<float2>(c.nb_frow * nf);
    w = std::max(w, padded_len<float2>(c.C_f * gf.NY) + padded_len<float2>(Pf * c.C_f * gf.NY));
    w = std::max(w, inv_rows(c.nb_finv, nf));
    w = std::max(w, padded_len<float2>(c.nb_prow * nv));
    w = std::max(w, padded_len<float2>(c.C_p * gv.NY) + padded_len<float2>(Pp * c.C_p * gp.NY));
    w = std::max(w, inv_rows(c.nb_pinv, np));
    *tab = (t + 1) / 2 * 2;   // the work area starts 16-byte aligned
    *work = w;
}

template <int TI, int MINB>
static cudaError_t launch_fused_ti(const EnsFusedArgs& a, int blocks, cudaStream_t s)
{
    // (the shared-memory limit was raised by ens_fused_blocks_per_sm, before any capture)
    const size_t smem = sizeof(float2) * ((size_t)a.tab_values + (size_t)a.work_values);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(ensf::kT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, ensf::k_ens_fused<TI, MINB>, a);
}

template <int MINB>
static cudaError_t launch_fused_minb(int TI, const EnsFusedArgs& a, int blocks, cudaStream_t s)
{
    switch (TI) {
        case 10: return launch_fused_ti<10, MINB>(a, blocks, s);
        case 21: return launch_fused_ti<21, MINB>(a, blocks, s);
        case 30: return launch_fused_ti<30, MINB>(a, blocks, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_ens_fused(int TI, int minb, const EnsFusedArgs& a, int blocks, cudaStream_t s)
{
    if (blocks <= 0 || a.M <= 0 || a.M > kEnsFusedMaxMembers || a.g <= 0) return cudaErrorInvalidValue;
    if (minb == 4) return launch_fused_minb<4>(TI, a, blocks, s);
    if (minb == 6) return launch_fused_minb<6>(TI, a, blocks, s);
    return cudaErrorInvalidValue;
}

template <int TI, int MINB>
static int blocks_per_sm_ti(const EnsFusedArgs& a)
{
    const size_t smem = sizeof(float2) * ((size_t)a.tab_values + (size_t)a.work_values);
    if (cudaFuncSetAttribute(ensf::k_ens_fused<TI, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ensf::k_ens_fused<TI, MINB>, ensf::kT, smem) != cudaSuccess)
        return 0;
    return n;
}

template <int MINB>
static int blocks_per_sm_minb(int TI, const EnsFusedArgs& a)
{
    switch (TI) {
        case 10: return blocks_per_sm_ti<10, MINB>(a);
        case 21: return blocks_per_sm_ti<21, MINB>(a);
        case 30: return blocks_per_sm_ti<30, MINB>(a);
        default: return 0;
    }
}

int ens_fused_blocks_per_sm(int TI, int minb, const EnsFusedArgs& a)
{
    if (minb == 4) return blocks_per_sm_minb<4>(TI, a);
    if (minb == 6) return blocks_per_sm_minb<6>(TI, a);
    return 0;
}

}  // namespace cmm
