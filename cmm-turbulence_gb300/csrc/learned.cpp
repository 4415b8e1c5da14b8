// learned.cpp -- the upsampler network on the device: parameters, Adam state, training
// pairs, work buffers, and the forward / backward passes as sequences of the kernels of
// learned_kernels.cu.
#include "learned.hpp"


#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>

namespace cmm {
namespace lrn {

namespace {
constexpr char kMagic[8] = {'C', 'M', 'M', 'U', 'P', 'S', '0', '3'};
constexpr float kB1 = 0.9f, kB2 = 0.999f, kEps = 1e-8f;

template <typename T>
cudaError_t alloc(T** p, long long n)
{
    *p = nullptr;
    if (n <= 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (size_t)n);
}
template <typename T>
void release(T*& p)
{
    if (p) cudaFree(const_cast<void*>(static_cast<const void*>(p)));
    p = nullptr;
}
}  // namespace

#define LRN_CHECK(call, what)                        \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return fail(what, e_); \
    } while (0)

int Upsampler::fail(const char* what, cudaError_t e)
{
    err = std::string("upsampler: ") + what + ": " + cudaGetErrorString(e);
    return 1;
}

Upsampler::Upsampler(int blocks, int channels) : nb_(blocks), ch_(channels)
{
    long long off = 0, offw = 0;
    auto add = [&](int cin, int cout) {
        LayerDesc L;
        L.cin = cin;
        L.cout = cout;
        L.w = off;
        off += 9ll * cin * cout;
        L.b = off;
        off += cout;
        L.wf = L.wb = offw;
        offw += 9ll * cin * cout;
        layers_.push_back(L);
        max_w_ = std::max(max_w_, 9 * cin * cout);
    };
    add(kHeadIn, ch_);
    for (int i = 0; i < nb_; ++i) {
        add(ch_, ch_);
        add(ch_, ch_);
    }
    add(ch_, kTailOut);
    n_params_ = off;
    n_wf_ = offw;
    if (ch_ != 32 || nb_ < 0 || nb_ > 64) {
        err = "upsampler: channels must be 32 and blocks 0..64";
        return;
    }
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = alloc(&params_, n_params_);
    if (e == cudaSuccess) e = alloc(&grads_, n_params_);
    if (e == cudaSuccess) e = alloc(&adam_m_, n_params_);
    if (e == cudaSuccess) e = alloc(&adam_v_, n_params_);
    if (e == cudaSuccess) e = alloc(&wf_, n_wf_);
    if (e == cudaSuccess) e = alloc(&wb_, n_wf_);
    if (e == cudaSuccess) e = alloc(&d_layers_, (long long)layers_.size());
    if (e == cudaSuccess) e = alloc(&d_sin_, kInCh);
    if (e == cudaSuccess) e = alloc(&d_loss_, 2 * kMaxBatch);
    if (e == cudaSuccess) e = alloc(&d_status_, 1);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_layers_, layers_.data(), sizeof(LayerDesc) * layers_.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_status_, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(grads_, 0, sizeof(float) * n_params_);
    if (e != cudaSuccess) {
        fail("allocation", e);
        return;
    }
    set_scales(s_in_, s_out_);
    scaled_ = false;
    init_weights(0);
}

Upsampler::~Upsampler()
{
    clear_dataset();
    release(params_);
    release(grads_);
    release(adam_m_);
    release(adam_v_);
    release(wf_);
    release(wb_);
    release(d_layers_);
    release(d_sin_);
    release(d_loss_);
    release(d_status_);
    release(x0_);
    for (auto& p : act_) release(p);
    for (auto& p : hid_) release(p);
    release(da_[0]);
    release(da_[1]);
    release(dh_);
    release(dout_);
    release(out32_);
    release(tgt_);
    release(part_);
    release(dbpart_);
    release(d_ptrs_);
    release(rbuf_);
    release(rspec_);
    release(tspec_);
    fft::plan_destroy(fft_);
}

int Upsampler::init_weights(uint64_t seed)
{
    if (!params_) return 1;
    std::vector<float> p((size_t)n_params_, 0.f);
    std::mt19937_64 g(seed);
    auto uni = [&]() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); };
    for (size_t l = 0; l < layers_.size(); ++l) {
        const LayerDesc& L = layers_[l];
        const int cin_real = l == 0 ? kInCh : L.cin;
        const int cout_real = l + 1 == layers_.size() ? 4 : L.cout;
        double bound = std::sqrt(6.0 / (9.0 * cin_real));
        if (l + 1 == layers_.size() || (l > 0 && l % 2 == 0)) bound *= 0.1;   // tail, second conv of a block
        for (int tap = 0; tap < 9; ++tap)
            for (int ci = 0; ci < L.cin; ++ci)
                for (int co = 0; co < L.cout; ++co) {
                    const double u = (2.0 * uni() - 1.0) * bound;
                    p[(size_t)(L.w + ((long long)tap * L.cin + ci) * L.cout + co)] =
                        (ci < cin_real && co < cout_real) ? (float)u : 0.f;
                }
    }
    return set_params(p.data(), n_params_);
}

int Upsampler::set_params(const float* host, long long n)
{
    if (n != n_params_ || !params_) {
        err = "upsampler: parameter count mismatch";
        return 1;
    }
    LRN_CHECK(cudaMemcpy(params_, host, sizeof(float) * n, cudaMemcpyHostToDevice), "set_params");
    LRN_CHECK(cudaMemset(adam_m_, 0, sizeof(float) * n), "set_params");
    LRN_CHECK(cudaMemset(adam_v_, 0, sizeof(float) * n), "set_params");
    adam_t_ = 0;
    prepared_ = false;
    return 0;
}

int Upsampler::get_params(float* host, long long n) const
{
    if (n != n_params_ || !params_) return 1;
    return cudaMemcpy(host, params_, sizeof(float) * n, cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : 1;
}

int Upsampler::get_grads(float* host, long long n) const
{
    if (n != n_params_ || !grads_) return 1;
    return cudaMemcpy(host, grads_, sizeof(float) * n, cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : 1;
}

void Upsampler::set_scales(const double* s_in, double s_out)
{
    float f[kInCh];
    for (int c = 0; c < kInCh; ++c) {
        s_in_[c] = s_in[c] > 0 ? s_in[c] : 1.0;
        f[c] = (float)s_in_[c];
    }
    s_out_ = s_out > 0 ? s_out : 1.0;
    if (d_sin_) cudaMemcpy(d_sin_, f, sizeof(f), cudaMemcpyHostToDevice);
    scaled_ = true;
}

void Upsampler::get_scales(double* s_in, double* s_out) const
{
    for (int c = 0; c < kInCh; ++c) s_in[c] = s_in_[c];
    *s_out = s_out_;
}

void Upsampler::clear_dataset()
{
    for (auto& p : snaps_) release(p);
    snaps_.clear();
}

int Upsampler::append(const float* planes4, const float* omega, const float* target, int h, int w, cudaStream_t s)
{
    if (!snaps_.empty() && (h != snap_h_ || w != snap_w_)) {
        err = "upsampler: training pairs must share one grid";
        return 1;
    }
    const long long hw = (long long)h * w;
    size_t free_b = 0, total_b = 0;
    LRN_CHECK(cudaMemGetInfo(&free_b, &total_b), "append");
    if ((double)free_b < 11.0 * hw * sizeof(float) + 8e9) {
        err = "upsampler: device memory full (training pairs keep 8 GB free)";
        return 1;
    }
    float* p = nullptr;
    LRN_CHECK(alloc(&p, 11 * hw), "append");
    LRN_CHECK(cudaMemcpyAsync(p, planes4, sizeof(float) * 4 * hw, cudaMemcpyDeviceToDevice, s), "append");
    LRN_CHECK(cudaMemcpyAsync(p + 4 * hw, omega, sizeof(float) * 3 * hw, cudaMemcpyDeviceToDevice, s), "append");
    LRN_CHECK(cudaMemcpyAsync(p + 7 * hw, target, sizeof(float) * 4 * hw, cudaMemcpyDeviceToDevice, s), "append");
    snaps_.push_back(p);
    snap_h_ = h;
    snap_w_ = w;
    return 0;
}

int Upsampler::fit_scales(cudaStream_t s)
{
    if (snaps_.empty()) {
        err = "upsampler: no training pairs";
        return 1;
    }
    const int n = (int)snaps_.size();
    const long long hw = (long long)snap_h_ * snap_w_;
    const float** dp = nullptr;
    double* acc = nullptr;
    LRN_CHECK(alloc(&dp, n), "fit_scales");
    LRN_CHECK(alloc(&acc, kInCh + 1), "fit_scales");
    LRN_CHECK(cudaMemcpyAsync(dp, snaps_.data(), sizeof(float*) * n, cudaMemcpyHostToDevice, s), "fit_scales");
    LRN_CHECK(cudaMemsetAsync(acc, 0, sizeof(double) * (kInCh + 1), s), "fit_scales");
    for (int c = 0; c < kInCh; ++c) LRN_CHECK(launch_sumsq_ptrs(dp, n, c * hw, hw, acc + c, s), "fit_scales");
    LRN_CHECK(launch_sumsq_ptrs(dp, n, 7 * hw, 4 * hw, acc + kInCh, s), "fit_scales");
    double h[kInCh + 1];
    LRN_CHECK(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s), "fit_scales");
    LRN_CHECK(cudaStreamSynchronize(s), "fit_scales");
    release(dp);
    release(acc);
    double sin[kInCh];
    for (int c = 0; c < kInCh; ++c) sin[c] = std::sqrt(h[c] / ((double)n * hw));
    set_scales(sin, std::sqrt(h[kInCh] / ((double)n * 4 * hw)));
    return 0;
}

int Upsampler::ensure(int B, int h, int w)
{
    if (w % kTile != 0 || h < 1 || B < 1) {
        err = "upsampler: the map grid width must be a multiple of 128";
        return 1;
    }
    const long long n = (long long)B * h * w;
    if (B > cap_B_ || h != cap_h_ || w != cap_w_ || n > (long long)cap_B_ * cap_h_ * cap_w_) {
        release(x0_);
        for (auto& p : act_) release(p);
        for (auto& p : hid_) release(p);
        act_.assign(nb_ + 1, nullptr);
        hid_.assign(std::max(1, nb_), nullptr);
        release(da_[0]);
        release(da_[1]);
        release(dh_);
        release(dout_);
        release(out32_);
        release(tgt_);
        release(part_);
        release(dbpart_);
        LRN_CHECK(alloc(&x0_, n * kHeadIn), "buffers");
        for (auto& p : act_) LRN_CHECK(alloc(&p, n * ch_), "buffers");
        for (auto& p : hid_) LRN_CHECK(alloc(&p, n * ch_), "buffers");
        LRN_CHECK(alloc(&da_[0], n * ch_), "buffers");
        LRN_CHECK(alloc(&da_[1], n * ch_), "buffers");
        LRN_CHECK(alloc(&dh_, n * ch_), "buffers");
        LRN_CHECK(alloc(&dout_, n * kTailOut), "buffers");
        LRN_CHECK(alloc(&out32_, n * kTailOut), "buffers");
        LRN_CHECK(alloc(&tgt_, 4 * n), "buffers");
        const int rows = B * h;
        part_cap_ = conv_grid(rows, w, dw_rows_per_cta(rows, w));
        LRN_CHECK(alloc(&part_, (long long)part_cap_ * 3 * 128 * 32), "buffers");
        LRN_CHECK(alloc(&dbpart_, (long long)part_cap_ * 32), "buffers");
        cap_B_ = B;
        cap_h_ = h;
        cap_w_ = w;
    }
    return ensure_ptrs(B);
}

int Upsampler::ensure_fft(int B, int h, int w)
{
    const long long n = (long long)B * h * w;
    if (B != fft_B_ || h != fft_h_ || w != fft_w_) {
        fft::plan_destroy(fft_);
        fft_B_ = 0;
        release(rbuf_);
        release(rspec_);
        release(tspec_);
        const long long nspec = (long long)B * 2 * h * (w + 1);
        LRN_CHECK(alloc(&rbuf_, 4 * n), "buffers");
        LRN_CHECK(alloc(&rspec_, nspec), "buffers");
        LRN_CHECK(alloc(&tspec_, nspec), "buffers");
        if (fft::plan_create(fft_, 2 * w, 2 * h, false, nullptr)) {
            err = "upsampler: FFT plan creation failed";
            return 1;
        }
        fft_B_ = B;
        fft_h_ = h;
        fft_w_ = w;
    }
    return 0;
}

int Upsampler::ensure_ptrs(int B)
{
    if (3 * B > ptr_cap_) {
        release(d_ptrs_);
        LRN_CHECK(alloc(&d_ptrs_, 3 * B), "buffers");
        ptr_cap_ = 3 * B;
    }
    return 0;
}

int Upsampler::prepare(cudaStream_t s)
{
    if (prepared_) return 0;
    LRN_CHECK(launch_prepare_weights(d_layers_, (int)layers_.size(), max_w_, params_, wf_, wb_, s), "prepare");
    ++launches;
    prepared_ = true;
    return 0;
}

int Upsampler::conv(int layer, bool flipped, const bf16* in, const bf16* mask, const bf16* res, bf16* out,
                    float* out32, bool bias, bool relu, int B, int h, int w, cudaStream_t s)
{
    const LayerDesc& L = layers_[(size_t)layer];
    ConvArgs a;
    a.in = in;
    a.wt = flipped ? wb_ + L.wb : wf_ + L.wf;
    a.bias = bias ? params_ + L.b : nullptr;
    a.mask = mask;
    a.res = res;
    a.out = out;
    a.out_f32 = out32;
    a.H = h;
    a.W = w;
    a.rows = B * h;
    a.relu = relu ? 1 : 0;
    a.rows_per_cta = conv_rows_per_cta(a.rows, h, w);
    a.status = d_status_;
    LRN_CHECK(launch_conv3x3(flipped ? L.cout : L.cin, flipped ? L.cin : L.cout, a, s), "conv3x3");
    ++launches;
    return 0;
}

int Upsampler::dw(int layer, const bf16* x, const bf16* dy, int B, int h, int w, cudaStream_t s)
{
    const LayerDesc& L = layers_[(size_t)layer];
    DwArgs d;
    d.x = x;
    d.dy = dy;
    d.part = part_;
    d.dbpart = dbpart_;
    d.H = h;
    d.W = w;
    d.rows = B * h;
    d.rows_per_cta = dw_rows_per_cta(d.rows, w);
    d.status = d_status_;
    const int grid = conv_grid(d.rows, w, d.rows_per_cta);
    if (grid > part_cap_) {
        err = "upsampler: gradient partials buffer too small";
        return 1;
    }
    LRN_CHECK(launch_conv3x3_dw(L.cin, L.cout, d, grid, s), "conv3x3 weight gradient");
    LRN_CHECK(launch_dw_reduce(L.cin, L.cout, part_, dbpart_, grid, grads_ + L.w, grads_ + L.b, s), "reduce");
    launches += 2;
    return 0;
}

int Upsampler::forward(int B, int h, int w, bool keep, cudaStream_t s)
{
    auto a = [&](int i) { return keep ? act_[(size_t)i] : act_[(size_t)(i & 1)]; };
    auto hb = [&](int i) { return keep ? hid_[(size_t)i] : hid_[0]; };
    if (conv(0, false, x0_, nullptr, nullptr, a(0), nullptr, true, false, B, h, w, s)) return 1;
    for (int i = 0; i < nb_; ++i) {
        if (conv(1 + 2 * i, false, a(i), nullptr, nullptr, hb(i), nullptr, true, true, B, h, w, s)) return 1;
        if (conv(2 + 2 * i, false, hb(i), nullptr, a(i), a(i + 1), nullptr, true, false, B, h, w, s)) return 1;
    }
    return conv(2 * nb_ + 1, false, a(nb_), nullptr, nullptr, nullptr, out32_, true, false, B, h, w, s);
}

int Upsampler::backward(int B, int h, int w, cudaStream_t s)
{
    const int tail = 2 * nb_ + 1;
    if (dw(tail, act_[(size_t)nb_], dout_, B, h, w, s)) return 1;
    if (conv(tail, true, dout_, nullptr, nullptr, da_[0], nullptr, false, false, B, h, w, s)) return 1;
    int cur = 0;
    for (int i = nb_ - 1; i >= 0; --i) {
        if (dw(2 + 2 * i, hid_[(size_t)i], da_[cur], B, h, w, s)) return 1;
        if (conv(2 + 2 * i, true, da_[cur], hid_[(size_t)i], nullptr, dh_, nullptr, false, false, B, h, w, s)) return 1;
        if (dw(1 + 2 * i, act_[(size_t)i], dh_, B, h, w, s)) return 1;
        if (conv(1 + 2 * i, true, dh_, nullptr, da_[cur], da_[cur ^ 1], nullptr, false, false, B, h, w, s)) return 1;
        cur ^= 1;
    }
    return dw(0, x0_, da_[cur], B, h, w, s);
}

double Upsampler::mean_ratio(const double* acc, int B)
{
    double m = 0;
    for (int b = 0; b < B; ++b) m += acc[2 * b + 1] > 0 ? acc[2 * b] / acc[2 * b + 1] : 0.0;
    return m / B;
}

int Upsampler::loss(int B, int h, int w, double* acc, cudaStream_t s)
{
    if (cut_ <= 0) {
        LRN_CHECK(launch_loss(out32_, tgt_, B, h, w, dout_, acc, s), "loss");
        ++launches;
        return 0;
    }
    if (ensure_fft(B, h, w)) return 1;
    LRN_CHECK(launch_shuffle_resid(out32_, tgt_, B, h, w, rbuf_, s), "loss");
    const long long rd = 4ll * h * w, sd = 2ll * h * (w + 1);
    LRN_CHECK(fft::r2c(fft_, rbuf_, rspec_, B, s, rd, sd), "loss FFT");
    LRN_CHECK(fft::r2c(fft_, tgt_, tspec_, B, s, rd, sd), "loss FFT");
    LRN_CHECK(launch_spec_loss(rspec_, tspec_, B, 2 * h, 2 * w, cut_, acc, s), "loss");
    LRN_CHECK(fft::c2r(fft_, rspec_, rbuf_, B, s, sd, rd), "loss FFT");
    LRN_CHECK(launch_grad_pack(rbuf_, acc, B, h, w, dout_, s), "loss");
    launches += 3;
    return 0;
}

int Upsampler::loss_grad(const float* const* planes, const float* const* omega, const float* const* target, int B,
                         int h, int w, double* loss, cudaStream_t s)
{
    if (!params_) return 1;
    if (B > kMaxBatch) {
        err = "upsampler: at most 256 samples";
        return 1;
    }
    if (ensure(B, h, w) || prepare(s)) return 1;
    std::vector<const float*> ptr(3 * (size_t)B);
    for (int b = 0; b < B; ++b) {
        ptr[(size_t)b] = planes[b];
        ptr[(size_t)(B + b)] = omega[b];
        ptr[(size_t)(2 * B + b)] = target[b];
    }
    LRN_CHECK(cudaMemcpyAsync(d_ptrs_, ptr.data(), sizeof(float*) * 3 * B, cudaMemcpyHostToDevice, s), "loss_grad");
    LRN_CHECK(launch_assemble(d_ptrs_, d_ptrs_ + B, d_ptrs_ + 2 * B, B, h, w, d_sin_, (float)(1.0 / s_out_), x0_, tgt_,
                              s),
              "assemble");
    if (forward(B, h, w, true, s)) return 1;
    LRN_CHECK(cudaMemsetAsync(d_loss_, 0, 2 * sizeof(double) * B, s), "loss_grad");
    if (this->loss(B, h, w, d_loss_, s)) return 1;
    if (backward(B, h, w, s)) return 1;
    int st = 0;
    std::vector<double> acc(2 * (size_t)B);
    LRN_CHECK(cudaMemcpyAsync(acc.data(), d_loss_, 2 * sizeof(double) * B, cudaMemcpyDeviceToHost, s), "loss_grad");
    LRN_CHECK(cudaMemcpyAsync(&st, d_status_, sizeof(int), cudaMemcpyDeviceToHost, s), "loss_grad");
    LRN_CHECK(cudaStreamSynchronize(s), "loss_grad");
    if (st) {
        err = "upsampler: a tensor-core wait ran out";
        return 1;
    }
    *loss = cut_ > 0 ? mean_ratio(acc.data(), B) : acc[0];
    return 0;
}

int Upsampler::train(int iters, int batch, double lr, uint64_t seed, double* loss, cudaStream_t s)
{
    if (snaps_.empty()) {
        err = "upsampler: no training pairs";
        return 1;
    }
    if (iters < 1 || batch < 1 || batch > kMaxBatch) {
        err = "upsampler: iterations >= 1 and 1 <= batch <= 256";
        return 1;
    }
    if (!scaled_ && fit_scales(s)) return 1;
    const int h = snap_h_, w = snap_w_;
    const long long hw = (long long)h * w;
    if (ensure(batch, h, w) || prepare(s)) return 1;
    launches = 0;
    // every iteration's batch: 3 x batch pointers, drawn up front
    std::mt19937_64 g(seed);
    std::vector<const float*> ptr(3 * (size_t)batch * iters);
    for (int it = 0; it < iters; ++it)
        for (int b = 0; b < batch; ++b) {
            const float* p = snaps_[(size_t)(g() % snaps_.size())];
            const size_t base = 3 * (size_t)batch * it;
            ptr[base + b] = p;
            ptr[base + batch + b] = p + 4 * hw;
            ptr[base + 2 * batch + b] = p + 7 * hw;
        }
    const float** dptr = nullptr;
    double* dloss = nullptr;
    LRN_CHECK(alloc(&dptr, (long long)ptr.size()), "train");
    LRN_CHECK(alloc(&dloss, 2ll * batch * iters), "train");
    LRN_CHECK(cudaMemcpyAsync(dptr, ptr.data(), sizeof(float*) * ptr.size(), cudaMemcpyHostToDevice, s), "train");
    LRN_CHECK(cudaMemsetAsync(dloss, 0, sizeof(double) * 2 * batch * iters, s), "train");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    for (int it = 0; it < iters; ++it) {
        const float* const* p = dptr + 3 * (size_t)batch * it;
        LRN_CHECK(launch_assemble(p, p + batch, p + 2 * batch, batch, h, w, d_sin_, (float)(1.0 / s_out_), x0_, tgt_, s),
                  "assemble");
        if (forward(batch, h, w, true, s)) return 1;
        if (this->loss(batch, h, w, dloss + 2ll * batch * it, s)) return 1;
        if (backward(batch, h, w, s)) return 1;
        ++adam_t_;
        const float c1 = (float)(1.0 - std::pow((double)kB1, (double)adam_t_));
        const float c2 = (float)(1.0 - std::pow((double)kB2, (double)adam_t_));
        LRN_CHECK(launch_adam(params_, grads_, adam_m_, adam_v_, n_params_, (float)lr, kB1, kB2, kEps, c1, c2, s),
                  "adam");
        launches += 2;
        prepared_ = false;
        if (prepare(s)) return 1;
    }
    cudaEventRecord(e1, s);
    std::vector<double> hl(2 * (size_t)batch * iters);
    int st = 0;
    LRN_CHECK(cudaMemcpyAsync(hl.data(), dloss, sizeof(double) * hl.size(), cudaMemcpyDeviceToHost, s), "train");
    LRN_CHECK(cudaMemcpyAsync(&st, d_status_, sizeof(int), cudaMemcpyDeviceToHost, s), "train");
    LRN_CHECK(cudaStreamSynchronize(s), "train");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    release(dptr);
    release(dloss);
    train_seconds = ms * 1e-3;
    train_steps += iters;
    if (st) {
        err = "upsampler: a tensor-core wait ran out";
        return 1;
    }
    const int k = std::min(iters, 16);
    double m = 0;
    for (int i = iters - k; i < iters; ++i)
        m += cut_ > 0 ? mean_ratio(hl.data() + 2 * (size_t)batch * i, batch) : hl[2 * (size_t)batch * i];
    if (loss) *loss = m / k;
    return 0;
}

int Upsampler::infer(const float* planes4, const float* omega, int h, int w, float* fine, cudaStream_t s)
{
    if (!params_) return 1;
    if (ensure(1, h, w) || prepare(s)) return 1;
    launches = 0;
    const float* ptr[3] = {planes4, omega, nullptr};
    LRN_CHECK(cudaMemcpyAsync(d_ptrs_, ptr, sizeof(ptr), cudaMemcpyHostToDevice, s), "infer");
    LRN_CHECK(launch_assemble(d_ptrs_, d_ptrs_ + 1, nullptr, 1, h, w, d_sin_, 1.f, x0_, nullptr, s), "assemble");
    if (forward(1, h, w, false, s)) return 1;
    LRN_CHECK(launch_shuffle_out(out32_, nullptr, h, w, (float)s_out_, fine, s), "shuffle");
    launches += 2;
    return 0;
}

int Upsampler::time_infer(int h, int w, int iters, double* ms, cudaStream_t s)
{
    const long long hw = (long long)h * w;
    float* in = nullptr;
    float* fine = nullptr;
    LRN_CHECK(alloc(&in, kInCh * hw), "time_infer");
    LRN_CHECK(alloc(&fine, 4 * hw), "time_infer");
    LRN_CHECK(cudaMemsetAsync(in, 0, sizeof(float) * kInCh * hw, s), "time_infer");
    int rc = 0;
    for (int i = 0; i < 2 && !rc; ++i) rc = infer(in, in + 4 * hw, h, w, fine, s);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    for (int i = 0; i < iters && !rc; ++i) rc = infer(in, in + 4 * hw, h, w, fine, s);
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    release(in);
    release(fine);
    if (rc) return rc;
    LRN_CHECK(e, "time_infer");
    *ms = iters > 0 ? t / iters : 0.0;
    return 0;
}

int Upsampler::save(const std::string& path) const
{
    std::vector<float> p((size_t)n_params_);
    if (get_params(p.data(), n_params_)) return 1;
    std::ofstream f(path, std::ios::binary);
    if (!f) return 1;
    const int32_t hdr[3] = {nb_, ch_, cut_};
    const int64_t n = n_params_;
    f.write(kMagic, 8);
    f.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
    f.write(reinterpret_cast<const char*>(&n), sizeof(n));
    f.write(reinterpret_cast<const char*>(s_in_), sizeof(s_in_));
    f.write(reinterpret_cast<const char*>(&s_out_), sizeof(s_out_));
    f.write(reinterpret_cast<const char*>(p.data()), sizeof(float) * p.size());
    return f ? 0 : 1;
}

int Upsampler::load(const std::string& path)
{
    std::ifstream f(path, std::ios::binary);
    char magic[8];
    int32_t hdr[3];
    int64_t n = 0;
    double sin[kInCh], sout = 1;
    if (!f.read(magic, 8) || std::memcmp(magic, kMagic, 8) != 0 || !f.read(reinterpret_cast<char*>(hdr), sizeof(hdr)) ||
        !f.read(reinterpret_cast<char*>(&n), sizeof(n))) {
        err = "upsampler: " + path + " is not an upsampler file";
        return 1;
    }
    if (hdr[0] != nb_ || hdr[1] != ch_ || n != n_params_) {
        err = "upsampler: " + path + " holds a network of another shape";
        return 1;
    }
    std::vector<float> p((size_t)n);
    if (!f.read(reinterpret_cast<char*>(sin), sizeof(sin)) || !f.read(reinterpret_cast<char*>(&sout), sizeof(sout)) ||
        !f.read(reinterpret_cast<char*>(p.data()), sizeof(float) * p.size())) {
        err = "upsampler: " + path + " is truncated";
        return 1;
    }
    set_scales(sin, sout);
    cut_ = hdr[2];
    return set_params(p.data(), n);
}

}  // namespace lrn
}  // namespace cmm
