// learned.hpp -- the learned psi upsampler.
//
// A residual network of 3x3 periodic convolutions maps the cheap coarse-grid fields (psi
// and its Hermite derivatives from omega sampled on the map grid, that omega and its
// gradient) to the vorticity the map-grid samples miss, on the psi grid (twice the map
// grid: the 2 x 2 sub-pixels of each map cell): omega sampled through the map on the psi
// grid minus the spectral interpolation of the map-grid samples.  That sub-grid content is
// local, and small where the flow is resolved, so BF16 relative errors on it become small
// psi errors: the learned psi is the cheap psi plus the psi solve of the prediction.  Layout: activations BF16,
// pixel-major [rows][W][C] with rows = images x H; the image is periodic in both
// directions.  Layers: head conv 7(16) -> C, B residual blocks (conv, ReLU, conv, + skip),
// tail conv C -> 4(16) whose four channels are the 2 x 2 sub-pixels of the psi grid.
//
// Kernels (learned_kernels.cu): forward / input-gradient convolution and weight-gradient
// convolution on the tcgen05 tensor cores (BF16 operands, FP32 accumulation in TMEM),
// and the small elementwise steps (input assembly, loss and its gradient, sub-pixel
// shuffle, weight preparation, Adam).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "fft.hpp"

#include <cstdint>
#include <random>
#include <string>
#include <vector>

namespace cmm {
namespace lrn {

using bf16 = __nv_bfloat16;

constexpr int kTile = 128;     // pixels per tile: one row segment (W must be a multiple)
constexpr int kPitch = 130;    // staged pixels per row (the tile and one halo pixel each side)
constexpr int kInCh = 7;       // psi, psi_x, psi_y, psi_xy (cheap), omega, omega_x, omega_y (map grid)
constexpr int kHeadIn = 16;    // input channels padded to the K = 16 MMA slice
constexpr int kTailOut = 16;   // output channels padded to N = 16 (4 used: the 2 x 2 sub-pixels)
constexpr int kMaxBatch = 256;

// out = [relu](conv3x3(in, w) + bias) [* (mask > 0)] [+ res]
struct ConvArgs {
    const bf16* in = nullptr;    // [rows][W][cin]
    const bf16* wt = nullptr;    // prepared weights [9][cin / 8][cout][8]
    const float* bias = nullptr; // [cout] or null
    const bf16* mask = nullptr;  // [rows][W][cout] or null
    const bf16* res = nullptr;   // [rows][W][cout] or null
    bf16* out = nullptr;         // [rows][W][cout] or null
    float* out_f32 = nullptr;    // [rows][W][cout] or null
    int H = 0, W = 0, rows = 0, relu = 0, rows_per_cta = 1;
    int* status = nullptr;       // set to 1 when a tensor-core wait ran out
};
// strip height of the forward kernel for rows / H images of H x W
int conv_rows_per_cta(int rows, int H, int W);
int conv_grid(int rows, int W, int rows_per_cta);
cudaError_t launch_conv3x3(int cin, int cout, const ConvArgs& a, cudaStream_t s);

// per-CTA partial weight and bias gradients: part[cta][dy][dx * cin + ci][co], dbpart[cta][co]
struct DwArgs {
    const bf16* x = nullptr;     // [rows][W][cin]
    const bf16* dy = nullptr;    // [rows][W][cout]
    float* part = nullptr;
    float* dbpart = nullptr;
    int H = 0, W = 0, rows = 0, rows_per_cta = 1;
    int* status = nullptr;
};
int dw_rows_per_cta(int rows, int W);
cudaError_t launch_conv3x3_dw(int cin, int cout, const DwArgs& a, int grid, cudaStream_t s);
// dw[tap][ci][co] (tap = 3 dy + dx, offsets dy - 1, dx - 1), db[co]; fixed summation order
cudaError_t launch_dw_reduce(int cin, int cout, const float* part, const float* dbpart, int grid, float* dw,
                             float* db, cudaStream_t s);

struct LayerDesc {
    int cin, cout;
    long long w, b;      // offsets of W[9][cin][cout] and b[cout] in the parameter vector
    long long wf, wb;    // offsets of the prepared forward / input-gradient weights
};
// FP32 parameters -> BF16 forward weights [9][cin/8][cout][8] and input-gradient weights
// (taps flipped, channels swapped) [9][cout/8][cin][8]
cudaError_t launch_prepare_weights(const LayerDesc* d_layers, int n_layers, int max_w, const float* params, bf16* wf,
                                   bf16* wb, cudaStream_t s);
cudaError_t launch_adam(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                        float eps, float c1, float c2, cudaStream_t s);
// network input (BF16, 16 channels, scaled by 1/s_in) and scaled target (FP32, 2h x 2w) of
// B samples; planes[b] -> 4 planes of h x w, omega[b] -> 3 planes (omega, omega_x, omega_y),
// target[b] -> 2h x 2w or null
cudaError_t launch_assemble(const float* const* planes, const float* const* omega, const float* const* target, int B,
                            int h, int w, const float* s_in, float inv_out, bf16* x0, float* tgt, cudaStream_t s);
// mean squared error of the shuffled tail output against tgt, its gradient (BF16, 16
// channels) and the loss (added to *loss)
cudaError_t launch_loss(const float* out16, const float* tgt, int B, int h, int w, bf16* dout, double* loss,
                        cudaStream_t s);
// tail output (channels 0..3) -> 2h x 2w field: fine[2y + i][2x + j] = base[y][x] + scale out[y][x][2i + j]
// (base may be null)
cudaError_t launch_shuffle_out(const float* out16, const float* base, int h, int w, float scale, float* fine,
                               cudaStream_t s);
// out = a - b
cudaError_t launch_sub(const float* a, const float* b, long long n, float* out, cudaStream_t s);
// spectral (psi-space) loss: r = shuffled tail output - target (B x 2h x 2w); on the half
// spectra of r and the target, per sample acc[2b..2b+1] += {sum w |R|^2, sum w |T|^2} with
// w = 1/|k|^4 on 0 < |k| <= cut and R *= w; the loss is the mean over samples of
// num / den, the tail's output gradient 2 C2R(w R_b) / (B den_b)
cudaError_t launch_shuffle_resid(const float* out16, const float* tgt, int B, int h, int w, float* r, cudaStream_t s);
cudaError_t launch_spec_loss(float2* R, const float2* T, int B, int H2, int W2, int cut, double* acc, cudaStream_t s);
cudaError_t launch_grad_pack(const float* g, const double* acc, int B, int h, int w, bf16* dout, cudaStream_t s);
// sum of squares per channel over n fields of `count` values each: out[k] += sum x^2
cudaError_t launch_sumsq_ptrs(const float* const* ptrs, int n, long long offset, long long count, double* out,
                              cudaStream_t s);

// out4 += {max |a - e|, max |e|, sum (a - e)^2, sum e^2} over a[i sa], e[i se], i < n
// (out4 zeroed by the caller; maxima of non-negative values through their bit patterns)
cudaError_t launch_diff_stats(const float* a, long long sa, const float* e, long long se, long long n, double* out4,
                              cudaStream_t s);

// The network, its optimiser, its training pairs and its work buffers.
class Upsampler {
public:
    Upsampler(int blocks = 6, int channels = 32);
    ~Upsampler();
    Upsampler(const Upsampler&) = delete;
    Upsampler& operator=(const Upsampler&) = delete;

    int init_weights(uint64_t seed);
    long long n_params() const { return n_params_; }
    int blocks() const { return nb_; }
    int set_params(const float* host, long long n);
    int get_params(float* host, long long n) const;
    int get_grads(float* host, long long n) const;
    void set_scales(const double* s_in, double s_out);
    void get_scales(double* s_in, double* s_out) const;

    // one training pair from device fields of the map grid (h x w) and the psi grid
    // (2h x 2w): the 4 cheap psi planes, omega and its gradient (3 planes), and the target
    // (omega on the psi grid minus the spectral interpolation of the map-grid samples)
    int append(const float* planes4, const float* omega, const float* target, int h, int w, cudaStream_t s);
    int dataset_size() const { return (int)snaps_.size(); }
    void clear_dataset();
    int fit_scales(cudaStream_t s);                 // RMS of each input channel and of the target
    // Loss: with a spectral cut-off set (the psi solve's, in integer wavenumbers of the 2 pi
    // periodic domain) the mean over the batch of each sample's relative psi-space error
    // sum w |FFT(pred - target)|^2 / sum w |FFT(target)|^2, w = 1/|k|^4 on 0 < |k| <= cut,
    // i.e. the part of the prediction the psi solve keeps, weighted as psi; with cut 0 the
    // mean squared error.
    void set_spectral_cut(int cut) { cut_ = cut; }
    int spectral_cut() const { return cut_; }
    // iters Adam steps on batches drawn from the pairs (mt19937_64(seed)); the mean loss of
    // the last min(iters, 16) steps in *loss
    int train(int iters, int batch, double lr, uint64_t seed, double* loss, cudaStream_t s);
    // loss and gradient (kept for get_grads) of B samples given as device fields
    int loss_grad(const float* const* planes, const float* const* omega, const float* const* target, int B, int h,
                  int w, double* loss, cudaStream_t s);
    // the predicted sub-grid vorticity on the psi grid (2h x 2w)
    int infer(const float* planes4, const float* omega, int h, int w, float* fine, cudaStream_t s);

    // device time of one inference on an h x w map grid (iters repeats after 2 warm-ups,
    // zero inputs: the cost does not depend on the values)
    int time_infer(int h, int w, int iters, double* ms, cudaStream_t s);

    int save(const std::string& path) const;
    int load(const std::string& path);

    std::string err;
    long long train_steps = 0;
    double train_seconds = 0;       // device time of the last train() call
    long long launches = 0;         // kernels launched by the last train() / infer()

private:
    int ensure(int B, int h, int w);
    int ensure_fft(int B, int h, int w);
    int ensure_ptrs(int B);
    int prepare(cudaStream_t s);
    int forward(int B, int h, int w, bool keep, cudaStream_t s);
    int loss(int B, int h, int w, double* acc, cudaStream_t s);   // acc: {loss} or B x {num, den}
    static double mean_ratio(const double* acc, int B);
    int backward(int B, int h, int w, cudaStream_t s);
    int fail(const char* what, cudaError_t e);
    int conv(int layer, bool flipped, const bf16* in, const bf16* mask, const bf16* res, bf16* out, float* out32,
             bool bias, bool relu, int B, int h, int w, cudaStream_t s);
    int dw(int layer, const bf16* x, const bf16* dy, int B, int h, int w, cudaStream_t s);

    int nb_, ch_;
    std::vector<LayerDesc> layers_;
    long long n_params_ = 0, n_wf_ = 0;
    float *params_ = nullptr, *grads_ = nullptr, *adam_m_ = nullptr, *adam_v_ = nullptr;
    bf16 *wf_ = nullptr, *wb_ = nullptr;
    LayerDesc* d_layers_ = nullptr;
    bool prepared_ = false;
    long long adam_t_ = 0;
    double s_in_[kInCh] = {1, 1, 1, 1, 1, 1, 1};
    double s_out_ = 1;
    bool scaled_ = false;
    float* d_sin_ = nullptr;
    int max_w_ = 0;

    // pairs: each one block of 11 h w floats ([4][h][w] psi planes, [3][h][w] omega planes,
    // [2h][2w] target)
    std::vector<float*> snaps_;
    int snap_h_ = 0, snap_w_ = 0;

    // work buffers for B x h x w
    int cap_B_ = 0, cap_h_ = 0, cap_w_ = 0;
    bf16* x0_ = nullptr;                 // [rows][w][16]
    std::vector<bf16*> act_;             // a_0 .. a_B (C channels)
    std::vector<bf16*> hid_;             // h_0 .. h_{B-1}
    bf16 *da_[2] = {nullptr, nullptr}, *dh_ = nullptr, *dout_ = nullptr;
    float* out32_ = nullptr;             // [rows][w][16]
    float* tgt_ = nullptr;               // [B][2h][2w]
    float *part_ = nullptr, *dbpart_ = nullptr;
    int part_cap_ = 0;
    double* d_loss_ = nullptr;
    int cut_ = 0;
    float* rbuf_ = nullptr;              // B x 2h x 2w residual / gradient
    float2 *rspec_ = nullptr, *tspec_ = nullptr;
    fft::Plan2D fft_;                    // transforms of 2h x 2w (loss)
    int fft_B_ = 0, fft_h_ = 0, fft_w_ = 0;
    int* d_status_ = nullptr;
    const float** d_ptrs_ = nullptr;     // 3 x B device pointers for assemble
    int ptr_cap_ = 0;
};

}  // namespace lrn
}  // namespace cmm
