// abi_learned.cpp -- extern "C" entry points of the learned psi (include/cmm_abi.h).
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/cmm_abi.h"
#include "abi_internal.hpp"
#include "learned.hpp"

struct cmm_upsampler {
    cmm::lrn::Upsampler* u = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
};

namespace {

constexpr size_t kIn = cmm::lrn::kInCh;

int fail(int code, const std::string& msg)
{
    cmm::set_last_error(msg);
    return code;
}

int up_rc(cmm_upsampler* u, int rc)
{
    if (rc) return fail(CMM_ERR_CUDA, u->u->err);
    return CMM_OK;
}

// device copies of host buffers, freed with the object
struct DevBuf {
    std::vector<void*> ptrs;
    ~DevBuf()
    {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    T* up(const T* host, size_t n, cudaError_t* e)
    {
        void* p = nullptr;
        if (*e != cudaSuccess) return nullptr;
        if ((*e = cudaMalloc(&p, sizeof(T) * (n ? n : 1))) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        if (host) *e = cudaMemcpy(p, host, sizeof(T) * n, cudaMemcpyHostToDevice);
        return static_cast<T*>(p);
    }
};

bool conv_shape_ok(int B, int H, int W, int cin, int cout)
{
    return B > 0 && H > 0 && W > 0 && W % cmm::lrn::kTile == 0 && (cin == 16 || cin == 32) &&
           (cout == 16 || cout == 32);
}

}  // namespace

extern "C" {

int cmm_upsampler_create(int blocks, int channels, unsigned long long seed, void* stream, cmm_upsampler** out)
{
    if (!out) return fail(CMM_ERR_PARAM, "out is NULL");
    *out = nullptr;
    if (channels != 32 || blocks < 0 || blocks > 64) return fail(CMM_ERR_UNSUPPORTED, "upsampler: 32 channels, 0..64 blocks");
    cmm_upsampler* u = new (std::nothrow) cmm_upsampler();
    if (!u) return fail(CMM_ERR_PARAM, "out of host memory");
    u->u = new (std::nothrow) cmm::lrn::Upsampler(blocks, channels);
    if (!u->u || !u->u->err.empty()) {
        std::string e = u->u ? u->u->err : "out of host memory";
        delete u->u;
        delete u;
        return fail(CMM_ERR_CUDA, e);
    }
    if (stream) {
        u->stream = static_cast<cudaStream_t>(stream);
    } else {
        if (cudaStreamCreateWithFlags(&u->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete u->u;
            delete u;
            return fail(CMM_ERR_CUDA, "cudaStreamCreate failed");
        }
        u->own_stream = true;
    }
    if (u->u->init_weights(seed)) {
        std::string e = u->u->err;
        cmm_upsampler_destroy(u);
        return fail(CMM_ERR_CUDA, e);
    }
    *out = u;
    return CMM_OK;
}

int cmm_upsampler_destroy(cmm_upsampler* u)
{
    if (!u) return CMM_OK;
    if (u->stream) cudaStreamSynchronize(u->stream);
    delete u->u;
    if (u->own_stream) cudaStreamDestroy(u->stream);
    delete u;
    return CMM_OK;
}

long long cmm_upsampler_num_params(const cmm_upsampler* u) { return u && u->u ? u->u->n_params() : 0; }

int cmm_upsampler_get_params(const cmm_upsampler* u, float* out, long long n)
{
    if (!u || !out) return fail(CMM_ERR_PARAM, "NULL argument");
    if (n != u->u->n_params()) return fail(CMM_ERR_PARAM, "parameter count mismatch");
    return u->u->get_params(out, n) ? fail(CMM_ERR_CUDA, "get_params failed") : CMM_OK;
}

int cmm_upsampler_set_params(cmm_upsampler* u, const float* in, long long n)
{
    if (!u || !in) return fail(CMM_ERR_PARAM, "NULL argument");
    if (n != u->u->n_params()) return fail(CMM_ERR_PARAM, "parameter count mismatch");
    return up_rc(u, u->u->set_params(in, n));
}

int cmm_upsampler_get_grads(const cmm_upsampler* u, float* out, long long n)
{
    if (!u || !out) return fail(CMM_ERR_PARAM, "NULL argument");
    if (n != u->u->n_params()) return fail(CMM_ERR_PARAM, "parameter count mismatch");
    return u->u->get_grads(out, n) ? fail(CMM_ERR_CUDA, "get_grads failed") : CMM_OK;
}

int cmm_upsampler_set_scales(cmm_upsampler* u, const double* s_in5, double s_out)
{
    if (!u || !s_in5) return fail(CMM_ERR_PARAM, "NULL argument");
    u->u->set_scales(s_in5, s_out);
    return CMM_OK;
}

int cmm_upsampler_get_scales(const cmm_upsampler* u, double* s_in5, double* s_out)
{
    if (!u || !s_in5 || !s_out) return fail(CMM_ERR_PARAM, "NULL argument");
    u->u->get_scales(s_in5, s_out);
    return CMM_OK;
}

int cmm_upsampler_collect(cmm_upsampler* u, cmm_ctx* c)
{
    if (!u || !c || !c->sim) return fail(CMM_ERR_STATE, "cmm_upsampler_collect needs an initialised context");
    int rc = c->sim->learned_collect(*u->u);
    if (rc) return fail(rc, c->sim->err);
    return CMM_OK;
}

int cmm_upsampler_dataset_size(const cmm_upsampler* u) { return u ? u->u->dataset_size() : 0; }

int cmm_upsampler_clear_dataset(cmm_upsampler* u)
{
    if (!u) return fail(CMM_ERR_PARAM, "upsampler is NULL");
    u->u->clear_dataset();
    return CMM_OK;
}

int cmm_upsampler_train(cmm_upsampler* u, int iters, int batch, double lr, unsigned long long seed, double* loss,
                        double* seconds)
{
    if (!u) return fail(CMM_ERR_PARAM, "upsampler is NULL");
    double l = 0;
    int rc = u->u->train(iters, batch, lr, seed, &l, u->stream);
    if (rc) return fail(CMM_ERR_CUDA, u->u->err);
    if (loss) *loss = l;
    if (seconds) *seconds = u->u->train_seconds;
    return CMM_OK;
}

int cmm_upsampler_loss_grad(cmm_upsampler* u, const float* inputs, const float* targets, int B, int h, int w,
                            int cut, double* loss)
{
    if (!u || !inputs || !targets || !loss) return fail(CMM_ERR_PARAM, "NULL argument");
    if (B < 1 || h < 1 || w < 1 || w % cmm::lrn::kTile != 0) return fail(CMM_ERR_PARAM, "bad shape (w % 128 != 0?)");
    const size_t hw = (size_t)h * w;
    DevBuf d;
    cudaError_t e = cudaSuccess;
    float* din = d.up(inputs, (size_t)B * kIn * hw, &e);
    float* dt = d.up(targets, (size_t)B * 4 * hw, &e);
    if (e != cudaSuccess) return fail(CMM_ERR_CUDA, cudaGetErrorString(e));
    std::vector<const float*> pl((size_t)B), om((size_t)B), tg((size_t)B);
    for (int b = 0; b < B; ++b) {
        pl[(size_t)b] = din + (size_t)b * kIn * hw;
        om[(size_t)b] = din + (size_t)b * kIn * hw + 4 * hw;
        tg[(size_t)b] = dt + (size_t)b * 4 * hw;
    }
    const int keep = u->u->spectral_cut();
    u->u->set_spectral_cut(cut);
    const int rc = u->u->loss_grad(pl.data(), om.data(), tg.data(), B, h, w, loss, u->stream);
    u->u->set_spectral_cut(keep);
    return up_rc(u, rc);
}

int cmm_upsampler_infer(cmm_upsampler* u, const float* inputs, int h, int w, float* fine)
{
    if (!u || !inputs || !fine) return fail(CMM_ERR_PARAM, "NULL argument");
    if (h < 1 || w < 1 || w % cmm::lrn::kTile != 0) return fail(CMM_ERR_PARAM, "bad shape (w % 128 != 0?)");
    const size_t hw = (size_t)h * w;
    DevBuf d;
    cudaError_t e = cudaSuccess;
    float* din = d.up(inputs, kIn * hw, &e);
    float* dout = d.up<float>(nullptr, 4 * hw, &e);
    if (e != cudaSuccess) return fail(CMM_ERR_CUDA, cudaGetErrorString(e));
    int rc = u->u->infer(din, din + 4 * hw, h, w, dout, u->stream);
    if (rc) return up_rc(u, rc);
    e = cudaMemcpyAsync(fine, dout, sizeof(float) * 4 * hw, cudaMemcpyDeviceToHost, u->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(u->stream);
    return e == cudaSuccess ? CMM_OK : fail(CMM_ERR_CUDA, cudaGetErrorString(e));
}

int cmm_upsampler_evaluate(cmm_upsampler* u, cmm_ctx* c, double* out6)
{
    if (!u || !c || !c->sim || !out6) return fail(CMM_ERR_STATE, "cmm_upsampler_evaluate needs an initialised context");
    int rc = c->sim->learned_evaluate(*u->u, out6);
    if (rc) return fail(rc, c->sim->err);
    return CMM_OK;
}

int cmm_upsampler_time_infer(cmm_upsampler* u, int h, int w, int iters, double* ms)
{
    if (!u || !ms) return fail(CMM_ERR_PARAM, "NULL argument");
    if (h < 1 || w < 1 || w % cmm::lrn::kTile != 0 || iters < 1) return fail(CMM_ERR_PARAM, "bad shape or iters");
    return up_rc(u, u->u->time_infer(h, w, iters, ms, u->stream));
}

int cmm_upsampler_save(const cmm_upsampler* u, const char* path)
{
    if (!u || !path) return fail(CMM_ERR_PARAM, "NULL argument");
    return u->u->save(path) ? fail(CMM_ERR_IO, std::string("cannot write ") + path) : CMM_OK;
}

int cmm_upsampler_load(cmm_upsampler* u, const char* path)
{
    if (!u || !path) return fail(CMM_ERR_PARAM, "NULL argument");
    return u->u->load(path) ? fail(CMM_ERR_IO, u->u->err) : CMM_OK;
}

int cmm_attach_upsampler(cmm_ctx* c, cmm_upsampler* u, int exact_every, double tol)
{
    if (!c || !c->sim) return fail(CMM_ERR_STATE, "cmm_attach_upsampler before cmm_init");
    int rc = c->sim->attach_upsampler(u ? u->u : nullptr, exact_every, tol);
    if (rc) return fail(rc, c->sim->err);
    return CMM_OK;
}

int cmm_conv3x3(const unsigned short* x, const unsigned short* w, const float* bias, const unsigned short* mask,
                const unsigned short* res, int relu, int B, int H, int W, int cin, int cout, float* out_f32,
                unsigned short* out_bf16)
{
    using namespace cmm::lrn;
    if (!x || !w || (!out_f32 && !out_bf16)) return fail(CMM_ERR_PARAM, "NULL argument");
    if (!conv_shape_ok(B, H, W, cin, cout)) return fail(CMM_ERR_PARAM, "cmm_conv3x3: cin, cout in {16, 32}, W % 128 == 0");
    const size_t n = (size_t)B * H * W;
    // weights [9][cin][cout] -> [9][cin / 8][cout][8]
    std::vector<unsigned short> wp((size_t)9 * cin * cout);
    for (int tap = 0; tap < 9; ++tap)
        for (int ci = 0; ci < cin; ++ci)
            for (int co = 0; co < cout; ++co)
                wp[(((size_t)tap * (cin / 8) + ci / 8) * cout + co) * 8 + ci % 8] = w[((size_t)tap * cin + ci) * cout + co];
    DevBuf d;
    cudaError_t e = cudaSuccess;
    ConvArgs a;
    a.in = reinterpret_cast<const bf16*>(d.up(x, n * cin, &e));
    a.wt = reinterpret_cast<const bf16*>(d.up(wp.data(), wp.size(), &e));
    a.bias = bias ? d.up(bias, (size_t)cout, &e) : nullptr;
    a.mask = mask ? reinterpret_cast<const bf16*>(d.up(mask, n * cout, &e)) : nullptr;
    a.res = res ? reinterpret_cast<const bf16*>(d.up(res, n * cout, &e)) : nullptr;
    a.out = out_bf16 ? reinterpret_cast<bf16*>(d.up<unsigned short>(nullptr, n * cout, &e)) : nullptr;
    a.out_f32 = out_f32 ? d.up<float>(nullptr, n * cout, &e) : nullptr;
    int* status = d.up<int>(nullptr, 1, &e);
    if (e == cudaSuccess) e = cudaMemset(status, 0, sizeof(int));
    if (e != cudaSuccess) return fail(CMM_ERR_CUDA, cudaGetErrorString(e));
    a.status = status;
    a.H = H;
    a.W = W;
    a.rows = B * H;
    a.relu = relu ? 1 : 0;
    a.rows_per_cta = conv_rows_per_cta(a.rows, H, W);
    e = launch_conv3x3(cin, cout, a, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && out_f32) e = cudaMemcpy(out_f32, a.out_f32, sizeof(float) * n * cout, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && out_bf16)
        e = cudaMemcpy(out_bf16, a.out, sizeof(unsigned short) * n * cout, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(CMM_ERR_CUDA, cudaGetErrorString(e));
    if (st) return fail(CMM_ERR_CUDA, "cmm_conv3x3: a tensor-core wait ran out");
    return CMM_OK;
}

int cmm_conv3x3_weight_grad(const unsigned short* x, const unsigned short* dy, int B, int H, int W, int cin, int cout,
                            float* dw, float* db)
{
    using namespace cmm::lrn;
    if (!x || !dy || !dw || !db) return fail(CMM_ERR_PARAM, "NULL argument");
    if (!conv_shape_ok(B, H, W, cin, cout)) return fail(CMM_ERR_PARAM, "cmm_conv3x3_weight_grad: cin, cout in {16, 32}, W % 128 == 0");
    const size_t n = (size_t)B * H * W;
    DwArgs a;
    a.H = H;
    a.W = W;
    a.rows = B * H;
    a.rows_per_cta = dw_rows_per_cta(a.rows, W);
    const int grid = conv_grid(a.rows, W, a.rows_per_cta);
    DevBuf d;
    cudaError_t e = cudaSuccess;
    a.x = reinterpret_cast<const bf16*>(d.up(x, n * cin, &e));
    a.dy = reinterpret_cast<const bf16*>(d.up(dy, n * cout, &e));
    a.part = d.up<float>(nullptr, (size_t)grid * 3 * 128 * cout, &e);
    a.dbpart = d.up<float>(nullptr, (size_t)grid * cout, &e);
    float* ddw = d.up<float>(nullptr, (size_t)9 * cin * cout, &e);
    float* ddb = d.up<float>(nullptr, (size_t)cout, &e);
    int* status = d.up<int>(nullptr, 1, &e);
    if (e == cudaSuccess) e = cudaMemset(status, 0, sizeof(int));
    if (e != cudaSuccess) return fail(CMM_ERR_CUDA, cudaGetErrorString(e));
    a.status = status;
    e = launch_conv3x3_dw(cin, cout, a, grid, nullptr);
    if (e == cudaSuccess) e = launch_dw_reduce(cin, cout, a.part, a.dbpart, grid, ddw, ddb, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(dw, ddw, sizeof(float) * 9 * cin * cout, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(db, ddb, sizeof(float) * cout, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(CMM_ERR_CUDA, cudaGetErrorString(e));
    if (st) return fail(CMM_ERR_CUDA, "cmm_conv3x3_weight_grad: a tensor-core wait ran out");
    return CMM_OK;
}

}  // extern "C"
