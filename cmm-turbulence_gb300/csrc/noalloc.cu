// noalloc.cu -- cmm_diagnostics_noalloc: the energy / enstrophy / max|omega|
// reductions of cmm_diagnostics without any device allocation.
//
// Who needs this: cmm_diagnostics obtains its reduction scratch with
// cudaMalloc and returns it with cudaFree.  Some callers cannot do that --
// a host that reserves all device memory up front and forbids allocation
// inside its time loop, a framework whose caching allocator already holds the
// GPU's memory, or a real-time loop that cannot afford cudaFree's implicit
// device-wide synchronisation (it waits for work on every stream).  This
// variant keeps its scratch in a file-scope device array instead.
//
// The array is loaded with the library and stays resident on every GPU that
// loads it until the process exits: kScratchDoubles doubles (about 393 KB).
// It holds one partial sum per 256 input values, so each reduced array may
// have at most kMaxValues = 4,194,304 values: 2 * Npsi (the two slope planes
// of psi) and Ncoarse must not exceed it.  Larger grids are rejected with
// CMM_ERR_PARAM.
//
// Every call shares the one array and it keeps the contents of the last call;
// nothing in it has to start at zero (each kernel writes its partials before
// they are read).  Calls that overlap on the GPU -- concurrent streams or host
// threads -- race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/cmm_abi.h"
#include "kernels.hpp"

namespace cmm {
void set_last_error(const std::string& msg);
}

namespace {
constexpr int kPartials = 16384;                          // one partial per 256 inputs
constexpr long long kMaxValues = 256LL * kPartials;       // 4,194,304 values per reduction
constexpr int kScratchDoubles = 3 * kPartials + 8;        // min/max/sum partials + 8 results
constexpr int kMaxDevices = 64;
}  // namespace

static __device__ __align__(256) double g_diag_scratch[kScratchDoubles];

namespace {
std::mutex g_scratch_mu;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of g_diag_scratch on the current device.  The array's name
// in host code is only a host-side stand-in, so the address is looked up once
// per device, with that device current, and cached.
int scratch_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cmm::set_last_error(std::string("cmm_diagnostics_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return CMM_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        cmm::set_last_error("cmm_diagnostics_noalloc: device index out of range");
        return CMM_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        double* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_diag_scratch);
        if (e != cudaSuccess || !p) {
            cmm::set_last_error(std::string("cmm_diagnostics_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return CMM_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return CMM_OK;
}

// one block of 256 threads reduces 256 consecutive values to one partial
__global__ void __launch_bounds__(256) k_na_sumsq(const double* __restrict__ v, long long n, double* __restrict__ part)
{
    __shared__ double s[256];
    long long i = blockIdx.x * 256LL + threadIdx.x;
    double x = i < n ? v[i] : 0.0;
    s[threadIdx.x] = x * x;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void __launch_bounds__(256) k_na_minmax(const double* __restrict__ v, long long n, double* __restrict__ part)
{
    __shared__ double smin[256], smax[256];
    long long i = blockIdx.x * 256LL + threadIdx.x;
    double inf = __longlong_as_double(0x7ff0000000000000ll);
    smin[threadIdx.x] = i < n ? v[i] : inf;
    smax[threadIdx.x] = i < n ? v[i] : -inf;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = smin[0];
        part[2 * blockIdx.x + 1] = smax[0];
    }
}

// one block folds nb partials (stride 1: sums; stride 2: min/max pairs)
__global__ void k_na_fold(const double* __restrict__ part, int nb, int pairs, double* __restrict__ out)
{
    __shared__ double a[256], b[256];
    double inf = __longlong_as_double(0x7ff0000000000000ll);
    double x = pairs ? inf : 0.0, y = -inf;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        if (pairs) { x = fmin(x, part[2 * k]); y = fmax(y, part[2 * k + 1]); }
        else x += part[k];
    }
    a[threadIdx.x] = x;
    b[threadIdx.x] = y;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            if (pairs) { a[threadIdx.x] = fmin(a[threadIdx.x], a[threadIdx.x + o]); b[threadIdx.x] = fmax(b[threadIdx.x], b[threadIdx.x + o]); }
            else a[threadIdx.x] += a[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = a[0];
        if (pairs) out[1] = b[0];
    }
}

int fail(int code, const char* msg)
{
    cmm::set_last_error(msg);
    return code;
}
}  // namespace

extern "C" int cmm_diagnostics_noalloc(const cmm_grid* grid_psi, const double* psi, const cmm_grid* grid_coarse,
                                       const double* vort, double* out3, void* stream)
{
    if (!grid_psi || !grid_coarse || grid_psi->NX <= 0 || grid_psi->NY <= 0 || grid_coarse->NX <= 0 ||
        grid_coarse->NY <= 0 || !(grid_psi->bounds[1] > grid_psi->bounds[0]) ||
        !(grid_psi->bounds[3] > grid_psi->bounds[2]) || !(grid_coarse->bounds[1] > grid_coarse->bounds[0]) ||
        !(grid_coarse->bounds[3] > grid_coarse->bounds[2]))
        return fail(CMM_ERR_PARAM, "cmm_diagnostics_noalloc: bad grid");
    if (!psi || !vort || !out3) return fail(CMM_ERR_PARAM, "cmm_diagnostics_noalloc: NULL pointer");
    cmm::Grid gp = cmm::make_grid(grid_psi->NX, grid_psi->NY, grid_psi->bounds);
    cmm::Grid gc = cmm::make_grid(grid_coarse->NX, grid_coarse->NY, grid_coarse->bounds);
    if (2 * gp.N > kMaxValues || gc.N > kMaxValues)
        return fail(CMM_ERR_PARAM, "cmm_diagnostics_noalloc: grid too large for the built-in scratch "
                                   "(at most 4194304 values per reduction: 2*NX*NY of psi and NX*NY of omega)");
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    double* part = scratch;
    double* res = scratch + 3 * kPartials;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    long long ne = 2 * gp.N;
    int nbe = (int)((ne + 255) / 256), nbc = (int)((gc.N + 255) / 256);
    k_na_sumsq<<<nbe, 256, 0, s>>>(psi + gp.N, ne, part);
    k_na_fold<<<1, 256, 0, s>>>(part, nbe, 0, res + 0);
    k_na_sumsq<<<nbc, 256, 0, s>>>(vort, gc.N, part);
    k_na_fold<<<1, 256, 0, s>>>(part, nbc, 0, res + 1);
    k_na_minmax<<<nbc, 256, 0, s>>>(vort, gc.N, part);
    k_na_fold<<<1, 256, 0, s>>>(part, nbc, 1, res + 2);
    cudaError_t e = cudaGetLastError();
    double h[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, res, sizeof(double) * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cmm::set_last_error(std::string("cmm_diagnostics_noalloc: ") + cudaGetErrorString(e));
        return CMM_ERR_CUDA;
    }
    out3[0] = 0.5 * gp.hx * gp.hy * h[0];
    out3[1] = 0.5 * gc.hx * gc.hy * h[1];
    double w_max = h[3] > 0 ? h[3] : 0.0, w_min = h[2] < 0 ? h[2] : 0.0;
    out3[2] = w_max > -w_min ? w_max : -w_min;
    return CMM_OK;
}
