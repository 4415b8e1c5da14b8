// fft.hpp -- host side of the library's own FFT (csrc/fft.cu, engine in fft.cuh).
//
// Replaces the cuFFT D2Z / Z2D (and FP32 R2C / C2R) plans the reference builds
// per grid (Cuda-CMM/src/grid/cmm-grid2d.cu:123-131): a Plan2D holds the radix
// plans and device twiddle tables of one NX x NY real shape in FP32 or FP64; the
// transforms are batched, stream-ordered and allocate nothing.
//
// Layouts are cuFFT's: real input NY rows of NX values (row stride NX), half
// spectrum NY rows of NX/2+1 complex values.  c2r may overwrite its input, as
// cuFFT's does.  Supported lengths: NX even with NX/2 <= 8192, NY <= 8192, every
// prime factor of NX/2 and NY in {2, 3, 5, 7, 11, 13}.
#pragma once
#include <cuda_runtime.h>

#include "fft.cuh"

namespace cmm {
namespace fft {

constexpr int kMaxLen = 8192;   // longest complex transform (values per transform in shared memory)

// true when a complex transform of length n runs here (n <= kMaxLen, primes <= 13)
bool supported_length(int n);
bool make_radix_plan(int n, RadixPlan& p);
// blocks of a persistent launch of func: as many as stay resident on the GPU, at most groups
int resident_grid(const void* func, int threads, size_t smem, long long groups);

struct Plan2D {
    int nx = 0, ny = 0;
    bool dbl = false;
    RadixPlan rx{}, ry{};      // rx: complex length nx/2 (packed rows), ry: ny (columns)
    void* twx = nullptr;       // rx's pass twiddles, then exp(-2 pi i k / nx) for k <= nx/2 (float2 / double2)
    void* twy = nullptr;       // ry's pass twiddles
    bool ok() const { return twx != nullptr; }
};

// 0 on success; -1 for an unsupported shape, -2 for a CUDA error (device tables)
int plan_create(Plan2D& p, int nx, int ny, bool dbl, cudaStream_t s);
void plan_destroy(Plan2D& p);
// a 1D plan of nx-point rows (ny = 1: no column tables)
inline int plan_create_rows(Plan2D& p, int nx, bool dbl, cudaStream_t s) { return plan_create(p, nx, 1, dbl, s); }

// batched 2D transforms; idist / odist = elements between batch items (0: dense)
cudaError_t r2c(const Plan2D& p, const void* in, void* out, int batch, cudaStream_t s, long long idist = 0,
                long long odist = 0);
cudaError_t c2r(const Plan2D& p, void* in, void* out, int batch, cudaStream_t s, long long idist = 0,
                long long odist = 0);

// the two passes on their own
// rows: R2C of `rows` real rows (row stride ild, every rows_per_item rows a new item at idist)
// writing bins 0..kout-1 (row stride old, item stride odist)
cudaError_t rows_r2c(const Plan2D& p, const void* in, long long ild, long long idist, void* out, long long old,
                     long long odist, int rows_per_item, int items, int kout, cudaStream_t s);
// rows: R2C of one item of `rows` FP32 rows (16-byte aligned, row stride ild a multiple of 4
// floats) writing bins 0..kout-1 column-major: bin k of row r at out[k ocol + r] (ocol even,
// at least rows; out 16-byte aligned).  Only the compile-time power-of-two kernels
// (rows_r2c_t_supported); cudaErrorInvalidValue otherwise
cudaError_t rows_r2c_t(const Plan2D& p, const void* in, long long ild, void* out, long long ocol, int rows, int kout,
                       cudaStream_t s);
bool rows_r2c_t_supported(const Plan2D& p);
// rows: C2R reading bins 0..kin-1 (the rest zero) of each row
cudaError_t rows_c2r(const Plan2D& p, const void* in, long long ild, long long idist, int kin, void* out,
                     long long old, long long odist, int rows_per_item, int items, cudaStream_t s);
// columns: in-place complex transforms of columns 0..ncols-1 (length p.ny) of a row-major
// complex array with row stride ld, batch items bdist apart
cudaError_t cols_c2c(const Plan2D& p, void* data, long long ld, long long bdist, int ncols, int batch, bool inverse,
                     cudaStream_t s);

}  // namespace fft
}  // namespace cmm
