// vlasov.hpp -- the Vlasov-Poisson potential of the CMM step (1D1V: x the
// periodic space coordinate, v the velocity coordinate of a 2D grid).
//
// The reference builds psi = phi(x) - h(v) on the psi grid and takes its 2D
// FFT to get the Hermite planes (evaluate_potential_from_density_hermite,
// src/simulation/cmm-simulation-host.cu:385-415).  psi is separable, so that
// 2D transform is exactly
//   psi = phi(x) - h(v),  psi_x = phi'(x),  psi_y = -h'(v),  psi_xy = 0
// with phi' and h' the 1D spectral derivatives of the same samples; this
// library computes those 1D spectra only (1D transforms, csrc/fft.hpp).  h depends on the
// grid alone and is built once.
#pragma once
#include <cuda_runtime.h>

#include "kernels.hpp"

namespace cmm {

constexpr int kVlasovRowChunk = 64;   // rows per partial sum of the v-integral

struct VlasovPlans {
    fft::Plan2D v;           // 1D transforms of length NX of the vort grid
    fft::Plan2D p;           // 1D transforms of length NX of the psi grid (x, and v since NX == NY)
};
bool make_vlasov_plans(VlasovPlans& p, const Grid& gv, const Grid& gp, cudaStream_t s);
void destroy_vlasov_plans(VlasovPlans& p);
// one 1D D2Z / Z2D of a plan's length (unnormalised; the Z2D input is not modified)
cudaError_t fft_d2z_1d(const fft::Plan2D& p, const double* in, double2* out, cudaStream_t s);
cudaError_t fft_z2d_1d(const fft::Plan2D& p, const double2* in, double* out, cudaStream_t s);

// rho[ix] = hy * (f[0][ix] + sum_iy f[iy][ix]) - 1 on the vort grid (row 0
// enters twice, as in the reference, whose integral_v output aliases it);
// f is FP64 (fd) or FP32 (ff); partial holds ceil(NY / kVlasovRowChunk) * NX doubles
cudaError_t launch_vlasov_rho(const double* fd, const float* ff, const Grid& gv, double* partial, double* rho,
                              cudaStream_t s);
// rho_hat (NX_fft of the vort grid, unnormalised D2Z) -> phi_hat and (i kx) phi_hat on
// the psi x-grid: /NXv, /kx^2 (mode 0 -> 0), zero padding (solve_1D_laplace,
// zero_padding_1D: cmm-simulation-host.cu:417-432, cmm-fft.cu:81-101,367-391)
cudaError_t launch_vlasov_phi_spec(const double2* rho_hat, const Grid& gv, const Grid& gp, double2* phi_hat,
                                   double2* dphi_hat, cudaStream_t s);
// normalised bump of compute_periodification_function (cmm-simulation-host.cu:478-494,
// 534-559) on the psi grid's v-nodes: one block, NY values
cudaError_t launch_vlasov_bump(const Grid& gp, double* sigma, cudaStream_t s);
// sigma_hat -> h_hat = sigma_hat / (NY ky^2) (mode 0 -> 0) and (i ky) h_hat (cmm-fft.cu:104-124)
cudaError_t launch_vlasov_h_spec(const double2* sig_hat, const Grid& gp, double2* h_hat, double2* dh_hat,
                                 cudaStream_t s);
// Hermite planes of psi = phi(x) - h(v) on the psi grid (plain form)
cudaError_t launch_vlasov_assemble(const double* phi, const double* dphi, const double* h, const double* dh,
                                   const Grid& gp, double* psi4, cudaStream_t s);
// phi(x), phi'(x) (2 x NX) of Hermite planes of psi = phi(x) - h(v): row 0 of psi plus h(v_0), row 0 of psi_x
cudaError_t launch_vlasov_phi_from_psi(const double* psi4, const double* h, const Grid& gp, double* phi, cudaStream_t s);
// sums of f, f v and f v^2 over the coarse grid (v = b2 + iY hy) -> out3 (device)
cudaError_t launch_vlasov_moments(const double* f, const Grid& gc, double* partial, double* out3, cudaStream_t s);
// 1D Hermite table of a Lagrange combination c_l of phi levels: table[i] =
// (F(x_{i+1}) - F(x_i), F'(x_i)) (phi_l: n values then n derivatives); also
// used for h with one level
cudaError_t launch_vlasov_table(const double* const* levels, const double* coef, int n_levels, int n, double2* table,
                                cudaStream_t s);
// |F_k| / N for k = 1..4 of a 1D spectrum (Compute_kth_Mode, cmm-mesure.cu:187-202) -> out4 (device)
cudaError_t launch_vlasov_modes(const double2* spec, int n, int nfft, double* out4, cudaStream_t s);

}  // namespace cmm
