// sim_learned.cpp -- the learned psi of the mixed Euler form.
//
// Exact psi (the method): omega sampled through the map on the vorticity grid, FFT,
// Poisson solve with the psi cut-off, Hermite planes on the psi grid.
// Cheap psi: the same solve from omega sampled on the map grid (16x fewer samples at the
// metric's 512^2 map / 2048^2 vorticity grids), which aliases the vorticity scales the map
// grid cannot hold into the retained modes.
// Learned psi: the upsampler's network sees the cheap psi planes, omega and omega's
// gradient on the map grid (the gradient, through the map's Jacobian, tells the vorticity
// scales the map grid cannot hold apart from the ones it can) and predicts, on the psi grid,
// the vorticity the map-grid samples miss (omega on the psi grid minus the spectral
// interpolation of the samples); the learned psi solves the cheap vorticity plus that
// prediction with the method's cut-off, Poisson step and Hermite derivatives.

#include <algorithm>
#include <cmath>

#include "learned.hpp"
#include "mixed.hpp"
#include "sim.hpp"

namespace cmm {

#define CMM_CUDA(call) do { int rc_ = check((call), #call); if (rc_) return rc_; } while (0)
#define CMM_LAUNCH(k, call) do { kernel_launches += (k); int rc_ = check((call), #call); if (rc_) return rc_; } while (0)
#define CMM_FFT(call) do { fft_calls++; cudaError_t e_ = (call); if (e_ != cudaSuccess) { err = std::string("FFT: ") + #call + ": " + cudaGetErrorString(e_); return kErrCuda; } } while (0)

int EulerSim::learned_check() const
{
    if (!mixed_ || vlasov_) return 0;
    if (gp.NX != 2 * gc.NX || gp.NY != 2 * gc.NY) return 0;
    if (gc.NX % lrn::kTile != 0) return 0;
    return 1;
}

int EulerSim::learned_setup()
{
    if (lc_omega_) return kOk;
    if (!learned_check()) {
        err = "the learned psi needs precision=mixed, a 2D Euler run, a psi grid twice the map grid and a map grid "
              "width that is a multiple of 128";
        return kErrUnsupported;
    }
    auto falloc = [&](void** p, size_t bytes) { return check(cudaMalloc(p, bytes), "cudaMalloc"); };
    int rc;
    if ((rc = falloc((void**)&lc_omega_, sizeof(float) * 3 * (size_t)gc.N)) ||
        (rc = falloc((void**)&lc_planes_, sizeof(float) * 4 * (size_t)gc.N)) ||
        (rc = falloc((void**)&l_delta_, sizeof(float) * (size_t)gp.N)) ||
        (rc = falloc((void**)&l_planes_, sizeof(float) * 4 * (size_t)gp.N)) ||
        (rc = falloc((void**)&lc_spec_, sizeof(float2) * (size_t)gc.Nfft)) ||
        (rc = falloc((void**)&lc_spec4_, sizeof(float2) * 4 * (size_t)gc.Nfft)) ||
        (rc = falloc((void**)&l_dspec_, sizeof(float2) * (size_t)gp.Nfft)) ||
        (rc = falloc((void**)&d_stats_, sizeof(double) * 4)))
        return rc;
    if (fft::plan_create(fc_, gc.NX, gc.NY, false, stream)) {
        err = "FFT plan creation for the learned psi failed";
        return kErrCuda;
    }
    return kOk;
}

void EulerSim::learned_release()
{
    auto f = [](void* p) { if (p) cudaFree(p); };
    f(lc_omega_); f(lc_planes_); f(l_delta_); f(l_planes_); f(lc_spec_); f(lc_spec4_); f(l_dspec_); f(d_stats_);
    lc_omega_ = lc_planes_ = l_delta_ = l_planes_ = nullptr;
    lc_spec_ = lc_spec4_ = l_dspec_ = nullptr;
    d_stats_ = nullptr;
    fft::plan_destroy(fc_);
    delete ups_owned_;
    ups_owned_ = nullptr;
    ups_ = nullptr;
}

int EulerSim::load_upsampler()
{
    auto* u = new lrn::Upsampler();
    if (!u->err.empty() || u->load(s.psi_upsampler)) {
        err = u->err.empty() ? "cannot read " + s.psi_upsampler : u->err;
        delete u;
        return kErrIO;
    }
    int rc = attach_upsampler(u, s.psi_exact_every, s.psi_learned_tol);
    if (rc) {
        delete u;
        return rc;
    }
    ups_owned_ = u;
    return kOk;
}

int EulerSim::attach_upsampler(lrn::Upsampler* u, int every, double tol)
{
    if (!u) {
        ups_ = nullptr;
        return kOk;
    }
    if (every < 1 || !(tol > 0)) {
        err = "psi_exact_every must be >= 1 and psi_learned_tol > 0";
        return kErrParam;
    }
    int rc = learned_setup();
    if (rc) return rc;
    ups_ = u;
    learned_every_ = every;
    learned_tol_ = tol;
    learned_level_ = 2;
    return kOk;
}

int EulerSim::cheap_fields()
{
    // omega and its gradient on the map grid, omega's spectrum, and the cheap psi's
    // Hermite planes there
    CMM_LAUNCH(1, launch_sample_grad_m(gc, gf, mapm_, wfm_, lc_omega_, stream));
    CMM_FFT(fft::r2c(fc_, lc_omega_, lc_spec_, 1, stream));
    CMM_LAUNCH(1, launch_spec_psi_f(lc_spec_, gc, gc, s.freq_cut_psi, lc_spec4_, stream));
    CMM_FFT(fft::c2r(fc_, lc_spec4_, lc_planes_, 4, stream));
    return kOk;
}

int EulerSim::learned_planes(lrn::Upsampler& u, float* out)
{
    int rc;
    if ((rc = cheap_fields())) return rc;
    if (u.infer(lc_planes_, lc_omega_, gc.NY, gc.NX, l_delta_, stream)) {
        err = u.err;
        return kErrCuda;
    }
    kernel_launches += u.launches;
    CMM_FFT(fft::r2c(fp_, l_delta_, l_dspec_, 1, stream));
    CMM_LAUNCH(1, launch_spec_psi_learned(lc_spec_, gc, l_dspec_, gp, s.freq_cut_psi, spec4f_, stream));
    if ((rc = psi_planes(spec4f_, out))) return rc;
    return kOk;
}

int EulerSim::diff_stats(const float* a, long long sa, const float* e, long long se, long long n, double* host4)
{
    CMM_CUDA(cudaMemsetAsync(d_stats_, 0, sizeof(double) * 4, stream));
    CMM_LAUNCH(1, lrn::launch_diff_stats(a, sa, e, se, n, d_stats_, stream));
    CMM_CUDA(cudaMemcpyAsync(host4, d_stats_, sizeof(double) * 4, cudaMemcpyDeviceToHost, stream));
    CMM_CUDA(cudaStreamSynchronize(stream));
    return kOk;
}

int EulerSim::cheap_planes(float* out)
{
    int rc;
    if ((rc = cheap_fields())) return rc;
    CMM_LAUNCH(1, launch_spec_psi_f(lc_spec_, gc, gp, s.freq_cut_psi, spec4f_, stream));
    if ((rc = psi_planes(spec4f_, out))) return rc;
    return kOk;
}

int EulerSim::learned_stream()
{
    // between judged steps: the level the last judgement chose
    if (loop_ctr_ % learned_every_ != 0) {
        if (learned_level_ == 0) {
            ++learned_steps_;
            return learned_planes(*ups_, realf_);
        }
        if (learned_level_ == 1) {
            ++cheap_steps_;
            return cheap_planes(realf_);
        }
    }
    ++exact_steps_;
    int rc;
    CMM_LAUNCH(1, launch_sample_m(gc, gv, gf, mapm_, wfm_, realf_, nullptr, stream));
    if ((rc = vort_spectrum())) return rc;
    CMM_LAUNCH(1, launch_spec_psi_f(specf_, gv, gp, s.freq_cut_psi, spec4f_, stream));
    if ((rc = psi_planes(spec4f_, realf_))) return rc;
    if (loop_ctr_ % learned_every_ != 0) return kOk;
    // the exact evaluation judges the learned and the cheap psi on the same state and picks
    // the level of the next every - 1 steps: the network where it meets the tolerance and
    // beats the cheap psi, else the cheap psi where that meets it, else the exact one
    double st[4];
    if ((rc = learned_planes(*ups_, l_planes_)) || (rc = diff_stats(l_planes_, 1, realf_, 1, gp.N, st))) return rc;
    const double el = st[1] > 0 ? st[0] / st[1] : 0.0;
    if ((rc = cheap_planes(l_planes_)) || (rc = diff_stats(l_planes_, 1, realf_, 1, gp.N, st))) return rc;
    const double ec = st[1] > 0 ? st[0] / st[1] : 0.0;
    ++learned_checks_;
    learned_last_err_ = el;
    learned_max_err_ = std::max(learned_max_err_, el);
    if (el <= learned_tol_ && el <= ec) {
        learned_level_ = 0;
    } else if (ec <= learned_tol_) {
        learned_level_ = 1;
        ++learned_cheaper_;
    } else {
        learned_level_ = 2;
        ++learned_fails_;
    }
    return kOk;
}

int EulerSim::learned_collect(lrn::Upsampler& u)
{
    if (!initialised_) { err = "learned_collect before init"; return kErrState; }
    int rc;
    if ((rc = learned_setup()) || (rc = cheap_fields())) return rc;
    // target: omega sampled through the map on the psi grid minus the spectral
    // interpolation of the map-grid samples there
    CMM_LAUNCH(1, launch_spec_pad(lc_spec_, gc, gp, l_dspec_, stream));
    CMM_FFT(fft::c2r(fp_, l_dspec_, l_planes_ + gp.N, 1, stream));
    CMM_LAUNCH(1, launch_sample_m(gc, gp, gf, mapm_, wfm_, l_planes_, nullptr, stream));
    CMM_LAUNCH(1, lrn::launch_sub(l_planes_, l_planes_ + gp.N, gp.N, l_delta_, stream));
    u.set_spectral_cut((int)std::floor(s.freq_cut_psi));
    if (u.append(lc_planes_, lc_omega_, l_delta_, gc.NY, gc.NX, stream)) {
        err = u.err;
        return kErrCuda;
    }
    CMM_CUDA(cudaStreamSynchronize(stream));
    return kOk;
}

int EulerSim::learned_evaluate(lrn::Upsampler& u, double* out6)
{
    if (!initialised_) { err = "learned_evaluate before init"; return kErrState; }
    int rc;
    if ((rc = learned_setup()) || (rc = cheap_fields())) return rc;
    const float* exact = reinterpret_cast<const float*>(psim_[0]);
    double st[4];
    CMM_LAUNCH(1, launch_spec_psi_f(lc_spec_, gc, gp, s.freq_cut_psi, spec4f_, stream));
    if ((rc = psi_planes(spec4f_, l_planes_))) return rc;
    auto rel = [&](double* o) {
        o[0] = st[1] > 0 ? st[0] / st[1] : 0.0;
        o[1] = st[3] > 0 ? std::sqrt(st[2] / st[3]) : 0.0;
    };
    if ((rc = diff_stats(l_planes_, 1, exact, 4, gp.N, st))) return rc;
    rel(out6);
    if ((rc = learned_planes(u, l_planes_))) return rc;
    if ((rc = diff_stats(l_planes_, 1, exact, 4, gp.N, st))) return rc;
    rel(out6 + 2);
    // the ceiling: psi of omega sampled exactly on the psi grid (what a perfect network gives)
    CMM_LAUNCH(1, launch_sample_m(gc, gp, gf, mapm_, wfm_, l_delta_, nullptr, stream));
    CMM_FFT(fft::r2c(fp_, l_delta_, l_dspec_, 1, stream));
    CMM_LAUNCH(1, launch_spec_psi_f(l_dspec_, gp, gp, s.freq_cut_psi, spec4f_, stream));
    if ((rc = psi_planes(spec4f_, l_planes_))) return rc;
    if ((rc = diff_stats(l_planes_, 1, exact, 4, gp.N, st))) return rc;
    rel(out6 + 4);
    return kOk;
}

}  // namespace cmm
