// abi.cpp -- extern "C" entry points declared in include/cmm_abi.h.
#include "../../include/cmm_abi.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>

#include "abi_internal.hpp"
#include "ensemble.hpp"
#include "kernels.hpp"
#include "settings.hpp"
#include "sim.hpp"
#include "vlasov.hpp"

struct cmm_ensemble {
    std::vector<cmm::Settings> settings;
    std::vector<std::vector<double>> discrete;
    cmm::EnsembleSim* ens = nullptr;
    cudaStream_t stream = nullptr;
    bool graphs = true;
    int fused = 2;
    long long wait_limit = 1ll << 24;
};

struct cmm_poisson {
    cmm::Grid gv, gp;
    double freq = 0;
    cudaStream_t stream = nullptr;
    cmm::FftPlans pv, pp;
    double2* spec = nullptr;
    double2* spec4 = nullptr;
};

struct cmm_fft {
    cmm::fft::Plan2D plan;
    cudaStream_t stream = nullptr;
};

struct cmm_vlasov {
    cmm::Grid gv, gp;
    cudaStream_t stream = nullptr;
    cmm::VlasovPlans plans;
    double* h = nullptr;       // h (NY), h' (NY)
    double* fs = nullptr;      // f on the vort grid
    double* rho = nullptr;
    double* part = nullptr;
    double* phi = nullptr;     // phi (NX), phi' (NX)
    double* red = nullptr;
    double* scal = nullptr;
    double* row = nullptr;
    double2* c[3] = {nullptr, nullptr, nullptr};
};

namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

int cuda_rc(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return CMM_OK;
    return fail(CMM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool to_grid(const cmm_grid* g, cmm::Grid* out)
{
    if (!g || g->NX <= 0 || g->NY <= 0 || !(g->bounds[1] > g->bounds[0]) || !(g->bounds[3] > g->bounds[2])) return false;
    *out = cmm::make_grid(g->NX, g->NY, g->bounds);
    return true;
}

int copy_text(const std::string& t, char* buf, size_t cap)
{
    if (buf && cap > 0) {
        size_t n = t.size() < cap - 1 ? t.size() : cap - 1;
        memcpy(buf, t.data(), n);
        buf[n] = 0;
    }
    return (int)t.size();
}

int sim_rc(cmm::EulerSim* sim, int rc)
{
    if (rc < 0) g_err = sim->err;
    return rc;
}
}  // namespace

// lets entry points defined in other translation units report through
// cmm_last_error
void cmm::set_last_error(const std::string& msg) { g_err = msg; }

extern "C" {

const char* cmm_last_error(void) { return g_err.c_str(); }
const char* cmm_version(void)
{
    return "cmm-gb300 0.2 (sm_103a; Euler 2D and Vlasov-Poisson 1D1V; plain FP64 and mixed forms)";
}

int cmm_create(int argc, const char* const* argv, cmm_ctx** out)
{
    if (!out) return fail(CMM_ERR_PARAM, "out is NULL");
    *out = nullptr;
    cmm_ctx* c = new (std::nothrow) cmm_ctx();
    if (!c) return fail(CMM_ERR_PARAM, "out of host memory");
    if (!c->settings.apply_cli(argc, argv)) {
        std::string e = c->settings.error;
        delete c;
        return fail(e.find("parameter file") != std::string::npos ? CMM_ERR_IO : CMM_ERR_PARAM, e);
    }
    c->settings.file_name = c->settings.derived_file_name();
    *out = c;
    g_err.clear();
    return CMM_OK;
}

int cmm_set_stream(cmm_ctx* c, void* stream)
{
    if (!c) return fail(CMM_ERR_PARAM, "ctx is NULL");
    if (c->sim) return fail(CMM_ERR_STATE, "cmm_set_stream after cmm_init");
    c->stream = static_cast<cudaStream_t>(stream);
    return CMM_OK;
}

int cmm_set_initial_discrete(cmm_ctx* c, const double* v, size_t n)
{
    if (!c || !v) return fail(CMM_ERR_PARAM, "NULL argument");
    if (c->sim) return fail(CMM_ERR_STATE, "cmm_set_initial_discrete after cmm_init");
    size_t need = (size_t)c->settings.initial_discrete_grid * c->settings.initial_discrete_grid;
    if (n != need) return fail(CMM_ERR_PARAM, "discrete initial condition needs initial_discrete_grid^2 values");
    c->discrete.assign(v, v + n);
    return CMM_OK;
}

int cmm_init(cmm_ctx* c)
{
    if (!c) return fail(CMM_ERR_PARAM, "ctx is NULL");
    if (c->sim) return fail(CMM_ERR_STATE, "cmm_init called twice");
    c->sim = new (std::nothrow) cmm::EulerSim(c->settings);
    if (!c->sim) return fail(CMM_ERR_PARAM, "out of host memory");
    if (c->stream) c->sim->set_stream(c->stream);
    if (!c->discrete.empty()) {
        int rc = c->sim->set_initial_discrete(c->discrete.data(), c->discrete.size());
        if (rc) return sim_rc(c->sim, rc);
    }
    int rc = c->sim->init();
    c->discrete.clear();
    return sim_rc(c->sim, rc);
}

int cmm_step(cmm_ctx* c, int n)
{
    if (!c || !c->sim) return fail(CMM_ERR_STATE, "cmm_step before cmm_init");
    for (int i = 0; i < n; ++i) {
        int rc = c->sim->step_once();
        if (rc != 0) return sim_rc(c->sim, rc);
    }
    return CMM_OK;
}

int cmm_run(cmm_ctx* c)
{
    if (!c || !c->sim) return fail(CMM_ERR_STATE, "cmm_run before cmm_init");
    int status = CMM_OK;
    while (true) {
        int rc = c->sim->step_once();
        if (rc == 1) break;
        if (rc == CMM_ERR_SATURATED) { status = rc; g_err = "map stack saturated"; break; }
        if (rc < 0) return sim_rc(c->sim, rc);
    }
    int rc = c->sim->finish();
    if (rc) return sim_rc(c->sim, rc);
    return status;
}

int cmm_get_field(cmm_ctx* c, const char* name, void* dst, size_t bytes)
{
    if (!c || !c->sim || !name || !dst) return fail(CMM_ERR_STATE, "cmm_get_field needs an initialised ctx, a name and a buffer");
    return sim_rc(c->sim, c->sim->get_field(name, dst, bytes));
}

size_t cmm_field_bytes(cmm_ctx* c, const char* name)
{
    if (!c || !c->sim || !name) return 0;
    return c->sim->field_bytes(name);
}

int cmm_get_scalar(cmm_ctx* c, const char* name, double* out)
{
    if (!c || !name || !out) return fail(CMM_ERR_PARAM, "NULL argument");
    if (!c->sim) {
        std::string n = name;
        if (n == "dt") { *out = c->settings.dt(); return CMM_OK; }
        if (n == "lagrange_order") { *out = c->settings.effective_lagrange_order(); return CMM_OK; }
        if (n == "stack_capacity") { *out = c->settings.cpu_map_num(); return CMM_OK; }
        return fail(CMM_ERR_STATE, "scalar needs cmm_init");
    }
    return sim_rc(c->sim, c->sim->get_scalar(name, out));
}

int cmm_set_profiling(cmm_ctx* c, int on)
{
    if (!c || !c->sim) return fail(CMM_ERR_STATE, "cmm_set_profiling needs an initialised ctx");
    c->sim->set_profiling(on != 0);
    return CMM_OK;
}

int cmm_settings_text(cmm_ctx* c, char* buf, size_t cap)
{
    if (!c) return fail(CMM_ERR_PARAM, "ctx is NULL");
    return copy_text(c->sim ? c->sim->s.param_text() : c->settings.param_text(), buf, cap);
}

int cmm_file_name(cmm_ctx* c, char* buf, size_t cap)
{
    if (!c) return fail(CMM_ERR_PARAM, "ctx is NULL");
    return copy_text(c->settings.derived_file_name(), buf, cap);
}

int cmm_destroy(cmm_ctx* c)
{
    if (!c) return CMM_OK;
    delete c->sim;
    delete c;
    return CMM_OK;
}

// ---------------------------------------------------------------- kernel API
int cmm_advect_map(const cmm_grid* grid_map, const cmm_grid* grid_psi, const double* chix, const double* chiy,
                   double* chix_out, double* chiy_out, const double* const* psi_levels, int l_order,
                   const double* L1, const double* L12, double dt, double map_epsilon, int time_integration_num,
                   int map_update_order_num, void* stream)
{
    cmm::AdvectArgs a{};
    if (!to_grid(grid_map, &a.gm) || !to_grid(grid_psi, &a.gp)) return fail(CMM_ERR_PARAM, "bad grid");
    if (!chix || !chiy || !chix_out || !chiy_out || !psi_levels || !L1 || !L12) return fail(CMM_ERR_PARAM, "NULL pointer");
    if (l_order < 1 || l_order > cmm::kMaxLagrange) return fail(CMM_ERR_PARAM, "l_order must be 1..4");
    if (map_update_order_num < 0 || map_update_order_num > 2) return fail(CMM_ERR_PARAM, "map_update_order_num must be 0..2");
    if (time_integration_num != 10 && time_integration_num != 21 && time_integration_num != 30)
        return fail(CMM_ERR_UNSUPPORTED, "time_integration_num must be 10, 21 or 30");
    if (time_integration_num == 30 && l_order < 3) return fail(CMM_ERR_PARAM, "RK3 needs l_order >= 3");
    a.ChiX = chix; a.ChiY = chiy; a.outX = chix_out; a.outY = chiy_out;
    for (int l = 0; l < l_order; ++l) {
        if (!psi_levels[l]) return fail(CMM_ERR_PARAM, "NULL psi level");
        a.psi[l] = psi_levels[l];
        a.L1[l] = L1[l];
        a.L12[l] = L12[l];
    }
    cmm::map_update_coefficients(map_update_order_num, map_epsilon, a.coef, &a.nfoot);
    a.dt = dt; a.ep = map_epsilon; a.time_integration_num = time_integration_num; a.l_order = l_order;
    return cuda_rc(cmm::launch_advect(a, static_cast<cudaStream_t>(stream)), "cmm_advect_map");
}

int cmm_incomp_max(const cmm_grid* grid_check, const cmm_grid* grid_map, const double* chix, const double* chiy,
                   double* d_result, void* stream)
{
    cmm::Grid gc, gm;
    if (!to_grid(grid_check, &gc) || !to_grid(grid_map, &gm)) return fail(CMM_ERR_PARAM, "bad grid");
    if (!chix || !chiy || !d_result) return fail(CMM_ERR_PARAM, "NULL pointer");
    return cuda_rc(cmm::launch_incomp(gc, gm, chix, chiy, d_result, static_cast<cudaStream_t>(stream)), "cmm_incomp_max");
}

int cmm_compose_stack(const cmm_grid* grid_map, const cmm_grid* grid_target, const double* chix, const double* chiy,
                      const double* stack, int n_maps, int ic_num, const double* discrete,
                      const cmm_grid* grid_discrete, double* out, void* stream)
{
    cmm::Grid gm, gt;
    if (!to_grid(grid_map, &gm) || !to_grid(grid_target, &gt)) return fail(CMM_ERR_PARAM, "bad grid");
    if (!chix || !chiy || !out || n_maps < 0 || (n_maps > 0 && !stack)) return fail(CMM_ERR_PARAM, "bad pointer / map count");
    cmm::InitSource src{};
    if (discrete) {
        if (!to_grid(grid_discrete, &src.gd)) return fail(CMM_ERR_PARAM, "bad discrete grid");
        src.kind = 3;
        src.discrete = discrete;
    } else {
        if (ic_num < 0 || ic_num > 11 || ic_num == 7 || ic_num == 8 || ic_num == 11)
            return fail(CMM_ERR_UNSUPPORTED, "ic_num not available in the kernel API (needs tables or parameters)");
        src.kind = 0;
        src.ic_num = ic_num;
    }
    return cuda_rc(cmm::launch_compose_sample(gm, gt, chix, chiy, stack, n_maps, src, out, static_cast<cudaStream_t>(stream)),
                   "cmm_compose_stack");
}

int cmm_compose_stack_var(const cmm_grid* grid_map, const cmm_grid* grid_target, const double* chix,
                          const double* chiy, const double* stack, int n_maps, int var_num, int ic_num,
                          const double* discrete, const cmm_grid* grid_discrete, double* out, void* stream)
{
    if (var_num == 0 || discrete)
        return cmm_compose_stack(grid_map, grid_target, chix, chiy, stack, n_maps, ic_num, discrete, grid_discrete, out,
                                 stream);
    cmm::Grid gm, gt;
    if (!to_grid(grid_map, &gm) || !to_grid(grid_target, &gt)) return fail(CMM_ERR_PARAM, "bad grid");
    if (!chix || !chiy || !out || n_maps < 0 || (n_maps > 0 && !stack)) return fail(CMM_ERR_PARAM, "bad pointer / map count");
    if ((var_num == 1 && (ic_num < 0 || ic_num > 2)) || (var_num == 2 && (ic_num < 0 || ic_num > 2)) || var_num < 0 ||
        var_num > 2)
        return fail(CMM_ERR_PARAM, "var_num / ic_num out of range");
    cmm::InitSource src{};
    src.kind = var_num;
    src.ic_num = ic_num;
    return cuda_rc(cmm::launch_compose_sample(gm, gt, chix, chiy, stack, n_maps, src, out, static_cast<cudaStream_t>(stream)),
                   "cmm_compose_stack_var");
}

int cmm_vlasov_create(const cmm_grid* grid_vort, const cmm_grid* grid_psi, void* stream, cmm_vlasov** out)
{
    if (!out) return fail(CMM_ERR_PARAM, "out is NULL");
    *out = nullptr;
    cmm_vlasov* p = new (std::nothrow) cmm_vlasov();
    if (!p) return fail(CMM_ERR_PARAM, "out of host memory");
    if (!to_grid(grid_vort, &p->gv) || !to_grid(grid_psi, &p->gp)) { delete p; return fail(CMM_ERR_PARAM, "bad grid"); }
    if (p->gv.NX > p->gp.NX || p->gv.NY > p->gp.NY) { delete p; return fail(CMM_ERR_PARAM, "vort grid finer than psi grid"); }
    if (p->gp.NX != p->gp.NY) { delete p; return fail(CMM_ERR_PARAM, "psi grid must be square"); }
    p->stream = static_cast<cudaStream_t>(stream);
    const int nchunks = (p->gv.NY + cmm::kVlasovRowChunk - 1) / cmm::kVlasovRowChunk;
    const int cn = p->gv.NX_fft > p->gp.NX_fft ? p->gv.NX_fft : p->gp.NX_fft;
    bool ok = cmm::make_vlasov_plans(p->plans, p->gv, p->gp, p->stream) &&
              cudaMalloc((void**)&p->h, sizeof(double) * 2 * p->gp.NY) == cudaSuccess &&
              cudaMalloc((void**)&p->fs, sizeof(double) * p->gv.N) == cudaSuccess &&
              cudaMalloc((void**)&p->rho, sizeof(double) * p->gv.NX) == cudaSuccess &&
              cudaMalloc((void**)&p->part, sizeof(double) * nchunks * p->gv.NX) == cudaSuccess &&
              cudaMalloc((void**)&p->phi, sizeof(double) * 2 * p->gp.NX) == cudaSuccess &&
              cudaMalloc((void**)&p->red, sizeof(double) * 3 * cmm::kReduceBlocks) == cudaSuccess &&
              cudaMalloc((void**)&p->scal, sizeof(double) * 16) == cudaSuccess &&
              cudaMalloc((void**)&p->row, sizeof(double) * (p->gp.NX > p->gp.NY ? p->gp.NX : p->gp.NY)) == cudaSuccess;
    for (int k = 0; k < 3 && ok; ++k) ok = cudaMalloc((void**)&p->c[k], sizeof(double2) * cn) == cudaSuccess;
    if (!ok) { cmm_vlasov_destroy(p); return fail(CMM_ERR_CUDA, "FFT plan or cudaMalloc failed"); }
    // the periodification h(v) and h'(v) once
    cudaError_t e = cmm::launch_vlasov_bump(p->gp, p->row, p->stream);
    if (e == cudaSuccess) e = cmm::fft_d2z_1d(p->plans.p, p->row, p->c[0], p->stream);
    if (e == cudaSuccess) e = cmm::launch_vlasov_h_spec(p->c[0], p->gp, p->c[1], p->c[2], p->stream);
    if (e == cudaSuccess) e = cmm::fft_z2d_1d(p->plans.p, p->c[1], p->h, p->stream);
    if (e == cudaSuccess) e = cmm::fft_z2d_1d(p->plans.p, p->c[2], p->h + p->gp.NY, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) { cmm_vlasov_destroy(p); return cuda_rc(e, "cmm_vlasov_create"); }
    *out = p;
    return CMM_OK;
}

int cmm_vlasov_potential(cmm_vlasov* p, const cmm_grid* grid_map, const cmm_grid* grid_fine, const double* chix,
                         const double* chiy, const double* f_fine_H, int molly_stencil, double* psi_out)
{
    if (!p || !chix || !chiy || !f_fine_H || !psi_out) return fail(CMM_ERR_PARAM, "NULL argument");
    cmm::Grid gm, gf;
    if (!to_grid(grid_map, &gm) || !to_grid(grid_fine, &gf)) return fail(CMM_ERR_PARAM, "bad grid");
    if (molly_stencil != 0 && molly_stencil != 4 && molly_stencil != 8) return fail(CMM_ERR_PARAM, "molly_stencil must be 0, 4 or 8");
    cudaStream_t s = p->stream;
    cudaError_t e = cmm::launch_sample_vort(gm, p->gv, gf, chix, chiy, f_fine_H, molly_stencil, p->fs, p->gv.NX, s);
    if (e == cudaSuccess) e = cmm::launch_vlasov_rho(p->fs, nullptr, p->gv, p->part, p->rho, s);
    if (e == cudaSuccess) e = cmm::fft_d2z_1d(p->plans.v, p->rho, p->c[0], s);
    if (e == cudaSuccess) e = cmm::launch_vlasov_phi_spec(p->c[0], p->gv, p->gp, p->c[1], p->c[2], s);
    if (e == cudaSuccess) e = cmm::fft_z2d_1d(p->plans.p, p->c[1], p->phi, s);
    if (e == cudaSuccess) e = cmm::fft_z2d_1d(p->plans.p, p->c[2], p->phi + p->gp.NX, s);
    if (e == cudaSuccess) e = cmm::launch_vlasov_assemble(p->phi, p->phi + p->gp.NX, p->h, p->h + p->gp.NY, p->gp, psi_out, s);
    return cuda_rc(e, "cmm_vlasov_potential");
}

int cmm_vlasov_diagnostics(cmm_vlasov* p, const cmm_grid* grid_coarse, const double* f_coarse, const double* psi,
                           double* out9)
{
    if (!p || !f_coarse || !psi || !out9) return fail(CMM_ERR_PARAM, "NULL argument");
    cmm::Grid gc;
    if (!to_grid(grid_coarse, &gc)) return fail(CMM_ERR_PARAM, "bad grid");
    const cmm::Grid& gp = p->gp;
    cudaStream_t s = p->stream;
    cudaError_t e = cmm::launch_vlasov_moments(f_coarse, gc, p->red, p->scal, s);
    if (e == cudaSuccess) e = cmm::launch_sumsq(psi + gp.N, gp.NX, p->red, p->scal + 3, s);   // first row of psi_x
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->row, psi + gp.N, sizeof(double) * gp.NX, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cmm::fft_d2z_1d(p->plans.p, p->row, p->c[0], s);
    if (e == cudaSuccess) e = cmm::launch_vlasov_modes(p->c[0], gp.NX, gp.NX_fft, p->scal + 4, s);
    double h[8] = {0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, p->scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_rc(e, "cmm_vlasov_diagnostics");
    double ekin = 0.5 * gc.hy * gc.hx * h[2], epot = 0.5 * gp.hx * h[3];
    out9[0] = ekin + epot; out9[1] = ekin; out9[2] = epot;
    out9[3] = gc.hy * gc.hx * h[0]; out9[4] = gc.hy * gc.hx * h[1];
    for (int k = 0; k < 4; ++k) out9[5 + k] = h[4 + k];
    return CMM_OK;
}

int cmm_vlasov_destroy(cmm_vlasov* p)
{
    if (!p) return CMM_OK;
    cmm::destroy_vlasov_plans(p->plans);
    auto f = [](void* q) { if (q) cudaFree(q); };
    f(p->h); f(p->fs); f(p->rho); f(p->part); f(p->phi); f(p->red); f(p->scal); f(p->row);
    for (int k = 0; k < 3; ++k) f(p->c[k]);
    delete p;
    return CMM_OK;
}

int cmm_sample_vort(const cmm_grid* grid_map, const cmm_grid* grid_out, const cmm_grid* grid_fine, const double* chix,
                    const double* chiy, const double* w_fine, int molly_stencil, double* out, void* stream)
{
    cmm::Grid gm, go, gf;
    if (!to_grid(grid_map, &gm) || !to_grid(grid_out, &go) || !to_grid(grid_fine, &gf)) return fail(CMM_ERR_PARAM, "bad grid");
    if (!chix || !chiy || !w_fine || !out) return fail(CMM_ERR_PARAM, "NULL pointer");
    if (molly_stencil != 0 && molly_stencil != 4 && molly_stencil != 8) return fail(CMM_ERR_PARAM, "molly_stencil must be 0, 4 or 8");
    return cuda_rc(cmm::launch_sample_vort(gm, go, gf, chix, chiy, w_fine, molly_stencil, out, go.NX,
                                           static_cast<cudaStream_t>(stream)), "cmm_sample_vort");
}

int cmm_fft_create(int nx, int ny, int precision, void* stream, cmm_fft** out)
{
    if (!out) return fail(CMM_ERR_PARAM, "out is NULL");
    *out = nullptr;
    if (precision != 0 && precision != 1) return fail(CMM_ERR_PARAM, "precision must be 0 (FP64) or 1 (FP32)");
    cmm_fft* f = new (std::nothrow) cmm_fft();
    if (!f) return fail(CMM_ERR_PARAM, "out of host memory");
    f->stream = static_cast<cudaStream_t>(stream);
    const int rc = cmm::fft::plan_create(f->plan, nx, ny, precision == 0, f->stream);
    if (rc) {
        delete f;
        return rc == -1 ? fail(CMM_ERR_PARAM, "unsupported FFT shape (nx even, nx/2 and ny <= 8192, prime factors <= 13)")
                        : fail(CMM_ERR_CUDA, "FFT twiddle tables: CUDA error");
    }
    *out = f;
    return CMM_OK;
}

int cmm_fft_r2c(cmm_fft* f, const void* in, void* out, int batch)
{
    if (!f || !in || !out || batch < 1) return fail(CMM_ERR_PARAM, "bad argument");
    return cuda_rc(cmm::fft::r2c(f->plan, in, out, batch, f->stream), "cmm_fft_r2c");
}

int cmm_fft_c2r(cmm_fft* f, void* in, void* out, int batch)
{
    if (!f || !in || !out || batch < 1) return fail(CMM_ERR_PARAM, "bad argument");
    return cuda_rc(cmm::fft::c2r(f->plan, in, out, batch, f->stream), "cmm_fft_c2r");
}

int cmm_fft_destroy(cmm_fft* f)
{
    if (!f) return CMM_OK;
    cmm::fft::plan_destroy(f->plan);
    delete f;
    return CMM_OK;
}

int cmm_poisson_create(const cmm_grid* grid_vort, const cmm_grid* grid_psi, double freq_cut_psi, void* stream,
                       cmm_poisson** out)
{
    if (!out) return fail(CMM_ERR_PARAM, "out is NULL");
    *out = nullptr;
    cmm_poisson* p = new (std::nothrow) cmm_poisson();
    if (!p) return fail(CMM_ERR_PARAM, "out of host memory");
    if (!to_grid(grid_vort, &p->gv) || !to_grid(grid_psi, &p->gp)) { delete p; return fail(CMM_ERR_PARAM, "bad grid"); }
    p->freq = freq_cut_psi;
    p->stream = static_cast<cudaStream_t>(stream);
    if (!cmm::make_plans(p->pv, p->gv, p->stream) || !cmm::make_plans(p->pp, p->gp, p->stream)) {
        cmm_poisson_destroy(p);
        return fail(CMM_ERR_PARAM, "FFT plan creation failed (grid sizes need NX even, sides <= 8192, prime factors <= 13)");
    }
    long long cmax = p->gv.Nfft > p->gp.Nfft ? p->gv.Nfft : p->gp.Nfft;
    if (cudaMalloc((void**)&p->spec, sizeof(double2) * (size_t)cmax) != cudaSuccess ||
        cudaMalloc((void**)&p->spec4, sizeof(double2) * 4 * (size_t)p->gp.Nfft) != cudaSuccess) {
        cmm_poisson_destroy(p);
        return fail(CMM_ERR_CUDA, "cudaMalloc failed");
    }
    *out = p;
    return CMM_OK;
}

int cmm_poisson_hermite(cmm_poisson* p, const double* vort, double* psi_out)
{
    if (!p || !vort || !psi_out) return fail(CMM_ERR_PARAM, "NULL argument");
    int rc = cuda_rc(cmm::fft_d2z(p->pv, vort, p->spec, p->stream), "FFT D2Z");
    if (!rc) rc = cuda_rc(cmm::launch_spec_psi(p->spec, p->gv, p->gp, p->freq, p->spec4, p->stream), "spec_psi");
    if (!rc) rc = cuda_rc(cmm::fft_z2d(p->pp, p->spec4, psi_out, 4, p->stream), "FFT Z2D");
    return rc;
}

int cmm_poisson_destroy(cmm_poisson* p)
{
    if (!p) return CMM_OK;
    cmm::destroy_plans(p->pv);
    cmm::destroy_plans(p->pp);
    if (p->spec) cudaFree(p->spec);
    if (p->spec4) cudaFree(p->spec4);
    delete p;
    return CMM_OK;
}

int cmm_particles_advect(const cmm_grid* grid_psi, double* pos, int num, const double* const* psi_levels, int l_order,
                         const double* Lp12, double dt, int time_integration_num, void* stream)
{
    cmm::ParticleArgs a{};
    if (!to_grid(grid_psi, &a.gp)) return fail(CMM_ERR_PARAM, "bad grid");
    if (num < 0 || (num > 0 && (!pos || !psi_levels || !Lp12))) return fail(CMM_ERR_PARAM, "bad arguments");
    if (l_order < 1 || l_order > cmm::kMaxLagrange) return fail(CMM_ERR_PARAM, "l_order must be 1..4");
    int need = time_integration_num == 30 ? 3 : time_integration_num == 20 ? 2 : 2;
    if (l_order < need) return fail(CMM_ERR_PARAM, "too few psi levels for this scheme");
    a.pos = pos; a.num = num;
    for (int l = 0; l < l_order; ++l) { a.psi[l] = psi_levels[l]; a.Lp12[l] = Lp12[l]; }
    a.dt = dt; a.time_integration_num = time_integration_num; a.l_order = l_order;
    cudaError_t e = cmm::launch_particles(a, static_cast<cudaStream_t>(stream));
    if (e == cudaErrorInvalidValue) return fail(CMM_ERR_UNSUPPORTED, "particle scheme not built (10, 20, 30 are)");
    return cuda_rc(e, "cmm_particles_advect");
}

int cmm_diagnostics(const cmm_grid* grid_psi, const double* psi, const cmm_grid* grid_coarse, const double* vort,
                    double* out3, void* stream)
{
    cmm::Grid gp, gc;
    if (!to_grid(grid_psi, &gp) || !to_grid(grid_coarse, &gc)) return fail(CMM_ERR_PARAM, "bad grid");
    if (!psi || !vort || !out3) return fail(CMM_ERR_PARAM, "NULL pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* scratch = nullptr;
    int rc = cuda_rc(cudaMalloc((void**)&scratch, sizeof(double) * (3 * cmm::kReduceBlocks + 8)), "cudaMalloc");
    if (rc) return rc;
    double* res = scratch + 3 * cmm::kReduceBlocks;
    cudaError_t e = cmm::launch_sumsq(psi + gp.N, 2 * gp.N, scratch, res, s);
    if (e == cudaSuccess) e = cmm::launch_sumsq(vort, gc.N, scratch, res + 1, s);
    if (e == cudaSuccess) e = cmm::launch_stats(vort, gc.N, 1, scratch, res + 4, s);
    double h[8] = {0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, res, sizeof(double) * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(scratch);
    if (e != cudaSuccess) return cuda_rc(e, "cmm_diagnostics");
    out3[0] = 0.5 * gp.hx * gp.hy * h[0];
    out3[1] = 0.5 * gc.hx * gc.hy * h[1];
    double w_max = h[5] > 0 ? h[5] : 0.0, w_min = h[4] < 0 ? h[4] : 0.0;
    out3[2] = w_max > -w_min ? w_max : -w_min;
    return CMM_OK;
}

// ---------------------------------------------------------------- ensembles
int cmm_ensemble_create(int n_members, const int* argc, const char* const* argv, void* stream, cmm_ensemble** out)
{
    if (!out) return fail(CMM_ERR_PARAM, "out is NULL");
    *out = nullptr;
    if (n_members <= 0 || !argc || !argv) return fail(CMM_ERR_PARAM, "an ensemble needs members and their arguments");
    cmm_ensemble* e = new (std::nothrow) cmm_ensemble();
    if (!e) return fail(CMM_ERR_PARAM, "out of host memory");
    e->stream = static_cast<cudaStream_t>(stream);
    const char* const* a = argv;
    for (int i = 0; i < n_members; ++i) {
        cmm::Settings st;
        if (argc[i] < 0 || !st.apply_cli(argc[i], a)) {
            std::string msg = "member " + std::to_string(i) + ": " + st.error;
            delete e;
            return fail(msg.find("parameter file") != std::string::npos ? CMM_ERR_IO : CMM_ERR_PARAM, msg);
        }
        st.file_name = st.derived_file_name();
        e->settings.push_back(st);
        a += argc[i];
    }
    e->discrete.resize((size_t)n_members);
    *out = e;
    g_err.clear();
    return CMM_OK;
}

int cmm_ensemble_set_initial_discrete(cmm_ensemble* e, int member, const double* v, size_t n)
{
    if (!e || !v) return fail(CMM_ERR_PARAM, "NULL argument");
    if (e->ens) return fail(CMM_ERR_STATE, "cmm_ensemble_set_initial_discrete after cmm_ensemble_init");
    if (member < 0 || member >= (int)e->settings.size()) return fail(CMM_ERR_PARAM, "no such member");
    size_t need = (size_t)e->settings[(size_t)member].initial_discrete_grid * e->settings[(size_t)member].initial_discrete_grid;
    if (n != need) return fail(CMM_ERR_PARAM, "discrete initial condition needs initial_discrete_grid^2 values");
    e->discrete[(size_t)member].assign(v, v + n);
    return CMM_OK;
}

int cmm_ensemble_set_graphs(cmm_ensemble* e, int on)
{
    if (!e) return fail(CMM_ERR_PARAM, "ensemble is NULL");
    e->graphs = on != 0;
    if (e->ens) e->ens->use_graphs = e->graphs;
    return CMM_OK;
}

int cmm_ensemble_init(cmm_ensemble* e)
{
    if (!e) return fail(CMM_ERR_PARAM, "ensemble is NULL");
    if (e->ens) return fail(CMM_ERR_STATE, "cmm_ensemble_init called twice");
    cmm::EnsembleSim* ens = new (std::nothrow) cmm::EnsembleSim(e->settings);
    if (!ens) return fail(CMM_ERR_PARAM, "out of host memory");
    ens->stream = e->stream;
    ens->use_graphs = e->graphs;
    ens->fused_mode = e->fused;
    ens->wait_limit = e->wait_limit;
    for (int i = 0; i < ens->size(); ++i) {
        const auto& d = e->discrete[(size_t)i];
        if (!d.empty() && ens->set_initial_discrete(i, d.data(), d.size())) {
            std::string msg = ens->err;
            delete ens;
            return fail(CMM_ERR_PARAM, msg);
        }
    }
    int rc = ens->init();
    if (rc) {
        std::string msg = ens->err;
        delete ens;
        return fail(rc, msg);
    }
    e->ens = ens;
    return CMM_OK;
}

int cmm_ensemble_step(cmm_ensemble* e, int n)
{
    if (!e || !e->ens) return fail(CMM_ERR_STATE, "cmm_ensemble_step before cmm_ensemble_init");
    for (int k = 0; k < n; ++k) {
        int rc = e->ens->step();
        if (rc == 1) return 1;
        if (rc) return fail(rc, e->ens->err);
    }
    return CMM_OK;
}

int cmm_ensemble_run(cmm_ensemble* e)
{
    if (!e || !e->ens) return fail(CMM_ERR_STATE, "cmm_ensemble_run before cmm_ensemble_init");
    int rc = e->ens->run();
    return rc ? fail(rc, e->ens->err) : CMM_OK;
}

int cmm_ensemble_get_scalar(cmm_ensemble* e, int member, const char* name, double* out)
{
    if (!e || !e->ens || !name || !out) return fail(CMM_ERR_STATE, "ensemble not initialised or NULL argument");
    if (member < 0 || member >= e->ens->size()) return fail(CMM_ERR_PARAM, "no such member");
    cmm::EulerSim& s = e->ens->member(member);
    int rc = s.get_scalar(name, out);
    return rc ? fail(rc, s.err) : CMM_OK;
}

int cmm_ensemble_get_field(cmm_ensemble* e, int member, const char* name, void* dst, size_t bytes)
{
    if (!e || !e->ens || !name || (!dst && bytes)) return fail(CMM_ERR_STATE, "ensemble not initialised or NULL argument");
    if (member < 0 || member >= e->ens->size()) return fail(CMM_ERR_PARAM, "no such member");
    cmm::EulerSim& s = e->ens->member(member);
    int rc = s.get_field(name, dst, bytes);
    return rc ? fail(rc, s.err) : CMM_OK;
}

size_t cmm_ensemble_field_bytes(cmm_ensemble* e, int member, const char* name)
{
    if (!e || !e->ens || !name || member < 0 || member >= e->ens->size()) return 0;
    return e->ens->member(member).field_bytes(name);
}

int cmm_ensemble_stats(cmm_ensemble* e, long long* out6)
{
    if (!e || !e->ens || !out6) return fail(CMM_ERR_STATE, "ensemble not initialised or NULL argument");
    cmm::EnsembleSim& x = *e->ens;
    out6[0] = x.member_steps;
    out6[1] = x.iterations;
    out6[2] = x.launches;
    out6[3] = x.size();
    out6[4] = x.blocks[cmm::kEnsAdvect];
    out6[5] = x.blocks[cmm::kEnsSampleVort];
    return CMM_OK;
}

int cmm_ensemble_set_fused(cmm_ensemble* e, int mode)
{
    if (!e) return fail(CMM_ERR_PARAM, "ensemble is NULL");
    if (e->ens) return fail(CMM_ERR_STATE, "cmm_ensemble_set_fused after cmm_ensemble_init");
    if (mode < 0 || mode > 2) return fail(CMM_ERR_PARAM, "iteration form 0 (two-phase), 1 (single launch) or 2 (tuned)");
    e->fused = mode;
    return CMM_OK;
}

int cmm_ensemble_set_wait_limit(cmm_ensemble* e, long long polls)
{
    if (!e) return fail(CMM_ERR_PARAM, "ensemble is NULL");
    if (polls < 0) return fail(CMM_ERR_PARAM, "the wait limit is a number of polls (>= 0)");
    e->wait_limit = polls;
    if (e->ens) e->ens->set_wait_limit(polls);
    return CMM_OK;
}

int cmm_ensemble_fused_info(cmm_ensemble* e, long long* out6, char* why, size_t why_cap)
{
    if (!e || !e->ens || !out6) return fail(CMM_ERR_STATE, "ensemble not initialised or NULL argument");
    cmm::EnsembleSim& x = *e->ens;
    out6[0] = x.fused_available() ? 1 : 0;
    out6[1] = x.fused() ? 1 : 0;
    out6[2] = x.fused_minb;
    out6[3] = x.fused_blocks;
    out6[4] = x.fused_g;
    out6[5] = x.last_waves;
    if (why && why_cap) {
        const size_t n = std::min(why_cap - 1, x.fused_why.size());
        std::memcpy(why, x.fused_why.data(), n);
        why[n] = 0;
    }
    return CMM_OK;
}

int cmm_ensemble_tuning(cmm_ensemble* e, long long* out4, int cap)
{
    if (!e || !e->ens || (!out4 && cap > 0)) return fail(CMM_ERR_STATE, "ensemble not initialised or NULL argument");
    const auto& t = e->ens->tuning;
    const int n = std::min(cap, (int)t.size());
    for (int k = 0; k < n; ++k) {
        out4[4 * k] = t[(size_t)k].minb;
        out4[4 * k + 1] = t[(size_t)k].blocks;
        out4[4 * k + 2] = t[(size_t)k].g;
        out4[4 * k + 3] = (long long)(t[(size_t)k].ms * 1e6);
    }
    return (int)t.size();
}

int cmm_ensemble_set_profiling(cmm_ensemble* e, int on)
{
    if (!e || !e->ens) return fail(CMM_ERR_STATE, "cmm_ensemble_set_profiling before cmm_ensemble_init");
    int rc = e->ens->set_profiling(on != 0);
    return rc ? fail(rc, e->ens->err) : CMM_OK;
}

int cmm_ensemble_profile(cmm_ensemble* e, unsigned long long* out56)
{
    if (!e || !e->ens || !out56) return fail(CMM_ERR_STATE, "ensemble not initialised or NULL argument");
    int rc = e->ens->read_profile(out56);
    return rc ? fail(rc, e->ens->err) : CMM_OK;
}

int cmm_ensemble_destroy(cmm_ensemble* e)
{
    if (!e) return CMM_OK;
    delete e->ens;
    delete e;
    return CMM_OK;
}

}  // extern "C"
