"""Python binding of libcmm_gb300.so (the C-ABI of include/cmm_abi.h) via ctypes.

This is the reference-facing host API used by tests, smoke() and bench.py:
`Simulation(argv)` mirrors the reference executable's COMMAND=VALUE /
param_file interface, and the module-level kernel functions mirror its host
functions on caller-owned device buffers.  There is no CPU fallback: loading
fails loudly when the CUDA library has not been built.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libcmm_gb300.so")
CLI_PATH = os.path.join(HERE, "lib", "SimulationCuda2d.out")

CMM_OK = 0
CMM_ERR_PARAM = -1
CMM_ERR_IO = -2
CMM_ERR_CUDA = -3
CMM_ERR_SATURATED = -4
CMM_ERR_STATE = -5
CMM_ERR_UNSUPPORTED = -6
CMM_ERR_NOT_FOUND = -7
CMM_ERR_TIMEOUT = -8

# every entry point declared in include/cmm_abi.h
EXPORTS = [
    "cmm_last_error", "cmm_version", "cmm_create", "cmm_set_stream", "cmm_set_initial_discrete", "cmm_init",
    "cmm_step", "cmm_run", "cmm_get_field", "cmm_field_bytes", "cmm_get_scalar", "cmm_set_profiling",
    "cmm_settings_text",
    "cmm_file_name", "cmm_destroy", "cmm_advect_map", "cmm_incomp_max", "cmm_compose_stack", "cmm_sample_vort",
    "cmm_poisson_create", "cmm_poisson_hermite", "cmm_poisson_destroy", "cmm_particles_advect", "cmm_diagnostics",
    "cmm_diagnostics_noalloc", "cmm_compose_stack_var", "cmm_vlasov_create", "cmm_vlasov_potential",
    "cmm_vlasov_diagnostics", "cmm_vlasov_destroy", "cmm_ensemble_create", "cmm_ensemble_set_initial_discrete",
    "cmm_ensemble_set_graphs", "cmm_ensemble_init", "cmm_ensemble_step", "cmm_ensemble_run",
    "cmm_ensemble_get_scalar", "cmm_ensemble_get_field", "cmm_ensemble_field_bytes", "cmm_ensemble_stats",
    "cmm_ensemble_set_fused", "cmm_ensemble_set_wait_limit", "cmm_ensemble_fused_info", "cmm_ensemble_tuning",
    "cmm_ensemble_set_profiling", "cmm_ensemble_profile",
    "cmm_ensemble_destroy", "cmm_upsampler_create", "cmm_upsampler_destroy", "cmm_upsampler_num_params",
    "cmm_upsampler_get_params", "cmm_upsampler_set_params", "cmm_upsampler_get_grads", "cmm_upsampler_set_scales",
    "cmm_upsampler_get_scales", "cmm_upsampler_collect", "cmm_upsampler_dataset_size", "cmm_upsampler_clear_dataset",
    "cmm_upsampler_train",
    "cmm_upsampler_loss_grad", "cmm_upsampler_infer", "cmm_upsampler_evaluate", "cmm_upsampler_save",
    "cmm_upsampler_load", "cmm_attach_upsampler", "cmm_conv3x3", "cmm_conv3x3_weight_grad", "cmm_upsampler_time_infer",
    "cmm_fft_create", "cmm_fft_r2c", "cmm_fft_c2r", "cmm_fft_destroy",
]


class CmmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("cmm error %d: %s" % (code, msg))
        self.code = code


class CmmGrid(C.Structure):
    _fields_ = [("NX", C.c_int), ("NY", C.c_int), ("bounds", C.c_double * 4)]


def grid(n, bounds=(0.0, 6.283185307179586, 0.0, 6.283185307179586)):
    g = CmmGrid()
    g.NX = g.NY = int(n)
    for i in range(4):
        g.bounds[i] = float(bounds[i])
    return g


_lib = None


def lib():
    """Load libcmm_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libcmm_gb300.so is missing: run __graft_entry__.build() (nvcc, sm_103a)")
    L = C.CDLL(LIB_PATH)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.c_int
    L.cmm_last_error.restype = C.c_char_p
    L.cmm_version.restype = C.c_char_p
    L.cmm_create.argtypes = [ip, C.POINTER(C.c_char_p), C.POINTER(vp)]
    L.cmm_set_stream.argtypes = [vp, vp]
    L.cmm_set_initial_discrete.argtypes = [vp, dp, C.c_size_t]
    L.cmm_init.argtypes = [vp]
    L.cmm_step.argtypes = [vp, ip]
    L.cmm_run.argtypes = [vp]
    L.cmm_get_field.argtypes = [vp, C.c_char_p, vp, C.c_size_t]
    L.cmm_field_bytes.argtypes = [vp, C.c_char_p]
    L.cmm_field_bytes.restype = C.c_size_t
    L.cmm_get_scalar.argtypes = [vp, C.c_char_p, dp]
    L.cmm_set_profiling.argtypes = [vp, ip]
    L.cmm_settings_text.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.cmm_file_name.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.cmm_destroy.argtypes = [vp]
    gp = C.POINTER(CmmGrid)
    L.cmm_advect_map.argtypes = [gp, gp, vp, vp, vp, vp, C.POINTER(vp), ip, dp, dp, C.c_double, C.c_double, ip, ip, vp]
    L.cmm_incomp_max.argtypes = [gp, gp, vp, vp, vp, vp]
    L.cmm_compose_stack.argtypes = [gp, gp, vp, vp, vp, ip, ip, vp, gp, vp, vp]
    L.cmm_sample_vort.argtypes = [gp, gp, gp, vp, vp, vp, ip, vp, vp]
    L.cmm_poisson_create.argtypes = [gp, gp, C.c_double, vp, C.POINTER(vp)]
    L.cmm_poisson_hermite.argtypes = [vp, vp, vp]
    L.cmm_poisson_destroy.argtypes = [vp]
    L.cmm_fft_create.argtypes = [ip, ip, ip, vp, C.POINTER(vp)]
    L.cmm_fft_r2c.argtypes = [vp, vp, vp, ip]
    L.cmm_fft_c2r.argtypes = [vp, vp, vp, ip]
    L.cmm_fft_destroy.argtypes = [vp]
    L.cmm_particles_advect.argtypes = [gp, vp, ip, C.POINTER(vp), ip, dp, C.c_double, ip, vp]
    L.cmm_diagnostics.argtypes = [gp, vp, gp, vp, dp, vp]
    L.cmm_diagnostics_noalloc.argtypes = [gp, vp, gp, vp, dp, vp]
    L.cmm_compose_stack_var.argtypes = [gp, gp, vp, vp, vp, ip, ip, ip, vp, gp, vp, vp]
    L.cmm_vlasov_create.argtypes = [gp, gp, vp, C.POINTER(vp)]
    L.cmm_vlasov_potential.argtypes = [vp, gp, gp, vp, vp, vp, ip, vp]
    L.cmm_vlasov_diagnostics.argtypes = [vp, gp, vp, vp, dp]
    L.cmm_vlasov_destroy.argtypes = [vp]
    L.cmm_ensemble_create.argtypes = [ip, C.POINTER(ip), C.POINTER(C.c_char_p), vp, C.POINTER(vp)]
    L.cmm_ensemble_set_initial_discrete.argtypes = [vp, ip, dp, C.c_size_t]
    L.cmm_ensemble_set_graphs.argtypes = [vp, ip]
    L.cmm_ensemble_init.argtypes = [vp]
    L.cmm_ensemble_step.argtypes = [vp, ip]
    L.cmm_ensemble_run.argtypes = [vp]
    L.cmm_ensemble_get_scalar.argtypes = [vp, ip, C.c_char_p, dp]
    L.cmm_ensemble_get_field.argtypes = [vp, ip, C.c_char_p, vp, C.c_size_t]
    L.cmm_ensemble_field_bytes.argtypes = [vp, ip, C.c_char_p]
    L.cmm_ensemble_field_bytes.restype = C.c_size_t
    L.cmm_ensemble_stats.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.cmm_ensemble_set_fused.argtypes = [vp, ip]
    L.cmm_ensemble_set_wait_limit.argtypes = [vp, C.c_longlong]
    L.cmm_ensemble_fused_info.argtypes = [vp, C.POINTER(C.c_longlong), C.c_char_p, C.c_size_t]
    L.cmm_ensemble_tuning.argtypes = [vp, C.POINTER(C.c_longlong), ip]
    L.cmm_ensemble_set_profiling.argtypes = [vp, ip]
    L.cmm_ensemble_profile.argtypes = [vp, C.POINTER(C.c_ulonglong)]
    L.cmm_ensemble_destroy.argtypes = [vp]
    fp, u16p, llp = C.POINTER(C.c_float), C.POINTER(C.c_ushort), C.POINTER(C.c_longlong)
    L.cmm_upsampler_create.argtypes = [ip, ip, C.c_ulonglong, vp, C.POINTER(vp)]
    L.cmm_upsampler_destroy.argtypes = [vp]
    L.cmm_upsampler_num_params.argtypes = [vp]
    L.cmm_upsampler_num_params.restype = C.c_longlong
    for name in ("cmm_upsampler_get_params", "cmm_upsampler_set_params", "cmm_upsampler_get_grads"):
        getattr(L, name).argtypes = [vp, fp, C.c_longlong]
    L.cmm_upsampler_set_scales.argtypes = [vp, dp, C.c_double]
    L.cmm_upsampler_get_scales.argtypes = [vp, dp, dp]
    L.cmm_upsampler_collect.argtypes = [vp, vp]
    L.cmm_upsampler_dataset_size.argtypes = [vp]
    L.cmm_upsampler_clear_dataset.argtypes = [vp]
    L.cmm_upsampler_train.argtypes = [vp, ip, ip, C.c_double, C.c_ulonglong, dp, dp]
    L.cmm_upsampler_loss_grad.argtypes = [vp, fp, fp, ip, ip, ip, ip, dp]
    L.cmm_upsampler_infer.argtypes = [vp, fp, ip, ip, fp]
    L.cmm_upsampler_evaluate.argtypes = [vp, vp, dp]
    L.cmm_upsampler_save.argtypes = [vp, C.c_char_p]
    L.cmm_upsampler_time_infer.argtypes = [vp, ip, ip, ip, dp]
    L.cmm_upsampler_load.argtypes = [vp, C.c_char_p]
    L.cmm_attach_upsampler.argtypes = [vp, vp, ip, C.c_double]
    L.cmm_conv3x3.argtypes = [u16p, u16p, fp, u16p, u16p, ip, ip, ip, ip, ip, ip, fp, u16p]
    L.cmm_conv3x3_weight_grad.argtypes = [u16p, u16p, ip, ip, ip, ip, ip, fp, fp]
    _lib = L
    return L


def last_error():
    return lib().cmm_last_error().decode()


def check(rc, allow=()):
    if rc < 0 and rc not in allow:
        raise CmmError(rc, last_error())
    return rc


def _dptr(a):
    """Device or host pointer of a numpy array / torch tensor / int."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def _darr(vals):
    arr = (C.c_double * max(1, len(vals)))(*[float(v) for v in vals])
    return arr


class Simulation:
    """One CMM run configured like `SimulationCuda2d.out [param_file=F] [KEY=VALUE ...]`."""

    def __init__(self, argv, stream=None):
        L = lib()
        args = ["cmm"] + [str(a) for a in argv]
        arr = (C.c_char_p * len(args))(*[a.encode() for a in args])
        h = C.c_void_p()
        check(L.cmm_create(len(args), arr, C.byref(h)))
        self.h = h
        self.L = L
        if stream is not None:
            check(L.cmm_set_stream(self.h, C.c_void_p(stream)))

    def close(self):
        if getattr(self, "h", None):
            self.L.cmm_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_initial_discrete(self, values):
        import numpy as np
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        check(self.L.cmm_set_initial_discrete(self.h, v.ctypes.data_as(C.POINTER(C.c_double)), v.size))

    def init(self):
        return check(self.L.cmm_init(self.h))

    def step(self, n=1):
        return check(self.L.cmm_step(self.h, int(n)), allow=(CMM_ERR_SATURATED,))

    def run(self):
        return check(self.L.cmm_run(self.h), allow=(CMM_ERR_SATURATED,))

    def field(self, name):
        import numpy as np
        nb = self.L.cmm_field_bytes(self.h, name.encode())
        if nb == 0 and name != "Map_stack":
            raise CmmError(CMM_ERR_NOT_FOUND, "unknown field " + name)
        out = np.empty(nb // 8, dtype=np.float64)
        check(self.L.cmm_get_field(self.h, name.encode(), out.ctypes.data_as(C.c_void_p), nb))
        return out

    def scalar(self, name):
        v = C.c_double()
        check(self.L.cmm_get_scalar(self.h, name.encode(), C.byref(v)))
        return v.value

    def set_profiling(self, on=True):
        check(self.L.cmm_set_profiling(self.h, 1 if on else 0))

    def settings_text(self):
        n = self.L.cmm_settings_text(self.h, None, 0)
        buf = C.create_string_buffer(n + 1)
        self.L.cmm_settings_text(self.h, buf, n + 1)
        return buf.value.decode()

    def attach_upsampler(self, ups, every=8, tol=1e-4):
        """Learned psi between exact evaluations every `every` steps (None detaches)."""
        check(self.L.cmm_attach_upsampler(self.h, ups.h if ups is not None else None, int(every), float(tol)))

    def file_name(self):
        buf = C.create_string_buffer(4096)
        self.L.cmm_file_name(self.h, buf, 4096)
        return buf.value.decode()


# ---------------------------------------------------------------- kernel API
def advect_map(gm, gp, chix, chiy, chix_out, chiy_out, psi_levels, L1, L12, dt, eps, ti=30, order=1, stream=None):
    levels = (C.c_void_p * len(psi_levels))(*[_dptr(p) for p in psi_levels])
    return check(lib().cmm_advect_map(C.byref(gm), C.byref(gp), _dptr(chix), _dptr(chiy), _dptr(chix_out),
                                      _dptr(chiy_out), levels, len(psi_levels), _darr(L1), _darr(L12), dt, eps, ti,
                                      order, stream))


def incomp_max(gcheck, gm, chix, chiy, d_result, stream=None):
    return check(lib().cmm_incomp_max(C.byref(gcheck), C.byref(gm), _dptr(chix), _dptr(chiy), _dptr(d_result), stream))


def compose_stack(gm, gt, chix, chiy, stack, n_maps, ic_num, out, discrete=None, gd=None, stream=None):
    return check(lib().cmm_compose_stack(C.byref(gm), C.byref(gt), _dptr(chix), _dptr(chiy), _dptr(stack), n_maps,
                                         ic_num, _dptr(discrete), C.byref(gd) if gd is not None else None,
                                         _dptr(out), stream))


def sample_vort(gm, gout, gf, chix, chiy, w_fine, out, molly=0, stream=None):
    return check(lib().cmm_sample_vort(C.byref(gm), C.byref(gout), C.byref(gf), _dptr(chix), _dptr(chiy),
                                       _dptr(w_fine), molly, _dptr(out), stream))


class Poisson:
    def __init__(self, gv, gp, freq, stream=None):
        self.h = C.c_void_p()
        check(lib().cmm_poisson_create(C.byref(gv), C.byref(gp), freq, stream, C.byref(self.h)))

    def __call__(self, vort, psi_out):
        return check(lib().cmm_poisson_hermite(self.h, _dptr(vort), _dptr(psi_out)))

    def close(self):
        if self.h:
            lib().cmm_poisson_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class FFT:
    """The library's 2D real FFT: ny x nx reals <-> ny x (nx/2+1) complex (unnormalised),
    precision 0 = FP64, 1 = FP32 (device buffers: torch tensors or raw pointers)."""

    def __init__(self, nx, ny, precision=0, stream=None):
        self.h = C.c_void_p()
        check(lib().cmm_fft_create(int(nx), int(ny), int(precision), stream, C.byref(self.h)))

    def r2c(self, x, out, batch=1):
        return check(lib().cmm_fft_r2c(self.h, _dptr(x), _dptr(out), int(batch)))

    def c2r(self, x, out, batch=1):
        return check(lib().cmm_fft_c2r(self.h, _dptr(x), _dptr(out), int(batch)))

    def close(self):
        if self.h:
            lib().cmm_fft_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def particles_advect(gp, pos, num, psi_levels, Lp12, dt, ti=30, stream=None):
    levels = (C.c_void_p * len(psi_levels))(*[_dptr(p) for p in psi_levels])
    return check(lib().cmm_particles_advect(C.byref(gp), _dptr(pos), num, levels, len(psi_levels), _darr(Lp12), dt,
                                            ti, stream))


def diagnostics(gp, psi, gc, vort, stream=None):
    out = (C.c_double * 3)()
    check(lib().cmm_diagnostics(C.byref(gp), _dptr(psi), C.byref(gc), _dptr(vort), out, stream))
    return list(out)


def diagnostics_noalloc(gp, psi, gc, vort, stream=None):
    """cmm_diagnostics without device allocation (fixed in-library scratch;
    serialise overlapping calls)."""
    out = (C.c_double * 3)()
    check(lib().cmm_diagnostics_noalloc(C.byref(gp), _dptr(psi), C.byref(gc), _dptr(vort), out, stream))
    return list(out)


def compose_stack_var(gm, gt, chix, chiy, stack, n_maps, var_num, ic_num, out, discrete=None, gd=None, stream=None):
    """cmm_compose_stack_var: var_num 0 vorticity, 1 passive scalar, 2 Vlasov distribution."""
    check(lib().cmm_compose_stack_var(C.byref(gm), C.byref(gt), _dptr(chix), _dptr(chiy), _dptr(stack), n_maps, var_num,
                                      ic_num, _dptr(discrete), C.byref(gd) if gd is not None else None, _dptr(out),
                                      stream))


class VlasovPotential:
    """cmm_vlasov_*: the Vlasov-Poisson potential and conservation targets on
    caller-owned device buffers."""

    def __init__(self, grid_vort, grid_psi, stream=None):
        self.h = C.c_void_p()
        self.gv, self.gp = grid_vort, grid_psi
        check(lib().cmm_vlasov_create(C.byref(grid_vort), C.byref(grid_psi), stream, C.byref(self.h)))

    def potential(self, gm, gf, chix, chiy, f_fine, psi_out, molly=0):
        check(lib().cmm_vlasov_potential(self.h, C.byref(gm), C.byref(gf), _dptr(chix), _dptr(chiy), _dptr(f_fine),
                                         molly, _dptr(psi_out)))

    def diagnostics(self, gc, f_coarse, psi):
        out = (C.c_double * 9)()
        check(lib().cmm_vlasov_diagnostics(self.h, C.byref(gc), _dptr(f_coarse), _dptr(psi), out))
        return list(out)

    def close(self):
        if self.h:
            lib().cmm_vlasov_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Ensemble:
    """Many mixed-form runs of uneven sizes advanced together (cmm_ensemble_*): members[i] is
    the argument list member i would get as a Simulation."""

    def __init__(self, members, stream=None, graphs=True, fused=None):
        """fused: None (default) the autotuner's choice of iteration form, True the single launch,
        False the two-phase iteration with the remaps on the host."""
        L = lib()
        flat, counts = [], []
        for argv in members:
            args = ["cmm"] + [str(a) for a in argv]
            flat += args
            counts.append(len(args))
        self._keep = [a.encode() for a in flat]
        arr = (C.c_char_p * len(flat))(*self._keep)
        cnt = (C.c_int * len(counts))(*counts)
        h = C.c_void_p()
        check(L.cmm_ensemble_create(len(counts), cnt, arr, stream, C.byref(h)))
        self.h, self.L, self.n = h, L, len(counts)
        check(L.cmm_ensemble_set_graphs(self.h, 1 if graphs else 0))
        check(L.cmm_ensemble_set_fused(self.h, 2 if fused is None else (1 if fused else 0)))

    def close(self):
        if self.h:
            self.L.cmm_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_initial_discrete(self, i, values):
        import numpy as np
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        check(self.L.cmm_ensemble_set_initial_discrete(self.h, i, v.ctypes.data_as(C.POINTER(C.c_double)), v.size))

    def init(self):
        check(self.L.cmm_ensemble_init(self.h))

    def step(self, n=1):
        return check(self.L.cmm_ensemble_step(self.h, int(n)), allow=(CMM_ERR_SATURATED,))

    def run(self):
        return check(self.L.cmm_ensemble_run(self.h), allow=(CMM_ERR_SATURATED,))

    def scalar(self, i, name):
        out = C.c_double()
        check(self.L.cmm_ensemble_get_scalar(self.h, i, name.encode(), C.byref(out)))
        return out.value

    def field(self, i, name):
        import numpy as np
        nb = self.L.cmm_ensemble_field_bytes(self.h, i, name.encode())
        if nb == 0:
            raise CmmError(CMM_ERR_NOT_FOUND, "unknown field " + name)
        out = np.empty(nb // 8, dtype=np.float64)
        check(self.L.cmm_ensemble_get_field(self.h, i, name.encode(), out.ctypes.data_as(C.c_void_p), nb))
        return out

    def stats(self):
        """{member_steps, iterations, launches, members, advect_blocks, sample_blocks}"""
        out = (C.c_longlong * 6)()
        check(self.L.cmm_ensemble_stats(self.h, out))
        return dict(zip(("member_steps", "iterations", "launches", "members", "advect_blocks", "sample_blocks"),
                        list(out)))

    def set_wait_limit(self, polls):
        """Polls after which a grid barrier of the single-launch iteration gives up (CMM_ERR_TIMEOUT)."""
        check(self.L.cmm_ensemble_set_wait_limit(self.h, C.c_longlong(int(polls))))

    def fused_info(self):
        """{available, fused, register_budget, blocks, tiles_per_task, waves, why}: whether the single
        launch is available and in use, the shape in use (register_budget 0: the two-phase iteration),
        or why it is unavailable."""
        out = (C.c_longlong * 6)()
        why = C.create_string_buffer(512)
        check(self.L.cmm_ensemble_fused_info(self.h, out, why, C.c_size_t(512)))
        return dict(available=bool(out[0]), fused=bool(out[1]), register_budget=out[2], blocks=out[3],
                    tiles_per_task=out[4], waves=out[5], why=why.value.decode())

    STAGES = ("precombine", "advect", "check", "compose", "fine_rows", "fine_columns", "fine_inverse_rows",
              "sample", "psi_rows", "psi_columns", "psi_inverse_rows")

    def set_profiling(self, on=True):
        """Count block cycles and tasks per stage of the single-launch iteration (on zeroes them)."""
        check(self.L.cmm_ensemble_set_profiling(self.h, 1 if on else 0))

    def profile(self):
        """{stage: (block cycles, tasks)}, barrier block cycles and ns per wave since profiling was switched on."""
        out = (C.c_ulonglong * 56)()
        check(self.L.cmm_ensemble_profile(self.h, out))
        stages = {n: (out[k], out[16 + k]) for k, n in enumerate(self.STAGES)}
        return dict(stages=stages, barrier_cycles=out[32], wave_ns=[out[40 + w] for w in range(16)])

    def tuning(self):
        """The autotuner's table: [(register_budget, blocks, tiles_per_task, median iteration ms), ...]
        (empty until tuned)."""
        out = (C.c_longlong * 128)()
        n = self.L.cmm_ensemble_tuning(self.h, out, 32)
        if n < 0:
            check(n)
        return [(out[4 * k], out[4 * k + 1], out[4 * k + 2], out[4 * k + 3] / 1e6) for k in range(min(n, 32))]



class Upsampler:
    """The learned psi network (cmm_upsampler_*): BF16 tensor-core training and inference."""

    def __init__(self, blocks=6, channels=32, seed=0, stream=None):
        L = lib()
        h = C.c_void_p()
        check(L.cmm_upsampler_create(int(blocks), int(channels), int(seed), stream, C.byref(h)))
        self.h, self.L, self.blocks, self.channels = h, L, blocks, channels

    def close(self):
        if getattr(self, "h", None):
            self.L.cmm_upsampler_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def num_params(self):
        return int(self.L.cmm_upsampler_num_params(self.h))

    def _vec(self, fn):
        import numpy as np
        out = np.empty(self.num_params(), dtype=np.float32)
        check(fn(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), out.size))
        return out

    def params(self):
        return self._vec(self.L.cmm_upsampler_get_params)

    def grads(self):
        return self._vec(self.L.cmm_upsampler_get_grads)

    def set_params(self, p):
        import numpy as np
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self.L.cmm_upsampler_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size))

    def set_scales(self, s_in, s_out):
        arr = (C.c_double * 7)(*[float(v) for v in s_in])
        check(self.L.cmm_upsampler_set_scales(self.h, arr, float(s_out)))

    def scales(self):
        arr = (C.c_double * 7)()
        out = C.c_double()
        check(self.L.cmm_upsampler_get_scales(self.h, arr, C.byref(out)))
        return list(arr), out.value

    def collect(self, sim):
        check(self.L.cmm_upsampler_collect(self.h, sim.h))

    def dataset_size(self):
        return int(self.L.cmm_upsampler_dataset_size(self.h))

    def clear_dataset(self):
        """Drop the collected pairs (streamed training: collect, train, clear)."""
        check(self.L.cmm_upsampler_clear_dataset(self.h))

    def train(self, iters, batch=8, lr=1e-3, seed=0):
        """-> (mean loss of the last steps, device seconds)"""
        loss, sec = C.c_double(), C.c_double()
        check(self.L.cmm_upsampler_train(self.h, int(iters), int(batch), float(lr), int(seed), C.byref(loss),
                                         C.byref(sec)))
        return loss.value, sec.value

    def loss_grad(self, inputs, targets, cut=0):
        """inputs[B, 7, h, w], targets[B, 2h, 2w] -> loss (gradient via grads()); cut > 0: the
        psi-space spectral loss of training"""
        import numpy as np
        x = np.ascontiguousarray(inputs, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        B, _, h, w = x.shape
        loss = C.c_double()
        fp = C.POINTER(C.c_float)
        check(self.L.cmm_upsampler_loss_grad(self.h, x.ctypes.data_as(fp), t.ctypes.data_as(fp), B, h, w, int(cut),
                                             C.byref(loss)))
        return loss.value

    def infer(self, inputs):
        """inputs[7, h, w] -> predicted sub-grid vorticity on the 2x grid [2h, 2w]"""
        import numpy as np
        x = np.ascontiguousarray(inputs, dtype=np.float32)
        _, h, w = x.shape
        out = np.empty((2 * h, 2 * w), dtype=np.float32)
        fp = C.POINTER(C.c_float)
        check(self.L.cmm_upsampler_infer(self.h, x.ctypes.data_as(fp), h, w, out.ctypes.data_as(fp)))
        return out

    def evaluate(self, sim):
        """relative differences from sim's exact psi of the cheap, learned and psi-grid psi"""
        arr = (C.c_double * 6)()
        check(self.L.cmm_upsampler_evaluate(self.h, sim.h, arr))
        return dict(zip(("cheap_linf", "cheap_l2", "learned_linf", "learned_l2", "grid_linf", "grid_l2"), list(arr)))

    def time_infer(self, h, w, iters=20):
        """device milliseconds of one inference on an h x w map grid"""
        ms = C.c_double()
        check(self.L.cmm_upsampler_time_infer(self.h, int(h), int(w), int(iters), C.byref(ms)))
        return ms.value

    def save(self, path):
        check(self.L.cmm_upsampler_save(self.h, str(path).encode()))

    def load(self, path):
        check(self.L.cmm_upsampler_load(self.h, str(path).encode()))


def conv3x3(x_bits, w_bits, bias=None, mask_bits=None, res_bits=None, relu=False):
    """One periodic 3x3 convolution of the network on BF16 bit arrays: x[B, H, W, cin],
    w[9, cin, cout] (uint16) -> (out float32, out BF16 bits), both [B, H, W, cout]."""
    import numpy as np
    L = lib()
    x = np.ascontiguousarray(x_bits, dtype=np.uint16)
    w = np.ascontiguousarray(w_bits, dtype=np.uint16)
    B, H, W, cin = x.shape
    cout = w.shape[2]
    u16 = C.POINTER(C.c_ushort)
    fp = C.POINTER(C.c_float)
    keep = []

    def opt(a, dt, ptr):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data_as(ptr)

    out = np.empty((B, H, W, cout), dtype=np.float32)
    outb = np.empty((B, H, W, cout), dtype=np.uint16)
    check(L.cmm_conv3x3(x.ctypes.data_as(u16), w.ctypes.data_as(u16), opt(bias, np.float32, fp),
                        opt(mask_bits, np.uint16, u16), opt(res_bits, np.uint16, u16), 1 if relu else 0, B, H, W,
                        cin, cout, out.ctypes.data_as(fp), outb.ctypes.data_as(u16)))
    return out, outb


def conv3x3_weight_grad(x_bits, dy_bits):
    """Weight and bias gradients of conv3x3 for x[B, H, W, cin], dy[B, H, W, cout] (BF16 bits)."""
    import numpy as np
    L = lib()
    x = np.ascontiguousarray(x_bits, dtype=np.uint16)
    dy = np.ascontiguousarray(dy_bits, dtype=np.uint16)
    B, H, W, cin = x.shape
    cout = dy.shape[3]
    dw = np.empty((9, cin, cout), dtype=np.float32)
    db = np.empty(cout, dtype=np.float32)
    u16 = C.POINTER(C.c_ushort)
    fp = C.POINTER(C.c_float)
    check(L.cmm_conv3x3_weight_grad(x.ctypes.data_as(u16), dy.ctypes.data_as(u16), B, H, W, cin, cout,
                                    dw.ctypes.data_as(fp), db.ctypes.data_as(fp)))
    return dw, db
