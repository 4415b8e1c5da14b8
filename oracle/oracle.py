"""ctypes wrapper of the CPU parity oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, never by the product.  The C sources restate
the reference's algorithm (see cmm_oracle.h for the citations).

`EulerOracle` drives og_init / og_step with the reference's host-side loop
logic (src/simulation/cmm-euler2d.cu:750-960: compute_next_timestep,
final-time clipping, save instants) so tests can compare with the golden
monitoring files the reference writes.
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


def build(force=False):
    """Compile liboracle.so with the committed Makefile (gcc + OpenMP)."""
    srcs = [os.path.join(HERE, f) for f in ("og_hermite.c", "og_fft.c", "og_euler.c", "og_vlasov.c", "og_sample.c", "og_learned.c",
                                          "cmm_oracle.h")]
    if not force and os.path.exists(LIB_PATH):
        if os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in srcs):
            return LIB_PATH
    subprocess.run(["make", "-s", "-C", HERE, "-B", "liboracle.so"], check=True)
    return LIB_PATH


class OgGrid(C.Structure):
    _fields_ = [("NX", C.c_int), ("NY", C.c_int), ("NX_fft", C.c_int),
                ("N", C.c_long), ("Nfft", C.c_long),
                ("hx", C.c_double), ("hy", C.c_double), ("bounds", C.c_double * 4)]


class OgParticleSet(C.Structure):
    _fields_ = [("num", C.c_int), ("tau", C.c_double), ("time_integration_num", C.c_int),
                ("init_time", C.c_double), ("init_vel", C.c_int)]


class OgFwdSet(C.Structure):
    _fields_ = [("num", C.c_int), ("init_time", C.c_double)]


class OgSettings(C.Structure):
    _fields_ = [("grid_coarse", C.c_int), ("grid_fine", C.c_int), ("grid_psi", C.c_int),
                ("grid_vort", C.c_int), ("bounds", C.c_double * 4), ("dt", C.c_double),
                ("time_integration_num", C.c_int), ("lagrange_order", C.c_int),
                ("lagrange_init_higher_order", C.c_int), ("map_update_order_num", C.c_int),
                ("map_epsilon", C.c_double), ("incomp_threshold", C.c_double),
                ("skip_remapping", C.c_int), ("molly_stencil", C.c_int),
                ("freq_cut_psi", C.c_double), ("initial_condition_num", C.c_int),
                ("initial_discrete", C.c_int), ("initial_discrete_grid", C.c_int),
                ("max_maps", C.c_int), ("n_particle_sets", C.c_int),
                ("psets", OgParticleSet * 8), ("simulation_type_num", C.c_int),
                ("forward_map", C.c_int), ("n_fwd_sets", C.c_int), ("fsets", OgFwdSet * 8)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        L.og_create.restype = C.c_void_p
        L.og_create.argtypes = [C.POINTER(OgSettings)]
        L.og_destroy.argtypes = [C.c_void_p]
        L.og_init.argtypes = [C.c_void_p]
        L.og_step.argtypes = [C.c_void_p, C.c_double, dp, C.POINTER(C.c_int)]
        L.og_set_particles.argtypes = [C.c_void_p, C.c_int, dp]
        L.og_set_discrete_initial.argtypes = [C.c_void_p, dp]
        for name in ("og_chix", "og_chiy", "og_psi", "og_vort_coarse", "og_vort_fine"):
            getattr(L, name).restype = dp
            getattr(L, name).argtypes = [C.c_void_p]
        L.og_particles.restype = dp
        L.og_particles.argtypes = [C.c_void_p, C.c_int]
        L.og_particle_vel.restype = dp
        L.og_particle_vel.argtypes = [C.c_void_p, C.c_int]
        L.og_grid_of.restype = C.POINTER(OgGrid)
        L.og_grid_of.argtypes = [C.c_void_p, C.c_int]
        for name in ("og_time", "og_energy_H", "og_enstrophy", "og_palinstrophy", "og_max_vorticity"):
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [C.c_void_p]
        for name in ("og_map_count", "og_loop_ctr", "og_old_ctr"):
            getattr(L, name).restype = C.c_int
            getattr(L, name).argtypes = [C.c_void_p]
        L.og_sample_points_dxdy.argtypes = [C.c_void_p, dp, dp, C.c_int]
        L.og_init.restype = C.c_int
        L.og_state_sample.argtypes = [C.c_void_p, C.c_int, C.c_int, dp, dp]
        L.og_state_vlasov_sample.argtypes = [C.c_void_p, C.c_int, dp, dp]
        L.og_vlasov_state_mesure.argtypes = [C.c_void_p, dp]
        L.og_set_init_data.argtypes = [dp, dp]
        L.og_state_zoom.argtypes = [C.c_void_p, C.c_int, dp, C.c_int, dp]
        for name in ("og_chix_f", "og_chiy_f"):
            getattr(L, name).restype = dp
            getattr(L, name).argtypes = [C.c_void_p]
        L.og_forward_monitors.argtypes = [C.c_void_p, dp, dp]
        L.og_set_forwarded_particles.argtypes = [C.c_void_p, C.c_int, dp]
        L.og_forward_sample.argtypes = [C.c_void_p, C.c_int, dp, dp, dp]
        L.og_restart.argtypes = [C.c_void_p, C.c_double, C.c_int, dp, dp, dp, dp, dp]
        L.og_restart.restype = C.c_int
        for name in ("og_stack_x", "og_stack_y"):
            getattr(L, name).restype = dp
            getattr(L, name).argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def stats_grid(v, hx, hy):
    """Debug-globals grid form (src/numerical/cmm-mesure.cu:217-232)."""
    v = np.asarray(v, dtype=np.float64)
    return [float(v.min()), float(v.max()), hx * hy * max(0.0, float(v.max())), hx * hy * float(v.sum())]


def stats_raw(v):
    """Debug-globals raw-array form (src/numerical/cmm-mesure.cu:234-249)."""
    v = np.asarray(v, dtype=np.float64)
    n = v.size
    return [float(v.min()), float(v.max()), max(0.0, float(v.max())) / n, float(v.sum()) / n]


class EulerOracle:
    """CPU restatement of one Euler-2D run, configured from a `Settings` object
    (cmm-turbulence_gb300 host-side settings mirror) or a plain dict."""

    def __init__(self, cfg):
        self.cfg = cfg
        L = lib()
        s = OgSettings()
        s.grid_coarse, s.grid_fine = cfg["grid_coarse"], cfg["grid_fine"]
        s.grid_psi, s.grid_vort = cfg["grid_psi"], cfg["grid_vort"]
        for i in range(4):
            s.bounds[i] = cfg["bounds"][i]
        s.dt = cfg["dt"]
        s.time_integration_num = cfg["time_integration_num"]
        s.lagrange_order = cfg["lagrange_order"]
        s.lagrange_init_higher_order = int(cfg["lagrange_init_higher_order"])
        s.map_update_order_num = cfg["map_update_order_num"]
        s.map_epsilon = cfg["map_epsilon"]
        s.incomp_threshold = cfg["incomp_threshold"]
        s.skip_remapping = int(cfg["skip_remapping"])
        s.molly_stencil = cfg["molly_stencil"]
        s.freq_cut_psi = cfg["freq_cut_psi"]
        s.initial_condition_num = cfg["initial_condition_num"]
        s.initial_discrete = int(cfg.get("initial_discrete", 0))
        s.initial_discrete_grid = cfg.get("initial_discrete_grid", 1)
        s.max_maps = cfg["max_maps"]
        s.simulation_type_num = int(cfg.get("simulation_type_num", 0))
        s.forward_map = int(cfg.get("forward_map", 0))
        fsets = cfg.get("forwarded", [])
        s.n_fwd_sets = len(fsets)
        for i, p in enumerate(fsets):
            s.fsets[i].num = p["num"]
            s.fsets[i].init_time = p["init_time"]
        psets = cfg.get("particles", [])
        s.n_particle_sets = len(psets)
        for i, p in enumerate(psets):
            s.psets[i].num = p["num"]
            s.psets[i].tau = p["tau"]
            s.psets[i].time_integration_num = p["time_integration_num"]
            s.psets[i].init_time = p["init_time"]
            s.psets[i].init_vel = int(p.get("init_vel", 0))
        self._s = s
        self.h = L.og_create(C.byref(s))
        self.L = L
        if "initial_params" in cfg:
            set_init_data(params=cfg["initial_params"])

    def close(self):
        if self.h:
            self.L.og_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def grid(self, which):
        g = self.L.og_grid_of(self.h, which).contents
        return g

    def set_discrete_initial(self, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self.L.og_set_discrete_initial(self.h, _dp(v))

    def set_particles(self, i, pos):
        p = np.ascontiguousarray(pos, dtype=np.float64)
        self.L.og_set_particles(self.h, i, _dp(p))

    def init(self):
        rc = self.L.og_init(self.h)
        if rc:
            raise ValueError("oracle initialisation rejected the grids (vort grid finer than psi grid?)")

    def restart(self, restart_time, files):
        """In place of init(): restart from a stored map stack given as the file
        contents of a MapStack folder (read_map_stack_dir / map_stack_files);
        readMapStack, src/simulation/cmm-simulation-host.cu:1256-1302."""
        nc4 = 4 * self.grid(0).N
        np4 = 4 * self.grid(2).N
        Lo = self.cfg["lagrange_order"]
        n = sum(1 for k in files if "Map_ChiX_H" in k) - 1
        sx = np.zeros(max(n, 1) * nc4)
        sy = np.zeros(max(n, 1) * nc4)
        for i in range(n):
            sx[i * nc4:(i + 1) * nc4] = files["Map_ChiX_H_%d" % i]
            sy[i * nc4:(i + 1) * nc4] = files["Map_ChiY_H_%d" % i]
        chix = np.ascontiguousarray(files["Map_ChiX_H_coarse"], dtype=np.float64)
        chiy = np.ascontiguousarray(files["Map_ChiY_H_coarse"], dtype=np.float64)
        prev = np.zeros(max(Lo - 1, 1) * np4)
        for l in range(1, Lo):
            prev[(l - 1) * np4:l * np4] = files["Stream_function_Psi_H_psi_%d" % l]
        for i, p in enumerate(self.cfg.get("particles", [])):
            self.set_particles(i, files["Particles_advected_pos_P%02d" % (i + 1)])
            if p["tau"] != 0:
                self.set_particle_velocity(i, files["Particles_advected_vel_U%02d" % (i + 1)])
        rc = self.L.og_restart(self.h, restart_time, n, _dp(sx), _dp(sy), _dp(chix), _dp(chiy), _dp(prev))
        if rc:
            raise ValueError("oracle restart rejected the stored map stack (%d maps, capacity %d)"
                             % (n, self.cfg["max_maps"]))
        return n

    def map_stack(self):
        """(X planes, Y planes) of the stacked sub-maps, shape (n, 4*Nc) each."""
        n, nc4 = self.map_count(), 4 * self.grid(0).N
        if n == 0:
            return np.zeros((0, nc4)), np.zeros((0, nc4))
        x = np.ctypeslib.as_array(self.L.og_stack_x(self.h), shape=(n * nc4,)).copy()
        y = np.ctypeslib.as_array(self.L.og_stack_y(self.h), shape=(n * nc4,)).copy()
        return x.reshape(n, nc4), y.reshape(n, nc4)

    def step(self, dt_now):
        e = C.c_double()
        r = C.c_int()
        rc = self.L.og_step(self.h, dt_now, C.byref(e), C.byref(r))
        return rc, e.value, bool(r.value)

    def _arr(self, fn, n):
        return np.ctypeslib.as_array(fn(self.h), shape=(n,)).copy()

    def chix(self):
        return self._arr(self.L.og_chix, 4 * self.grid(0).N)

    def chiy(self):
        return self._arr(self.L.og_chiy, 4 * self.grid(0).N)

    def psi(self, levels=1):
        return self._arr(self.L.og_psi, 4 * self.grid(2).N * levels)

    def vort(self):
        return self._arr(self.L.og_vort_coarse, self.grid(0).N)

    def vort_fine(self):
        return self._arr(self.L.og_vort_fine, 4 * self.grid(1).N)

    def particles(self, i):
        n = self.cfg["particles"][i]["num"]
        return np.ctypeslib.as_array(self.L.og_particles(self.h, i), shape=(2 * n,)).copy()

    def particle_velocity(self, i):
        """What the reference saves as Particles_advected_vel_U<i>: the velocity state of
        an inertial set (tau != 0), else (psi_x, psi_y) sampled at the tracers
        (k_h_sample_points_dxdy, src/ui/cmm-io.cu:580-600)."""
        p = self.cfg["particles"][i]
        if p["tau"] != 0:
            return np.ctypeslib.as_array(self.L.og_particle_vel(self.h, i), shape=(2 * p["num"],)).copy()
        pos = self.particles(i)
        out = np.empty_like(pos)
        self.L.og_sample_points_dxdy(self.h, _dp(pos), _dp(out), len(pos) // 2)
        return out

    def set_particle_velocity(self, i, vel):
        n = 2 * self.cfg["particles"][i]["num"]
        v = np.ascontiguousarray(vel, dtype=np.float64)
        np.ctypeslib.as_array(self.L.og_particle_vel(self.h, i), shape=(n,))[:] = v[:n]

    def time(self):
        return self.L.og_time(self.h)

    def map_count(self):
        return self.L.og_map_count(self.h)

    def loop_ctr(self):
        return self.L.og_loop_ctr(self.h)

    def old_ctr(self):
        return self.L.og_old_ctr(self.h)

    def energy(self):
        return self.L.og_energy_H(self.h)

    def enstrophy(self):
        return self.L.og_enstrophy(self.h)

    def palinstrophy(self):
        return self.L.og_palinstrophy(self.h)

    def max_vorticity(self):
        return self.L.og_max_vorticity(self.h)

    def sample(self, n, scalar_num):
        """Sampled outputs on an n x n grid: dict of the ten planes and the five
        conservation values (sample_compute_and_write, backward part)."""
        out = np.zeros(10 * n * n)
        mes = np.zeros(5)
        self.L.og_state_sample(self.h, n, scalar_num, _dp(out), _dp(mes))
        names = ("Map_ChiX", "Map_ChiY", "Scalar_Theta", "Vorticity_W", "Laplacian_W", "GradX_W", "GradY_W",
                 "Stream_function_Psi", "Velocity_UX", "Velocity_UY")
        planes = {k: out[i * n * n:(i + 1) * n * n].copy() for i, k in enumerate(names)}
        return planes, dict(zip(("Energy", "Enstrophy", "Palinstrophy", "Max_vorticity", "Scalar_integral"),
                                mes.tolist()))

    def vlasov_sample(self, n):
        """Vlasov sampled outputs on an n x n grid: dict of the four planes (Map_ChiX,
        Map_ChiY, Distribution_F, Stream_function_Psi) and the nine conservation values
        (sample_compute_and_write_vlasov, backward part)."""
        out = np.zeros(4 * n * n)
        mes = np.zeros(9)
        self.L.og_state_vlasov_sample(self.h, n, _dp(out), _dp(mes))
        names = ("Map_ChiX", "Map_ChiY", "Distribution_F", "Stream_function_Psi")
        planes = {k: out[i * n * n:(i + 1) * n * n].copy() for i, k in enumerate(names)}
        keys = ("Etot", "Ekin", "Epot", "Mass", "Momentum", "Emode1", "Emode2", "Emode3", "Emode4")
        return planes, dict(zip(keys, mes.tolist()))

    # forward map
    def chix_f(self):
        return self._arr(self.L.og_chix_f, 4 * self.grid(0).N)

    def chiy_f(self):
        return self._arr(self.L.og_chiy_f, 4 * self.grid(0).N)

    def forward_monitors(self):
        """(forward incompressibility error, invertibility error) of the last step"""
        a, b = C.c_double(), C.c_double()
        self.L.og_forward_monitors(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def set_forwarded_particles(self, i, pos):
        p = np.ascontiguousarray(pos, dtype=np.float64)
        if self.L.og_set_forwarded_particles(self.h, i, _dp(p)):
            raise ValueError("no forwarded particle set %d" % i)

    def forward_sample(self, n, bounds):
        """Forward map on an n x n frame (x planes, y planes) and the forwarded particle
        positions of every set (list of 2*num arrays, NaN outside the frame)."""
        xy = np.zeros(2 * n * n)
        nums = [p["num"] for p in self.cfg.get("forwarded", [])]
        parts = np.zeros(max(1, 2 * sum(nums)))
        b = np.ascontiguousarray(bounds[:4], dtype=np.float64)
        self.L.og_forward_sample(self.h, n, _dp(b), _dp(xy), _dp(parts))
        out, k = [], 0
        for m in nums:
            out.append(parts[k:k + 2 * m].copy())
            k += 2 * m
        return xy[0::2].copy(), xy[1::2].copy(), out

    def zoom(self, n, bounds, scalar_num):
        """compute_zoom planes on an n x n window (bounds = x_min, x_max, y_min, y_max):
        dict Map_ChiX, Map_ChiY, Scalar_Theta, Vorticity_W, Distribution, Stream_function_Psi."""
        out = np.zeros(6 * n * n)
        b = np.ascontiguousarray(bounds[:4], dtype=np.float64)
        self.L.og_state_zoom(self.h, n, _dp(b), scalar_num, _dp(out))
        names = ("Map_ChiX", "Map_ChiY", "Scalar_Theta", "Vorticity_W", "Distribution", "Stream_function_Psi")
        return {k: out[i * n * n:(i + 1) * n * n].copy() for i, k in enumerate(names)}

    def vlasov_mesure(self):
        """{Etot, Ekin, Epot, Mass, Momentum, Emode1..4} of the current state
        (Vlasov-Poisson conservation targets)."""
        out = np.zeros(9)
        self.L.og_vlasov_state_mesure(self.h, _dp(out))
        keys = ("Etot", "Ekin", "Epot", "Mass", "Momentum", "Emode1", "Emode2", "Emode3", "Emode4")
        return dict(zip(keys, out.tolist()))


def set_init_data(params=None, table=None):
    """initial_params (10 values) and the random table of the analytic initial conditions
    (1000 uniform(-1, 1) values then the 98 turbulence_gaussienne offsets: the product's
    "Init_random_table" field), shared by every oracle state of the process."""
    p = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
    t = None if table is None else np.ascontiguousarray(table, dtype=np.float64)
    if t is not None and t.size != 1098:
        raise ValueError("the initial-condition table has 1098 values")
    lib().og_set_init_data(None if p is None else _dp(p), None if t is None else _dp(t))


# ---------------------------------------------------------------- MapStack folder
def map_stack_files(o):
    """The files writeMapStack / writeParticlesState leave in the MapStack folder at
    the end of a run (src/ui/cmm-io.cu:611-657; src/simulation/cmm-euler2d.cu:1033-1051):
    every stacked sub-map (Map_ChiX_H_<i>, Map_ChiY_H_<i>, 4*Nc planar doubles), the
    active map (..._H_coarse) and Stream_function_Psi_H_psi_<l> for l = 1..L-1 -- each
    of them a copy of psi level 0, as the reference writes Psi.Dev_var for every l
    (src/ui/cmm-io.cu:631-633) -- the particle positions Particles_advected_pos_P<ii> and,
    for inertial sets, their velocities Particles_advected_vel_U<ii>."""
    files = {}
    sx, sy = o.map_stack()
    for i in range(sx.shape[0]):
        files["Map_ChiX_H_%d" % i] = sx[i]
        files["Map_ChiY_H_%d" % i] = sy[i]
    files["Map_ChiX_H_coarse"] = o.chix()
    files["Map_ChiY_H_coarse"] = o.chiy()
    p0 = o.psi(1)
    for l in range(1, o.cfg["lagrange_order"]):
        files["Stream_function_Psi_H_psi_%d" % l] = p0
    for i, p in enumerate(o.cfg.get("particles", [])):
        files["Particles_advected_pos_P%02d" % (i + 1)] = o.particles(i)
        if p["tau"] != 0:
            files["Particles_advected_vel_U%02d" % (i + 1)] = o.particle_velocity(i)
    return files


def read_map_stack_dir(path):
    """{name: float64 array} of the .data files of a MapStack folder."""
    out = {}
    for fn in sorted(os.listdir(path)):
        if fn.endswith(".data"):
            out[fn[:-len(".data")]] = np.fromfile(os.path.join(path, fn), dtype=np.float64)
    return out


# ---------------------------------------------------------------- kernel-level restatements
def make_grid(n, bounds=(0.0, 6.283185307179586, 0.0, 6.283185307179586)):
    g = OgGrid()
    L = lib()
    b = (C.c_double * 4)(*bounds)
    L.og_grid_fill(C.byref(g), int(n), int(n), b)
    return g


def _kernel_lib():
    L = lib()
    if not getattr(L, "_kernels_typed", False):
        dp = C.POINTER(C.c_double)
        gp = C.POINTER(OgGrid)
        L.og_grid_fill.argtypes = [gp, C.c_int, C.c_int, dp]
        L.og_advect_map.argtypes = [dp, dp, dp, dp, dp, gp, gp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                    dp, dp, dp, dp, dp, dp]
        L.og_map_update_coefficients.argtypes = [C.c_int, C.c_double, dp, dp, dp, dp]
        L.og_incompressibility_check.argtypes = [gp, gp, dp, dp]
        L.og_incompressibility_check.restype = C.c_double
        L.og_compose_sample.argtypes = [dp, dp, dp, C.c_int, gp, gp, C.c_int, dp, gp, dp]
        L.og_compose_sample_var.argtypes = [dp, dp, dp, C.c_int, gp, gp, C.c_int, C.c_int, dp, gp, dp]
        L.og_vlasov_potential.argtypes = [dp, dp, dp, gp, gp, gp, gp, C.c_int, dp]
        L.og_vlasov_potential.restype = C.c_int
        L.og_vlasov_mesure.argtypes = [dp, gp, dp, gp, dp]
        L.og_periodification.argtypes = [gp, dp]
        L.og_integral_v.argtypes = [dp, dp, C.c_int, C.c_int, C.c_double]
        L.og_apply_map_and_sample_from_hermite.argtypes = [dp, dp, dp, dp, gp, gp, gp, C.c_int, C.c_int]
        L.og_particle_advect.argtypes = [C.c_int, C.c_double, dp, dp, gp, C.c_int, C.c_int, dp]
        L.og_fft_d2z.argtypes = [gp, dp, dp]
        L.og_fft_z2d.argtypes = [gp, dp, dp]
        L.og_normalize_h.argtypes = [dp, gp]
        L.og_fft_grid_move.argtypes = [dp, dp, gp, gp]
        L.og_fft_cut_off_scale_h.argtypes = [dp, gp, C.c_double]
        L.og_fft_iLap_h.argtypes = [dp, dp, gp]
        L.og_fourier_hermite.argtypes = [gp, dp, dp]
        L.og_get_L_coefficient.argtypes = [dp, C.c_double, C.c_int, C.c_int, C.c_int]
        L.og_get_L_coefficient.restype = C.c_double
        L._kernels_typed = True
    return L


def advect_map(chix, chiy, psi_levels, gm, gp, dt, ep, ti, order, L1, L12):
    """og_advect_map on contiguous numpy inputs; psi_levels is a list of 4*Np arrays."""
    L = _kernel_lib()
    psi = np.ascontiguousarray(np.concatenate(psi_levels))
    outx = np.empty_like(chix)
    outy = np.empty_like(chiy)
    c = [np.zeros(12) for _ in range(4)]
    L.og_map_update_coefficients(order, ep, *[_dp(a) for a in c])
    l1 = np.array(list(L1) + [0] * 4, dtype=np.float64)
    l12 = np.array(list(L12) + [0] * 4, dtype=np.float64)
    L.og_advect_map(_dp(chix), _dp(chiy), _dp(outx), _dp(outy), _dp(psi), C.byref(gm), C.byref(gp), dt, ep, ti, order,
                    len(psi_levels), _dp(l1), _dp(l12), *[_dp(a) for a in c])
    return outx, outy


def incompressibility(gcheck, gm, chix, chiy):
    return _kernel_lib().og_incompressibility_check(C.byref(gcheck), C.byref(gm), _dp(chix), _dp(chiy))


def compose_sample(chix, chiy, stack, n, gm, gt, ic_num, discrete=None, gd=None, var_num=0):
    L = _kernel_lib()
    out = np.empty(gt.N, dtype=np.float64)
    st = np.ascontiguousarray(stack if stack is not None else np.zeros(1))
    L.og_compose_sample_var(_dp(chix), _dp(chiy), _dp(st), n, C.byref(gm), C.byref(gt), var_num, ic_num,
                            _dp(discrete) if discrete is not None else None, C.byref(gd) if gd is not None else None,
                            _dp(out))
    return out


def vlasov_potential(chix, chiy, f_fine, gm, gv, gf, gp, molly=0):
    """evaluate_potential_from_density_hermite on the CPU -> 4 Hermite planes of psi on gp."""
    L = _kernel_lib()
    out = np.empty(4 * gp.N)
    rc = L.og_vlasov_potential(_dp(chix), _dp(chiy), _dp(f_fine), C.byref(gm), C.byref(gv), C.byref(gf),
                               C.byref(gp), molly, _dp(out))
    if rc:
        raise ValueError("vort grid finer than psi grid, or psi grid not square")
    return out


def vlasov_mesure(f_coarse, gc, psi, gp):
    L = _kernel_lib()
    out = np.zeros(9)
    L.og_vlasov_mesure(_dp(np.ascontiguousarray(f_coarse)), C.byref(gc), _dp(np.ascontiguousarray(psi)),
                       C.byref(gp), _dp(out))
    return out


def periodification(gp):
    L = _kernel_lib()
    out = np.empty(gp.NY)
    L.og_periodification(C.byref(gp), _dp(out))
    return out


def sample_vort(chix, chiy, w_fine, gm, gout, gf, molly=0):
    L = _kernel_lib()
    out = np.empty(gout.N, dtype=np.float64)
    L.og_apply_map_and_sample_from_hermite(_dp(chix), _dp(chiy), _dp(out), _dp(w_fine), C.byref(gm), C.byref(gout),
                                           C.byref(gf), molly, 0)
    return out


def particle_advect(pos, psi_levels, g, dt, ti, Lp12):
    L = _kernel_lib()
    p = np.ascontiguousarray(pos, dtype=np.float64).copy()
    psi = np.ascontiguousarray(np.concatenate(psi_levels))
    lp = np.array(list(Lp12) + [0] * 4, dtype=np.float64)
    L.og_particle_advect(len(p) // 2, dt, _dp(p), _dp(psi), C.byref(g), ti, len(psi_levels), _dp(lp))
    return p


def poisson_hermite(vort, gv, gp, freq):
    """evaluate_stream_hermite's FFT part on the CPU: vort samples -> 4 Hermite planes."""
    L = _kernel_lib()
    cv = np.empty(2 * gv.Nfft)
    cp = np.empty(2 * max(gv.Nfft, gp.Nfft))
    v = np.ascontiguousarray(vort, dtype=np.float64)
    L.og_fft_d2z(C.byref(gv), _dp(v), _dp(cv))
    L.og_normalize_h(_dp(cv), C.byref(gv))
    if gv.NX != gp.NX:
        L.og_fft_grid_move(_dp(cv), _dp(cp), C.byref(gp), C.byref(gv))
    else:
        cp[: 2 * gv.Nfft] = cv
    L.og_fft_cut_off_scale_h(_dp(cp), C.byref(gp), freq)
    c2 = np.empty_like(cp)
    L.og_fft_iLap_h(_dp(cp), _dp(c2), C.byref(gp))
    out = np.empty(4 * gp.N)
    L.og_fourier_hermite(C.byref(gp), _dp(c2), _dp(out))
    return out


def lagrange(t, t_next, loop_ctr, i_point, l_order):
    tt = np.ascontiguousarray(t, dtype=np.float64)
    return _kernel_lib().og_get_L_coefficient(_dp(tt), t_next, loop_ctr, i_point, l_order)


# ---------------------------------------------------------------- learned psi upsampler
def _learned_lib():
    L = lib()
    if not getattr(L, "_learned", False):
        dp = C.POINTER(C.c_double)
        fp = C.POINTER(C.c_float)
        L.og_bf16_round.argtypes = [C.c_double]
        L.og_bf16_round.restype = C.c_double
        L.og_conv3x3.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int, dp, dp, C.c_int, dp, dp, C.c_int, dp]
        L.og_conv3x3_t.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int, dp, C.c_int, dp, dp, dp]
        L.og_conv3x3_dw.argtypes = [dp, dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, dp, dp]
        L.og_upsampler_loss_grad.argtypes = [dp, C.c_int, C.c_int, dp, C.c_double, fp, fp, C.c_int, C.c_int, C.c_int,
                                             C.c_int, C.c_int, dp]
        L.og_upsampler_loss_grad.restype = C.c_double
        L.og_upsampler_loss_grad_sq.argtypes = [dp, C.c_int, C.c_int, dp, C.c_double, fp, fp, C.c_int, C.c_int,
                                                C.c_int, C.c_int, C.c_int, dp, dp]
        L.og_upsampler_loss_grad_sq.restype = C.c_double
        L._learned = True
    return L


def bf16_round(a):
    """Round to the nearest BF16 value (ties to even), as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    f = (f + 0x7FFF + ((f >> 16) & 1)) & 0xFFFF0000
    return f.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(a):
    """BF16 bit patterns (uint16) of values already representable in BF16."""
    return (np.ascontiguousarray(a, dtype=np.float32).view(np.uint32) >> 16).astype(np.uint16)


def _opt(a):
    """A float64 array already kept alive by the caller, or None (NULL)."""
    return None if a is None else _dp(a)


def conv3x3(x, w, bias=None, mask=None, res=None, relu=False):
    """x[B, H, W, cin], w[9, cin, cout] -> out[B, H, W, cout] (periodic 3x3, FP64)."""
    L = _learned_lib()
    B, H, W, cin = x.shape
    cout = w.shape[2]
    x = np.ascontiguousarray(x, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    bias, mask, res = (None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in (bias, mask, res))
    out = np.empty((B, H, W, cout))
    L.og_conv3x3(_dp(x), B, H, W, cin, _dp(w), _opt(bias), cout, _opt(mask), _opt(res), 1 if relu else 0, _dp(out))
    return out


def conv3x3_input_grad(dy, w, mask=None, res=None):
    """dy[B, H, W, cout], w[9, cin, cout] -> dx[B, H, W, cin]."""
    L = _learned_lib()
    B, H, W, cout = dy.shape
    cin = w.shape[1]
    dy = np.ascontiguousarray(dy, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    mask, res = (None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in (mask, res))
    dx = np.empty((B, H, W, cin))
    L.og_conv3x3_t(_dp(dy), B, H, W, cin, _dp(w), cout, _opt(mask), _opt(res), _dp(dx))
    return dx


def conv3x3_weight_grad(x, dy):
    """x[B, H, W, cin], dy[B, H, W, cout] -> (dw[9, cin, cout], db[cout])."""
    L = _learned_lib()
    B, H, W, cin = x.shape
    cout = dy.shape[3]
    x = np.ascontiguousarray(x, dtype=np.float64)
    dy = np.ascontiguousarray(dy, dtype=np.float64)
    dw = np.empty((9, cin, cout))
    db = np.empty(cout)
    L.og_conv3x3_dw(_dp(x), _dp(dy), B, H, W, cin, cout, _dp(dw), _dp(db))
    return dw, db


def upsampler_loss_grad(params, blocks, channels, s_in, s_out, inputs, targets, emulate_bf16=True, cut=0,
                        dy_sq=False):
    """Loss and gradient of the upsampler: inputs[B, 7, h, w], targets[B, 2h, 2w] (float32);
    cut > 0: the psi-space spectral loss (w = 1/|k|^4 on 0 < |k| <= cut).  dy_sq: also return,
    at each layer's bias slots of the parameter layout, the sum over pixels of the squared
    output gradient of that channel (the scale of the rounding noise in its bias gradient)."""
    L = _learned_lib()
    params = np.ascontiguousarray(params, dtype=np.float64)
    s_in = np.ascontiguousarray(s_in, dtype=np.float64)
    inputs = np.ascontiguousarray(inputs, dtype=np.float32)
    targets = np.ascontiguousarray(targets, dtype=np.float32)
    B, _, h, w = inputs.shape
    grad = np.zeros_like(params)
    fp = C.POINTER(C.c_float)
    sq = np.zeros_like(params)
    loss = L.og_upsampler_loss_grad_sq(_dp(params), blocks, channels, _dp(s_in), float(s_out),
                                       inputs.ctypes.data_as(fp), targets.ctypes.data_as(fp), B, h, w,
                                       1 if emulate_bf16 else 0, int(cut), _dp(grad), _dp(sq))
    return (loss, grad, sq) if dy_sq else (loss, grad)


def upsampler_param_count(blocks, channels):
    n = 9 * 16 * channels + channels
    n += blocks * 2 * (9 * channels * channels + channels)
    n += 9 * channels * 16 + 16
    return n
