"""Test-side restatement of the reference's settings and loop control.

Used by the parity tests to configure the CPU oracle exactly as the reference
binary would be configured by a param file, and to reproduce the reference's
save instants.  The product has its own C++ implementation of the same logic
(cmm-turbulence_gb300/csrc/settings.cpp); tests/test_settings.py checks the two
agree.

Restates:
  presets            src/ui/settings.cu:18-327
  COMMAND=VALUE      src/ui/settings.cu:347-436
  records {k=v,...}  src/ui/settings.cu:556-823
  param file         src/ui/cmm-param.cu:149-229
  dt / lagrange      src/simulation/cmm-euler2d.cu:62-78
  next time step     src/simulation/cmm-simulation-host.cu:1307-1374
  save instants      src/ui/cmm-io.cu:300-317, cmm-simulation-host.cu:619-636
  loop               src/simulation/cmm-euler2d.cu:750-960
  Vlasov driver      src/simulation/cmm-vlasov1d.cu:62-105 (bounds x pi, dt, iter_max)
"""
import math

TWO_PI = 6.283185307179586476925286766559005768394338798750211641949889184615632812572417997256069650684234136
PI = TWO_PI / 2
T_MAX = 10000.0

IC_EULER = ["4_nodes", "quadropole", "one_vortex", "two_votices", "three_vortices", "single_shear_layer",
            "tanh_shear_layer", "turbulence_gaussienne", "gaussian_blobs", "shielded_vortex", "two_cosine",
            "vortex_sheets"]
IC_VLASOV = ["landau_damping", "two_stream", "nonlin_landau_damping"]
TI_MAP = {"EulerExp": (10, 1), "RK1": (10, 1), "Heun": (21, 2), "RK2": (21, 2), "AB2": (20, 2),
          "RK3": (30, 3), "RK4": (40, 4), "RK3Mod": (31, 3), "RK4Mod": (41, 4)}
TI_PART = {"EulerExp": 10, "RK1": 10, "Heun": 20, "RK2": 20, "RK3": 30, "RK4": 40, "RK3Mod": 31, "RK4Mod": 41}


def _bool(v):
    return v in ("true", "True", "1")


def _str_t(x):
    # str_t of settings.h:484 -- ostringstream with default precision 6... but
    # only used to build preset record strings; parse back with float()
    return repr(float(x))


def _record(text):
    """Parse "{k=v,k=v}" (settings.cu:556-579)."""
    out = {}
    if len(text) >= 2 and ((text[0] == "{" and text[-1] == "}") or (text[0] == '"' and text[-1] == '"')):
        for part in text[1:-1].split(","):
            if "=" in part:
                k, v = part.split("=", 1)
                out[k] = v
    return out


class SaveRec:
    def __init__(self, text, kind):
        self.is_instant = False
        self.time_start = 0.0
        self.time_end = 0.0
        self.time_step = 0.0
        self.var = ""
        self.conv = False
        self.grid = 0
        self.pos_x = self.pos_y = self.width_x = self.width_y = 0.0
        self.rep = 0
        self.rep_fac = 0.0
        for k, v in _record(text).items():
            if k == "is_instant": self.is_instant = _bool(v)
            elif k == "time_start": self.time_start = float(v)
            elif k == "time_end": self.time_end = float(v)
            elif k == "time_step": self.time_step = float(v)
            elif k == "var": self.var = v
            elif k == "conv" and kind == "comp": self.conv = _bool(v)
            elif k == "grid" and kind != "comp": self.grid = int(v)
            elif kind == "zoom" and k in ("pos_x", "pos_y", "width_x", "width_y", "rep_fac"): setattr(self, k, float(v))
            elif kind == "zoom" and k == "rep": self.rep = int(float(v))


class PartRec:
    def __init__(self, text):
        self.num = 0
        self.tau = 0.0
        self.seed = 0
        self.time_integration = ""
        self.time_integration_num = 0
        self.init_name = ""
        self.init_num = 0
        self.init_time = 0.0
        self.init_vel = False
        self.init_param = [0.0, 0.0, 0.0, 0.0]
        for k, v in _record(text).items():
            if k == "num": self.num = int(v)
            elif k == "tau": self.tau = float(v)
            elif k == "seed": self.seed = int(v)
            elif k == "time_integration":
                self.time_integration = v
                self.time_integration_num = TI_PART.get(v, -1)
            elif k == "init_name":
                self.init_name = v
                self.init_num = {"uniform": 0, "normal": 1, "gaussian": 1, "circular_ring": 2,
                                 "uniform_grid": 3, "sine_sheets": 4}.get(v, -1)
            elif k == "init_time": self.init_time = float(v)
            elif k == "init_vel": self.init_vel = _bool(v)
            elif k.startswith("init_param_"): self.init_param[int(k[-1]) - 1] = float(v)


class Settings:
    """Settings after presets, param file and CLI (src/main2d.cpp:66-89)."""

    def __init__(self):
        self.workspace = "./"
        self.simulation_type = "cmm_euler_2d"
        self.sim_name = "debug"
        self.grid_coarse, self.grid_fine, self.grid_psi, self.grid_vort = 512, 2048, 1024, 2048
        self.initial_condition = "4_nodes"
        self.initial_params = [0.0] * 10
        self.initial_discrete = False
        self.initial_discrete_grid = 2048
        self.initial_discrete_location = ""
        self.verbose = 3
        self.domain_bounds = [0, TWO_PI, 0, TWO_PI, 0, 0]
        self.final_time = 3.0
        self.set_dt_by_steps = True
        self.factor_dt_by_grid = 1.0
        self.steps_per_sec = 20
        self.save_comp = [SaveRec(s, "comp") for s in (
            "{is_instant=1,time_start=0,var=W-U,conv=1}",
            "{is_instant=1,time_start=%s,var=W-U,conv=1}" % T_MAX,
            "{is_instant=0,time_start=0,time_end=%s,time_step=0.5,var ,conv=1}" % T_MAX,
            "{is_instant=0,time_start=0,time_end=%s,time_step=0.5,var=PartA_01-PartA_02-PartA_03-PartA_04,conv=0}" % T_MAX)]
        self.incomp_threshold = 1e-5
        self.map_epsilon = 1e-3
        self.skip_remapping = False
        self.mem_RAM_CPU_remaps = 9000
        self.save_map_stack = True
        self.restart_time = 0.0
        self.lagrange_order = 0
        self.time_integration = ""
        self.time_integration_num = 0
        self.set_time_integration("RK3")
        self.lagrange_override = -1
        self.lagrange_init_higher_order = True
        self.map_update_order = "4th"
        self.molly_stencil = 0
        self.freq_cut_psi = 512 / 4.0
        self.save_sample = [SaveRec("{is_instant=0,time_start=0,time_end=%s,time_step=0.5,var=W,grid=1024}" % T_MAX, "sample")]
        self.save_zoom = []
        self.forward_map = False
        self.particles_forwarded = []
        pi_s = ",init_param_1=%r,init_param_2=%r,init_param_3=%r,init_param_4=%r}" % (PI, PI, 2 * PI, 2 * PI)
        self.particles_advected = [
            PartRec("{num=100000,tau=0,seed=0,time_integration=RK3,init_name=sine_sheets,init_time=0,init_vel=0" + pi_s),
            PartRec("{num=100000,tau=0.1,seed=0,time_integration=RK3,init_name=uniform,init_time=0,init_vel=0" + pi_s)]
        self.particles_steps = -1
        self.scalar_name = "rectangle"

    # settings.h:386-398 -- raises the Lagrange order, never lowers it
    def set_time_integration(self, v):
        self.time_integration = v
        num, lo = TI_MAP.get(v, (-1, 0))
        self.time_integration_num = num
        if num != -1 and self.lagrange_order < lo:
            self.lagrange_order = lo

    @property
    def map_update_order_num(self):
        return {"2nd": 0, "4th": 1, "6th": 2}.get(self.map_update_order, -1)

    @property
    def initial_condition_num(self):
        table = IC_VLASOV if self.simulation_type == "cmm_vlasov_poisson_1d" else IC_EULER
        return table.index(self.initial_condition) if self.initial_condition in table else -1

    @property
    def scalar_num(self):
        # settings.h:322-330
        return {"rectangle": 0, "gaussian": 1, "circular_ring": 2}.get(self.scalar_name, -1)

    @property
    def simulation_type_num(self):
        return 2 if self.simulation_type == "cmm_vlasov_poisson_1d" else 0

    def set_variable(self, line, delim):
        """settings.cu:347-436; returns the record-count code 0..5."""
        pos = line.find(delim)
        if pos < 0:
            return 0
        k, v = line[:pos], line[pos + len(delim):]
        ints = {"grid_coarse", "grid_fine", "grid_psi", "grid_vort", "steps_per_sec", "mem_RAM_CPU_remaps",
                "verbose", "initial_discrete_grid", "lagrange_override", "molly_stencil", "particles_steps"}
        floats = {"final_time", "factor_dt_by_grid", "restart_time", "incomp_threshold", "map_epsilon", "freq_cut_psi"}
        bools = {"set_dt_by_steps", "save_map_stack", "initial_discrete", "lagrange_init_higher_order",
                 "skip_remapping", "forward_map"}
        strs = {"workspace", "simulation_type", "sim_name", "initial_condition", "initial_discrete_location",
                "map_update_order", "scalar_name"}
        if k in ints: setattr(self, k, int(v))
        elif k in floats: setattr(self, k, float(v))
        elif k in bools: setattr(self, k, _bool(v))
        elif k in strs: setattr(self, k, v)
        elif k == "domain_bounds":
            b = [0.0] * 6
            if len(v) >= 2 and v[0] in "{\"" and v[-1] in "}\"":
                for i, x in enumerate(v[1:-1].split(",")[:6]):
                    b[i] = float(x)
            self.domain_bounds = b
        elif k == "initial_params":
            if len(v) >= 2 and v[0] in "{\"" and v[-1] in "}\"":
                for i, x in enumerate(v[1:-1].split(",")[:10]):
                    self.initial_params[i] = float(x)
        elif k == "time_integration": self.set_time_integration(v)
        elif k == "save_computational_num":
            self.save_comp = [SaveRec("", "comp") for _ in range(int(v))]
            return 1
        elif k == "save_sample_num":
            self.save_sample = [SaveRec("", "sample") for _ in range(int(v))]
            return 2
        elif k == "save_zoom_num":
            self.save_zoom = [SaveRec("", "zoom") for _ in range(int(v))]
            return 3
        elif k == "particles_advected_num":
            self.particles_advected = [PartRec("") for _ in range(int(v))]
            return 4
        elif k == "particles_forwarded_num":
            self.particles_forwarded = [PartRec("") for _ in range(int(v))]
            return 5
        return 0

    def load_param_text(self, text):
        """cmm-param.cu:149-229"""
        lines = text.split("\n")
        if len(lines) < 2 or lines[0] != "CMM Parameter file":
            return False
        d = "\t=\t"
        if not lines[1].startswith("param_version" + d):
            return False
        i = 3
        lists = {1: ("save_comp", "comp"), 2: ("save_sample", "sample"), 3: ("save_zoom", "zoom")}
        while i < len(lines):
            code = self.set_variable(lines[i], d)
            i += 1
            if code in lists:
                attr, kind = lists[code]
                for j in range(len(getattr(self, attr))):
                    line = lines[i] if i < len(lines) else ""
                    i += 1
                    p = line.find(d)
                    if p >= 0:
                        getattr(self, attr)[j] = SaveRec(line[p + len(d):], kind)
            elif code in (4, 5):
                attr = "particles_advected" if code == 4 else "particles_forwarded"
                for j in range(len(getattr(self, attr))):
                    line = lines[i] if i < len(lines) else ""
                    i += 1
                    p = line.find(d)
                    if p >= 0:
                        getattr(self, attr)[j] = PartRec(line[p + len(d):])
        return True

    # ---- derived quantities of cmm-euler2d.cu:62-83 ----
    def finalize(self):
        if self.simulation_type == "cmm_vlasov_poisson_1d":
            # cmm-vlasov1d.cu:72: the Vlasov driver multiplies the bounds by pi
            self.domain_bounds = [b * PI if i < 4 else b for i, b in enumerate(self.domain_bounds)]
        if self.set_dt_by_steps:
            self.dt = 1.0 / self.steps_per_sec
        else:
            self.dt = 1.0 / self.grid_coarse / self.factor_dt_by_grid
        for p in self.particles_advected:
            need = {20: 2, 30: 3, 31: 3, 40: 4, 41: 4}.get(p.time_integration_num, 0)
            if self.lagrange_order < need:
                self.lagrange_order = need
        if self.lagrange_override != -1:
            self.lagrange_order = self.lagrange_override
        self.iter_max = int(1.05 * math.ceil((self.final_time - self.restart_time) / self.dt))
        map_size = 8 * self.grid_coarse * self.grid_coarse * 8 / 1e6
        self.cpu_map_num = int(float(self.mem_RAM_CPU_remaps) / map_size)
        if self.forward_map:
            self.cpu_map_num = int(self.cpu_map_num / 2.0)
        return self

    def oracle_config(self):
        return dict(grid_coarse=self.grid_coarse, grid_fine=self.grid_fine, grid_psi=self.grid_psi,
                    grid_vort=self.grid_vort, bounds=list(self.domain_bounds[:4]), dt=self.dt,
                    time_integration_num=self.time_integration_num, lagrange_order=self.lagrange_order,
                    lagrange_init_higher_order=self.lagrange_init_higher_order,
                    map_update_order_num=self.map_update_order_num, map_epsilon=self.map_epsilon,
                    incomp_threshold=self.incomp_threshold, skip_remapping=self.skip_remapping,
                    molly_stencil=self.molly_stencil, freq_cut_psi=self.freq_cut_psi,
                    initial_condition_num=self.initial_condition_num,
                    initial_discrete=self.initial_discrete, initial_discrete_grid=self.initial_discrete_grid,
                    max_maps=self.cpu_map_num, simulation_type_num=self.simulation_type_num,
                    initial_params=list(self.initial_params), forward_map=int(self.forward_map),
                    forwarded=[dict(num=p.num, init_time=p.init_time) for p in self.particles_forwarded],
                    particles=[dict(num=p.num, tau=p.tau, time_integration_num=p.time_integration_num,
                                    init_time=p.init_time, init_vel=p.init_vel) for p in self.particles_advected])


def settings_from_param_text(text, cli=()):
    s = Settings()
    s.load_param_text(text)
    for c in cli:
        s.set_variable(c, "=")
    return s.finalize()


def compute_next_timestep(s, t, dt):
    """cmm-simulation-host.cu:1307-1374"""
    dt_now = dt
    dt_e = dt * 1e-5
    for p in s.particles_advected + s.particles_forwarded:
        if t + dt_e - p.init_time < 0 and t + dt_e + dt - p.init_time > 0:
            dt_now = min(dt_now, p.init_time - t)
    for recs in (s.save_comp, s.save_sample, s.save_zoom):
        for r in recs:
            if r.is_instant and t + dt_e - r.time_start < 0 and t + dt_e + dt - r.time_start > 0:
                dt_now = min(dt_now, r.time_start - t)
            if not r.is_instant:
                a = math.fmod(t + dt_e - r.time_start, r.time_step) if r.time_step else float("nan")
                b = math.fmod(t + dt + dt_e - r.time_start, r.time_step) if r.time_step else float("nan")
                if (a > b or (a < 0 and b > 0)) and t + dt + dt_e >= r.time_start and t - dt_e <= r.time_end:
                    dt_now = min(dt_now, r.time_step - math.fmod(t, r.time_step))
    return dt_now


def save_instant(recs, t_now, dt_now, dt, need_conv=False):
    """True when any record fires at t_now (cmm-io.cu:300-317 / cmm-simulation-host.cu:619-636)."""
    fired = False
    for r in recs:
        if need_conv and not r.conv:
            continue
        if r.is_instant and t_now - r.time_start + dt * 1e-5 < dt_now and t_now - r.time_start + dt * 1e-5 >= 0:
            fired = True
        if not r.is_instant:
            m = math.fmod(t_now - r.time_start + dt * 1e-5, r.time_step) if r.time_step else float("nan")
            if (m < dt_now and t_now + dt * 1e-5 >= r.time_start and t_now - dt * 1e-5 <= r.time_end) \
                    or t_now == r.time_end:
                fired = True
    return fired


def run_reference_loop(s, stepper, on_save, on_step=None):
    """Drive `stepper` (an object with init/step/time) through the loop of
    cmm-euler2d.cu:687-1060.  `on_save(t_now, dt_now)` fires at every
    save_functions call; `on_step(loop_ctr, t, e_inc, gap, maps)` after each step."""
    dt = s.dt
    L = s.lagrange_order
    stepper.init()
    on_save(s.restart_time, dt)
    t_vec = [s.restart_time - (L - 1 - i) * dt for i in range(L)]
    loop_ctr = 0
    cont = True
    while s.final_time - t_vec[-1] > dt * 1e-5 and loop_ctr < s.iter_max and cont:
        t = t_vec[-1]
        dt_now = compute_next_timestep(s, t, dt)
        if t + dt_now > s.final_time:
            dt_now = s.final_time - t
        rc, e_inc, remapped, gap, maps = stepper.step(dt_now)
        if rc == 2:
            raise RuntimeError("incompressibility error out of range: Vlasov run aborted (cmm-vlasov1d.cu:838-840)")
        if rc == 1:
            cont = False
        t_vec.append(t + dt_now)
        on_save(t + dt_now, dt_now)
        if on_step:
            on_step(loop_ctr, t + dt_now, e_inc, gap, maps)
        loop_ctr += 1
    on_save(T_MAX, dt)
    return loop_ctr
