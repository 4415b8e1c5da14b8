"""Benchmark of the CMM time step on one GB300 (and the CPU reference arm).

Workload (the metric's configuration): 2D Euler decaying turbulence, map grid
512^2, fine / vorticity grid 2048^2, psi grid 1024^2, dt = 1/256, random-phase
initial vorticity with energy spectrum E(k) ~ k^4 exp(-(k/8)^2) normalised to
unit enstrophy (Z = 1/2 hx hy sum w^2), map stack up to 200 sub-maps
(mem_RAM_CPU_remaps=3356), 10^6 RK3 tracer particles.  One "step" is one
iteration of the reference loop (map advection, incompressibility check,
remap when needed, psi solve, coarse vorticity, particles, monitors).

  python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is steps/s with the state resident in HBM,
timed with CUDA events on the library's stream; `e2e` is the same metric
through the C-ABI with the initial vorticity uploaded from pinned host memory,
the initialisation, and every step's monitoring record plus the final psi
read back to the host inside the timed region.  `--impl reference` times the
CPU implementation of the same step (the FP64 OpenMP oracle restating the
reference algorithm) on the host cores.
"""
import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TWO_PI = 6.283185307179586
WORKLOAD = dict(grid_coarse=512, grid_fine=2048, grid_psi=1024, grid_vort=2048, steps_per_sec=256,
                mem_RAM_CPU_remaps=3356, particles=1000000, seed=0, k0=8.0)
METRIC = "steps/s (512² map, 2048² fine): chosen vs plain FP64 at ≤1e-4 enstrophy err"


def initial_vorticity(n=2048, seed=0, k0=8.0):
    """Random-phase field with E(k) ~ k^4 exp(-(k/k0)^2), unit enstrophy."""
    rng = np.random.default_rng(seed)
    kx = np.fft.rfftfreq(n, 1.0 / n)
    ky = np.fft.fftfreq(n, 1.0 / n)
    k = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    ek = k ** 4 * np.exp(-(k / k0) ** 2)
    amp = np.zeros_like(k)
    nz = k > 0
    amp[nz] = np.sqrt(k[nz] ** 2 * ek[nz] / (2 * np.pi * k[nz]))   # |w_k|^2 ~ k^2 E(k) / (2 pi k)
    phase = rng.uniform(0.0, 2 * np.pi, size=k.shape)
    w = np.fft.irfft2(amp * np.exp(1j * phase), s=(n, n))
    h = TWO_PI / n
    z = 0.5 * h * h * np.sum(w * w)
    return np.ascontiguousarray(w / np.sqrt(z))


def sim_args(workspace, precision="fp64", particles=WORKLOAD["particles"]):
    w = WORKLOAD
    return ["workspace=%s/" % workspace, "sim_name=bench", "simulation_type=cmm_euler_2d",
            "grid_coarse=%d" % w["grid_coarse"], "grid_fine=%d" % w["grid_fine"], "grid_psi=%d" % w["grid_psi"],
            "grid_vort=%d" % w["grid_vort"], "set_dt_by_steps=1", "steps_per_sec=%d" % w["steps_per_sec"],
            "final_time=10", "initial_condition=4_nodes", "initial_discrete=1",
            "initial_discrete_grid=%d" % w["grid_fine"], "time_integration=RK3", "map_update_order=4th",
            "map_epsilon=0.001", "incomp_threshold=0.0001", "skip_remapping=0", "molly_stencil=0",
            "freq_cut_psi=128", "lagrange_init_higher_order=1", "mem_RAM_CPU_remaps=%d" % w["mem_RAM_CPU_remaps"],
            "save_computational_num=0", "save_sample_num=0", "save_zoom_num=0", "forward_map=0", "verbose=0",
            "save_map_stack=0", "precision=%s" % precision, "particles_advected_num=1"], \
           ["{num=%d,tau=0,seed=0,time_integration=RK3,init_name=uniform,init_time=0,init_vel=0,"
            "init_param_1=3.141592653589793,init_param_2=3.141592653589793,init_param_3=6.283185307179586,"
            "init_param_4=6.283185307179586}" % particles]


def write_param_file(path, args, records):
    """The reference's param-file format, so the record list can follow particles_advected_num."""
    lines = ["CMM Parameter file", "param_version\t=\t3", ""]
    for a in args:
        k, v = a.split("=", 1)
        lines.append("%s\t=\t%s" % (k, v))
    for r in records:
        lines.append("particles_advected\t=\t%s" % r)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                      "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.splitlines()[0].split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            self._t = threading.Thread(target=self._run, daemon=True)
            self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = sorted(float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit())
        mx = max(float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 5 + i and s[5 + i] == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


# ---------------------------------------------------------------- roofline bookkeeping
def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


FP64_PEAK_TFLOPS = 1.10   # GB300 FP64 rate: `python bench.py --fp64-peak` (cuBLAS DGEMM), profiles/fp64_peak.md

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the roofline kernel,
# from one ncu capture of the same kernel on this workload; the file named beside each figure
# holds the command and the raw numbers
NCU_TRAFFIC = {("mixed", "advect"): (58.74e6 + 1.05e6, "profiles/mixed_step_kernels_c2.md"),
               ("fp64", "advect"): (127.4e6, "profiles/k_advect_fp64_c2.md")}


def measure_fp64_peak():
    """FP64 throughput of a cuBLAS DGEMM (torch.matmul, float64, 8192^3,
    2 N^3 flops, best of 5 after 2 warm-up runs, CUDA events)."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    best = None
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    tflops = 2.0 * n ** 3 / (best / 1000.0) / 1e12
    print(json.dumps({"fp64_dgemm_tflops": tflops, "n": n, "best_ms": best, "how": "cuBLAS DGEMM via torch.matmul"}))


CPU_SAMPLE_STEPS = 60   # ~10 s of the CPU restatement on 16 host cores (~6 steps/s)


def cpu_oracle_steps(n_steps, ic, threads, particles=100000):
    """Time n_steps of the CPU oracle on the C2 workload (after its initialisation)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle as O
    w = WORKLOAD
    cfg = dict(grid_coarse=w["grid_coarse"], grid_fine=w["grid_fine"], grid_psi=w["grid_psi"],
               grid_vort=w["grid_vort"], bounds=[0, TWO_PI, 0, TWO_PI], dt=1.0 / w["steps_per_sec"],
               time_integration_num=30, lagrange_order=3, lagrange_init_higher_order=1, map_update_order_num=1,
               map_epsilon=1e-3, incomp_threshold=1e-4, skip_remapping=0, molly_stencil=0, freq_cut_psi=128.0,
               initial_condition_num=0, initial_discrete=1, initial_discrete_grid=w["grid_fine"],
               max_maps=200, particles=[dict(num=particles, tau=0.0, time_integration_num=30, init_time=0.0)])
    o = O.EulerOracle(cfg)
    o.set_discrete_initial(ic)
    rng = np.random.default_rng(0)
    o.set_particles(0, rng.uniform(0, TWO_PI, 2 * particles))
    o.init()
    t0 = time.perf_counter()
    for _ in range(n_steps):
        o.step(cfg["dt"])
    dt = time.perf_counter() - t0
    o.close()
    return n_steps / dt, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ic = initial_vorticity(WORKLOAD["grid_fine"], WORKLOAD["seed"], WORKLOAD["k0"])
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    # a bounded sample: at most CPU_SAMPLE_STEPS full steps of the workload (the requested
    # warm-up + steps when fewer), all timed; the figure is steps per second of that sample
    n = max(1, min(args.steps + args.warmup, CPU_SAMPLE_STEPS))
    sps, secs = cpu_oracle_steps(n, ic, threads, particles=WORKLOAD["particles"])
    line = {"impl": "reference", "metric": METRIC, "value": sps, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / sps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "euler2d-turbulence coarse512 fine2048 psi1024 dt1/256 1e6 tracers",
                       "form": "plain FP64 (CPU restatement of the reference algorithm)"},
            "cpu_baseline": {"value": sps, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": "%d full steps of the workload after the Lagrange initialisation, %.1f s"
                                       % (n, secs)},
            "e2e": {"value": sps, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def measure_form(m, torch, pf, ic, precision, args, world, clocks=None, profile=True):
    """W warm-up steps on a throw-away instance, then a fresh simulation of the
    workload in `precision`: its first K steps from t = 0 (with every remap
    they trigger; K = 2560 is the whole T = 10 run) timed with CUDA events on
    the library stream, then (optionally) a few more steps profiled phase by
    phase."""
    stream = torch.cuda.Stream()
    over = ["param_file=" + pf, "precision=" + precision,
            "final_time=%r" % ((args.steps + 32) / WORKLOAD["steps_per_sec"])]
    if args.warmup > 0:
        warm = m.Simulation(over, stream=stream.cuda_stream)
        warm.set_initial_discrete(ic)
        warm.init()
        for _ in range(args.warmup):
            warm.step(1)
        warm.close()
    sim = m.Simulation(over, stream=stream.cuda_stream)
    sim.set_initial_discrete(ic)
    sim.init()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    l0, maps0 = sim.scalar("kernel_launches"), sim.scalar("map_counter")
    ctx = clocks if clocks is not None else ClockSampler()
    with ctx:
        e0.record(stream)
        sim.step(args.steps)          # one C-ABI call: the library's own loop runs the K steps
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
        ms = float(t.item())
    out = {"ms": ms, "value": world * args.steps / (ms / 1000.0), "launches": int(sim.scalar("kernel_launches") - l0),
           "remaps": int(sim.scalar("map_counter") - maps0), "time": sim.scalar("time"),
           "enstrophy": sim.scalar("enstrophy"), "energy": sim.scalar("energy"),
           "palinstrophy": sim.scalar("palinstrophy"), "maps": int(sim.scalar("map_counter"))}
    if profile:
        sim.set_profiling(True)
        for _ in range(max(3, min(args.steps, 20))):
            sim.step(1)
        out["phases"] = {ph: {"ms_total": sim.scalar("prof_%s_ms" % ph), "launches": int(sim.scalar("prof_%s_count" % ph))}
                         for ph in ("advect", "incomp", "remap", "psi", "coarse", "particles", "save")}
    sim.close()
    return out


def full_run(m, torch, pf, ic, precision, every=64, final_time=10.0, ups=None, exact_every=8, tol=1e-4):
    """Run the workload to its final time (T = 10, 2560 steps with every remap)
    and record (t, enstrophy, energy, maps) every `every` steps (0.25 time units);
    with `ups` the learned psi form (exact evaluation every exact_every steps)."""
    stream = torch.cuda.Stream()
    sim = m.Simulation(["param_file=" + pf, "precision=" + precision, "final_time=%g" % final_time],
                       stream=stream.cuda_stream)
    sim.set_initial_discrete(ic)
    sim.init()
    if ups is not None:
        sim.attach_upsampler(ups, every=exact_every, tol=tol)
    rec = [(sim.scalar("time"), sim.scalar("enstrophy"), sim.scalar("energy"), 0)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n = 0
    steps_only = 0.0
    while True:
        ts = time.perf_counter()
        rc = sim.step(1)
        if rc == 1:
            break
        n += 1
        if n % every == 0:
            torch.cuda.synchronize()
            steps_only += time.perf_counter() - ts
            rec.append((sim.scalar("time"), sim.scalar("enstrophy"), sim.scalar("energy"), int(sim.scalar("map_counter"))))
        else:
            steps_only += time.perf_counter() - ts
        if rc == m.CMM_ERR_SATURATED:
            break
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    maps = int(sim.scalar("map_counter"))
    out = {"steps": n, "wall_s": wall, "steps_per_s": n / wall, "maps": maps, "series": rec}
    if ups is not None:
        out.update({k: sim.scalar(k) for k in ("learned_steps", "cheap_steps", "exact_steps", "learned_checks",
                                               "learned_cheaper", "learned_failures", "learned_max_err")})
    sim.close()
    return out


VLASOV = dict(grid_coarse=256, grid_fine=1024, grid_vort=1024, grid_psi=1024, steps_per_sec=32, final_time=40.0,
              bounds="{0,4,-2,2}", incomp_threshold=1e-4)


def vlasov_initial(n):
    """f0 = (1 + 0.01 cos(x/2)) v^2 exp(-v^2/2) / sqrt(2 pi) on the n x n nodes of
    x in [0, 4 pi), v in [-2 pi, 2 pi) (row-major, v the row index)."""
    x = 4 * np.pi / n * np.arange(n)
    v = -2 * np.pi + 4 * np.pi / n * np.arange(n)
    return np.ascontiguousarray((1 + 0.01 * np.cos(0.5 * x))[None, :] * (v * v * np.exp(-v * v / 2)
                                                                        / np.sqrt(2 * np.pi))[:, None])


def run_vlasov(args):
    """The Vlasov-Poisson configuration in both forms over the whole run:
    steps/s and the FP64 diagnostics (mass, L2 of f, energies) of the mixed
    form against plain FP64."""
    import __graft_entry__ as ge
    ge.build()
    m = ge.package()
    import torch
    w = VLASOV
    work = tempfile.mkdtemp(prefix="cmm_vlasov_")
    f0 = vlasov_initial(w["grid_fine"])
    final = args.vlasov_final
    out = {"validation": "Vlasov-Poisson, mixed vs plain FP64 over the whole run", "final_time": final,
           "workload": "vlasov1d1v f0=(1+0.01cos(x/2)) v^2 exp(-v^2/2)/sqrt(2pi) coarse256 fine1024 psi1024 dt1/32"}
    res = {}
    for prec in ("mixed", "fp64"):
        cli = ["workspace=%s/" % work, "sim_name=vp_%s" % prec, "simulation_type=cmm_vlasov_poisson_1d",
               "domain_bounds=%s" % w["bounds"], "grid_coarse=%d" % w["grid_coarse"], "grid_fine=%d" % w["grid_fine"],
               "grid_vort=%d" % w["grid_vort"], "grid_psi=%d" % w["grid_psi"], "set_dt_by_steps=1",
               "steps_per_sec=%d" % w["steps_per_sec"], "final_time=%r" % final, "initial_condition=landau_damping",
               "initial_discrete=1", "initial_discrete_grid=%d" % w["grid_fine"], "time_integration=RK3",
               "map_update_order=4th", "map_epsilon=0.001", "incomp_threshold=%r" % w["incomp_threshold"],
               "skip_remapping=0", "molly_stencil=0", "lagrange_init_higher_order=1", "mem_RAM_CPU_remaps=20000",
               "particles_advected_num=0", "save_computational_num=0", "save_sample_num=0", "verbose=0",
               "save_map_stack=0", "precision=%s" % prec]
        stream = torch.cuda.Stream()
        sim = m.Simulation(cli, stream=stream.cuda_stream)
        sim.set_initial_discrete(f0)
        sim.init()
        hc = 4 * np.pi / w["grid_coarse"]

        def diag():
            f = sim.field("Distribution_coarse")
            return {"t": sim.scalar("time"), "maps": int(sim.scalar("map_counter")), "mass": sim.scalar("mass"),
                    "l2": float(hc * hc * np.sum(f * f)), "etot": sim.scalar("etot"), "ekin": sim.scalar("ekin"),
                    "epot": sim.scalar("epot"), "emode1": sim.scalar("emode1")}

        series = [diag()]
        every = 5 * w["steps_per_sec"]
        torch.cuda.synchronize()
        wall = 0.0
        n = 0
        t0 = time.perf_counter()
        while True:
            rc = sim.step(1)
            if rc == 1:
                break
            n += 1
            if n % every == 0:
                torch.cuda.synchronize()
                wall += time.perf_counter() - t0
                series.append(diag())
                t0 = time.perf_counter()
        torch.cuda.synchronize()
        wall += time.perf_counter() - t0
        res[prec] = dict(series[-1], steps=n, wall_s=wall, steps_per_s=n / wall, series=series)
        sim.close()
    keys = ("mass", "l2", "etot", "ekin", "epot", "emode1")
    out["mixed"] = {k: v for k, v in res["mixed"].items() if k != "series"}
    out["plain_fp64"] = {k: v for k, v in res["fp64"].items() if k != "series"}
    out["speedup"] = res["mixed"]["steps_per_s"] / res["fp64"]["steps_per_s"]
    out["rel_err"] = {k: abs(res["mixed"][k] - res["fp64"][k]) / abs(res["fp64"][k]) for k in keys}
    out["rel_err_series"] = [dict({"t": round(a["t"], 3), "maps_mixed": a["maps"], "maps_plain": b["maps"]},
                                  **{k: abs(a[k] - b[k]) / abs(b[k]) for k in keys})
                             for a, b in zip(res["mixed"]["series"], res["fp64"]["series"])]
    print(json.dumps(out))
    shutil.rmtree(work, ignore_errors=True)


def run_t10(args):
    """Both forms to T = 10: the metric's enstrophy error over the whole run."""
    import __graft_entry__ as ge
    ge.build()
    m = ge.package()
    import torch
    ic = initial_vorticity(WORKLOAD["grid_fine"], WORKLOAD["seed"], WORKLOAD["k0"])
    work = tempfile.mkdtemp(prefix="cmm_t10_")
    cli, recs = sim_args(work, "mixed", particles=args.t10_particles)
    pf = os.path.join(work, "params.txt")
    write_param_file(pf, cli, recs)
    mixed = full_run(m, torch, pf, ic, "mixed", final_time=args.t10_final)
    plain = full_run(m, torch, pf, ic, "fp64", final_time=args.t10_final)
    zs = [(a[0], abs(a[1] - b[1]) / abs(b[1]), abs(a[2] - b[2]) / abs(b[2]))
          for a, b in zip(mixed["series"], plain["series"])]
    out = {"validation": "chosen (mixed) vs plain FP64 over the whole run", "final_time": args.t10_final,
           "workload": "euler2d-turbulence coarse512 fine2048 psi1024 dt1/256, %d tracers" % args.t10_particles,
           "mixed": {k: mixed[k] for k in ("steps", "wall_s", "steps_per_s", "maps")},
           "plain_fp64": {k: plain[k] for k in ("steps", "wall_s", "steps_per_s", "maps")},
           "speedup": mixed["steps_per_s"] / plain["steps_per_s"],
           "max_enstrophy_rel_err": max(z[1] for z in zs), "max_energy_rel_err": max(z[2] for z in zs),
           "enstrophy_series": [(round(z[0], 4), z[1]) for z in zs]}
    print(json.dumps(out))
    shutil.rmtree(work, ignore_errors=True)


class MT19937_64:
    """The 64-bit Mersenne Twister (Matsumoto and Nishimura, 2000) with the standard
    seeding (the engine std::mt19937_64 names), for drawing the ensemble's members."""
    def __init__(self, seed):
        m = (1 << 64) - 1
        self.mt = [seed & m]
        for i in range(1, 312):
            self.mt.append((6364136223846793005 * (self.mt[-1] ^ (self.mt[-1] >> 62)) + i) & m)
        self.i = 312

    def __call__(self):
        m = (1 << 64) - 1
        if self.i >= 312:
            mt = self.mt
            for k in range(312):
                y = (mt[k] & 0xFFFFFFFF80000000) | (mt[(k + 1) % 312] & 0x7FFFFFFF)
                mt[k] = mt[(k + 156) % 312] ^ (y >> 1) ^ (0xB5026F5AA96619E9 if y & 1 else 0)
            self.i = 0
        y = self.mt[self.i]
        self.i += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & m


ENSEMBLE = dict(members=64, sizes=(64, 96, 128, 192, 256), seed=0, final_time=5.0, incomp_threshold=1e-3)


def ensemble_members(n=ENSEMBLE["members"], seed=ENSEMBLE["seed"]):
    """Member i: N = sizes[g() % 5], k0 = 4 + 12 u with u = (g() >> 11) 2^-53, g = mt19937_64(seed)."""
    g = MT19937_64(seed)
    out = []
    for _ in range(n):
        size = ENSEMBLE["sizes"][g() % len(ENSEMBLE["sizes"])]
        k0 = 4.0 + 12.0 * ((g() >> 11) * 2.0 ** -53)
        out.append((size, k0))
    return out


def ensemble_args(work, i, n, precision="mixed", threshold=None):
    """N / 4N / 2N grids (map / fine = vort / psi), dt = 1/(N/2) (the metric workload's
    CFL ratio), remaps at 1e-3 (the run of record; at the metric workload's 1e-4 the small
    members remap on most steps, in FP64 as in the mixed form: both are reported)."""
    e = dict(ENSEMBLE, incomp_threshold=threshold or ENSEMBLE["incomp_threshold"])
    return ["workspace=%s/" % work, "sim_name=e%02d_%s" % (i, precision), "simulation_type=cmm_euler_2d",
            "grid_coarse=%d" % n, "grid_fine=%d" % (4 * n), "grid_vort=%d" % (4 * n), "grid_psi=%d" % (2 * n),
            "set_dt_by_steps=1", "steps_per_sec=%d" % (n // 2), "final_time=%r" % e["final_time"],
            "initial_condition=4_nodes", "initial_discrete=1", "initial_discrete_grid=%d" % (4 * n),
            "time_integration=RK3", "map_update_order=4th", "map_epsilon=0.001",
            "incomp_threshold=%r" % e["incomp_threshold"], "skip_remapping=0", "molly_stencil=0",
            "freq_cut_psi=%d" % n, "lagrange_init_higher_order=1", "mem_RAM_CPU_remaps=100000",
            "save_computational_num=0", "save_sample_num=0", "save_zoom_num=0", "forward_map=0",
            "particles_advected_num=0", "save_map_stack=0", "verbose=0", "precision=%s" % precision]


def run_ensemble(args):
    """The 64-member ensemble of uneven sizes to T = 5: member-steps/s batched
    (cmm_ensemble_*, autotuned persistent grids, CUDA graphs) against the same members
    run one after another as single simulations, and every member's energy and
    enstrophy against the member run alone in plain FP64."""
    import __graft_entry__ as ge
    ge.build()
    m = ge.package()
    import torch
    members = ensemble_members()
    ics = [initial_vorticity(4 * n, seed=i, k0=k0) for i, (n, k0) in enumerate(members)]
    work = tempfile.mkdtemp(prefix="cmm_ens_")
    stream = torch.cuda.Stream()

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, a.elapsed_time(b) / 1e3

    if args.ensemble_iterations or args.ensemble_profile:
        ens = m.Ensemble([ensemble_args(work, i, n) for i, (n, _) in enumerate(members)],
                         stream=stream.cuda_stream, graphs=not args.ensemble_iterations)
        for i, w in enumerate(ics):
            ens.set_initial_discrete(i, w)
        ens.init()
        if args.ensemble_profile:
            ens.set_profiling(True)
        wall, _ = timed((lambda: ens.step(args.ensemble_iterations)) if args.ensemble_iterations else ens.run)
        st = ens.stats()
        out = {"member_steps": st["member_steps"], "iterations": st["iterations"], "wall_s": wall,
               "member_steps_per_s": st["member_steps"] / wall, "fused_info": ens.fused_info(),
               "tuning": [list(r) for r in ens.tuning()]}
        if args.ensemble_profile:
            p = ens.profile()
            tot = sum(c for c, _ in p["stages"].values()) + p["barrier_cycles"]
            out["stages"] = {k: {"share": c / tot, "tasks": n, "cycles_per_task": c / max(n, 1)}
                             for k, (c, n) in p["stages"].items()}
            out["barrier_share"] = p["barrier_cycles"] / tot
            out["wave_ms"] = [x / 1e6 for x in p["wave_ns"] if x]
        ens.close()
        print(json.dumps(out))
        shutil.rmtree(work, ignore_errors=True)
        return
    res = {}
    # (graphs, form): the autotuned form (the headline), the single launch alone and the two-phase
    # iteration with host remaps (the earlier form), each with its CUDA graphs
    variants = ((True, None),) if args.ensemble_batched_only else ((True, None), (True, True), (True, False))
    for graphs, fused in variants:
        ens = m.Ensemble([ensemble_args(work, i, n) for i, (n, _) in enumerate(members)],
                         stream=stream.cuda_stream, graphs=graphs, fused=fused)
        for i, w in enumerate(ics):
            ens.set_initial_discrete(i, w)
        init_wall, _ = timed(ens.init)
        wall, dev = timed(ens.run)
        st = ens.stats()
        info = ens.fused_info()
        res[(graphs, fused)] = dict(st, init_s=init_wall, wall_s=wall, device_s=dev,
                                    member_steps_per_s=st["member_steps"] / wall,
                                    form="single launch" if info["fused"] else "two-phase",
                                    register_budget=info["register_budget"],
                                    fused_blocks=info["blocks"],
                                    tiles_per_task=info["tiles_per_task"], why=info["why"],
                                    tuning=[list(r) for r in ens.tuning()],
                                    diag=[(ens.scalar(i, "energy"), ens.scalar(i, "enstrophy"),
                                           int(ens.scalar(i, "map_counter"))) for i in range(len(members))])
        ens.close()
    if args.ensemble_batched_only:
        b = res[(True, None)]
        print(json.dumps({"batched_graphs": {k: v for k, v in b.items() if k != "diag"}}))
        return
    seq = {"mixed": dict(member_steps=0, wall_s=0.0, diag=[]), "fp64": dict(member_steps=0, wall_s=0.0, diag=[])}
    for prec in ("mixed", "fp64"):
        for i, (n, _) in enumerate(members):
            sim = m.Simulation(ensemble_args(work, i, n, prec), stream=stream.cuda_stream)
            sim.set_initial_discrete(ics[i])
            sim.init()

            def go():
                while sim.step(1) != 1:
                    seq[prec]["member_steps"] += 1

            wall, _ = timed(go)
            seq[prec]["wall_s"] += wall
            seq[prec]["diag"].append((sim.scalar("energy"), sim.scalar("enstrophy"), int(sim.scalar("map_counter"))))
            sim.close()
    # the whole ensemble again at the metric workload's remap threshold 1e-4: batched (the tuned
    # form) against every member run alone in plain FP64
    ens = m.Ensemble([ensemble_args(work, i, n, threshold=1e-4) for i, (n, _) in enumerate(members)],
                     stream=stream.cuda_stream)
    for i, w in enumerate(ics):
        ens.set_initial_discrete(i, w)
    ens.init()
    wall4, _ = timed(ens.run)
    st4 = ens.stats()
    diag4 = [(ens.scalar(i, "energy"), ens.scalar(i, "enstrophy"), int(ens.scalar(i, "map_counter")))
             for i in range(len(members))]
    form4 = "single launch" if ens.fused_info()["fused"] else "two-phase"
    ens.close()
    fp4 = []
    for i, (n, _) in enumerate(members):
        sim = m.Simulation(ensemble_args(work, i, n, "fp64", threshold=1e-4), stream=stream.cuda_stream)
        sim.set_initial_discrete(ics[i])
        sim.init()
        sim.run()
        fp4.append((sim.scalar("energy"), sim.scalar("enstrophy"), int(sim.scalar("map_counter"))))
        sim.close()
    study = {"member_steps": st4["member_steps"], "wall_s": wall4, "member_steps_per_s": st4["member_steps"] / wall4,
             "form": form4, "remaps_batched": sum(x[2] for x in diag4), "remaps_fp64": sum(y[2] for y in fp4),
             "members_with_equal_remaps": sum(1 for x, y in zip(diag4, fp4) if x[2] == y[2]),
             "max_energy_rel_err_vs_fp64": max(abs(x[0] - y[0]) / abs(y[0]) for x, y in zip(diag4, fp4)),
             "max_enstrophy_rel_err_vs_fp64": max(abs(x[1] - y[1]) / abs(y[1]) for x, y in zip(diag4, fp4))}
    b, plain = res[(True, None)], seq["fp64"]
    rel = [(abs(x[0] - y[0]) / abs(y[0]), abs(x[1] - y[1]) / abs(y[1])) for x, y in zip(b["diag"], plain["diag"])]
    counts = {str(s): sum(1 for n, _ in members if n == s) for s in ENSEMBLE["sizes"]}
    out = {"validation": "64-member ensemble of uneven sizes, batched vs one after another, vs plain FP64",
           "workload": "euler2d-ensemble 64 members N in {64,96,128,192,256} (mt19937_64 seed 0), fine 4N, psi 2N, "
                       "dt 1/(N/2), T=5, k0~U[4,16], remap 1e-3",
           "sizes": counts, "unit": "member-steps/s",
           "batched_graphs": {k: b[k] for k in ("member_steps", "iterations", "launches", "form", "register_budget",
                                                "fused_blocks", "tiles_per_task", "tuning", "init_s", "wall_s",
                                                "device_s", "member_steps_per_s")},
           "single_launch_graphs": {k: res[(True, True)][k] for k in ("launches", "register_budget", "fused_blocks",
                                                                      "tiles_per_task", "wall_s", "device_s",
                                                                      "member_steps_per_s")},
           "two_phase_host_remaps_graphs": {k: res[(True, False)][k] for k in ("launches", "advect_blocks",
                                                                               "sample_blocks", "wall_s", "device_s",
                                                                               "member_steps_per_s")},
           "single_launch_equals_two_phase_maps": sum(1 for x, y in zip(res[(True, True)]["diag"],
                                                                        res[(True, False)]["diag"]) if x[2] == y[2]),
           "sequential_mixed": {"member_steps": seq["mixed"]["member_steps"], "wall_s": seq["mixed"]["wall_s"],
                                "member_steps_per_s": seq["mixed"]["member_steps"] / seq["mixed"]["wall_s"]},
           "sequential_fp64": {"member_steps": plain["member_steps"], "wall_s": plain["wall_s"],
                               "member_steps_per_s": plain["member_steps"] / plain["wall_s"]},
           "speedup_vs_sequential_mixed": b["member_steps_per_s"] * seq["mixed"]["wall_s"] / seq["mixed"]["member_steps"],
           "speedup_vs_sequential_fp64": b["member_steps_per_s"] * plain["wall_s"] / plain["member_steps"],
           "max_energy_rel_err_vs_fp64": max(r[0] for r in rel),
           "max_enstrophy_rel_err_vs_fp64": max(r[1] for r in rel),
           "batched_equals_sequential_mixed_maps": sum(1 for x, y in zip(b["diag"], seq["mixed"]["diag"]) if x[2] == y[2]),
           "remaps_batched": sum(x[2] for x in b["diag"]), "remaps_fp64": sum(y[2] for y in plain["diag"]),
           "threshold_1e-4": study}
    print(json.dumps(out))
    shutil.rmtree(work, ignore_errors=True)


LEARNED = dict(blocks=6, channels=32, train_seeds=100, pairs_per_seed=200, passes=2, batch=8, lr=1e-3,
               exact_every=8, tol=1e-4)


def conv_flops_per_pixel(blocks, C=32):
    """Tensor-core FLOPs per map-grid pixel of one training step (padded channel counts as
    executed): forward of every layer, input gradient of every layer but the head, weight
    gradient of every layer (M padded to 128 rows: 3 dx x cin)."""
    layers = [(16, C)] + [(C, C)] * (2 * blocks) + [(C, 16)]
    fwd = sum(2 * 9 * ci * co for ci, co in layers)
    dx = sum(2 * 9 * ci * co for ci, co in layers[1:])
    dw = sum(2 * 3 * 128 * co for ci, co in layers)
    return fwd, fwd + dx + dw


def run_learned(args):
    """The learned psi on the metric workload: training pairs streamed from seeded runs
    (seeds 1..S to T = 10, P pairs per run at evenly spaced steps: 100 x 200 = 20 000 pairs
    by default, the size of the learned-psi configuration; the metric's seed 0 is held out),
    each run's pairs trained on (`passes` epochs of batches) and dropped before the next run,
    then the held-out seed 0 to T = 10 three ways (exact mixed form, learned form with exact
    evaluation every 8 steps at psi tolerance 1e-4, plain FP64) plus the psi errors of the
    cheap, learned and psi-grid evaluations along an exact run."""
    import __graft_entry__ as ge
    ge.build()
    m = ge.package()
    import torch
    L = LEARNED
    work = tempfile.mkdtemp(prefix="cmm_learned_")
    cli, _ = sim_args(work, "mixed", particles=1000)
    cli = [c for c in cli if not c.startswith("particles_advected_num")] + ["particles_advected_num=0"]
    pf = os.path.join(work, "params.txt")
    write_param_file(pf, cli, [])
    stream = torch.cuda.Stream()
    u = m.Upsampler(blocks=L["blocks"], channels=L["channels"], seed=1, stream=stream.cuda_stream)
    t0 = time.perf_counter()
    S, P = args.learned_seeds, args.learned_pairs_per_seed
    steps_run = int(round(args.t10_final * WORKLOAD["steps_per_sec"]))
    iters = max(1, L["passes"] * P // L["batch"])   # Adam steps on each run's pairs
    losses, train_s, pairs, iterations = [], 0.0, 0, 0
    for r, seed in enumerate(range(1, 1 + S)):
        sim = m.Simulation(["param_file=" + pf, "final_time=%g" % args.t10_final], stream=stream.cuda_stream)
        sim.set_initial_discrete(initial_vorticity(WORKLOAD["grid_fine"], seed, WORKLOAD["k0"]))
        sim.init()
        k = 0
        while sim.step(1) != 1:
            k += 1
            if (k * P) // steps_run != ((k - 1) * P) // steps_run:   # P evenly spaced steps of the run
                u.collect(sim)
        sim.close()
        pairs += u.dataset_size()
        loss, sec = u.train(iters, batch=L["batch"], lr=L["lr"] if r < 0.8 * S else L["lr"] / 5, seed=r)
        losses.append(loss)
        train_s += sec
        iterations += iters
        u.clear_dataset()
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0 - train_s
    fwd_pp, train_pp = conv_flops_per_pixel(L["blocks"], L["channels"])
    px = WORKLOAD["grid_coarse"] ** 2
    ic = initial_vorticity(WORKLOAD["grid_fine"], WORKLOAD["seed"], WORKLOAD["k0"])
    exact = full_run(m, torch, pf, ic, "mixed", final_time=args.t10_final)
    learned = full_run(m, torch, pf, ic, "mixed", final_time=args.t10_final, ups=u, exact_every=L["exact_every"],
                       tol=L["tol"])
    plain = full_run(m, torch, pf, ic, "fp64", final_time=args.t10_final)
    # psi errors along an exact run of the held-out seed
    sim = m.Simulation(["param_file=" + pf, "final_time=%g" % args.t10_final], stream=stream.cuda_stream)
    sim.set_initial_discrete(ic)
    sim.init()
    errs, k = [], 0
    while sim.step(1) != 1:
        k += 1
        if k % 256 == 0:
            e = u.evaluate(sim)
            errs.append({"t": round(sim.scalar("time"), 3), **{q: float("%.3e" % v) for q, v in e.items()}})
    sim.close()

    def zerr(a, b):
        return max(abs(x[1] - y[1]) / abs(y[1]) for x, y in zip(a["series"], b["series"]))

    keep = ("steps", "wall_s", "steps_per_s", "maps")
    out = {"validation": "learned psi on the metric workload (held-out seed 0), against the exact mixed form and plain FP64",
           "workload": "euler2d-turbulence coarse512 fine2048 psi1024 dt1/256 T=%g, no tracers" % args.t10_final,
           "network": {"blocks": L["blocks"], "channels": L["channels"], "params": u.num_params(),
                       "inputs": "psi, psi_x, psi_y, psi_xy (cheap), omega, omega_x, omega_y on 512^2",
                       "output": "sub-grid vorticity on the 1024^2 psi grid"},
           "training": {"pairs": pairs, "seeds": "1..%d (seed 0 held out)" % S, "pairs_per_run": P,
                        "streamed": "each run's pairs trained on (%d Adam steps) and dropped" % iters,
                        "pair_generation_s": gen_s, "iterations": iterations, "batch": L["batch"],
                        "device_s": train_s, "samples_per_s": iterations * L["batch"] / train_s,
                        "conv_tflops": iterations * L["batch"] * px * train_pp / train_s / 1e12,
                        "loss_first_last": [losses[0], losses[-1]], "loss": "mean relative psi-space error"},
           "exact_mixed": {k: exact[k] for k in keep},
           "learned": {k: learned[k] for k in keep + ("learned_steps", "cheap_steps", "exact_steps", "learned_checks",
                                                      "learned_cheaper", "learned_failures", "learned_max_err")},
           "plain_fp64": {k: plain[k] for k in keep},
           "learned_vs_plain_fp64": {"speedup": learned["steps_per_s"] / plain["steps_per_s"],
                                     "max_enstrophy_rel_err": zerr(learned, plain)},
           "exact_mixed_vs_plain_fp64": {"speedup": exact["steps_per_s"] / plain["steps_per_s"],
                                         "max_enstrophy_rel_err": zerr(exact, plain)},
           "learned_vs_exact_mixed_max_enstrophy_rel_err": zerr(learned, exact),
           "inference_conv_gflop_per_step": px * fwd_pp / 1e9,
           "inference": {"ms": u.time_infer(WORKLOAD["grid_coarse"], WORKLOAD["grid_coarse"]),
                         "note": "one forward pass at 512^2 (input assembly, 14 convs, sub-pixel output)"},
           "psi_errors_along_exact_run": errs}
    print(json.dumps(out))
    shutil.rmtree(work, ignore_errors=True)


def run_learned_profile(args):
    """Small runs of the learned psi's kernels for ncu captures.  infer: the metric workload
    (no tracers) with a 6-block network attached and only the first step exact, 3 + 4 steps;
    train: pairs every 8 steps of a 128^2 map / 512^2 vorticity run to T = 2, then 4 Adam
    steps of batch 32 (weights of either are untrained: the cost does not depend on them)."""
    import __graft_entry__ as ge
    ge.build()
    m = ge.package()
    import torch
    work = tempfile.mkdtemp(prefix="cmm_lprof_")
    if args.learned_profile == "infer":
        cli, _ = sim_args(work, "mixed", particles=1000)
        cli = [c for c in cli if not c.startswith("particles_advected_num")] + ["particles_advected_num=0",
                                                                                 "final_time=1"]
        sim = m.Simulation(cli)
        sim.set_initial_discrete(initial_vorticity(WORKLOAD["grid_fine"], 0, WORKLOAD["k0"]))
        sim.init()
        u = m.Upsampler(blocks=LEARNED["blocks"], seed=2)
        sim.attach_upsampler(u, every=1000000, tol=1e9)
        sim.step(3)
        ms = u.time_infer(WORKLOAD["grid_coarse"], WORKLOAD["grid_coarse"], 20)
        fwd_pp, _ = conv_flops_per_pixel(LEARNED["blocks"], LEARNED["channels"])
        print(json.dumps({"inference_ms": ms, "conv_tflops": WORKLOAD["grid_coarse"] ** 2 * fwd_pp / (ms * 1e-3) / 1e12}))
    else:
        n = 128
        cli = ["workspace=%s/" % work, "sim_name=prof", "grid_coarse=%d" % n, "grid_fine=%d" % (4 * n),
               "grid_vort=%d" % (4 * n), "grid_psi=%d" % (2 * n), "set_dt_by_steps=1", "steps_per_sec=%d" % (n // 2),
               "final_time=2", "initial_condition=4_nodes", "initial_discrete=1", "initial_discrete_grid=%d" % (4 * n),
               "time_integration=RK3", "map_update_order=4th", "map_epsilon=0.001", "incomp_threshold=1e-4",
               "molly_stencil=0", "freq_cut_psi=%d" % (n // 4), "mem_RAM_CPU_remaps=100000",
               "save_computational_num=0", "save_sample_num=0", "save_zoom_num=0", "particles_advected_num=0",
               "save_map_stack=0", "verbose=0", "precision=mixed"]
        sim = m.Simulation(cli)
        sim.set_initial_discrete(initial_vorticity(4 * n, 1, 8.0))
        sim.init()
        u = m.Upsampler(blocks=LEARNED["blocks"], seed=1)
        k = 0
        while sim.step(1) != 1:
            k += 1
            if k % 8 == 0:
                u.collect(sim)
        loss, sec = u.train(4, batch=32, lr=1e-3, seed=0)
        print(json.dumps({"pairs": u.dataset_size(), "loss": loss, "train_s": sec}))
    shutil.rmtree(work, ignore_errors=True)


def run_ours(args):
    import __graft_entry__ as ge
    ge.build()
    m = ge.package()
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ic = initial_vorticity(WORKLOAD["grid_fine"], WORKLOAD["seed"], WORKLOAD["k0"])
    work = tempfile.mkdtemp(prefix="cmm_bench_")
    cli, recs = sim_args(work, args.precision)
    pf = os.path.join(work, "params.txt")
    write_param_file(pf, cli, recs)

    # ---- the chosen form: value, clocks, phases
    clocks = ClockSampler()
    chosen = measure_form(m, torch, pf, ic, args.precision, args, world, clocks=clocks)
    # ---- plain FP64 over the same warm-up + K steps from the same state
    plain = None
    if args.precision != "fp64" and not args.no_plain:
        plain = measure_form(m, torch, pf, ic, "fp64", args, world, profile=False)
    # ---- e2e through the C-ABI with host buffers
    e2e_line = None if args.no_e2e else _e2e(m, torch, ic, pf, args, world)
    _report(args, world, rank, chosen, plain, clocks, e2e_line, ic)
    shutil.rmtree(work, ignore_errors=True)


def _e2e(m, torch, ic, pf, args, world):
    ic_pinned = torch.from_numpy(ic).pin_memory()
    stream2 = torch.cuda.Stream()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim2 = m.Simulation(["param_file=" + pf, "precision=" + args.precision,
                         "final_time=%r" % ((args.steps + 32) / WORKLOAD["steps_per_sec"])], stream=stream2.cuda_stream)
    sim2.set_initial_discrete(ic_pinned.numpy())
    sim2.init()
    d2h = 0
    for _ in range(args.steps):
        sim2.step(1)
        sim2.scalar("e_inc")          # the step's monitoring record (read back inside the step)
        d2h += 8
    psi = sim2.field("Stream_function_Psi_H_psi")
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    d2h += psi.nbytes
    sim2.close()
    e2e = world * args.steps / e2e_s
    return {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": ic.nbytes / args.steps,
            "d2h_bytes_per_step": d2h / args.steps,
            "includes": "IC upload + init (Lagrange history) + every step + final psi readback"}


def roofline_model():
    import importlib.util
    path = os.path.join(ROOT, "cmm-turbulence_gb300", "roofline_model.py")
    spec = importlib.util.spec_from_file_location("cmm_gb300_roofline_model", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def phase_models(w, precision):
    """Algorithmic (compulsory) HBM bytes of each loop phase per step (word 8
    for the plain FP64 form, 4 for the FP32 nodes of the mixed form) and the
    counted FLOPs of the advection."""
    rm = roofline_model()
    return rm.phase_bytes(w, 8 if precision == "fp64" else 4), rm.step_flops(w)["advect"]


def _report(args, world, rank, chosen, plain, clocks, e2e_line, ic):
    phases = chosen["phases"]
    per = {k: v["ms_total"] / max(1, v["launches"]) for k, v in phases.items() if v["launches"]}
    models, flops = phase_models(WORKLOAD, args.precision)
    peak, peak_kind = load_peaks()
    # the coarse vorticity is sampled only when read (not per step) in the 2D Euler form
    per.pop("coarse", None)
    # the roofline kernel: the single-kernel phase (advection, incompressibility check,
    # tracers) with the largest measured time; the psi phase (sample, row transform, column
    # transforms with the spectral step, inverse rows with the node pass) is reported in the
    # breakdown with its own HBM fraction
    single = [k for k in ("advect", "incomp", "particles") if k in per and k in models]
    dom = max(single, key=lambda k: per[k])
    ms = per[dom]
    achieved = models[dom] / (ms / 1000.0) / 1e9
    kernels = {"advect": "k_advect (GALS map advection)", "incomp": "k_incomp (det grad X, max)",
               "psi": "psi solve (k_sample + k_rows_r2c + k_psi_cols + k_psi_rows_inv)", "coarse": "k_sample (coarse omega)",
               "particles": "k_particles (RK3 tracers)"}
    roof = {"kernel": kernels.get(dom, dom), "phase": dom, "bound": "hbm", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_source": "of " + peak_kind,
            "traffic": NCU_TRAFFIC.get((args.precision, dom), (None, None))[0],
            "traffic_source": NCU_TRAFFIC.get((args.precision, dom), (None, None))[1],
            "ms_per_launch": ms, "algorithmic_bytes": models[dom],
            "phases": {k: {"ms": per[k], "GBps": models[k] / (per[k] / 1000.0) / 1e9,
                           "frac": models[k] / (per[k] / 1000.0) / 1e9 / peak} for k in per if k in models}}
    if args.precision == "fp64":
        adv = per.get("advect", 1.0)
        roof["fp64"] = {"achieved_tflops": flops / (adv / 1000.0) / 1e12, "peak_tflops": FP64_PEAK_TFLOPS,
                        "frac": flops / (adv / 1000.0) / 1e12 / FP64_PEAK_TFLOPS,
                        "note": "the plain FP64 form is bound by GB300's FP64 issue rate, not HBM"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n = CPU_SAMPLE_STEPS
        sps, secs = cpu_oracle_steps(n, ic, threads, particles=WORKLOAD["particles"])
        cpu = {"value": sps, "unit": "steps/s", "cores": threads, "kind": "port",
               "sample": "%d full workload steps after the oracle's Lagrange initialisation (%.1f s)" % (n, secs)}
    if rank != 0:
        return
    comparison = None
    if plain is not None:
        comparison = {"plain_fp64_value": plain["value"], "plain_fp64_ms_per_step": plain["ms"] / args.steps,
                      "speedup_vs_plain_fp64": chosen["value"] / plain["value"],
                      "time": chosen["time"], "maps_chosen": chosen["maps"], "maps_plain": plain["maps"],
                      "enstrophy_rel_err": abs(chosen["enstrophy"] - plain["enstrophy"]) / abs(plain["enstrophy"]),
                      "energy_rel_err": abs(chosen["energy"] - plain["energy"]) / abs(plain["energy"]),
                      "palinstrophy_rel_err": abs(chosen["palinstrophy"] - plain["palinstrophy"]) / abs(plain["palinstrophy"])}
    form = {"fp64": "plain FP64", "mixed": "mixed: FP32 displacement maps + FP32 Hermite psi/omega, FP64 "
                                           "composition, FP64 det deviation, FP64 diagnostics"}.get(args.precision, args.precision)
    line = {"metric": METRIC, "value": chosen["value"], "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": chosen["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic",
            "config": {"workload": "euler2d-turbulence coarse512 fine2048 psi1024 dt1/256 1e6 tracers",
                       "form": form, "remaps_in_timed_region": chosen["remaps"],
                       "l2": "working set per step > 129 MB L2 (psi levels, fine vorticity, map)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "clocks": clocks.summary(), "gpu_launches": chosen["launches"], "e2e": e2e_line,
            "vs_plain_fp64": comparison, "roofline": roof, "cpu_baseline": cpu}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2560, help="timed steps from t = 0 (2560 = the whole T = 10 run)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--t10", action="store_true", help="run both forms to the final time and report the enstrophy error")
    ap.add_argument("--t10-final", type=float, default=10.0)
    ap.add_argument("--t10-particles", type=int, default=WORKLOAD["particles"])
    ap.add_argument("--fp64-peak", action="store_true", help="measure the FP64 rate (cuBLAS DGEMM) and exit")
    ap.add_argument("--vlasov", action="store_true", help="run the Vlasov-Poisson configuration in both forms")
    ap.add_argument("--vlasov-final", type=float, default=VLASOV["final_time"])
    ap.add_argument("--ensemble", action="store_true", help="run the 64-member ensemble batched and one by one")
    ap.add_argument("--ensemble-batched-only", action="store_true", help="with --ensemble: only the batched run")
    ap.add_argument("--ensemble-profile", action="store_true",
                    help="with --ensemble: the batched run with the single launch's per-stage counters")
    ap.add_argument("--ensemble-iterations", type=int, default=0,
                    help="with --ensemble: only this many batched iterations, without graphs (for an ncu capture)")
    ap.add_argument("--learned", action="store_true", help="train the psi upsampler and run the learned form")
    ap.add_argument("--learned-seeds", type=int, default=LEARNED["train_seeds"])
    ap.add_argument("--learned-pairs-per-seed", type=int, default=LEARNED["pairs_per_seed"])
    ap.add_argument("--learned-profile", choices=["infer", "train"], help="small learned-psi runs for ncu captures")
    args = ap.parse_args()
    if args.fp64_peak:
        measure_fp64_peak()
    elif args.ensemble:
        run_ensemble(args)
    elif args.learned:
        run_learned(args)
    elif args.learned_profile:
        run_learned_profile(args)
    elif args.vlasov:
        run_vlasov(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.t10:
        run_t10(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
