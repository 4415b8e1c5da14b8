"""GPU tests of the Vlasov-Poisson path (simulation_type=cmm_vlasov_poisson_1d).

Plain FP64 against the CPU oracle step by step (same inputs, FP64; the
oracle takes the reference's 2D FFT of the assembled psi, the product the
equivalent 1D spectra of its separable parts), the mixed form against plain
FP64, the analytic t = 0 answers of Landau damping, the reference golden's
t = 0 rows through the reference's own parameter file, and the reference's
rejection of a vort grid finer than the psi grid.

Tolerances as in test_gpu_parity.py: maps and spectral Hermite fields in
units of their conditioning (map_err, herm_err), distribution and
diagnostics relative 1e-10 after a run with remaps; E_inc absolutely, in
units of the map's conditioning (einc_tol).
"""
import numpy as np
import pytest

import oracle as O
import refloop
from goldens import DebugRecorder, compare_series, goldens
from product import cmm, read_monitoring
from test_gpu_parity import herm_err, map_err, rel_linf

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

PI = np.pi
CASES = {
    # name: (initial condition, domain_bounds in units of pi)
    "landau": ("landau_damping", "{0,4,-2.5,2.5}"),
    "two_stream": ("two_stream", "{0,10,-2.5,2.5}"),
}


def _args(work, ic, bounds, precision="fp64", coarse=64, fine=128, psi=128, vort=128, sps=32, final_time=2.0,
          threshold=1e-4):
    return ["workspace=%s/" % work, "sim_name=vp", "simulation_type=cmm_vlasov_poisson_1d",
            "initial_condition=%s" % ic, "domain_bounds=%s" % bounds, "grid_coarse=%d" % coarse,
            "grid_fine=%d" % fine, "grid_vort=%d" % vort, "grid_psi=%d" % psi, "set_dt_by_steps=1",
            "steps_per_sec=%d" % sps, "final_time=%g" % final_time, "time_integration=RK3", "map_update_order=4th",
            "map_epsilon=0.001", "incomp_threshold=%r" % threshold, "skip_remapping=0", "molly_stencil=0",
            "lagrange_init_higher_order=1", "freq_cut_psi=%d" % (psi // 2), "particles_advected_num=0",
            "save_sample_num=0", "save_zoom_num=0", "forward_map=0", "mem_RAM_CPU_remaps=4000",
            "save_computational_num=0", "verbose=0", "precision=%s" % precision]


def einc_tol(max_x, h, eps=1e-3):
    """E_inc = max |1 - det grad X| inherits the map's conditioning: the
    X_xy plane carries footpoint rounding (relative to max|X|) times 1/eps^2,
    and enters det scaled by the cell size h.  5 u max|X| h / eps^2 is 1.7e-10
    for C1's Euler map and 8.5e-9 for the two-stream domain (10 pi)."""
    return 5 * 1.1e-16 * max_x * h / eps ** 2


def _oracle(args):
    s = refloop.Settings()
    for a in args:
        s.set_variable(a, "=")
    s.finalize()
    return O.EulerOracle(s.oracle_config()), s


@pytest.mark.parametrize("case", sorted(CASES))
def test_vlasov_plain_fp64_matches_oracle(tmp_path, case):
    ic, bounds = CASES[case]
    args = _args(tmp_path, ic, bounds)
    m = cmm()
    sim = m.Simulation(args)
    sim.init()
    o, s = _oracle(args)
    o.init()
    n = 128
    psi0 = sim.field("Stream_function_Psi_H_psi_all").reshape(3, -1)
    ref0 = o.psi(levels=3).reshape(3, -1)
    for lvl in range(3):
        assert herm_err(psi0[lvl], ref0[lvl], n) < 1e-12, lvl
    maps_gpu, maps_cpu = [], []
    b = s.domain_bounds
    tol = einc_tol(max(abs(x) for x in b[:4]), (b[1] - b[0]) / s.grid_coarse)
    while sim.step(1) != 1:
        _, e, _ = o.step(s.dt)
        assert abs(sim.scalar("e_inc") - e) < tol
        maps_gpu.append(int(sim.scalar("map_counter")))
        maps_cpu.append(o.map_count())
    assert len(maps_gpu) == 64 and maps_gpu == maps_cpu and maps_gpu[-1] >= 2
    assert map_err(sim.field("Map_ChiX_H_coarse"), o.chix()) < 1e-10
    assert map_err(sim.field("Map_ChiY_H_coarse"), o.chiy()) < 1e-10
    assert herm_err(sim.field("Vorticity_W_fine_H"), o.vort_fine(), 128) < 1e-10
    assert herm_err(sim.field("Stream_function_Psi_H_psi"), o.psi(), n) < 1e-10
    assert rel_linf(sim.field("Distribution_coarse"), o.vort()) < 1e-10
    ref = o.vlasov_mesure()
    for k in ("Etot", "Ekin", "Epot", "Mass", "Emode1"):
        assert abs(sim.scalar(k.lower()) - ref[k]) <= 1e-10 * abs(ref[k]), k
    assert abs(sim.scalar("momentum") - ref["Momentum"]) <= 1e-10 * ref["Mass"]
    sim.close()


def test_vlasov_forward_map_matches_oracle(tmp_path):
    """forward_map=1 in the Vlasov driver (cmm-vlasov1d.cu:815, 845): the forward map advected
    on the same separable psi history, its incompressibility and the invertibility check each
    step, and the forward map after a run with remaps, against the oracle."""
    ic, bounds = CASES["landau"]
    args = [a for a in _args(tmp_path, ic, bounds) if not a.startswith("forward_map")] + ["forward_map=1"]
    m = cmm()
    sim = m.Simulation(args)
    sim.init()
    o, s = _oracle(args)
    o.init()
    b = s.domain_bounds
    tol = einc_tol(max(abs(x) for x in b[:4]), (b[1] - b[0]) / s.grid_coarse)
    steps = 0
    while sim.step(1) != 1:
        o.step(s.dt)
        ef, ev = o.forward_monitors()
        assert abs(sim.scalar("e_inc_forward") - ef) < tol, steps
        assert abs(sim.scalar("e_invertibility") - ev) < 1e-9, steps
        steps += 1
    assert steps == 64 and int(sim.scalar("map_counter")) == o.map_count() >= 2
    assert map_err(sim.field("Map_ChiX_f_H_coarse"), o.chix_f()) < 1e-10
    assert map_err(sim.field("Map_ChiY_f_H_coarse"), o.chiy_f()) < 1e-10
    sim.close()


def test_vlasov_known_answers_at_t0(tmp_path):
    """Landau damping at t = 0: Epot = pi/100, |E_1| = 0.05, Ekin = 2 pi,
    Mass = 4 pi (derivation in test_oracle_golden.py)."""
    m = cmm()
    sim = m.Simulation(_args(tmp_path, "landau_damping", "{0,4,-2.5,2.5}", coarse=128, fine=256, psi=256, vort=256))
    sim.init()
    assert abs(sim.scalar("epot") - PI / 100) < 1e-12
    assert abs(sim.scalar("emode1") - 0.05) < 1e-12
    assert abs(sim.scalar("ekin") - 2 * PI) < 1e-11 and abs(sim.scalar("mass") - 4 * PI) < 1e-11
    psi = sim.field("Stream_function_Psi_H_psi").reshape(4, 256, 256)
    v = -2.5 * PI + (5 * PI / 256) * np.arange(256)
    centre = np.abs(v) < 3.0
    # 1e-9: on 256 v-nodes the bump's tanh edges span a few points, and the
    # spectral double integral of the bump is v there only to ~2e-10
    assert np.max(np.abs(psi[2][centre, :] - v[centre, None])) < 1e-9
    sim.close()


@pytest.mark.parametrize("case", sorted(CASES))
def test_vlasov_mixed_matches_plain_fp64(tmp_path, case):
    """Mixed form (FP32 displacement maps and distribution nodes, separable
    psi from 1D FP32 tables, FP64 potential and diagnostics) against plain
    FP64 over 64 steps with remaps."""
    ic, bounds = CASES[case]
    m = cmm()
    res = {}
    for prec in ("fp64", "mixed"):
        sim = m.Simulation(_args(tmp_path, ic, bounds, precision=prec))
        sim.init()
        while sim.step(1) != 1:
            pass
        res[prec] = ({k: sim.scalar(k) for k in ("etot", "ekin", "epot", "mass", "emode1")},
                     sim.field("Distribution_coarse"), int(sim.scalar("map_counter")))
        sim.close()
    (dp, fp, mp), (dm, fm, mm) = res["fp64"], res["mixed"]
    for k in ("etot", "ekin", "mass"):
        assert abs(dm[k] - dp[k]) <= 1e-6 * abs(dp[k]), (k, dm[k], dp[k])
    for k in ("epot", "emode1"):
        assert abs(dm[k] - dp[k]) <= 1e-4 * abs(dp[k]), (k, dm[k], dp[k])
    assert np.max(np.abs(fm - fp)) <= 1e-5 * np.max(np.abs(fp))
    assert abs(mm - mp) <= 1


def _sample_files(run, n):
    """{time directory: {plane name: array}} of the sampled outputs on the n grid"""
    import os
    base = os.path.join(run, "Time_data")
    out = {}
    for d in os.listdir(base):
        planes = {}
        for k in ("Map_ChiX", "Map_ChiY", "Distribution_F", "Stream_function_Psi"):
            f = os.path.join(base, d, "%s_%d.data" % (k, n))
            if os.path.exists(f):
                planes[k] = np.fromfile(f, dtype="<f8")
        if planes:
            out[d] = planes
    return out


def _periods(bounds):
    b = [float(v) * PI for v in bounds.strip("{}").split(",")[:4]]
    return b[1] - b[0], b[3] - b[2]


def _with_sample(work, args, rec):
    """the run's settings as a parameter file with one save_sample record (record lists are
    read from parameter files only, as in the reference) -> command-line arguments"""
    kv = [a.split("=", 1) for a in args if not a.startswith(("workspace=", "save_sample_num"))]
    lines = ["CMM Parameter file", "param_version\t=\t3", ""]
    lines += ["%s\t=\t%s" % (k, v) for k, v in kv]
    lines += ["save_sample_num\t=\t1", "save_sample\t=\t" + rec]
    pf = work / "params_sample.txt"
    pf.write_text("\n".join(lines) + "\n")
    return ["param_file=%s" % pf, "workspace=%s/" % work]


def wrap_err(a, b, period):
    """relative L-infinity of composed positions modulo whole periods (a point within rounding
    of the periodic boundary may land on either side)"""
    d = np.asarray(a) - np.asarray(b)
    d -= period * np.round(d / period)
    return float(np.max(np.abs(d)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("case", sorted(CASES))
def test_vlasov_sampled_outputs_match_oracle(tmp_path, case):
    """sample_compute_and_write_vlasov on a 96 x 96 sample grid (non-power-of-two 1D
    transforms) at t = 0, 1 and 2 of a run with remaps: the composed map, the distribution
    function, the written stream buffer (d phi / dx of the sample grid's own potential in
    its first 96 entries, the distribution from entry N / 8 on) and the nine Mesure series,
    against the oracle at the same instants; at t = 0 Landau damping's known answers."""
    import os
    ic, bounds = CASES[case]
    lx, ly = _periods(bounds)
    n = 96
    args = _args(tmp_path, ic, bounds)
    m = cmm()
    sim = m.Simulation(_with_sample(tmp_path, args, "{is_instant=0,time_start=0,time_end=2,time_step=1,var=All,grid=%d}" % n))
    sim.init()
    o, s = _oracle(args)
    o.init()
    expect = [o.vlasov_sample(n)]
    k = 0
    while sim.step(1) != 1:
        o.step(s.dt)
        k += 1
        if k % 32 == 0:
            expect.append(o.vlasov_sample(n))
    run = os.path.join(str(tmp_path), "data", sim.file_name())
    maps = int(sim.scalar("map_counter"))
    sim.close()
    assert maps >= 2
    mon = read_monitoring(run)
    assert np.allclose(mon["Mesure/Time_s_%d" % n], [0.0, 1.0, 2.0], atol=1e-12)
    files = _sample_files(run, n)
    assert len(files) == 3
    N = n * n
    for i, d in enumerate(sorted(files, key=lambda t: float(t.split("_")[-1]) if t[-1].isdigit() else 1e9)):
        planes, mes = expect[i]
        got = files[d]
        assert wrap_err(got["Map_ChiX"], planes["Map_ChiX"], lx) < 1e-10, (d, "x")
        assert wrap_err(got["Map_ChiY"], planes["Map_ChiY"], ly) < 1e-10, (d, "y")
        assert rel_linf(got["Distribution_F"], planes["Distribution_F"]) < 1e-10, d
        e, er = got["Stream_function_Psi"][:n], planes["Stream_function_Psi"][:n]
        assert np.max(np.abs(e - er)) <= 1e-9 * np.max(np.abs(er)), d
        assert np.array_equal(got["Stream_function_Psi"][N // 8:], got["Distribution_F"][N // 8:])
        assert not np.any(got["Stream_function_Psi"][n:N // 8])
        for key in ("Etot", "Ekin", "Epot", "Mass", "Emode1"):
            assert abs(mon["Mesure/%s_%d" % (key, n)][i] - mes[key]) <= 1e-9 * abs(mes[key]), (d, key)
        assert abs(mon["Mesure/Momentum_%d" % n][i] - mes["Momentum"]) <= 1e-10 * mes["Mass"], d
    if case == "landau":
        assert abs(mon["Mesure/Epot_%d" % n][0] - PI / 100) < 1e-12
        assert abs(mon["Mesure/Mass_%d" % n][0] - 4 * PI) < 1e-11
        assert abs(mon["Mesure/Ekin_%d" % n][0] - 2 * PI) < 1e-11
        assert abs(mon["Mesure/Emode1_%d" % n][0] - 0.05) < 1e-12


def test_vlasov_sampled_outputs_mixed_form(tmp_path):
    """The mixed form's sampled outputs (fixed-point composition through the FP32 stack) against
    the plain FP64 form's after a run with remaps."""
    import os
    ic, bounds = CASES["two_stream"]
    n = 64
    res = {}
    for prec in ("fp64", "mixed"):
        work = tmp_path / prec
        work.mkdir()
        args = _args(work, ic, bounds, precision=prec)
        m = cmm()
        sim = m.Simulation(_with_sample(work, args, "{is_instant=1,time_start=2,var=Dist Map_b,grid=%d}" % n))
        sim.init()
        sim.run()
        run = os.path.join(str(work), "data", sim.file_name())
        sim.close()
        res[prec] = (_sample_files(run, n), read_monitoring(run))
    (fp, mp), (fm, mm) = res["fp64"], res["mixed"]
    assert len(fp) == len(fm) == 1
    a, b = list(fp.values())[0], list(fm.values())[0]
    assert set(a) == set(b) == {"Map_ChiX", "Map_ChiY", "Distribution_F"}
    lx, ly = _periods(bounds)
    assert wrap_err(b["Map_ChiX"], a["Map_ChiX"], lx) < 1e-5 and wrap_err(b["Map_ChiY"], a["Map_ChiY"], ly) < 1e-5
    assert np.max(np.abs(b["Distribution_F"] - a["Distribution_F"])) <= 1e-5 * np.max(np.abs(a["Distribution_F"]))
    for key in ("Mass", "Ekin"):
        x, y = mp["Mesure/%s_%d" % (key, n)][0], mm["Mesure/%s_%d" % (key, n)][0]
        assert abs(y - x) <= 1e-6 * abs(x), key


def test_vlasov_golden_initial_state_through_param_file(tmp_path):
    """The reference's Vlasov parameter file with grid_psi raised to the vort
    grid (the current reference rejects its own 256 < 512): the t = 0
    monitoring rows that do not depend on the potential match the golden."""
    m = cmm()
    g = goldens()["vlasov_15"]
    pf = tmp_path / "params.txt"
    pf.write_text(g["params_in"])
    sim = m.Simulation(["param_file=%s" % pf, "workspace=%s/" % tmp_path, "grid_psi=512", "final_time=0"])
    sim.init()
    sim.run()
    import os
    got = read_monitoring(os.path.join(str(tmp_path), "data", sim.file_name()))
    sim.close()
    from test_oracle_golden import RTOL, VLASOV_T0_KEYS
    first = {k: [got[k][0]] for k in VLASOV_T0_KEYS if k in got}
    gold = {k: [g["files"][k][0]] for k in VLASOV_T0_KEYS}
    worst, fails = compare_series(first, gold, VLASOV_T0_KEYS, RTOL)
    assert len(worst) == len(VLASOV_T0_KEYS)
    assert not fails, fails


def test_vlasov_rejects_vort_grid_finer_than_psi_grid(tmp_path):
    m = cmm()
    sim = m.Simulation(_args(tmp_path, "landau_damping", "{0,4,-2.5,2.5}", psi=64, vort=128))
    with pytest.raises(m.CmmError) as e:
        sim.init()
    assert e.value.code == m.CMM_ERR_PARAM
    sim.close()


def test_vlasov_kernel_api_matches_oracle():
    """cmm_compose_stack_var (distribution function), cmm_vlasov_potential and
    cmm_vlasov_diagnostics on caller-owned device buffers, against the oracle,
    on a map deformed by six oracle steps."""
    from test_gpu_parity import dev, host
    m = cmm()
    b = (0.0, 4 * PI, -2.5 * PI, 2.5 * PI)
    cfg = dict(grid_coarse=32, grid_fine=64, grid_psi=64, grid_vort=64, bounds=list(b), dt=1.0 / 32,
               time_integration_num=30, lagrange_order=3, lagrange_init_higher_order=1, map_update_order_num=1,
               map_epsilon=1e-3, incomp_threshold=1.0, skip_remapping=1, molly_stencil=0, freq_cut_psi=32.0,
               initial_condition_num=0, max_maps=4, particles=[], simulation_type_num=2)
    o = O.EulerOracle(cfg)
    o.init()
    for _ in range(6):
        o.step(cfg["dt"])
    chix, chiy, f_fine = o.chix(), o.chiy(), o.vort_fine()
    go = {n: O.make_grid(n, b) for n in (32, 64)}
    gq = {n: m.grid(n, b) for n in (32, 64)}
    out = dev(np.zeros(64 * 64))
    m.compose_stack_var(gq[32], gq[64], dev(chix), dev(chiy), None, 0, 2, 0, out)
    ref = O.compose_sample(chix, chiy, None, 0, go[32], go[64], 0, var_num=2)
    assert rel_linf(host(out), ref) < 1e-12
    vp = m.VlasovPotential(gq[64], gq[64])
    psi = dev(np.zeros(4 * 64 * 64))
    vp.potential(gq[32], gq[64], dev(chix), dev(chiy), dev(f_fine), psi)
    ref_psi = O.vlasov_potential(chix, chiy, f_fine, go[32], go[64], go[64], go[64])
    assert herm_err(host(psi), ref_psi, 64) < 1e-12
    d = vp.diagnostics(gq[32], dev(o.vort()), dev(ref_psi))
    r = O.vlasov_mesure(o.vort(), go[32], ref_psi, go[64])
    for k in range(9):
        # relative, with the mass as the scale of the cancelling momentum sum
        assert abs(d[k] - r[k]) <= 1e-12 * max(abs(r[k]), abs(r[3])), k
    vp.close()
