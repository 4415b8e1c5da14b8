"""Ensembles of uneven-size runs advanced together (cmm_ensemble_*).

Each member of an ensemble runs the single-member kernels' device bodies on its own
descriptor, and the psi solve transforms every member of a size class in one batched
transform (the library's FFT).  The batched kernels are separate instantiations of those bodies (their
arguments come from shared memory rather than the parameter space), so the compiler
may contract and share FP32 products differently: a member agrees with its single run
to FP32 rounding, not bit for bit (one step moves the map's cross-derivative plane, whose
conditioning is 1/eps^2, by a few FP32 ulps).  Checked here, for the single-launch iteration and the
two-phase one: every member's map (in units of its conditioning), psi and coarse vorticity
after a run without remaps against the member run alone, with and without the CUDA graphs; a
run with remaps (counts within one, conserved quantities to 1e-6); the two iterations against
each other through remaps; the members' conserved quantities against plain FP64 runs; the
autotuner's table and the graph replay; a grid barrier made to give up (CMM_ERR_TIMEOUT, the
context usable afterwards); and the members the ensemble rejects or keeps on the two-phase path.
"""
import os

import numpy as np
import pytest

from product import cmm, read_monitoring

pytestmark = pytest.mark.gpu
TWO_PI = 2 * np.pi
SIZES = [32, 48, 64, 32, 96, 48, 64]


def random_vorticity(n, seed, k0):
    """Random-phase field with E(k) ~ k^4 exp(-(k/k0)^2), unit enstrophy Z = 1/2 hx hy sum w^2."""
    rng = np.random.default_rng(seed)
    kx = np.fft.rfftfreq(n, 1.0 / n)
    ky = np.fft.fftfreq(n, 1.0 / n)
    k = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    ek = k ** 4 * np.exp(-(k / k0) ** 2)
    amp = np.zeros_like(k)
    nz = k > 0
    amp[nz] = np.sqrt(k[nz] ** 2 * ek[nz] / (2 * np.pi * k[nz]))
    w = np.fft.irfft2(amp * np.exp(1j * rng.uniform(0.0, 2 * np.pi, size=k.shape)), s=(n, n))
    h = TWO_PI / n
    return np.ascontiguousarray(w / np.sqrt(0.5 * h * h * np.sum(w * w)))


def member_args(tmp, i, n, precision="mixed", final_time=0.5, threshold=1e-3):
    # N / 4N / 2N grids (map / fine = vort / psi), dt = 1 / (N / 2).  At 1e-4 members this small
    # remap on most steps (in plain FP64 as in the mixed form); 1e-3 keeps a few remaps per run
    return ["workspace=%s/" % tmp, "sim_name=m%02d" % i, "simulation_type=cmm_euler_2d",
            "grid_coarse=%d" % n, "grid_fine=%d" % (4 * n), "grid_vort=%d" % (4 * n), "grid_psi=%d" % (2 * n),
            "set_dt_by_steps=1", "steps_per_sec=%d" % (n // 2), "final_time=%r" % final_time,
            "initial_condition=4_nodes", "initial_discrete=1", "initial_discrete_grid=%d" % (4 * n),
            "time_integration=RK3", "map_update_order=4th", "map_epsilon=0.001", "incomp_threshold=%r" % threshold,
            "skip_remapping=0", "molly_stencil=0", "freq_cut_psi=%d" % n, "lagrange_init_higher_order=1",
            "mem_RAM_CPU_remaps=400", "save_computational_num=0", "save_sample_num=0", "save_zoom_num=0",
            "forward_map=0", "particles_advected_num=0", "save_map_stack=0", "verbose=0",
            "precision=%s" % precision]


def fields(get):
    return [get("Map_ChiX_H_coarse"), get("Map_ChiY_H_coarse"), get("Stream_function_Psi_H_psi"),
            get("Vorticity_W_coarse")]


def _close(a, b, tol):
    return float(np.max(np.abs(a - b))) <= tol * max(1e-300, float(np.max(np.abs(b))))


def _same_run(get_a, get_b, scalar_a, scalar_b):
    """Two runs of one member through different batched paths.  E_inc is a cancellation-prone
    determinant deviation whose FP32 rounding differs between kernel builds by up to ~1e-2
    relative, so a check that lands within that of incomp_threshold may remap in one run and not
    in the other: then the remap counts differ by one and the conserved quantities by the remap
    error (1e-5); otherwise the fields agree to FP32 rounding.  Returns the remap count."""
    from test_gpu_parity import map_err
    a, b = int(scalar_a("map_counter")), int(scalar_b("map_counter"))
    assert abs(a - b) <= 1, (a, b)
    tol = 1e-6 if a == b else 1e-5
    for name in ("energy", "enstrophy"):
        assert abs(scalar_a(name) - scalar_b(name)) <= tol * abs(scalar_b(name)), (name, a, b)
    if a == b:
        mx, my, psi, w = fields(get_a)
        mx1, my1, psi1, w1 = fields(get_b)
        assert map_err(mx, mx1) < 1e-5 and map_err(my, my1) < 1e-5
        assert _close(psi, psi1, 1e-5) and _close(w, w1, 1e-5)
    return a


@pytest.mark.parametrize("graphs,fused", [(True, True), (False, True), (True, False), (False, False)])
def test_ensemble_members_equal_their_single_runs(tmp_path, graphs, fused):
    from test_gpu_parity import map_err
    m = cmm()
    (tmp_path / "e").mkdir()
    (tmp_path / "s").mkdir()
    ics = [random_vorticity(4 * n, seed=i, k0=3.0 + i) for i, n in enumerate(SIZES)]
    ens = m.Ensemble([member_args(tmp_path / "e", i, n, threshold=1.0) for i, n in enumerate(SIZES)], graphs=graphs,
                     fused=fused)
    for i, w in enumerate(ics):
        ens.set_initial_discrete(i, w)
    ens.init()
    info = ens.fused_info()
    assert info["available"] == fused and info["fused"] == fused, info
    ens.run()
    if fused:
        assert ens.stats()["launches"] == ens.stats()["iterations"]   # one kernel launch per iteration
        assert ens.fused_info()["waves"] == 6   # advect, check, sample, rows, columns, inverse rows
    st = ens.stats()
    assert st["member_steps"] == sum(int(0.5 * n / 2) for n in SIZES)
    assert st["iterations"] == max(int(0.5 * n / 2) for n in SIZES)
    for i, n in enumerate(SIZES):
        sim = m.Simulation(member_args(tmp_path / "s", i, n, threshold=1.0))
        sim.set_initial_discrete(ics[i])
        sim.init()
        sim.run()
        assert ens.scalar(i, "time") == sim.scalar("time")
        assert ens.scalar(i, "map_counter") == sim.scalar("map_counter") == 0
        mx, my, psi, w = fields(lambda k: ens.field(i, k))
        mx1, my1, psi1, w1 = fields(sim.field)
        assert map_err(mx, mx1) < 1e-5 and map_err(my, my1) < 1e-5, i
        assert _close(psi, psi1, 1e-5) and _close(w, w1, 1e-5), i
        for name in ("energy", "enstrophy"):
            assert abs(ens.scalar(i, name) - sim.scalar(name)) <= 1e-6 * abs(sim.scalar(name)), (i, name)
        sim.close()
    ens.close()


@pytest.mark.parametrize("fused", [True, False])
def test_ensemble_members_remap_like_their_single_runs(tmp_path, fused):
    m = cmm()
    (tmp_path / "e").mkdir()
    (tmp_path / "s").mkdir()
    ics = [random_vorticity(4 * n, seed=i, k0=3.0 + i) for i, n in enumerate(SIZES)]
    ens = m.Ensemble([member_args(tmp_path / "e", i, n, final_time=1.0) for i, n in enumerate(SIZES)], fused=fused)
    for i, w in enumerate(ics):
        ens.set_initial_discrete(i, w)
    ens.init()
    ens.run()
    remaps = 0
    for i, n in enumerate(SIZES):
        sim = m.Simulation(member_args(tmp_path / "s", i, n, final_time=1.0))
        sim.set_initial_discrete(ics[i])
        sim.init()
        sim.run()
        a, b = int(ens.scalar(i, "map_counter")), int(sim.scalar("map_counter"))
        assert abs(a - b) <= 1, (i, a, b)
        mon_e = {k: np.asarray(v) for k, v in
                 read_monitoring(os.path.join(str(tmp_path / "e"), "data", sim.file_name())).items()}
        mon_s = {k: np.asarray(v) for k, v in
                 read_monitoring(os.path.join(str(tmp_path / "s"), "data", sim.file_name())).items()}
        for key in ("Time_s", "Error_incompressibility", "Map_gaps", "Map_counter"):
            assert mon_e[key].shape == mon_s[key].shape, (i, key)
        assert np.array_equal(mon_e["Time_s"], mon_s["Time_s"]), i
        assert mon_e["Map_counter"][-1] == a
        remaps += a
        tol = 1e-6 if a == b else 1e-5   # a check at the threshold can flip (see _same_run)
        for name in ("energy", "enstrophy"):
            assert abs(ens.scalar(i, name) - sim.scalar(name)) <= tol * abs(sim.scalar(name)), (i, name)
        sim.close()
    assert remaps >= 3
    ens.close()


def test_ensemble_members_follow_plain_fp64(tmp_path):
    m = cmm()
    sizes = [32, 64, 96]
    ics = [random_vorticity(4 * n, seed=10 + i, k0=4.0) for i, n in enumerate(sizes)]
    ens = m.Ensemble([member_args(tmp_path, i, n, final_time=1.0) for i, n in enumerate(sizes)])
    for i, w in enumerate(ics):
        ens.set_initial_discrete(i, w)
    ens.init()
    ens.run()
    for i, n in enumerate(sizes):
        sim = m.Simulation(member_args(tmp_path, 10 + i, n, precision="fp64", final_time=1.0))
        sim.set_initial_discrete(ics[i])
        sim.init()
        sim.run()
        for name in ("energy", "enstrophy", "palinstrophy"):
            a, b = ens.scalar(i, name), sim.scalar(name)
            assert abs(a - b) <= 1e-5 * abs(b), (i, name, a, b)
        sim.close()


def test_ensemble_rejects_members_it_cannot_batch(tmp_path):
    m = cmm()
    args = [member_args(tmp_path, 0, 32), member_args(tmp_path, 1, 32, precision="fp64")]
    ens = m.Ensemble(args)
    w = random_vorticity(128, 0, 3.0)
    ens.set_initial_discrete(0, w)
    ens.set_initial_discrete(1, w)
    with pytest.raises(m.CmmError) as e:
        ens.init()
    assert e.value.code == m.CMM_ERR_UNSUPPORTED
    assert "member 1" in str(e.value)


def test_fused_iteration_equals_two_phase_with_remaps(tmp_path):
    """The single-launch iteration (device-side remap decision, batched remaps) against the
    two-phase one (remaps on the host): the same remap steps and fields to FP32 rounding."""
    m = cmm()
    sizes = [32, 48, 64]
    ics = [random_vorticity(4 * n, seed=20 + i, k0=5.0) for i, n in enumerate(sizes)]
    runs = []
    for fused in (True, False):
        d = tmp_path / ("f" if fused else "t")
        d.mkdir()
        ens = m.Ensemble([member_args(d, i, n, final_time=1.0) for i, n in enumerate(sizes)], fused=fused)
        for i, w in enumerate(ics):
            ens.set_initial_discrete(i, w)
        ens.init()
        ens.run()
        runs.append((d, ens))
    (df, ef), (dt, et) = runs
    remaps = 0
    for i, n in enumerate(sizes):
        a = _same_run(lambda k: ef.field(i, k), lambda k: et.field(i, k), lambda k: ef.scalar(i, k),
                      lambda k: et.scalar(i, k))
        remaps += a
        if a == int(et.scalar(i, "map_counter")):
            name = "m%02d" % i
            mon = [[read_monitoring(os.path.join(str(d), "data", p)) for p in os.listdir(os.path.join(str(d), "data"))
                    if p.startswith(name)][0] for d in (df, dt)]
            assert np.array_equal(np.asarray(mon[0]["Map_gaps"]), np.asarray(mon[1]["Map_gaps"])), i
    assert remaps >= 3
    ef.close()
    et.close()


def test_autotuner_picks_the_fastest_form_and_shape(tmp_path):
    """The autotuner times every single-launch shape (register budget, blocks, tiles per task) and
    the two-phase iteration with batched remaps on live iterations, keeps the fastest, and the run
    equals the single-launch run (same remaps, fields to FP32 rounding) whichever it picked."""
    m = cmm()
    sizes = [32, 64, 48]
    ics = [random_vorticity(4 * n, seed=30 + i, k0=5.0) for i, n in enumerate(sizes)]
    runs = []
    for fused in (None, True):
        d = tmp_path / ("auto" if fused is None else "one")
        d.mkdir()
        ens = m.Ensemble([member_args(d, i, n, final_time=3.0) for i, n in enumerate(sizes)], fused=fused)
        for i, w in enumerate(ics):
            ens.set_initial_discrete(i, w)
        ens.init()
        ens.run()
        runs.append(ens)
    auto, one = runs
    table = auto.tuning()
    info = auto.fused_info()
    assert info["available"] and len(table) >= 4, table
    assert 0 in {r[0] for r in table} and 4 in {r[0] for r in table}, table
    best = min(table, key=lambda r: r[3])
    assert (info["register_budget"], info["blocks"], info["tiles_per_task"]) == best[:3]
    assert info["fused"] == (best[0] != 0)
    assert all(r[3] > 0 for r in table)
    assert auto.stats()["iterations"] == int(3.0 * 64 / 2)
    for i in range(len(sizes)):
        _same_run(lambda k: auto.field(i, k), lambda k: one.field(i, k), lambda k: auto.scalar(i, k),
                  lambda k: one.scalar(i, k))
    auto.close()
    one.close()


def test_fused_barrier_wait_limit_times_out_and_context_survives(tmp_path):
    """A grid barrier that may poll zero times gives up (some block arrives before the last),
    the step reports CMM_ERR_TIMEOUT, the ensemble refuses further steps, and the CUDA context
    still runs a simulation afterwards."""
    m = cmm()
    sizes = [32, 48, 64]
    ics = [random_vorticity(4 * n, seed=40 + i, k0=4.0) for i, n in enumerate(sizes)]
    ens = m.Ensemble([member_args(tmp_path, i, n) for i, n in enumerate(sizes)], fused=True)
    for i, w in enumerate(ics):
        ens.set_initial_discrete(i, w)
    ens.init()
    assert ens.fused_info()["fused"]
    ens.step(1)   # a normal iteration first
    ens.set_wait_limit(0)
    with pytest.raises(m.CmmError) as e:
        ens.step(1)
    assert e.value.code == m.CMM_ERR_TIMEOUT, str(e.value)
    assert "gave up" in str(e.value)
    with pytest.raises(m.CmmError) as e2:
        ens.step(1)
    assert e2.value.code == m.CMM_ERR_STATE
    ens.close()
    (tmp_path / "after").mkdir()
    sim = m.Simulation(member_args(tmp_path / "after", 9, 32, final_time=0.25))
    sim.set_initial_discrete(ics[0])
    sim.init()
    sim.run()
    assert abs(sim.scalar("time") - 0.25) < 1e-12
    sim.close()


def test_fused_iteration_declines_what_it_cannot_run(tmp_path):
    """A member that writes its map stack at remaps keeps the ensemble on the two-phase path."""
    m = cmm()
    args = [member_args(tmp_path, 0, 32), member_args(tmp_path, 1, 32)]
    args[1] = [a if not a.startswith("save_map_stack=") else "save_map_stack=1" for a in args[1]]
    ens = m.Ensemble(args)
    w = random_vorticity(128, 0, 3.0)
    ens.set_initial_discrete(0, w)
    ens.set_initial_discrete(1, w)
    ens.init()
    info = ens.fused_info()
    assert not info["available"] and not info["fused"] and "member 1" in info["why"], info
    ens.step(2)
    ens.close()
