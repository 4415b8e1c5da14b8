"""Restart from a stored map stack on the GPU (save_map_stack, restart_time,
restart_location).

The reference writes a MapStack folder at every remap and at the end of a run
(writeMapStack / writeParticlesState, src/ui/cmm-io.cu:611-657) and restarts
from it (readMapStack, src/simulation/cmm-simulation-host.cu:1256-1302; the
restart branch of src/simulation/cmm-euler2d.cu:634-715).  Checked here:

* the reference's own restart test (tests/euler2D_remap: params-1 to t = 1,
  params-2 restarts to t = 2) through the CLI interface against its goldens;
* the files a plain FP64 run writes against the oracle's restatement of the
  same files (maps, the psi history with its level-0 copies, tracers);
* a restarted plain run against the oracle restarted from the same files,
  step by step (Euler and Vlasov-Poisson);
* the mixed form restarting from FP64 files, and writing files a plain run
  restarts from;
* the reported errors for a missing folder and for a stack larger than
  mem_RAM_CPU_remaps allows.

Tolerances as in test_gpu_parity.py (map_err, rel_linf) and test_gpu_vlasov.py
(einc_tol).
"""
import os

import numpy as np
import pytest

import oracle as O
import refloop
from goldens import compare_series, goldens
from oracle_adapter import OracleRun
from product import cmm, read_monitoring
from test_gpu_parity import map_err, rel_linf
from test_gpu_vlasov import einc_tol

pytestmark = pytest.mark.gpu
TWO_PI = 2 * np.pi
TRACERS = ("{num=500,tau=0,seed=3,time_integration=RK3,init_name=uniform,init_time=0,init_vel=0,"
           "init_param_1=3.141592653589793,init_param_2=3.141592653589793,init_param_3=6.283185307179586,"
           "init_param_4=6.283185307179586}")


def _param_text(final_time, restart_time=0.0, save=1, precision="fp64", threshold=1e-5):
    # 4_nodes on a 64^2 map (fine = vort 256, psi 128), dt = 1/64, 500 tracers
    kv = [("simulation_type", "cmm_euler_2d"), ("sim_name", "rs"), ("initial_condition", "4_nodes"),
          ("grid_coarse", "64"), ("grid_fine", "256"), ("grid_vort", "256"), ("grid_psi", "128"),
          ("set_dt_by_steps", "1"), ("steps_per_sec", "64"), ("final_time", repr(final_time)),
          ("time_integration", "RK3"), ("map_update_order", "4th"), ("map_epsilon", "0.001"),
          ("incomp_threshold", repr(threshold)), ("skip_remapping", "0"), ("molly_stencil", "0"),
          ("lagrange_init_higher_order", "1"), ("lagrange_override", "-1"), ("freq_cut_psi", "64"),
          ("mem_RAM_CPU_remaps", "100"), ("save_map_stack", str(save)), ("restart_time", repr(restart_time)),
          ("save_computational_num", "0"), ("save_sample_num", "0"), ("save_zoom_num", "0"), ("forward_map", "0"),
          ("verbose", "0"), ("precision", precision)]
    lines = ["CMM Parameter file", "param_version\t=\t3", ""] + ["%s\t=\t%s" % p for p in kv]
    lines += ["particles_advected_num\t=\t1", "particles_advected\t=\t" + TRACERS]
    return "\n".join(lines) + "\n"


def _sim(tmp, text, cli=()):
    m = cmm()
    pf = os.path.join(str(tmp), "params_%d.txt" % len(os.listdir(str(tmp))))
    with open(pf, "w") as f:
        f.write(text)
    return m.Simulation(["param_file=%s" % pf, "workspace=%s/" % tmp] + list(cli))


def _oracle(text, restart_files=None, cli=()):
    s = refloop.settings_from_param_text(text, cli)
    return OracleRun(s, restart_files=restart_files), s


def _first_run(tmp, precision="fp64"):
    """A run to t = 0.5 that writes its MapStack; returns (sim, folder)."""
    sim = _sim(tmp, _param_text(0.5, precision=precision))
    sim.init()
    sim.run()
    return sim, os.path.join(str(tmp), "data", sim.file_name(), "MapStack")


def _wrap_diff(a, b):
    d = np.abs(np.asarray(a) - np.asarray(b))
    return float(np.max(np.minimum(d, TWO_PI - d)))


def test_restart_golden_through_the_cli_interface(tmp_path):
    """The reference's restart test: its params-1 run writes the MapStack folder,
    its params-2 run restarts from it; the restarted run's monitoring files match
    the goldens (3 maps loaded, the remap steps, E_inc per step, the t = 1 and t = 2
    statistics of map, psi, vorticity, the fluid tracers and the inertial set with
    its velocity state read back from the folder)."""
    m = cmm()
    g = goldens()["restart_remap"]
    p1, p2 = tmp_path / "params-1.txt", tmp_path / "params-2.txt"
    p1.write_text(g["params_pre"])
    p2.write_text(g["params_in"])
    sim = m.Simulation(["param_file=%s" % p1, "workspace=%s/" % tmp_path])
    sim.init()
    sim.run()
    stack_dir = os.path.join(str(tmp_path), "data", sim.file_name(), "MapStack")
    names = sorted(os.listdir(stack_dir))
    assert [n for n in names if n.startswith("Map_ChiX_H")] == ["Map_ChiX_H_0.data", "Map_ChiX_H_1.data",
                                                               "Map_ChiX_H_2.data", "Map_ChiX_H_coarse.data"]
    sim.close()
    sim = m.Simulation(["param_file=%s" % p2, "workspace=%s/" % tmp_path, "restart_location=%s" % stack_dir])
    sim.init()
    sim.run()
    run_dir = os.path.join(str(tmp_path), "data", sim.file_name())
    ours = read_monitoring(run_dir)
    keys = list(g["files"])
    worst, fails = compare_series(ours, g["files"], keys, 1e-9)
    assert len(worst) >= 60
    assert not fails, fails
    assert ours["Map_counter"] == g["files"]["Map_counter"]
    log = open(os.path.join(run_dir, "log.txt")).read()
    assert log.startswith("\nContinuing simulation\n")


def test_map_stack_files_match_the_oracle(tmp_path):
    """A plain FP64 run to t = 0.5 with remaps: every file of its MapStack folder
    against the oracle's restatement of writeMapStack after the same run (the
    oracle starts from the GPU's cuRAND tracer positions)."""
    text = _param_text(0.5)
    sim = _sim(tmp_path, text)
    sim.init()
    p0 = sim.field("Particles_advected_pos_P01").copy()
    sim.run()
    stack_dir = os.path.join(str(tmp_path), "data", sim.file_name(), "MapStack")
    files = O.read_map_stack_dir(stack_dir)
    run, s = _oracle(text)
    run.particle_init = {0: p0}
    refloop.run_reference_loop(s, run, lambda t, dt: None)
    ref = O.map_stack_files(run.o)
    assert sorted(files) == sorted(ref)
    n = sum(1 for k in ref if k.startswith("Map_ChiX_H_")) - 1
    assert n >= 2
    for k in ref:
        assert files[k].shape == ref[k].shape, k
        if k.startswith("Map_"):
            assert map_err(files[k], ref[k]) < 1e-10, k
        elif k.startswith("Stream"):
            assert rel_linf(files[k], ref[k]) < 1e-10, k
        else:
            assert _wrap_diff(files[k], ref[k]) < 1e-10, k
    # the reference's psi history: level 0 under every level's name
    np.testing.assert_array_equal(files["Stream_function_Psi_H_psi_1"], files["Stream_function_Psi_H_psi_2"])


def test_restart_matches_the_oracle_restart(tmp_path):
    """Restart at t = 0.5 from the files of a plain run, on to t = 1: the GPU and
    the oracle, both restarted from the same files, agree step by step."""
    _, stack_dir = _first_run(tmp_path)
    files = O.read_map_stack_dir(stack_dir)
    text = _param_text(1.0, restart_time=0.5, save=0)
    sim = _sim(tmp_path, text, ["restart_location=%s" % stack_dir])
    sim.init()
    run, s = _oracle(text, restart_files=files)
    run.init()
    o = run.o
    assert sim.scalar("map_counter") == o.map_count() == run.loaded_maps
    assert map_err(sim.field("Map_ChiX_H_coarse"), o.chix()) < 1e-12
    assert rel_linf(sim.field("Stream_function_Psi_H_psi"), o.psi()) < 1e-10
    assert rel_linf(sim.field("Vorticity_W_coarse"), o.vort()) < 1e-10
    tol = einc_tol(TWO_PI, TWO_PI / 64)
    steps = 0
    while sim.step(1) != 1:
        _, e, _ = o.step(1.0 / 64)
        assert abs(sim.scalar("e_inc") - e) < tol
        assert sim.scalar("map_counter") == o.map_count()
        steps += 1
    assert steps == 32
    assert abs(sim.scalar("time") - 1.0) < 1e-12
    assert map_err(sim.field("Map_ChiX_H_coarse"), o.chix()) < 1e-10
    assert map_err(sim.field("Map_ChiY_H_coarse"), o.chiy()) < 1e-10
    assert rel_linf(sim.field("Stream_function_Psi_H_psi"), o.psi()) < 1e-10
    assert _wrap_diff(sim.field("Particles_advected_pos_P01"), o.particles(0)) < 1e-10
    for name, ref in (("energy", o.energy()), ("enstrophy", o.enstrophy())):
        assert abs(sim.scalar(name) - ref) <= 1e-11 * abs(ref), name


def test_mixed_form_restarts_from_fp64_files_and_writes_restartable_files(tmp_path):
    """The mixed form reads the FP64 planar files (maps become FP32 displacements,
    tracers 64-bit fixed point) and continues like the plain restart to the mixed
    form's accuracy; the files it writes are its state in the reference layout and
    restart a plain run.  The restarted runs remap at 1e-3: on this 64^2 map with
    dt = 1/64 the FP32 rounding of E_inc is ~1e-4."""
    (tmp_path / "a").mkdir()
    _, stack_dir = _first_run(tmp_path / "a")
    runs = {}
    for prec in ("fp64", "mixed"):
        sim = _sim(tmp_path, _param_text(1.0, restart_time=0.5, save=0, precision=prec, threshold=1e-3),
                   ["restart_location=%s" % stack_dir, "sim_name=rs_%s" % prec])
        sim.init()
        assert sim.scalar("map_counter") >= 2
        sim.run()
        runs[prec] = sim
    for name in ("energy", "enstrophy", "palinstrophy"):
        a, b = runs["fp64"].scalar(name), runs["mixed"].scalar(name)
        assert abs(a - b) <= 1e-5 * abs(a), name
    assert _wrap_diff(runs["fp64"].field("Particles_advected_pos_P01"),
                      runs["mixed"].field("Particles_advected_pos_P01")) < 1e-4
    # a mixed run writing its own folder: its state in the reference layout
    (tmp_path / "b").mkdir()
    sim = _sim(tmp_path / "b", _param_text(0.5, precision="mixed", threshold=1e-3))
    sim.init()
    sim.run()
    stack_m = os.path.join(str(tmp_path / "b"), "data", sim.file_name(), "MapStack")
    fm = O.read_map_stack_dir(stack_m)
    n = int(sim.scalar("map_counter"))
    assert sum(1 for k in fm if k.startswith("Map_ChiX_H_")) == n + 1
    np.testing.assert_array_equal(fm["Map_ChiX_H_coarse"], sim.field("Map_ChiX_H_coarse"))
    np.testing.assert_array_equal(fm["Map_ChiY_H_coarse"], sim.field("Map_ChiY_H_coarse"))
    np.testing.assert_array_equal(fm["Stream_function_Psi_H_psi_1"], sim.field("Stream_function_Psi_H_psi"))
    np.testing.assert_array_equal(fm["Particles_advected_pos_P01"], sim.field("Particles_advected_pos_P01"))
    if n:
        st = sim.field("Map_stack").reshape(n, 2, -1)
        for i in range(n):
            np.testing.assert_array_equal(fm["Map_ChiX_H_%d" % i], st[i, 0])
    sims = {}
    for prec in ("fp64", "mixed"):
        sims[prec] = _sim(tmp_path / "b", _param_text(1.0, restart_time=0.5, save=0, precision=prec, threshold=1e-3),
                          ["restart_location=%s" % stack_m, "sim_name=rb_%s" % prec])
        sims[prec].init()
        assert sims[prec].scalar("map_counter") == n
        sims[prec].run()
    a, b = sims["fp64"].scalar("enstrophy"), sims["mixed"].scalar("enstrophy")
    assert abs(a - b) <= 1e-5 * abs(a)


def test_mixed_form_forward_map_writes_and_restarts(tmp_path):
    """precision=mixed with forward_map=1: the MapStack folder holds the FP64 forward map and
    one forward sub-map per remap beside the backward ones, equal to the run's state; both
    forms restart from it at t = 1 with that forward map: over a window without remaps their
    forward maps agree to the FP32 psi's rounding, and to t = 1.5 with remaps (at 5e-4, above
    the FP32 maps' ~1e-4 of E_inc on this 64^2 map) their enstrophy agrees."""
    text = _param_text(1.0, precision="mixed", threshold=5e-4).replace("forward_map\t=\t0", "forward_map\t=\t1")
    (tmp_path / "a").mkdir()
    sim = _sim(tmp_path / "a", text)
    sim.init()
    sim.run()
    n = int(sim.scalar("map_counter"))
    assert n >= 1
    stack_dir = os.path.join(str(tmp_path / "a"), "data", sim.file_name(), "MapStack")
    files = O.read_map_stack_dir(stack_dir)
    assert sum(1 for k in files if k.startswith("Map_ChiX_f_H_") and k != "Map_ChiX_f_H_coarse") == n
    fx, fy = sim.field("Map_ChiX_f_H_coarse").copy(), sim.field("Map_ChiY_f_H_coarse").copy()
    np.testing.assert_array_equal(files["Map_ChiX_f_H_coarse"], fx)
    np.testing.assert_array_equal(files["Map_ChiY_f_H_coarse"], fy)
    sim.close()
    ends = {}
    for prec in ("fp64", "mixed"):
        # a window with no remap (threshold 1): both forms advect the restarted forward map over
        # the same 16 steps, so their forward maps differ only by the mixed form's FP32 psi
        wtext = _param_text(1.25, restart_time=1.0, save=0, precision=prec, threshold=1.0).replace(
            "forward_map\t=\t0", "forward_map\t=\t1")
        r = _sim(tmp_path, wtext, ["restart_location=%s" % stack_dir, "sim_name=rw_%s" % prec])
        r.init()
        assert int(r.scalar("map_counter")) == n
        np.testing.assert_array_equal(r.field("Map_ChiX_f_H_coarse"), fx)
        r.run()
        assert int(r.scalar("map_counter")) == n
        ends[prec] = r.field("Map_ChiX_f_H_coarse").copy()
        r.close()
    xp, xm = ends["fp64"], ends["mixed"]
    assert np.max(np.abs(xm[: xm.size // 4] - xp[: xp.size // 4])) < 1e-4
    # and with remaps to t = 1.5: the forward maps there depend on the steps at which each form
    # remapped (a step apart is u dt ~ 1e-2 apart), so the conserved quantities are compared
    ends = {}
    for prec in ("fp64", "mixed"):
        rtext = _param_text(1.5, restart_time=1.0, save=0, precision=prec, threshold=5e-4).replace(
            "forward_map\t=\t0", "forward_map\t=\t1")
        r = _sim(tmp_path, rtext, ["restart_location=%s" % stack_dir, "sim_name=rf_%s" % prec])
        r.init()
        r.run()
        ends[prec] = (int(r.scalar("map_counter")), r.scalar("enstrophy"))
        r.close()
    (cp, zp), (cm, zm) = ends["fp64"], ends["mixed"]
    assert cp > n and cm > n
    assert abs(zm - zp) <= 1e-5 * abs(zp)


def test_restart_reports_missing_files_and_oversized_stacks(tmp_path):
    m = cmm()
    empty = tmp_path / "nothing"
    empty.mkdir()
    sim = _sim(tmp_path, _param_text(1.0, restart_time=0.5, save=0), ["restart_location=%s" % empty])
    with pytest.raises(m.CmmError) as e:
        sim.init()
    assert e.value.code == m.CMM_ERR_IO
    assert "Map_ChiX_H_coarse.data" in str(e.value)
    sim.close()
    _, stack_dir = _first_run(tmp_path)
    n = len([f for f in os.listdir(stack_dir) if "Map_ChiX_H" in f]) - 1
    # capacity int(mem / map size) with a 64^2 map of 0.262 MB: room for n - 1 maps
    mem = 0.262144 * (n - 1) + 0.1
    sim = _sim(tmp_path, _param_text(1.0, restart_time=0.5, save=0),
               ["restart_location=%s" % stack_dir, "mem_RAM_CPU_remaps=%r" % mem])
    with pytest.raises(m.CmmError) as e:
        sim.init()
    assert e.value.code == m.CMM_ERR_PARAM


def test_vlasov_restart_matches_the_oracle_restart(tmp_path):
    """Vlasov-Poisson (landau_damping, 64^2 map, 128^2 fine and psi): a plain run to
    t = 1 writes its MapStack, then the GPU and the oracle restart from it to t = 2."""
    from test_gpu_vlasov import _args
    base = [a for a in _args(tmp_path, "landau_damping", "{0,4,-2.5,2.5}", final_time=1.0, threshold=1e-5)
            if not a.startswith("workspace")]
    m = cmm()
    sim = m.Simulation(["workspace=%s/" % tmp_path] + base + ["save_map_stack=1"])
    sim.init()
    sim.run()
    stack_dir = os.path.join(str(tmp_path), "data", sim.file_name(), "MapStack")
    files = O.read_map_stack_dir(stack_dir)
    assert sum(1 for k in files if k.startswith("Map_ChiX_H_")) >= 2
    cli = base + ["final_time=2", "restart_time=1", "restart_location=%s" % stack_dir, "save_map_stack=0"]
    s = refloop.Settings()
    for a in cli:
        s.set_variable(a, "=")
    s.finalize()
    run = OracleRun(s, restart_files=files)
    run.init()
    o = run.o
    sim = m.Simulation(["workspace=%s/" % tmp_path] + cli + ["sim_name=vr_fp64"])
    sim.init()
    assert sim.scalar("map_counter") == run.loaded_maps
    tol = einc_tol(2.5 * np.pi, 4 * np.pi / 64)
    steps = 0
    while sim.step(1) != 1:
        _, e, _ = o.step(s.dt)
        assert abs(sim.scalar("e_inc") - e) < tol
        assert sim.scalar("map_counter") == o.map_count()
        steps += 1
    assert steps == 32
    mo = o.vlasov_mesure()
    plain = {k: sim.scalar(k) for k in ("etot", "ekin", "mass")}
    for k, ref in (("etot", mo["Etot"]), ("ekin", mo["Ekin"]), ("mass", mo["Mass"])):
        assert abs(plain[k] - ref) <= 1e-10 * abs(ref), k
    assert map_err(sim.field("Map_ChiX_H_coarse"), o.chix()) < 1e-10
    assert rel_linf(sim.field("Stream_function_Psi_H_psi"), o.psi()) < 1e-10
    sim.close()
    # the mixed form from the same FP64 files (phi levels taken from the stored psi planes)
    sim = m.Simulation(["workspace=%s/" % tmp_path] + cli + ["precision=mixed", "sim_name=vr_mixed"])
    sim.init()
    sim.run()
    for k in ("etot", "ekin", "mass"):
        assert abs(sim.scalar(k) - plain[k]) <= 1e-6 * abs(plain[k]), k
