"""The remaining time integrators and inertial particles on the GPU, against the oracle.

Map advection (backward characteristics, src/numerical/cmm-timestep.cu): AB2 with
its ten fixed-point sweeps, RK4, RK3Mod and RK4Mod, including the order-4 Lagrange
initialisation that RK4 makes possible.  Particles (src/numerical/cmm-particles.cu):
fluid tracers with EulerExp, Heun, RK3, RK4, RK3Mod and RK4Mod, and inertial
particles (tau != 0) with the same six schemes, starting at rest or at the fluid
velocity, and with a start time inside the run (the velocity restarts there,
src/simulation/cmm-euler2d.cu:883-895).

Each case runs the plain FP64 product through its parameter-file interface and the
oracle on the same settings (the oracle starts from the product's initial particle
positions), and compares E_inc per step (in units of the map's conditioning), the
final map, psi and every particle set; the mixed form is compared with plain FP64.
"""
import os

import numpy as np
import pytest

import refloop
from oracle_adapter import OracleRun
from product import cmm, read_monitoring
from test_gpu_parity import herm_err, map_err, rel_linf
from test_gpu_vlasov import einc_tol

pytestmark = pytest.mark.gpu
TWO_PI = 2 * np.pi


def _record(num, tau, ti, init="uniform", init_time=0.0, init_vel=0, seed=1):
    return ("{num=%d,tau=%r,seed=%d,time_integration=%s,init_name=%s,init_time=%r,init_vel=%d,"
            "init_param_1=3.141592653589793,init_param_2=3.141592653589793,init_param_3=6.283185307179586,"
            "init_param_4=6.283185307179586}" % (num, tau, seed, ti, init, init_time, init_vel))


def _param_text(map_ti, records, final_time=0.25, precision="fp64", threshold=1e-5):
    # 4_nodes on a 64^2 map (fine = vort 128, psi 64), dt = 1/64, remaps at 1e-5
    kv = [("simulation_type", "cmm_euler_2d"), ("sim_name", "ti"), ("initial_condition", "4_nodes"),
          ("grid_coarse", "64"), ("grid_fine", "128"), ("grid_vort", "128"), ("grid_psi", "64"),
          ("set_dt_by_steps", "1"), ("steps_per_sec", "64"), ("final_time", repr(final_time)),
          ("time_integration", map_ti), ("map_update_order", "4th"), ("map_epsilon", "0.001"),
          ("incomp_threshold", repr(threshold)), ("skip_remapping", "0"), ("molly_stencil", "0"),
          ("lagrange_init_higher_order", "1"), ("lagrange_override", "-1"), ("freq_cut_psi", "32"),
          ("mem_RAM_CPU_remaps", "100"), ("save_map_stack", "0"), ("save_computational_num", "0"),
          ("save_sample_num", "0"), ("save_zoom_num", "0"), ("forward_map", "0"), ("verbose", "0"),
          ("precision", precision)]
    lines = ["CMM Parameter file", "param_version\t=\t3", ""] + ["%s\t=\t%s" % p for p in kv]
    lines.append("particles_advected_num\t=\t%d" % len(records))
    lines += ["particles_advected\t=\t" + r for r in records]
    return "\n".join(lines) + "\n"


def _wrap_diff(a, b):
    d = np.abs(np.asarray(a) - np.asarray(b))
    return float(np.max(np.minimum(d, TWO_PI - d)))


def _run_pair(tmp, text):
    """Plain FP64 product run and the oracle on the same settings -> (sim, oracle run, E_inc GPU, E_inc oracle)."""
    m = cmm()
    pf = os.path.join(str(tmp), "params.txt")
    with open(pf, "w") as f:
        f.write(text)
    sim = m.Simulation(["param_file=%s" % pf, "workspace=%s/" % tmp])
    sim.init()
    s = refloop.settings_from_param_text(text)
    p0 = {i: sim.field("Particles_advected_pos_P%02d" % (i + 1)).copy() for i in range(len(s.particles_advected))}
    sim.run()
    run = OracleRun(s, particle_init=p0)
    einc = []
    refloop.run_reference_loop(s, run, lambda t, dt: None, lambda c, t, e, g, n: einc.append(e))
    ours = read_monitoring(os.path.join(str(tmp), "data", sim.file_name()))
    return sim, run, np.asarray(ours["Error_incompressibility"]), np.asarray(einc), s


def _check_pair(sim, run, e_gpu, e_cpu, s):
    o = run.o
    assert e_gpu.shape == e_cpu.shape and e_gpu.size >= 16
    assert np.max(np.abs(e_gpu - e_cpu)) < einc_tol(TWO_PI, TWO_PI / 64)
    assert sim.scalar("map_counter") == o.map_count()
    assert map_err(sim.field("Map_ChiX_H_coarse"), o.chix()) < 1e-10
    assert map_err(sim.field("Map_ChiY_H_coarse"), o.chiy()) < 1e-10
    assert rel_linf(sim.field("Stream_function_Psi_H_psi"), o.psi()) < 1e-10
    for i, p in enumerate(s.particles_advected):
        assert _wrap_diff(sim.field("Particles_advected_pos_P%02d" % (i + 1)), o.particles(i)) < 1e-10, i
        if p.tau != 0:
            v, vo = sim.field("Particles_advected_vel_U%02d" % (i + 1)), o.particle_velocity(i)
            assert np.max(np.abs(v - vo)) <= 1e-10 * max(1.0, np.max(np.abs(vo))), i


@pytest.mark.parametrize("map_ti", ["AB2", "RK4", "RK3Mod", "RK4Mod"])
def test_map_integrators_match_oracle(tmp_path, map_ti):
    text = _param_text(map_ti, [_record(300, 0, "RK3")])
    _check_pair(*_run_pair(tmp_path, text))


@pytest.mark.parametrize("ti", ["EulerExp", "Heun", "RK3", "RK4", "RK3Mod", "RK4Mod"])
def test_tracers_and_inertial_particles_match_oracle(tmp_path, ti):
    recs = [_record(300, 0, ti, seed=1), _record(300, 0.5, ti, seed=2),
            _record(256, 0.2, ti, init="uniform_grid", init_vel=1),
            _record(300, 1.0, ti, init_time=0.125, init_vel=1, seed=4)]
    text = _param_text("RK3", recs)
    _check_pair(*_run_pair(tmp_path, text))


@pytest.mark.parametrize("map_ti,part_ti", [("AB2", "Heun"), ("RK4", "RK4"), ("RK3Mod", "RK3Mod"),
                                            ("RK4Mod", "RK4Mod")])
def test_mixed_form_follows_plain_fp64_for_every_scheme(tmp_path, map_ti, part_ti):
    """FP32 maps and nodes with the same schemes: energy and enstrophy within 1e-6,
    tracers and inertial particles within 1e-4 of plain FP64 (remaps at 1e-3: FP32
    E_inc rounding on this 64^2 map is ~1e-4)."""
    m = cmm()
    recs = [_record(300, 0, part_ti, seed=1), _record(300, 0.5, part_ti, seed=2, init_vel=1)]
    res = {}
    for prec in ("fp64", "mixed"):
        pf = tmp_path / ("p_%s.txt" % prec)
        pf.write_text(_param_text(map_ti, recs, precision=prec, threshold=1e-3))
        sim = m.Simulation(["param_file=%s" % pf, "workspace=%s/" % tmp_path, "sim_name=mx_" + prec])
        sim.init()
        sim.run()
        res[prec] = sim
    a, b = res["fp64"], res["mixed"]
    for name in ("energy", "enstrophy"):
        assert abs(a.scalar(name) - b.scalar(name)) <= 1e-6 * abs(a.scalar(name)), name
    for i in range(2):
        assert _wrap_diff(a.field("Particles_advected_pos_P%02d" % (i + 1)),
                          b.field("Particles_advected_pos_P%02d" % (i + 1))) < 1e-4
    v, w = a.field("Particles_advected_vel_U02"), b.field("Particles_advected_vel_U02")
    assert np.max(np.abs(v - w)) < 1e-4 * max(1.0, np.max(np.abs(v)))


IC_EULER = ["4_nodes", "quadropole", "one_vortex", "two_votices", "three_vortices", "single_shear_layer",
            "tanh_shear_layer", "turbulence_gaussienne", "gaussian_blobs", "shielded_vortex", "two_cosine",
            "vortex_sheets"]


@pytest.mark.parametrize("ic", IC_EULER)
def test_every_analytic_initial_condition_matches_oracle(tmp_path, ic):
    """Each analytic Euler initial condition (src/simulation/cmm-init.cu:30-241), composed
    through the Lagrange start and 8 steps with remaps: fine and coarse vorticity and psi
    against the oracle.  The oracle receives the product's random table (mt19937_64 values
    for gaussian_blobs and the cuRAND blob offsets of turbulence_gaussienne, both library
    draws, the latter checked here for its range and granularity)."""
    m = cmm()
    text = _param_text("RK3", [], final_time=0.125).replace(
        "initial_condition\t=\t4_nodes", "initial_condition\t=\t%s" % ic) + "initial_params\t=\t{500,0,0,0,0,0,0,0,0,0}\n"
    pf = tmp_path / "params.txt"
    pf.write_text(text)
    sim = m.Simulation(["param_file=%s" % pf, "workspace=%s/" % tmp_path])
    sim.init()
    table = sim.field("Init_random_table")
    assert table.size == 1098 and np.all(np.abs(table[:1000]) <= 1)
    off = table[1000:]
    assert np.all(np.abs(off) <= 0.005) and np.allclose(off * 1e5, np.round(off * 1e5), atol=1e-6)
    import oracle as O
    O.set_init_data(table=table)
    s = refloop.settings_from_param_text(text)
    o = O.EulerOracle(s.oracle_config())
    o.init()
    assert herm_err(sim.field("Vorticity_W_fine_H"), o.vort_fine(), 128) < 1e-10
    while sim.step(1) != 1:
        o.step(1.0 / 64)
    assert sim.scalar("map_counter") == o.map_count()
    w, wo = sim.field("Vorticity_W_coarse"), o.vort()
    assert np.max(np.abs(w - wo)) <= 1e-10 * np.max(np.abs(wo))
    assert rel_linf(sim.field("Stream_function_Psi_H_psi"), o.psi()) < 1e-10


def test_mixed_tracer_storage_order_is_invisible(tmp_path):
    """Sets of at least 4096 tracers are kept sorted by 4 x 4 psi-cell bucket in the mixed
    form (re-sorted every 32 steps); positions and velocities read back through the
    permutation.  Over 64 steps (two sorts), with a tracer set and an inertial set, the
    mixed form's positions and velocities follow plain FP64 tracer by tracer."""
    m = cmm()
    recs = [_record(6000, 0, "RK3", seed=3), _record(5000, 0.5, "RK3", seed=4, init_vel=1)]
    res = {}
    for prec in ("fp64", "mixed"):
        pf = tmp_path / ("p_%s.txt" % prec)
        pf.write_text(_param_text("RK3", recs, final_time=1.0, precision=prec, threshold=1e-3))
        sim = m.Simulation(["param_file=%s" % pf, "workspace=%s/" % tmp_path, "sim_name=ord_" + prec])
        sim.init()
        p0 = sim.field("Particles_advected_pos_P01").copy()
        sim.run()
        res[prec] = (sim, p0)
    (a, a0), (b, b0) = res["fp64"], res["mixed"]
    assert np.array_equal(a0, b0)
    for i in range(2):
        pa = a.field("Particles_advected_pos_P%02d" % (i + 1))
        pb = b.field("Particles_advected_pos_P%02d" % (i + 1))
        assert _wrap_diff(pa, pb) < 1e-4, i
    v, w = a.field("Particles_advected_vel_U02"), b.field("Particles_advected_vel_U02")
    assert np.max(np.abs(v - w)) < 1e-4 * max(1.0, np.max(np.abs(v)))
