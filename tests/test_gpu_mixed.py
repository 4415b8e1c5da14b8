"""GPU tests of the mixed-precision form (precision=mixed: FP32 displacement
maps, FP32 Hermite psi / fine vorticity, fixed-point tracer positions, FP64
composition, FP64-accurate determinant deviation, FP64 diagnostic sums)
against the plain FP64 form of the same library, which the other GPU tests
pin to the CPU oracle and the reference.

Acceptance: relative enstrophy error <= 1e-4 against plain FP64 at the end
of the run; energy, palinstrophy and max |omega| are held to the same bound;
the remap count may differ by one where FP32 rounding moves E_inc across the
threshold.
"""
import os
import sys

import numpy as np
import pytest

from product import cmm

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _args(work, precision, coarse, fine, psi, steps_per_sec, final_time, threshold, discrete=False):
    a = ["workspace=%s/" % work, "sim_name=mx_%s" % precision, "grid_coarse=%d" % coarse, "grid_fine=%d" % fine,
         "grid_vort=%d" % fine, "grid_psi=%d" % psi, "set_dt_by_steps=1", "steps_per_sec=%d" % steps_per_sec,
         "final_time=%g" % final_time, "time_integration=RK3", "map_update_order=4th", "map_epsilon=0.001",
         "incomp_threshold=%r" % threshold, "skip_remapping=0", "molly_stencil=0", "freq_cut_psi=%d" % (psi // 2),
         "particles_advected_num=0", "save_sample_num=0", "save_computational_num=0", "verbose=0",
         "mem_RAM_CPU_remaps=4000", "precision=%s" % precision]
    if discrete:
        a += ["initial_discrete=1", "initial_discrete_grid=%d" % fine]
    return a


def _run(m, args, ic=None):
    sim = m.Simulation(args)
    if ic is not None:
        sim.set_initial_discrete(ic)
    sim.init()
    series = []
    while True:
        rc = sim.step(1)
        if rc == 1:
            break
        series.append((sim.scalar("time"), sim.scalar("e_inc"), int(sim.scalar("map_counter"))))
    diag = {k: sim.scalar(k) for k in ("energy", "enstrophy", "palinstrophy", "max_vorticity")}
    fields = {k: sim.field(k) for k in ("Stream_function_Psi_H_psi", "Vorticity_W_coarse", "Map_ChiX_H_coarse")}
    sim.close()
    return series, diag, fields


def _compare(plain, mixed, tol=1e-4, same_remaps=True):
    sp, dp, fp = plain
    sm, dm, fm = mixed
    assert len(sp) == len(sm)
    if same_remaps:
        assert [s[2] for s in sp] == [s[2] for s in sm], "remap steps differ"
    for k in ("energy", "enstrophy", "palinstrophy", "max_vorticity"):
        assert abs(dm[k] - dp[k]) <= tol * abs(dp[k]), (k, dm[k], dp[k])
    for k in ("Stream_function_Psi_H_psi", "Vorticity_W_coarse"):
        a, b = fm[k], fp[k]
        assert np.max(np.abs(a - b)) <= 1e-3 * np.max(np.abs(b)), k


def test_mixed_c1_matches_plain_fp64(tmp_path):
    """C1 (map 128^2, dt = 1/64) moves footpoints 4x further per step than the
    metric's configuration; the FP32 footpoint rounding then reaches the
    Jacobian through the 1/eps^2 GALS X_xy plane at the 1e-5 level, so the
    remap instants may shift.  The transported fields and the conserved
    quantities must still agree to 1e-4."""
    m = cmm()
    for thr in (1e-4, 1e-5):
        plain = _run(m, _args(tmp_path, "fp64", 128, 512, 256, 64, 1.0, thr))
        mixed = _run(m, _args(tmp_path, "mixed", 128, 512, 256, 64, 1.0, thr))
        _compare(plain, mixed, same_remaps=False)
        einc_p = np.array([s[1] for s in plain[0]])
        einc_m = np.array([s[1] for s in mixed[0]])
        assert np.max(np.abs(einc_p - einc_m)) <= 2.5e-4


def test_mixed_turbulence_matches_plain_fp64(tmp_path):
    """The metric's random-phase turbulence, scaled down (map 128^2, fine
    512^2, psi 256^2, dt = 1/64, T = 1, with remaps)."""
    import bench
    m = cmm()
    ic = bench.initial_vorticity(512, seed=1, k0=8.0)
    plain = _run(m, _args(tmp_path, "fp64", 128, 512, 256, 64, 1.0, 1e-4, discrete=True), ic)
    mixed = _run(m, _args(tmp_path, "mixed", 128, 512, 256, 64, 1.0, 1e-4, discrete=True), ic)
    assert plain[0][-1][2] >= 1, "the case should remap"
    _compare(plain, mixed, same_remaps=False)
    assert abs(plain[0][-1][2] - mixed[0][-1][2]) <= 1


def test_mixed_tracers_follow_plain_fp64(tmp_path):
    """The mixed form keeps tracer positions as 64-bit fixed point: after the
    initialisation they must read back as the FP64 positions, and after 64
    RK3 steps (with remaps) they must stay on the plain FP64 trajectories."""
    import bench
    m = cmm()
    args = [a for a in _args(tmp_path, "fp64", 128, 512, 256, 64, 1.0, 1e-5)
            if not a.startswith(("particles_advected_num", "precision"))] + ["particles_advected_num=1"]
    rec = ("{num=4096,tau=0,seed=0,time_integration=RK3,init_name=uniform,init_time=0,init_vel=0,"
           "init_param_1=3.141592653589793,init_param_2=3.141592653589793,"
           "init_param_3=6.283185307179586,init_param_4=6.283185307179586}")
    pf = str(tmp_path / "params.txt")
    bench.write_param_file(pf, args, [rec])
    start, end = {}, {}
    for prec in ("fp64", "mixed"):
        sim = m.Simulation(["param_file=" + pf, "precision=" + prec])
        sim.init()
        start[prec] = sim.field("Particles_advected_pos_P01")
        while sim.step(1) != 1:
            pass
        end[prec] = sim.field("Particles_advected_pos_P01")
        sim.close()
    two_pi = 2 * np.pi
    assert np.max(np.abs(start["mixed"] - start["fp64"])) <= 1e-14
    assert np.all((end["mixed"] >= 0) & (end["mixed"] < two_pi))
    d = np.mod(end["mixed"] - end["fp64"] + np.pi, two_pi) - np.pi
    assert np.max(np.abs(d)) <= 1e-4, np.max(np.abs(d))


def test_mixed_fields_convert_to_reference_layout(tmp_path):
    m = cmm()
    sim = m.Simulation(_args(tmp_path, "mixed", 32, 128, 64, 16, 0.25, 1e-4))
    sim.init()
    x = sim.field("Map_ChiX_H_coarse").reshape(4, 32, 32)
    h = 6.283185307179586 / 32
    # identity map after the Lagrange initialisation: X = x, X_x = 1, X_y = X_xy = 0
    assert np.allclose(x[0], np.arange(32)[None, :] * h)
    assert np.allclose(x[1], 1.0) and np.allclose(x[2], 0.0) and np.allclose(x[3], 0.0)
    sim.step(2)
    psi = sim.field("Stream_function_Psi_H_psi")
    assert psi.shape == (4 * 64 * 64,) and np.isfinite(psi).all()
    sim.close()


def test_mixed_captured_and_plain_launches_agree(tmp_path):
    """The mixed step's front (advection, Jacobian check, psi solve) is replayed as a CUDA
    graph; profiled steps launch the same kernels plainly.  Both chains launch them as
    programmatic dependents of one another (each kernel waits for its predecessor before
    it reads or writes) and fork the E_inc readback to a side stream; both must give the
    same bits, with remaps and tracers, at sizes that run the compile-time transform
    kernels (vorticity 512^2, psi 256^2)."""
    import bench
    m = cmm()
    args = [a for a in _args(tmp_path, "mixed", 128, 512, 256, 64, 0.5, 1e-5, discrete=True)
            if not a.startswith("particles_advected_num")] + ["particles_advected_num=1"]
    rec = ("{num=4096,tau=0,seed=0,time_integration=RK3,init_name=uniform,init_time=0,init_vel=0,"
           "init_param_1=3.141592653589793,init_param_2=3.141592653589793,"
           "init_param_3=6.283185307179586,init_param_4=6.283185307179586}")
    pf = str(tmp_path / "params.txt")
    bench.write_param_file(pf, args, [rec])
    ic = bench.initial_vorticity(512, seed=3, k0=8.0)
    out = {}
    for profiled in (False, True):
        sim = m.Simulation(["param_file=" + pf])
        sim.set_initial_discrete(ic)
        sim.init()
        sim.set_profiling(profiled)
        einc = []
        while sim.step(1) != 1:
            einc.append(sim.scalar("e_inc"))
        out[profiled] = (np.array(einc), int(sim.scalar("map_counter")),
                         {k: sim.field(k) for k in ("Stream_function_Psi_H_psi", "Map_ChiX_H_coarse",
                                                    "Particles_advected_pos_P01")})
        sim.close()
    (e0, n0, f0), (e1, n1, f1) = out[False], out[True]
    assert n0 >= 1 and n0 == n1, (n0, n1)
    assert np.array_equal(e0, e1)
    for k in f0:
        assert np.array_equal(f0[k], f1[k]), k


@pytest.mark.parametrize("coarse,fine,psi", [(256, 1024, 512), (1024, 4096, 2048)])
def test_mixed_psi_solve_sizes_match_plain_fp64(tmp_path, coarse, fine, psi):
    """The FP32 psi solve's compile-time kernels at the vorticity / psi sizes the other tests
    do not reach (1024^2 / 512^2 and 4096^2 / 2048^2): the psi of the mixed form after its
    initialisation and two steps against plain FP64 (relative L-infinity per Hermite plane,
    FP32 rounding of the vorticity sample and transforms: 1e-4)."""
    import bench
    m = cmm()
    ic = bench.initial_vorticity(fine, seed=2, k0=8.0)
    out = {}
    for prec in ("fp64", "mixed"):
        sim = m.Simulation(_args(tmp_path, prec, coarse, fine, psi, 256, 2.0 / 256, 1e-4, discrete=True))
        sim.set_initial_discrete(ic)
        sim.init()
        sim.step(2)
        out[prec] = sim.field("Stream_function_Psi_H_psi").reshape(4, psi, psi)
        sim.close()
    for q in range(4):
        ref = out["fp64"][q]
        err = np.max(np.abs(out["mixed"][q] - ref)) / np.max(np.abs(ref))
        assert err < 1e-4, (q, err)
