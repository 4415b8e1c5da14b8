"""The forward map (forward_map = 1) on the GPU against the oracle.

A run with remaps: the forward map is advected beside the backward one
(k_advect_using_stream_hermite, direction 1), checked for invertibility and
incompressibility each step, pushed onto its own stack at every remap, and composed
oldest-first on the sample grid and on zoom windows (apply_map_stack, direction 1).
Two forwarded particle sets: one from t = 0, one whose start time forces a remap and
which is mapped only from the sub-map after it (apply_map_stack_points); particles
leaving a zoom frame are NaN.  Every Debug_globals series, the two forward monitors per
step and the raw forwarded-particle files are compared with the oracle, for each forward
integrator (the reference's RK4 and RK4Mod quirks included).
"""
import os

import numpy as np
import pytest

import refloop
from goldens import DebugRecorder, compare_series
from oracle_adapter import OracleRun
from product import cmm, read_monitoring
from test_gpu_parity import map_err

pytestmark = pytest.mark.gpu


def _text(ti):
    rec = ("{num=%d,seed=%d,time_integration=RK3,init_name=uniform,init_time=%r,"
           "init_param_1=3.141592653589793,init_param_2=3.141592653589793,init_param_3=6.283185307179586,"
           "init_param_4=6.283185307179586}")
    return "\n".join([
        "CMM Parameter file", "param_version\t=\t3", "",
        "simulation_type\t=\tcmm_euler_2d", "sim_name\t=\tfw", "initial_condition\t=\t4_nodes",
        "grid_coarse\t=\t64", "grid_fine\t=\t128", "grid_vort\t=\t128", "grid_psi\t=\t64", "set_dt_by_steps\t=\t1",
        "steps_per_sec\t=\t64", "final_time\t=\t0.25", "time_integration\t=\t%s" % ti, "map_update_order\t=\t4th",
        "map_epsilon\t=\t0.001", "incomp_threshold\t=\t1e-05", "skip_remapping\t=\t0", "molly_stencil\t=\t0",
        "lagrange_init_higher_order\t=\t1", "freq_cut_psi\t=\t32", "mem_RAM_CPU_remaps\t=\t200",
        "save_map_stack\t=\t0", "verbose\t=\t4", "scalar_name\t=\tgaussian",
        "save_computational_num\t=\t1",
        "save_computational\t=\t{is_instant=0,time_start=0,time_end=10000,time_step=0.0625,var=All,conv=1}",
        "save_sample_num\t=\t1",
        "save_sample\t=\t{is_instant=0,time_start=0,time_end=10000,time_step=0.0625,var=All,grid=64}",
        "save_zoom_num\t=\t1",
        "save_zoom\t=\t{is_instant=0,time_start=0,time_end=10000,time_step=0.125,var=AllPartF_01,grid=48,"
        "pos_x=2.5,pos_y=4.0,width_x=3.0,width_y=3.0,rep=2,rep_fac=0.5}",
        "forward_map\t=\t1", "particles_advected_num\t=\t0", "particles_forwarded_num\t=\t2",
        "particles_forwarded\t=\t" + rec % (400, 5, 0.0), "particles_forwarded\t=\t" + rec % (300, 6, 0.109375), ""])


@pytest.mark.parametrize("ti", ["EulerExp", "Heun", "AB2", "RK3", "RK4", "RK3Mod", "RK4Mod"])
def test_forward_map_run_matches_oracle(tmp_path, ti):
    m = cmm()
    text = _text(ti)
    pf = tmp_path / "params.txt"
    pf.write_text(text)
    sim = m.Simulation(["param_file=%s" % pf, "workspace=%s/" % tmp_path])
    sim.init()
    f0 = [sim.field("Particles_forwarded_pos_P%02d" % (i + 1)).copy() for i in range(2)]
    assert all(np.isfinite(f).all() for f in f0)
    sim.run()
    run_dir = os.path.join(str(tmp_path), "data", sim.file_name())
    ours = read_monitoring(run_dir)
    s = refloop.settings_from_param_text(text)
    run = OracleRun(s, forwarded_init={0: f0[0], 1: f0[1]})
    rec = DebugRecorder(s, run)
    refloop.run_reference_loop(s, run, rec.on_save, rec.on_step)
    assert max(rec.series["Map_counter"]) >= 2
    assert len(ours["Error_invertibility"]) == 16
    keys = list(rec.series)
    assert len([k for k in keys if "_f_" in k]) >= 4 * 6
    worst, fails = compare_series(ours, rec.series, keys, 1e-9)
    assert not fails, fails
    assert map_err(sim.field("Map_ChiX_f_H_coarse"), run.o.chix_f()) < 1e-10
    # raw forwarded-particle files at every sample instant (the whole domain as frame)
    n_files = 0
    for (t, i), pos in rec.forwarded.items():
        # folders are named with 3 significant digits (the reference's to_str), "final" at the end
        folder = "Time_final" if t > 1e3 else "Time_%.3g" % t
        got = np.fromfile(os.path.join(run_dir, "Particle_data", folder, "Particles_forwarded_pos_P%02d.data" % (i + 1)))
        assert got.shape == pos.shape
        assert np.array_equal(np.isnan(got), np.isnan(pos))
        ok = ~np.isnan(pos)
        dd = np.abs(got[ok] - pos[ok])
        assert np.all(np.minimum(dd, 2 * np.pi - dd) < 1e-10), (t, i)
        n_files += 1
    assert n_files >= 8
    # zoom frames: the first set's file (named P00 as in the reference), NaN outside the frame
    zf = os.path.join(run_dir, "Zoom_data", "Time_final", "Zoom_1_rep_1", "Particles_forwarded_pos_P00.data")
    z = np.fromfile(zf)
    assert z.size == 800 and np.isnan(z).any() and np.isfinite(z).any()


def test_forward_map_in_the_mixed_form(tmp_path):
    """precision=mixed with forward_map=1: the forward map stays FP64, advected on FP64 copies
    of the FP32 psi levels and checked against the FP32 backward map.  Against the plain FP64
    run of the same parameter file (RK3, remaps, both forwarded sets) up to the first step
    where the two remap histories part (E_inc meets the threshold within FP32 noise): the same
    remap steps, both forward monitors per step and the forwarded particles (modulo the
    period) at every sample instant before it.  Threshold 1e-4 (the FP32 maps sit near 2e-5
    of incompressibility error right after a remap on a 64^2 map, above this file's 1e-5),
    T = 1.  The mixed Vlasov-Poisson form keeps refusing the option."""
    m = cmm()
    text = _text("RK3").replace("incomp_threshold\t=\t1e-05", "incomp_threshold\t=\t0.0001").replace(
        "final_time\t=\t0.25", "final_time\t=\t1")
    res = {}
    for prec in ("fp64", "mixed"):
        work = tmp_path / prec
        work.mkdir()
        pf = work / "params.txt"
        pf.write_text(text)
        sim = m.Simulation(["param_file=%s" % pf, "workspace=%s/" % work, "precision=%s" % prec])
        sim.init()
        sim.run()
        run_dir = os.path.join(str(work), "data", sim.file_name())
        parts = {}
        pdir = os.path.join(run_dir, "Particle_data")
        for folder in os.listdir(pdir):
            for i in range(2):
                f = os.path.join(pdir, folder, "Particles_forwarded_pos_P%02d.data" % (i + 1))
                if os.path.exists(f):
                    parts[(folder, i)] = np.fromfile(f)
        res[prec] = (read_monitoring(run_dir), sim.field("Map_ChiX_f_H_coarse").copy(),
                     sim.field("Map_ChiY_f_H_coarse").copy(), parts)
        sim.close()
    (mp, xp, yp, pp), (mm, xm, ym, pm) = res["fp64"], res["mixed"]
    # the two runs remap at the same steps until E_inc meets the threshold within FP32 noise
    # (a remap one step apart); everything before that step is compared
    cp, cm = mp["Map_counter"], mm["Map_counter"]
    assert len(cp) == len(cm) == 64
    div = next((i for i in range(64) if cp[i] != cm[i]), 64)
    assert div >= 30 and cp[div - 1] >= 3, (div, cp, cm)
    assert abs(cp[-1] - cm[-1]) <= 1
    for k in ("Error_incompressibility_forward", "Error_invertibility"):
        a, b = np.array(mm[k][:div]), np.array(mp[k][:div])
        # the forward map is advected on FP32-accurate psi: its determinant deviation carries
        # the rounding of the psi_xy plane (a floor of ~2e-6 on a 64^2 map), and E_inv the
        # FP32 backward map's (~1e-7 of the domain)
        assert np.all(np.abs(a - b) <= 2e-2 * np.abs(b) + 5e-6), (k, a, b)
    if div == 64:
        assert np.max(np.abs(xm[: xm.size // 4] - xp[: xp.size // 4])) < 1e-5
        assert np.max(np.abs(ym[: ym.size // 4] - yp[: yp.size // 4])) < 1e-5
    # (the Debug_globals statistics of the sampled forward map are not compared: points within
    # rounding of the periodic boundary flip between 0 and 2 pi in either run)
    assert set(pm) == set(pp) and len(pp) >= 8
    n_cmp = 0
    for (folder, i), a in pp.items():
        t = 1e9 if folder == "Time_final" else float(folder.split("_")[1])
        if t * 64 >= div - 0.5:
            continue
        b = pm[(folder, i)]
        assert np.array_equal(np.isnan(a), np.isnan(b))
        ok = ~np.isnan(a)
        d = np.abs(b[ok] - a[ok])
        assert np.all(np.minimum(d, 2 * np.pi - d) < 1e-4), (folder, i)
        n_cmp += 1
    assert n_cmp >= 8
    bad = m.Simulation(["workspace=%s/" % tmp_path, "sim_name=vfw", "simulation_type=cmm_vlasov_poisson_1d",
                        "initial_condition=landau_damping", "domain_bounds={0,4,-2.5,2.5}", "grid_coarse=32",
                        "grid_fine=64", "grid_vort=64", "grid_psi=64", "forward_map=1", "precision=mixed",
                        "verbose=0"])
    with pytest.raises(m.CmmError) as e:
        bad.init()
    assert e.value.code == m.CMM_ERR_UNSUPPORTED


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_discrete_scalar_samples_the_discrete_initial_vorticity(tmp_path, precision):
    """scalar_discrete=1: the reference's k_h_sample_from_init reads Vort_discrete_init for
    the passive scalar (cmm-simulation-host.cu:803-805), so on a sample grid the scalar equals
    the composed discrete initial vorticity, i.e. the sampled vorticity, value for value;
    without a discrete initial field the option is refused."""
    m = cmm()
    n = 64
    rng = np.random.default_rng(5)
    k = np.fft.rfftfreq(4 * n, 1.0 / (4 * n))
    w = np.fft.irfft2(np.exp(-((k[None, :] ** 2 + np.fft.fftfreq(4 * n, 1.0 / (4 * n))[:, None] ** 2) / 40.0))
                      * np.exp(2j * np.pi * rng.uniform(size=(4 * n, 2 * n + 1))), s=(4 * n, 4 * n)) * 1e3
    lines = ["CMM Parameter file", "param_version\t=\t3", ""]
    kv = [("sim_name", "dscal"), ("grid_coarse", n), ("grid_fine", 4 * n), ("grid_vort", 4 * n), ("grid_psi", 2 * n),
          ("set_dt_by_steps", 1), ("steps_per_sec", 32), ("final_time", 0.5), ("initial_discrete", 1),
          ("initial_discrete_grid", 4 * n), ("incomp_threshold", 1e-4), ("freq_cut_psi", n // 2),
          ("scalar_discrete", 1), ("save_computational_num", 0), ("save_zoom_num", 0), ("particles_advected_num", 0),
          ("save_map_stack", 0), ("verbose", 0), ("precision", precision), ("save_sample_num", 1)]
    lines += ["%s\t=\t%s" % (a, b) for a, b in kv]
    lines.append("save_sample\t=\t{is_instant=0,time_start=0,time_end=0.5,time_step=0.25,var=Vorticity Scalar,grid=64}")
    pf = tmp_path / "p.txt"
    pf.write_text("\n".join(lines) + "\n")
    sim = m.Simulation(["param_file=%s" % pf, "workspace=%s/" % tmp_path])
    sim.set_initial_discrete(np.ascontiguousarray(w))
    sim.init()
    sim.run()
    run = os.path.join(str(tmp_path), "data", sim.file_name(), "Time_data")
    found = 0
    for d in sorted(os.listdir(run)):
        sc = os.path.join(run, d, "Scalar_Theta_64.data")
        vo = os.path.join(run, d, "Vorticity_W_64.data")
        if os.path.exists(sc) and os.path.exists(vo):
            a, b = np.fromfile(sc, dtype="<f8"), np.fromfile(vo, dtype="<f8")
            assert a.size == 64 * 64 and np.array_equal(a, b), d
            found += 1
    assert found >= 2
    sim.close()
    bad = m.Simulation(["workspace=%s/" % tmp_path, "sim_name=dscal_bad", "scalar_discrete=1", "initial_discrete=0",
                        "grid_coarse=32", "grid_fine=64", "grid_vort=64", "grid_psi=32", "verbose=0"])
    with pytest.raises(m.CmmError) as e:
        bad.init()
    assert e.value.code == m.CMM_ERR_UNSUPPORTED
