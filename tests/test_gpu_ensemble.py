"""Ensembles of uneven-size runs advanced together (cmm_ensemble_*).

Each member of an ensemble runs the single-member kernels' device bodies on its own
descriptor, and the psi solve transforms every member of a size class in one batched
transform (the library's FFT).  The batched kernels are separate instantiations of those bodies (their
arguments come from shared memory rather than the parameter space), so the compiler
may contract and share FP32 products differently: a member agrees with its single run
to FP32 rounding, not bit for bit (one step moves the map's cross-derivative plane, whose
conditioning is 1/eps^2, by a few FP32 ulps).  Checked here: every member's map (in units
of its conditioning), psi and coarse vorticity after a run without remaps against the
member run alone, with and without the CUDA graphs; a run with remaps (counts within one,
conserved quantities to 1e-6); the members' conserved quantities against plain FP64 runs;
and the members the ensemble rejects.
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
    # N / 4N / 2N grids (map / fine = vort / psi), dt = 1 / (N / 2).  The FP32 rounding of E_inc
    # grows like dt h / eps^2 ~ 0.75 / N^2 (7e-4 at N = 32), so these small members remap at 1e-3
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


@pytest.mark.parametrize("graphs", [True, False])
def test_ensemble_members_equal_their_single_runs(tmp_path, graphs):
    from test_gpu_parity import map_err
    m = cmm()
    (tmp_path / "e").mkdir()
    (tmp_path / "s").mkdir()
    ics = [random_vorticity(4 * n, seed=i, k0=3.0 + i) for i, n in enumerate(SIZES)]
    ens = m.Ensemble([member_args(tmp_path / "e", i, n, threshold=1.0) for i, n in enumerate(SIZES)], graphs=graphs)
    for i, w in enumerate(ics):
        ens.set_initial_discrete(i, w)
    ens.init()
    ens.run()
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


def test_ensemble_members_remap_like_their_single_runs(tmp_path):
    m = cmm()
    (tmp_path / "e").mkdir()
    (tmp_path / "s").mkdir()
    ics = [random_vorticity(4 * n, seed=i, k0=3.0 + i) for i, n in enumerate(SIZES)]
    ens = m.Ensemble([member_args(tmp_path / "e", i, n, final_time=1.0) for i, n in enumerate(SIZES)])
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
        for name in ("energy", "enstrophy"):
            assert abs(ens.scalar(i, name) - sim.scalar(name)) <= 1e-6 * abs(sim.scalar(name)), (i, name)
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
