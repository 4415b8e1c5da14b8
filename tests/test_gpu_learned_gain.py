"""What the trained upsampler gains over the method without it, and the learned form's
exact-evaluation judge.

A 2-block network is trained on the GPU (its own tensor-core forward / backward kernels,
Adam, the psi-space loss) on pairs collected every 4 steps from six decaying-turbulence
runs (map 128^2, vorticity 512^2, psi 256^2, random-phase omega_0 with k0 = 8, seeds 1-6),
then judged on a seventh run (seed 0) it never saw: at 8 instants of that run, the relative
L2 difference from the exact psi of the cheap psi (omega sampled on the map grid, the method
without the network) and of the learned psi (the same plus the network's sub-grid
vorticity).  The learned psi must be closer on average (ratio < 0.95) and at most instants.

The learned form inside a run: every 8th step is exact and judges the learned and the cheap
psi; with a tolerance nothing meets, every check fails and the run falls back to exact
steps; with a tolerance everything meets, only the judged steps are exact and the others
use whichever of the network and the cheap psi was closer at the last check.
"""
import numpy as np
import pytest

import bench
from product import cmm

pytestmark = pytest.mark.gpu
N = 128


def _args(tmp, name, final=4.0):
    n = N
    return ["workspace=%s/" % tmp, "sim_name=%s" % name, "simulation_type=cmm_euler_2d",
            "grid_coarse=%d" % n, "grid_fine=%d" % (4 * n), "grid_vort=%d" % (4 * n), "grid_psi=%d" % (2 * n),
            "set_dt_by_steps=1", "steps_per_sec=%d" % (n // 2), "final_time=%r" % final,
            "initial_condition=4_nodes", "initial_discrete=1", "initial_discrete_grid=%d" % (4 * n),
            "time_integration=RK3", "map_update_order=4th", "map_epsilon=0.001", "incomp_threshold=1e-4",
            "skip_remapping=0", "molly_stencil=0", "freq_cut_psi=%d" % (n // 4), "lagrange_init_higher_order=1",
            "mem_RAM_CPU_remaps=100000", "save_computational_num=0", "save_sample_num=0", "save_zoom_num=0",
            "forward_map=0", "particles_advected_num=0", "save_map_stack=0", "verbose=0", "precision=mixed"]


@pytest.fixture(scope="module")
def trained(tmp_path_factory):
    m = cmm()
    tmp = tmp_path_factory.mktemp("learned")
    u = m.Upsampler(blocks=2, seed=1)
    for seed in range(1, 7):
        sim = m.Simulation(_args(tmp, "tr%d" % seed))
        sim.set_initial_discrete(bench.initial_vorticity(4 * N, seed=seed, k0=8.0))
        sim.init()
        k = 0
        while sim.step(1) != 1:
            k += 1
            if k % 4 == 0:
                u.collect(sim)
        sim.close()
    losses = [u.train(100, batch=8, lr=1e-3 if r < 16 else 2e-4, seed=r)[0] for r in range(20)]
    return m, u, tmp, losses


def test_training_lowers_the_psi_space_loss(trained):
    _, u, _, losses = trained
    assert u.dataset_size() == 6 * 64
    assert np.mean(losses[-4:]) < 0.8 * np.mean(losses[:2]), losses


def test_trained_network_gains_over_the_method_without_it(trained):
    m, u, tmp, _ = trained
    ev = m.Simulation(_args(tmp, "held_out"))
    ev.set_initial_discrete(bench.initial_vorticity(4 * N, seed=0, k0=8.0))
    ev.init()
    cheap, learned, k = [], [], 0
    while ev.step(1) != 1:
        k += 1
        if k % 32 == 0:
            e = u.evaluate(ev)
            cheap.append(e["cheap_l2"])
            learned.append(e["learned_l2"])
            # the learned psi may not be worse than the exact evaluation of omega on the psi grid
            assert e["grid_l2"] <= e["learned_l2"]
    ev.close()
    cheap, learned = np.array(cheap), np.array(learned)
    ratio = learned / cheap
    assert len(ratio) == 8
    assert np.mean(ratio) < 0.95, ratio
    assert np.sum(ratio < 1.0) >= 6, ratio


def test_learned_form_judge_and_fallback(trained):
    m, u, tmp, _ = trained
    runs = {}
    for name, tol in (("strict", 1e-12), ("loose", 1.0)):
        sim = m.Simulation(_args(tmp, "judge_" + name, final=1.0))
        sim.set_initial_discrete(bench.initial_vorticity(4 * N, seed=0, k0=8.0))
        sim.init()
        sim.attach_upsampler(u, every=8, tol=tol)
        sim.run()
        runs[name] = {k: sim.scalar(k) for k in ("learned_steps", "cheap_steps", "exact_steps", "learned_checks",
                                                "learned_cheaper", "learned_failures", "learned_max_err",
                                                "enstrophy", "energy")}
        sim.close()
    s, l_ = runs["strict"], runs["loose"]
    steps = int(1.0 * N / 2)
    # strict: every judged step fails, so everything after a check is exact
    assert s["learned_steps"] == s["cheap_steps"] == 0 and s["exact_steps"] == steps
    assert s["learned_checks"] == s["learned_failures"] == steps // 8
    # loose: exactly every 8th step is exact (and judged), the others learned or cheap as judged,
    # and the trained network is chosen at some checks
    assert l_["exact_steps"] == l_["learned_checks"] == steps // 8 and l_["learned_failures"] == 0
    assert l_["learned_steps"] + l_["cheap_steps"] == steps - steps // 8
    assert l_["cheap_steps"] == 7 * l_["learned_cheaper"]
    assert l_["learned_steps"] > 0
    assert 0 < l_["learned_max_err"] < 1e-2
    # a run of learned steps conserves like the exact one
    for q in ("enstrophy", "energy"):
        assert abs(l_[q] - s[q]) <= 1e-4 * abs(s[q]), q


def test_dataset_clear_streams_pairs(tmp_path):
    """Streamed training collects a run's pairs, trains on them and drops them: after
    cmm_upsampler_clear_dataset the set is empty, collection starts again, and training
    on the new pairs runs."""
    m = cmm()
    u = m.Upsampler(blocks=1, seed=2)
    sim = m.Simulation(_args(tmp_path, "clr", final=0.25))
    sim.set_initial_discrete(bench.initial_vorticity(4 * N, seed=5, k0=8.0))
    sim.init()
    for _ in range(2):
        sim.step(1)
        u.collect(sim)
    assert u.dataset_size() == 2
    u.clear_dataset()
    assert u.dataset_size() == 0
    sim.step(1)
    u.collect(sim)
    assert u.dataset_size() == 1
    loss, sec = u.train(2, batch=1)
    assert np.isfinite(loss) and sec > 0
    sim.close()
    u.close()
