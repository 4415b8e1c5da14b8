"""The oracle's forward map (forward_map = 1) on the CPU.

The reference's forward-map golden (tests/euler2D_init_fields, reference-results_forward)
holds only t = 0, where every forward quantity is the identity; it is matched in
test_oracle_golden.py.  Over a run the forward map must invert the backward one: the
invertibility error max |x - X_b(X_f(x))| (k_invertibility_check,
src/simulation/cmm-simulation-kernel.cu:177-198) stays at the schemes' truncation
level -- except for RK4Mod, whose forward integrator in the reference is a copy of the
backward one (src/numerical/cmm-timestep.cu:385-420) and moves the forward map backwards;
the restatement keeps that, and this test pins it.
"""
import numpy as np
import pytest

import refloop
from oracle_adapter import OracleRun


def _text(ti, final_time=0.25):
    return "\n".join(["CMM Parameter file", "param_version\t=\t3", "", "simulation_type\t=\tcmm_euler_2d",
                      "initial_condition\t=\t4_nodes", "grid_coarse\t=\t64", "grid_fine\t=\t128", "grid_vort\t=\t128",
                      "grid_psi\t=\t64", "set_dt_by_steps\t=\t1", "steps_per_sec\t=\t64",
                      "final_time\t=\t%r" % final_time, "time_integration\t=\t%s" % ti, "incomp_threshold\t=\t1e-5",
                      "skip_remapping\t=\t0", "freq_cut_psi\t=\t32", "forward_map\t=\t1", "mem_RAM_CPU_remaps\t=\t100",
                      "save_computational_num\t=\t0", "save_sample_num\t=\t0", "particles_advected_num\t=\t0", ""])


@pytest.mark.parametrize("ti,bound", [("Heun", 2e-5), ("AB2", 5e-5), ("RK3", 2e-5), ("RK4", 1e-4), ("RK3Mod", 2e-5)])
def test_forward_map_inverts_the_backward_map(ti, bound):
    s = refloop.settings_from_param_text(_text(ti))
    run = OracleRun(s)
    mon = []
    refloop.run_reference_loop(s, run, lambda t, dt: None,
                               lambda c, t, e, g, n: mon.append(run.forward_monitors() + (n,)))
    mon = np.asarray(mon)
    assert mon.shape[0] == 16 and mon[-1, 2] >= 2          # 16 steps, remaps on both stacks
    assert mon[:, 1].max() < bound                          # invertibility
    assert mon[:, 0].max() < 1e-4                           # forward incompressibility


def test_reference_rk4mod_forward_scheme_runs_backwards():
    s = refloop.settings_from_param_text(_text("RK4Mod"))
    run = OracleRun(s)
    mon = []
    refloop.run_reference_loop(s, run, lambda t, dt: None, lambda c, t, e, g, n: mon.append(run.forward_monitors()))
    assert np.asarray(mon)[:, 1].max() > 0.05
