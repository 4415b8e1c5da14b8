"""CPU-only tests of the product's boundary: the C-ABI library loads and
exports every symbol of include/cmm_abi.h, and the reference's settings /
param-file interface resolves exactly like the reference (checked against the
test-side restatement in tests/refloop.py and against the reference's own
output-folder names).  No GPU work is launched here; the one call that needs
a GPU checks that it fails with a status code instead of exiting."""
import ctypes as C
import os

import pytest

import refloop
from goldens import goldens
from product import cmm, header_functions

GOLDEN_DIRS = {
    "init_comp": "init_fields_comp_4_nodes_C256_F512_t1_T0",
    "one_step": "one_step_4_nodes_C256_F512_t1_T1",
    "remap_11b": "11b-4nodes-reference-remapping_4_nodes_C256_F512_t32_T2",
}


def test_library_exports_every_declared_symbol():
    m = cmm()
    L = m.lib()
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(m.EXPORTS) == set(names)
    assert b"sm_103a" in L.cmm_version()


@pytest.mark.parametrize("name", sorted(GOLDEN_DIRS))
def test_param_files_resolve_like_the_reference(tmp_path, name):
    m = cmm()
    text = goldens()[name]["params_in"]
    pf = tmp_path / "params.txt"
    pf.write_text(text)
    sim = m.Simulation(["param_file=%s" % pf])
    ref = refloop.settings_from_param_text(text)
    assert sim.file_name() == GOLDEN_DIRS[name]
    assert sim.scalar("dt") == ref.dt
    assert int(sim.scalar("lagrange_order")) == ref.lagrange_order
    assert int(sim.scalar("stack_capacity")) == ref.cpu_map_num
    # the written parameter text parses back to the same settings
    back = refloop.settings_from_param_text(sim.settings_text())
    for key in ("grid_coarse", "grid_fine", "grid_psi", "grid_vort", "final_time", "steps_per_sec",
                "incomp_threshold", "map_epsilon", "time_integration", "map_update_order", "freq_cut_psi",
                "skip_remapping", "verbose", "initial_condition"):
        assert getattr(back, key) == getattr(ref, key), key
    assert len(back.save_comp) == len(ref.save_comp)
    for a, b in zip(back.save_comp, ref.save_comp):
        assert (a.is_instant, a.time_start, a.var, a.conv) == (b.is_instant, b.time_start, b.var, b.conv)
    assert [(p.num, p.tau, p.seed, p.init_name) for p in back.particles_advected] == \
           [(p.num, p.tau, p.seed, p.init_name) for p in ref.particles_advected]


def test_cli_overrides_param_file_and_presets(tmp_path):
    m = cmm()
    pf = tmp_path / "p.txt"
    pf.write_text(goldens()["one_step"]["params_in"])
    sim = m.Simulation(["param_file=%s" % pf, "grid_coarse=64", "steps_per_sec=8", "final_time=0.5"])
    assert sim.file_name() == "one_step_4_nodes_C64_F512_t8_T0.5"
    assert sim.scalar("dt") == 1.0 / 8
    preset = m.Simulation([])
    assert preset.file_name() == "debug_4_nodes_C512_F2048_t20_T3"
    t = preset.settings_text()
    assert "freq_cut_psi\t=\t128\n" in t and "domain_bounds\t=\t{0,6.28319,0,6.28319,0,0}\n" in t


def test_errors_are_status_codes_not_exits(tmp_path):
    m = cmm()
    with pytest.raises(m.CmmError) as e:
        m.Simulation(["initial_condition=not_a_flow"])
    assert e.value.code == m.CMM_ERR_PARAM
    with pytest.raises(m.CmmError) as e:
        m.Simulation(["param_file=%s" % (tmp_path / "missing.txt")])
    assert e.value.code == m.CMM_ERR_IO
    sim = m.Simulation(["workspace=%s/" % tmp_path])
    with pytest.raises(m.CmmError) as e:
        sim.step(1)
    assert e.value.code == m.CMM_ERR_STATE
    # kernel API argument validation happens before any device work
    g = m.grid(16)
    bad = m.grid(0)
    rc = m.lib().cmm_incomp_max(C.byref(bad), C.byref(g), None, None, None, None)
    assert rc == m.CMM_ERR_PARAM
    assert "grid" in m.last_error()


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES") is None and os.path.exists("/dev/nvidia0"),
                    reason="a GPU is present; the no-GPU failure path is only observable without one")
def test_init_without_gpu_returns_cuda_error(tmp_path):
    m = cmm()
    sim = m.Simulation(["workspace=%s/" % tmp_path, "grid_coarse=16", "grid_fine=32", "grid_psi=16",
                        "grid_vort=32", "particles_advected_num=0", "verbose=0"])
    with pytest.raises(m.CmmError) as e:
        sim.init()
    assert e.value.code == m.CMM_ERR_CUDA


def test_fft_rejects_unsupported_shapes_before_any_gpu_work():
    """Shapes the library's FFT does not run are a status code at creation (checked
    before any CUDA call): odd row length, a prime factor above 13, too long a side."""
    m = cmm()
    for nx, ny in ((63, 64), (64, 17 * 4), (2 * 17, 64), (2 * 16384, 64), (64, 16384)):
        with pytest.raises(m.CmmError) as e:
            m.FFT(nx, ny, 0)
        assert e.value.code == m.CMM_ERR_PARAM, (nx, ny)
    with pytest.raises(m.CmmError):
        m.FFT(64, 64, 2)
