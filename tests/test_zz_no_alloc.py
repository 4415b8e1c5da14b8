"""GPU test of cmm_diagnostics_noalloc, the diagnostics entry point that keeps
its reduction scratch in a fixed in-library device array instead of
allocating.  It must give the results of cmm_diagnostics (same grids, same
inputs) to rounding, on consecutive calls that reuse the scratch, and reject
grids larger than its scratch before launching anything.

The file is named to be collected last, so the entry point is also exercised
after every other test has run in the same process.
"""
import numpy as np
import pytest

from product import cmm

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 1e-12   # sums of squares grouped differently; max|omega| is exact


def _fields(n_psi, n_coarse, seed):
    rng = np.random.default_rng(seed)
    psi = torch.tensor(rng.standard_normal(4 * n_psi * n_psi), dtype=torch.float64, device="cuda")
    vort = torch.tensor(rng.standard_normal(n_coarse * n_coarse) * 3.0, dtype=torch.float64, device="cuda")
    return psi, vort


def _numpy_diagnostics(psi, vort, n_psi, n_coarse):
    p = psi.cpu().numpy().reshape(4, -1)
    w = vort.cpu().numpy()
    hp, hc = 2 * np.pi / n_psi, 2 * np.pi / n_coarse
    return [0.5 * hp * hp * float(np.sum(p[1] ** 2) + np.sum(p[2] ** 2)), 0.5 * hc * hc * float(np.sum(w * w)),
            float(np.max(np.abs(w)))]


def _close(a, b):
    for x, y in zip(a, b):
        assert abs(x - y) <= RTOL * abs(y), (a, b)


def test_noalloc_matches_diagnostics_on_consecutive_calls():
    m = cmm()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(256, 128, 1), (100, 300, 2), (1448, 2048, 3)]   # last: the scratch's maximum sizes
    for n_psi, n_coarse, seed in cases:
        gp, gc = m.grid(n_psi), m.grid(n_coarse)
        psi, vort = _fields(n_psi, n_coarse, seed)
        want = m.diagnostics(gp, psi, gc, vort, stream)
        first = m.diagnostics_noalloc(gp, psi, gc, vort, stream)
        second = m.diagnostics_noalloc(gp, psi, gc, vort, stream)
        _close(first, want)
        _close(_numpy_diagnostics(psi, vort, n_psi, n_coarse), want)
        assert first == second, "the second call over the reused scratch must repeat the first"


def test_noalloc_leaves_device_memory_untouched():
    """After the first call on the device (which looks up the scratch array's address), calls
    at the largest sizes change the device's free memory by nothing: no allocation, cached
    or leaked, happens inside the entry point."""
    m = cmm()
    stream = torch.cuda.current_stream().cuda_stream
    gp, gc = m.grid(1448), m.grid(2048)
    psi, vort = _fields(1448, 2048, 5)
    m.diagnostics_noalloc(gp, psi, gc, vort, stream)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        m.diagnostics_noalloc(gp, psi, gc, vort, stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_grids_beyond_its_scratch():
    m = cmm()
    psi, vort = _fields(8, 8, 4)
    stream = torch.cuda.current_stream().cuda_stream
    for n_psi, n_coarse in ((1449, 64), (64, 2049)):
        with pytest.raises(m.CmmError) as e:
            m.diagnostics_noalloc(m.grid(n_psi), psi, m.grid(n_coarse), vort, stream)
        assert e.value.code == m.CMM_ERR_PARAM
        assert "too large" in m.last_error()
    # the entry point stays usable after a rejection
    gp, gc = m.grid(8), m.grid(8)
    _close(m.diagnostics_noalloc(gp, psi, gc, vort, stream), m.diagnostics(gp, psi, gc, vort, stream))
