"""Algorithmic work of one CMM Euler time step: compulsory HBM bytes and
counted FP64 FLOPs per kernel, the denominators of the roofline figures.

Bytes = each distinct input array read once and each output written once.
`w` is the word of the map / Hermite nodes (8 for the plain FP64 form, 4 for
the mixed form, whose maps, psi and fine vorticity are FP32); spectra are
complex words (2w).  Grid sizes are sides: N_c coarse (map), N_f fine,
N_v vorticity (the psi solve's source grid), N_psi; L psi levels; P tracers.

FLOPs follow the reference's arithmetic (FMA = 2): 1D cubic weights 20,
tensor weights 16, one 16-term plane contraction 32, value interpolation 88,
map (diffeo) interpolation 120, velocity gradient over n_l levels
112 + 64 n_l, det grad X 243, RK arithmetic 30 per footpoint, FFT
2.5 N log2 N per real transform.  The operations they count are in
src/numerical/cmm-hermite.cu:30-503 (interpolation), src/numerical/cmm-timestep.cu:175-207
(RK3), src/simulation/cmm-simulation-kernel.cu:159-173,207-298,402-461 (the kernels).
"""
import math


def _sizes(cfg):
    return (cfg["grid_coarse"] ** 2, cfg["grid_fine"] ** 2, cfg["grid_vort"], cfg["grid_psi"],
            cfg.get("lagrange_levels", 3), cfg.get("particles", 0))


def step_bytes(cfg, w=8):
    """Compulsory bytes per time step, by kernel."""
    Nc2, Nf2, nv, npsi, L, P = _sizes(cfg)
    c = 2 * w                                   # complex word
    spec_v = nv * (nv // 2 + 1)
    spec_p = npsi * (npsi // 2 + 1)
    return {
        "advect": w * (8 * Nc2 + 4 * L * npsi * npsi + 8 * Nc2),
        "incomp": w * 8 * Nc2,
        "sample_vort": w * (8 * Nc2 + 4 * Nf2) + w * nv * (nv + 2),
        "fft_forward": w * nv * (nv + 2) + c * spec_v,
        "spectral": c * spec_p * 5,
        "fft_inverse4": 4 * c * spec_p + 4 * w * npsi * npsi,
        "coarse": w * (8 * Nc2 + 4 * Nf2) + 8 * Nc2,
        "particles": 32 * P + w * 4 * L * npsi * npsi,
    }


def step_flops(cfg, nfoot=8):
    """Counted FP64-convention FLOPs per time step, by kernel."""
    Nc2, Nf2, nv, npsi, L, P = _sizes(cfg)
    grad_L, grad_1 = 112 + 64 * L, 112 + 64
    fft = lambda n: 2.5 * n * n * math.log2(n * n)
    return {
        "advect": nfoot * (grad_L + grad_L + grad_1 + 120 + 30) * Nc2 + 128 * Nc2,
        "incomp": 243 * Nf2,
        "sample_vort": 208 * nv * nv,
        "coarse": 208 * Nc2,
        "ffts": fft(nv) + 4 * fft(npsi),
        "particles": (grad_1 + grad_L + grad_1 + 40) * P,
    }


def remap_flops(cfg, n_maps):
    """FLOPs of one remap at stack depth n_maps (composition through every
    sub-map plus the initial-condition evaluation) on the fine grid."""
    Nf2 = cfg["grid_fine"] ** 2
    return (120 * (n_maps + 1) + 88) * Nf2


def remap_bytes(cfg, n_maps, w=8):
    """Compulsory bytes of one fused remap: every sub-map read once, the fine
    vorticity Hermite written once."""
    Nc2, Nf2 = cfg["grid_coarse"] ** 2, cfg["grid_fine"] ** 2
    return w * 8 * Nc2 * (n_maps + 1) + w * 4 * Nf2


# the loop phases the library times with CUDA events, as sums of the kernels above
PHASES = {
    "advect": ("advect",),
    "incomp": ("incomp",),
    "psi": ("sample_vort", "fft_forward", "spectral", "fft_inverse4"),
    "coarse": ("coarse",),
    "particles": ("particles",),
}


def phase_bytes(cfg, w=8):
    b = step_bytes(cfg, w)
    return {ph: sum(b[k] for k in ks) for ph, ks in PHASES.items()}
