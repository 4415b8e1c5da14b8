"""The CPU oracle of the learned psi upsampler (no GPU): its FP64 gradients (mean squared
error and psi-space spectral loss) against central finite differences, its BF16 rounding,
its convolution against a direct numpy restatement of the periodic 3x3 stencil, and its
spectral loss against numpy's FFT."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle as O  # noqa: E402


def test_bf16_rounding_ties_to_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e-40, 65504.0])
    r = O.bf16_round(vals)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0 and r[4] == -2.5
    for v in vals:
        assert O._learned_lib().og_bf16_round(float(v)) == O.bf16_round(np.array([v]))[0]


def test_conv_matches_numpy_stencil():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(2, 5, 6, 3))
    w = rng.normal(size=(9, 3, 4))
    b = rng.normal(size=4)
    ref = np.zeros((2, 5, 6, 4)) + b
    for dy in range(3):
        for dx in range(3):
            sh = np.roll(np.roll(x, -(dy - 1), axis=1), -(dx - 1), axis=2)
            ref += sh @ w[3 * dy + dx]
    assert np.allclose(O.conv3x3(x, w, b), ref, rtol=1e-12, atol=1e-12)
    # input gradient = adjoint of the convolution: <conv(x), g> = <x, conv_t(g)>
    g = rng.normal(size=(2, 5, 6, 4))
    lhs = np.sum(O.conv3x3(x, w) * g)
    rhs = np.sum(x * O.conv3x3_input_grad(g, w))
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
    dw, db = O.conv3x3_weight_grad(x, g)
    # d<conv(x, w), g>/dw = dw
    e = 1e-6
    w2 = w.copy()
    w2[4, 1, 2] += e
    fd = (np.sum(O.conv3x3(x, w2) * g) - lhs) / e
    assert abs(fd - dw[4, 1, 2]) < 1e-5 * max(1.0, abs(fd))
    assert np.allclose(db, g.sum(axis=(0, 1, 2)))


import pytest  # noqa: E402


@pytest.mark.parametrize("cut", [0, 3])
def test_network_gradient_matches_finite_differences(cut):
    rng = np.random.default_rng(1 + cut)
    nb, C = 1, 32
    n = O.upsampler_param_count(nb, C)
    p = rng.normal(0, 0.1, n)
    inputs = rng.normal(0, 1, (1, 7, 4, 8)).astype(np.float32)
    targets = rng.normal(0, 1, (1, 8, 16)).astype(np.float32)
    s_in = np.array([1.0, 2.0, 0.5, 1.0, 3.0, 5.0, 4.0])
    loss, g = O.upsampler_loss_grad(p, nb, C, s_in, 0.5, inputs, targets, emulate_bf16=False, cut=cut)
    for i in rng.choice(n, 16, replace=False):
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        lp, _ = O.upsampler_loss_grad(pp, nb, C, s_in, 0.5, inputs, targets, emulate_bf16=False, cut=cut)
        lm, _ = O.upsampler_loss_grad(pm, nb, C, s_in, 0.5, inputs, targets, emulate_bf16=False, cut=cut)
        fd = (lp - lm) / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9 * np.max(np.abs(g)), (i, fd, g[i])


def test_spectral_loss_matches_numpy_fft():
    """The oracle's psi-space loss restated with numpy.fft on the network's shuffled output."""
    rng = np.random.default_rng(4)
    nb, C, cut = 0, 32, 4
    n = O.upsampler_param_count(nb, C)
    p = rng.normal(0, 0.1, n)
    inputs = rng.normal(0, 1, (2, 7, 4, 8)).astype(np.float32)
    targets = rng.normal(0, 1, (2, 8, 16)).astype(np.float32)
    s_in = np.ones(7)
    loss, _ = O.upsampler_loss_grad(p, nb, C, s_in, 1.0, inputs, targets, emulate_bf16=False, cut=cut)
    # forward by the oracle's convolutions: head then tail (no blocks)
    off = 9 * 16 * C
    wh, bh = p[:off].reshape(9, 16, C), p[off:off + C]
    off2 = off + C + 9 * C * 16
    wt, bt = p[off + C:off2].reshape(9, C, 16), p[off2:off2 + 16]
    x0 = np.zeros((2, 4, 8, 16))
    x0[..., :7] = inputs.transpose(0, 2, 3, 1)
    out = O.conv3x3(O.conv3x3(x0, wh, bh), wt, bt)
    pred = np.zeros((2, 8, 16))
    for k in range(4):
        pred[:, k // 2::2, k % 2::2] = out[..., k]
    ky = np.fft.fftfreq(8, 1.0 / 8)[:, None]
    kx = np.fft.fftfreq(16, 1.0 / 16)[None, :]
    k2 = kx ** 2 + ky ** 2
    wk = np.where((k2 > 0) & (k2 <= cut * cut), 1.0 / np.where(k2 > 0, k2, 1) ** 2, 0.0)
    num = np.sum(wk * np.abs(np.fft.fft2(pred - targets)) ** 2, axis=(1, 2))
    den = np.sum(wk * np.abs(np.fft.fft2(targets.astype(np.float64))) ** 2, axis=(1, 2))
    ref = np.mean(num / den)
    assert abs(loss - ref) <= 1e-10 * ref
