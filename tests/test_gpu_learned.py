"""The learned psi upsampler's tensor-core kernels and network against the CPU oracle.

Kernels (cmm_conv3x3, cmm_conv3x3_weight_grad): BF16 operands from the same random
values the oracle gets, so the only difference is the product's FP32 accumulation order
(checked at 1e-5 of the largest output); every channel pair the network uses, the fused
epilogue (bias, ReLU, ReLU mask, residual), several images per batch (the periodic wrap
is per image) and strips of rows that cross image boundaries.

Network (cmm_upsampler_loss_grad): loss and every layer's gradient, for the mean squared
error and for the psi-space spectral loss training uses, against the oracle's network with
BF16 rounding at the points where the product stores BF16 (weights, input, activations,
output gradient, propagated gradients).  Where an FP32 sum lands on the other
side of a BF16 rounding boundary the two round differently, so the gradients are compared
in relative L2 per layer (2e-2), each bias gradient channel by channel against a bound derived
from that rounding, and the loss to 1e-3.
"""
import os
import sys

import numpy as np
import pytest

from product import cmm

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle as O  # noqa: E402  (the CPU oracle)


def _bf16(rng, shape, scale=1.0):
    v = O.bf16_round(rng.normal(0.0, scale, size=shape))
    return v, O.bf16_bits(v)


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32), (32, 16), (16, 16)])
@pytest.mark.parametrize("flags", ["plain", "bias_relu", "mask_res"])
def test_conv3x3_matches_oracle(cin, cout, flags):
    m = cmm()
    rng = np.random.default_rng(cin * 100 + cout + len(flags))
    B, H, W = 3, 7, 256
    x, xb = _bf16(rng, (B, H, W, cin))
    w, wb = _bf16(rng, (9, cin, cout), 0.2)
    bias = rng.normal(0, 1, cout).astype(np.float32) if flags == "bias_relu" else None
    mask = res = maskb = resb = None
    if flags == "mask_res":
        mask, maskb = _bf16(rng, (B, H, W, cout))
        res, resb = _bf16(rng, (B, H, W, cout))
    out, outb = m.conv3x3(xb, wb, bias, maskb, resb, relu=(flags == "bias_relu"))
    ref = O.conv3x3(x, w, bias, mask, res, relu=(flags == "bias_relu"))
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(out - ref)) <= 1e-5 * scale
    assert np.array_equal(O.bf16_bits(O.bf16_round(out)), outb)   # the epilogue's BF16 store


@pytest.mark.parametrize("B,H,W", [(2, 70, 1024), (1, 512, 512)])
def test_conv3x3_tall_strips_match_oracle(B, H, W):
    """Images wide enough that the persistent grid takes strips of several rows (4 rows for
    70 x 1024 with a 2-row last strip, 14 rows for 512 x 512 with an 8-row last strip): the
    source-row accumulators of a strip, their release counts and the periodic wrap at
    both image edges."""
    m = cmm()
    rng = np.random.default_rng(H + W)
    x, xb = _bf16(rng, (B, H, W, 32))
    w, wb = _bf16(rng, (9, 32, 32), 0.2)
    bias = rng.normal(0, 1, 32).astype(np.float32)
    res, resb = _bf16(rng, (B, H, W, 32))
    out, outb = m.conv3x3(xb, wb, bias, None, resb, relu=True)
    ref = O.conv3x3(x, w, bias, None, res, relu=True)
    assert np.max(np.abs(out - ref)) <= 1e-5 * np.max(np.abs(ref))
    assert np.array_equal(O.bf16_bits(O.bf16_round(out)), outb)


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32), (32, 16), (16, 16)])
def test_conv3x3_weight_grad_matches_oracle(cin, cout):
    m = cmm()
    rng = np.random.default_rng(7 + cin + cout)
    B, H, W = 3, 70, 256      # 210 rows x 2 segments: strips of 3 rows crossing image boundaries
    x, xb = _bf16(rng, (B, H, W, cin))
    dy, dyb = _bf16(rng, (B, H, W, cout), 1e-3)
    dw, db = m.conv3x3_weight_grad(xb, dyb)
    rw, rb = O.conv3x3_weight_grad(x, dy)
    assert np.max(np.abs(dw - rw)) <= 1e-5 * np.max(np.abs(rw))
    assert np.max(np.abs(db - rb)) <= 1e-5 * np.max(np.abs(rb))


def test_input_gradient_is_the_flipped_convolution():
    """The network's input gradient runs the forward kernel on flipped, channel-swapped
    weights: check that restatement against the oracle's transposed convolution."""
    rng = np.random.default_rng(3)
    m = cmm()
    B, H, W, cin, cout = 2, 5, 128, 32, 16
    w, _ = _bf16(rng, (9, cin, cout), 0.2)
    dy, dyb = _bf16(rng, (B, H, W, cout))
    wflip = np.ascontiguousarray(w[::-1].transpose(0, 2, 1))      # tap' = 8 - tap, [co][ci]
    out, _ = m.conv3x3(dyb, O.bf16_bits(wflip))
    ref = O.conv3x3_input_grad(dy, w)
    assert np.max(np.abs(out - ref)) <= 1e-5 * np.max(np.abs(ref))


def _net_case(blocks, seed, B=2, h=8, w=128):
    rng = np.random.default_rng(seed)
    m = cmm()
    u = m.Upsampler(blocks=blocks, seed=seed)
    p = u.params().astype(np.float64)
    n = p.size
    # random biases (the product starts them at zero) so every path carries signal
    layers = [(16, 32)] + [(32, 32)] * (2 * blocks) + [(32, 16)]
    off = 0
    for li, (ci, co) in enumerate(layers):
        off += 9 * ci * co
        p[off:off + co] = rng.normal(0, 0.05, co) * (1 if li + 1 < len(layers) else (np.arange(co) < 4))
        off += co
    assert off == n == O.upsampler_param_count(blocks, 32)
    u.set_params(p.astype(np.float32))
    s_in = [1.5, 0.7, 0.8, 2.0, 3.0, 9.0, 11.0]
    u.set_scales(s_in, 0.01)
    inputs = rng.normal(0, 1, (B, 7, h, w)).astype(np.float32) * np.array(s_in, dtype=np.float32)[None, :, None, None]
    targets = (0.01 * rng.normal(0, 1, (B, 2 * h, 2 * w))).astype(np.float32)
    return u, p.astype(np.float32).astype(np.float64), s_in, inputs, targets, layers


@pytest.mark.parametrize("blocks,cut", [(1, 0), (2, 0), (1, 5), (2, 3)])
def test_network_loss_and_gradient_match_oracle(blocks, cut):
    """cut 0: mean squared error; cut > 0: the psi-space spectral loss of training (batched
    transforms on the GPU, a direct DFT in the oracle)."""
    u, p, s_in, inputs, targets, layers = _net_case(blocks, 11 + blocks + cut)
    loss = u.loss_grad(inputs, targets, cut=cut)
    g = u.grads().astype(np.float64)
    lo, go, dy_sq = O.upsampler_loss_grad(p, blocks, 32, s_in, 0.01, inputs, targets, emulate_bf16=True, cut=cut,
                                          dy_sq=True)
    assert abs(loss - lo) <= 1e-3 * lo
    off = 0
    for li, (ci, co) in enumerate(layers):
        # a layer's weights and bias together in relative L2
        n_el = 9 * ci * co + co
        a, b = g[off:off + n_el], go[off:off + n_el]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b), (li, np.linalg.norm(a - b) / np.linalg.norm(b))
        # each bias gradient, channel by channel: db_c = sum over pixels of the BF16 output
        # gradient dy_c.  The product and the oracle round the same values, reached by sums in
        # another order, so an element may land one BF16 step (at most 2^-7 of |dy|) on the other
        # side; with independent signs the sum of n such steps stays within 6 sigma of
        # 2^-7 sqrt(sum dy_c^2).  (A bias gradient under the spectral loss nearly cancels, so a
        # relative bound on it would be meaningless; this one is absolute and holds for both losses.)
        ab, bb, sq = a[-co:], b[-co:], dy_sq[off + n_el - co:off + n_el]
        bound = 6.0 * 2.0 ** -7 * np.sqrt(sq) + 1e-6 * np.abs(bb)
        assert np.all(np.abs(ab - bb) <= bound), (li, float(np.max(np.abs(ab - bb) / np.maximum(bound, 1e-300))))
        assert np.all(ab[sq == 0] == 0), li
        off += n_el
    # unused channels carry no gradient: head inputs 7..15, tail outputs 4..15
    head = g[:9 * 16 * 32].reshape(9, 16, 32)
    assert np.all(head[:, 7:, :] == 0)
    tail_off = off - (9 * 32 * 16 + 16)
    tail = g[tail_off:tail_off + 9 * 32 * 16].reshape(9, 32, 16)
    assert np.all(tail[:, :, 4:] == 0) and np.all(g[off - 16 + 4:off] == 0)
    u.close()


def test_network_gradient_agrees_with_fp64_direction():
    """Against the oracle's unrounded FP64 gradient (itself checked by finite differences
    in test_learned_oracle.py): the BF16 network's gradient points the same way."""
    u, p, s_in, inputs, targets, _ = _net_case(1, 5)
    u.loss_grad(inputs, targets)
    g = u.grads().astype(np.float64)
    _, go = O.upsampler_loss_grad(p, 1, 32, s_in, 0.01, inputs, targets, emulate_bf16=False)
    cos = float(g @ go / (np.linalg.norm(g) * np.linalg.norm(go)))
    assert cos > 0.999, cos
    u.close()
