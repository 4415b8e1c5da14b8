"""The library's own FFT (csrc/fft.cu) through the C-ABI against numpy's.

Forward: the unnormalised 2D R2C of ny x nx reals equals numpy.fft.rfft2.
Inverse: the unnormalised C2R equals the column inverse transform followed by the
row C2R with the imaginary parts of the kx = 0 and kx = nx/2 columns dropped
(cuFFT's and the CPU oracle's convention), times ny * nx.

Tolerances: relative L-infinity against the largest output magnitude,
2e-15 * log2(N) in FP64 (rounding of a Stockham FFT grows like log N) and
3e-7 * log2(N) in FP32.  Lengths cover the radix families (powers of two,
3 * 2^k of the ensemble sizes, factors 5, 7, 11, 13), the longest rows (16384
reals) and columns (8192), batches, and the psi solve's sizes; FP32 rows of 256 to
4096 reals run the compile-time-length kernel.
"""
import numpy as np
import pytest

from product import cmm

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SHAPES = [(64, 64), (128, 96), (96, 128), (256, 256), (384, 192), (1024, 1024), (2048, 2048), (60, 40),
          (154, 52), (70, 26), (16384, 4), (8, 8192), (4, 4096), (4096, 16), (512, 8)]


def tol(nx, ny, prec):
    return (2e-15 if prec == 0 else 3e-7) * np.log2(nx * ny)


def _c2r_reference(Y, nx):
    Z = np.fft.ifft(Y, axis=-2) * Y.shape[-2]
    Z[..., 0] = Z[..., 0].real
    Z[..., nx // 2] = Z[..., nx // 2].real
    return np.fft.irfft(Z, n=nx, axis=-1) * nx


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("shape", SHAPES)
def test_fft_matches_numpy(shape, prec):
    m = cmm()
    nx, ny = shape
    batch = 3 if nx * ny <= 1 << 20 else 1
    rng = np.random.default_rng(nx * 7 + ny)
    x = rng.standard_normal((batch, ny, nx))
    dt_r = torch.float64 if prec == 0 else torch.float32
    dt_c = torch.complex128 if prec == 0 else torch.complex64
    f = m.FFT(nx, ny, prec)
    xin = torch.from_numpy(x).to(dt_r).cuda()
    X = torch.empty((batch, ny, nx // 2 + 1), dtype=dt_c, device="cuda")
    f.r2c(xin, X, batch)
    torch.cuda.synchronize()
    ref = np.fft.rfft2(xin.cpu().double().numpy())
    got = X.cpu().numpy().astype(np.complex128)
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err < tol(nx, ny, prec), ("r2c", err)
    Y = rng.standard_normal((batch, ny, nx // 2 + 1)) + 1j * rng.standard_normal((batch, ny, nx // 2 + 1))
    yin = torch.from_numpy(Y).to(dt_c).cuda()
    yref = _c2r_reference(yin.cpu().numpy().astype(np.complex128), nx)
    out = torch.empty((batch, ny, nx), dtype=dt_r, device="cuda")
    f.c2r(yin, out, batch)
    torch.cuda.synchronize()
    err = np.max(np.abs(out.cpu().double().numpy() - yref)) / np.max(np.abs(yref))
    assert err < tol(nx, ny, prec), ("c2r", err)
    f.close()


def test_fft_round_trip_is_identity_times_n():
    """C2R(R2C(x)) = N x at the psi solve's size, FP64."""
    m = cmm()
    nx = ny = 1024
    rng = np.random.default_rng(5)
    x = torch.from_numpy(rng.standard_normal((ny, nx))).cuda()
    f = m.FFT(nx, ny, 0)
    X = torch.empty((ny, nx // 2 + 1), dtype=torch.complex128, device="cuda")
    y = torch.empty_like(x)
    f.r2c(x, X)
    f.c2r(X, y)
    torch.cuda.synchronize()
    assert float(torch.max(torch.abs(y / (nx * ny) - x))) < 1e-13 * float(torch.max(torch.abs(x)))
    f.close()
