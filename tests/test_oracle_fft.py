"""The oracle's FFT against numpy.fft (pocketfft): an independent DFT check."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("shape", [(8, 6, 4), (16, 16, 16), (12, 10, 16), (32, 96, 160), (64, 64, 64), (6, 20, 18)])
def test_r2c_matches_numpy(shape):
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(shape)
    s = O.fft_r2c(a)
    ref = np.fft.rfftn(a).transpose(1, 0, 2)  # reference layout [ky][kz][kx]
    assert np.abs(s - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("shape", [(8, 6, 4), (16, 12, 10), (32, 96, 160)])
def test_c2r_roundtrip_and_numpy(shape):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape)
    s = O.fft_r2c(a)
    b = O.fft_c2r(s, shape)
    assert np.abs(b / np.prod(shape) - a).max() < 1e-13
    # numpy irfftn uses the same projection onto Hermitian spectra
    ref = np.fft.irfftn(s.transpose(1, 0, 2), s=shape, axes=(0, 1, 2)) * np.prod(shape)
    assert np.abs(b - ref).max() < 1e-11 * np.abs(ref).max()


def test_c2r_ignores_imaginary_dc_and_nyquist_after_yz():
    # a multi-dimensional c2r uses Re of the kx=0 / kx=Nx/2 entries after the
    # complex y, z inverse: a purely imaginary constant there contributes 0
    shape = (8, 8, 8)
    s = np.zeros((8, 8, 5), np.complex128)
    s[0, 0, 0] = 1j
    s[0, 0, 4] = 2j
    assert np.abs(O.fft_c2r(s, shape)).max() == 0.0
