"""Oracle restatement of the mode-3 centring (calc_center.f90, calc_center_selfrot180.f90,
img2d_lowpass.f90, guass_regression.f90, cross_correlation.f90, img3d_mask.f90): known
answers and independent numpy restatements."""
import numpy as np
import pytest

from _data import small_case


@pytest.mark.parametrize("dx0,dy0,c", [(0.3, -0.2, 0.7), (-0.45, 0.1, 1.3), (0.0, 0.0, 0.5)])
def test_gauss_regression_recovers_a_gaussian_peak(orc, dx0, dy0, c):
    j, i = np.meshgrid([-1, 0, 1], [-1, 0, 1], indexing="ij")
    z = np.exp(np.log(c) - ((i - dx0) ** 2 + (j - dy0) ** 2) / 1.7)
    dx, dy, cc = orc.gauss_regression(z, "f64")
    assert abs(dx - dx0) < 1e-12 and abs(dy - dy0) < 1e-12 and abs(cc - c) < 1e-12
    dx32, dy32, cc32 = orc.gauss_regression(z, "f32")
    assert abs(dx32 - dx0) < 1e-5 and abs(cc32 - c) < 1e-5


def test_lowpass_matches_numpy(orc):
    """img2d_FFT returns (Re, -Im) but its backward call reads (a, b) as Re + i Im, so a
    forward/backward pair conjugates the spectrum: the reference's low pass comes back
    scaled by 1/nx^2 and point-reflected about pixel (0, 0)."""
    n, lp = 32, 6
    a = np.random.default_rng(2).normal(size=(n, n))
    got = orc.lowpass(a, lp, "f64")
    k = np.arange(n) - n // 2
    H = np.exp(-(k[None, :] ** 2 + k[:, None] ** 2) / (2.0 * lp * lp))
    filt = np.real(np.fft.ifft2(np.fft.fft2(a) * np.fft.ifftshift(H))) / n ** 2
    want = np.roll(filt[::-1, ::-1], 1, axis=(0, 1))  # index i -> (n - i) mod n
    assert np.abs(got - want).max() < 1e-12 * np.abs(want).max() + 1e-15


def _centrosymmetric(n, sx, sy):
    """Gaussian blobs in +/- pairs about (n/2 + sx, n/2 + sy)."""
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    img = np.zeros((n, n))
    for px, py, a in [(5.0, 2.0, 1.0), (-3.0, 7.0, 0.6), (0.0, 0.0, 0.8), (9.0, -4.0, 0.5)]:
        for s in (1, -1):
            cx, cy = n / 2 + sx + s * px, n / 2 + sy + s * py
            img += a * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / 6.0)
    return img.astype(np.float32)


@pytest.mark.parametrize("sx,sy", [(1.5, -2.25), (-3.0, 0.75)])
def test_selfrot180_finds_the_centre_of_a_centrosymmetric_image(orc, sx, sy):
    import cryoim_gb300 as ci
    n = 64
    p = ci.default_params(n, apix=4.0, minRes=60.0, maxRes=12.0, imgmask=(n // 2 - 2) * 4.0)
    parts = ci.particles(1)
    out = orc.center(p, _centrosymmetric(n, sx, sy)[None], parts, None, "f64")
    assert abs(out[0, 0] - sx) < 0.15 and abs(out[0, 1] - sy) < 0.15, out
    assert out[0, 2] > 0.9


def test_calc_center_recovers_the_origin_of_projections(orc):
    """Noise-free projections (with CTF) at their true orientation, shifted by their
    origin: the centring against the model returns that origin (to a tenth of a pixel)."""
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(n=64, P=3, snr=0.0, apply_ctf=1)
    q = parts.copy()
    out = orc.center(p, imgs, q, vol, "f64")
    assert np.abs(out[:, 0] - parts["x"]).max() < 0.1, (out, parts["x"])
    assert np.abs(out[:, 1] - parts["y"]).max() < 0.1, (out, parts["y"])
    assert np.all(out[:, 2] > 0.9)
    out32 = orc.center(p, imgs, q, vol, "f32")
    assert np.abs(out32 - out).max() < 1e-3


def test_calc_center_without_ctf_keeps_the_reference_parity(orc):
    """Each img2d_FFT forward/backward pair point-reflects (see the low-pass test): the
    model's projection comes back reflected once by project2d_FT3dTo2d, once by the CTF
    pass and once by the low pass, the image once by its low pass.  With applyCTF=y the
    two agree; with applyCTF=n the projection is the image's mirror and the peak is lost
    (the reference's behaviour, kept)."""
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(n=64, P=3, snr=0.0, apply_ctf=0)
    out = orc.center(p, imgs, parts.copy(), vol, "f64")
    assert np.all(out[:, 2] < 0.5)
