"""Known-answer tests of the oracle's 2D routines (FFT convention, CTF, origin shift,
amplitude-cut fit, mask, central section) and FP32-vs-FP64 agreement."""
import numpy as np
import pytest


@pytest.mark.parametrize("n", [32, 64, 48])
def test_fft_convention_matches_numpy(orc, n):
    """img2d_FFT.f90 + FFTW.f90:179-194: forward /N^2, returns (Re, -Im)."""
    rng = np.random.default_rng(n)
    a0, b0 = rng.normal(size=(2, n, n))
    a, b = orc.fft2d(a0, b0, 1, "f64")
    F = np.fft.fft2(a0 + 1j * b0) / (n * n)
    assert np.abs(a - F.real).max() < 1e-12 and np.abs(b + F.imag).max() < 1e-12
    a1, b1 = orc.fft2d(a0, b0, -1, "f64")
    G = np.fft.ifft2(a0 + 1j * b0) * (n * n)
    assert np.abs(a1 - G.real).max() < 1e-9 and np.abs(b1 + G.imag).max() < 1e-9
    a32, b32 = orc.fft2d(a0, b0, 1, "f32")
    assert np.abs(a32 - a).max() < 1e-5 * np.abs(a).max() + 1e-7


def test_fft3d_matches_numpy(orc):
    rng = np.random.default_rng(3)
    re, im = rng.normal(size=(2, 16, 16, 16))
    r, i = orc.fft3d(re, im, -1, "f64")
    F = np.fft.fftn(re + 1j * im)
    assert np.abs(r - F.real).max() < 1e-10 and np.abs(i - F.imag).max() < 1e-10


def test_ctf_matches_independent_formula(orc):
    from synth import ctf2d
    for args in [(1.5, 1.5, 0.0, 2.0), (2.0, 2.1, 37.0, 1.5)]:
        c64 = orc.ctf2d(64, *args, 300.0, 2.7, 0.07, fp="f64")
        ref = ctf2d(64, *args, 300.0, 2.7, 0.07)
        assert np.abs(c64 - ref).max() < 1e-9
        c32 = orc.ctf2d(64, *args, 300.0, 2.7, 0.07, fp="f32")
        assert np.abs(c32 - ref).max() < 2e-4
    # at zero frequency the phase is 0: ctf = -ampwg
    c = orc.ctf2d(32, 1.0, 1.0, 0.0, 2.0, 300.0, 2.7, 0.07, fp="f64")
    assert abs(c[16, 16] + 0.07) < 1e-12


def test_centshift_round_trip_and_shift_theorem(orc):
    n = 32
    rng = np.random.default_rng(4)
    a0, b0 = rng.normal(size=(2, n, n))
    a, b = orc.centshift(a0, b0, 2.5, -1.25, "f64")
    # the phase includes nx/2: undo with x' = -x - n
    a2, b2 = orc.centshift(a, b, -2.5 - n, 1.25 - n, "f64")
    assert np.abs(a2 - a0).max() < 1e-9 and np.abs(b2 - b0).max() < 1e-9
    # an object at (n/2 + x, n/2 + y) is re-referenced to its centre
    img = np.zeros((n, n))
    img[n // 2 + 3, n // 2 + 2] = 1.0  # x=2, y=3
    cb = np.where((np.add.outer(np.arange(n), np.arange(n)) % 2) == 1, -1.0, 1.0)
    a, b = orc.fft2d(img * cb, np.zeros((n, n)), 1, "f64")
    a, b = orc.centshift(a, b, 2.0, 3.0, "f64")
    assert np.allclose(a, 1.0 / (n * n), atol=1e-12) and np.allclose(b, 0.0, atol=1e-12)


def test_expfit_constant_amplitude(orc):
    n, mn, mx = 64, 3, 20
    a = np.full((n, n), 0.6)
    b = np.full((n, n), 0.8)
    f = orc.expfit(a, b, mn, mx, "f64")
    assert np.allclose(f, 0.8, atol=1e-9)  # 0.8 * |F| with |F| = 1


def test_expfit_exponential_profile(orc):
    n, mn, mx = 64, 4, 24
    ky, hx = np.meshgrid(np.arange(n) - n // 2, np.arange(n) - n // 2, indexing="ij")
    r = np.sqrt(hx ** 2 + ky ** 2)
    amp = np.exp(-0.1 * r + 1.0)
    f = orc.expfit(amp, np.zeros_like(amp), mn, mx, "f64")
    # Fcut is evaluated at each ring's mean radius (ky >= 0 half plane, |hx| <= maxR);
    # the ring mean of exp(-0.1 r) equals exp(-0.1 <r>) to within the ring's spread
    half = (ky >= 0) & (np.abs(hx) <= mx)
    rbar = np.array([r[half & (np.floor(r + 0.5) == k)].mean() for k in range(mn, mx + 1)])
    assert np.allclose(f / (0.8 * np.exp(-0.1 * rbar + 1.0)), 1.0, atol=2e-3)


def test_mask_edges(orc):
    n = 64
    img = np.ones((n, n))
    img[n // 2 - 10:n // 2 + 10, n // 2 - 10:n // 2 + 10] = 5.0
    m = orc.mask(img, 20.0, 0.0, 0.0, "f64")
    assert np.allclose(m[n // 2, n // 2], 5.0)
    assert np.allclose(m[0, 0], 1.0)  # outside R2: the edge-ring mean (ring lies in the ones)
    y, x = np.indices((n, n))
    r = np.hypot(x - n // 2, y - n // 2)
    assert np.allclose(m[r <= 17], img[r <= 17])


def test_central_section_of_point_source(orc):
    """A point at the map centre has a constant FT; every central section is constant
    inside radius nx/2-2 and zero outside."""
    n = 32
    fre = np.ones((n, n, n))
    fim = np.zeros((n, n, n))
    ore, oim = orc.central_section(fre, fim, 37.0, 12.0, 250.0, "f64")
    ky, hx = np.meshgrid(np.arange(n) - n // 2, np.arange(n) - n // 2, indexing="ij")
    inside = np.hypot(hx, ky) <= n // 2 - 2
    assert np.allclose(ore[inside], 1.0) and np.allclose(ore[~inside], 0.0)
    assert np.allclose(oim, 0.0)


def test_norm(orc):
    rng = np.random.default_rng(5)
    img = rng.normal(3.0, 2.0, size=(32, 32))
    o = orc.norm(img, "f64")
    assert abs(o.mean()) < 1e-12 and abs(np.sqrt((o ** 2).mean()) - 1) < 1e-12


def test_gaussian_section_known_answers(orc):
    """The Gaussian-kernel section: a constant map gives the constant inside the cut;
    at any orientation each sample equals the normalised 27-voxel sum restated in numpy."""
    n, sig = 32, 0.7
    c = np.full((n, n, n), 2.5)
    sr, si = orc.central_section_gauss(c, 0 * c, 17.0, -40.0, 123.0, sig)
    h = n // 2
    iy, ix = np.meshgrid(np.arange(n) - h, np.arange(n) - h, indexing="ij")
    inside = np.hypot(ix, iy) <= h - 2.5
    assert np.abs(sr[inside] - 2.5).max() < 1e-12 and np.abs(si).max() == 0.0
    rng = np.random.default_rng(4)
    fr, fi = rng.normal(size=(2, n, n, n))
    th, ph, om = 33.0, 71.0, -12.0
    sr, si = orc.central_section_gauss(fr, fi, th, ph, om, sig)
    R = orc.euler(th, ph, om, "f64")
    for (y, x) in [(3, 4), (-7, 2), (0, -9), (10, 1)]:
        X = R @ np.array([x, y, 0.0])
        c0 = np.rint(X).astype(int)
        acc, ws = 0j, 0.0
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    v = c0 + np.array([dx, dy, dz])
                    w = np.exp(-np.sum((X - v) ** 2) / (2 * sig * sig))
                    acc += w * (fr[v[2] + h, v[1] + h, v[0] + h] + 1j * fi[v[2] + h, v[1] + h, v[0] + h])
                    ws += w
        k = (y + h) * n + (x + h)
        assert abs(sr.ravel()[k] - (acc / ws).real) < 1e-12 and abs(si.ravel()[k] - (acc / ws).imag) < 1e-12
