"""The oracle's restatement of local_box's sub-image stack mode (loc_box.f90:34-91),
pinned by known answers and by an independent numpy restatement.  No GPU needed."""
import numpy as np
import pytest


def _parts(n, seed, orc, x=None, y=None):
    rng = np.random.default_rng(seed)
    p = np.zeros(n, orc.PARTICLE_DTYPE)
    p["particle_id"] = p["img_id"] = p["img_particle_id"] = np.arange(1, n + 1)
    p["theta"], p["phi"], p["omega"] = rng.uniform(5, 175, n), rng.uniform(-170, 170, n), rng.uniform(-170, 170, n)
    p["x"] = rng.uniform(-4, 4, n) if x is None else x
    p["y"] = rng.uniform(-4, 4, n) if y is None else y
    p["pr"] = rng.uniform(10, 60, n)
    p["df1"], p["df2"], p["astigang"] = 1.5, 1.6, 20.0
    return p


def _numpy_extract(imgs, parts, sym, loc, apix, sub):
    """loc_box.f90 in numpy FP64: centre by the Fourier shift theorem, equalort, cut with
    wrap, normalise (the whole-image normalisation cancels in the sub-image's own)."""
    from synth import euler_mat
    n = imgs.shape[-1]
    h = np.arange(n) - n // 2
    ky, hx = np.meshgrid(h, h, indexing="ij")
    out, cents = [], []
    for img, q in zip(imgs, parts):
        F = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(img.astype(np.float64))))
        F *= np.exp(2j * np.pi * (q["x"] * hx + q["y"] * ky) / n)
        a = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(F))).real
        E = euler_mat(q["theta"], q["phi"], q["omega"])
        for S in sym.astype(np.float64):
            r = S @ E
            th = np.degrees(np.arccos(np.clip(r[2, 2], -1, 1)))
            ph = np.degrees(np.arctan2(r[1, 2], r[0, 2]))
            om = np.degrees(np.arctan2(r[2, 1], -r[2, 0]))
            c = euler_mat(th, ph, om).T @ np.asarray(loc, np.float64)
            hx0 = int(c[0]) + n // 2 - sub // 2
            ky0 = int(c[1]) + n // 2 - sub // 2
            rows = (np.arange(sub) + ky0) % n
            cols = (np.arange(sub) + hx0) % n
            b = a[np.ix_(rows, cols)]
            b = b - b.mean()
            out.append(b / np.sqrt((b * b).mean()))
            cents.append(c)
    return np.array(out), np.array(cents)


def test_delta_lands_at_the_box_centre(orc):
    n, sub = 64, 16
    img = np.zeros((1, n, n), np.float32)
    img[0, n // 2 - 5, n // 2 + 3] = 1.0
    p = _parts(1, 1, orc, x=3.0, y=-5.0)
    so, rec = orc.local_box_extract(img, p, np.eye(3, dtype=np.float32)[None], (0.0, 0.0, 0.0), 1.0, sub, fp="f64")
    assert so.shape == (1, sub, sub)
    assert np.unravel_index(np.argmax(so[0]), so[0].shape) == (sub // 2, sub // 2)
    assert rec["local_hx0"][0] == rec["local_ky0"][0] == n // 2 - sub // 2
    assert abs(so[0].mean()) < 1e-6 and abs(np.sqrt((so[0].astype(np.float64) ** 2).mean()) - 1) < 1e-6


@pytest.mark.parametrize("sym", ["c5", "i5"])
def test_stack_mode_matches_numpy_restatement(orc, sym):
    import cryoim_gb300 as ci
    n, sub = 64, 24
    rng = np.random.default_rng(5)
    imgs = rng.normal(size=(3, n, n)).astype(np.float32)
    p = _parts(3, 6, orc)
    s = ci.local_sym_matrices(sym)[:12]
    loc = (6.0, -9.5, 21.0)
    so, rec = orc.local_box_extract(imgs, p, s, loc, 1.5, sub, fp="f64")
    want, cents = _numpy_extract(imgs, p, s, loc, 1.5, sub)
    assert len(so) == len(want) == 3 * len(s)
    assert np.abs(so - want).max() < 1e-5
    np.testing.assert_allclose(rec["local_z0"], cents[:, 2] * 1.5, atol=1e-4)
    frac = cents[:, 0] - np.trunc(cents[:, 0])
    np.testing.assert_allclose(rec["local_x0"], frac, atol=1e-5)
    assert np.array_equal(rec["local_img_id"], np.tile(np.arange(1, len(s) + 1), 3))
    assert np.array_equal(rec["particle_id"], np.arange(1, len(so) + 1))


def test_selection_and_wrap(orc):
    n, sub = 32, 32
    rng = np.random.default_rng(9)
    imgs = rng.normal(size=(4, n, n)).astype(np.float32)
    p = _parts(4, 10, orc, x=np.zeros(4), y=np.zeros(4))
    p["pr"] = [10.0, 95.0, 20.0, 30.0]          # the second is above PR_threshold
    p["x"][3] = 150.0                            # the fourth is beyond boundX
    so, rec = orc.local_box_extract(imgs, p, np.eye(3, dtype=np.float32)[None], (0.0, 0.0, 0.0), 1.0, sub,
                                    pr_threshold=90.0, boundx=100.0, fp="f64")
    assert len(so) == 2 and list(rec["img_id"]) == [1, 3]
    # a box as large as the image is the whole centred image, wrapped into place
    a = imgs[0].astype(np.float64)
    a = (a - a.mean()) / np.sqrt(((a - a.mean()) ** 2).mean())
    assert np.abs(so[0] - a).max() < 1e-5
