"""The localized-reconstruction inputs (local_box's coordinate mode, local_refine's
refine_PR): symmetry sets, sub-particle coordinates against the oracle, the local
orientation files, and the oracle's refinement restatement."""
import numpy as np
import pytest


def _rot_ok(m, tol=2e-6):
    return (np.abs(m @ m.T - np.eye(3)).max() < tol) and abs(np.linalg.det(m) - 1) < tol


@pytest.mark.parametrize("sym,n", [("c1", 1), ("c5", 5), ("C12", 12), ("i2", 60), ("i3", 60), ("i5", 60)])
def test_local_symmetry_sets_are_groups(built, sym, n):
    import cryoim_gb300 as ci
    s = ci.local_sym_matrices(sym).astype(np.float64)
    assert len(s) == n and all(_rot_ok(m, 5e-6) for m in s)
    for a in s[: min(n, 12)]:
        for b in s[: min(n, 12)]:
            d = np.abs(s - a @ b).reshape(n, -1).max(1)
            assert d.min() < 5e-5  # closure
    assert np.abs(s - np.eye(3)).reshape(n, -1).max(1).min() < 5e-6  # contains the identity
    if sym.lower() == "i5":  # the 5-fold frame: a 72-degree turn about z
        c, sn = np.cos(np.radians(72.0)), np.sin(np.radians(72.0))
        rz = np.array([[c, -sn, 0], [sn, c, 0], [0, 0, 1]])
        assert np.abs(s - rz).reshape(n, -1).max(1).min() < 1e-5 or \
            np.abs(s - rz.T).reshape(n, -1).max(1).min() < 1e-5


def _parts(n, seed=3):
    import cryoim_gb300 as ci
    rng = np.random.default_rng(seed)
    p = ci.particles(n)
    p["particle_id"] = np.arange(1, n + 1)
    p["img_id"] = np.arange(1, n + 1)
    p["img_particle_id"] = np.arange(1, n + 1)
    p["theta"] = rng.uniform(5, 175, n)
    p["phi"] = rng.uniform(-179, 179, n)
    p["omega"] = rng.uniform(-179, 179, n)
    p["x"], p["y"] = rng.uniform(-3, 3, (2, n))
    p["pr"] = rng.uniform(10, 100, n)
    p["df1"], p["df2"], p["astigang"] = 1.5, 1.6, 30.0
    return p


@pytest.mark.parametrize("sym", ["c1", "c5", "i5"])
def test_local_box_coordinates_match_oracle(built, orc, sym):
    import cryoim_gb300 as ci
    p = _parts(12)
    s = ci.local_sym_matrices(sym)
    got = ci.local_box_coordinates(p, s, (30.0, -12.5, 41.0), 1.5, 256, pr_threshold=90.0, boundx=100.0)
    want = orc.local_box_coordinates(p, s, (30.0, -12.5, 41.0), 1.5, 256, 90.0, 100.0, "f64")
    sel = p["pr"] <= 90.0
    assert len(got) == len(want) == sel.sum() * len(s)
    assert np.array_equal(got["local_img_id"], want["local_img_id"])
    # the integer box centre can differ only where the FP32 coordinate sits on an integer
    d = (got["local_hx0"] + got["local_x0"]) - (want["local_hx0"] + want["local_x0"])
    assert np.abs(d).max() < 1e-3
    for f in ("local_theta0", "local_z0"):
        assert np.abs(got[f] - want[f]).max() < 2e-3, f
    for f in ("local_phi0", "local_omega0"):
        e = np.abs(got[f] - want[f])
        assert np.minimum(e, 360 - e).max() < 2e-3, f
    assert np.allclose(got["df1"], p["df1"][0] * 1e4)


def test_local_box_identity_keeps_the_particle(built):
    import cryoim_gb300 as ci
    p = _parts(5)
    p["pr"] = 10.0
    got = ci.local_box_coordinates(p, ci.local_sym_matrices("c1"), (0.0, 0.0, 0.0), 2.0, 128)
    assert np.allclose(got["local_theta0"], p["theta"], atol=1e-3)
    e = np.abs(got["local_phi0"] - p["phi"])
    assert np.minimum(e, 360 - e).max() < 1e-3
    cx = 64 + p["x"]
    assert np.array_equal(got["local_hx0"], np.trunc(cx).astype(np.int32))
    assert np.allclose(got["local_x0"], cx - np.trunc(cx), atol=1e-5)
    assert np.allclose(got["local_z0"], 0.0, atol=1e-4)


def test_local_ort_round_trip(built, tmp_path):
    import ctypes as C
    import cryoim_gb300 as ci
    from cryoim_gb300._abi import load
    L = load()
    q = ci.local_box_coordinates(_parts(4), ci.local_sym_matrices("c5"), (10.0, 5.0, 20.0), 1.0, 128,
                                 pr_threshold=1000.0)
    names = np.zeros((len(q), 64), np.uint8)
    for i in range(len(q)):
        names[i, :9] = np.frombuffer(b"stack.mrc", np.uint8)
    f = str(tmp_path / "loc.dat").encode()
    assert L.cryoim_local_ort_write(f, q.ctypes.data, names.ctypes.data, 64, len(q), 23, 0) == 0
    back = ci.local_particles(len(q))
    nb = np.zeros((len(q), 64), np.uint8)
    assert L.cryoim_local_ort_read(f, 1, len(q), back.ctypes.data, nb.ctypes.data, 64) == 0
    for fld in ("local_hx0", "local_ky0", "local_img_id", "particle_id"):
        assert np.array_equal(back[fld], q[fld])
    for fld in ("local_theta0", "local_x0", "local_z0", "df1"):
        assert np.allclose(back[fld], q[fld], atol=1e-4)
    assert bytes(nb[0][:9]) == b"stack.mrc"
    line = open(tmp_path / "loc.dat").readline()
    assert len(line.rstrip("\n")) == 64 + 8 + 60 + 12 + 6 + 30 + 10 + 9 + 12 + 50 + 22
    assert L.cryoim_local_ort_write(str(tmp_path / "r.dat").encode(), q.ctypes.data, names.ctypes.data, 64,
                                    len(q), 28, 0) == 0
    line = open(tmp_path / "r.dat").readline()
    assert len(line.rstrip("\n")) == 64 + 9 + 60 + 11 + 7 + 30 + 10 + 21 + 50 + 21 + 50


def local_case(n=32, n0=48, P=3, seed=11, snr=0.0, sign=1.0):
    """A blob map in an n box, whole images n0 x n0 holding its projections at known
    sub-particle orientations, centres and origins (noise-free unless snr); the content
    of each window is moved by sign x (local_x0, local_y0)."""
    import cryoim_gb300 as ci
    import synth
    rng = np.random.default_rng(seed)
    z, y, x = np.mgrid[0:n, 0:n, 0:n] - n // 2
    vol = np.zeros((n, n, n), np.float32)
    for _ in range(10):
        c = rng.uniform(-8, 8, 3)
        vol += rng.uniform(0.5, 1.5) * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / 4.0)
    e = np.stack([rng.uniform(20, 160, P), rng.uniform(-170, 170, P), rng.uniform(-170, 170, P)], 1)
    proj = synth.project_numpy(vol, e.astype(np.float32))
    q = ci.local_particles(P)
    imgs = np.zeros((P, n0, n0), np.float32)
    for i in range(P):
        hx0, ky0 = int(rng.integers(n // 2 + 2, n0 - n // 2 - 2)), int(rng.integers(n // 2 + 2, n0 - n // 2 - 2))
        sx, sy = rng.uniform(0, 1, 2)
        # sub-pixel shift by (sx, sy) in Fourier space, then paste centred at (hx0, ky0)
        k = np.fft.fftfreq(n)
        ph = np.exp(-2j * np.pi * sign * (k[None, :] * sx + k[:, None] * sy))
        sub = np.real(np.fft.ifft2(np.fft.fft2(proj[i]) * ph)).astype(np.float32)
        imgs[i, ky0 - n // 2:ky0 + n // 2, hx0 - n // 2:hx0 + n // 2] = sub
        if snr:
            imgs[i] += rng.normal(scale=np.sqrt(sub.var() / snr), size=(n0, n0)).astype(np.float32)
        q["particle_id"][i] = i + 1
        q["local_hx0"][i], q["local_ky0"][i] = hx0, ky0
        q["local_theta0"][i], q["local_phi0"][i], q["local_omega0"][i] = e[i]
        q["local_x0"][i], q["local_y0"][i] = sx, sy
        q["df1"][i] = q["df2"][i] = 15000.0
    return vol, imgs, q, e


def test_local_refine_oracle_fp32_agrees_with_fp64(orc):
    import cryoim_gb300 as ci
    vol, imgs, q, e = local_case()
    q["local_theta0"] += 2.0
    q["local_x0"] += 0.3
    lp = ci.local_params(32, 48, apix=2.0, max_res=8.0, ncycle=4, apply_ctf=0)
    r64 = orc.local_refine(lp, vol, imgs, q, "f64")
    r32 = orc.local_refine(lp, vol, imgs, q, "f32")
    for f in ("local_theta", "local_phi", "local_omega", "local_x", "local_y"):
        assert np.abs(r64[f] - r32[f]).max() < 1e-3, f
    assert np.abs(r64["local_pr"] - r32["local_pr"]).max() < 1e-3
    assert np.allclose(r64["local_dtheta"], r64["local_theta"] - q["local_theta0"], atol=1e-4)


def test_local_refine_oracle_conventions(orc):
    """refine_PR compares the model's central section in the standard sign (img3d_FFT.f90
    keeps +Im) with the sub-particle's img2d_FFT transform (-Im): data consistent with it
    are the point inversion of the map, with the window content at minus the origin.  On
    such data the oracle finds the origin with a low phase residual; the projected map
    itself scores near random phases."""
    import cryoim_gb300 as ci
    vol, imgs, q0, e = local_case(P=3, sign=-1.0)
    inv = np.roll(vol[::-1, ::-1, ::-1], 1, axis=(0, 1, 2))
    q = q0.copy()
    q["local_x0"] += 0.4
    lp = ci.local_params(32, 48, apix=2.0, max_res=6.0, ncycle=12, apply_ctf=0, refine_angle=1.0, refine_shift=0.5)
    r = orc.local_refine(lp, inv, imgs, q, "f64")
    assert np.abs(r["local_x"] - q0["local_x0"]).max() < 0.15
    assert np.abs(r["local_y"] - q0["local_y0"]).max() < 0.15
    assert r["local_pr"].max() < 10.0
    r2 = orc.local_refine(lp, vol, imgs, q, "f64")
    assert r2["local_pr"].min() > 30.0
