"""local_box's sub-image stack mode on the GPU (cryoim_local_box_extract) against the
oracle: the box geometry (equivalent orientations, box corners, fractions) bit-exact to
the FP32 restatement (same host arithmetic), the sub-images within 2e-5 of the FP64
restatement (unit-variance values; cuFFT FP32 against an FP64 FFT)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 2e-5


def _case(n=128, P=5, seed=21):
    import cryoim_gb300 as ci
    import synth
    rng = np.random.default_rng(seed)
    vol = synth.phantom(n, seed)
    e = synth.random_rotations(P, rng)
    imgs = synth.project_numpy(vol, e) + rng.normal(scale=0.5, size=(P, n, n))
    p = ci.particles(P)
    p["particle_id"] = p["img_id"] = p["img_particle_id"] = np.arange(1, P + 1)
    p["theta"], p["phi"], p["omega"] = e[:, 0], e[:, 1], e[:, 2]
    p["x"], p["y"] = rng.uniform(-5, 5, (2, P))
    p["pr"] = rng.uniform(20, 60, P)
    p["pr"][1] = 120.0  # not selected
    p["df1"], p["df2"], p["astigang"] = 1.8, 1.9, 40.0
    return imgs.astype(np.float32), p


@pytest.mark.parametrize("sym,loc,sub", [("c5", (0.0, 0.0, 30.0), 64), ("i5", (12.0, -7.5, 50.0), 48),
                                         ("i2", (55.0, 40.0, 10.0), 96)])
def test_local_box_extract_matches_oracle(built, orc, sym, loc, sub):
    import cryoim_gb300 as ci
    imgs, p = _case()
    s = ci.local_sym_matrices(sym)
    if sym == "i5":
        s = s[:12]
    with ci.Context(0, ci.default_params(128)) as c:
        got, rec = c.local_box_extract(imgs, p, s, loc, 1.25, sub)
    want32, rec32 = orc.local_box_extract(imgs, p, s, loc, 1.25, sub, fp="f32")
    want, rec64 = orc.local_box_extract(imgs, p, s, loc, 1.25, sub, fp="f64")
    assert len(rec) == len(rec32) == 4 * len(s)
    for f in ("particle_id", "img_id", "local_img_id", "local_hx0", "local_ky0", "local_theta0", "local_phi0",
              "local_omega0", "local_x0", "local_y0", "local_z0", "df1", "pr"):
        assert np.array_equal(rec[f], rec32[f]), f
    assert np.array_equal(rec["local_hx0"], rec64["local_hx0"])
    err = np.abs(got - want)
    assert err.max() < TOL, err.max()


def test_local_box_extract_device_equals_host(built):
    import torch
    import cryoim_gb300 as ci
    imgs, p = _case(P=4, seed=3)
    s = ci.local_sym_matrices("c5")
    with ci.Context(0, ci.default_params(128)) as c:
        h, rh = c.local_box_extract(imgs, p, s, (20.0, 5.0, 30.0), 1.0, 64)
        d_in = torch.from_numpy(imgs).cuda()
        d_out = torch.zeros((len(p) * len(s), 64, 64), device="cuda")
        _, rd = c.local_box_extract(d_in.data_ptr(), p, s, (20.0, 5.0, 30.0), 1.0, 64, d_out=d_out.data_ptr(),
                                    fftsize=128)
        torch.cuda.synchronize()
    assert np.array_equal(rh, rd)
    assert np.array_equal(h, d_out[: len(rd)].cpu().numpy())


def test_local_box_stack_mode_executable(built, tmp_path):
    """local_box local_imgstck=... on files: the sub-image stack and the 14-column rows
    as the library gives them for the particles the file holds."""
    import os
    import subprocess
    import cryoim_gb300 as ci
    from conftest import ROOT
    from test_io import lib, write_stack
    imgs, p = _case(P=4, seed=8)
    L = lib()
    write_stack(L, tmp_path / "stack.mrc", imgs, 1.25)
    with open(tmp_path / "icos.dat", "w") as f:
        for i, q in enumerate(p):
            f.write(f"{tmp_path / 'stack.mrc'} {i + 1} {q['theta']:.4f} {q['phi']:.4f} {q['omega']:.4f} "
                    f"{q['x']:.4f} {q['y']:.4f} {q['pr']:.4f} {q['img_id']} {i + 1} {q['df1']:.4f} "
                    f"{q['df2']:.4f} {q['astigang']:.4f}\n")
    r = subprocess.run([os.path.join(ROOT, "cryoim_gb300", "bin", "local_box"), f"icos_ort={tmp_path / 'icos.dat'}",
                        f"local_ort={tmp_path / 'loc.dat'}", f"local_imgstck={tmp_path / 'sub.mrc'}",
                        "local_x=10", "local_y=-4", "local_z=33", "apix=1.25", "sym=c5", "sub_FFTsize=48"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    parts = ci.particles(len(p))
    assert L.cryoim_ort_read(str(tmp_path / "icos.dat").encode(), 1, len(p), parts.ctypes.data, None, 0) == 0
    with ci.Context(0, ci.default_params(128)) as c:
        want, rec = c.local_box_extract(imgs, parts, ci.local_sym_matrices("c5"), (10.0, -4.0, 33.0), 1.25, 48)
    raw = open(tmp_path / "sub.mrc", "rb").read()
    hdr = np.frombuffer(raw[:12], np.int32)
    assert list(hdr) == [48, 48, 5 * len(p)]  # nz = Nsym x rows of icos_ort (loc_box.f90:29)
    got = np.frombuffer(raw[1024:], np.float32).reshape(-1, 48, 48)
    assert np.array_equal(got, want)
    rows = open(tmp_path / "loc.dat").read().splitlines()
    assert len(rows) == len(rec)
    for line, q in zip(rows, rec):
        assert len(line) == 64 + 8 + 60 + 12 + 6 + 30 + 12
        assert int(line[64:72]) == q["particle_id"]
        v = [float(line[72 + 10 * k:82 + 10 * k]) for k in range(6)]
        np.testing.assert_allclose(v, [q["local_theta0"], q["local_phi0"], q["local_omega0"], q["local_x0"],
                                       q["local_y0"], q["pr"]], atol=6e-5)
        assert int(line[132:144]) == q["img_id"] and int(line[144:150]) == q["local_img_id"]
        assert abs(float(line[180:192]) - q["local_z0"]) < 6e-5
