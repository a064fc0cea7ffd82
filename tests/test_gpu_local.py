"""local_refine on the GPU (cryoim_local_refine) against the oracle's refine_PR
restatement, and the local_box -> local_refine executables on files.

Tolerances: every refined orientation within 1e-3 degree and origin within 1e-3 px of
the FP32 oracle (the descent takes the same branch at every step), final phase
residuals within 1e-3 relative; the FP64 oracle ends on the same candidates.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from test_local import local_case

pytestmark = pytest.mark.gpu
BIN = os.path.join(ROOT, "cryoim_gb300", "bin")


def consistent_case(P=6, seed=11, snr=0.0):
    """Sub-particles as local_refine's conventions see them: the model is the point
    inversion of the projected map and the content sits at minus the local origin."""
    vol, imgs, q, e = local_case(P=P, seed=seed, snr=snr, sign=-1.0)
    inv = np.roll(vol[::-1, ::-1, ::-1], 1, axis=(0, 1, 2))
    return inv, imgs, q


def _compare(got, want):
    for f in ("local_theta", "local_phi", "local_omega", "local_x", "local_y"):
        assert np.abs(got[f] - want[f]).max() < 1e-3, (f, got[f], want[f])
    assert np.abs(got["local_pr"] - want["local_pr"]).max() < 1e-3 * max(1.0, np.abs(want["local_pr"]).max())
    for f in ("local_dtheta", "local_dx"):
        assert np.abs(got[f] - want[f]).max() < 1e-3


@pytest.mark.parametrize("nsym,ctf", [(1, 0), (5, 0), (1, 1), (5, 1)])
def test_local_refine_matches_oracle(built, orc, nsym, ctf):
    import cryoim_gb300 as ci
    vol, imgs, q = consistent_case()
    q["local_theta0"] += 1.5
    q["local_phi0"] -= 1.0
    q["local_x0"] += 0.4
    lp = ci.local_params(32, 48, apix=2.0, max_res=6.0, ncycle=8, apply_ctf=ctf, nsym=nsym,
                         refine_angle=1.0, refine_shift=0.5)
    got = q.copy()
    with ci.Context(0) as ctx:
        ctx.local_refine(lp, vol, imgs, got)
    _compare(got, orc.local_refine(lp, vol, imgs, q, "f32"))
    w64 = orc.local_refine(lp, vol, imgs, q, "f64")
    same = np.abs(got["local_theta"] - w64["local_theta"]) < 1e-3
    assert same.mean() >= 5 / 6


def test_local_refine_recovers_the_origin(built):
    """On data that follow local_refine's own conventions the refinement finds the
    sub-particle origin and a low phase residual."""
    import cryoim_gb300 as ci
    vol, imgs, q0 = consistent_case(P=4)
    q = q0.copy()
    q["local_x0"] += 0.4
    lp = ci.local_params(32, 48, apix=2.0, max_res=6.0, ncycle=12, apply_ctf=0, refine_angle=1.0,
                         refine_shift=0.5)
    with ci.Context(0) as ctx:
        ctx.local_refine(lp, vol, imgs, q)
    assert np.abs(q["local_x"] - q0["local_x0"]).max() < 0.15
    assert np.abs(q["local_y"] - q0["local_y0"]).max() < 0.15
    assert q["local_pr"].max() < 10.0


def test_local_box_and_local_refine_executables(built, tmp_path):
    """local_box (coordinate mode) then local_refine on files: rows as the library gives."""
    import cryoim_gb300 as ci
    from test_io import lib, write_stack
    vol, imgs, q = consistent_case(P=3)
    L = lib()
    write_stack(L, tmp_path / "parts.mrc", imgs, 2.0)
    write_stack(L, tmp_path / "local.mrc", vol, 2.0)
    # whole-particle rows whose local_box output reproduces q's boxes: identity symmetry,
    # local point at the origin, the sub-particle centre carried by the particle origin;
    # stack names relative (the local files hold 64 characters of name, format a64)
    with open(tmp_path / "icos.dat", "w") as f:
        for i in range(len(q)):
            x = q["local_hx0"][i] + q["local_x0"][i] - 24
            y = q["local_ky0"][i] + q["local_y0"][i] - 24
            f.write(f"parts.mrc {i + 1} {q['local_theta0'][i]:.4f} {q['local_phi0'][i]:.4f} "
                    f"{q['local_omega0'][i]:.4f} {x:.4f} {y:.4f} 10.0 {i + 1} {i + 1} 1.5 1.5 0.0\n")
    r = subprocess.run([os.path.join(BIN, "local_box"), f"icos_ort={tmp_path / 'icos.dat'}",
                        f"local_ort={tmp_path / 'loc.dat'}", "local_x=0", "local_y=0", "local_z=0", "apix=2.0",
                        "sym=c1"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([os.path.join(BIN, "local_refine"), f"local_ort0={tmp_path / 'loc.dat'}",
                        f"local_newort={tmp_path / 'new.dat'}", f"model3d={tmp_path / 'local.mrc'}", "apix=2.0",
                        "maxRes=6.0", "Ncycle=6", "applyCTF=n", "refine_angle=1.0", "refine_shift=0.5"],
                       capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = [line.split() for line in open(tmp_path / "new.dat")]
    assert len(rows) == len(q) and all(len(t) == 28 for t in rows)
    got = np.array([[float(t[16]), float(t[19]), float(t[20]), float(t[22])] for t in rows])
    back = ci.local_particles(len(q))
    assert L.cryoim_local_ort_read(str(tmp_path / "loc.dat").encode(), 1, len(q), back.ctypes.data, None, 0) == 0
    lp = ci.local_params(32, 48, apix=2.0, max_res=6.0, ncycle=6, apply_ctf=0, refine_angle=1.0, refine_shift=0.5)
    with ci.Context(0) as ctx:
        ctx.local_refine(lp, vol, imgs, back)
    assert np.allclose(got[:, 0], back["local_theta"], atol=2e-4)
    assert np.allclose(got[:, 1], back["local_x"], atol=2e-4) and np.allclose(got[:, 3], back["local_pr"], atol=2e-4)
