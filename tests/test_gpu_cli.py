"""The drop-in executables on real files: icosprocess modes 0/1/4/5 (+ contract=y),
merge_icosprocess_subrec, against the library entry points on the same inputs."""
import os
import subprocess

import numpy as np
import pytest

from _data import small_case
from conftest import ROOT
from test_io import lib, write_stack

pytestmark = pytest.mark.gpu
BIN = os.path.join(ROOT, "cryoim_gb300", "bin")


def read_rows(path):
    out = []
    for line in open(path).read().splitlines():
        v = [float(line[62 + 10 * k:72 + 10 * k]) for k in range(6)]  # theta phi omega x y PR
        out.append(v)
    return np.array(out)


def read_map(path, n):
    raw = open(path, "rb").read()
    return np.frombuffer(raw[1024:], np.float32).reshape(n, n, n)


@pytest.fixture(scope="module")
def files(built, tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    p, vol, tmpl, timgs, imgs, parts, truth = small_case()
    L = lib()
    write_stack(L, d / "stack.mrc", imgs, p.apix)
    write_stack(L, d / "tmpl.mrc", timgs, p.apix)
    write_stack(L, d / "model.mrc", vol, p.apix)
    with open(d / "ort.dat", "w") as f:
        for i, q in enumerate(parts):
            f.write(f"{d / 'stack.mrc'} {i + 1} {q['theta']:.4f} {q['phi']:.4f} {q['omega']:.4f} "
                    f"{q['x']:.6f} {q['y']:.6f} 10.0 {q['img_id']} {i + 1} {q['df1']:.6f} {q['df2']:.6f} "
                    f"{q['astigang']:.6f}\n")
    with open(d / "tort.dat", "w") as f:
        for t in tmpl:
            f.write(f"{t['particle_id']} {t['theta']:.6f} {t['phi']:.6f} {t['omega']:.6f} 0 0\n")
    common = [f"ortfile={d / 'ort.dat'}", "apix=4.0", "minRes=60", "maxRes=12", "searchstep=4",
              f"imgmask={(p.fftsize // 2 - 2) * 4.0}", "ampwg=0.07"]
    return d, common, (p, vol, tmpl, timgs, imgs, parts, truth)


def run(args, cwd=None):
    r = subprocess.run([os.path.join(BIN, args[0])] + args[1:], capture_output=True, text=True, cwd=cwd)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def read_tnf(path):
    import ctypes as C
    L = lib()
    ih, fh = np.zeros(4, np.int32), np.zeros(2, np.float32)
    assert L.cryoim_tnf_read(str(path).encode(), ih.ctypes.data, fh.ctypes.data, None, None, None) == 0
    R = int(ih[1])
    t = 2 * R + 1
    a, b, w = (np.zeros((R + 1, t, t), np.float32) for _ in range(3))
    assert L.cryoim_tnf_read(str(path).encode(), ih.ctypes.data, fh.ctypes.data, a.ctypes.data,
                             b.ctypes.data, w.ctypes.data) == 0
    return ih, fh, (a, b, w)


def library_parts(d, case):
    """Particles as the executable reads them (ort values rounded by the file)."""
    import ctypes as C
    import cryoim_gb300 as ci
    p = case[0]
    parts = ci.particles(len(case[5]))
    assert lib().cryoim_ort_read(str(d / "ort.dat").encode(), 1, len(parts), parts.ctypes.data, None, 0) == 0
    return parts


def test_mode4_matches_library(files):
    import cryoim_gb300 as ci
    d, common, case = files
    p, vol, tmpl, timgs, imgs, parts, truth = case
    run(["icosprocess", "mode=4", *common, f"templateort={d / 'tort.dat'}",
         f"templatestck={d / 'tmpl.mrc'}", f"newortfile={d / 'new4.dat'}"])
    rows = read_rows(d / "new4.dat")
    q = library_parts(d, case)
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.globesearch(imgs, q)
    assert np.allclose(rows[:, 0], q["theta"], atol=1e-4) and np.allclose(rows[:, 2], q["omega"], atol=1e-4)
    assert np.allclose(rows[:, 5], q["pr"], atol=2e-4)


def test_mode4_contract_matches_exhaustive(files):
    d, common, case = files
    run(["icosprocess", "mode=4", *common, f"templateort={d / 'tort.dat'}", f"model3d={d / 'model.mrc'}",
         f"newortfile={d / 'new4c.dat'}", "contract=y", "originmax=2", "originstep=0.5", "topk=8"])
    run(["icosprocess", "mode=4", *common, f"templateort={d / 'tort.dat'}", f"model3d={d / 'model.mrc'}",
         f"newortfile={d / 'new4e.dat'}"])
    a, b = read_rows(d / "new4c.dat"), read_rows(d / "new4e.dat")
    assert np.allclose(a[:, :3], b[:, :3], atol=1e-4)


def test_mode5_matches_library(files):
    import cryoim_gb300 as ci
    d, common, case = files
    p, vol, tmpl, timgs, imgs, parts, truth = case
    run(["icosprocess", "mode=5", *common, "Ncycle=3", f"templateort={d / 'tort.dat'}",
         f"templatestck={d / 'tmpl.mrc'}", f"newortfile={d / 'new5.dat'}"])
    rows = read_rows(d / "new5.dat")
    q = library_parts(d, case)
    p5 = ci.Params.from_buffer_copy(p)
    p5.ncycle = 3
    with ci.Context(0, p5) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.refine(imgs, q)
    assert np.allclose(rows[:, 0], q["theta"], atol=2e-4) and np.allclose(rows[:, 3], q["x"], atol=2e-4)


def test_mode1_and_subrec_merge(files):
    import cryoim_gb300 as ci
    d, common, case = files
    p, vol, tmpl, timgs, imgs, parts, truth = case
    n = p.fftsize
    run(["icosprocess", "mode=1", *common, f"result3d={d / 'map.mrc'}"])
    m = read_map(d / "map.mrc", n)
    q = library_parts(d, case)
    with ci.Context(0, p) as ctx:
        ctx.rec_begin()
        ctx.rec_insert(imgs, q)
        want = ctx.rec_finish()
    assert np.linalg.norm(m - want) / np.linalg.norm(want) < 1e-5
    # partial reconstructions of two particle ranges merge to the partial of all.  Every
    # reconstruct run masks all its images at particle(first)'s origin
    # (reconstruct.f90:92), so the ranges are given one common origin here.
    lines = open(d / "ort.dat").read().splitlines()
    with open(d / "ort0.dat", "w") as f:
        for line in lines:
            v = line.split()
            v[5] = v[6] = "0.0"
            f.write(" ".join(v) + "\n")
    c0 = [a if not a.startswith("ortfile=") else f"ortfile={d / 'ort0.dat'}" for a in common]
    run(["icosprocess", "mode=1", *c0, "subrec=y", "first=1", "last=1", f"result3d={d / 'a.tnf'}"])
    run(["icosprocess", "mode=1", *c0, "subrec=y", "first=2", "last=3", f"result3d={d / 'b.tnf'}"])
    run(["icosprocess", "mode=1", *c0, "subrec=y", f"result3d={d / 'all.tnf'}"])
    run(["merge_icosprocess_subrec", str(d / "a.tnf"), str(d / "b.tnf"), str(d / "m2.mrc")])
    run(["merge_icosprocess_subrec", str(d / "all.tnf"), str(d / "m1.mrc")])
    # merge_reconstruct.f90 writes the central (n-8)^3 box under an (n-8) header
    m1, m2 = read_map(d / "m1.mrc", n - 8), read_map(d / "m2.mrc", n - 8)
    assert np.linalg.norm(m1 - m2) / np.linalg.norm(m1) < 1e-4
    assert tuple(np.frombuffer(open(d / "m1.mrc", "rb").read(12), np.int32)) == (n - 8,) * 3
    # the crop, with its index: voxel i (1-based) from section i // (n-8)^2 + 4
    ih, fh, part = read_tnf(d / "all.tnf")
    with ci.Context(0, p) as ctx:
        ctx.rec_begin()
        ctx.rec_add_partial(*part)
        full = ctx.rec_finish_merge()
    m = n - 8
    i = np.arange(1, m ** 3 + 1)
    lz, ky, hx = i // (m * m) + 4, (i - 1) % (m * m) // m + 4, (i - 1) % (m * m) % m + 4
    want = full[lz, ky, hx].reshape(m, m, m)
    assert np.linalg.norm(m1 - want) <= 1e-5 * np.linalg.norm(want)


def test_mode1_fsc_half_maps(files):
    """FSC=y (0main.f90:216-222): oddtnf, evetnf, FSC.txt and the FSC-weighted map in
    result3d; with subrec=y only the two tnf files, named result3d//'oddtnf' etc."""
    import cryoim_gb300 as ci
    d, common, case = files
    p, vol, tmpl, timgs, imgs, parts, truth = case
    n = p.fftsize
    run(["icosprocess", "mode=1", *common, "FSC=y", f"result3d={d / 'fsc.mrc'}"], cwd=d)
    q = library_parts(d, case)
    with ci.Context(0, p) as ctx:
        odd, even = ctx.half_maps(imgs, q)
        fsc, want = ctx.fsc_combine(odd, even)
    for name, ref in (("oddtnf", odd), ("evetnf", even)):
        ih, fh, got = read_tnf(d / name)
        assert ih[0] == n and ih[1] == p.max_r and ih[2] == 0  # header flag: subrec
        for k in range(3):
            assert np.linalg.norm(got[k] - ref[k]) <= 1e-5 * np.linalg.norm(ref[k])
    rows = np.array([[float(v) for v in line.split()[:2]] for line in open(d / "FSC.txt")])
    assert np.array_equal(rows[:, 0], np.arange(p.max_r + 1))
    assert np.abs(rows[:, 1] - fsc).max() < 1e-5
    m = read_map(d / "fsc.mrc", n)
    assert np.linalg.norm(m - want) / np.linalg.norm(want) < 1e-5
    # the header is the particle stack's, as reconstruct_FSC.f90:181 writes it
    nz = np.frombuffer(open(d / "fsc.mrc", "rb").read(12), np.int32)[2]
    assert nz == len(imgs)
    run(["icosprocess", "mode=1", *common, "FSC=y", "subrec=y", f"result3d={d / 'h'}"], cwd=d)
    ih, fh, got = read_tnf(d / "hevetnf")
    assert ih[2] == 1
    assert np.linalg.norm(got[2] - even[2]) <= 1e-5 * np.linalg.norm(even[2])
    # merge_icosprocess_subrec on the prefix: header flag 1 -> merge_reconstruct_FSC.f90
    os.remove(d / "FSC.txt")
    run(["merge_icosprocess_subrec", "h", "mfsc.mrc"], cwd=d)
    rows = np.array([[float(v) for v in line.split()[:2]] for line in open(d / "FSC.txt")])
    assert np.abs(rows[:, 1] - fsc).max() < 1e-5
    with ci.Context(0, p) as ctx:
        fm, full = ctx.fsc_combine(odd, even, merge=True)
    m = n - 8
    raw = open(d / "mfsc.mrc", "rb").read()
    assert tuple(np.frombuffer(raw[:12], np.int32)) == (m, m, m)
    got = np.frombuffer(raw[1024:], np.float32)
    want = full.ravel()[:m ** 3]  # the routine writes the first (n-8)^3 values of its n^3 array
    assert np.linalg.norm(got - want) <= 1e-5 * np.linalg.norm(want)


def test_mode3_centring(files):
    """mode=3 (0main.f90:237-241): calc_center with model3d, calc_center_selfrot180
    without; every particle of first..last written to newortfile."""
    import cryoim_gb300 as ci
    d, common, case = files
    p, vol, tmpl, timgs, imgs, parts, truth = case
    run(["icosprocess", "mode=3", *common, f"model3d={d / 'model.mrc'}", f"newortfile={d / 'c3.dat'}"])
    rows = read_rows(d / "c3.dat")
    q = library_parts(d, case)
    with ci.Context(0, p) as ctx:
        ctx.center(imgs, q, vol)
    assert len(rows) == len(parts)
    assert np.allclose(rows[:, 3], q["x"], atol=2e-4) and np.allclose(rows[:, 4], q["y"], atol=2e-4)
    assert np.allclose(rows[:, 0], q["theta"], atol=2e-4)
    run(["icosprocess", "mode=3", *common, f"newortfile={d / 'c3s.dat'}"])
    rows = read_rows(d / "c3s.dat")
    q = library_parts(d, case)
    with ci.Context(0, p) as ctx:
        ctx.center(imgs, q)
    assert np.allclose(rows[:, 3], q["x"], atol=2e-4) and np.allclose(rows[:, 5], q["pr"], atol=2e-3)


def test_mode0_projections(files):
    import cryoim_gb300 as ci
    d, common, case = files
    p, vol, tmpl, *_ = case
    run(["icosprocess", "mode=0", "apix=4.0", f"model3d={d / 'model.mrc'}", f"templateort={d / 'tort.dat'}",
         f"templatestck={d / 'proj.mrc'}"])
    raw = open(d / "proj.mrc", "rb").read()
    n = p.fftsize
    got = np.frombuffer(raw[1024:], np.float32).reshape(-1, n, n)
    t = ci.templates(len(tmpl))
    for i, line in enumerate(open(d / "tort.dat").read().splitlines()):
        v = line.split()
        t["theta"][i], t["phi"][i], t["omega"][i] = float(v[1]), float(v[2]), float(v[3])
    with ci.Context(0, p) as ctx:
        want = ctx.project_templates(vol, t)
    assert np.array_equal(got, want)


def test_bad_inputs_stop_cleanly(files):
    d, common, case = files
    bad = d / "bad_ort.dat"
    bad.write_text(f"{d / 'stack.mrc'} 1 70 0 0 0 0 0 1 99 1 1 0\n")  # section 99 does not exist
    r = subprocess.run([os.path.join(BIN, "icosprocess"), "mode=4", f"ortfile={bad}", "apix=4",
                        f"templateort={d / 'tort.dat'}", f"templatestck={d / 'tmpl.mrc'}"],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "not match" in r.stdout
    r = subprocess.run([os.path.join(BIN, "icosprocess"), "mode=4", "bogus=1", "ortfile=x"],
                       capture_output=True, text=True)
    assert r.returncode == 0 and "usage" in r.stdout
