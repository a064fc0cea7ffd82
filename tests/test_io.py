"""File formats (host code, no GPU): MRC header/stack, orientation rows (list-directed in,
format 900 out), template rows, tnf partials, and the proc_icos executable."""
import ctypes as C
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT

BIN = os.path.join(ROOT, "cryoim_gb300", "bin")


class Hdr(C.Structure):
    _fields_ = [("raw", C.c_char * 1024)]


def lib():
    import cryoim_gb300._abi as abi
    L = abi.load()
    L.cryoim_mrc_write.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int64]
    L.cryoim_map_header.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float]
    L.cryoim_mrc_read_header.argtypes = [C.c_char_p, C.c_void_p]
    L.cryoim_mrc_read_sections.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_void_p]
    L.cryoim_ort_count.argtypes = [C.c_char_p, C.POINTER(C.c_int32)]
    L.cryoim_ort_read.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]
    L.cryoim_ort_write.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.cryoim_template_ort_read.argtypes = [C.c_char_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
    L.cryoim_tnf_write.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_int32, C.c_int32,
                                   C.c_void_p, C.c_void_p, C.c_void_p]
    L.cryoim_tnf_read.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return L


def write_stack(L, path, data, apix=1.0):
    h = Hdr()
    nz, ny, nx = data.shape
    assert L.cryoim_map_header(C.byref(h), nx, ny, nz, apix) == 0
    d = np.ascontiguousarray(data, np.float32)
    assert L.cryoim_mrc_write(str(path).encode(), C.byref(h), d.ctypes.data, d.size) == 0


def test_mrc_round_trip_and_header_layout(built, tmp_path):
    L = lib()
    data = np.random.default_rng(0).normal(size=(3, 16, 12)).astype(np.float32)
    p = tmp_path / "s.mrc"
    write_stack(L, p, data, 1.5)
    raw = p.read_bytes()
    assert len(raw) == 1024 + data.nbytes
    nx, ny, nz, mode = struct.unpack("<4i", raw[:16])
    assert (nx, ny, nz, mode) == (12, 16, 3, 2)
    assert struct.unpack("<3i", raw[16:28]) == (-6, -8, -1)          # n*start = -n/2 (mrchead.f90:17-19)
    assert struct.unpack("<f", raw[28 + 12:28 + 16])[0] == np.float32(11 * 1.5)  # a = mx * apix
    # map(4), machinestamp(4), label(10,80) are arrays of single characters: the strings
    # assigned in mrchead.f90:60-66 leave their first letter in every element
    assert raw[208:216] == b"mmmmllll" and raw[224:1024] == b"H" * 800
    assert struct.unpack("<3f", raw[196:208]) == (-12.0, -16.0, -3.0)  # x/y/zorigin = -n
    out = np.zeros((2, 16, 12), np.float32)
    assert L.cryoim_mrc_read_sections(str(p).encode(), 2, 2, out.ctypes.data) == 0
    assert np.array_equal(out, data[1:])
    assert L.cryoim_mrc_read_sections(str(p).encode(), 3, 2, out.ctypes.data) == -8  # beyond nz
    assert L.cryoim_mrc_read_sections(b"/nonexistent.mrc", 1, 1, out.ctypes.data) == -7


def fortran_f(v, w, d):
    s = f"{v:{w}.{d}f}"
    return "*" * w if len(s) > w else s


def test_ort_rows_read_and_write_format_900(built, tmp_path):
    import cryoim_gb300 as ci
    L = lib()
    src = tmp_path / "in.dat"
    src.write_text("stack_a.mrc 1 70.5 -12.25 300.0 1.5 -2.0 45.0 7 1 1.5 1.6 30.0\n"
                   "\n"
                   "stack_b.mrc,2,\t80,10,20,0,0,99,8,3,2.5,2.5,0\n")
    n = C.c_int32()
    assert L.cryoim_ort_count(str(src).encode(), C.byref(n)) == 0 and n.value == 2
    parts = ci.particles(2)
    names = np.zeros((2, 64), np.uint8)
    assert L.cryoim_ort_read(str(src).encode(), 1, 2, parts.ctypes.data, names.ctypes.data, 64) == 0
    assert bytes(names[1]).rstrip(b"\0") == b"stack_b.mrc"
    assert parts["img_particle_id"][1] == 3 and parts["phi"][0] == np.float32(-12.25)
    parts["dtheta"][0] = 123456.0  # overflows F10.4 -> asterisks
    out = tmp_path / "out.dat"
    assert L.cryoim_ort_write(str(out).encode(), parts.ctypes.data, names.ctypes.data, 64, 2, 54, 0) == 0
    rows = out.read_text().splitlines()
    q = parts[0]
    want = ("stack_a.mrc".ljust(54) + f"{1:8d}" +
            "".join(fortran_f(float(q[k]), 10, 4) for k in ("theta", "phi", "omega", "x", "y", "pr")) +
            f"{7:12d}{1:6d}" +
            "".join(fortran_f(float(q[k]), 10, 4) for k in ("df1", "df2", "astigang", "dtheta", "dphi", "domega",
                                                            "dx", "dy", "dpr")))
    assert rows[0] == want
    assert "**********" in rows[0]
    assert len(rows[1]) == 54 + 8 + 60 + 12 + 6 + 90
    # short file and bad values are errors, not garbage
    bad = tmp_path / "bad.dat"
    bad.write_text("s 1 2 3\n")
    assert L.cryoim_ort_read(str(bad).encode(), 1, 1, parts.ctypes.data, None, 0) == -7
    bad.write_text("s x 70 0 0 0 0 0 1 1 1 1 0\n")
    assert L.cryoim_ort_read(str(bad).encode(), 1, 1, parts.ctypes.data, None, 0) == -6
    assert L.cryoim_ort_read(str(src).encode(), 1, 3, parts.ctypes.data, None, 0) == -7


def test_template_rows_and_tnf_round_trip(built, tmp_path):
    import cryoim_gb300 as ci
    L = lib()
    t = tmp_path / "t.dat"
    t.write_text("1 70 10 20 0 0\n2 80 -5 300 1 -1\n")
    tm = ci.templates(4)
    n = C.c_int32()
    assert L.cryoim_template_ort_read(str(t).encode(), tm.ctypes.data, 4, C.byref(n)) == 0 and n.value == 2
    assert tm["omega"][1] == 300 and tm["x"][1] == 1
    R = 5
    sz = (2 * R + 1) ** 2 * (R + 1)
    fa, fb, wg = (np.random.default_rng(k).normal(size=sz).astype(np.float32) for k in range(3))
    f = tmp_path / "p.tnf"
    assert L.cryoim_tnf_write(str(f).encode(), 64, R, 1.5, 30.0, 1, 0, fa.ctypes.data, fb.ctypes.data,
                              wg.ctypes.data) == 0
    raw = f.read_bytes()
    assert struct.unpack("<2i2f2i", raw[:24]) == (64, R, 1.5, 30.0, 1, 0)
    assert len(raw) == 24 + 3 * sz * 4
    ih = np.zeros(4, np.int32)
    fh = np.zeros(2, np.float32)
    a, b, c = (np.zeros(sz, np.float32) for _ in range(3))
    assert L.cryoim_tnf_read(str(f).encode(), ih.ctypes.data, fh.ctypes.data, a.ctypes.data, b.ctypes.data,
                             c.ctypes.data) == 0
    assert list(ih) == [64, R, 1, 0] and np.array_equal(a, fa) and np.array_equal(c, wg)


def test_proc_icos_transforms_and_random_equivalents(built, orc, tmp_path):
    src = tmp_path / "in.dat"
    src.write_text("a.mrc 1 70 10 33 0 0 20 1 1 1.5 1.5 0\nb.mrc 2 85 -20 120 1 1 30 2 2 2 2 0\n")
    out = tmp_path / "out.dat"
    r = subprocess.run([os.path.join(BIN, "proc_icos"), f"ort0={src}", f"newort={out}", "transform_ort_2fTo5f=y"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rows = out.read_text().splitlines()
    assert len(rows) == 2 and len(rows[0]) == 64 + 8 + 60 + 12 + 6 + 15 + 15 + 10
    t, p, o = orc.transform_ort(5, [70.0, 85.0], [10.0, -20.0], [33.0, 120.0], "f32")
    got = [float(rows[0][72:82]), float(rows[0][82:92]), float(rows[0][92:102])]
    assert np.allclose(got, [t[0], p[0], o[0]], atol=2e-4)
    r = subprocess.run([os.path.join(BIN, "proc_icos"), f"ort0={src}", f"newort={out}", "calc_randort_2f=y",
                        "seed=3"], capture_output=True, text=True)
    assert r.returncode == 0
    from synth import euler_mat
    ops = orc.icos_ops("f64")
    for row, (t0, p0, o0) in zip(out.read_text().splitlines(), [(70, 10, 33), (85, -20, 120)]):
        e = [float(row[72 + 10 * k:82 + 10 * k]) for k in range(3)]
        R0, R1 = euler_mat(t0, p0, o0), euler_mat(*e)
        assert min(np.abs(S @ R0 - R1).max() for S in ops) < 2e-3
    r = subprocess.run([os.path.join(BIN, "proc_icos"), "nonsense=1"], capture_output=True, text=True)
    assert r.returncode == 0 and "usage" in r.stdout
