"""ctypes wrapper of the CPU oracle (oracle/cryoim_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU-baseline
legs of bench.py as the checker.  The product (libcryoim_gb300.so and the
cryoim_gb300 package) never imports this module.

Every function takes an `fp` argument: "f32" (FP32 in the Fortran's operation order)
or "f64" (the same algorithm in FP64).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libcryoim_oracle.so")
_lib = None

# Records and parameters as laid out in include/cryoim.h (the C oracle compiles against
# that header); the same layouts as the library's, so arrays of either pass to both.
_PF = ["theta0", "phi0", "omega0", "x0", "y0", "pr0", "df1", "df2", "astigang",
       "theta", "phi", "omega", "x", "y", "pr", "dtheta", "dphi", "domega", "dx", "dy", "dpr"]
PARTICLE_DTYPE = np.dtype([("particle_id", "<i4"), ("img_id", "<i4"), ("img_particle_id", "<i4")]
                          + [(f, "<f4") for f in _PF])
TEMPLATE_DTYPE = np.dtype([("particle_id", "<i4"), ("theta", "<f4"), ("phi", "<f4"),
                           ("omega", "<f4"), ("x", "<f4"), ("y", "<f4")])
_LI = ["particle_id", "img_id", "img_particle_id", "local_img_id", "local_hx0", "local_ky0"]
_LF = ["theta", "phi", "omega", "x", "y", "pr", "df1", "df2", "astigang",
       "local_theta0", "local_phi0", "local_omega0", "local_x0", "local_y0", "local_z0", "local_pr0",
       "local_theta", "local_phi", "local_omega", "local_x", "local_y", "local_z", "local_pr",
       "local_dtheta", "local_dphi", "local_domega", "local_dx", "local_dy"]
LOCAL_PARTICLE_DTYPE = np.dtype([(f, "<i4") for f in _LI] + [(f, "<f4") for f in _LF])


class Params(C.Structure):
    """cryoim_params of include/cryoim.h."""
    _fields_ = [(n, C.c_int32) for n in (
        "fftsize", "mode", "first", "last", "ncycle", "apply_ctf", "use_imgmask", "realspaceavg",
        "subrec", "fsc", "imgstck")] + [(n, C.c_float) for n in (
        "apix", "min_res", "max_res", "imgmask", "vol", "cs", "ampwg", "bfactor", "pr_threshold",
        "searchstep", "maxcentshift", "boundx")] + [(n, C.c_int32) for n in (
        "min_r", "max_r", "nsym", "nlin")] + [(n, C.c_float) for n in (
        "imgmask_px", "delta_angle", "delta_trans")]


def default_params(fftsize: int, **kw) -> Params:
    """0initialvalue.f90 defaults for nx = fftsize, keyword overrides by icosprocess key
    name (apix, minRes, maxRes, searchstep, ampwg, imgmask, ...), then the derived values
    of 0calc_initialvalues.f90 (oracle restatement)."""
    p = Params()
    lib().orc_params_default(C.byref(p), C.c_int(int(fftsize)))
    alias = {"minRes": "min_res", "maxRes": "max_res", "applyCTF": "apply_ctf", "Cs": "cs",
             "PR_threshold": "pr_threshold", "boundX": "boundx", "Ncycle": "ncycle", "Bfactor": "bfactor"}
    for k, v in kw.items():
        k = alias.get(k, k)
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    lib().orc_params_derive(C.byref(p))
    return p


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        for s, R in (("f32", C.c_float), ("f64", C.c_double)):
            getattr(_lib, f"orc_pr_single_{s}").restype = R
    return _lib


def _dt(fp):
    return np.float32 if fp == "f32" else np.float64


def _R(fp):
    return C.c_float if fp == "f32" else C.c_double


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _fn(name, fp):
    f = getattr(lib(), f"orc_{name}_{fp}")
    return f


# --- single routines ---------------------------------------------------------
def ctf2d(nx, df1, df2, astig, apix, vol, cs, ampwg, fp="f32"):
    R = _R(fp)
    out = np.zeros(nx * nx, _dt(fp))
    _fn("ctf2d", fp)(C.c_int(nx), R(df1), R(df2), R(astig), R(apix), R(vol), R(cs), R(ampwg), _p(out))
    return out.reshape(nx, nx)


def mask(img, radius, ox, oy, fp="f32"):
    a = np.ascontiguousarray(img, _dt(fp)).copy()
    R = _R(fp)
    _fn("mask", fp)(_p(a), C.c_int(a.shape[-1]), R(radius), R(ox), R(oy))
    return a


def fft2d(a, b, nbit=1, fp="f32"):
    a = np.ascontiguousarray(a, _dt(fp)).copy()
    b = np.ascontiguousarray(b, _dt(fp)).copy()
    _fn("fft2d", fp)(_p(a), _p(b), C.c_int(a.shape[-1]), C.c_int(a.shape[-2]), C.c_int(nbit))
    return a, b


def fft3d(re, im, sign, fp="f64"):
    re = np.ascontiguousarray(re, _dt(fp)).copy()
    im = np.ascontiguousarray(im, _dt(fp)).copy()
    _fn("fft3d", fp)(_p(re), _p(im), C.c_int(re.shape[-1]), C.c_int(sign))
    return re, im


def expfit(a, b, min_r, max_r, fp="f32"):
    a = np.ascontiguousarray(a, _dt(fp))
    b = np.ascontiguousarray(b, _dt(fp))
    out = np.zeros(max_r - min_r + 1, _dt(fp))
    _fn("expfit", fp)(_p(a), _p(b), C.c_int(a.shape[-1]), C.c_int(min_r), C.c_int(max_r), _p(out))
    return out


def centshift(a, b, x0, y0, fp="f32"):
    a = np.ascontiguousarray(a, _dt(fp)).copy()
    b = np.ascontiguousarray(b, _dt(fp)).copy()
    R = _R(fp)
    _fn("centshift", fp)(_p(a), _p(b), C.c_int(a.shape[-1]), R(x0), R(y0))
    return a, b


def norm(img, fp="f32"):
    a = np.ascontiguousarray(img, _dt(fp)).copy()
    _fn("norm", fp)(_p(a), C.c_int(a.shape[-1]))
    return a


def euler(theta, phi, omega, fp="f32"):
    m = np.zeros(9, _dt(fp))
    R = _R(fp)
    _fn("euler", fp)(R(theta), R(phi), R(omega), _p(m))
    return m.reshape(3, 3)


def icos_ops(fp="f64"):
    m = np.zeros(540, _dt(fp))
    _fn("icos_ops", fp)(_p(m))
    return m.reshape(60, 3, 3)


def icos_gen(fp="f64"):
    m = np.zeros(540, _dt(fp))
    _fn("icos_gen", fp)(_p(m))
    return m.reshape(60, 3, 3)


def crosslin(o1, o2, fp="f32"):
    a1 = np.zeros(60, _dt(fp))
    a2 = np.zeros(60, _dt(fp))
    R = _R(fp)
    _fn("crosslin", fp)(*(R(v) for v in (*o1, *o2)), _p(a1), _p(a2))
    return a1, a2


def asu_fold(theta, phi, omega, fp="f32"):
    R = _R(fp)
    t, p, o = R(theta), R(phi), R(omega)
    _fn("asu_fold", fp)(C.byref(t), C.byref(p), C.byref(o))
    return t.value, p.value, o.value


def fill_lin(a, b, min_r, max_r, alpha, fp="f32"):
    a = np.ascontiguousarray(a, _dt(fp))
    b = np.ascontiguousarray(b, _dt(fp))
    al = np.ascontiguousarray(alpha, _dt(fp))
    nr = max_r - min_r + 1
    out = np.zeros((len(al), nr, 2), _dt(fp))
    _fn("fill_lin", fp)(C.c_int(len(al)), _p(a), _p(b), C.c_int(a.shape[-1]), C.c_int(min_r),
                        C.c_int(max_r), _p(al), _p(out))
    return out


def pr_omega(pa, pb, fcut0, tmpl, tort, tfcut, ctf, min_r, max_r, step, theta, phi, omega=0.0,
             fp="f64"):
    dt = _dt(fp)
    R = _R(fp)
    nx = pa.shape[-1]
    nom = int(np.float32(360.0) / np.float32(step))
    out = np.zeros(nom, dt)
    args = [np.ascontiguousarray(x, dt) if x is not None else None
            for x in (pa, pb, fcut0, tmpl, tort, tfcut, ctf)]
    _fn("pr_omega", fp)(*[_p(x) for x in args], C.c_int(len(tort)), C.c_int(nx), C.c_int(min_r),
                        C.c_int(max_r), R(step), C.c_int(nom), R(theta), R(phi), R(omega), _p(out))
    return out


def pr_single(pa, pb, fcut0, tmpl, tort, tfcut, ctf, min_r, max_r, theta, phi, omega, x, y,
              fp="f64"):
    dt = _dt(fp)
    R = _R(fp)
    args = [np.ascontiguousarray(v, dt) if v is not None else None
            for v in (pa, pb, fcut0, tmpl, tort, tfcut, ctf)]
    return _fn("pr_single", fp)(*[_p(v) for v in args], C.c_int(len(tort)), C.c_int(pa.shape[-1]),
                                C.c_int(min_r), C.c_int(max_r), R(theta), R(phi), R(omega), R(x), R(y))


def prep_particle(img, use_mask, mask_px, x, y, shift, min_r, max_r, fp="f64"):
    dt = _dt(fp)
    R = _R(fp)
    im = np.ascontiguousarray(img, np.float32)
    nx = im.shape[-1]
    a = np.zeros((nx, nx), dt)
    b = np.zeros((nx, nx), dt)
    f = np.zeros(max_r - min_r + 1, dt)
    _fn("prep_particle", fp)(_p(im), C.c_int(nx), C.c_int(int(use_mask)), R(mask_px), R(x), R(y),
                             C.c_int(int(shift)), C.c_int(min_r), C.c_int(max_r), _p(a), _p(b), _p(f))
    return a, b, f


def load_templates(imgs, tmpl, params, fp="f64"):
    dt = _dt(fp)
    im = np.ascontiguousarray(imgs, np.float32)
    t = np.ascontiguousarray(tmpl)
    T, nx = len(t), params.fftsize
    nr = params.max_r - params.min_r + 1
    tm = np.zeros((T, 2, nx, nx), dt)
    tf = np.zeros((T, nr), dt)
    _fn("load_templates", fp)(_p(im), _p(t), C.c_int(T), C.byref(params), _p(tm), _p(tf))
    return tm, tf


def globesearch(params, tm, tf, tmpl, imgs, parts, want_pr_array=False, nthreads=0, fp="f64"):
    dt = _dt(fp)
    nth, nph, nom = grid_sizes(params.searchstep)
    pra = None
    if want_pr_array:
        pra = np.zeros((len(parts), nth + 1, 2 * nph + 1, nom), np.float32)
    im = np.ascontiguousarray(imgs, np.float32)
    r = _fn("globesearch", fp)(C.byref(params), _p(np.ascontiguousarray(tm, dt)),
                               _p(np.ascontiguousarray(tf, dt)), _p(np.ascontiguousarray(tmpl)),
                               C.c_int(len(tmpl)), _p(im), _p(parts), C.c_int(len(parts)), _p(pra),
                               C.c_int(nthreads))
    assert r == 0
    return pra


def refine(params, tm, tf, tmpl, imgs, parts, nthreads=0, fp="f64"):
    dt = _dt(fp)
    im = np.ascontiguousarray(imgs, np.float32)
    r = _fn("refine", fp)(C.byref(params), _p(np.ascontiguousarray(tm, dt)),
                          _p(np.ascontiguousarray(tf, dt)), _p(np.ascontiguousarray(tmpl)),
                          C.c_int(len(tmpl)), _p(im), _p(parts), C.c_int(len(parts)), C.c_int(nthreads))
    assert r == 0


def search_views(params, tm, tf, tmpl, img, part, views, nthreads=0, fp="f32"):
    """PR(omega) of one particle at the listed (theta, phi) views (CPU baseline sample)."""
    dt = _dt(fp)
    nth, nph, nom = grid_sizes(params.searchstep)
    v = np.ascontiguousarray(views, np.float32).reshape(-1, 2)
    out = np.zeros((len(v), nom), np.float32)
    q = np.ascontiguousarray(part).reshape(1)
    r = _fn("search_views", fp)(C.byref(params), _p(np.ascontiguousarray(tm, dt)),
                                _p(np.ascontiguousarray(tf, dt)), _p(np.ascontiguousarray(tmpl)),
                                C.c_int(len(tmpl)), _p(np.ascontiguousarray(img, np.float32)), _p(q),
                                _p(v), C.c_int(len(v)), C.c_int(nthreads), _p(out))
    assert r == 0
    return out


def project_template2d(map3d, theta, phi, omega, fp="f32"):
    m = np.ascontiguousarray(map3d, np.float32)
    nx = m.shape[-1]
    out = np.zeros((nx, nx), _dt(fp))
    R = _R(fp)
    _fn("project_template2d", fp)(_p(m), C.c_int(nx), R(theta), R(phi), R(omega), _p(out))
    return out


def central_section(fre, fim, theta, phi, omega, fp="f32"):
    dt = _dt(fp)
    fre = np.ascontiguousarray(fre, dt)
    fim = np.ascontiguousarray(fim, dt)
    nx = fre.shape[-1]
    ore = np.zeros((nx, nx), dt)
    oim = np.zeros((nx, nx), dt)
    R = _R(fp)
    _fn("central_section", fp)(_p(fre), _p(fim), C.c_int(nx), R(theta), R(phi), R(omega), _p(ore), _p(oim))
    return ore, oim


def central_section_gauss(fre, fim, theta, phi, omega, sigma, fp="f64"):
    """The central section with the 27-voxel Gaussian kernel of width sigma voxels."""
    dt = _dt(fp)
    fre = np.ascontiguousarray(fre, dt)
    fim = np.ascontiguousarray(fim, dt)
    nx = fre.shape[-1]
    ore = np.zeros((nx, nx), dt)
    oim = np.zeros((nx, nx), dt)
    R = _R(fp)
    _fn("central_section_gauss", fp)(_p(fre), _p(fim), C.c_int(nx), R(theta), R(phi), R(omega), R(sigma),
                                     _p(ore), _p(oim))
    return ore, oim


def reconstruct(params, imgs, parts, want_acc=False, fp="f64"):
    dt = _dt(fp)
    nx = params.fftsize
    im = np.ascontiguousarray(imgs, np.float32)
    out = np.zeros((nx, nx, nx), np.float32)
    acc = np.zeros((3, nx, nx, nx), dt) if want_acc else None
    r = _fn("reconstruct", fp)(C.byref(params), _p(im), _p(np.ascontiguousarray(parts)),
                               C.c_int(len(parts)), _p(out), _p(acc))
    assert r == 0
    return (out, acc) if want_acc else out


def reconstruct_half(params, imgs, parts, parity, fp="f64"):
    """reconstruct_half.f90: tnf partial (fa, fb, wg), each (R+1, 2R+1, 2R+1), of the
    particles parity, parity+2, ... of `parts`."""
    dt = _dt(fp)
    R = params.max_r
    t = 2 * R + 1
    im = np.ascontiguousarray(imgs, np.float32)
    fa, fb, wg = (np.zeros((R + 1, t, t), dt) for _ in range(3))
    r = _fn("reconstruct_half", fp)(C.byref(params), _p(im), _p(np.ascontiguousarray(parts)),
                                    C.c_int(len(parts)), C.c_int(parity), _p(fa), _p(fb), _p(wg))
    assert r == 0
    return fa, fb, wg


def fsc_combine(nx, max_r, odd, even, fp="f64"):
    """reconstruct_FSC.f90: (FSC per shell 0..R, FSC-weighted map nx^3) from the odd and
    even tnf partials (each a (fa, fb, wg) triple, float32)."""
    a = [np.ascontiguousarray(x, np.float32) for x in (*odd, *even)]
    fsc = np.zeros(max_r + 1, _dt(fp))
    out = np.zeros((nx, nx, nx), np.float32)
    r = _fn("fsc_combine", fp)(C.c_int(nx), C.c_int(max_r), *[_p(x) for x in a], _p(fsc), _p(out))
    assert r == 0
    return fsc, out


def merge_fsc(nx, max_r, odd, even, imgmask, fp="f64"):
    """merge_reconstruct_FSC.f90: (FSC per shell, nx^3 map before the output quirks)."""
    a = [np.ascontiguousarray(x, np.float32) for x in (*odd, *even)]
    fsc = np.zeros(max_r + 1, _dt(fp))
    out = np.zeros((nx, nx, nx), np.float32)
    r = _fn("merge_fsc", fp)(C.c_int(nx), C.c_int(max_r), *[_p(x) for x in a], _R(fp)(imgmask),
                             _p(fsc), _p(out))
    assert r == 0
    return fsc, out


def merge_finish(nx, max_r, part, fp="f64"):
    """merge_reconstruct.f90:20-140 on a summed tnf partial (fa, fb, wg): the nx^3 map."""
    a = [np.ascontiguousarray(x, np.float32) for x in part]
    out = np.zeros((nx, nx, nx), np.float32)
    assert _fn("merge_finish", fp)(C.c_int(nx), C.c_int(max_r), *[_p(x) for x in a], _p(out)) == 0
    return out


def icosavg(map3d, r0, fp="f64"):
    """img3d_icosavg.f90: real-space icosahedral average of a cubic map."""
    m = np.ascontiguousarray(map3d, np.float32)
    out = np.zeros_like(m)
    _fn("icosavg", fp)(_p(m), C.c_int(m.shape[0]), _R(fp)(r0), _p(out))
    return out


def center(params, imgs, parts, map3d=None, fp="f64"):
    """calc_center.f90 (map3d given) / calc_center_selfrot180.f90: (P, 3) of (centx,
    centy, cc) before the record update."""
    dt = _dt(fp)
    im = np.ascontiguousarray(imgs, np.float32)
    m = None if map3d is None else np.ascontiguousarray(map3d, np.float32)
    out = np.zeros((len(parts), 3), dt)
    r = _fn("center", fp)(C.byref(params), _p(m), _p(im), _p(np.ascontiguousarray(parts)),
                          C.c_int(len(parts)), _p(out))
    assert r == 0
    return out


def lowpass(img, lp, fp="f64"):
    a = np.array(img, _dt(fp), copy=True, order="C")
    _fn("lowpass", fp)(_p(a), C.c_int(a.shape[0]), C.c_int(lp))
    return a


def gauss_regression(z, fp="f64"):
    """z[j+1][i+1] = z(i, j) of guass_regression.f90; returns (dx, dy, cc)."""
    zz = np.ascontiguousarray(z, _dt(fp)).reshape(9)
    out = np.zeros(3, _dt(fp))
    _fn("gauss_regression", fp)(_p(zz), _p(out))
    return out


def local_box_coordinates(parts, sym, loc, apix, fftsize, pr_threshold=90.0, boundx=100.0, fp="f64"):
    """loc_box_coordinate.f90: sub-particle records (LOCAL_PARTICLE_DTYPE)."""
    p = np.ascontiguousarray(parts)
    s = np.ascontiguousarray(sym, np.float32).reshape(-1, 3, 3)
    out = np.zeros(len(p) * len(s), LOCAL_PARTICLE_DTYPE)
    R = _R(fp)
    k = _fn("local_box_coordinates", fp)(_p(p), C.c_int(len(p)), _p(s), C.c_int(len(s)), R(loc[0]), R(loc[1]),
                                         R(loc[2]), R(apix), C.c_int(fftsize), R(pr_threshold), R(boundx), _p(out))
    return out[:k].copy()


def local_refine(lp, map3d, imgs, lparts, fp="f64"):
    """refine_PR.f90 on sub-particle records (a refined copy is returned)."""
    q = np.array(lparts, copy=True)
    m = np.ascontiguousarray(map3d, np.float32)
    im = np.ascontiguousarray(imgs, np.float32)
    r = _fn("local_refine", fp)(C.byref(lp), _p(m), _p(im), _p(q), C.c_int(len(q)))
    assert r == 0
    return q


def equalort(theta, phi, omega, fp="f32"):
    out = np.zeros((60, 3), _dt(fp))
    R = _R(fp)
    _fn("equalort", fp)(R(theta), R(phi), R(omega), _p(out))
    return out


def transform_ort(to, theta, phi, omega, fp="f32"):
    dt = _dt(fp)
    t = np.array(theta, dt).ravel().copy()
    p = np.array(phi, dt).ravel().copy()
    o = np.array(omega, dt).ravel().copy()
    _fn("transform_ort", fp)(C.c_int(to), _p(t), _p(p), _p(o), C.c_int(len(t)))
    return t, p, o


def grid_sizes(step):
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    lib().orc_grid_sizes(C.c_float(step), C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value


def num_threads():
    return lib().orc_num_threads()


def local_box_extract(imgs, parts, sym, loc, apix, sub, pr_threshold=90.0, boundx=100.0, fp="f64"):
    """loc_box.f90 (sub-image stack mode): (sub images (K, sub, sub) float32, records
    LOCAL_PARTICLE_DTYPE) for the selected particles x nsym rotations."""
    im = np.ascontiguousarray(imgs, np.float32)
    p = np.ascontiguousarray(parts)
    s = np.ascontiguousarray(sym, np.float32).reshape(-1, 3, 3)
    nx0 = im.shape[-1]
    so = np.zeros((len(p) * len(s), sub, sub), np.float32)
    out = np.zeros(len(p) * len(s), LOCAL_PARTICLE_DTYPE)
    R = _R(fp)
    k = _fn("local_box_extract", fp)(_p(im), _p(p), C.c_int(len(p)), C.c_int(nx0), _p(s), C.c_int(len(s)),
                                     R(loc[0]), R(loc[1]), R(loc[2]), R(apix), C.c_int(sub), R(pr_threshold),
                                     R(boundx), _p(so), _p(out))
    return so[:k].copy(), out[:k].copy()
