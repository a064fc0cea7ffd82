"""ctypes view of libcryoim_gb300.so (include/cryoim.h).

Record layouts are numpy structured dtypes so arrays of particles / templates pass
to C without copies.  Loading fails loudly when the library has not been built:
there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libcryoim_gb300.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_SIZE, ERR_INPUT, ERR_IO, ERR_MISMATCH = (
    -1, -2, -3, -4, -5, -6, -7, -8)
ERR_NAMES = {0: "OK", -1: "ERR_ARG", -2: "ERR_CUDA", -3: "ERR_NOMEM", -4: "ERR_STATE",
             -5: "ERR_SIZE", -6: "ERR_INPUT", -7: "ERR_IO", -8: "ERR_MISMATCH"}

_F = ["theta0", "phi0", "omega0", "x0", "y0", "pr0", "df1", "df2", "astigang",
      "theta", "phi", "omega", "x", "y", "pr", "dtheta", "dphi", "domega", "dx", "dy", "dpr"]
# cryoim_particle: the `particles` type of icosprocess/SRC/0common_icosproc.f90:28-34
PARTICLE_DTYPE = np.dtype([("particle_id", "<i4"), ("img_id", "<i4"), ("img_particle_id", "<i4")]
                          + [(f, "<f4") for f in _F])
# cryoim_template: the `templates` type of 0common_icosproc.f90:37-40
TEMPLATE_DTYPE = np.dtype([("particle_id", "<i4"), ("theta", "<f4"), ("phi", "<f4"),
                           ("omega", "<f4"), ("x", "<f4"), ("y", "<f4")])
assert PARTICLE_DTYPE.itemsize == 24 * 4 and TEMPLATE_DTYPE.itemsize == 24
# cryoim_local_particle: the sub-particle rows of local_box / local_refine
_LI = ["particle_id", "img_id", "img_particle_id", "local_img_id", "local_hx0", "local_ky0"]
_LF = ["theta", "phi", "omega", "x", "y", "pr", "df1", "df2", "astigang",
       "local_theta0", "local_phi0", "local_omega0", "local_x0", "local_y0", "local_z0", "local_pr0",
       "local_theta", "local_phi", "local_omega", "local_x", "local_y", "local_z", "local_pr",
       "local_dtheta", "local_dphi", "local_domega", "local_dx", "local_dy"]
LOCAL_PARTICLE_DTYPE = np.dtype([(f, "<i4") for f in _LI] + [(f, "<f4") for f in _LF])
assert LOCAL_PARTICLE_DTYPE.itemsize == 34 * 4


class LocalParams(C.Structure):
    """cryoim_local_params (include/cryoim.h)."""
    _fields_ = [(n, C.c_int32) for n in ("fftsize", "fftsize0", "nsym", "ncycle", "apply_ctf", "normalize")] + \
               [(n, C.c_float) for n in ("apix", "max_res", "imgmask", "vol", "cs", "ampwg", "refine_angle",
                                         "refine_shift", "convf", "max_r", "imgmask_px")]


class Params(C.Structure):
    """cryoim_params (include/cryoim.h)."""
    _fields_ = [(n, C.c_int32) for n in (
        "fftsize", "mode", "first", "last", "ncycle", "apply_ctf", "use_imgmask", "realspaceavg",
        "subrec", "fsc", "imgstck")] + [(n, C.c_float) for n in (
        "apix", "min_res", "max_res", "imgmask", "vol", "cs", "ampwg", "bfactor", "pr_threshold",
        "searchstep", "maxcentshift", "boundx")] + [(n, C.c_int32) for n in (
        "min_r", "max_r", "nsym", "nlin")] + [(n, C.c_float) for n in (
        "imgmask_px", "delta_angle", "delta_trans")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ContractOpts(C.Structure):
    """cryoim_contract_opts (include/cryoim.h)."""
    _fields_ = [("origin_max", C.c_float), ("origin_step", C.c_float), ("topk", C.c_int32),
                ("pick", C.c_int32), ("precision", C.c_int32), ("nbr", C.c_int32), ("coarse", C.c_int32),
                ("learned", C.c_int32), ("nbr_best", C.c_int32), ("local_range", C.c_float),
                ("local_step", C.c_float), ("fallback", C.c_float), ("centred_origins", C.c_int32),
                ("proposal_nbr", C.c_int32)]


class LearnOpts(C.Structure):
    """cryoim_learn_opts (include/cryoim.h)."""
    _fields_ = [("samples", C.c_int32), ("batch", C.c_int32), ("seed", C.c_int32)] + \
               [(n, C.c_float) for n in ("lr", "snr", "df_min", "df_max", "astig_max", "origin_max")]


_vp, _fp, _ip, _i32, _f32 = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int32), C.c_int32, C.c_float
_pp = C.POINTER(Params)
_op = C.POINTER(ContractOpts)

# name -> argtypes (every function returns int status unless listed in _RESTYPES)
SIGNATURES = {
    "cryoim_version": [],
    "cryoim_last_error": [],
    "cryoim_params_default": [_pp, _i32],
    "cryoim_params_derive": [_pp],
    "cryoim_ctx_create": [_i32, C.POINTER(_vp)],
    "cryoim_ctx_destroy": [_vp],
    "cryoim_ctx_set_stream": [_vp, _vp],
    "cryoim_ctx_set_batch": [_vp, _i32],
    "cryoim_ctx_set_lanes": [_vp, _i32],
    "cryoim_set_params": [_vp, _pp],
    "cryoim_ctx_set_profiling": [_vp, _i32],
    "cryoim_ctx_kernel_time": [_vp, C.POINTER(C.c_double), C.POINTER(C.c_int64)],
    "cryoim_search_terms": [_vp, C.POINTER(C.c_double)],
    "cryoim_project_templates": [_vp, _vp, _vp, _i32, _vp],
    "cryoim_load_templates": [_vp, _vp, _vp, _i32],
    "cryoim_globesearch": [_vp, _vp, _vp, _i32, _vp],
    "cryoim_globesearch_device": [_vp, _vp, _vp, _i32, _vp],
    "cryoim_search_grid": [_vp, _ip, _ip, _ip, _ip],
    "cryoim_prscore_omega": [_vp, _vp, _vp, _vp, _vp, _f32, _f32, _vp],
    "cryoim_refine": [_vp, _vp, _vp, _i32],
    "cryoim_refine_device": [_vp, _vp, _vp, _i32],
    "cryoim_prscore": [_vp, _vp, _vp, _vp, _vp, _f32, _f32, _f32, _f32, _f32, _fp],
    "cryoim_prscore_noalloc": [_i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _i32,
                               _vp, _vp],
    "cryoim_gemm_bf16_argmax": [_vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp],
    "cryoim_gemm_e4m3_argmax": [_vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp],
    "cryoim_set_reference_map": [_vp, _vp],
    "cryoim_contract_search": [_vp, _vp, _vp, _i32, _op, _vp],
    "cryoim_contract_search_device": [_vp, _vp, _vp, _i32, _op, _vp],
    "cryoim_contract_stats": [_vp, _vp],
    "cryoim_rescore_stats": [_vp, _vp],
    "cryoim_rec_add_partial": [_vp, _vp, _vp, _vp],
    "cryoim_mrc_read_header": [C.c_char_p, _vp],
    "cryoim_mrc_read_sections": [C.c_char_p, _i32, _i32, _vp],
    "cryoim_map_header": [_vp, _i32, _i32, _i32, _f32],
    "cryoim_mrc_write": [C.c_char_p, _vp, _vp, C.c_int64],
    "cryoim_ort_count": [C.c_char_p, _ip],
    "cryoim_ort_read": [C.c_char_p, _i32, _i32, _vp, _vp, _i32],
    "cryoim_ort_write": [C.c_char_p, _vp, _vp, _i32, _i32, _i32, _i32],
    "cryoim_template_ort_read": [C.c_char_p, _vp, _i32, _ip],
    "cryoim_tnf_write": [C.c_char_p, _i32, _i32, _f32, _f32, _i32, _i32, _vp, _vp, _vp],
    "cryoim_tnf_read": [C.c_char_p, _vp, _vp, _vp, _vp, _vp],
    "cryoim_rec_begin": [_vp],
    "cryoim_rec_insert": [_vp, _vp, _vp, _i32, _ip],
    "cryoim_rec_insert_device": [_vp, _vp, _vp, _i32, _ip],
    "cryoim_rec_finish": [_vp, _vp],
    "cryoim_rec_get_partial": [_vp, _vp, _vp, _vp],
    "cryoim_rec_begin_half": [_vp, _f32, _f32],
    "cryoim_fsc_combine": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "cryoim_merge_fsc_combine": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "cryoim_rec_finish_merge": [_vp, _vp],
    "cryoim_icosavg": [_vp, _vp, _i32, _f32],
    "cryoim_center": [_vp, _vp, _vp, _vp, _i32],
    "cryoim_local_sym_matrices": [C.c_char_p, _vp, _ip],
    "cryoim_local_box_coordinates": [_vp, _i32, _vp, _i32, _f32, _f32, _f32, _f32, _i32, _f32, _f32, _vp, _ip],
    "cryoim_local_params_default": [_vp, _i32, _i32],
    "cryoim_local_params_derive": [_vp],
    "cryoim_local_refine": [_vp, _vp, _vp, _vp, _vp, _i32],
    "cryoim_contract_fallbacks": [_vp, _ip],
    "cryoim_gemm_bf16_argmax_withhold": [_vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _i32, _i32, _vp],
    "cryoim_set_interpolation": [_vp, _i32, _f32],
    "cryoim_local_box_extract": [_vp, _vp, _vp, _i32, _i32, _vp, _i32, _f32, _f32, _f32, _f32, _i32, _f32, _f32,
                                 _vp, _vp, _ip],
    "cryoim_local_box_extract_device": [_vp, _vp, _vp, _i32, _i32, _vp, _i32, _f32, _f32, _f32, _f32, _i32, _f32,
                                        _f32, _vp, _vp, _ip],
    "cryoim_local_ort_read": [C.c_char_p, _i32, _i32, _vp, _vp, _i32],
    "cryoim_local_ort_write": [C.c_char_p, _vp, _vp, _i32, _i32, _i32, _i32],
    "cryoim_learn_opts_default": [_vp],
    "cryoim_learn_train": [_vp, _vp, _vp, _fp],
    "cryoim_learn_save": [_vp, C.c_char_p],
    "cryoim_learn_load": [_vp, C.c_char_p],
    "cryoim_learn_params": [_vp, _vp, _vp, C.POINTER(C.c_int64)],
    "cryoim_learn_forward": [_vp, _vp, _vp, _i32, _vp, _vp, _vp],
    "cryoim_learn_set_conv": [_vp, _i32],
    "cryoim_conv3_check": [_i32, _vp, _i32, _i32, _i32, _vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp],
    "cryoim_learn_features": [_vp, _vp, _vp, _i32, _vp],
    "cryoim_learn_views": [_vp, _vp, _ip],
    "cryoim_learn_render": [_vp, _vp, _vp, _vp, _i32, _f32, _i32, _vp],
    "cryoim_central_sections": [_vp, _vp, _vp, _vp, _i32, _vp, _vp],
    "cryoim_icos_ops": [_vp],
    "cryoim_asu_fold": [_fp, _fp, _fp],
    "cryoim_equalort": [_f32, _f32, _f32, _vp],
    "cryoim_transform_ort": [_i32, _vp, _vp, _vp, _i32],
}
_RESTYPES = {"cryoim_version": C.c_int32, "cryoim_last_error": C.c_char_p}

_lib = None


class CryoimError(RuntimeError):
    def __init__(self, code: int, fn: str, msg: str):
        super().__init__(f"{fn} -> {ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: str | None = None) -> C.CDLL:
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build the CUDA library first "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(p)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int)
    if path is None:
        _lib = lib
    return lib


def call(name: str, *args) -> int:
    lib = load()
    r = getattr(lib, name)(*args)
    if r != OK:
        raise CryoimError(r, name, lib.cryoim_last_error().decode())
    return r


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data_as(C.c_void_p)
