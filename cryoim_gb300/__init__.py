"""cryoim_gb300 — GB300 (sm_103a) implementation of cryoIM's icosahedral
projection-matching refinement loop (icosprocess modes 4/5/1 and proc_icos).

The compute lives in libcryoim_gb300.so behind the C ABI of include/cryoim.h; this
package is the host-side mirror of the reference's drivers for Python callers (tests,
bench).  Every call goes to the CUDA library; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import (PARTICLE_DTYPE, TEMPLATE_DTYPE, CryoimError, Params, call, load, ptr)

__all__ = ["Context", "Params", "PARTICLE_DTYPE", "TEMPLATE_DTYPE", "CryoimError", "default_params",
           "icos_ops", "asu_fold", "equalort", "transform_ort", "load"]


def default_params(fftsize: int, **kw) -> Params:
    """Reference defaults for a stack of nx=fftsize (0initialvalue.f90), with keyword
    overrides by icosprocess key name (apix, minRes, maxRes, searchstep, ...), then
    the derived values of 0calc_initialvalues.f90."""
    p = Params()
    call("cryoim_params_default", C.byref(p), int(fftsize))
    alias = {"minRes": "min_res", "maxRes": "max_res", "applyCTF": "apply_ctf", "Cs": "cs",
             "PR_threshold": "pr_threshold", "boundX": "boundx", "Ncycle": "ncycle",
             "Bfactor": "bfactor"}
    for k, v in kw.items():
        k = alias.get(k, k)
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    call("cryoim_params_derive", C.byref(p))
    return p


def particles(n: int) -> np.ndarray:
    return np.zeros(n, dtype=PARTICLE_DTYPE)


def templates(n: int) -> np.ndarray:
    return np.zeros(n, dtype=TEMPLATE_DTYPE)


class Context:
    """One device context (cryoim_ctx): params, resident templates, scratch, stream."""

    def __init__(self, device: int = 0, params: Params | None = None):
        load()
        h = C.c_void_p()
        call("cryoim_ctx_create", int(device), C.byref(h))
        self._h = h
        self.params: Params | None = None
        if params is not None:
            self.set_params(params)

    # -- lifetime -------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            call("cryoim_ctx_destroy", self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- configuration --------------------------------------------------------
    def set_params(self, p: Params) -> None:
        call("cryoim_set_params", self._h, C.byref(p))
        self.params = p

    def set_stream(self, stream_handle: int | None) -> None:
        call("cryoim_ctx_set_stream", self._h, C.c_void_p(stream_handle) if stream_handle else None)

    def set_batch(self, b: int) -> None:
        call("cryoim_ctx_set_batch", self._h, int(b))

    def set_lanes(self, n: int) -> None:
        """Pass lanes of the contraction search (1..8, default 6)."""
        call("cryoim_ctx_set_lanes", self._h, int(n))

    def set_profiling(self, on: bool) -> None:
        call("cryoim_ctx_set_profiling", self._h, int(bool(on)))

    def kernel_time(self) -> tuple[float, int]:
        """(total ms, launches) of the hot search kernel since the last call."""
        ms, n = C.c_double(), C.c_int64()
        call("cryoim_ctx_kernel_time", self._h, C.byref(ms), C.byref(n))
        return ms.value, n.value

    def search_terms(self) -> float:
        t = C.c_double()
        call("cryoim_search_terms", self._h, C.byref(t))
        return t.value

    # -- templates ------------------------------------------------------------
    def project_templates(self, map3d: np.ndarray, tmpl: np.ndarray) -> np.ndarray:
        n = self.params.fftsize
        m = np.ascontiguousarray(map3d, dtype=np.float32)
        t = np.ascontiguousarray(tmpl, dtype=TEMPLATE_DTYPE)
        out = np.zeros((len(t), n, n), np.float32)
        call("cryoim_project_templates", self._h, ptr(m), ptr(t), len(t), ptr(out))
        return out

    def load_templates(self, imgs: np.ndarray, tmpl: np.ndarray) -> None:
        im = np.ascontiguousarray(imgs, dtype=np.float32)
        t = np.ascontiguousarray(tmpl, dtype=TEMPLATE_DTYPE)
        call("cryoim_load_templates", self._h, ptr(im), ptr(t), len(t))

    # -- mode 4 ---------------------------------------------------------------
    def search_grid(self) -> tuple[int, int, int, int]:
        a = [C.c_int32() for _ in range(4)]
        call("cryoim_search_grid", self._h, *[C.byref(x) for x in a])
        return tuple(x.value for x in a)

    def globesearch(self, imgs, parts: np.ndarray, want_pr_array: bool = False):
        """Global search; parts (PARTICLE_DTYPE) is updated in place.  imgs may be a
        host array (P, nx, nx) or a device pointer (int) for the _device entry point."""
        assert parts.dtype == PARTICLE_DTYPE and parts.flags["C_CONTIGUOUS"]
        pra = None
        if want_pr_array:
            nth, nph, nom, _ = self.search_grid()
            pra = np.zeros((len(parts), nth + 1, 2 * nph + 1, nom), np.float32)
        if isinstance(imgs, int):
            call("cryoim_globesearch_device", self._h, C.c_void_p(imgs), ptr(parts), len(parts), ptr(pra))
        else:
            im = np.ascontiguousarray(imgs, dtype=np.float32)
            call("cryoim_globesearch", self._h, ptr(im), ptr(parts), len(parts), ptr(pra))
        return pra

    def prscore_omega(self, ft_a, ft_b, fcut0, ctf, theta: float, phi: float) -> np.ndarray:
        nom = int(360.0 / np.float32(self.params.searchstep))
        out = np.zeros(nom, np.float32)
        a = np.ascontiguousarray(ft_a, np.float32)
        b = np.ascontiguousarray(ft_b, np.float32)
        f = np.ascontiguousarray(fcut0, np.float32)
        c = None if ctf is None else np.ascontiguousarray(ctf, np.float32)
        call("cryoim_prscore_omega", self._h, ptr(a), ptr(b), ptr(f), ptr(c), float(theta), float(phi), ptr(out))
        return out

    # -- contraction form ------------------------------------------------------
    def set_reference_map(self, map3d: np.ndarray) -> None:
        m = np.ascontiguousarray(map3d, dtype=np.float32)
        call("cryoim_set_reference_map", self._h, ptr(m))

    def contract_search(self, imgs, parts: np.ndarray, origin_max: float = 6.0,
                        origin_step: float = 0.5, topk: int = 16, pick: int = 0,
                        want_cands: bool = False, precision: str = "bf16", nbr: int = 1,
                        coarse: int = 0, learned: int = 0, nbr_best: int = 0,
                        local_range: float = 0.0, local_step: float = 0.0, fallback: float = 0.0,
                        centred_origins: bool = False, proposal_nbr: int = 0):
        """Tensor-core cross-correlation search with FP64 / phase-residual rescoring of
        the top-k and their grid neighbours within nbr steps; parts is updated in place.
        precision: "bf16" or "fp8" (e4m3 operands with per-band scales); coarse > 0: the
        proposal form (a coarse contraction names `coarse` orientations per particle,
        only their fine neighbourhoods are correlated); learned > 0: the same with the
        trained proposer's `learned` cells (learn_train / learn_load first); nbr_best > 0:
        only the neighbourhoods of the nbr_best candidates of least phase residual are
        rescored; local_range > 0: local grid search of +-local_range degrees at
        local_step around each particle's own orientation (pick 1, BF16); fallback > 0
        (learned form): particles whose phase residual lies more than `fallback` robust
        standard deviations above the call's median are searched again exhaustively
        (contract_fallbacks() counts them); centred_origins: the origin grid is centred
        on each particle's own origin; proposal_nbr: the proposals' fine neighbourhood
        (+- steps, 0 = 2).  Returns (P, topk, 8) candidates if asked: theta,
        phi, omega, x, y, CC (contraction), CC (FP64), PR."""
        assert parts.dtype == PARTICLE_DTYPE and parts.flags["C_CONTIGUOUS"]
        if precision not in ("bf16", "fp8"):
            raise ValueError("precision must be 'bf16' or 'fp8'")
        o = _abi.ContractOpts(float(origin_max), float(origin_step), int(topk), int(pick),
                              int(precision == "fp8"), int(nbr), int(coarse), int(learned), int(nbr_best),
                              float(local_range), float(local_step), float(fallback), int(bool(centred_origins)),
                              int(proposal_nbr))
        out = np.zeros((len(parts), topk, 8), np.float32) if want_cands else None
        if isinstance(imgs, int):
            call("cryoim_contract_search_device", self._h, C.c_void_p(imgs), ptr(parts), len(parts),
                 C.byref(o), ptr(out))
        else:
            im = np.ascontiguousarray(imgs, dtype=np.float32)
            call("cryoim_contract_search", self._h, ptr(im), ptr(parts), len(parts), C.byref(o), ptr(out))
        return out

    # -- learned orientation proposer ------------------------------------------
    def learn_train(self, map3d: np.ndarray, **opts) -> dict:
        """Trains the proposer on projections of map3d rendered by the library (keys of
        cryoim_learn_opts: samples, batch, seed, lr, snr, df_min, df_max, astig_max,
        origin_max).  Returns the mean loss of the last tenth of the steps, the time,
        the angle sign and the number of views."""
        o = _abi.LearnOpts()
        call("cryoim_learn_opts_default", C.byref(o))
        for k, v in opts.items():
            if not hasattr(o, k):
                raise KeyError(k)
            setattr(o, k, v)
        m = np.ascontiguousarray(map3d, dtype=np.float32)
        st = (C.c_float * 4)()
        call("cryoim_learn_train", self._h, ptr(m), C.byref(o), st)
        return {"loss": st[0], "seconds": st[1], "sign": int(st[2]), "views": int(st[3])}

    def learn_save(self, path: str) -> None:
        call("cryoim_learn_save", self._h, str(path).encode())

    def learn_load(self, path: str) -> None:
        call("cryoim_learn_load", self._h, str(path).encode())

    def learn_params(self, set_to: np.ndarray | None = None) -> np.ndarray:
        n = C.c_int64()
        call("cryoim_learn_params", self._h, None, None, C.byref(n))
        out = np.zeros(n.value, np.float32)
        s = None if set_to is None else np.ascontiguousarray(set_to, np.float32)
        if s is not None and s.size != n.value:
            raise ValueError(f"expected {n.value} parameters")
        call("cryoim_learn_params", self._h, ptr(out), ptr(s), C.byref(n))
        return out

    def learn_set_conv(self, tensor_cores: bool) -> None:
        """The proposer's convolutions on the tensor cores (TF32 operands, the default)
        or on the CUDA cores (FP32)."""
        call("cryoim_learn_set_conv", self._h, 1 if tensor_cores else 0)

    def learn_forward(self, feat: np.ndarray, truth: np.ndarray | None = None, views: int = 0):
        """Scores (B, views, 128); with truth (B, 4) also the loss (B,) and the
        parameter gradients."""
        f = np.ascontiguousarray(feat, np.float32)
        B = f.shape[0]
        nparam = self.learn_params().size
        sc = np.zeros((B, views, 128), np.float32) if views else None
        loss = np.zeros(B, np.float32) if truth is not None else None
        gr = np.zeros(nparam, np.float32) if truth is not None else None
        t = None if truth is None else np.ascontiguousarray(truth, np.float32)
        call("cryoim_learn_forward", self._h, ptr(f), ptr(t), B, ptr(sc), ptr(loss), ptr(gr))
        return sc, loss, gr

    def learn_render(self, map3d: np.ndarray, eulers: np.ndarray, par: np.ndarray, snr: float = 0.0,
                     seed: int = 0) -> np.ndarray:
        """Training renderer: (B, nx, nx) particles of map3d at eulers (B, 3) with par
        (B, 5) = (df1, df2, astig, x, y)."""
        m = np.ascontiguousarray(map3d, np.float32)
        e = np.ascontiguousarray(eulers, np.float32).reshape(-1, 3)
        pr = np.ascontiguousarray(par, np.float32).reshape(-1, 5)
        n = self.params.fftsize
        out = np.zeros((len(e), n, n), np.float32)
        call("cryoim_learn_render", self._h, ptr(m), ptr(e), ptr(pr), len(e), float(snr), int(seed), ptr(out))
        return out

    def learn_views(self) -> np.ndarray:
        """(V, 2) theta, phi of the proposer's view classes."""
        n = C.c_int32()
        call("cryoim_learn_views", self._h, None, C.byref(n))
        out = np.zeros((n.value, 2), np.float32)
        call("cryoim_learn_views", self._h, ptr(out), C.byref(n))
        return out

    def learn_features(self, imgs: np.ndarray, parts: np.ndarray) -> np.ndarray:
        im = np.ascontiguousarray(imgs, np.float32)
        out = np.zeros((len(parts), 64, 128), np.float32)
        call("cryoim_learn_features", self._h, ptr(im), ptr(parts), len(parts), ptr(out))
        return out

    def set_interpolation(self, kind: str = "trilinear", sigma: float = 0.0) -> None:
        """Sections of the contraction forms: "trilinear", "gaussian" (kernel width sigma
        voxels, 27 taps) or "oversampled" (trilinear on the transform of the map padded to
        twice its side)."""
        k = {"trilinear": 0, "gaussian": 1, "oversampled": 2}[kind]
        call("cryoim_set_interpolation", self._h, k, float(sigma))

    def contract_fallbacks(self) -> int:
        n = C.c_int32()
        call("cryoim_contract_fallbacks", self._h, C.byref(n))
        return n.value

    def contract_stats(self) -> dict:
        v = np.zeros(6, np.float64)
        call("cryoim_contract_stats", self._h, ptr(v))
        return {"slice_ms": v[0], "gemm_ms": v[1], "gemm_launches": int(v[2]), "gemm_flops": v[3],
                "orientations": int(v[4]), "kpad": int(v[5])}

    def rescore_stats(self) -> dict:
        """The contraction forms' phase-residual rescoring since the last call (timed
        while profiling is on): launch ms, launches, candidates scored."""
        v = np.zeros(3, np.float64)
        call("cryoim_rescore_stats", self._h, ptr(v))
        return {"ms": v[0], "launches": int(v[1]), "candidates": v[2]}

    # -- mode 5 ---------------------------------------------------------------
    def refine(self, imgs, parts: np.ndarray) -> None:
        assert parts.dtype == PARTICLE_DTYPE and parts.flags["C_CONTIGUOUS"]
        if isinstance(imgs, int):
            call("cryoim_refine_device", self._h, C.c_void_p(imgs), ptr(parts), len(parts))
        else:
            im = np.ascontiguousarray(imgs, dtype=np.float32)
            call("cryoim_refine", self._h, ptr(im), ptr(parts), len(parts))

    def prscore(self, ft_a, ft_b, fcut0, ctf, theta, phi, omega, x, y) -> float:
        out = C.c_float()
        a = np.ascontiguousarray(ft_a, np.float32)
        b = np.ascontiguousarray(ft_b, np.float32)
        f = np.ascontiguousarray(fcut0, np.float32)
        c = None if ctf is None else np.ascontiguousarray(ctf, np.float32)
        call("cryoim_prscore", self._h, ptr(a), ptr(b), ptr(f), ptr(c), float(theta), float(phi),
             float(omega), float(x), float(y), C.byref(out))
        return out.value

    # -- mode 1 ---------------------------------------------------------------
    def rec_begin(self) -> None:
        call("cryoim_rec_begin", self._h)

    def rec_insert(self, imgs, parts: np.ndarray) -> int:
        used = C.c_int32()
        p = np.ascontiguousarray(parts, dtype=PARTICLE_DTYPE)
        if isinstance(imgs, int):
            call("cryoim_rec_insert_device", self._h, C.c_void_p(imgs), ptr(p), len(p), C.byref(used))
        else:
            im = np.ascontiguousarray(imgs, dtype=np.float32)
            call("cryoim_rec_insert", self._h, ptr(im), ptr(p), len(p), C.byref(used))
        return used.value

    def rec_finish(self) -> np.ndarray:
        n = self.params.fftsize
        out = np.zeros((n, n, n), np.float32)
        call("cryoim_rec_finish", self._h, ptr(out))
        return out

    def rec_get_partial(self):
        R = self.params.max_r
        t = 2 * R + 1
        fa, fb, wg = (np.zeros((R + 1, t, t), np.float32) for _ in range(3))
        call("cryoim_rec_get_partial", self._h, ptr(fa), ptr(fb), ptr(wg))
        return fa, fb, wg

    def rec_begin_half(self, mask_x: float, mask_y: float) -> None:
        """One half map of a gold-standard pair (reconstruct_half.f90); images are masked
        at (mask_x, mask_y), particle(first)'s origin in the reference."""
        call("cryoim_rec_begin_half", self._h, float(mask_x), float(mask_y))

    def half_maps(self, imgs, parts: np.ndarray):
        """Odd and even tnf half maps of `parts` (particles 0, 2, ... and 1, 3, ...), both
        masked at parts[0]'s origin, as icosprocess FSC=y builds them."""
        p = np.ascontiguousarray(parts, dtype=PARTICLE_DTYPE)
        im = np.ascontiguousarray(imgs, dtype=np.float32)
        out = []
        for parity in (0, 1):
            self.rec_begin_half(p["x"][0], p["y"][0])
            if parity < len(p):
                self.rec_insert(im[parity::2], p[parity::2])
            out.append(self.rec_get_partial())
        return out

    def fsc_combine(self, odd, even, want_map: bool = True, merge: bool = False):
        """(FSC per shell 0..maxR, FSC-weighted map or None) from two tnf half maps;
        merge=True follows merge_reconstruct_FSC.f90 instead of reconstruct_FSC.f90."""
        n, R = self.params.fftsize, self.params.max_r
        a = [np.ascontiguousarray(x, np.float32) for x in (*odd, *even)]
        t = 2 * R + 1
        for x in a:
            if x.size != (R + 1) * t * t:
                raise ValueError("tnf arrays must hold (maxR+1)(2maxR+1)^2 floats")
        fsc = np.zeros(R + 1, np.float32)
        out = np.zeros((n, n, n), np.float32) if want_map else None
        call("cryoim_merge_fsc_combine" if merge else "cryoim_fsc_combine", self._h,
             *[ptr(x) for x in a], ptr(fsc), ptr(out) if want_map else None)
        return fsc, out

    # -- local_refine ---------------------------------------------------------
    def local_refine(self, lp, map3d, imgs, lparts: np.ndarray) -> None:
        """local_refine's refine_PR on sub-particle records (LOCAL_PARTICLE_DTYPE, updated in
        place); imgs: one whole-particle image per record (P, fftsize0, fftsize0)."""
        assert lparts.dtype == _abi.LOCAL_PARTICLE_DTYPE and lparts.flags["C_CONTIGUOUS"]
        m = np.ascontiguousarray(map3d, np.float32)
        im = np.ascontiguousarray(imgs, np.float32)
        call("cryoim_local_refine", self._h, C.byref(lp), ptr(m), ptr(im), ptr(lparts), len(lparts))

    # -- mode 3 ---------------------------------------------------------------
    def local_box_extract(self, imgs, parts: np.ndarray, sym: np.ndarray, loc, apix: float, sub: int,
                          pr_threshold: float = 90.0, boundx: float = 100.0, d_out: int | None = None,
                          fftsize: int | None = None):
        """local_box's sub-image stack mode: (sub images (K, sub, sub) float32 or None when
        written to the device pointer d_out, sub-particle records (LOCAL_PARTICLE_DTYPE)).
        imgs: host array (P, n, n) or a device pointer (int, with fftsize)."""
        p = np.ascontiguousarray(parts, dtype=PARTICLE_DTYPE)
        s = np.ascontiguousarray(sym, dtype=np.float32).reshape(-1, 3, 3)
        out = np.zeros(len(p) * len(s), _abi.LOCAL_PARTICLE_DTYPE)
        n = C.c_int32()
        if isinstance(imgs, int):
            assert d_out is not None and fftsize is not None
            call("cryoim_local_box_extract_device", self._h, C.c_void_p(imgs), ptr(p), len(p), int(fftsize), ptr(s),
                 len(s), float(loc[0]), float(loc[1]), float(loc[2]), float(apix), int(sub), float(pr_threshold),
                 float(boundx), C.c_void_p(d_out), ptr(out), C.byref(n))
            return None, out[: n.value].copy()
        im = np.ascontiguousarray(imgs, dtype=np.float32)
        so = np.zeros((len(p) * len(s), sub, sub), np.float32)
        call("cryoim_local_box_extract", self._h, ptr(im), ptr(p), len(p), im.shape[-1], ptr(s), len(s),
             float(loc[0]), float(loc[1]), float(loc[2]), float(apix), int(sub), float(pr_threshold), float(boundx),
             ptr(so), ptr(out), C.byref(n))
        return so[: n.value].copy(), out[: n.value].copy()

    def center(self, imgs, parts: np.ndarray, map3d=None) -> None:
        """Origin centring (calc_center.f90 against map3d, or calc_center_selfrot180.f90
        without); parts is updated in place."""
        assert parts.dtype == PARTICLE_DTYPE and parts.flags["C_CONTIGUOUS"]
        im = np.ascontiguousarray(imgs, dtype=np.float32)
        m = None if map3d is None else np.ascontiguousarray(map3d, dtype=np.float32)
        call("cryoim_center", self._h, ptr(m), ptr(im), ptr(parts), len(parts))

    def rec_add_partial(self, fa, fb, wg) -> None:
        """Add a tnf partial (each (maxR+1, 2maxR+1, 2maxR+1)) into the accumulation."""
        a = [np.ascontiguousarray(x, np.float32) for x in (fa, fb, wg)]
        R = self.params.max_r
        if any(x.size != (R + 1) * (2 * R + 1) ** 2 for x in a):
            raise ValueError("tnf arrays must hold (maxR+1)(2maxR+1)^2 floats")
        call("cryoim_rec_add_partial", self._h, *[ptr(x) for x in a])

    def rec_finish_merge(self) -> np.ndarray:
        n = self.params.fftsize
        out = np.zeros((n, n, n), np.float32)
        call("cryoim_rec_finish_merge", self._h, ptr(out))
        return out

    def icosavg(self, map3d, r0: float) -> np.ndarray:
        """Real-space icosahedral average (img3d_icosavg.f90) of a cubic map."""
        m = np.array(map3d, np.float32, copy=True, order="C")
        n = m.shape[0]
        if m.shape != (n, n, n):
            raise ValueError("map must be cubic")
        call("cryoim_icosavg", self._h, ptr(m), n, float(r0))
        return m

    # -- central sections ----------------------------------------------------
    def central_sections(self, ft_re, ft_im, eulers) -> tuple[np.ndarray, np.ndarray]:
        n = self.params.fftsize
        e = np.ascontiguousarray(eulers, np.float32).reshape(-1, 3)
        re = np.ascontiguousarray(ft_re, np.float32)
        im = np.ascontiguousarray(ft_im, np.float32)
        ore = np.zeros((len(e), n, n), np.float32)
        oim = np.zeros((len(e), n, n), np.float32)
        call("cryoim_central_sections", self._h, ptr(re), ptr(im), ptr(e), len(e), ptr(ore), ptr(oim))
        return ore, oim


# -- proc_icos (host geometry in the library) ----------------------------------
def local_particles(n: int) -> np.ndarray:
    return np.zeros(n, dtype=_abi.LOCAL_PARTICLE_DTYPE)


def local_params(fftsize: int, fftsize0: int, **kw) -> "_abi.LocalParams":
    """local_refine defaults (0input_parameters.f90) with keyword overrides by field name
    (apix, max_res, imgmask, nsym, ncycle, apply_ctf, normalize, vol, cs, ampwg,
    refine_angle, refine_shift, convf), then the derived values."""
    p = _abi.LocalParams()
    call("cryoim_local_params_default", C.byref(p), int(fftsize), int(fftsize0))
    p.refine_angle = p.refine_shift = 0.0
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    call("cryoim_local_params_derive", C.byref(p))
    return p


def local_sym_matrices(sym: str) -> np.ndarray:
    out = np.zeros((60, 3, 3), np.float32)
    n = C.c_int32()
    call("cryoim_local_sym_matrices", sym.encode(), ptr(out), C.byref(n))
    return out[:n.value].copy()


def local_box_coordinates(parts: np.ndarray, sym: np.ndarray, loc, apix: float, fftsize: int,
                          pr_threshold: float = 90.0, boundx: float = 100.0) -> np.ndarray:
    """local_box's coordinate mode: sub-particle records for the selected particles."""
    p = np.ascontiguousarray(parts, dtype=PARTICLE_DTYPE)
    s = np.ascontiguousarray(sym, np.float32).reshape(-1, 3, 3)
    out = local_particles(len(p) * len(s))
    n = C.c_int32()
    call("cryoim_local_box_coordinates", ptr(p), len(p), ptr(s), len(s), float(loc[0]), float(loc[1]),
         float(loc[2]), float(apix), int(fftsize), float(pr_threshold), float(boundx), ptr(out), C.byref(n))
    return out[:n.value].copy()


def icos_ops() -> np.ndarray:
    out = np.zeros((60, 3, 3), np.float32)
    call("cryoim_icos_ops", ptr(out))
    return out


def asu_fold(theta: float, phi: float, omega: float) -> tuple[float, float, float]:
    t, p, o = C.c_float(theta), C.c_float(phi), C.c_float(omega)
    call("cryoim_asu_fold", C.byref(t), C.byref(p), C.byref(o))
    return t.value, p.value, o.value


def equalort(theta: float, phi: float, omega: float) -> np.ndarray:
    out = np.zeros((60, 3), np.float32)
    call("cryoim_equalort", float(theta), float(phi), float(omega), ptr(out))
    return out


def transform_ort(to: int, theta, phi, omega):
    t = np.ascontiguousarray(theta, np.float32).copy()
    p = np.ascontiguousarray(phi, np.float32).copy()
    o = np.ascontiguousarray(omega, np.float32).copy()
    call("cryoim_transform_ort", int(to), ptr(t), ptr(p), ptr(o), len(t))
    return t, p, o


def conv3_check(x: np.ndarray, W: np.ndarray, bias: np.ndarray | None = None, relu: bool = False,
                dpre: np.ndarray | None = None, tensor_cores: bool = True):
    """Test hook of the proposer's 3x3 convolution kernels (circular in the 128 angles,
    zero-padded in radius): x (B, Cin, H, 128), W (Cout, Cin, 3, 3) -> out (B, Cout, H,
    128); with dpre (B, Cout, H, 128) also the weight and bias gradients.  Returns
    (out, dW, db)."""
    x = np.ascontiguousarray(x, np.float32)
    W = np.ascontiguousarray(W, np.float32)
    B, Cin, H, T = x.shape
    Cout = W.shape[0]
    if T != 128 or W.shape != (Cout, Cin, 3, 3):
        raise ValueError("x must be (B, Cin, H, 128) and W (Cout, Cin, 3, 3)")
    b = None if bias is None else np.ascontiguousarray(bias, np.float32)
    g = None if dpre is None else np.ascontiguousarray(dpre, np.float32)
    out = np.zeros((B, Cout, H, T), np.float32)
    dW = np.zeros_like(W) if g is not None else None
    db = np.zeros(Cout, np.float32) if g is not None else None
    call("cryoim_conv3_check", 1 if tensor_cores else 0, ptr(x), B, Cin, H, ptr(W), ptr(b), Cout,
         1 if relu else 0, ptr(out), ptr(g), ptr(dW), ptr(db))
    return out, dW, db
