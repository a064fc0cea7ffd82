"""cryoim_prscore_noalloc: the allocation-free refinement scorer, for callers that
cannot allocate device memory while they score.  It must give the same scores as
cryoim_prscore (the allocating entry point) on the same particle and templates, within
the 1e-4 relative tolerance of the other parity tests, on two calls in a row (its
scratch array keeps the previous call's contents, which must not leak into the next).

This file is collected last so that a run that stops at the first failure has run
every other test first; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from _data import small_case

pytestmark = pytest.mark.gpu


def _window(a, n, r):
    w, off = 2 * r + 2, n // 2 - r
    return np.ascontiguousarray(a[off:off + w, off:off + w])


def test_noalloc_scores_match_prscore(built, orc):
    import torch
    import cryoim_gb300 as ci
    from cryoim_gb300._abi import call

    p, vol, tmpl, timgs, imgs, parts, truth = small_case()
    n, R = p.fftsize, p.max_r
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    tm, tf = orc.load_templates(timgs, tmpl, p, "f64")
    tort = np.stack([tmpl["theta"], tmpl["phi"], tmpl["omega"]], 1).astype(np.float32)
    rng = np.random.default_rng(3)
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        for call_no, i in enumerate([0, 1]):  # two calls in a row, different particles
            a, b, f = orc.prep_particle(imgs[i], 1, p.imgmask_px, parts["x"][i], parts["y"][i], 0,
                                        p.min_r, p.max_r, "f64")
            ctf = orc.ctf2d(n, parts["df1"][i], parts["df2"][i], parts["astigang"][i], p.apix, p.vol,
                            p.cs, p.ampwg, "f64")
            K = 11 if call_no == 0 else 7
            cand = np.stack([rng.uniform(69, 90, K), rng.uniform(-30, 30, K), rng.uniform(0, 360, K),
                             rng.uniform(-3, 3, K), rng.uniform(-3, 3, K)], 1).astype(np.float32)
            want = np.array([ctx.prscore(a, b, f, ctf, *c) for c in cand], np.float32)
            # device inputs: band windows of the same transforms
            band = np.stack([_window(a, n, R), _window(b, n, R)], -1).astype(np.float32)
            tband = np.stack([np.stack([_window(tm[t, 0], n, R), _window(tm[t, 1], n, R)], -1)
                              for t in range(len(tmpl))]).astype(np.float32)
            d = {k: torch.from_numpy(np.ascontiguousarray(v, np.float32)).to(dev) for k, v in dict(
                band=band, fcut0=f, ctf=_window(ctf, n, R), tband=tband, tfcut=tf, tort=tort,
                cand=cand).items()}
            out = torch.full((K,), -1.0, device=dev)
            s = torch.cuda.current_stream().cuda_stream
            call("cryoim_prscore_noalloc", n, p.min_r, p.max_r, C.c_void_p(d["band"].data_ptr()),
                 C.c_void_p(d["fcut0"].data_ptr()), C.c_void_p(d["ctf"].data_ptr()),
                 C.c_void_p(d["tband"].data_ptr()), C.c_void_p(d["tfcut"].data_ptr()),
                 C.c_void_p(d["tort"].data_ptr()), len(tmpl), C.c_void_p(d["cand"].data_ptr()), K,
                 C.c_void_p(out.data_ptr()), C.c_void_p(s))
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            np.testing.assert_allclose(got, want, rtol=1e-4, err_msg=f"call {call_no}")
        # without a CTF: the caller's own template cuts (no scratch cuts)
        i = 2
        a, b, f = orc.prep_particle(imgs[i], 1, p.imgmask_px, parts["x"][i], parts["y"][i], 0,
                                    p.min_r, p.max_r, "f64")
        cand = np.stack([rng.uniform(69, 90, 5), rng.uniform(-30, 30, 5), rng.uniform(0, 360, 5),
                         rng.uniform(-3, 3, 5), rng.uniform(-3, 3, 5)], 1).astype(np.float32)
        pn = ci.Params.from_buffer_copy(p)
        pn.apply_ctf = 0
        ctx.set_params(pn)
        ctx.load_templates(timgs, tmpl)
        want = np.array([ctx.prscore(a, b, f, None, *c) for c in cand], np.float32)
        band = np.stack([_window(a, n, R), _window(b, n, R)], -1).astype(np.float32)
        d = {k: torch.from_numpy(np.ascontiguousarray(v, np.float32)).to(dev) for k, v in dict(
            band=band, fcut0=f, tband=tband, tfcut=tf, tort=tort, cand=cand).items()}
        out = torch.full((5,), -1.0, device=dev)
        call("cryoim_prscore_noalloc", n, p.min_r, p.max_r, C.c_void_p(d["band"].data_ptr()),
             C.c_void_p(d["fcut0"].data_ptr()), None, C.c_void_p(d["tband"].data_ptr()),
             C.c_void_p(d["tfcut"].data_ptr()), C.c_void_p(d["tort"].data_ptr()), len(tmpl),
             C.c_void_p(d["cand"].data_ptr()), 5, C.c_void_p(out.data_ptr()),
             C.c_void_p(torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-4, err_msg="no CTF")


def test_noalloc_rejects_sizes_beyond_its_limits(built):
    import cryoim_gb300._abi as abi
    lib = abi.load()
    dummy = C.c_void_p(16)  # never dereferenced: the size checks come first
    r = lib.cryoim_prscore_noalloc(64, 4, 22, dummy, dummy, dummy, dummy, dummy, dummy, 65, dummy, 1,
                                   dummy, None)
    assert r == abi.ERR_SIZE
    r = lib.cryoim_prscore_noalloc(64, 4, 22, dummy, dummy, dummy, dummy, dummy, dummy, 4, dummy, 12,
                                   dummy, None)
    assert r == abi.ERR_SIZE
    r = lib.cryoim_prscore_noalloc(64, 4, 22, None, dummy, dummy, dummy, dummy, dummy, 4, dummy, 1,
                                   dummy, None)
    assert r == abi.ERR_ARG
