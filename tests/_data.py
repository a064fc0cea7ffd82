"""Small seeded cases shared by the CPU and GPU tests (numpy projections)."""
from __future__ import annotations

import functools

import numpy as np


def projector(map3d, eulers):
    import synth
    return synth.project_numpy(map3d, eulers)


@functools.lru_cache(maxsize=8)
def small_case(n=64, P=3, T=4, step=4.0, apix=4.0, min_res=60.0, max_res=12.0, snr=0.0, seed=7,
               apply_ctf=1):
    import cryoim_gb300 as ci
    import synth
    p = ci.default_params(n, apix=apix, minRes=min_res, maxRes=max_res, searchstep=step,
                          ampwg=0.07, apply_ctf=apply_ctf, imgmask=(n // 2 - 2) * apix)
    vol = synth.phantom(n, seed)
    rng = np.random.default_rng(seed + 1)
    te = synth.random_asu_orientations(T, rng)
    timgs = projector(vol, te.astype(np.float32))
    tmpl = ci.templates(T)
    tmpl["particle_id"] = np.arange(1, T + 1)
    tmpl["theta"], tmpl["phi"], tmpl["omega"] = te[:, 0], te[:, 1], te[:, 2]
    imgs, parts, truth = synth.make_particles(vol, P, seed + 2, projector, apix,
                                              origin_max=2.0, snr=snr)
    return p, vol, tmpl, timgs, imgs, parts, truth
