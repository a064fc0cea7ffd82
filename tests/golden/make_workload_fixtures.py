"""Oracle fixtures of the global search and the reconstruction at production sizes.

Runs the FP64 CPU oracle (oracle/cryoim_oracle.cpp, OpenMP over particles) on the seeded
workloads of tests/_workloads.py and writes, per workload, tests/golden/<name>_search.npz:

  fingerprint  per particle image (sum, sum of squares, first, last pixel), FP64, and the
               same for the templates -- the GPU test regenerates the inputs and checks
               them against these before comparing anything;
  pick         (P, 3) the oracle's (theta, phi, omega): ort_globesearch.f90's minloc;
  pr           (P,) the minimum phase residual;
  gap          (P,) (second smallest - smallest) / smallest over the whole PR array
               (a different grid entry can only win where the scores differ by less);
  pick_index   (P, 3) grid indices (theta, phi, omega) of the pick;
  pr_row       (R, Nomega) the PR(omega) row of the pick's view for the first R particles;
  map_coef     (box128 only) the centred 3D transform, half space, |h| <= maxR, of the
               map reconstruct.f90 makes from all particles at the oracle's picks
               (tests/_workloads.py band_coefficients), complex64.

Usage: python tests/golden/make_workload_fixtures.py box256 box128 box128_fine (hours of
CPU for box128 on a few cores: 500 particles x ~75 core-seconds; box128_fine searches the
first 24 of the same particles on the 0.5-degree grid, ~650 core-seconds each).
"""
from __future__ import annotations

import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

ROWS = {"box128": 64, "box256": 16, "box128_fine": 24}
SEARCHED = {"box128_fine": 24}  # the oracle searches only the first particles of this set
CHUNK = 40


def run(name: str) -> None:
    import _workloads as W
    import pyoracle
    t0 = time.time()
    p, vol, tmpl, timgs, imgs, parts, truth = W.make(name)
    print(f"{name}: inputs in {time.time() - t0:.0f} s", flush=True)
    tm, tf = pyoracle.load_templates(timgs, tmpl, p, "f64")
    nth, nph, nom = pyoracle.grid_sizes(p.searchstep)
    P = SEARCHED.get(name, len(parts))
    imgs, parts = imgs[:P], parts[:P]
    q = parts.copy()
    pick_index = np.zeros((P, 3), np.int32)
    gap = np.zeros(P)
    rows = np.zeros((min(P, ROWS[name]), nom), np.float32)
    for c0 in range(0, P, CHUNK):
        sl = slice(c0, min(P, c0 + CHUNK))
        qq = q[sl].copy()
        pra = pyoracle.globesearch(p, tm, tf, tmpl, imgs[sl], qq, want_pr_array=True, fp="f64")
        q[sl] = qq
        for k in range(len(qq)):
            i = c0 + k
            flat = pra[k].ravel()
            b = int(np.argmin(flat))
            it, iph, iom = np.unravel_index(b, pra[k].shape)
            pick_index[i] = (it, iph, iom)
            v = np.partition(flat, 1)[:2]
            gap[i] = (v[1] - v[0]) / v[0]
            if i < len(rows):
                rows[i] = pra[k][it, iph]
        print(f"{name}: {sl.stop}/{P} particles searched, {time.time() - t0:.0f} s", flush=True)
    out = dict(fingerprint=W.fingerprint(imgs), tmpl_fingerprint=W.fingerprint(timgs),
               pick=np.stack([q["theta"], q["phi"], q["omega"]], 1).astype(np.float32),
               pr=q["pr"].astype(np.float64), gap=gap, pick_index=pick_index, pr_row=rows,
               grid=np.array([nth, nph, nom], np.int32))
    if name == "box128":
        m = pyoracle.reconstruct(p, imgs, q, fp="f64")
        coef, _ = W.band_coefficients(m, p.max_r)
        out["map_coef"] = coef.astype(np.complex64)
        out["map_particles_used"] = np.array([int(np.sum((q["pr"] <= p.pr_threshold)
                                                         & (np.abs(q["x"]) <= p.boundx)
                                                         & (np.abs(q["y"]) <= p.boundx)))])
    out["made_on"] = np.array(f"{platform.machine()} {pyoracle.num_threads()} threads, "
                              f"{time.time() - t0:.0f} s")
    path = os.path.join(HERE, f"{name}_search.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: wrote {path} ({os.path.getsize(path)} bytes) in {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    for n in sys.argv[1:] or ["box256", "box128"]:
        run(n)
