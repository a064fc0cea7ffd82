"""The seeded synthetic workloads the parity fixtures are made from, at the sizes of the
production runs the GPU path is built for:

* box128 -- the CPU-runnable search: 128^3 phantom (240 Gaussian blobs at radius 40-52 px
  plus a shell at 30-34 px), 500 particles of 128^2 at 2.0 A/px, defocus U(1.0, 3.0) um
  without astigmatism, origins U(+-3 px), white noise at SNR 0.1, 20 templates at random
  asymmetric-unit orientations, band 1/60-1/10 A^-1 (minR 4, maxR 26), 1-degree grid.
* box128_fine -- the same data searched on the 0.5-degree grid (the precision form).
* box256 -- the production shapes: 256^3 phantom (radii x2) at 1.5 A/px, 256^2
  particles, defocus U(0.8, 3.5) um with astigmatism up to 0.1 um at a random angle,
  origins U(+-6 px), SNR 0.05, 20 templates, band 1/50-1/6 A^-1 (minR 7, maxR 64),
  1-degree grid.

Projections are taken by synth.project_numpy (FP64 real-space line integrals with the
geometry of project_template2d.f90), so the inputs do not depend on the GPU and the
fixture script (which runs the CPU oracle) and the GPU tests see the same images.  The
projections are spread over a spawn process pool: no worker is forked from a process
that has touched the GPU.  A spawn worker re-imports the caller's main module, so a
script that calls make() must keep its work under `if __name__ == "__main__":`.  `fingerprint()` summarises the inputs so a test can check
that it regenerated exactly the images the fixture was made from.
"""
from __future__ import annotations

import functools
import multiprocessing as mp
import os

import numpy as np

SPECS = {
    "box128": dict(n=128, apix=2.0, min_res=60.0, max_res=10.0, searchstep=1.0, ntemplates=20,
                   particles=500, df=(1.0, 3.0), astig=0.0, origin=3.0, snr=0.1, ampwg=0.07,
                   seed=20261204),
    # the box128 particles on the 0.5-degree grid (the precision form's search)
    "box128_fine": dict(n=128, apix=2.0, min_res=60.0, max_res=10.0, searchstep=0.5, ntemplates=20,
                        particles=500, df=(1.0, 3.0), astig=0.0, origin=3.0, snr=0.1, ampwg=0.07,
                        seed=20261204),
    "box256": dict(n=256, apix=1.5, min_res=50.0, max_res=6.0, searchstep=1.0, ntemplates=20,
                   particles=16, df=(0.8, 3.5), astig=0.1, origin=6.0, snr=0.05, ampwg=0.07,
                   seed=20261205),
}


def params(name: str):
    import cryoim_gb300 as ci
    s = SPECS[name]
    n = s["n"]
    return ci.default_params(n, apix=s["apix"], minRes=s["min_res"], maxRes=s["max_res"],
                             searchstep=s["searchstep"], ampwg=s["ampwg"],
                             imgmask=(n // 2 - 2) * s["apix"])


def _project_chunk(args):
    vol, eulers = args
    import synth
    return synth.project_numpy(vol, eulers)


class _PoolProjector:
    """synth.project_numpy over a spawn pool, chunked by orientation (same FP64 result
    per image as the serial call)."""

    def __init__(self, workers: int):
        self.workers = workers

    def __call__(self, vol, eulers):
        e = np.asarray(eulers)
        if self.workers <= 1 or len(e) < 4:
            import synth
            return synth.project_numpy(vol, e)
        chunks = [c for c in np.array_split(e, min(len(e), 4 * self.workers)) if len(c)]
        with mp.get_context("spawn").Pool(self.workers) as pool:
            parts = pool.map(_project_chunk, [(vol, c) for c in chunks])
        return np.concatenate(parts, 0)


def _workers() -> int:
    return max(1, min(16, (os.cpu_count() or 2)))


@functools.lru_cache(maxsize=2)
def make(name: str):
    """(params, vol, tmpl, timgs, imgs, parts, truth) of the named workload (every
    particle of it: the draws of particle i depend on the particle count)."""
    if name == "box128_fine":  # the box128 data, searched on the finer grid
        return (params(name),) + make("box128")[1:]
    import cryoim_gb300 as ci
    import synth
    s = SPECS[name]
    P = s["particles"]
    proj = _PoolProjector(_workers())
    p = params(name)
    vol = synth.phantom(s["n"], s["seed"])
    rng = np.random.default_rng(s["seed"])
    te = synth.random_asu_orientations(s["ntemplates"], rng)
    tmpl = ci.templates(s["ntemplates"])
    tmpl["particle_id"] = np.arange(1, s["ntemplates"] + 1)
    tmpl["theta"], tmpl["phi"], tmpl["omega"] = te[:, 0], te[:, 1], te[:, 2]
    timgs = proj(vol, te.astype(np.float32))
    imgs, parts, truth = synth.make_particles(vol, P, s["seed"] + 1, proj, s["apix"], df_range=s["df"],
                                              astig_max=s["astig"], origin_max=s["origin"], snr=s["snr"],
                                              ampwg=s["ampwg"])
    return p, vol, tmpl, timgs, imgs, parts, truth


def fingerprint(imgs: np.ndarray) -> np.ndarray:
    """Per image (sum, sum of squares, first pixel, last pixel) in FP64."""
    x = np.asarray(imgs, np.float64).reshape(len(imgs), -1)
    return np.stack([x.sum(1), (x * x).sum(1), x[:, 0], x[:, -1]], 1)


def band_coefficients(map3d: np.ndarray, max_r: int):
    """The map's centred 3D transform on the half space (z > 0, or z == 0 with y > 0, or
    z == y == 0 with x >= 0) within |h| <= max_r: the whole content of a reconstruction
    (insertion fills no other frequency), as (coefficients complex128, shell index)."""
    n = map3d.shape[0]
    F = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(np.asarray(map3d, np.float64))))
    h = np.arange(n) - n // 2
    z, y, x = np.meshgrid(h, h, h, indexing="ij")
    r = np.sqrt(x * x + y * y + z * z)
    half = (z > 0) | ((z == 0) & (y > 0)) | ((z == 0) & (y == 0) & (x >= 0))
    sel = half & (r <= max_r)
    return F[sel], np.rint(r[sel]).astype(np.int32)


def fsc_shells(a: np.ndarray, b: np.ndarray, shell: np.ndarray, max_r: int) -> np.ndarray:
    """FSC per integer shell 1..max_r between two coefficient sets on the same samples."""
    out = np.zeros(max_r + 1)
    for s in range(1, max_r + 1):
        k = shell == s
        num = np.real(np.vdot(a[k], b[k]))
        den = np.sqrt(np.vdot(a[k], a[k]).real * np.vdot(b[k], b[k]).real)
        out[s] = num / den if den > 0 else 1.0
    return out[1:]
