"""Seeded synthetic icosahedral data with the shapes of the reference workloads.

The reference ships no data; its workloads are described by size only.  This module
builds a phantom (Gaussian blobs placed by the 60 icosahedral rotations plus a solid
shell), random orientations, CTF-modulated noisy projections and template sets.  It is
numpy only and imports nothing of the cryoim_gb300 package: the 60 rotations and the
particle record type are passed in (`ops`, `dtype`), and only when they are not is the
package asked for its own.  The bench's CPU reference arm passes the oracle's.

Conventions follow icosprocess: ZYZ Euler angles R = Rz(phi) Ry(theta) Rz(omega)
(euler_mat.f90), a projection samples the map at R*(x, y, z) (project_template2d.f90),
an origin (x, y) means the object centre sits at pixel (nx/2 + x, nx/2 + y), and the
phantom is generated directly in the 2-fold frame icosprocess works in.

Projection itself is delegated to a `projector(map3d, eulers) -> images` callable so
that CPU tests can use the oracle and GPU runs the library's projector.
"""
from __future__ import annotations

import numpy as np


def _ops(ops):
    if ops is None:
        import cryoim_gb300
        ops = cryoim_gb300.icos_ops()
    return np.asarray(ops).astype(np.float64)


def euler_mat(theta, phi, omega) -> np.ndarray:
    t, p, o = np.deg2rad([theta, phi, omega])
    c1, c2, c3, s1, s2, s3 = np.cos(p), np.cos(t), np.cos(o), np.sin(p), np.sin(t), np.sin(o)
    return np.array([[c1 * c2 * c3 - s1 * s3, -c1 * c2 * s3 - c3 * s1, c1 * s2],
                     [c2 * c3 * s1 + c1 * s3, -c2 * s1 * s3 + c1 * c3, s1 * s2],
                     [-c3 * s2, s2 * s3, c2]])


def euler_from_matrix(r: np.ndarray) -> tuple[float, float, float]:
    th = np.degrees(np.arccos(np.clip(r[2, 2], -1.0, 1.0)))
    ph = np.degrees(np.arctan2(r[1, 2], r[0, 2]))
    om = np.degrees(np.arctan2(r[2, 1], -r[2, 0]))
    return float(th), float(ph), float(om)


def random_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    """Haar-uniform rotations (unit quaternions) as ZYZ Euler angles, (n, 3) degrees."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z); R[:, 0, 1] = 2 * (x * y - z * w); R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w); R[:, 1, 1] = 1 - 2 * (x * x + z * z); R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w); R[:, 2, 1] = 2 * (y * z + x * w); R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return np.array([euler_from_matrix(r) for r in R])


_A = None


def asu_planes():
    d2r = np.pi / 180
    c31, s31, c69, s69 = np.cos(31.717 * d2r), np.sin(31.717 * d2r), np.cos(69.09 * d2r), np.sin(69.09 * d2r)
    return (-s31 * c69, -c31 * c69, s31 * s69, -s31 * c69, c31 * c69, s31 * s69)


def in_asu(v: np.ndarray) -> np.ndarray:
    A1, B1, C1, A2, B2, C2 = asu_planes()
    x, y, z = v[..., 0], v[..., 1], v[..., 2]
    return (z >= 0) & (z <= -(A1 * x + B1 * y) / C1) & (z <= -(A2 * x + B2 * y) / C2)


def random_asu_orientations(n: int, rng: np.random.Generator) -> np.ndarray:
    """Orientations whose view direction lies in the asymmetric unit; omega uniform."""
    out = []
    while len(out) < n:
        v = rng.normal(size=(4096, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        for u in v[in_asu(v)]:
            th = np.degrees(np.arccos(np.clip(u[2], -1, 1)))
            ph = np.degrees(np.arctan2(u[1], u[0]))
            out.append((th, ph, rng.uniform(0, 360)))
            if len(out) == n:
                break
    return np.array(out)


def phantom(n: int, seed: int, ops=None, nblob_seeds: int = 4) -> np.ndarray:
    """240 Gaussian blobs (sigma 2.5 px, amplitude U(0.5,1.5) per seed, radius 40-52 px)
    plus a shell (radius 30-34 px, density 0.3), all scaled by n/128.  ops: the 60
    icosahedral rotations (FP32 table, 2-fold frame)."""
    rng = np.random.default_rng(seed)
    s = n / 128.0
    ops = _ops(ops)
    vol = np.zeros((n, n, n), np.float32)
    c = n // 2
    zz, yy, xx = np.meshgrid(np.arange(n) - c, np.arange(n) - c, np.arange(n) - c, indexing="ij")
    r = np.sqrt(xx ** 2 + yy ** 2 + zz ** 2)
    vol[(r >= 30 * s) & (r <= 34 * s)] = 0.3
    sigma = 2.5 * s
    half = int(np.ceil(4 * sigma))
    g = np.arange(-half, half + 1)
    for _ in range(nblob_seeds):
        while True:
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            if in_asu(u):
                break
        pos = u * rng.uniform(40 * s, 52 * s)
        amp = rng.uniform(0.5, 1.5)
        for S in ops:
            p = S @ pos
            ip = np.round(p).astype(int)
            lo = ip - half + c
            if lo.min() < 0 or (ip + half + c).max() >= n:
                continue
            dz = (g + ip[2] - p[2])[:, None, None]
            dy = (g + ip[1] - p[1])[None, :, None]
            dx = (g + ip[0] - p[0])[None, None, :]
            blob = amp * np.exp(-(dx ** 2 + dy ** 2 + dz ** 2) / (2 * sigma ** 2))
            vol[lo[2]:lo[2] + 2 * half + 1, lo[1]:lo[1] + 2 * half + 1, lo[0]:lo[0] + 2 * half + 1] += blob
    return vol


def project_numpy(map3d: np.ndarray, eulers: np.ndarray) -> np.ndarray:
    """Real-space projections in FP64 with the geometry of project_template2d.f90:
    pixel (ix, iy) sums map(R*(x, y, z)) over z inside the sphere of radius nx/2-1.
    For the small boxes of tests and smoke runs (input generation only)."""
    n = map3d.shape[-1]
    h = n // 2
    z, y, x = np.indices((n, n, n)) - h
    keep = np.sqrt(x ** 2 + y ** 2 + z ** 2) < (h - 1)
    X = np.stack([x[keep], y[keep], z[keep]]).astype(np.float64)
    pix = (y[keep] + h) * n + (x[keep] + h)
    m = map3d.astype(np.float64).ravel()
    out = np.empty((len(eulers), n, n), np.float32)
    for k, e in enumerate(np.asarray(eulers, np.float64)):
        u = euler_mat(*e) @ X + h
        i0 = np.floor(u).astype(np.int64)
        f = u - i0
        acc = np.zeros(X.shape[1])
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    w = ((f[0] if dx else 1 - f[0]) * (f[1] if dy else 1 - f[1]) *
                         (f[2] if dz else 1 - f[2]))
                    acc += w * m[((i0[2] + dz) * n + (i0[1] + dy)) * n + (i0[0] + dx)]
        out[k] = np.bincount(pix, weights=acc, minlength=n * n).reshape(n, n)
    return out


def project_fourier(map3d: np.ndarray, eulers: np.ndarray) -> np.ndarray:
    """Projections by the projection-slice theorem (one 3D FFT, trilinear central
    sections, 2D inverse FFTs): same geometry as project_numpy, for large boxes where
    only the inputs' statistics matter (CPU-side input generation)."""
    from scipy.ndimage import map_coordinates
    n = map3d.shape[-1]
    h = n // 2
    F = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(map3d.astype(np.float32)))).astype(np.complex64)
    iy, ix = np.meshgrid(np.arange(n) - h, np.arange(n) - h, indexing="ij")
    pts = np.stack([ix.ravel(), iy.ravel(), np.zeros(n * n)]).astype(np.float64)
    out = np.empty((len(eulers), n, n), np.float32)
    for k, e in enumerate(np.asarray(eulers, np.float64)):
        x = euler_mat(*e) @ pts + h
        coords = np.stack([x[2], x[1], x[0]])
        s = (map_coordinates(F.real, coords, order=1, mode="constant") +
             1j * map_coordinates(F.imag, coords, order=1, mode="constant")).reshape(n, n)
        out[k] = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(s))).real
    return out


def ctf2d(n, df1, df2, astig, apix, vol=300.0, cs=2.7, ampwg=0.1) -> np.ndarray:
    """getCTF2d.f90 in FP64 on the centred grid (defocus um, Cs mm)."""
    lam = 0.387818 / np.sqrt(vol * (1 + 0.978459e-3 * vol))
    ky, hx = np.meshgrid(np.arange(n) - n // 2, np.arange(n) - n // 2, indexing="ij")
    phi = np.arctan2(ky, hx)
    phi = np.where(phi < 0, phi + 2 * np.pi, phi) - np.deg2rad(astig)
    df = df1 * 1e4 * np.cos(phi) ** 2 + df2 * 1e4 * np.sin(phi) ** 2
    res = np.sqrt(hx ** 2 + ky ** 2) / n / apix
    ph = 2 * np.pi * (-cs * 1e7 * lam ** 3 * res ** 4 / 4 + df * lam * res ** 2 / 2)
    return -(np.sqrt(1 - ampwg ** 2) * np.sin(ph) + ampwg * np.cos(ph))


def apply_ctf_shift(img: np.ndarray, ctf: np.ndarray | None, x: float, y: float) -> np.ndarray:
    n = img.shape[-1]
    F = np.fft.fftshift(np.fft.fft2(img))
    if ctf is not None:
        F = F * ctf
    ky, hx = np.meshgrid(np.arange(n) - n // 2, np.arange(n) - n // 2, indexing="ij")
    F = F * np.exp(-2j * np.pi * (hx * x + ky * y) / n)
    return np.fft.ifft2(np.fft.ifftshift(F)).real


def make_particles(map3d: np.ndarray, P: int, seed: int, projector, apix: float,
                   df_range=(1.0, 3.0), astig_max=0.0, origin_max=3.0, snr=0.1,
                   vol=300.0, cs=2.7, ampwg=0.1, eulers: np.ndarray | None = None, dtype=None):
    """Projections at Haar-random orientations, CTF, origin shift and white noise.
    Returns (images (P,n,n) float32, particle records (dtype: the cryoim_particle
    layout), true eulers)."""
    if dtype is None:
        import cryoim_gb300
        dtype = cryoim_gb300.PARTICLE_DTYPE
    rng = np.random.default_rng(seed)
    n = map3d.shape[-1]
    e = random_rotations(P, rng) if eulers is None else np.asarray(eulers, np.float64)
    proj = projector(map3d, e.astype(np.float32))
    rec = np.zeros(P, dtype)
    imgs = np.empty((P, n, n), np.float32)
    yy, xx = np.meshgrid(np.arange(n) - n // 2, np.arange(n) - n // 2, indexing="ij")
    inside = (xx ** 2 + yy ** 2) <= (0.4 * n) ** 2
    for i in range(P):
        df1 = rng.uniform(*df_range)
        da = rng.uniform(0, astig_max) if astig_max > 0 else 0.0
        ang = rng.uniform(0, 180) if astig_max > 0 else 0.0
        x, y = rng.uniform(-origin_max, origin_max, size=2)
        c = ctf2d(n, df1, df1 + da, ang, apix, vol, cs, ampwg)
        sig = apply_ctf_shift(proj[i].astype(np.float64), c, x, y)
        v = sig[inside].var()
        noise = rng.normal(scale=np.sqrt(v / snr), size=(n, n)) if snr and snr > 0 else 0.0
        imgs[i] = (sig + noise).astype(np.float32)
        r = rec[i]
        r["particle_id"] = i + 1
        r["img_id"] = i + 1           # unique imgID per particle (the CTF cache keys on it)
        r["img_particle_id"] = i + 1
        r["df1"], r["df2"], r["astigang"] = df1, df1 + da, ang
        r["x"], r["y"] = x, y
        r["theta"], r["phi"], r["omega"] = e[i]
    return imgs, rec, e


def orientation_error(e1, e2, ops=None) -> float:
    """Smallest rotation angle (degrees) between e1 and any icosahedral equivalent of e2."""
    ops = _ops(ops)
    R1 = euler_mat(*e1)
    R2 = euler_mat(*e2)
    best = 180.0
    for S in ops:
        M = R1.T @ (S @ R2)
        c = np.clip((np.trace(M) - 1) / 2, -1, 1)
        best = min(best, float(np.degrees(np.arccos(c))))
    return best
