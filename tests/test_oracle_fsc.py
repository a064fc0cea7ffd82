"""Oracle restatements of the map-side routines: gold-standard half maps and FSC
(reconstruct_half.f90, reconstruct_FSC.f90), the merges of merge_icosprocess_subrec
(merge_reconstruct.f90, merge_reconstruct_FSC.f90) and the real-space icosahedral average
(img3d_icosavg.f90), checked against the full reconstruction, independent numpy
restatements and symmetry properties."""
import numpy as np
import pytest

from _data import small_case


def fsc_numpy(nx, R, odd, even):
    """reconstruct_FSC.f90:25-178 restated with whole-array numpy operations (FP64)."""
    t = 2 * R + 1
    fa1, fb1, wg1 = (np.asarray(x, np.float64).reshape(R + 1, t, t) for x in odd)
    fa2, fb2, wg2 = (np.asarray(x, np.float64).reshape(R + 1, t, t) for x in even)
    w1, w2 = wg1 + 1.0, wg2 + 1.0
    a1, b1, a2, b2 = fa1 / w1, fb1 / w1, fa2 / w2, fb2 / w2
    lz, ky, hx = np.meshgrid(np.arange(R + 1), np.arange(-R, R + 1), np.arange(-R, R + 1), indexing="ij")
    ir = np.sqrt((hx * hx + ky * ky + lz * lz).astype(np.float32)).astype(np.int64)
    m = ir <= R
    F = np.bincount(ir[m], (a1 * a2 + b1 * b2)[m], R + 1)
    F1 = 1e-10 + np.bincount(ir[m], (a1 * a1 + b1 * b1)[m], R + 1)
    F2 = 1e-10 + np.bincount(ir[m], (a2 * a2 + b2 * b2)[m], R + 1)
    fsc = F / np.sqrt(F1 * F2)
    wt = np.where(fsc <= 0, 0.0, np.sqrt(np.maximum(2 * fsc / (1 + fsc), 0)))
    A = a1 * w1 + a2 * w2
    B = b1 * w1 + b2 * w2
    W = w1 + w2 - 2.0
    wc = wt[np.minimum(ir, R)]
    A = np.where(m, A * wc, 0.0)
    B = np.where(m, B * wc, 0.0)
    W = np.where(m, W * wc, W) + 1.0
    h = nx // 2
    V = np.zeros((nx, nx, nx), np.complex128)
    s = np.where((hx + ky + lz) % 2 == 0, 1.0, -1.0)
    up = m & (lz >= 1)
    val = (A / W * s + 1j * (B / W * s))[up]
    V[lz[up] + h, ky[up] + h, hx[up] + h] = val
    V[-lz[up] + h, -ky[up] + h, -hx[up] + h] = np.conj(val)
    # plane lz = 0: (hx, ky) paired with (-hx, -ky)
    A0, B0, W0 = A[0], B[0], W[0]
    w = W0 + W0[::-1, ::-1]
    fa = (A0 + A0[::-1, ::-1]) / w
    fb = (B0 - B0[::-1, ::-1]) / w
    k0, h0 = ky[0], hx[0]
    half = m[0] & ((k0 >= 1) | ((k0 == 0) & (h0 >= 1)))
    s0 = np.where((h0 + k0) % 2 == 0, 1.0, -1.0)
    v0 = (fa * s0 + 1j * fb * s0)[half]
    V[h, k0[half] + h, h0[half] + h] = v0
    V[h, -k0[half] + h, -h0[half] + h] = np.conj(v0)
    V[h, h, h] = A0[R, R] / W0[R, R]
    out = np.real(np.fft.ifftn(V)) * nx ** 3
    z, y, x = np.meshgrid(*(np.arange(nx),) * 3, indexing="ij")
    out = np.where((x + y + z) % 2 == 0, out, -out)
    return fsc, out


def _random_tnf(rng, R, scale=1.0):
    t = 2 * R + 1
    fa = rng.normal(size=(R + 1, t, t)).astype(np.float32) * scale
    fb = rng.normal(size=(R + 1, t, t)).astype(np.float32) * scale
    wg = rng.uniform(0.0, 3.0, size=(R + 1, t, t)).astype(np.float32)
    return fa, fb, wg


@pytest.mark.parametrize("nx,R", [(16, 5), (24, 10)])
def test_fsc_combine_matches_numpy_restatement(orc, nx, R):
    rng = np.random.default_rng(nx + R)
    odd = _random_tnf(rng, R)
    even = tuple(x + 0.5 * y for x, y in zip(odd[:2], _random_tnf(rng, R)[:2])) + (odd[2] * 1.5,)
    fsc, m = orc.fsc_combine(nx, R, odd, even, "f64")
    fsc_np, m_np = fsc_numpy(nx, R, odd, even)
    assert np.abs(fsc - fsc_np).max() < 1e-12
    assert np.abs(m - m_np).max() < 1e-5 * np.abs(m_np).max()
    fsc32, m32 = orc.fsc_combine(nx, R, odd, even, "f32")
    assert np.abs(fsc32 - fsc).max() < 1e-5
    assert np.linalg.norm(m32 - m) < 1e-5 * np.linalg.norm(m)


def test_fsc_of_identical_halves_is_one(orc):
    rng = np.random.default_rng(5)
    R, nx = 6, 16
    odd = _random_tnf(rng, R)
    fsc, _ = orc.fsc_combine(nx, R, odd, odd, "f64")
    assert np.all(np.abs(fsc - 1.0) < 1e-9)
    neg = (-odd[0], -odd[1], odd[2])
    fsc_n, _ = orc.fsc_combine(nx, R, odd, neg, "f64")
    assert np.all(np.abs(fsc_n + 1.0) < 1e-9)


def test_fsc_map_is_point_inversion_of_conjugate_convention(orc):
    """reconstruct_FSC.f90:173 builds cmplx(fa, fb) where reconstruct.f90:241 builds
    cmplx(fa, -fb): the FSC map is the other one reflected through the box centre."""
    rng = np.random.default_rng(9)
    R, nx = 5, 16
    odd = _random_tnf(rng, R)
    _, m = orc.fsc_combine(nx, R, odd, odd, "f64")
    conj_odd = (odd[0], -odd[1], odd[2])
    _, mc = orc.fsc_combine(nx, R, conj_odd, conj_odd, "f64")
    # x -> -x about the centre nx/2: index i -> (nx - i) mod nx
    inv = np.roll(mc[::-1, ::-1, ::-1], 1, axis=(0, 1, 2))
    assert np.abs(m - inv).max() < 1e-9 * np.abs(m).max()


def test_half_maps_sum_to_the_full_accumulator(orc):
    """Odd + even half maps (reconstruct_half) = the full-box accumulation of
    reconstruct.f90 at the tnf cells, less its 0.01 weight start."""
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(n=32, P=3, min_res=40.0, max_res=10.0, apix=4.0)
    q = parts.copy()
    q["pr"] = 10.0
    R = p.max_r
    odd = orc.reconstruct_half(p, imgs, q, 0, "f64")
    even = orc.reconstruct_half(p, imgs, q, 1, "f64")
    _, acc = orc.reconstruct(p, imgs, q, want_acc=True, fp="f64")
    h = p.fftsize // 2
    box = acc[:, h:h + R + 1, h - R:h + R + 1, h - R:h + R + 1]
    for k, (o, e) in enumerate(zip(odd, even)):
        ref = box[k] - (0.01 if k == 2 else 0.0)
        assert np.abs(o + e - ref).max() < 1e-9 * np.abs(ref).max(), k
    # one particle per half when P == 2: the even half holds particle 2 alone
    e2 = orc.reconstruct_half(p, imgs[1:2], q[1:2], 0, "f64")
    assert np.abs(e2[2]).max() > 0
    # stride: particles 0 and 2 in the odd half
    odd_only0 = orc.reconstruct_half(p, imgs[:1], q[:1], 0, "f64")
    assert np.abs(odd[2] - odd_only0[2]).max() > 0


def test_half_map_fsc_of_noiseless_projections(orc):
    """Two halves of a noiseless, correctly oriented data set agree at low resolution."""
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(n=32, P=6, min_res=40.0, max_res=10.0, apix=4.0)
    q = parts.copy()  # true orientations and origins
    q["pr"] = 10.0
    odd = [x.astype(np.float32) for x in orc.reconstruct_half(p, imgs, q, 0, "f64")]
    even = [x.astype(np.float32) for x in orc.reconstruct_half(p, imgs, q, 1, "f64")]
    fsc, m = orc.fsc_combine(p.fftsize, p.max_r, odd, even, "f64")
    assert fsc[1:4].min() > 0.8, fsc
    assert np.isfinite(m).all()


def icosavg_numpy(m, r0, ops):
    """img3d_icosavg.f90:45-123 with whole-array numpy operations (FP64)."""
    n = m.shape[0]
    h = n // 2
    flat = m.astype(np.float64).ravel()
    lz, ky, hx = np.meshgrid(*(np.arange(n) - h,) * 3, indexing="ij")
    x0 = np.stack([hx, ky, lz], -1).reshape(-1, 3).astype(np.float64)
    inside = np.sqrt((x0 ** 2).sum(1)) <= r0
    acc = np.zeros(len(x0))
    nn = n * n
    for S in ops.astype(np.float64):
        x = x0 @ S.T + h
        i = np.trunc(x).astype(np.int64)
        a = x - i
        base = i[:, 2] * nn + i[:, 1] * n + i[:, 0]
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    idx = base + dz * nn + dy * n + dx
                    ok = (idx >= 0) & (idx < flat.size)
                    v = np.where(ok, flat[np.clip(idx, 0, flat.size - 1)], 0.0)
                    w = ((a[:, 0] if dx else 1 - a[:, 0]) * (a[:, 1] if dy else 1 - a[:, 1])
                         * (a[:, 2] if dz else 1 - a[:, 2]))
                    acc += w * v
    return np.where(inside, acc / 60.0, 0.0).reshape(n, n, n)


def test_icosavg_matches_numpy_and_is_symmetric(orc, golden_ops):
    rng = np.random.default_rng(11)
    n = 16
    m = rng.normal(size=(n, n, n)).astype(np.float32)
    r0 = n / 2 - 2
    out = orc.icosavg(m, r0, "f64")
    ref = icosavg_numpy(m, r0, golden_ops)
    assert np.abs(out - ref).max() < 1e-6 * np.abs(ref).max()
    out32 = orc.icosavg(m, r0, "f32")
    assert np.abs(out32 - out).max() < 1e-5 * np.abs(out).max()
    # the 2-fold frame has 2-fold axes on x, y and z: (x, y, z) -> (-x, -y, z) maps grid
    # points to grid points, so the average is invariant under it (up to summation order)
    h = n // 2
    a = out[:, 1:, 1:]
    b = out[:, 1:, 1:][:, ::-1, ::-1]
    assert np.abs(a - b).max() < 1e-6 * np.abs(out).max()
    # a constant map stays constant where no sample leaves the map
    c = orc.icosavg(np.full((n, n, n), 2.5, np.float32), r0, "f64")
    lz, ky, hx = np.meshgrid(*(np.arange(n) - h,) * 3, indexing="ij")
    r = np.sqrt(hx ** 2 + ky ** 2 + lz ** 2)
    assert np.abs(c[r <= r0] - 2.5).max() < 1e-6 and np.all(c[r > r0] == 0)


def test_merge_finish_equals_reconstruct_for_band_limited_partials(orc):
    """merge_reconstruct.f90 on the tnf view of reconstruct.f90's accumulator (weights less
    the 0.01 start, nothing beyond maxR) gives reconstruct.f90's map."""
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(n=32, P=3, min_res=40.0, max_res=10.0, apix=4.0)
    q = parts.copy()
    q["pr"] = 10.0
    R, h = p.max_r, p.fftsize // 2
    m_rec, acc = orc.reconstruct(p, imgs, q, want_acc=True, fp="f64")
    box = acc[:, h:h + R + 1, h - R:h + R + 1, h - R:h + R + 1].copy()
    box[2] -= 0.01
    lz, ky, hx = np.meshgrid(np.arange(R + 1), np.arange(-R, R + 1), np.arange(-R, R + 1), indexing="ij")
    far = np.sqrt(hx ** 2 + ky ** 2 + lz ** 2) > R
    box[:, far] = 0.0
    m = orc.merge_finish(p.fftsize, R, [x.astype(np.float32) for x in box], "f64")
    assert np.linalg.norm(m - m_rec) < 1e-5 * np.linalg.norm(m_rec)


def test_merge_fsc_is_the_uninverted_masked_fsc_map(orc):
    """merge_reconstruct_FSC.f90 transforms with the opposite exponent sign to
    reconstruct_FSC.f90 (its map is not point-inverted) and cuts at imgmask."""
    rng = np.random.default_rng(4)
    R, nx, r0 = 5, 16, 5.5
    odd = _random_tnf(rng, R)
    even = _random_tnf(rng, R)
    f1, m1 = orc.fsc_combine(nx, R, odd, even, "f64")
    f2, m2 = orc.merge_fsc(nx, R, odd, even, r0, "f64")
    assert np.array_equal(f1, f2)
    inv = np.roll(m1[::-1, ::-1, ::-1], 1, axis=(0, 1, 2))
    h = nx // 2
    lz, ky, hx = np.meshgrid(*(np.arange(nx) - h,) * 3, indexing="ij")
    inside = np.sqrt((hx ** 2 + ky ** 2 + lz ** 2).astype(np.float32)) <= r0
    assert np.abs(m2[inside] - inv[inside]).max() < 1e-9 * np.abs(inv).max()
    assert np.all(m2[~inside] == 0)
