"""The local form of the contraction search (cryoim_contract_opts.local_range): each
particle's own grid of orientations around its input (theta, phi, omega), sliced from
the map's band cube for the pass and correlated against the origin grid on the tensor
cores (BF16), the top candidates rescored in FP64.  Noise-free particles whose true
orientation lies on their grid come back within half a grid step of it, at the origin
next to the truth, from differently centred grids alike; every returned candidate's FP64 correlation equals
an independent FP64 restatement of the unbiased score sum Re(P conj(CTF S)) / (|P| |CTF S|)
(oracle central section x oracle-prepared particle, CTF, origin shift); passes split across lanes give the same result; bad options are
refused."""
import numpy as np
import pytest

from _data import small_case
from test_gpu_contract import cc_fp64, map_cube_full

pytestmark = pytest.mark.gpu

STEP, M = 2.0, 3  # local grid: +-3 steps of 2 degrees (343 orientations)


@pytest.fixture(scope="module")
def case(built):
    return small_case(P=4, T=4, step=4.0)


def offsets(P, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(-(M - 1), M, size=(P, 3))


def run_local(case, off, lanes=4, batch=64, topk=8):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["theta"] = truth[:, 0] + STEP * off[:, 0]
    q["phi"] = truth[:, 1] + STEP * off[:, 1]
    q["omega"] = truth[:, 2] + STEP * off[:, 2]
    with ci.Context(0, p) as ctx:
        ctx.set_reference_map(vol)
        ctx.set_lanes(lanes)
        ctx.set_batch(batch)
        cands = ctx.contract_search(imgs, q, origin_max=2.0, origin_step=0.5, topk=topk, pick=1,
                                    want_cands=True, local_range=M * STEP, local_step=STEP)
    return q, cands


def test_noise_free_particles_land_on_their_true_grid_point(case):
    import synth
    p, vol, tmpl, timgs, imgs, parts, truth = case
    for seed in (1, 2):
        q, cands = run_local(case, offsets(len(parts), seed))
        for i in range(len(parts)):
            # compared as rotations: near theta = 0 or 180 degrees grid points that shift
            # phi and omega together lie within a fraction of a step of the truth, and the
            # best of them can win by interpolation; the search resolves half a step
            got = tuple(float(q[f][i]) for f in ("theta", "phi", "omega"))
            err = synth.orientation_error(got, truth[i])
            assert err < 0.5 * STEP, (i, err, got, truth[i])
            assert abs(q["x"][i] - parts["x"][i]) <= 0.5 and abs(q["y"][i] - parts["y"][i]) <= 0.5
            # the pick is the best FP64 CC among the candidates
            assert q["pr"][i] == pytest.approx(cands[i, :, 6].max(), rel=1e-6)


def test_fp64_scores_match_independent_cc(case, orc):
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q, cands = run_local(case, offsets(len(parts), 3))
    vft = map_cube_full(vol)
    for i in range(len(parts)):
        for j in range(3):
            ref = cc_fp64(orc, p, vft, imgs[i], parts[i], cands[i, j, :5].astype(np.float64), unbiased=True)
            assert abs(cands[i, j, 6] - ref) < 1e-6, (i, j, cands[i, j, 6], ref)
            # the BF16 tensor-core score tracks it
            assert abs(cands[i, j, 5] - ref) < 2e-2, (i, j, cands[i, j, 5], ref)
        # candidates lie on the particle's own grid
        for j in range(cands.shape[1]):
            d = (cands[i, j, :3] - np.array([q["theta"][i], q["phi"][i], q["omega"][i]])) / STEP
            assert np.all(np.abs(d - np.round(d)) < 1e-3) and np.all(np.abs(d) <= 2 * M + 1e-3)


def test_lanes_and_passes_do_not_change_the_result(case):
    off = offsets(len(case[5]), 4)
    q1, c1 = run_local(case, off, lanes=1, batch=64)
    q4, c4 = run_local(case, off, lanes=3, batch=1)
    assert np.array_equal(q1, q4)
    assert np.array_equal(c1, c4)


def test_bad_local_options_are_refused(case):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    with ci.Context(0, p) as ctx:
        ctx.set_reference_map(vol)
        for kw in (dict(pick=0), dict(pick=1, precision="fp8"), dict(pick=1, local_step=0.0),
                   dict(pick=1, coarse=4)):
            args = dict(origin_max=2.0, origin_step=0.5, topk=8, local_range=3.0, local_step=1.0)
            args.update(kw)
            with pytest.raises(ci.CryoimError):
                ctx.contract_search(imgs, parts.copy(), **args)


def test_centred_origin_grid_is_a_window_of_the_absolute_one(case):
    """centred_origins: the origin grid sits around each particle's own (x, y).  With the
    records' origins on the absolute grid, the centred +-1 px window is a subset of the
    absolute +-3 px grid: where the absolute pick falls inside the window both forms
    return the same orientation, origin and FP64 score."""
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    off = offsets(len(parts), 5)
    q0 = parts.copy()
    q0["theta"] = truth[:, 0] + STEP * off[:, 0]
    q0["phi"] = truth[:, 1] + STEP * off[:, 1]
    q0["omega"] = truth[:, 2] + STEP * off[:, 2]
    q0["x"] = np.round(parts["x"] * 2) / 2 + 0.5
    q0["y"] = np.round(parts["y"] * 2) / 2 - 0.5
    kw = dict(origin_step=0.5, topk=8, pick=1, local_range=M * STEP, local_step=STEP)
    with ci.Context(0, p) as ctx:
        ctx.set_reference_map(vol)
        qa = q0.copy()
        ctx.contract_search(imgs, qa, origin_max=3.0, **kw)
        qc = q0.copy()
        cc = ctx.contract_search(imgs, qc, origin_max=1.0, centred_origins=True, want_cands=True, **kw)
    assert np.all(np.abs(cc[:, :, 3] - q0["x"][:, None]) <= 1.0 + 1e-6)
    assert np.all(np.abs(cc[:, :, 4] - q0["y"][:, None]) <= 1.0 + 1e-6)
    inside = (np.abs(qa["x"] - q0["x"]) <= 1.0 + 1e-6) & (np.abs(qa["y"] - q0["y"]) <= 1.0 + 1e-6)
    assert inside.sum() >= len(parts) // 2
    for f in ("theta", "phi", "omega", "x", "y"):
        np.testing.assert_allclose(qc[f][inside], qa[f][inside], atol=1e-5)
    np.testing.assert_allclose(qc["pr"][inside], qa["pr"][inside], rtol=1e-6)


def test_oversampled_sections_score_and_land_on_the_truth(case, orc):
    """Interpolation kind 2 (trilinear on the transform of the map zero-padded to twice
    its side): every returned candidate's FP64 score equals an independent FP64
    restatement on the padded transform (numpy, trilinear), and noise-free particles on a
    grid of half-degree steps land on their true grid point."""
    import cryoim_gb300 as ci
    import synth
    from scipy.ndimage import map_coordinates
    p, vol, tmpl, timgs, imgs, parts, truth = case
    n, R, r0 = p.fftsize, p.max_r, p.min_r
    step, mm = 0.5, 3
    rng = np.random.default_rng(11)
    q = parts.copy()
    off = rng.integers(-(mm - 1), mm, size=(len(parts), 3))
    q["theta"] = truth[:, 0] + step * off[:, 0]
    q["phi"] = truth[:, 1] + step * off[:, 1]
    q["omega"] = truth[:, 2] + step * off[:, 2]
    with ci.Context(0, p) as ctx:
        ctx.set_reference_map(vol)
        ctx.set_interpolation("oversampled")
        cands = ctx.contract_search(imgs, q, origin_max=2.0, origin_step=0.5, topk=6, pick=1, want_cands=True,
                                    local_range=mm * step, local_step=step)
    m = 2 * n
    pad = np.zeros((m, m, m))
    pad[n // 2:n // 2 + n, n // 2:n // 2 + n, n // 2:n // 2 + n] = vol
    F = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(pad)))
    h = n // 2
    ky, hx = np.meshgrid(np.arange(n) - h, np.arange(n) - h, indexing="ij")
    d2 = hx ** 2 + ky ** 2
    half = ((hx > 0) | ((hx == 0) & (ky > 0))) & (d2 >= r0 * r0) & (d2 <= R * R)
    hs = np.stack([hx[half], ky[half], np.zeros(int(half.sum()))]).astype(np.float64)
    for i in range(len(parts)):
        a, b, _ = orc.prep_particle(imgs[i], 1, p.imgmask_px, parts["x"][i], parts["y"][i], 0, r0, R, "f64")
        ctf = orc.ctf2d(n, parts["df1"][i], parts["df2"][i], parts["astigang"][i], p.apix, p.vol, p.cs, p.ampwg,
                        "f64")
        for j in range(3):
            c = cands[i, j].astype(np.float64)
            X = 2.0 * (synth.euler_mat(*c[:3]) @ hs) + m // 2
            s = (map_coordinates(F.real, [X[2], X[1], X[0]], order=1) +
                 1j * map_coordinates(F.imag, [X[2], X[1], X[0]], order=1))
            aa, bb = orc.centshift(a, b, c[3], c[4], "f64")
            pr, pi = (aa * ctf)[half], (-bb * ctf)[half]
            cw = ctf[half]
            want = np.sum(pr * s.real + pi * s.imag) / np.sqrt(
                np.sum(aa[half] ** 2 + bb[half] ** 2) * np.sum(cw * cw * np.abs(s) ** 2))
            assert abs(c[6] - want) < 2e-5, (i, j, c[6], want)
        err = synth.orientation_error((q["theta"][i], q["phi"][i], q["omega"][i]), truth[i])
        assert err < 0.5 * step, (i, err)
