"""The projection-matching contraction form (cryoim_contract_search): every returned
candidate's FP64 cross-correlation equals an independent FP64 restatement (oracle
central section of the map's centred transform x oracle-prepared particle, CTF and
origin shift), the BF16 tensor-core score tracks it, the phase-residual rescoring
matches the oracle's cal_crosslin_PR, and noise-free particles land on their true
orientation (up to symmetry)."""
import numpy as np
import pytest

from _data import small_case

pytestmark = pytest.mark.gpu


def map_cube_full(vol):
    """Centred FT of the map (phase at the map centre), standard complex, / n^3."""
    n = vol.shape[-1]
    z, y, x = np.indices(vol.shape)
    chk = np.where((x + y + z) % 2 == 1, -1.0, 1.0)
    ft = np.fft.fftn(vol.astype(np.float64) * chk) / n ** 3
    k = np.arange(n) - n // 2
    sg = np.where((k[:, None, None] + k[None, :, None] + k[None, None, :]) % 2 == 1, -1.0, 1.0)
    return ft * sg


def cc_fp64(orc, p, vol_ft, img, part, cand, unbiased=False):
    """The FP64 score of one candidate: sum Re(CTF P conj S) over the half-plane band,
    normalised by |CTF P| |S| (the global forms, whose sections are shared by all
    particles) or, unbiased, by |P| |CTF S| (the local form)."""
    n, R, r0 = p.fftsize, p.max_r, p.min_r
    h = n // 2
    sre, sim = orc.central_section(vol_ft.real, vol_ft.imag, *cand[:3], fp="f64")
    a, b, _ = orc.prep_particle(img, 1, p.imgmask_px, part["x"], part["y"], 0, r0, R, "f64")
    a, b = orc.centshift(a, b, cand[3], cand[4], "f64")
    ctf = orc.ctf2d(n, part["df1"], part["df2"], part["astigang"], p.apix, p.vol, p.cs, p.ampwg, "f64")
    ky, hx = np.meshgrid(np.arange(n) - h, np.arange(n) - h, indexing="ij")
    d2 = hx ** 2 + ky ** 2
    half = ((hx > 0) | ((hx == 0) & (ky > 0))) & (d2 >= r0 * r0) & (d2 <= R * R)
    pr, pi = (a * ctf)[half], (-b * ctf)[half]
    qr, qi = sre[half], sim[half]
    if unbiased:
        c = ctf[half]
        return float(np.sum(pr * qr + pi * qi) /
                     np.sqrt(np.sum(a[half] ** 2 + b[half] ** 2) * np.sum(c * c * (qr * qr + qi * qi))))
    return float(np.sum(pr * qr + pi * qi) / np.sqrt(np.sum(pr * pr + pi * pi) * np.sum(qr * qr + qi * qi)))


@pytest.fixture(scope="module")
def run(built, orc):
    import cryoim_gb300 as ci
    case = small_case(P=3, T=4, step=4.0)
    p, vol, tmpl, timgs, imgs, parts, truth = case
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        q = parts.copy()
        cands = ctx.contract_search(imgs, q, origin_max=2.0, origin_step=0.5, topk=8, want_cands=True)
        stats = ctx.contract_stats()
    return case, q, cands, stats


def test_fp64_rescoring_matches_independent_cc(run, orc):
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    vol_ft = map_cube_full(vol)
    for i in range(len(parts)):
        for j in range(3):
            c = cands[i, j]
            want = cc_fp64(orc, p, vol_ft, imgs[i], parts[i], c[:5].astype(np.float64))
            assert abs(c[6] - want) < 2e-5, (i, j, c[6], want)
            # BF16 operands, FP32 accumulation
            assert abs(c[5] - c[6]) < 2e-2, (i, j, c[5], c[6])


def test_candidates_are_sorted_and_distinct(run):
    (p, *_), q, cands, stats = run
    for i in range(cands.shape[0]):
        cc = cands[i, :, 5]
        assert np.all(np.diff(cc) <= 1e-6)
        keys = {tuple(np.round(c[:5], 4)) for c in cands[i]}
        assert len(keys) == cands.shape[1]
    assert stats["orientations"] > 0 and stats["kpad"] % 64 == 0


def test_pr_rescoring_matches_oracle(run, orc):
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    tm, tf = orc.load_templates(timgs, tmpl, p, "f64")
    tort = np.stack([tmpl["theta"], tmpl["phi"], tmpl["omega"]], 1)
    for i in range(len(parts)):
        a, b, f = orc.prep_particle(imgs[i], 1, p.imgmask_px, parts["x"][i], parts["y"][i], 0,
                                    p.min_r, p.max_r, "f64")
        ctf = orc.ctf2d(p.fftsize, parts["df1"][i], parts["df2"][i], parts["astigang"][i], p.apix,
                        p.vol, p.cs, p.ampwg, "f64")
        for j in range(cands.shape[1]):
            c = cands[i, j]
            # scored at the particle's own origin, as ort_globesearch does
            want = orc.pr_single(a, b, f, tm, tort, tf, ctf, p.min_r, p.max_r, *c[:3],
                                 parts["x"][i], parts["y"][i], fp="f64")
            assert abs(c[7] - want) / want < 5e-3
        # the pick is the minimum over the candidates and their grid neighbours
        assert q["pr"][i] <= cands[i, :, 7].min() + 1e-6
        want = orc.pr_single(a, b, f, tm, tort, tf, ctf, p.min_r, p.max_r, q["theta"][i], q["phi"][i],
                             q["omega"][i], parts["x"][i], parts["y"][i], fp="f64")
        assert abs(q["pr"][i] - want) / want < 5e-3
        assert q["x"][i] == parts["x"][i] and q["y"][i] == parts["y"][i]


def test_pick_matches_exhaustive_pr_search(run, built):
    """On noise-free particles the exhaustive FP32 search's minimum lies next to a
    contraction candidate, so the two forms return the same grid orientation."""
    import cryoim_gb300 as ci
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        qe = parts.copy()
        ctx.globesearch(imgs, qe)
    for i in range(len(parts)):
        assert (q["theta"][i], q["phi"][i], q["omega"][i]) == (qe["theta"][i], qe["phi"][i], qe["omega"][i])
        assert abs(q["pr"][i] - qe["pr"][i]) / qe["pr"][i] < 1e-3


def test_noise_free_particles_find_their_orientation(run):
    import synth
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    for i in range(len(parts)):
        top = cands[i, 0]
        err = synth.orientation_error(tuple(top[:3]), truth[i])
        assert err < 1.5 * p.searchstep, (i, err)
        assert abs(top[3] - parts["x"][i]) <= 0.5 and abs(top[4] - parts["y"][i]) <= 0.5


def test_fp8_form_tracks_fp64_and_picks_the_same_orientation(run, built):
    """FP8-e4m3 operands with per-band power-of-two scales: the descaled tensor-core CC of
    every candidate tracks its FP64 CC, the candidates carry the same FP64 rescoring, and
    the pick equals the BF16 form's."""
    import cryoim_gb300 as ci
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        q8 = parts.copy()
        c8 = ctx.contract_search(imgs, q8, origin_max=2.0, origin_step=0.5, topk=8, want_cands=True,
                                 precision="fp8")
        st8 = ctx.contract_stats()
    assert st8["kpad"] % 128 == 0
    for i in range(len(parts)):
        for j in range(c8.shape[1]):
            assert abs(c8[i, j, 5] - c8[i, j, 6]) < 5e-2, (i, j, c8[i, j, 5], c8[i, j, 6])
        assert (q8["theta"][i], q8["phi"][i], q8["omega"][i]) == (q["theta"][i], q["phi"][i], q["omega"][i])
        # the BF16 form's best candidate is among the FP8 form's best three
        assert any(np.allclose(c8[i, j, :3], cands[i, 0, :3]) for j in range(3))


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_proposal_form_picks_the_exhaustive_orientation(run, built, precision):
    """coarse > 0: the coarse level's proposals and their fine neighbourhoods contain the
    exhaustive contraction's best candidates on these particles, so the pick is the same."""
    import cryoim_gb300 as ci
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        qp = parts.copy()
        cp = ctx.contract_search(imgs, qp, origin_max=2.0, origin_step=0.5, topk=8, want_cands=True,
                                 precision=precision, coarse=8)
    for i in range(len(parts)):
        assert (qp["theta"][i], qp["phi"][i], qp["omega"][i]) == (q["theta"][i], q["phi"][i], q["omega"][i])
        # k distinct orientations, sorted by the contraction score
        assert len({tuple(np.round(c[:3], 4)) for c in cp[i]}) == cp.shape[1]
        assert np.all(np.diff(cp[i, :, 5]) <= 1e-6)
        # the best FP64 CC among the candidates is no worse than the exhaustive BF16 form's;
        # FP8 scores may place an orientation at a neighbouring 0.5 px origin
        tol = 1e-4 if precision == "bf16" else 5e-3
        assert cp[i, :, 6].max() > cands[i, :, 6].max() - tol, (i, cp[i, :, 6], cands[i, :, 6])


def test_proposal_neighbourhood_width(run, built):
    """proposal_nbr: the proposals' fine neighbourhood; the widths that cover the coarse
    grid's gaps (+-2 and +-3 fine steps) give the exhaustive pick on these particles, +-1
    runs, and widths outside 0..4 are refused."""
    import cryoim_gb300 as ci
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        for pn in (2, 3):
            qp = parts.copy()
            ctx.contract_search(imgs, qp, origin_max=2.0, origin_step=0.5, topk=8, coarse=8, proposal_nbr=pn)
            for i in range(len(parts)):
                assert (qp["theta"][i], qp["phi"][i], qp["omega"][i]) == (q["theta"][i], q["phi"][i], q["omega"][i])
        qp = parts.copy()
        ctx.contract_search(imgs, qp, origin_max=2.0, origin_step=0.5, topk=8, coarse=8, proposal_nbr=1)
        assert np.all(qp["pr"] < 999)
        for bad in (-1, 5):
            with pytest.raises(ci.CryoimError):
                ctx.contract_search(imgs, parts.copy(), origin_max=2.0, origin_step=0.5, topk=8, coarse=8,
                                    proposal_nbr=bad)


@pytest.mark.parametrize("form", [dict(), dict(coarse=8)])
def test_pass_lanes_give_the_same_results(run, built, form):
    """Passes dealt to 1, 2 or 3 lanes (own streams, buffers and host threads) return
    bit-identical orientations, scores and candidates: one particle per pass here, so
    every lane runs at least one pass."""
    import cryoim_gb300 as ci
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    out = []
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        ctx.set_batch(1)
        for lanes in (1, 2, 3):
            ctx.set_lanes(lanes)
            ql = parts.copy()
            cl = ctx.contract_search(imgs, ql, origin_max=2.0, origin_step=0.5, topk=8, want_cands=True, **form)
            out.append((ql, cl))
    for ql, cl in out[1:]:
        assert np.array_equal(ql, out[0][0])
        assert np.array_equal(cl, out[0][1])


@pytest.mark.parametrize("sigma", [0.5, 0.8])
def test_gaussian_kernel_sections_match_oracle(run, built, orc, sigma):
    """cryoim_set_interpolation(kind 1): the section bank, the FP64 rescoring and the
    pick use the 27-voxel Gaussian kernel.  Every candidate's FP64 CC equals the
    independent restatement with the oracle's Gaussian central section; the BF16 score of
    the tensor-core contraction tracks it; noise-free particles still land on their
    orientation."""
    import cryoim_gb300 as ci
    import synth
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        ctx.set_interpolation("gaussian", sigma)
        qg = parts.copy()
        cg = ctx.contract_search(imgs, qg, origin_max=2.0, origin_step=0.5, topk=8, want_cands=True, pick=1)
        with pytest.raises(ci.CryoimError):
            ctx.set_interpolation("gaussian", 5.0)
    vol_ft = map_cube_full(vol)
    n, R, r0 = p.fftsize, p.max_r, p.min_r
    h = n // 2
    ky, hx = np.meshgrid(np.arange(n) - h, np.arange(n) - h, indexing="ij")
    d2 = hx ** 2 + ky ** 2
    half = ((hx > 0) | ((hx == 0) & (ky > 0))) & (d2 >= r0 * r0) & (d2 <= R * R)
    for i in range(len(parts)):
        a, b, _ = orc.prep_particle(imgs[i], 1, p.imgmask_px, parts["x"][i], parts["y"][i], 0, r0, R, "f64")
        ctf = orc.ctf2d(n, parts["df1"][i], parts["df2"][i], parts["astigang"][i], p.apix, p.vol, p.cs, p.ampwg,
                        "f64")
        for j in range(3):
            c = cg[i, j].astype(np.float64)
            sre, sim = orc.central_section_gauss(vol_ft.real, vol_ft.imag, *c[:3], sigma, fp="f64")
            aa, bb = orc.centshift(a, b, c[3], c[4], "f64")
            pr, pi = (aa * ctf)[half], (-bb * ctf)[half]
            qr, qi = sre[half], sim[half]
            want = np.sum(pr * qr + pi * qi) / np.sqrt(np.sum(pr * pr + pi * pi) * np.sum(qr * qr + qi * qi))
            assert abs(c[6] - want) < 2e-5, (i, j, c[6], want)
            assert abs(c[5] - c[6]) < 2e-2, (i, j, c[5], c[6])
        err = synth.orientation_error((qg["theta"][i], qg["phi"][i], qg["omega"][i]), truth[i])
        assert err < 1.5 * p.searchstep, (i, err)


def test_rescoring_stats_count_the_scored_candidates(run, built):
    """cryoim_rescore_stats: with profiling on, the phase-residual rescoring's launches,
    their time and the candidates they scored (the candidates and, with nbr = 1, their grid
    neighbours: at least topk per particle); reset by the read."""
    import cryoim_gb300 as ci
    (p, vol, tmpl, timgs, imgs, parts, truth), q, cands, stats = run
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        ctx.set_lanes(1)
        ctx.set_profiling(True)
        ctx.contract_search(imgs, parts.copy(), origin_max=2.0, origin_step=0.5, topk=8)
        st = ctx.rescore_stats()
        assert st["launches"] >= 1 and st["ms"] > 0.0
        assert st["candidates"] >= 8 * len(parts)
        assert ctx.rescore_stats()["launches"] == 0
