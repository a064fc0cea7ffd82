"""End-to-end behaviour of the oracle on a small noise-free case: the global search
(ort_globesearch) finds each particle's orientation up to icosahedral symmetry, the
refinement (ort_refinement) does not lose it, and the symmetrised reconstruction
(reconstruct) of the particles at their true orientations correlates with the phantom."""
import numpy as np

from _data import small_case


def test_globesearch_recovers_orientation(orc):
    import synth
    p, vol, tmpl, timgs, imgs, parts, truth = small_case()
    tm, tf = orc.load_templates(timgs, tmpl, p, "f64")
    q = parts.copy()
    pra = orc.globesearch(p, tm, tf, tmpl, imgs, q, want_pr_array=True, fp="f64")
    for i in range(len(q)):
        found = (q["theta"][i], q["phi"][i], q["omega"][i])
        assert synth.orientation_error(found, truth[i]) < 1.5 * p.searchstep
        assert q["pr"][i] == pra[i].min()
        # the output row keeps the previous values and the deltas (ort_globesearch.f90:109-126)
        assert q["theta0"][i] == parts["theta"][i] and q["x"][i] == parts["x"][i]
        assert np.isclose(q["dtheta"][i], q["theta"][i] - q["theta0"][i])


def test_fp32_oracle_agrees_with_fp64(orc):
    p, vol, tmpl, timgs, imgs, parts, truth = small_case()
    a64, b64, f64 = orc.prep_particle(imgs[0], 1, p.imgmask_px, parts["x"][0], parts["y"][0], 1,
                                      p.min_r, p.max_r, "f64")
    a32, b32, f32 = orc.prep_particle(imgs[0], 1, p.imgmask_px, parts["x"][0], parts["y"][0], 1,
                                      p.min_r, p.max_r, "f32")
    assert np.abs(a32 - a64).max() < 1e-5 * np.abs(a64).max()
    tm64, tf64 = orc.load_templates(timgs, tmpl, p, "f64")
    tm32, tf32 = orc.load_templates(timgs, tmpl, p, "f32")
    ctf = orc.ctf2d(p.fftsize, parts["df1"][0], parts["df2"][0], parts["astigang"][0], p.apix,
                    p.vol, p.cs, p.ampwg, "f64")
    tort = np.stack([tmpl["theta"], tmpl["phi"], tmpl["omega"]], 1)
    pr64 = orc.pr_omega(a64, b64, f64, tm64, tort, tf64, ctf, p.min_r, p.max_r, p.searchstep, 81.0, 8.0, fp="f64")
    pr32 = orc.pr_omega(a32, b32, f32, tm32, tort, tf32, ctf.astype(np.float32), p.min_r, p.max_r,
                        p.searchstep, 81.0, 8.0, fp="f32")
    assert np.abs(pr32 - pr64).max() / pr64.max() < 5e-4


def test_refine_keeps_or_improves(orc):
    import synth
    p, vol, tmpl, timgs, imgs, parts, truth = small_case()
    tm, tf = orc.load_templates(timgs, tmpl, p, "f64")
    q = parts.copy()
    orc.globesearch(p, tm, tf, tmpl, imgs, q, fp="f64")
    r = q.copy()
    p.ncycle = 3
    orc.refine(p, tm, tf, tmpl, imgs, r, fp="f64")
    for i in range(len(r)):
        e0 = synth.orientation_error((q["theta"][i], q["phi"][i], q["omega"][i]), truth[i])
        e1 = synth.orientation_error((r["theta"][i], r["phi"][i], r["omega"][i]), truth[i])
        assert e1 < e0 + 1.0
        assert r["pr0"][i] == q["pr"][i]
    p.ncycle = 6


def test_reconstruction_correlates_with_phantom(orc):
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(P=3)
    q = parts.copy()
    q["pr"] = 0.0
    m = orc.reconstruct(p, imgs, q, fp="f64")
    n = p.fftsize
    # compare within the band: low-pass both to maxR
    F1 = np.fft.fftshift(np.fft.fftn(m))
    F2 = np.fft.fftshift(np.fft.fftn(vol))
    z, y, x = np.indices((n, n, n)) - n // 2
    band = np.sqrt(x ** 2 + y ** 2 + z ** 2) <= p.max_r - 2
    c = np.abs(np.vdot(F1[band], F2[band])) / np.linalg.norm(F1[band]) / np.linalg.norm(F2[band])
    assert c > 0.5, c


def test_view_set_is_decided_in_fp32(orc):
    """ort_globesearch.f90:7-8,70-78 tests the asymmetric unit in `real`: at theta = 90
    degrees cos rounds to -4.4e-8 in FP32, so the equator's views are never searched.
    The FP64 oracle makes the same decision in FP32: the views it searches are exactly
    those of an independent numpy restatement of the FP32 test (bench.asu_views)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    step = 3.0  # 69 + 7 x 3 = 90: the equator is on this grid
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(P=1, step=step)
    tm, tf = orc.load_templates(timgs, tmpl, p, "f64")
    pra = orc.globesearch(p, tm, tf, tmpl, imgs, parts.copy(), want_pr_array=True, fp="f64")[0]
    searched = pra.min(axis=-1) < 999.0
    nph = (searched.shape[1] - 1) // 2
    want = np.zeros_like(searched)
    for th, ph in bench.asu_views(step):
        want[int(round((th - 69.0) / step)), int(round(ph / step)) + nph] = True
    assert np.array_equal(searched, want)
    assert not searched[int(round((90.0 - 69.0) / step))].any()
    assert searched.sum() > 0
