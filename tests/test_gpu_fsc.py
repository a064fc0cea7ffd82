"""Gold-standard half maps and FSC on the GPU (cryoim_rec_begin_half + cryoim_rec_insert +
cryoim_rec_get_partial, cryoim_fsc_combine) against the oracle's reconstruct_half and
reconstruct_FSC restatements.

Tolerances: half-map accumulators within 1e-4 relative L2 (FP32 transforms and FP32
atomics against the FP64 oracle, as for the full reconstruction); from identical tnf
inputs, FSC within 1e-5 absolute and the weighted map within 1e-5 relative L2.
"""
import numpy as np
import pytest

from _data import small_case

pytestmark = pytest.mark.gpu
RTOL = 1e-4


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def case():
    return small_case()


def test_half_maps_match_oracle(built, orc, case):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["pr"] = 10.0
    q["pr"][2] = 95.0  # above PR_threshold: left out of the odd half
    with ci.Context(0, p) as ctx:
        odd, even = ctx.half_maps(imgs, q)
    for parity, got in ((0, odd), (1, even)):
        want = orc.reconstruct_half(p, imgs, q, parity, "f64")
        for k in range(3):
            assert _rel(got[k], want[k]) < RTOL, (parity, k, _rel(got[k], want[k]))


def test_half_map_masks_at_the_range_origin(built, orc, case):
    """Both halves mask at particle(first)'s origin, not at their own first particle."""
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["pr"] = 10.0
    q["x"][0], q["y"][0] = 9.0, -7.0  # far from particle 2's origin: the mask moves
    with ci.Context(0, p) as ctx:
        _, even = ctx.half_maps(imgs, q)
        ctx.rec_begin_half(q["x"][1], q["y"][1])
        ctx.rec_insert(imgs[1::2], q[1::2])
        own = ctx.rec_get_partial()
    want = orc.reconstruct_half(p, imgs, q, 1, "f64")
    assert _rel(even[0], want[0]) < RTOL
    assert _rel(own[0], want[0]) > 10 * RTOL


def test_fsc_combine_matches_oracle(built, orc, case):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["pr"] = 10.0
    odd = [x.astype(np.float32) for x in orc.reconstruct_half(p, imgs, q, 0, "f64")]
    even = [x.astype(np.float32) for x in orc.reconstruct_half(p, imgs, q, 1, "f64")]
    f_orc, m_orc = orc.fsc_combine(p.fftsize, p.max_r, odd, even, "f64")
    with ci.Context(0, p) as ctx:
        f_gpu, m_gpu = ctx.fsc_combine(odd, even)
        f_only, none = ctx.fsc_combine(odd, even, want_map=False)
    assert none is None and np.array_equal(f_only, f_gpu)
    assert np.abs(f_gpu - f_orc).max() < 1e-5, np.abs(f_gpu - f_orc).max()
    assert _rel(m_gpu, m_orc) < 1e-5, _rel(m_gpu, m_orc)


def test_fsc_of_identical_halves_is_one_on_gpu(built, case):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["pr"] = 10.0
    with ci.Context(0, p) as ctx:
        odd, _ = ctx.half_maps(imgs, q)
        f, _ = ctx.fsc_combine(odd, odd, want_map=False)
    assert np.all(np.abs(f - 1.0) < 1e-6), f


def test_half_map_pipeline_end_to_end(built, orc, case):
    """GPU half maps -> GPU FSC and map against the oracle chain on the same particles."""
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["pr"] = 10.0
    with ci.Context(0, p) as ctx:
        odd, even = ctx.half_maps(imgs, q)
        f_gpu, m_gpu = ctx.fsc_combine(odd, even)
    o = [x.astype(np.float32) for x in orc.reconstruct_half(p, imgs, q, 0, "f64")]
    e = [x.astype(np.float32) for x in orc.reconstruct_half(p, imgs, q, 1, "f64")]
    f_orc, m_orc = orc.fsc_combine(p.fftsize, p.max_r, o, e, "f64")
    assert np.abs(f_gpu - f_orc).max() < 1e-3
    assert _rel(m_gpu, m_orc) < RTOL


def test_finish_refuses_half_maps(built, case):
    import cryoim_gb300 as ci
    p, *_ = case
    with ci.Context(0, p) as ctx:
        ctx.rec_begin_half(0.0, 0.0)
        with pytest.raises(ci.CryoimError):
            ctx.rec_finish()


def test_icosavg_matches_oracle(built, orc, case):
    import cryoim_gb300 as ci
    p, vol, *_ = case
    r0 = p.imgmask_px
    with ci.Context(0, p) as ctx:
        got = ctx.icosavg(vol, r0)
    want = orc.icosavg(vol, r0, "f64")
    assert _rel(got, want) < 1e-5, _rel(got, want)
    assert np.all(got[np.abs(want) == 0] == 0)


def test_finish_applies_realspaceavg(built, orc, case):
    """realspaceavg=y: reconstruct.f90:253-255 and reconstruct_FSC.f90:185-187 average the
    map in real space before writing it."""
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["pr"] = 10.0
    pa = ci.Params.from_buffer_copy(p)
    pa.realspaceavg = 1
    with ci.Context(0, pa) as ctx:
        ctx.rec_begin()
        ctx.rec_insert(imgs, q)
        m = ctx.rec_finish()
        odd, even = ctx.half_maps(imgs, q)
        _, mf = ctx.fsc_combine(odd, even)
    want = orc.icosavg(orc.reconstruct(p, imgs, q, fp="f64"), p.imgmask_px, "f64")
    assert _rel(m, want) < RTOL, _rel(m, want)
    with ci.Context(0, p) as ctx:
        _, plain = ctx.fsc_combine(odd, even)
    assert _rel(mf, orc.icosavg(plain, p.imgmask_px, "f64")) < 1e-5


def test_merge_finish_and_merge_fsc_match_oracle(built, orc, case):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["pr"] = 10.0
    odd = [x.astype(np.float32) for x in orc.reconstruct_half(p, imgs, q, 0, "f64")]
    even = [x.astype(np.float32) for x in orc.reconstruct_half(p, imgs, q, 1, "f64")]
    total = [a + b for a, b in zip(odd, even)]
    with ci.Context(0, p) as ctx:
        ctx.rec_begin()
        ctx.rec_add_partial(*odd)
        ctx.rec_add_partial(*even)
        m = ctx.rec_finish_merge()
        f, mf = ctx.fsc_combine(odd, even, merge=True)
    want = orc.merge_finish(p.fftsize, p.max_r, total, "f64")
    assert _rel(m, want) < 1e-5, _rel(m, want)
    f_orc, mf_orc = orc.merge_fsc(p.fftsize, p.max_r, odd, even, p.imgmask_px, "f64")
    assert np.abs(f - f_orc).max() < 1e-5
    assert _rel(mf, mf_orc) < 1e-5, _rel(mf, mf_orc)


def test_particle_shards_exchange_tnf_partials(built, case, tmp_path):
    """Two particle shards, as two ranks of a sharded run would own them (one context
    each): each inserts its range and writes its tnf partial with the library's writer;
    the partials read back, summed (the reduction shard.allreduce_partials performs) and
    added to a fresh accumulation finish to the map of one context that inserted every
    particle.  reconstruct.f90:92 masks every image at particle(first)'s origin, so the
    records share one origin here (as merge_icosprocess_subrec's users must)."""
    import cryoim_gb300 as ci
    from test_io import lib
    p, vol, tmpl, timgs, imgs, parts, truth = case
    q = parts.copy()
    q["pr"] = 0.0
    q["x"] = q["y"] = 0.0
    L = lib()
    R = p.max_r
    t = 2 * R + 1
    ps = ci.Params.from_buffer_copy(p)
    ps.subrec = 1  # tnf partials: weights start at 0 (reconstruct_substep.f90:25)
    shards = [slice(0, 1), slice(1, len(q))]
    got = []
    for k, sl in enumerate(shards):
        with ci.Context(0, ps) as c:
            c.rec_begin()
            c.rec_insert(imgs[sl], q[sl])
            fa, fb, wg = c.rec_get_partial()
        path = str(tmp_path / f"shard{k}.tnf").encode()
        assert L.cryoim_tnf_write(path, p.fftsize, R, p.apix, p.imgmask, 0, 0, fa.ctypes.data, fb.ctypes.data,
                                  wg.ctypes.data) == 0
        ih, fh = np.zeros(4, np.int32), np.zeros(2, np.float32)
        back = [np.zeros((R + 1, t, t), np.float32) for _ in range(3)]
        assert L.cryoim_tnf_read(path, ih.ctypes.data, fh.ctypes.data, back[0].ctypes.data, back[1].ctypes.data,
                                 back[2].ctypes.data) == 0
        assert all(np.array_equal(a, b) for a, b in zip((fa, fb, wg), back))
        got.append(back)
    with ci.Context(0, p) as c:
        c.rec_begin()
        for part in got:
            c.rec_add_partial(*part)
        merged = c.rec_finish_merge()
    with ci.Context(0, ps) as c:
        c.rec_begin()
        c.rec_insert(imgs, q)
        whole = c.rec_get_partial()
    with ci.Context(0, p) as c:
        c.rec_begin()
        c.rec_add_partial(*whole)
        want = c.rec_finish_merge()
    assert _rel(sum(g[0].astype(np.float64) for g in got), whole[0]) < 1e-5
    assert _rel(merged, want) < 1e-5
