"""Edge cases of the device entry points: empty particle ranges are a no-op (the
reference's loops over first..last simply do not run when first > last), a single
particle searches like the same particle inside a batch, and the contraction forms and
the reconstruction accept them too."""
import numpy as np
import pytest

from _data import small_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(built):
    return small_case(P=3, T=4, step=6.0)


def test_empty_ranges_are_a_no_op(case):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        empty = parts[:0].copy()
        ctx.globesearch(imgs[:0], empty)
        ctx.refine(imgs[:0], empty)
        ctx.contract_search(imgs[:0], empty, origin_max=2.0, origin_step=0.5, topk=4)
        ctx.rec_begin()
        ctx.rec_insert(imgs[:0], empty)
        m = ctx.rec_finish()
        assert np.all(np.isfinite(m))


def test_one_particle_alone_equals_its_batch_result(case):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = case
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        qb = parts.copy()
        ctx.globesearch(imgs, qb)
        cb = parts.copy()
        ctx.contract_search(imgs, cb, origin_max=2.0, origin_step=0.5, topk=4)
        for i in range(len(parts)):
            q1 = parts[i:i + 1].copy()
            ctx.globesearch(imgs[i:i + 1], q1)
            assert (q1["theta"][0], q1["phi"][0], q1["omega"][0]) == (qb["theta"][i], qb["phi"][i], qb["omega"][i])
            assert q1["pr"][0] == pytest.approx(qb["pr"][i], rel=1e-6)
            c1 = parts[i:i + 1].copy()
            ctx.contract_search(imgs[i:i + 1], c1, origin_max=2.0, origin_step=0.5, topk=4)
            assert (c1["theta"][0], c1["phi"][0], c1["omega"][0]) == (cb["theta"][i], cb["phi"][i], cb["omega"][i])
