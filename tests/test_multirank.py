"""Two CPU ranks (gloo): particle shards give the same search results as one process,
and the all_reduce of partial reconstruction accumulators equals the single-process
accumulation (the exchange merge_icosprocess_subrec does through tnf files).  Each
rank's partial goes through the library's tnf writer and reader (cryoim_tnf_write /
cryoim_tnf_read, host code of libcryoim_gb300.so) before the reduction, and the
merged map of the reduced partial (merge_reconstruct.f90, oracle restatement) equals
the one of the single-process partial."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT


def test_particle_ranges_cover_exactly():
    from cryoim_gb300.shard import particle_range
    for n in (0, 1, 7, 100):
        for w in (1, 2, 3, 8):
            seen = []
            for r in range(w):
                f, l = particle_range(n, r, w)
                seen += list(range(f, l + 1))
            assert seen == list(range(1, n + 1))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import pyoracle
    from _data import small_case
    from cryoim_gb300.shard import allreduce_partials, particle_range
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(P=4, T=3, step=6.0)
    first, last = particle_range(len(parts), rank, world)
    mine = slice(first - 1, last)
    # search shard
    tm, tf = pyoracle.load_templates(timgs, tmpl, p, "f64")
    q = parts[mine].copy()
    pyoracle.globesearch(p, tm, tf, tmpl, imgs[mine], q, nthreads=1, fp="f64")
    got = [None] * world
    dist.all_gather_object(got, [tuple(r) for r in q[["theta", "phi", "omega", "pr"]]])
    # reconstruction shard -> partial accumulators -> sum.  reconstruct.f90:92 masks every
    # image at particle(first)'s origin, so shards with different `first` would mask
    # differently (as separate reference runs do); the reduction is checked unmasked.
    from cryoim_gb300 import Params
    pm = Params.from_buffer_copy(p)
    pm.use_imgmask = 0
    qq = parts.copy()
    qq["pr"] = 0.0
    _, acc = pyoracle.reconstruct(pm, imgs[mine], qq[mine], want_acc=True, fp="f64")
    fa, fb, wg = allreduce_partials(acc[0], acc[1], acc[2], wg_init=0.01)
    # the tnf exchange: this rank's half-box partial (reconstruct_substep.f90) written and
    # read back by the library, then summed over the ranks
    import ctypes as C
    from cryoim_gb300 import load
    L = load()
    R = p.max_r
    t = 2 * R + 1
    sub = [np.ascontiguousarray(x, np.float32) for x in pyoracle.reconstruct_half(pm, imgs[mine], qq[mine], 0)]
    sub2 = [np.ascontiguousarray(x, np.float32) for x in pyoracle.reconstruct_half(pm, imgs[mine], qq[mine], 1)]
    part = [a + b for a, b in zip(sub, sub2)]
    path = os.path.join(os.path.dirname(out), f"rank{rank}.tnf")
    assert L.cryoim_tnf_write(path.encode(), p.fftsize, R, p.apix, p.imgmask, 0, 0, part[0].ctypes.data,
                              part[1].ctypes.data, part[2].ctypes.data) == 0
    ih, fh = np.zeros(4, np.int32), np.zeros(2, np.float32)
    back = [np.zeros((R + 1, t, t), np.float32) for _ in range(3)]
    assert L.cryoim_tnf_read(path.encode(), ih.ctypes.data, fh.ctypes.data, back[0].ctypes.data,
                             back[1].ctypes.data, back[2].ctypes.data) == 0
    assert all(np.array_equal(a, b) for a, b in zip(part, back)) and list(ih[:2]) == [p.fftsize, R]
    tsum = allreduce_partials(*[b.astype(np.float64) for b in back])
    if rank == 0:
        np.savez(out, fa=fa, fb=fb, wg=wg, res=np.array(sum(got, []), dtype=np.float64),
                 tfa=tsum[0], tfb=tsum[1], twg=tsum[2])
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.slow
def test_two_ranks_match_one_process(built, orc, tmp_path):
    import torch.multiprocessing as mp
    from _data import small_case
    out = str(tmp_path / "r.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    r = np.load(out)
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(P=4, T=3, step=6.0)
    tm, tf = orc.load_templates(timgs, tmpl, p, "f64")
    q = parts.copy()
    orc.globesearch(p, tm, tf, tmpl, imgs, q, nthreads=1, fp="f64")
    want = np.array([tuple(x) for x in q[["theta", "phi", "omega", "pr"]]], np.float64)
    assert np.array_equal(r["res"], want)
    from cryoim_gb300 import Params
    pm = Params.from_buffer_copy(p)
    pm.use_imgmask = 0
    qq = parts.copy()
    qq["pr"] = 0.0
    _, acc = orc.reconstruct(pm, imgs, qq, want_acc=True, fp="f64")
    for k, a in zip(("fa", "fb", "wg"), acc):
        assert np.allclose(r[k], a, rtol=1e-10, atol=1e-12 * np.abs(a).max())
    # the tnf partials summed over the ranks = the partial of all particles, and so is
    # the merged map
    whole = [a + b for a, b in zip(orc.reconstruct_half(pm, imgs, qq, 0), orc.reconstruct_half(pm, imgs, qq, 1))]
    for k, a in zip(("tfa", "tfb", "twg"), whole):
        assert np.allclose(r[k], a, rtol=1e-5, atol=1e-6 * np.abs(a).max())
    m_ranks = orc.merge_finish(p.fftsize, p.max_r, [r["tfa"], r["tfb"], r["twg"]])
    m_one = orc.merge_finish(p.fftsize, p.max_r, whole)
    assert np.linalg.norm(m_ranks - m_one) <= 1e-5 * np.linalg.norm(m_one)
