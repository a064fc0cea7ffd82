"""The learned orientation proposer (cryoim_learn_*): its CUDA forward and backward pass
against a plain PyTorch FP32 restatement of the same network (same weights, features
and targets), its input features against a numpy restatement on the oracle's particle
transform, and a trained proposer whose proposals lead the contraction to the same
pick as the exhaustive form."""
import math

import numpy as np
import pytest

from _data import small_case

pytestmark = pytest.mark.gpu

NR, NT, CM, MIXK = 64, 128, 16, 256
CONV = [(1, 16), (16, 32), (32, 32), (32, 32)]


def tf32_round(t):
    """FP32 -> TF32 (10 mantissa bits), to nearest with ties away from zero, as
    cvt.rna.tf32.f32 rounds the tensor-core convolutions' operands."""
    import torch
    u = t.detach().to(torch.float32).contiguous().view(torch.int32)
    return ((u + 0x1000) & -8192).view(torch.float32)


def conv_tf32_function():
    """A 3x3 convolution (circular in angle, zero-padded in radius) whose operands are
    rounded to TF32 and whose products are summed in FP64, forward and backward, as
    conv_tc.cu computes it: the data gradient from the rounded output gradient and
    weights, the weight gradient from the rounded output gradient and inputs, the bias
    gradient from the unrounded output gradient."""
    import torch
    F = torch.nn.functional

    def pad(a):
        return F.pad(F.pad(a, (1, 1, 0, 0), mode="circular"), (0, 0, 1, 1))

    class ConvTF32(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, W, b):
            xr, Wr = tf32_round(x).double(), tf32_round(W).double()
            ctx.save_for_backward(xr, Wr)
            return (F.conv2d(pad(xr), Wr) + b.double()[None, :, None, None]).float()

        @staticmethod
        def backward(ctx, gy):
            xr, Wr = ctx.saved_tensors
            gr = tf32_round(gy).double()
            dx = F.conv2d(pad(gr), Wr.flip(2, 3).transpose(0, 1))
            xp = pad(xr)
            H, T = xr.shape[2], xr.shape[3]
            dW = torch.zeros_like(Wr)
            for dh in range(3):
                for dt in range(3):
                    dW[:, :, dh, dt] = torch.einsum("boht,bcht->oc", gr, xp[:, :, dh:dh + H, dt:dt + T])
            return dx.float(), dW.float(), gy.double().sum((0, 2, 3)).float()

    return ConvTF32.apply


def torch_reference(w, feat, truth, views, sv, tf32=False):
    """The network of learn.cu in torch FP32 (CPU): scores, per-particle loss and the
    gradients of the mean loss, flattened in the library's parameter order.  tf32: the
    convolutions as the tensor-core kernels compute them (conv_tf32_function)."""
    torch = pytest.importorskip("torch")
    F = torch.nn.functional
    conv_tf32 = conv_tf32_function() if tf32 else None
    wt = torch.tensor(w, dtype=torch.float32, requires_grad=True)
    x = torch.tensor(feat, dtype=torch.float32)[:, None]
    B = x.shape[0]
    off = 0

    def take(n):
        nonlocal off
        t = wt[off:off + n]
        off += n
        return t

    for layer, (ci, co) in enumerate(CONV):
        W = take(co * ci * 9).reshape(co, ci, 3, 3)
        b = take(co)
        if tf32:
            x = F.relu(conv_tf32(x, W, b))
        else:
            x = F.pad(x, (1, 1, 0, 0), mode="circular")
            x = F.pad(x, (0, 0, 1, 1))
            x = F.relu(F.conv2d(x, W, b))
        if layer >= 1:
            x = F.avg_pool2d(x, (2, 1))
    W5 = take(CM * MIXK).reshape(CM, MIXK)
    b5 = take(CM)
    g = torch.einsum("ok,bkt->bot", W5, x.reshape(B, MIXK, NT)) + b5[None, :, None]
    V = len(views)
    T = take(V * CM * NT).reshape(V, CM, NT)
    idx = (torch.arange(NT)[:, None] + torch.arange(NT)[None, :]) % NT  # [s, t] -> (t + s) % NT
    sc = torch.einsum("bcst,vct->bvs", g[:, :, idx], T)
    d2r = math.pi / 180.0
    th, ph = torch.tensor(views[:, 0] * d2r), torch.tensor(views[:, 1] * d2r)
    vv = torch.stack([torch.sin(th) * torch.cos(ph), torch.sin(th) * torch.sin(ph), torch.cos(th)], 1).float()
    tr = torch.tensor(truth, dtype=torch.float32)
    dot = torch.clamp(tr[:, None, :3] @ vv.T[None], -1, 1)[:, 0]  # [B, V]
    av = torch.rad2deg(torch.acos(dot)) / sv
    s = torch.arange(NT)[None]
    ds = (s - tr[:, 3:4].long()).abs() % NT
    ds = torch.minimum(ds, NT - ds).float()
    tgt = torch.exp(-av[:, :, None] ** 2 - ds[:, None, :] ** 2)
    tgt = tgt / tgt.sum(dim=(1, 2), keepdim=True)
    logp = F.log_softmax(sc.reshape(B, -1), dim=1).reshape(sc.shape)
    loss = -(tgt * logp).sum(dim=(1, 2))
    loss.mean().backward()
    return sc.detach().numpy(), loss.detach().numpy(), wt.grad.numpy()


@pytest.fixture(scope="module")
def lctx(built):
    import cryoim_gb300 as ci
    p, *_ = small_case()
    with ci.Context(0, p) as ctx:
        yield ctx, p


def random_weights(n, V, rng):
    w = np.zeros(n, np.float32)
    off = 0
    for ci, co in CONV:
        w[off:off + co * ci * 9] = rng.normal(0, math.sqrt(2.0 / (9 * ci)), co * ci * 9)
        off += co * ci * 9
        w[off:off + co] = rng.normal(0, 0.05, co)
        off += co
    w[off:off + CM * MIXK] = rng.normal(0, 1 / math.sqrt(MIXK), CM * MIXK)
    off += CM * MIXK
    w[off:off + CM] = rng.normal(0, 0.05, CM)
    off += CM
    assert n - off == V * CM * NT
    w[off:] = rng.normal(0, 0.05, n - off)
    return w


@pytest.mark.parametrize("tensor_cores", [False, True])
def test_forward_backward_match_torch(lctx, tensor_cores):
    """FP32 convolutions against the FP32 restatement; tensor-core convolutions against
    the restatement whose convolutions round their operands to TF32 the same way."""
    ctx, p = lctx
    ctx.learn_set_conv(tensor_cores)
    rng = np.random.default_rng(5)
    views = ctx.learn_views()
    V = len(views)
    n = ctx.learn_params().size
    w = random_weights(n, V, rng)
    ctx.learn_params(w)
    B = 6
    feat = rng.normal(size=(B, NR, NT)).astype(np.float32)
    d2r = math.pi / 180.0
    truth = np.zeros((B, 4), np.float32)
    for b in range(B):
        th, ph = views[rng.integers(V)] + rng.normal(0, 1.0, 2)
        truth[b, :3] = [math.sin(th * d2r) * math.cos(ph * d2r), math.sin(th * d2r) * math.sin(ph * d2r),
                        math.cos(th * d2r)]
        truth[b, 3] = rng.integers(NT)
    sc, loss, gr = ctx.learn_forward(feat, truth, views=V)
    rsc, rloss, rgr = torch_reference(w, feat, truth, views.astype(np.float64), 2.0 * p.searchstep,
                                      tf32=tensor_cores)
    ctx.learn_set_conv(True)
    assert np.abs(sc - rsc).max() < 1e-4 * np.abs(rsc).max() + 1e-6
    assert np.allclose(loss, rloss, rtol=1e-4, atol=1e-5)
    # gradients, block by block (conv 1-4 weights and biases, mix, templates)
    sizes = []
    for ci, co in CONV:
        sizes += [co * ci * 9, co]
    sizes += [CM * MIXK, CM, V * CM * NT]
    # TF32: an activation the kernels and the restatement compute one FP32 ulp apart can
    # round to TF32 values one TF32 ulp (2^-10 relative) apart; through the backward
    # pass such flips move a gradient block by a few 1e-3 of its maximum.  The
    # convolutions' own arithmetic is pinned exactly by tests/test_gpu_conv_tc.py.
    gtol = 5e-3 if tensor_cores else 2e-3
    off = 0
    for k, sz in enumerate(sizes):
        a, b = gr[off:off + sz], rgr[off:off + sz]
        assert np.abs(a - b).max() <= gtol * np.abs(b).max() + 1e-7, (k, np.abs(a - b).max(), np.abs(b).max())
        off += sz


def features_numpy(a, b, n, r0, R):
    P = a.astype(np.float64) ** 2 + b.astype(np.float64) ** 2
    out = np.zeros((NR, NT))
    for ir in range(NR):
        r = r0 + (R - r0) * ir / (NR - 1)
        for it in range(NT):
            ang = math.pi * it / NT
            x, y = r * math.cos(ang) + n // 2, r * math.sin(ang) + n // 2
            lx, ly = math.floor(x), math.floor(y)
            ax, ay = x - lx, y - ly
            out[ir, it] = ((1 - ay) * ((1 - ax) * P[ly, lx] + ax * P[ly, lx + 1]) +
                           ay * ((1 - ax) * P[ly + 1, lx] + ax * P[ly + 1, lx + 1]))
    out = np.log(out + 1e-6 * out.mean())
    out = (out - out.mean(axis=1, keepdims=True)) / (out.std(axis=1, keepdims=True) + 1e-6)
    return out


def test_features_match_numpy(lctx, orc):
    ctx, p = lctx
    _, vol, tmpl, timgs, imgs, parts, truth = small_case()
    got = ctx.learn_features(imgs, parts)
    for i in range(len(parts)):
        a, b, _ = orc.prep_particle(imgs[i], 1, p.imgmask_px, parts["x"][i], parts["y"][i], 0,
                                    p.min_r, p.max_r, "f64")
        want = features_numpy(a, b, p.fftsize, p.min_r, p.max_r)
        d = np.abs(got[i] - want)
        assert np.median(d) < 1e-3 and np.quantile(d, 0.999) < 2e-2, (i, np.median(d), d.max())


def test_trained_proposer_leads_to_the_exhaustive_pick(built, tmp_path):
    """Trained on library-rendered projections of the map (noisy, CTF, shifted), the
    proposer's 16 cells per particle, expanded to their +-2-step neighbourhoods, contain
    the exhaustive contraction's pick on noise-free particles; a saved and reloaded
    proposer proposes the same."""
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(P=8)
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        st = ctx.learn_train(vol, samples=24576, batch=128, seed=3, snr=1.0, df_min=1.0, df_max=3.0,
                             origin_max=2.0)
        assert st["views"] == len(ctx.learn_views()) and st["sign"] in (1, -1)
        assert np.isfinite(st["loss"])
        qe = parts.copy()
        ctx.contract_search(imgs, qe, origin_max=2.0, origin_step=0.5, topk=8)
        ql = parts.copy()
        cl = ctx.contract_search(imgs, ql, origin_max=2.0, origin_step=0.5, topk=8, learned=16, want_cands=True)
        path = str(tmp_path / "proposer.bin")
        ctx.learn_save(path)
    for i in range(len(parts)):
        assert (ql["theta"][i], ql["phi"][i], ql["omega"][i]) == (qe["theta"][i], qe["phi"][i], qe["omega"][i]), i
    with ci.Context(0, p) as c2:
        c2.load_templates(timgs, tmpl)
        c2.set_reference_map(vol)
        c2.learn_load(path)
        q2 = parts.copy()
        c2b = c2.contract_search(imgs, q2, origin_max=2.0, origin_step=0.5, topk=8, learned=16, want_cands=True)
        # one particle per pass, dealt to 3 lanes: each lane runs the borrowed proposer
        c2.set_batch(1)
        c2.set_lanes(3)
        q3 = parts.copy()
        c3 = c2.contract_search(imgs, q3, origin_max=2.0, origin_step=0.5, topk=8, learned=16, want_cands=True)
    assert np.array_equal(q2, ql)
    assert np.array_equal(c2b, cl)
    assert np.array_equal(q3, ql)
    assert np.array_equal(c3, cl)


def test_learned_form_needs_a_trained_proposer(built):
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = small_case()
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        with pytest.raises(ci.CryoimError):
            ctx.contract_search(imgs, parts.copy(), learned=8)
        with pytest.raises(ci.CryoimError):
            ctx.contract_search(imgs, parts.copy(), learned=8, coarse=8)


def test_render_matches_real_space_projection(built):
    """The training renderer (Fourier slice of the twice-padded map's transform, CTF,
    origin shift) against the numpy real-space projector with the same CTF and shift,
    over |h| <= maxR."""
    import cryoim_gb300 as ci
    import synth
    p, vol, *_ = small_case()
    n, R = p.fftsize, p.max_r
    rng = np.random.default_rng(9)
    e = synth.random_rotations(4, rng)
    par = np.zeros((4, 5), np.float32)
    par[:, 0] = rng.uniform(1.0, 3.0, 4)
    par[:, 1] = par[:, 0] + 0.05
    par[:, 2] = 30.0
    par[:, 3:] = rng.uniform(-2, 2, (4, 2))
    with ci.Context(0, p) as ctx:
        got = ctx.learn_render(vol, e, par)
    ky, hx = np.meshgrid(np.arange(n) - n // 2, np.arange(n) - n // 2, indexing="ij")
    disc = hx ** 2 + ky ** 2 <= R * R
    for i in range(4):
        proj = synth.project_numpy(vol, e[i:i + 1].astype(np.float32))[0]
        c = synth.ctf2d(n, par[i, 0], par[i, 1], par[i, 2], p.apix, p.vol, p.cs, p.ampwg)
        want = synth.apply_ctf_shift(proj.astype(np.float64), c, par[i, 3], par[i, 4])
        fa = np.fft.fftshift(np.fft.fft2(got[i]))[disc]
        fb = np.fft.fftshift(np.fft.fft2(want))[disc]
        cc = np.real(np.vdot(fa, fb)) / np.sqrt(np.vdot(fa, fa).real * np.vdot(fb, fb).real)
        ratio = np.linalg.norm(fa) / np.linalg.norm(fb)
        assert cc > 0.99 and 0.95 < ratio < 1.05, (i, cc, ratio)


def test_learned_form_fallback_to_the_exhaustive_contraction(built):
    """cryoim_contract_opts.fallback: particles whose phase residual lies more than t
    robust standard deviations above the call's median are searched again by the
    exhaustive contraction and keep the lower phase residual.  t = 1e9 sends none and
    changes nothing; t = 1e-6 sends every particle above the median, each of which ends
    with min(learned, exhaustive) phase residual and that form's pick."""
    import cryoim_gb300 as ci
    p, vol, tmpl, timgs, imgs, parts, truth = small_case(P=8, snr=0.5)
    kw = dict(origin_max=2.0, origin_step=0.5, topk=8)
    with ci.Context(0, p) as ctx:
        ctx.load_templates(timgs, tmpl)
        ctx.set_reference_map(vol)
        ctx.learn_train(vol, samples=8192, batch=128, seed=3, snr=0.5, df_min=1.0, df_max=3.0, origin_max=2.0)
        ql = parts.copy()
        ctx.contract_search(imgs, ql, learned=16, **kw)
        assert ctx.contract_fallbacks() == 0
        qe = parts.copy()
        ctx.contract_search(imgs, qe, **kw)
        qn = parts.copy()
        ctx.contract_search(imgs, qn, learned=16, fallback=1e9, **kw)
        assert ctx.contract_fallbacks() == 0
        assert np.array_equal(qn, ql)
        qf = parts.copy()
        ctx.contract_search(imgs, qf, learned=16, fallback=1e-6, **kw)
        nf = ctx.contract_fallbacks()
        with pytest.raises(ci.CryoimError):
            ctx.contract_search(imgs, parts.copy(), fallback=1.0, **kw)  # not the learned form
    sent = ql["pr"] > np.sort(ql["pr"])[len(ql) // 2]  # the library's median: the upper one
    assert nf == int(sent.sum()) and nf >= 1
    assert np.array_equal(qf[~sent], ql[~sent])
    for i in np.nonzero(sent)[0]:
        want = qe[i] if qe["pr"][i] < ql["pr"][i] else ql[i]
        assert qf[i] == want, i
