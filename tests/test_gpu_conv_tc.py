"""The learned proposer's 3x3 convolutions (circular in the 128 angles, zero-padded in
radius) through the C-ABI test hook cryoim_conv3_check: the tcgen05 TF32 kernels
(conv_tc.cu) against an FP64 numpy restatement on operands rounded to TF32 the way the
kernels round them (to nearest, ties away from zero), and the FP32 CUDA-core kernels
(learn.cu) against the same restatement on unrounded operands.  Shapes cover every layer
of the network (1 -> 16, 16 -> 32, 32 -> 32 channels; the data gradient 32 -> 16), single-
and multi-row blocks, and blocks whose rows cross from one sample to the next."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tf32(a):
    u = np.ascontiguousarray(a, np.float32).view(np.uint32)
    return ((u + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def shifted(x):
    """xs[dh][dt][..., h, t] = x[..., h + dh - 1, t + dt - 1] (zero outside h, circular in t)."""
    H = x.shape[2]
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (0, 0)))
    return [[np.roll(xp[:, :, dh:dh + H, :], -(dt - 1), axis=3) for dt in range(3)] for dh in range(3)]


def conv_ref(x, W, bias, relu):
    x, W = x.astype(np.float64), W.astype(np.float64)
    xs = shifted(x)
    out = np.zeros((x.shape[0], W.shape[0], x.shape[2], x.shape[3]))
    for dh in range(3):
        for dt in range(3):
            out += np.einsum("oc,bcht->boht", W[:, :, dh, dt], xs[dh][dt])
    if bias is not None:
        out += bias[None, :, None, None]
    return np.maximum(out, 0.0) if relu else out


def wgrad_ref(x, g):
    xs = shifted(x.astype(np.float64))
    g = g.astype(np.float64)
    dW = np.zeros((g.shape[1], x.shape[1], 3, 3))
    for dh in range(3):
        for dt in range(3):
            dW[:, :, dh, dt] = np.einsum("boht,bcht->oc", g, xs[dh][dt])
    return dW


CASES = [  # B, Cin, Cout, H
    (3, 1, 16, 64),
    (2, 16, 32, 64),
    (3, 32, 32, 32),
    (2, 32, 32, 16),
    (2, 32, 16, 64),
    (20, 32, 32, 32),   # several rows per block, blocks crossing samples
    (9, 16, 32, 64),
]


@pytest.mark.parametrize("B,Cin,Cout,H", CASES)
@pytest.mark.parametrize("tensor_cores", [True, False])
def test_conv3_forward_and_weight_gradient(built, B, Cin, Cout, H, tensor_cores):
    import cryoim_gb300 as ci
    rng = np.random.default_rng(B * 1000 + Cin * 10 + Cout + H)
    x = rng.normal(size=(B, Cin, H, 128)).astype(np.float32)
    W = (rng.normal(size=(Cout, Cin, 3, 3)) / np.sqrt(9 * Cin)).astype(np.float32)
    bias = rng.normal(0, 0.1, Cout).astype(np.float32)
    g = rng.normal(size=(B, Cout, H, 128)).astype(np.float32)
    relu = Cin != 32 or Cout != 16
    out, dW, db = ci.conv3_check(x, W, bias, relu=relu, dpre=g, tensor_cores=tensor_cores)
    xr, Wr, gr = (tf32(x), tf32(W), tf32(g)) if tensor_cores else (x, W, g)
    ref = conv_ref(xr, Wr, bias.astype(np.float64), relu)
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 3e-6, err
    dref = wgrad_ref(xr, gr)
    derr = np.abs(dW - dref).max() / np.abs(dref).max()
    assert derr < 3e-5, derr
    bref = g.astype(np.float64).sum(axis=(0, 2, 3))
    assert np.abs(db - bref).max() <= 3e-5 * np.abs(bref).max() + 1e-3


def test_tf32_rounding_is_what_the_kernel_does(built):
    """Operands exactly halfway between two TF32 values round away from zero: the
    restatement above holds only if the kernel rounds as cvt.rna does."""
    import cryoim_gb300 as ci
    B, Cin, Cout, H = 1, 1, 16, 8
    one_half_ulp = np.float32(1.0 + 2.0 ** -11)  # halfway between 1 and 1 + 2^-10
    x = np.zeros((B, Cin, H, 128), np.float32)
    x[0, 0, 3, 5] = one_half_ulp
    x[0, 0, 4, 9] = -one_half_ulp
    W = np.zeros((Cout, Cin, 3, 3), np.float32)
    W[:, 0, 1, 1] = 1.0
    out, _, _ = ci.conv3_check(x, W, tensor_cores=True)
    assert out[0, 0, 3, 5] == np.float32(1.0 + 2.0 ** -10)
    assert out[0, 0, 4, 9] == -np.float32(1.0 + 2.0 ** -10)
