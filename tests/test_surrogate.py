"""The learned WFF2 surrogate: the FP64 oracle (CPU) and the CUDA network
(tensor-core convolutions, forward, backward) against it (GPU).

Tolerances: the GPU stores activations and activation gradients in BF16 and
sums in FP32; the oracle emulates the BF16 rounding and sums in FP64, so
elementwise results agree except where an FP32-vs-FP64 difference moves a
value across a BF16 rounding boundary (one BF16 ulp, 2^-8 relative).
"""
import numpy as np
import pytest

from oracle import surrogate as S

DIL = [1, 2, 4, 8, 16, 8, 4, 1]


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125 + 2 ** -9, -3.14159, 0.0, 65504.0], np.float32)
    r = S.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                    # exactly halfway between 1 and 1+2^-7: ties to even (1.0)
    assert r[2] == 1.0078125              # above halfway rounds up
    assert r[3] == 1.0078125              # below the next halfway rounds down
    assert abs(r[4] - (-3.140625)) < 1e-12
    assert r[5] == 0.0


@pytest.mark.parametrize("wscale", [1.0, 10.0])
def test_oracle_gradient_matches_finite_differences(wscale):
    rng = np.random.default_rng(0)
    p = S.init_params(1, scale_last=1.0).astype(np.float64)
    z = np.exp(1j * rng.uniform(-np.pi, np.pi, (1, 9, 11)))
    # target magnitudes on both sides of 1 / wscale
    t = rng.uniform(0.02, 1.2, (1, 9, 11)) * np.exp(1j * rng.uniform(-np.pi, np.pi, (1, 9, 11)))
    dil = [1, 2, 1, 3, 1, 2, 1, 1]
    loss, g = S.loss_and_grad(p, z, t, dil, bf16_emul=False, wscale=wscale)
    idx = rng.choice(p.size, 40, replace=False)
    # include every layer's bias and one weight of each layer
    offs = np.cumsum([0] + [co * ci * 9 + co for co, ci in S.SIZES])
    idx = np.concatenate([idx, offs[1:] - 1, offs[:-1]])
    eps = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        lp, _ = S.loss_and_grad(pp, z, t, dil, bf16_emul=False, wscale=wscale)
        lm, _ = S.loss_and_grad(pm, z, t, dil, bf16_emul=False, wscale=wscale)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-9, (k, fd, g[k])


def test_oracle_conv_matches_direct_sum():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2, 7, 9, 3))
    w = rng.standard_normal((4, 3, 3, 3))
    b = rng.standard_normal(4)
    d = 2
    out = S.conv(x, w, b, d)
    ref = np.zeros_like(out)
    for bi in range(2):
        for y in range(7):
            for xx in range(9):
                acc = b.copy()
                for ky in range(3):
                    for kx in range(3):
                        yy, xs = y + (ky - 1) * d, xx + (kx - 1) * d
                        if 0 <= yy < 7 and 0 <= xs < 9:
                            acc += w[:, :, ky, kx] @ x[bi, yy, xs]
                ref[bi, y, xx] = acc
    assert np.allclose(out, ref, atol=1e-12)


# ---------------------------------------------------------------------------
def _torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def _bf16_bits(a):
    f = np.ascontiguousarray(S.bf16(a), np.float64).astype(np.float32)
    return (f.view(np.uint32) >> 16).astype(np.uint16)


def _from_bits(u):
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,dil,relu,mask", [((1, 37, 150), 1, True, False), ((2, 40, 128), 3, True, True),
                                                 ((1, 70, 300), 16, False, False), ((3, 19, 64), 8, True, False),
                                                 ((1, 5, 7), 2, True, True)])
def test_tensor_core_conv_matches_oracle(glsu, shape, dil, relu, mask):
    """One 32 -> 32 layer: tcgen05 MMAs over TMA-loaded rows (ragged widths,
    dilations up to 16, batches, masks) against the FP64 oracle."""
    torch = _torch()
    rng = np.random.default_rng(dil * 100 + shape[1])
    B, H, W = shape
    x = rng.standard_normal((B, H, W, 32)).astype(np.float32)
    w = (rng.standard_normal((32, 32, 3, 3)) * 0.1).astype(np.float32)
    b = (rng.standard_normal(32) * 0.1).astype(np.float32)
    xb = _bf16_bits(x)
    xin = torch.from_numpy(xb.view(np.int16)).cuda()
    out = torch.zeros_like(xin)
    mb = None
    m_arr = None
    if mask:
        m_arr = np.where(rng.random((B, H, W, 32)) < 0.5, 1.0, 0.0).astype(np.float32)
        mb = torch.from_numpy(_bf16_bits(m_arr).view(np.int16)).cuda()
    glsu.conv32(xin.data_ptr(), out.data_ptr(), B, W, H, dil, w, b, relu, mb.data_ptr() if mask else 0)
    got = _from_bits(out.cpu().numpy().view(np.uint16))
    ref = S.conv(_from_bits(xb), S.bf16(w), b.astype(np.float64), dil)
    if relu:
        ref = np.maximum(ref, 0)
    if mask:
        ref = ref * (m_arr > 0)
    refb = S.bf16(ref)
    diff = np.abs(got - refb)
    ulp = np.maximum(np.abs(refb), 1e-30) * 2.0 ** -7
    bad = diff > ulp + 1e-6
    print("conv32 %s d=%d: max |diff| %.3g, elements off by more than one BF16 ulp: %d, exact %.4f"
          % (shape, dil, diff.max(), bad.sum(), (diff == 0).mean()))
    assert not bad.any()
    assert (diff == 0).mean() > 0.99


@pytest.mark.gpu
@pytest.mark.parametrize("shape,dil", [((1, 5, 40), 1), ((2, 36, 136), 16), ((1, 70, 300), 3), ((3, 17, 129), 24),
                                       ((1, 64, 128), 64), ((2, 33, 257), 2)])
def test_tensor_core_weight_gradient_matches_fp64(glsu, shape, dil):
    """Weight and bias gradient of one 32 -> 32 layer: tcgen05 MMAs with
    MN-major operands (rows of the gradient and the activation by TMA) and
    the CUDA-core bias sums, against FP64 sums of the same BF16 values
    (ragged widths, widths below one 128-pixel segment, dilations up to 64,
    rows beyond the image)."""
    torch = _torch()
    rng = np.random.default_rng(dil * 10 + shape[2])
    B, H, W = shape
    gb = _bf16_bits(rng.uniform(-1, 1, (B, H, W, 32)).astype(np.float32))
    ab = _bf16_bits(rng.uniform(-1, 1, (B, H, W, 32)).astype(np.float32))
    dg = torch.from_numpy(gb.view(np.int16)).cuda()
    da = torch.from_numpy(ab.view(np.int16)).cuda()
    dw, db = glsu.wgrad32(dg.data_ptr(), da.data_ptr(), B, W, H, dil)
    g, a = _from_bits(gb), _from_bits(ab)
    ap = np.zeros((B, H + 2 * dil, W + 2 * dil, 32))
    ap[:, dil:dil + H, dil:dil + W] = a
    ref = np.zeros((32, 32, 3, 3))
    for ky in range(3):
        for kx in range(3):
            sh = ap[:, ky * dil:ky * dil + H, kx * dil:kx * dil + W]
            ref[:, :, ky, kx] = np.einsum("bhwo,bhwi->oi", g, sh)
    rdb = g.sum((0, 1, 2))
    e = np.abs(dw - ref).max() / np.abs(ref).max()
    eb = np.abs(db - rdb).max() / np.abs(rdb).max()
    print("wgrad32 %s d=%d: max |dW - ref| / max |ref| %.3g, bias %.3g" % (shape, dil, e, eb))
    assert e < 1e-5 and eb < 1e-5


def _net_case(glsu, B, H, W, seed):
    torch = _torch()
    rng = np.random.default_rng(seed)
    p = S.init_params(seed, scale_last=1.0)
    phase = rng.uniform(-np.pi, np.pi, (B, H, W))
    z = np.exp(1j * phase).astype(np.complex64)
    t = (rng.uniform(0.2, 1.2, (B, H, W)) * np.exp(1j * (phase + rng.normal(0, 0.3, (B, H, W))))).astype(np.complex64)
    return torch, p, z, t


@pytest.mark.gpu
@pytest.mark.parametrize("wscale", [1.0, 10.0])
def test_network_forward_and_gradients_match_oracle(glsu, wscale):
    """Every parameter gradient of the CUDA training pass (tensor-core
    forward, backward-data with the flipped weights, tensor-core weight
    gradients of the hidden layers) against the oracle with the same BF16
    rounding points, for two loss weightings."""
    B, H, W = 2, 36, 136
    torch, p, z, t = _net_case(glsu, B, H, W, 7)
    net = glsu.Surrogate(B, W, H, DIL, training=True)
    net.params = p
    if wscale != 1.0:
        net.set_loss_scale(wscale)
    dz, dt = torch.from_numpy(z).cuda(), torch.from_numpy(t).cuda()
    loss, g = net.backward(dz.data_ptr(), dt.data_ptr(), want_grad=True)
    out = net.output()
    rout, cache = S.forward(p, z.astype(np.complex128), DIL)
    rloss, rg = S.loss_and_grad(p, z.astype(np.complex128), t.astype(np.complex128), DIL, wscale=wscale)
    d = np.abs(out - rout)
    # out = y/|y|: where |y| is small a one-ulp BF16 difference upstream turns the direction
    firm = cache["n"][..., 0] >= 0.05
    print("network: loss %.6f vs %.6f, |out diff| rms %.3g, max %.3g (|y| >= 0.05: %.3g)"
          % (loss, rloss, np.sqrt(np.mean(d ** 2)), d.max(), d[firm].max()))
    assert abs(loss - rloss) <= 2e-3 * rloss
    assert np.sqrt(np.mean(d ** 2)) < 2e-3 and d[firm].max() < 2e-2
    offs = np.cumsum([0] + [co * ci * 9 + co for co, ci in S.SIZES])
    for l in range(8):
        a, b = g[offs[l]:offs[l + 1]].astype(np.float64), rg[offs[l]:offs[l + 1]]
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        print("layer %d: |grad| %.4g, relative error %.3g, cosine %.6f" % (l, np.linalg.norm(b), rel, cos))
        assert rel < 2e-2 and cos > 0.9995
    net.close()


@pytest.mark.gpu
def test_inference_forward_equals_training_forward(glsu):
    B, H, W = 1, 50, 130
    torch, p, z, t = _net_case(glsu, B, H, W, 3)
    tr = glsu.Surrogate(B, W, H, DIL, training=True)
    tr.params = p
    dz, dt = torch.from_numpy(z).cuda(), torch.from_numpy(t).cuda()
    tr.backward(dz.data_ptr(), dt.data_ptr())
    a = tr.output()
    inf = glsu.Surrogate(B, W, H, DIL)
    inf.params = p
    o = torch.empty_like(dz)
    inf.forward(dz.data_ptr(), o.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(o.cpu().numpy(), a)
    assert np.allclose(np.abs(a), 1, atol=1e-5)
    tr.close()
    inf.close()


@pytest.mark.gpu
def test_adam_step_decreases_loss(glsu):
    B, H, W = 2, 32, 128
    torch, p, z, t = _net_case(glsu, B, H, W, 5)
    net = glsu.Surrogate(B, W, H, DIL, training=True)
    net.params = p
    dz, dt = torch.from_numpy(z).cuda(), torch.from_numpy(t).cuda()
    l0, _ = net.backward(dz.data_ptr(), dt.data_ptr())
    for _ in range(20):
        net.adam(1e-3)
        l1, _ = net.backward(dz.data_ptr(), dt.data_ptr())
    print("adam: loss %.5f -> %.5f" % (l0, l1))
    assert l1 < 0.9 * l0
    net.close()
