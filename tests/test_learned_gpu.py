"""The warm-start CNN kernels and network against the float64 CPU reference (torch autograd).

Layer checks use inputs that are exact BF16 values, so the kernels' only error is FP32
accumulation: forward, input gradient (convolution with flipped weights), weight and bias
gradients, pooling, upsampling, loss and Adam. The network check runs the whole forward and
backward against autograd with BF16 rounding at the same storage points."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from cnn_reference import LAYERS, bf16_round, conv3, forward, from_c8, pool2, to_c8, unpack, up2

pytestmark = pytest.mark.gpu


def _lib():
    from iane_gb300._lib import lib

    return lib()


def _check(rc):
    from iane_gb300._lib import check

    check(rc)


def _bf16_tensor(gen, shape, scale=1.0, device="cuda"):
    """(float64 reference, BF16 device copy) of N(0, scale^2) values rounded to BF16."""
    import torch

    t = torch.randn(shape, generator=gen, dtype=torch.float64) * scale
    return bf16_round(t), t.to(torch.bfloat16).to(device)


def _act(gen, shape, scale=1.0, device="cuda"):
    """An activation: float64 planar reference and its BF16 C8 device copy."""
    ref, dev = _bf16_tensor(gen, shape, scale, device)
    return ref, to_c8(dev)


def _p(t):
    return None if t is None else t.data_ptr()


def _rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("shape,c0,c1,co", [((6, 10, 12), 3, 0, 16), ((5, 9, 17), 3, 5, 20), ((4, 8, 8), 16, 0, 64),
                                             ((7, 3, 11), 2, 0, 1), ((4, 8, 16), 64, 32, 32)])
def test_conv3_forward(cuda, shape, c0, c1, co):
    import torch

    gen = torch.Generator().manual_seed(1 + c0 + co)
    x0r, x0 = _act(gen, (c0,) + shape)
    x1r, x1 = _act(gen, (max(c1, 1),) + shape)
    wr, w = _bf16_tensor(gen, (co, c0 + c1, 27), 0.2)
    b = torch.randn(co, generator=gen, dtype=torch.float32) * 0.1
    y32 = torch.empty((co,) + shape, dtype=torch.float32, device=cuda)
    y16 = to_c8(torch.zeros((co,) + shape, dtype=torch.bfloat16, device=cuda))
    mr, m = _act(gen, (co,) + shape)
    bd = b.to(cuda)
    _check(_lib().iane_gb_cnn_conv3(_p(x0), c0, _p(x1) if c1 else None, c1, *shape, _p(w), _p(bd), co,
                                    _p(y16), _p(y32), None, 1, _p(m), None))
    torch.cuda.synchronize()
    inp = torch.cat([x0r, x1r[:c1]], 0) if c1 else x0r
    ref = torch.relu(conv3(inp, wr, b.double())) * (mr > 0)
    mag = conv3(inp.abs(), wr.abs()) + b.double().abs().unsqueeze(1).unsqueeze(1).unsqueeze(1)
    got = y32.cpu().double()
    assert float(((got - ref).abs() / (mag + 1e-30)).max()) < 2e-6
    # BF16 output is the rounded FP32 value
    assert torch.equal(from_c8(y16.cpu(), co), y32.cpu().to(torch.bfloat16))


def test_conv3_residual_f32_output(cuda):
    import torch

    gen = torch.Generator().manual_seed(7)
    shape = (8, 12, 20)
    xr, x = _act(gen, (16,) + shape)
    wr, w = _bf16_tensor(gen, (1, 16, 27), 0.2)
    res = torch.randn((1,) + shape, generator=gen, dtype=torch.float32)
    b = torch.tensor([0.25], dtype=torch.float32)
    y = torch.empty((1,) + shape, dtype=torch.float32, device=cuda)
    bd, rd = b.to(cuda), res.to(cuda)  # keep the device copies alive until the kernel has run
    _check(_lib().iane_gb_cnn_conv3(_p(x), 16, None, 0, *shape, _p(w), _p(bd), 1, None, _p(y), _p(rd), 0, None,
                                    None))
    torch.cuda.synchronize()
    ref = conv3(xr, wr, b.double()) + res.double()
    mag = conv3(xr.abs(), wr.abs()) + 0.25 + res.double().abs()
    assert float(((y.cpu().double() - ref).abs() / mag).max()) < 2e-6


@pytest.mark.parametrize("shape,ci,co", [((6, 10, 12), 16, 32), ((4, 8, 8), 64, 64), ((5, 7, 9), 2, 16),
                                         ((8, 8, 8), 48, 16)])
def test_conv3_input_gradient_by_flipped_weights(cuda, shape, ci, co):
    import torch

    gen = torch.Generator().manual_seed(ci * 100 + co)
    xr = torch.randn((ci,) + shape, generator=gen, dtype=torch.float64).requires_grad_(True)
    dyr, dy = _act(gen, (co,) + shape)
    wr, w = _bf16_tensor(gen, (co, ci, 27), 0.2)
    (conv3(xr, wr) * dyr).sum().backward()
    ref = xr.grad
    flipped = torch.empty(ci * co * 27, dtype=torch.bfloat16, device=cuda)
    _check(_lib().iane_gb_cnn_flip(_p(w), co, ci, _p(flipped), None))
    dx = torch.empty((ci,) + shape, dtype=torch.float32, device=cuda)
    _check(_lib().iane_gb_cnn_conv3(_p(dy), co, None, 0, *shape, _p(flipped), None, ci, None, _p(dx), None, 0, None,
                                    None))
    torch.cuda.synchronize()
    wt = wr.transpose(0, 1).flip(2)  # [ci][co][26 - t]
    mag = conv3(dyr.abs(), wt.abs())
    assert float(((dx.cpu().double() - ref).abs() / (mag + 1e-30)).max()) < 2e-6
    assert torch.equal(flipped.cpu(), wt.to(torch.bfloat16).reshape(-1))


@pytest.mark.parametrize("shape,c0,c1,co", [((6, 10, 12), 16, 0, 16), ((5, 9, 17), 8, 5, 20), ((8, 8, 8), 32, 16, 48),
                                             ((16, 16, 16), 2, 0, 16), ((7, 3, 11), 16, 0, 1)])
def test_conv3_weight_gradient(cuda, shape, c0, c1, co):
    import torch

    gen = torch.Generator().manual_seed(3 * c0 + co)
    x0r, x0 = _act(gen, (c0,) + shape)
    x1r, x1 = _act(gen, (max(c1, 1),) + shape)
    dyr, dy = _act(gen, (co,) + shape)
    inp = torch.cat([x0r, x1r[:c1]], 0) if c1 else x0r
    wr = torch.zeros((co, c0 + c1, 27), dtype=torch.float64, requires_grad=True)
    br = torch.zeros(co, dtype=torch.float64, requires_grad=True)
    (conv3(inp, wr, br) * dyr).sum().backward()
    # accumulate onto existing values (+=)
    dw0 = torch.randn(wr.shape, generator=gen, dtype=torch.float32)
    db0 = torch.randn(co, generator=gen, dtype=torch.float32)
    dw, db = dw0.to(cuda), db0.to(cuda)
    need = _lib().iane_gb_cnn_wgrad_scratch_bytes(c0, c1, *shape, co)
    scratch = torch.empty(int(need), dtype=torch.uint8, device=cuda)
    _check(_lib().iane_gb_cnn_conv3_wgrad(_p(x0), c0, _p(x1) if c1 else None, c1, *shape, _p(dy), co, _p(dw), _p(db),
                                          _p(scratch), scratch.numel(), None))
    torch.cuda.synchronize()
    # magnitude: the same sums over absolute values
    wa = torch.zeros_like(wr, requires_grad=True)
    ba = torch.zeros_like(br, requires_grad=True)
    (conv3(inp.abs(), wa, ba) * dyr.abs()).sum().backward()
    for got, start, ref, mag in ((dw, dw0, wr.grad, wa.grad), (db, db0, br.grad, ba.grad)):
        want = start.double() + ref
        err = (got.cpu().double() - want).abs()
        assert bool((err <= 1e-5 * mag + 2 ** -22 * want.abs() + 1e-30).all()), float((err - 1e-5 * mag).max())
    # deterministic: the same call gives bit-identical results
    dw2, db2 = dw0.to(cuda), db0.to(cuda)
    _check(_lib().iane_gb_cnn_conv3_wgrad(_p(x0), c0, _p(x1) if c1 else None, c1, *shape, _p(dy), co, _p(dw2),
                                          _p(db2), _p(scratch), scratch.numel(), None))
    assert torch.equal(dw, dw2) and torch.equal(db, db2)


def test_conv3_wgrad_scratch_too_small_is_a_length_error(cuda):
    import torch

    from iane_gb300 import abi

    x = torch.zeros((1, 8, 8, 8, 8), dtype=torch.bfloat16, device=cuda)
    dy = torch.zeros((1, 8, 8, 8, 8), dtype=torch.bfloat16, device=cuda)
    dw = torch.zeros(4 * 4 * 27, dtype=torch.float32, device=cuda)
    scratch = torch.empty(16, dtype=torch.uint8, device=cuda)
    rc = _lib().iane_gb_cnn_conv3_wgrad(_p(x), 4, None, 0, 8, 8, 8, _p(dy), 4, _p(dw), None, _p(scratch), 16, None)
    assert rc == abi.LENGTH_ERROR


def test_pool_and_upsample(cuda):
    import torch

    gen = torch.Generator().manual_seed(11)
    c, shape = 5, (6, 8, 10)
    half = tuple(s // 2 for s in shape)
    xr, x = _act(gen, (c,) + shape)
    y = to_c8(torch.zeros((c,) + half, dtype=torch.bfloat16, device=cuda))
    _check(_lib().iane_gb_cnn_pool2(_p(x), c, *shape, _p(y), None))
    torch.cuda.synchronize()
    # 8 BF16 values summed in FP32 and scaled by 1/8: the FP32 sum is exact to 2^-24 relative
    assert torch.allclose(from_c8(y.cpu(), c).double(), bf16_round(pool2(xr)), rtol=2 ** -8, atol=0)

    dyr, dy = _act(gen, (c,) + half)
    mr, m = _act(gen, (c,) + shape)
    for accumulate in (0, 1):
        pr, prev = _act(gen, (c,) + shape)
        dx = prev.clone()
        _check(_lib().iane_gb_cnn_pool2_grad(_p(dy), c, *shape, _p(dx), _p(m), accumulate, None))
        torch.cuda.synchronize()
        ref = (up2(dyr) / 8 + (pr if accumulate else 0)) * (mr > 0)
        assert torch.allclose(from_c8(dx.cpu(), c).double(), bf16_round(ref), rtol=2 ** -8, atol=0)

    u = to_c8(torch.zeros((c,) + tuple(2 * s for s in shape), dtype=torch.bfloat16, device=cuda))
    _check(_lib().iane_gb_cnn_up2(_p(x), c, *shape, _p(u), None))
    torch.cuda.synchronize()
    assert torch.equal(from_c8(u.cpu(), c).double(), up2(xr))

    gr, g = _act(gen, (c,) + tuple(2 * s for s in shape))
    dx = to_c8(torch.zeros((c,) + shape, dtype=torch.bfloat16, device=cuda))
    _check(_lib().iane_gb_cnn_up2_grad(_p(g), c, *shape, _p(dx), _p(m), None))
    torch.cuda.synchronize()
    ref = (gr.reshape(c, shape[0], 2, shape[1], 2, shape[2], 2).sum((2, 4, 6))) * (mr > 0)
    assert torch.allclose(from_c8(dx.cpu(), c).double(), bf16_round(ref), rtol=2 ** -8, atol=0)


def test_mse_and_adam(cuda):
    import torch

    gen = torch.Generator().manual_seed(5)
    n = 100003
    y = torch.randn(n, generator=gen, dtype=torch.float32)
    t = torch.randn(n, generator=gen, dtype=torch.float32)
    dy = torch.zeros(8 * n, dtype=torch.bfloat16, device=cuda)  # one channel, C8
    loss = torch.full((1,), 0.5, dtype=torch.float64, device=cuda)
    yd, td = y.to(cuda), t.to(cuda)
    _check(_lib().iane_gb_cnn_mse(_p(yd), _p(td), n, _p(dy), _p(loss), None))
    torch.cuda.synchronize()
    e = (y - t).double()
    assert abs(float(loss.item()) - 0.5 - float((e * e).mean())) < 1e-12
    assert torch.equal(dy.cpu()[::8], (2.0 * (y - t) / n).to(torch.bfloat16))
    assert not bool(dy.cpu().reshape(n, 8)[:, 1:].any())

    p = torch.randn(n, generator=gen, dtype=torch.float32)
    g = torch.randn(n, generator=gen, dtype=torch.float32)
    m = torch.randn(n, generator=gen, dtype=torch.float32) * 0.1
    v = torch.rand(n, generator=gen, dtype=torch.float32) * 0.1
    dp, dp16, dm, dv = p.to(cuda), torch.empty(n, dtype=torch.bfloat16, device=cuda), m.to(cuda), v.to(cuda)
    lr, b1, b2, eps, step, scale = 1e-3, 0.9, 0.999, 1e-8, 3, 0.5
    gd_dev = g.to(cuda)
    _check(_lib().iane_gb_cnn_adam(_p(dp), _p(dp16), _p(gd_dev), _p(dm), _p(dv), n, ctypes.c_float(lr),
                                   ctypes.c_float(b1), ctypes.c_float(b2), ctypes.c_float(eps), step,
                                   ctypes.c_float(scale), None))
    torch.cuda.synchronize()
    gd = g.double() * scale
    m1 = b1 * m.double() + (1 - b1) * gd
    v1 = b2 * v.double() + (1 - b2) * gd * gd
    p1 = p.double() - lr * (m1 / (1 - b1 ** step)) / ((v1 / (1 - b2 ** step)).sqrt() + eps)
    assert float((dm.cpu().double() - m1).abs().max()) < 1e-6
    assert float((dv.cpu().double() - v1).abs().max()) < 1e-6
    assert float((dp.cpu().double() - p1).abs().max()) < 1e-6
    assert torch.equal(dp16.cpu(), dp.cpu().to(torch.bfloat16))


@pytest.mark.parametrize("shape,c0,c1,co", [((6, 10, 12), 16, 0, 16), ((5, 9, 30), 2, 0, 16), ((4, 8, 16), 64, 32, 32),
                                             ((3, 5, 7), 32, 0, 64), ((8, 12, 29), 32, 16, 16), ((9, 17, 15), 16, 0, 32)])
def test_conv3_tensor_core_forward(cuda, shape, c0, c1, co):
    """tcgen05 forward against float64 (BF16 products are exact in FP32; the error is the
    FP32 accumulation) and against the SIMT kernel."""
    import torch

    gen = torch.Generator().manual_seed(17 + c0 + co + shape[2])
    x0r, x0 = _act(gen, (c0,) + shape)
    x1r, x1 = _act(gen, (max(c1, 1),) + shape)
    wr, w = _bf16_tensor(gen, (co, c0 + c1, 27), 0.2)
    b = (torch.randn(co, generator=gen, dtype=torch.float32) * 0.1).to(cuda)
    packed = torch.empty(int(_lib().iane_gb_cnn_tc_packed_bytes(co, c0, c1)) // 2, dtype=torch.bfloat16, device=cuda)
    _check(_lib().iane_gb_cnn_tc_pack(_p(w), co, c0, c1, _p(packed), None))
    y16 = to_c8(torch.zeros((co,) + shape, dtype=torch.bfloat16, device=cuda))
    y32 = torch.zeros((co,) + shape, dtype=torch.float32, device=cuda)
    _check(_lib().iane_gb_cnn_conv3_tc(_p(x0), c0, _p(x1) if c1 else None, c1, *shape, _p(packed), _p(b), co,
                                       _p(y16), _p(y32), None, 1, None))
    s16 = to_c8(torch.zeros((co,) + shape, dtype=torch.bfloat16, device=cuda))
    s32 = torch.zeros((co,) + shape, dtype=torch.float32, device=cuda)
    _check(_lib().iane_gb_cnn_conv3(_p(x0), c0, _p(x1) if c1 else None, c1, *shape, _p(w), _p(b), co, _p(s16),
                                    _p(s32), None, 1, None, None))
    torch.cuda.synchronize()
    from iane_gb300 import device_status

    device_status()
    inp = torch.cat([x0r, x1r[:c1]], 0) if c1 else x0r
    ref = torch.relu(conv3(inp, wr, b.cpu().double()))
    mag = conv3(inp.abs(), wr.abs()) + b.cpu().double().abs().reshape(-1, 1, 1, 1)
    got = y32.cpu().double()
    assert float(((got - ref).abs() / mag).max()) < 1e-5
    assert float(((got - s32.cpu().double()).abs() / mag).max()) < 1e-5
    assert torch.equal(from_c8(y16.cpu(), co), y32.cpu().to(torch.bfloat16))


def test_conv3_tensor_core_head_with_residual(cuda):
    import torch

    gen = torch.Generator().manual_seed(23)
    shape = (7, 13, 33)
    xr, x = _act(gen, (16,) + shape)
    wr, w = _bf16_tensor(gen, (1, 16, 27), 0.2)
    res = torch.randn((1,) + shape, generator=gen, dtype=torch.float32).to(cuda)
    b = torch.tensor([0.25], dtype=torch.float32, device=cuda)
    packed = torch.empty(int(_lib().iane_gb_cnn_tc_packed_bytes(1, 16, 0)) // 2, dtype=torch.bfloat16, device=cuda)
    _check(_lib().iane_gb_cnn_tc_pack(_p(w), 1, 16, 0, _p(packed), None))
    y = torch.zeros((1,) + shape, dtype=torch.float32, device=cuda)
    _check(_lib().iane_gb_cnn_conv3_tc(_p(x), 16, None, 0, *shape, _p(packed), _p(b), 1, None, _p(y), _p(res), 0,
                                       None))
    torch.cuda.synchronize()
    ref = conv3(xr, wr, b.cpu().double()) + res.cpu().double()
    mag = conv3(xr.abs(), wr.abs()) + 0.25 + res.cpu().double().abs()
    assert float(((y.cpu().double() - ref).abs() / mag).max()) < 1e-5


def test_network_tensor_core_forward_matches_simt(cuda):
    import torch

    from iane_gb300.learned import WarmStartNet

    net = WarmStartNet(cuda, seed=6)
    gen = torch.Generator().manual_seed(4)
    w0, b0 = net.offsets["head"]
    net.master[w0:b0] = (torch.randn(b0 - w0, generator=gen) * 0.3).to(cuda)
    net.p16.copy_(net.master.to(torch.bfloat16))
    obs = (torch.rand((16, 36, 44), generator=gen, dtype=torch.float32) * 2.0).to(cuda)
    a = net.forward(obs, 1.5).clone()
    b = net.forward(obs, 1.5, tensor_cores=True).clone()
    torch.cuda.synchronize()
    # the paths sum in different FP32 orders (each layer agrees to 1e-5 of its magnitude, see
    # above), which flips the BF16 rounding (2^-8 relative) of some stored activations; over
    # eleven layers that leaves a few 1e-3 of difference in the output
    assert _rel_l2(b.cpu(), a.cpu()) < 1e-2


def test_network_forward_and_gradients_match_float64(cuda):
    """Whole network, forward and backward, against float64 autograd with BF16 rounding of the
    activations and activation gradients at the points where the kernels store BF16."""
    import torch

    from iane_gb300.learned import WarmStartNet

    shape = (8, 12, 16)
    net = WarmStartNet(cuda, seed=3)
    # a head with real weights, so every layer receives gradient
    gen = torch.Generator().manual_seed(9)
    w0, b0 = net.offsets["head"]
    net.master[w0:b0] = (torch.randn(b0 - w0, generator=gen) * 0.3).to(cuda)
    net.p16.copy_(net.master.to(torch.bfloat16))
    obs = (torch.rand(shape, generator=gen, dtype=torch.float32) * 2.0).to(cuda)
    target = (torch.rand(shape, generator=gen, dtype=torch.float32) * 2.0).to(cuda)
    sigma = 2.0

    net.zero_grad()
    out = net.forward(obs, sigma)
    loss = net.loss_and_grad(target)
    net.backward(shape)
    torch.cuda.synchronize()

    params = net.master.cpu()
    p = unpack(params)
    for name, _, _ in LAYERS:  # the kernels multiply BF16 copies of the weights
        with torch.no_grad():
            p[name][0].copy_(bf16_round(p[name][0]))
    x = torch.stack([obs.cpu().double(), torch.full(shape, sigma / 3.0, dtype=torch.float64)])
    ref_out = forward(p, x, obs.cpu().double())
    ref_loss = ((ref_out[0] - target.cpu().double()) ** 2).mean()
    ref_loss.backward()

    assert _rel_l2(out.cpu(), ref_out.detach()) < 1e-3
    ref_value = float(ref_loss.detach())
    assert abs(float(loss.detach().item()) - ref_value) < 2e-2 * ref_value
    for name, ci, co in LAYERS:
        gw = net.dw(name).cpu().double().reshape(co, ci, 27)
        gb = net.db(name).cpu().double()
        rw, rb = p[name][0].grad, p[name][1].grad
        err_w = _rel_l2(gw, rw)
        err_b = _rel_l2(gb, rb)
        assert err_w < 3e-2, (name, err_w)
        assert err_b < 3e-2, (name, err_b)


def test_training_reduces_the_loss(cuda):
    """A few Adam steps on small synthetic pairs lower the loss."""
    import torch

    from iane_gb300.learned import WarmStartNet, make_pair, train

    rng = np.random.default_rng(2)
    pairs = [make_pair(rng, size=32, iterations=30, device=cuda, ellipsoids=10) for _ in range(4)]
    net = WarmStartNet(cuda, seed=1)

    def total_loss():
        s = 0.0
        for observed, sigma, target, _ in pairs:
            mean = observed.double().mean().float()
            net.zero_grad()
            net.forward(observed / mean, sigma)
            s += float(net.loss_and_grad((target / mean).contiguous()).item())
        return s

    before = total_loss()
    train(net, pairs, epochs=25, lr=2e-3)
    after = total_loss()
    assert after < 0.7 * before, (before, after)


def test_learned_start_gains_over_the_flat_start(cuda):
    """The shipped weights on a held-out 64^3 volume: the network's start is much closer to
    the 200-iteration FP32 result than the flat start, stays closer after 10 iterations (BF16
    tensor-core RL from the learned start, FP32 from the flat start), and reaches a relative
    change of 1e-3 per iteration in far fewer iterations."""
    import torch

    import iane_gb300
    from iane_gb300.learned import load_default, make_pair

    net = load_default(cuda)
    observed, sigma, target, psf = make_pair(np.random.default_rng(987654), size=64)
    flat = torch.full_like(observed, float(observed.double().mean()))
    start = net.warm_start(observed, sigma)
    e_flat0, e_learn0 = _rel_l2(flat.cpu(), target.cpu()), _rel_l2(start.cpu(), target.cpu())
    assert e_learn0 < 0.3 * e_flat0, (e_learn0, e_flat0)

    rl32 = iane_gb300.RichardsonLucy(psf, observed.shape)
    rl16 = iane_gb300.RichardsonLucy(psf, observed.shape, precision="bf16")
    est32, est16 = torch.empty_like(observed), start.clone()
    rl32.run(observed, est32, 10, 1e-6, init=rl32.INIT_MEAN)
    rl16.run(observed, est16, 10, 1e-6, init=rl16.INIT_GIVEN)
    e_plain10, e_learn10 = _rel_l2(est32.cpu(), target.cpu()), _rel_l2(est16.cpu(), target.cpu())
    assert e_learn10 < 0.5 * e_plain10, (e_learn10, e_plain10)

    def iterations_to_converge(rl, est, init):
        stats = torch.zeros(2, dtype=torch.float64, device=cuda)
        for k in range(1, 201):
            rl.run(observed, est, 1, 1e-6, init=init if k == 1 else rl.INIT_GIVEN, stats=stats)
            if float(stats[1]) <= 1e-3:
                return k
        return 201

    n_plain = iterations_to_converge(rl32, torch.empty_like(observed), rl32.INIT_MEAN)
    n_learn = iterations_to_converge(rl16, start.clone(), rl16.INIT_GIVEN)
    assert n_learn <= n_plain // 2, (n_learn, n_plain)
    rl32.close()
    rl16.close()
