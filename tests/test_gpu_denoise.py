"""The denoiser's GPU kernels against the fp32 CPU reference (oracle/denoise_ref.py).

Inputs are rounded to bf16 first, so the reference sees exactly the operands the tensor cores
see.  Tolerances: outputs stored as bf16 (convolution forward and data gradient, pooling,
upsampling) within 1 bf16 rounding (2^-8 relative) plus fp32 summation-order noise; fp32
outputs (weight and bias gradients, head gradients, AdamW) within 1e-4 relative to the largest
reference value.  The whole network -- bf16 activations through 14 convolutions -- is compared on
its output correction within 3% and on every parameter gradient by direction (cosine >= 0.99)
and size (norm within 10%).  Then a short training run on engine-generated pairs must lower the
loss, and the committed checkpoint must beat the raw low-photon map on held-out volumes.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import denoise_ref as R

pytestmark = pytest.mark.gpu

BF = torch.bfloat16


@pytest.fixture(scope="module")
def dn(engine):
    from mcx_gb300 import denoise

    return denoise


@pytest.fixture(scope="module")
def lib(engine):
    from mcx_gb300._lib import lib as L

    return L


def _call(lib, fn, *args):
    rc = getattr(lib, fn)(*args)
    assert rc == 0, (fn, rc, lib.mcxg_dn_last_error())


def _gpu(a, dtype=torch.float32):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to("cuda").to(dtype).contiguous()


def _st():
    return torch.cuda.current_stream().cuda_stream


def _close_bf16(got, ref, extra=0.0):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref).max() + 1e-30
    err = np.abs(got - ref)
    assert (err <= np.abs(ref) * 2.0 ** -8 + scale * (1e-3 + extra)).all(), float((err / scale).max())


def _nchw(a, n, d, h, w):
    return torch.from_numpy(np.asarray(a, np.float32).reshape(n, d, h, w, -1)).permute(0, 4, 1, 2, 3)


def _ndhwc(t):
    return t.permute(0, 2, 3, 4, 1).reshape(-1, t.shape[1]).detach().numpy()


SHAPES = [(16, 16), (16, 32), (32, 64), (64, 128), (128, 128), (192, 64), (96, 32), (48, 16)]
GRID = (2, 5, 7, 9)     # 630 voxels: a ragged last tile, every face of the stencil clipped


@pytest.mark.parametrize("cin,cout", SHAPES)
def test_conv_forward(lib, cin, cout):
    rng = np.random.default_rng(cin * 1000 + cout)
    n, d, h, w = GRID
    vox = n * d * h * w
    x = R.bf16(rng.standard_normal((vox, cin)))
    wt = R.bf16(rng.standard_normal((cout, 27, cin)) * R.he_std(cin))
    b = (rng.standard_normal(cout) * 0.1).astype(np.float32)
    y = torch.empty(vox * cout, dtype=BF, device="cuda")
    X, W, B = _gpu(x, BF), _gpu(wt, BF), _gpu(b)
    _call(lib, "mcxg_dn_conv_fwd", X.data_ptr(), W.data_ptr(), B.data_ptr(), None, y.data_ptr(), n, d, h, w, cin, cout, 27, 1,
          _st())
    assert lib.mcxg_dn_check(_st()) == 0, lib.mcxg_dn_last_error()
    ref = _ndhwc(R.conv(_nchw(x, n, d, h, w), torch.from_numpy(wt), torch.from_numpy(b)))
    _close_bf16(y.float().cpu().numpy().reshape(vox, cout), ref)


def test_conv_forward_pointwise_no_relu(lib):
    rng = np.random.default_rng(5)
    n, d, h, w = GRID
    vox, cin, cout = n * d * h * w, 32, 16
    x = R.bf16(rng.standard_normal((vox, cin)))
    wt = R.bf16(rng.standard_normal((cout, 1, cin)) * 0.2)
    y = torch.empty(vox * cout, dtype=BF, device="cuda")
    X, W = _gpu(x, BF), _gpu(wt, BF)
    _call(lib, "mcxg_dn_conv_fwd", X.data_ptr(), W.data_ptr(), None, None, y.data_ptr(), n, d, h, w, cin, cout, 1, 0, _st())
    _close_bf16(y.float().cpu().numpy().reshape(vox, cout), x @ wt[:, 0, :].T)


def _transposed(lib, wt):
    """The optimiser's flipped transposed bf16 copy of fp32 weights (an AdamW step with lr 0)."""
    cout, taps, cin = wt.shape
    m = _gpu(wt.reshape(-1))
    z = torch.zeros_like(m)
    w16 = torch.empty(m.numel(), dtype=BF, device="cuda")
    wt16 = torch.empty(m.numel(), dtype=BF, device="cuda")
    _call(lib, "mcxg_dn_adamw", m.data_ptr(), z.clone().data_ptr(), z.clone().data_ptr(), z.clone().data_ptr(), w16.data_ptr(),
          wt16.data_ptr(), m.numel(), cout, taps, cin, 0.0, 0.9, 0.999, 1e-8, 0.0, 1, _st())
    return w16, wt16


@pytest.mark.parametrize("cin,cout", SHAPES)
def test_conv_data_gradient(lib, cin, cout):
    rng = np.random.default_rng(7 + cin + cout)
    n, d, h, w = GRID
    vox = n * d * h * w
    wt = R.bf16(rng.standard_normal((cout, 27, cin)) * R.he_std(cin))
    dy = R.bf16(rng.standard_normal((vox, cout)))
    mask = R.bf16(rng.standard_normal((vox, cin)))
    w16, wt16 = _transposed(lib, wt)
    assert np.array_equal(w16.float().cpu().numpy(), wt.reshape(-1))
    dx = torch.empty(vox * cin, dtype=BF, device="cuda")
    DY, M = _gpu(dy, BF), _gpu(mask, BF)
    _call(lib, "mcxg_dn_conv_fwd", DY.data_ptr(), wt16.data_ptr(), None, M.data_ptr(), dx.data_ptr(), n, d, h, w, cout, cin, 27,
          0, _st())
    xt = torch.zeros(n, cin, d, h, w, requires_grad=True)
    y = R.conv(xt, torch.from_numpy(wt), None, relu=False)
    y.backward(_nchw(dy, n, d, h, w))
    ref = _ndhwc(xt.grad) * (mask > 0)
    _close_bf16(dx.float().cpu().numpy().reshape(vox, cin), ref)


@pytest.mark.parametrize("cin,cout", SHAPES)
def test_conv_weight_and_bias_gradient(lib, cin, cout):
    rng = np.random.default_rng(11 + cin + cout)
    n, d, h, w = GRID
    vox = n * d * h * w
    x = R.bf16(rng.standard_normal((vox, cin)))
    dy = R.bf16(rng.standard_normal((vox, cout)))
    dw = torch.zeros(cout * 27 * cin, device="cuda")
    db = torch.zeros(cout, device="cuda")
    X, DY = _gpu(x, BF), _gpu(dy, BF)
    _call(lib, "mcxg_dn_conv_wgrad", DY.data_ptr(), X.data_ptr(), dw.data_ptr(), n, d, h, w, cin, cout, 27, _st())
    _call(lib, "mcxg_dn_bias_grad", DY.data_ptr(), db.data_ptr(), vox, cout, _st())
    wt = torch.zeros(cout, cin, 3, 3, 3, requires_grad=True)
    y = torch.nn.functional.conv3d(_nchw(x, n, d, h, w), wt, padding=1)
    y.backward(_nchw(dy, n, d, h, w))
    ref = R.engine_weight(wt.grad).numpy().reshape(-1)
    got = dw.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max(), np.abs(got - ref).max()
    np.testing.assert_allclose(db.cpu().numpy(), dy.sum(0), rtol=1e-4, atol=1e-4 * np.abs(dy.sum(0)).max())


def test_weight_gradient_large_grid(lib):
    """Split-K over many voxel slices (64^3 x 2 volumes): the atomics sum every slice once."""
    rng = np.random.default_rng(3)
    n, d, h, w, cin, cout = 2, 64, 64, 64, 16, 16
    vox = n * d * h * w
    x = R.bf16(rng.standard_normal((vox, cin)) * 0.5)
    dy = R.bf16(rng.standard_normal((vox, cout)) * 0.5)
    dw = torch.zeros(cout * 27 * cin, device="cuda")
    X, DY = _gpu(x, BF), _gpu(dy, BF)
    _call(lib, "mcxg_dn_conv_wgrad", DY.data_ptr(), X.data_ptr(), dw.data_ptr(), n, d, h, w, cin, cout, 27, _st())
    wt = torch.zeros(cout, cin, 3, 3, 3, requires_grad=True)
    y = torch.nn.functional.conv3d(_nchw(x, n, d, h, w), wt, padding=1)
    y.backward(_nchw(dy, n, d, h, w))
    ref = R.engine_weight(wt.grad).numpy().reshape(-1)
    assert np.abs(dw.cpu().numpy() - ref).max() <= 1e-4 * np.abs(ref).max()


def test_pool_upcat_and_backward(lib):
    rng = np.random.default_rng(4)
    n, d, h, w, c1, c2 = 2, 8, 6, 4, 32, 16
    fine, coarse = n * d * h * w, n * d * h * w // 8
    x = R.bf16(rng.standard_normal((fine, c2)))
    low = R.bf16(rng.standard_normal((coarse, c1)))
    X, L = _gpu(x, BF), _gpu(low, BF)
    p = torch.empty(coarse * c2, dtype=BF, device="cuda")
    _call(lib, "mcxg_dn_pool", X.data_ptr(), p.data_ptr(), n, d, h, w, c2, _st())
    ref = _ndhwc(torch.nn.functional.avg_pool3d(_nchw(x, n, d, h, w), 2))
    _close_bf16(p.float().cpu().numpy().reshape(coarse, c2), ref)
    cat = torch.empty(fine * (c1 + c2), dtype=BF, device="cuda")
    _call(lib, "mcxg_dn_upcat", L.data_ptr(), X.data_ptr(), cat.data_ptr(), n, d, h, w, c1, c2, _st())
    up = torch.nn.functional.interpolate(_nchw(low, n, d // 2, h // 2, w // 2), scale_factor=2, mode="nearest")
    ref = _ndhwc(torch.cat([up, _nchw(x, n, d, h, w)], 1))
    assert np.array_equal(cat.float().cpu().numpy().reshape(fine, c1 + c2), ref)
    # backward: the upsampled half sums to the parents (masked by low > 0), the skip half adds
    # to the pooled gradient spread over the children (masked by x > 0)
    dcat = R.bf16(rng.standard_normal((fine, c1 + c2)))
    dp = R.bf16(rng.standard_normal((coarse, c2)))
    DC, DP = _gpu(dcat, BF), _gpu(dp, BF)
    dlow = torch.empty(coarse * c1, dtype=BF, device="cuda")
    _call(lib, "mcxg_dn_upcat_bwd", DC.data_ptr(), L.data_ptr(), dlow.data_ptr(), n, d, h, w, c1, c2, _st())
    lt = _nchw(low, n, d // 2, h // 2, w // 2).clone().requires_grad_(True)
    upt = torch.nn.functional.interpolate(lt, scale_factor=2, mode="nearest")
    upt.backward(_nchw(dcat[:, :c1], n, d, h, w))
    _close_bf16(dlow.float().cpu().numpy().reshape(coarse, c1), _ndhwc(lt.grad) * (low > 0))
    dx = torch.empty(fine * c2, dtype=BF, device="cuda")
    _call(lib, "mcxg_dn_unpool_add", DP.data_ptr(), DC.data_ptr(), X.data_ptr(), dx.data_ptr(), n, d, h, w, c1, c2, _st())
    xt = _nchw(x, n, d, h, w).clone().requires_grad_(True)
    torch.nn.functional.avg_pool3d(xt, 2).backward(_nchw(dp, n, d // 2, h // 2, w // 2))
    ref = (_ndhwc(xt.grad) + dcat[:, c1:]) * (x > 0)
    _close_bf16(dx.float().cpu().numpy().reshape(fine, c2), ref)


def test_head_and_loss(lib):
    rng = np.random.default_rng(6)
    m = 5000
    act = R.bf16(np.maximum(rng.standard_normal((m, 16)), 0) * (rng.random((m, 16)) < 0.7))
    xres = rng.standard_normal(m).astype(np.float32)
    hw = rng.standard_normal(16).astype(np.float32) * 0.3
    hb = np.array([0.2], np.float32)
    tgt = (xres + rng.standard_normal(m)).astype(np.float32)
    valid = (rng.random(m) < 0.6).astype(np.float32)
    inv = 1.0 / valid.sum()
    A, XR, W, B, T, V = (_gpu(act, BF), _gpu(xres), _gpu(hw), _gpu(hb), _gpu(tgt), _gpu(valid))
    out = torch.empty(m, device="cuda")
    _call(lib, "mcxg_dn_head", A.data_ptr(), XR.data_ptr(), W.data_ptr(), B.data_ptr(), None, None, out.data_ptr(), None, None,
          None, None, m, 0.0, _st())
    ref_out = xres + hb[0] + act @ hw
    np.testing.assert_allclose(out.cpu().numpy(), ref_out, rtol=1e-5, atol=1e-5)
    dact = torch.empty(m * 16, dtype=BF, device="cuda")
    dw, db, loss = torch.zeros(16, device="cuda"), torch.zeros(1, device="cuda"), torch.zeros(1, device="cuda")
    _call(lib, "mcxg_dn_head", A.data_ptr(), XR.data_ptr(), W.data_ptr(), B.data_ptr(), T.data_ptr(), V.data_ptr(), None,
          dact.data_ptr(), dw.data_ptr(), db.data_ptr(), loss.data_ptr(), m, float(inv), _st())
    at = torch.from_numpy(act).requires_grad_(True)
    wt = torch.from_numpy(hw).requires_grad_(True)
    bt = torch.from_numpy(hb).requires_grad_(True)
    o = torch.from_numpy(xres) + bt + at @ wt
    L = ((o - torch.from_numpy(tgt)).abs() * torch.from_numpy(valid)).sum() * inv
    L.backward()
    assert abs(loss.item() * inv - L.item()) <= 1e-4 * L.item()
    np.testing.assert_allclose(dw.cpu().numpy(), wt.grad.numpy(), rtol=1e-3, atol=1e-6)
    np.testing.assert_allclose(db.cpu().numpy(), bt.grad.numpy(), rtol=1e-3, atol=1e-6)
    _close_bf16(dact.float().cpu().numpy().reshape(m, 16), at.grad.numpy() * (act > 0))


def test_pack(lib):
    rng = np.random.default_rng(8)
    nvol, d, h, w, nprop = 3, 12, 10, 14, 5
    vox = d * h * w
    flux = (10.0 ** rng.uniform(-9, 0, (nvol, vox))).astype(np.float32) * (rng.random((nvol, vox)) < 0.9)
    labels = rng.integers(0, nprop + 2, (nvol, vox)).astype(np.uint8)
    props = np.stack([np.c_[rng.uniform(1e-3, 5e-2, nprop), rng.uniform(0.5, 20, nprop), rng.uniform(0.7, 0.95, nprop),
                            np.full(nprop, 1.37)] for _ in range(nvol)]).astype(np.float32)
    props[:, 0] = [0, 0, 1, 1]
    lp = np.log10([1e5, 1e6, 3e5]).astype(np.float32)
    F, Lb, P, LP = _gpu(flux), torch.from_numpy(labels).cuda(), _gpu(props), _gpu(lp)
    x0 = torch.empty(nvol * vox * 16, dtype=BF, device="cuda")
    xres = torch.empty(nvol * vox, device="cuda")
    _call(lib, "mcxg_dn_pack", F.data_ptr(), Lb.data_ptr(), P.data_ptr(), LP.data_ptr(), x0.data_ptr(), xres.data_ptr(), nvol,
          d, h, w, nprop, _st())
    rx, rl = R.features(flux, labels, props, lp, (d, h, w))
    np.testing.assert_allclose(xres.cpu().numpy().reshape(nvol, vox), rl, rtol=1e-5, atol=1e-4)
    _close_bf16(x0.float().cpu().numpy().reshape(nvol, vox, 16), R.bf16(rx), extra=1e-3)


def test_adamw(lib):
    rng = np.random.default_rng(9)
    cout, taps, cin = 32, 27, 16
    n = cout * taps * cin
    p = rng.standard_normal(n) * 0.1
    P = _gpu(p)
    M1, M2 = torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
    w16 = torch.empty(n, dtype=BF, device="cuda")
    wt16 = torch.empty(n, dtype=BF, device="cuda")
    m1 = np.zeros(n)
    m2 = np.zeros(n)
    for step in range(1, 4):
        g = rng.standard_normal(n) * 0.01
        G = _gpu(g)
        _call(lib, "mcxg_dn_adamw", P.data_ptr(), G.data_ptr(), M1.data_ptr(), M2.data_ptr(), w16.data_ptr(), wt16.data_ptr(), n,
              cout, taps, cin, 1e-3, 0.9, 0.999, 1e-8, 1e-2, step, _st())
        p, m1, m2 = R.adamw(p, g.astype(np.float32).astype(np.float64), m1, m2, 1e-3, 0.9, 0.999, 1e-8, 1e-2, step)
        assert not G.any().item()      # the gradient is cleared
    np.testing.assert_allclose(P.cpu().numpy(), p, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(M1.cpu().numpy(), m1, rtol=1e-4, atol=1e-9)
    np.testing.assert_allclose(M2.cpu().numpy(), m2, rtol=1e-4, atol=1e-12)
    pw = R.bf16(P.cpu().numpy())
    assert np.array_equal(w16.float().cpu().numpy(), pw)
    flipped = pw.reshape(cout, taps, cin)[:, ::-1, :].transpose(2, 1, 0).reshape(-1)
    assert np.array_equal(wt16.float().cpu().numpy(), flipped)


def _net_case(dn, seed=5):
    rng = np.random.default_rng(seed)
    params = dn.init_params(seed)
    for name, _, cout, _ in dn.LAYERS:
        params[name + ".b"] = (rng.standard_normal(cout) * 0.05).astype(np.float32)
        params[name + ".w"] = R.bf16(params[name + ".w"])
    params["head.w"] = (rng.standard_normal(16) * 0.2).astype(np.float32)
    params["head.b"] = np.array([0.1], np.float32)
    nvol, d, h, w = 2, 16, 16, 16
    vox = nvol * d * h * w
    x0 = np.zeros((vox, 16), np.float32)
    x0[:, :4] = rng.standard_normal((vox, 4))
    x0 = R.bf16(x0)
    xres = rng.standard_normal(vox).astype(np.float32)
    tgt = (xres + rng.standard_normal(vox) * 0.5).astype(np.float32)
    valid = (rng.random(vox) < 0.7).astype(np.float32)
    return params, (nvol, d, h, w), x0, xres, tgt, valid


def test_network_forward_and_gradients(dn):
    params, (nvol, d, h, w), x0, xres, tgt, valid = _net_case(dn)
    inv = 1.0 / valid.sum()
    net = dn.UNet(params)
    out = torch.empty(nvol * d * h * w, device="cuda")
    A = net.forward(_gpu(x0, BF), _gpu(xres), nvol, d, h, w, out=out)
    net.loss_acc.zero_()
    net.backward(A, _gpu(tgt), _gpu(valid), inv)
    torch.cuda.synchronize()
    L, ref_out, ref_g = R.grads(params, x0, xres, tgt, valid, inv, nvol, d, h, w)
    corr, ref_corr = out.cpu().numpy() - xres, ref_out.numpy() - xres
    assert np.abs(corr - ref_corr).max() <= 0.03 * np.abs(ref_corr).max(), np.abs(corr - ref_corr).max()
    assert abs(net.loss_acc.item() * inv - L) <= 0.01 * L
    got = net.grads()
    for k, r in ref_g.items():
        g = got[k].reshape(-1).astype(np.float64)
        r = r.reshape(-1).astype(np.float64)
        cos = g @ r / (np.linalg.norm(g) * np.linalg.norm(r) + 1e-30)
        ratio = np.linalg.norm(g) / (np.linalg.norm(r) + 1e-30)
        print(f"{k}: cosine {cos:.5f} norm ratio {ratio:.4f}")
        assert cos >= 0.99 and 0.9 <= ratio <= 1.1, (k, cos, ratio)


def test_training_lowers_the_loss(dn):
    """Engine-made pairs (eight 32^3 volumes, 1e4 / 1e5 photons against 2e6): 400 AdamW steps
    lower the loss over the training set, at both photon counts, below the network's starting
    point (about the 3x3x3 box filter its head corrects)."""
    data = dn.make_pairs(8, edge=32, seed=77, target_photons=2e6, input_photons=(1e4, 1e5), valid_frac=1e-4)
    net = dn.UNet(seed=1)
    before = dn.evaluate_loss(net, data)
    dn.train(net, data, steps=400, batch=2, lr=1e-3, log_every=100, verbose=False)
    after = dn.evaluate_loss(net, data)
    print("loss before", before, "after", after)
    assert np.isfinite(after).all()
    assert all(a <= 0.93 * b for a, b in zip(after, before)), (before, after)


def test_checkpoint_beats_raw_low_photon_maps(dn):
    """Held-out 64^3 volumes (a seed the checkpoint never saw): against a 1e8-photon run, the
    denoised 1e5-photon map has a smaller median relative error than the raw 1e5-photon map
    (what the network gains over plain MC) and than its 3x3x3 box filter (the network's
    starting point, so the gain is learned)."""
    from mcx_gb300.api import run

    if not dn.DEFAULT_WEIGHTS.exists():
        pytest.skip("no trained checkpoint in the package")
    net = dn.UNet(dn.load_params())
    raw, box, den = [], [], []
    for cfg in dn.problems.denoise_instances(3, 64, seed=424242):
        judge = run(dict(cfg, nphoton=1e8))["flux"][..., 0]
        f = run(dict(cfg, nphoton=1e5, seed=cfg["seed"] + 5))["flux"][..., 0]
        d = net.denoise(f, cfg["vol"], cfg["prop"], 1e5)
        b3 = R.box_means(f.reshape(1, -1, order="F"), (64, 64, 64))[0].reshape(f.shape, order="F")
        raw.append(dn.median_rel_error(f, judge))
        box.append(dn.median_rel_error(b3, judge))
        den.append(dn.median_rel_error(d, judge))
    print("raw", raw, "box", box, "denoised", den)
    assert np.median(den) <= 0.7 * np.median(raw), (raw, den)
    assert np.median(den) < np.median(box), (box, den)


def test_denoise_on_the_device_equals_the_host_call():
    """UNet.denoise_device on a map already on the GPU gives the host call's map bit for bit (the
    same kernels in the same order), and several volumes can be queued before one synchronise."""
    import torch

    from mcx_gb300 import denoise as dn
    from mcx_gb300 import problems

    net = dn.UNet(seed=3)
    cfgs = problems.denoise_instances(2, 32, seed=9)
    rng = np.random.default_rng(1)
    maps = [rng.random(c["vol"].shape).astype(np.float32) for c in cfgs]
    want = [net.denoise(m, c["vol"], c["prop"], 1e5) for m, c in zip(maps, cfgs)]
    dev = [torch.from_numpy(m.ravel(order="F").copy()).cuda() for m in maps]
    outs = [torch.empty_like(d) for d in dev]
    for d, o, c in zip(dev, outs, cfgs):
        net.denoise_device(d, c["vol"], c["prop"], 1e5, out=o)
    torch.cuda.synchronize()
    for o, w, c in zip(outs, want, cfgs):
        assert np.array_equal(o.cpu().numpy(), w.ravel(order="F"))


def test_denoise_many_volumes_in_one_pass_equals_one_at_a_time():
    """UNet.denoise_many_device (the volumes of one shape as one batch through every kernel) gives
    each volume exactly what denoise_device gives it alone; media tables of different lengths are
    padded with rows no label reads."""
    import torch

    from mcx_gb300 import denoise as dn
    from mcx_gb300 import problems

    net = dn.UNet(seed=4)
    cfgs = problems.denoise_instances(3, 32, seed=21)
    rng = np.random.default_rng(2)
    block = torch.from_numpy(rng.random((3, 32 ** 3)).astype(np.float32)).cuda()
    budgets = [1e5, 3e5, 1e6]
    alone = [net.denoise_device(block[i].clone(), c["vol"], c["prop"], n).cpu().numpy()
             for i, (c, n) in enumerate(zip(cfgs, budgets))]
    many = net.denoise_many_device(block.clone(), [c["vol"] for c in cfgs], [c["prop"] for c in cfgs], budgets)
    torch.cuda.synchronize()
    for i in range(3):
        assert np.array_equal(many[i].cpu().numpy(), alone[i]), i
