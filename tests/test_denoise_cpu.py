"""CPU checks of the denoiser's host side and of its CPU reference (oracle/denoise_ref.py).

* the layer plan of the package and of the reference agree, and channels flow through the
  skip concatenations;
* the reference's convolution, in the engine's [cout, 27, cin] weight order, equals a direct
  loop over the 3x3x3 stencil (pins the tap order dz*9 + dy*3 + dx and the zero padding);
* the reference's gradients equal central finite differences in float64 (pins the reference
  as a gradient oracle);
* the input features, the error metric and the training-volume generator.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import denoise_ref as R


@pytest.fixture(scope="module")
def dn(engine):
    from mcx_gb300 import denoise

    return denoise


def test_layer_plan(dn):
    assert dn.LAYERS == R.LAYERS
    spec = {n: (ci, co) for n, ci, co, _ in dn.LAYERS}
    assert spec["dec3a"][0] == spec["botb"][1] + spec["enc3b"][1]
    assert spec["dec2a"][0] == spec["dec3b"][1] + spec["enc2b"][1]
    assert spec["dec1a"][0] == spec["dec2b"][1] + spec["enc1b"][1]
    assert spec["enc1a"][0] == dn.IN_CH
    assert [spec[n][1] for n in ("enc1b", "enc2b", "enc3b", "botb")] == [16, 32, 64, 128]
    for _, ci, co, _ in dn.LAYERS:
        assert ci % 16 == 0 and co in (16, 32, 64, 128)


def test_conv_tap_order_against_direct_loop():
    rng = np.random.default_rng(0)
    n, d, h, w, cin, cout = 2, 4, 5, 3, 3, 2
    x = rng.standard_normal((n, cin, d, h, w)).astype(np.float64)
    wt = rng.standard_normal((cout, 27, cin)).astype(np.float64)
    b = rng.standard_normal(cout)
    y = R.conv(torch.from_numpy(x), torch.from_numpy(wt), torch.from_numpy(b), relu=False).numpy()
    ref = np.zeros((n, cout, d, h, w))
    for t in range(27):
        dz, dy, dx = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
        for z in range(d):
            for yy in range(h):
                for xx in range(w):
                    zs, ys, xs = z + dz, yy + dy, xx + dx
                    if 0 <= zs < d and 0 <= ys < h and 0 <= xs < w:
                        ref[:, :, z, yy, xx] += np.einsum("oc,nc->no", wt[:, t, :], x[:, :, zs, ys, xs])
    ref += b[None, :, None, None, None]
    np.testing.assert_allclose(y, ref, rtol=1e-10, atol=1e-10)
    assert np.array_equal(R.engine_weight(R.torch_weight(torch.from_numpy(wt))).numpy(), wt)


def test_reference_gradients_match_finite_differences(dn):
    rng = np.random.default_rng(1)
    nvol, d, h, w = 1, 8, 8, 8
    params = {k: v.astype(np.float64) for k, v in dn.init_params(3).items()}
    params["head.w"] = rng.standard_normal(16) * 0.3
    for n, _, co, _ in dn.LAYERS:
        params[n + ".b"] = rng.standard_normal(co) * 0.05
    vox = nvol * d * h * w
    x0 = np.zeros((vox, 16))
    x0[:, :4] = rng.standard_normal((vox, 4))
    xres = rng.standard_normal(vox)
    target = xres + rng.standard_normal(vox) * 0.5
    valid = (rng.random(vox) < 0.8).astype(np.float64)
    L, _, g = R.grads(params, x0, xres, target, valid, 1.0 / valid.sum(), nvol, d, h, w, dtype=torch.float64)
    eps = 1e-6
    checked = 0
    for key in ("enc1a.w", "bota.w", "dec3a.w", "dec1b.w", "enc2b.b", "head.w", "head.b"):
        flat = params[key].reshape(-1)
        for i in rng.choice(flat.size, size=min(3, flat.size), replace=False):
            ps = {k: v.copy() for k, v in params.items()}
            ps[key].reshape(-1)[i] += eps
            lp = R.grads(ps, x0, xres, target, valid, 1.0 / valid.sum(), nvol, d, h, w, dtype=torch.float64)[0]
            ps[key].reshape(-1)[i] -= 2 * eps
            lm = R.grads(ps, x0, xres, target, valid, 1.0 / valid.sum(), nvol, d, h, w, dtype=torch.float64)[0]
            fd = (lp - lm) / (2 * eps)
            an = g[key].reshape(-1)[i]
            assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)) + 1e-7, (key, i, fd, an)
            checked += 1
    assert checked >= 15


def test_features():
    flux = np.array([[0.0, 1.0, 1e-3, -1.0]], np.float32)            # a 1 x 1 x 4 grid
    labels = np.array([[0, 1, 2, 9]], np.uint8)
    props = np.array([[[0, 0, 1, 1], [0.01, 10.0, 0.9, 1.37], [0.001, 2.0, 0.5, 1.37]]], np.float32)
    x, l = R.features(flux, labels, props, np.array([5.0], np.float32), (1, 1, 4))
    f = np.maximum(flux[0], 0)
    b3 = np.array([f[:2].mean(), f[:3].mean(), f[1:].mean(), f[2:].mean()])
    b5 = np.array([f[:3].mean(), f.mean(), f.mean(), f[1:].mean()])
    lg = lambda a: np.log10(a + 1e-10)  # noqa: E731
    np.testing.assert_allclose(l[0], lg(b3), rtol=1e-6)
    np.testing.assert_allclose(x[0, :, 0], (lg(b3) + 5) / 3, rtol=1e-6)
    np.testing.assert_allclose(x[0, :, 1], np.clip(4 * (lg(f) - lg(b3)), -4, 4), rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(x[0, :, 2], np.clip(4 * (lg(b5) - lg(b3)), -4, 4), rtol=1e-5, atol=1e-5)
    np.testing.assert_array_equal(x[0, :, 3], [1, 0, 0, 1])
    np.testing.assert_allclose(x[0, :, 4], [-2.0, 0.0, -1.0, -1.0], atol=1e-6)      # label 9 clamps to the last row
    np.testing.assert_allclose(x[0, :, 5], [-3.0, 0.0, 0.0, 0.0], atol=1e-6)
    np.testing.assert_allclose(x[0, :, 6], -1.0)
    assert not x[..., 7:].any()


def test_box_means_against_scipy():
    from scipy.ndimage import uniform_filter

    rng = np.random.default_rng(2)
    f = rng.random((2, 5 * 6 * 7)).astype(np.float32)
    b3, b5 = R.box_means(f, (5, 6, 7))
    for r, b in ((3, b3), (5, b5)):
        g = f.reshape(2, 5, 6, 7).astype(np.float64)
        s = np.stack([uniform_filter(v, r, mode="constant") for v in g])
        c = uniform_filter(np.ones((5, 6, 7)), r, mode="constant")
        np.testing.assert_allclose(b, (s / c).reshape(2, -1), rtol=1e-9)


def test_median_rel_error(dn):
    ref = np.array([1.0, 0.5, 1e-7, 0.2])
    est = np.array([1.1, 0.5, 5.0, 0.1])
    # scored: ref >= 1e-6 * 1.0 -> voxels 0, 1, 3 with errors 0.1, 0, 0.5
    assert dn.VALID_FRAC == 1e-6
    assert dn.median_rel_error(est, ref) == pytest.approx(0.1)
    assert dn.median_rel_error(est, ref, frac=1e-8) == pytest.approx(0.3)


def test_denoise_instances(engine):
    from mcx_gb300 import problems

    a = problems.denoise_instances(4, 32, 11)
    b = problems.denoise_instances(4, 32, 11)
    for x, y in zip(a, b):
        assert np.array_equal(x["vol"], y["vol"]) and np.array_equal(x["prop"], y["prop"]) and x["seed"] == y["seed"]
    for c in a:
        assert c["vol"].shape == (32, 32, 32) and c["vol"].max() == c["prop"].shape[0] - 1 or c["vol"].max() < c["prop"].shape[0]
        p = c["prop"][1:]
        assert (p[:, 0] >= 1e-3).all() and (p[:, 0] <= 5e-2).all() and (p[:, 1] >= 0.5).all() and (p[:, 1] <= 20).all()
        assert (p[:, 2] >= 0.7).all() and (p[:, 2] <= 0.95).all() and (p[:, 3] == np.float32(1.37)).all()
        assert 8 <= c["srcpos"][0] < 24 and 8 <= c["srcpos"][1] < 24 and c["srcpos"][2] == 0
