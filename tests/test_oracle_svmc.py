"""The oracle's split-voxel Monte Carlo (MEDIA_2LABEL_SPLIT; src/mcx_core.cu:688-830, 2112-2133,
2295-2310, 2386-2404, 2474-2507) checked by geometry on the CPU, as the engine's is on the GPU:

  * a volume whose every voxel is split between label 1 and label 1 runs the plain label-1
    volume's photons (the flights are only cut at the planes);
  * a layered medium whose interface runs through the middle of a voxel layer, as split voxels
    at 1 mm, absorbs what the same medium as labels at 0.5 mm absorbs, with and without a
    refractive-index step at the interface (Fresnel reflection and refraction at the planes).
"""

from __future__ import annotations

import numpy as np
import pytest

N, K0 = 30, 10


def _deck(vol, prop, unit=1.0, nphoton=300_000):
    return {"nphoton": nphoton, "seed": 4321, "vol": vol, "prop": np.asarray(prop, np.float32), "unitinmm": unit,
            "tstart": 0.0, "tend": 5e-9, "tstep": 5e-9, "srcpos": [N / 2 / unit, N / 2 / unit, 0.0],
            "srcdir": [0.0, 0.0, 1.0], "issrcfrom0": 1, "isreflect": 1, "issavedet": 0}


def _absorbed(r):
    return r["stat"]["energyabs"] / r["stat"]["energytot"]


def test_same_label_split_is_the_plain_volume(engine, oracle):
    prop = [[0, 0, 1, 1], [0.01, 5.0, 0.8, 1.37]]
    v = np.zeros((8, N, N, N), np.uint8)
    v[0], v[1] = 1, 1
    v[2:5] = np.asarray((100, 150, 80), np.uint8)[:, None, None, None]
    v[5:8] = np.asarray((200, 90, 160), np.uint8)[:, None, None, None]
    a = oracle.run(engine.prepare(_deck(np.ones((N, N, N), np.uint8), prop, nphoton=100_000)))
    b = oracle.run(engine.prepare(_deck(v, prop, nphoton=100_000)))
    assert abs(_absorbed(a) - _absorbed(b)) < 2e-5
    assert abs(a["stat"]["n_scatter"] - b["stat"]["n_scatter"]) <= 1e-4 * a["stat"]["n_scatter"]


@pytest.mark.parametrize("n2", [1.37, 1.5])
def test_half_voxel_interface_equals_double_resolution(engine, oracle, n2):
    prop = [[0, 0, 1, 1], [0.01, 5.0, 0.8, 1.37], [0.03, 10.0, 0.9, n2]]
    v = np.zeros((8, N, N, N), np.uint8)
    v[0] = np.where(np.arange(N) > K0, 2, 1)[None, None, :]
    v[0, :, :, K0] = 1
    v[1, :, :, K0] = 2
    v[2:5, :, :, K0] = 128
    v[5, :, :, K0], v[6, :, :, K0], v[7, :, :, K0] = 128, 128, 255
    lab = np.where(np.arange(2 * N) >= 2 * K0 + 1, 2, 1).astype(np.uint8)
    vol2 = np.broadcast_to(lab[None, None, :], (2 * N, 2 * N, 2 * N)).copy()
    a = oracle.run(engine.prepare(_deck(v, prop)))
    b = oracle.run(engine.prepare(_deck(vol2, prop, unit=0.5)))
    fa, fb = _absorbed(a), _absorbed(b)
    se = np.sqrt(fa * (1 - fa) / 3e5 + fb * (1 - fb) / 3e5)
    print("n2", n2, "split voxels", fa, "labels at 0.5 mm", fb, "SE", se)
    assert abs(fa - fb) <= 5 * se
