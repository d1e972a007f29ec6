"""Split-voxel Monte Carlo (MEDIA_2LABEL_SPLIT, SVMC; src/mcx_core.cu:688-830, 2112-2133,
2295-2310, 2386-2404) on the GPU, checked by geometry rather than against the oracle:

  * a volume whose every voxel is split between label 1 and label 1 (any plane) is the plain
    label-1 volume: the same photons, the flights only cut at the planes;
  * a layered medium whose interface runs through the middle of a voxel layer, written as split
    voxels at 1 mm, is the same medium written as labels at 0.5 mm (twice the resolution), with
    a refractive-index step at the interface (Fresnel reflection and refraction at the split
    voxels' planes): absorbed fraction and escaped weight within 5 standard errors.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _deck(vol, prop, n=30, unit=1.0, nphoton=1_000_000, reflect=1):
    return {
        "nphoton": nphoton, "seed": 4321, "vol": vol, "prop": np.asarray(prop, np.float32), "unitinmm": unit,
        "tstart": 0.0, "tend": 5e-9, "tstep": 5e-9, "srcpos": [n / 2 / unit, n / 2 / unit, 0.0],
        "srcdir": [0.0, 0.0, 1.0], "issrcfrom0": 1, "isreflect": reflect, "issavedet": 0,
    }


def _split(n, lower, upper, point, normal):
    v = np.zeros((8, n, n, n), np.uint8)
    v[0], v[1] = lower, upper
    v[2:5] = np.asarray(point, np.uint8)[:, None, None, None]
    v[5:8] = np.asarray(normal, np.uint8)[:, None, None, None]
    return v


def test_same_label_split_is_the_plain_volume(engine):
    n = 30
    prop = [[0, 0, 1, 1], [0.01, 5.0, 0.8, 1.37]]
    a = engine.run(_deck(np.ones((n, n, n), np.uint8), prop))["stat"]
    pc = engine.prepare(_deck(_split(n, 1, 1, (100, 150, 80), (200, 90, 160)), prop))
    assert pc.c.mediabyte == 97
    b = engine.run(_deck(_split(n, 1, 1, (100, 150, 80), (200, 90, 160)), prop))["stat"]
    assert b["error_flags"] == 0
    fa, fb = a["energyabs"] / a["energytot"], b["energyabs"] / b["energytot"]
    assert abs(fa - fb) < 2e-4, (fa, fb)
    assert abs(a["n_scatter"] - b["n_scatter"]) <= 1e-3 * a["n_scatter"]


@pytest.mark.parametrize("n2", [1.37, 1.5])
def test_half_voxel_interface_equals_double_resolution(engine, n2):
    n, k0 = 30, 10
    prop = [[0, 0, 1, 1], [0.01, 5.0, 0.8, 1.37], [0.03, 10.0, 0.9, n2]]
    # split voxels at 1 mm: layers z < k0 label 1, z > k0 label 2, layer k0 split at its middle
    # (plane point z = 128/255, normal +z: label 2 (upper) lies on the normal's side)
    v = np.zeros((8, n, n, n), np.uint8)
    v[0] = np.where(np.arange(n) > k0, 2, 1)[None, None, :]
    v[0, :, :, k0] = 1
    v[1, :, :, k0] = 2
    v[2:5, :, :, k0] = 128
    v[5, :, :, k0], v[6, :, :, k0], v[7, :, :, k0] = 128, 128, 255
    ng = 1_000_000
    a = engine.run(_deck(v, prop, n=n, nphoton=ng))["stat"]
    # the same medium as labels at 0.5 mm: the interface at z = k0 + 0.5 mm = voxel 2 k0 + 1
    lab = np.where(np.arange(2 * n) >= 2 * k0 + 1, 2, 1).astype(np.uint8)
    vol2 = np.broadcast_to(lab[None, None, :], (2 * n, 2 * n, 2 * n)).copy()
    b = engine.run(_deck(vol2, prop, n=n, unit=0.5, nphoton=ng))["stat"]
    assert a["error_flags"] == 0 and b["error_flags"] == 0
    fa, fb = a["energyabs"] / a["energytot"], b["energyabs"] / b["energytot"]
    se = np.sqrt(fa * (1 - fa) / ng + fb * (1 - fb) / ng)
    print("n2", n2, "split voxels", fa, "labels at 0.5 mm", fb, "SE", se)
    assert abs(fa - fb) <= 5 * se, (fa, fb, se)


@pytest.mark.parametrize("n2", [1.37, 1.5])
def test_split_voxels_against_the_reference(engine, n2):
    """The half-voxel interface deck run by MCX's own build from the same split-voxel volume
    (MediaFormat "svmc", 8 bytes per voxel): absorbed fraction within 5 standard errors of two
    independent 1e6-photon runs, depth profile of the fluence within 5% where it is well sampled."""
    from oracle import ref_mcx

    if not ref_mcx.available():
        pytest.skip("reference sources are not staged in baseline/_ref/src")
    n, k0, ng = 30, 10, 1_000_000
    prop = [[0, 0, 1, 1], [0.01, 5.0, 0.8, 1.37], [0.03, 10.0, 0.9, n2]]
    v = np.zeros((8, n, n, n), np.uint8)
    v[0] = np.where(np.arange(n) > k0, 2, 1)[None, None, :]
    v[0, :, :, k0] = 1
    v[1, :, :, k0] = 2
    v[2:5, :, :, k0] = 128
    v[5, :, :, k0], v[6, :, :, k0], v[7, :, :, k0] = 128, 128, 255
    deck = _deck(v, prop, n=n, nphoton=ng)
    r = ref_mcx.run(dict(deck, seed=9876))
    o = engine.run(deck)
    fo = o["stat"]["energyabs"] / o["stat"]["energytot"]
    fr = r["absorbed"]
    se = np.sqrt(fo * (1 - fo) / ng + fr * (1 - fr) / ng)
    print("n2", n2, "engine", fo, "reference", fr, "SE", se)
    assert abs(fo - fr) <= 5 * se + 1e-4, (fo, fr, se)
    zo = o["flux"][..., 0].sum(axis=(0, 1)).astype(np.float64)
    zr = r["flux"][..., 0].sum(axis=(0, 1)).astype(np.float64)
    good = zr > 1e-3 * zr.max()
    assert np.all(np.abs(zo[good] / zr[good] - 1) < 0.05), (zo[good] / zr[good])


@pytest.mark.parametrize("n2", [1.37, 1.5])
def test_split_voxels_against_the_oracle(engine, oracle, n2):
    """The half-voxel interface deck run by the oracle's split-voxel restatement: absorbed fraction
    within 5 standard errors of two independent 1e6-photon runs, depth profile of the fluence
    within 5% where it is well sampled."""
    n, k0, ng = 30, 10, 1_000_000
    prop = [[0, 0, 1, 1], [0.01, 5.0, 0.8, 1.37], [0.03, 10.0, 0.9, n2]]
    v = np.zeros((8, n, n, n), np.uint8)
    v[0] = np.where(np.arange(n) > k0, 2, 1)[None, None, :]
    v[0, :, :, k0] = 1
    v[1, :, :, k0] = 2
    v[2:5, :, :, k0] = 128
    v[5, :, :, k0], v[6, :, :, k0], v[7, :, :, k0] = 128, 128, 255
    o = engine.run(_deck(v, prop, n=n, nphoton=ng))
    r = oracle.run(engine.prepare(dict(_deck(v, prop, n=n, nphoton=ng), seed=8765)))
    fo = o["stat"]["energyabs"] / o["stat"]["energytot"]
    fr = r["stat"]["energyabs"] / r["stat"]["energytot"]
    se = np.sqrt(fo * (1 - fo) / ng + fr * (1 - fr) / ng)
    print("n2", n2, "engine", fo, "oracle", fr, "SE", se)
    assert abs(fo - fr) <= 5 * se
    zo = o["flux"][..., 0].sum(axis=(0, 1)).astype(np.float64)
    zr = r["flux"][..., 0].sum(axis=(0, 1)).astype(np.float64)
    good = zr > 1e-3 * zr.max()
    assert np.all(np.abs(zo[good] / zr[good] - 1) < 0.05), (zo[good] / zr[good])
