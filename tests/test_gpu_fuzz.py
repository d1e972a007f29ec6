"""Randomised decks: the GPU path against the oracle over seeded random inputs.

Each deck draws its volume (16-48 voxels a side, up to three inclusions and a void pocket),
media, boundary conditions, reflection, time gates, output type, source shape and detectors
from one seed.  Checked per deck: energy balance to 1e-5, error-free run, absorbed fraction and
launched weight per photon within 5 combined standard errors of the oracle, photons that
entered equal within 5 SE, detected-photon counts within 5 Poisson SE.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SOURCES = ["pencil", "isotropic", "cone", "gaussian", "planar", "disk", "zgaussian", "line", "slit", "arcsine",
           "fourier", "ring"]


def deck(seed: int, nphoton: int) -> dict:
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(v) for v in rng.integers(16, 49, 3))
    vol = np.ones((nx, ny, nz), np.uint8)
    nmed = 1
    for k in range(int(rng.integers(0, 4))):
        lo = [int(rng.integers(0, d - 4)) for d in (nx, ny, nz)]
        hi = [int(rng.integers(l + 2, d)) for l, d in zip(lo, (nx, ny, nz))]
        nmed += 1
        vol[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = nmed
    if rng.random() < 0.3:                                   # a void pocket inside
        c = [int(rng.integers(4, d - 4)) for d in (nx, ny, nz)]
        vol[c[0] - 1:c[0] + 2, c[1] - 1:c[1] + 2, c[2] - 1:c[2] + 2] = 0
    prop = np.zeros((nmed + 1, 4), np.float32)
    prop[0] = [0, 0, 1, 1]
    for m in range(1, nmed + 1):
        prop[m] = [rng.uniform(0.001, 0.05), rng.uniform(0.5, 10.0), rng.uniform(0.0, 0.95), rng.uniform(1.0, 1.5)]
    ngates = int(rng.integers(1, 6))
    tend = float(rng.uniform(1e-9, 5e-9))
    src = str(rng.choice(SOURCES))
    cfg = {
        "nphoton": nphoton, "seed": int(rng.integers(1, 2**31 - 1)), "vol": vol, "prop": prop,
        "tstart": 0.0, "tend": tend, "tstep": tend / ngates,
        "srctype": src, "srcpos": [nx / 2, ny / 2, 0.0], "srcdir": [0.0, 0.0, 1.0], "issrcfrom0": 1,
        "isreflect": int(rng.integers(0, 2)), "outputtype": str(rng.choice(["x", "f", "e"])),
        "bc": "".join(rng.choice(list("_ramc")) for _ in range(6)),
    }
    if src in ("isotropic", "arcsine", "line"):
        cfg["srcpos"] = [nx / 2, ny / 2, nz / 2]
    if src == "line":
        cfg["srcparam1"] = [nx / 3, 0, 0, 0]
    elif src == "slit":
        cfg["srcparam1"] = [nx / 3, 0, 0, 0]
    elif src in ("planar", "fourier"):
        cfg.update(srcpos=[nx / 4, ny / 4, -3.0], srcparam1=[nx / 2, 0, 0, 2], srcparam2=[0, ny / 2, 0, 1])
    elif src in ("disk", "gaussian", "ring"):
        cfg["srcparam1"] = [min(nx, ny) / 6, 1.0, 0, 0]
    elif src in ("cone", "zgaussian"):
        cfg["srcparam1"] = [0.4, 0, 0, 0]
    if rng.random() < 0.6:
        cfg["detpos"] = np.array([[nx / 2 + 4, ny / 2, 0, 2.0], [nx / 2, ny / 2 - 6, 0, 2.0]], np.float32)
        cfg["issavedet"] = 1
    else:
        cfg["issavedet"] = 0
    return cfg


@pytest.mark.parametrize("seed", list(range(12)))
def test_random_deck_matches_oracle(engine, oracle, seed):
    ng, no = 1_000_000, 200_000
    g = engine.run(deck(seed, ng))
    s = g["stat"]
    assert s["error_flags"] == 0
    bal = abs(s["e_launch"] - (s["e_absdep"] + s["e_absother"] + s["e_escape"] + s["e_detect"]))
    assert bal <= 1e-5 * max(1.0, s["e_launch"])
    o = oracle.run(engine.prepare(deck(seed, no)), nphoton=no, seed=seed + 1000)["stat"]
    if s["energytot"] == 0 or o["energytot"] == 0:
        assert s["energytot"] == o["energytot"] == 0
        return
    fg, fo = s["energyabs"] / s["energytot"], o["energyabs"] / o["energytot"]
    se = np.sqrt(max(fg * (1 - fg), 1e-4) / ng + max(fo * (1 - fo), 1e-4) / no)
    assert abs(fg - fo) <= 5 * se, (seed, fg, fo)
    lg, lo = s["energytot"] / ng, o["energytot"] / no
    assert abs(lg - lo) <= 5 * np.sqrt(0.25 / ng + 0.25 / no), (seed, lg, lo)
    pg, po = s["n_photon"] / ng, o["n_photon"] / no
    assert abs(pg - po) <= 5 * np.sqrt(0.25 / ng + 0.25 / no) + 1e-9, (seed, pg, po)
    if "detp" in g or s["detected"]:
        dg, do = s["detected"] / ng, o.get("detected", 0) / no
        assert abs(dg - do) <= 5 * np.sqrt(dg / ng + do / no) + 2.0 / no, (seed, dg, do)
