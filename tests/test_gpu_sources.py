"""Source shapes other than the pencil beam (src/mcx_core.cu:1261-1640) on the GPU.

Each shape is sampled per photon on the device, void skipping and specular loss included.
Checks, through the C-ABI:
  * the absorbed fractions the reference's own tests assert for the planar, isotropic, cone,
    Fourier and pencil-array sources (test/testmcx.sh:84-102);
  * every MCX_SRC_* shape (and the focusing options of the area sources) against the oracle's
    restatement: absorbed fraction within 5 combined standard errors, launched energy per photon
    and the fraction of photons that enter within 5 standard errors;
  * per-voxel fluence of the planar deck over 16 independent seeds per side (tests/stats.py);
  * energy balance launched = absorbed + escaped + detected to 1e-5.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

from .stats import assert_parity

pytestmark = pytest.mark.gpu


def _base(n, planar=True):
    cfg = problems.cube60planar(n) if planar else problems.cube60(n)
    cfg.pop("detpos", None)
    cfg["issavedet"] = 0
    return cfg


def _pattern2d():
    i, j = np.meshgrid(np.arange(20), np.arange(20), indexing="ij")
    return ((i // 5 + j // 5) % 2).astype(np.float32) * 0.8 + 0.1


def _pattern3d():
    i, j, k = np.meshgrid(np.arange(10), np.arange(10), np.arange(10), indexing="ij")
    return ((i + 2 * j + 3 * k) % 7 / 6.0).astype(np.float32)


# name -> (planar base?, overrides)
CASES = {
    "planar": (True, {}),
    "planar_focus": (True, {"srcdir": [0, 0, 1, 25.0]}),
    "planar_isotropic": (True, {"srcdir": [0, 0, 1, float("nan")]}),
    "planar_lambertian": (True, {"srcdir": [0, 0, 1, float("-inf")]}),
    "pattern": (True, {"srctype": "pattern", "srcparam1": [40, 0, 0, 20], "srcparam2": [0, 40, 0, 20],
                       "srcpattern": _pattern2d()}),
    "pattern3d": (True, {"srctype": "pattern3d", "srcpos": [10, 10, 10], "srcparam1": [10, 10, 10, 0],
                         "srcparam2": [0, 0, 0, 0], "srcpattern": _pattern3d()}),
    "fourier": (True, {"srctype": "fourier", "srcparam1": [40, 0, 0, 2]}),
    "fourierx": (True, {"srctype": "fourierx", "srcparam1": [40, 0, 0, 40], "srcparam2": [2, 1, 0.25, 0.5]}),
    "fourierx2d": (True, {"srctype": "fourierx2d", "srcparam1": [40, 0, 0, 40], "srcparam2": [2, 1, 0.25, 0]}),
    "pencilarray": (True, {"srctype": "pencilarray", "srcparam1": [40, 0, 0, 4], "srcparam2": [0, 20, 0, 2]}),
    "disk": (False, {"srctype": "disk", "srcparam1": [6, 0, 0, 0]}),
    "ring": (False, {"srctype": "ring", "srcparam1": [6, 3, 0.5, 2.5]}),
    "gaussian": (False, {"srctype": "gaussian", "srcparam1": [3, 0, 0, 0]}),
    "gaussian_focus": (False, {"srctype": "gaussian", "srcparam1": [3, 0.8, 0, 0], "srcdir": [0, 0, 1, 20.0]}),
    "isotropic": (False, {"srctype": "isotropic", "srcpos": [29, 29, 29]}),
    "cone": (False, {"srctype": "cone", "srcparam1": [0.5, 0, 0, 0]}),
    "cone_uniform": (False, {"srctype": "cone", "srcparam1": [0.7, 1, 0, 0]}),
    "arcsine": (False, {"srctype": "arcsine", "srcpos": [29, 29, 29]}),
    "zgaussian": (False, {"srctype": "zgaussian", "srcparam1": [0.3, 0, 0, 0]}),
    "hyperboloid": (False, {"srctype": "hyperboloid", "srcparam1": [2, 10, 5, 0]}),
    "line": (False, {"srctype": "line", "srcpos": [10, 29, 29], "srcparam1": [40, 0, 0, 0]}),
    "line_sector": (False, {"srctype": "line", "srcpos": [10, 29, 29], "srcdir": [0, 0, 1], "srcparam1": [40, 0, 0, 0],
                            "srcparam2": [1.0, 0, 0, 0]}),
    "slit": (False, {"srctype": "slit", "srcpos": [10, 29, 0], "srcparam1": [40, 0, 0, 0]}),
    "slit_spread": (False, {"srctype": "slit", "srcpos": [10, 29, 0], "srcparam1": [40, 0, 0, 0],
                            "srcparam2": [0.1, 0.2, 0, 0]}),
    "isotropic_outside": (False, {"srctype": "isotropic", "srcpos": [29, 29, -5]}),
}


def _cfg(name, n):
    planar, over = CASES[name]
    cfg = _base(n, planar)
    cfg.update(over)
    return cfg


@pytest.mark.parametrize("name", ["planar", "isotropic", "cone", "fourier", "pencilarray"])
def test_source_goldens(engine, goldens, name):
    g = next(x for x in goldens["sources"] if x["name"] == name)
    r = engine.run(problems.source_deck(g))
    s = r["stat"]
    frac = s["energyabs"] / s["energytot"]
    assert g["lo"] <= frac < g["hi"], (name, frac, g["source"])
    assert s["error_flags"] == 0


@pytest.mark.parametrize("name", sorted(CASES))
def test_source_shape_matches_oracle(engine, oracle, name):
    ng, no = 1_000_000, 200_000
    r = engine.run(_cfg(name, ng))
    sg = r["stat"]
    assert sg["error_flags"] == 0
    balance = abs(sg["e_launch"] - (sg["e_absdep"] + sg["e_absother"] + sg["e_escape"] + sg["e_detect"]))
    assert balance <= 1e-5 * sg["e_launch"], name
    so = oracle.run(engine.prepare(_cfg(name, no)), nphoton=no, seed=4321)["stat"]
    fg, fo = sg["energyabs"] / sg["energytot"], so["energyabs"] / so["energytot"]
    # per-photon absorbed weight lies in [0, w]: its variance is at most f(1-f) per unit weight
    se = np.sqrt(fg * (1 - fg) / ng + fo * (1 - fo) / no) + 1e-6
    assert abs(fg - fo) <= 5 * se, (name, fg, fo, se)
    # launched weight per attempted photon (pattern and Fourier weights, specular loss)
    lg, lo = sg["energytot"] / ng, so["energytot"] / no
    assert abs(lg - lo) <= 5 * np.sqrt(0.25 / ng + 0.25 / no), (name, lg, lo)
    # photons that entered the medium
    pg, po = sg["n_photon"] / ng, so["n_photon"] / no
    assert abs(pg - po) <= 5 * np.sqrt(0.25 / ng + 0.25 / no) + 1e-9, (name, pg, po)


def test_planar_voxel_parity_16_seeds(engine, oracle):
    seeds = [300 + 7 * i for i in range(16)]
    n = 100_000
    gpu = []
    for sd in seeds:
        cfg = _cfg("planar", n)
        cfg["seed"] = sd
        gpu.append(engine.run(cfg)["flux"])
    pc = engine.prepare(_cfg("planar", n))
    cpu, hits = [], None
    for sd in seeds:
        o = oracle.run(pc, seed=sd + 99991, hits=True)
        cpu.append(o["flux"])
        hits = o["hits"] if hits is None else hits + o["hits"]
    rep = assert_parity(np.stack(gpu), np.stack(cpu), hits > 1000)
    print("planar", rep)
