"""Per-voxel media formats (src/mcx_core.cu:582-730) on the GPU.

MCX's 32-bit voxel words encode the properties of every voxel: mua as a float (MEDIA_MUA_FLOAT),
mua and mus as binary16 (MEDIA_AS_F2H), interpolation fractions between prop rows 2 and 3
(MEDIA_ASGN_BYTE, MEDIA_AS_SHORT), a label with one property replaced by a binary16 value
(MEDIA_LABEL_HALF), all four properties as binary16 in two words (MEDIA_ASGN_F2H), or a mix of
two labels chosen at random on entry (MEDIA_2LABEL_MIX); the fields a format does not store come
from row 2 (the label's row).  Checked:
a label volume rewritten per voxel gives the label run's result; each format against the oracle's
decode (absorbed fraction, launched weight, detected count within 5 standard errors); detectors
keep only format-independent record columns.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu


def _grid(n=40):
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return i, j, k


def deck(fmt: str, n: int, nphoton: int) -> dict:
    i, j, k = _grid(n)
    cfg = {
        "nphoton": nphoton, "seed": 777, "tstart": 0.0, "tend": 5e-9, "tstep": 1e-9,
        "srcpos": [n / 2, n / 2, 0.0], "srcdir": [0.0, 0.0, 1.0], "issrcfrom0": 1, "isreflect": 1,
        "prop": np.array([[0, 0, 1, 1], [0.01, 2.0, 0.8, 1.37], [0.05, 8.0, 0.95, 1.45]], np.float32),
        "detpos": np.array([[n / 2 + 5, n / 2, 0, 2.0]], np.float32), "issavedet": 1,
    }
    if fmt == "mua_float":
        cfg["vol"] = (0.002 + 0.02 * k / n).astype(np.float32)
    elif fmt == "f2h":
        cfg["vol"] = np.stack([(0.002 + 0.02 * k / n), (0.5 + 5.0 * i / n)]).astype(np.float32)
    elif fmt == "asgn_byte":
        cfg["vol"] = np.stack([(255 * k / n), (255 * i / n), (255 * j / n), (127 * (k > n / 2))]).astype(np.uint8)
    elif fmt == "as_short":
        cfg["vol"] = np.stack([(65535 * k / n), (32767 * i / n)]).astype(np.uint16)
    elif fmt == "asgn_f2h":
        cfg["vol"] = np.stack([(0.002 + 0.02 * k / n), (0.5 + 5.0 * i / n), np.full((n, n, n), 0.8),
                               np.where(k > n / 2, 1.45, 1.37)]).astype(np.float32)
    elif fmt == "mix":
        # label 1 or 2, label 2's share growing with depth
        cfg["vol"] = np.stack([np.ones((n, n, n)), np.full((n, n, n), 2), 32767 * k / n]).astype(np.int16)
    elif fmt == "label_half":
        # labels 1 / 2 by x; deeper than n/2 the mus of the label is replaced by 4, elsewhere its g by 0.5
        lab = np.where(i < n / 2, 1.0, 2.0)
        fld = np.where(k > n / 2, 1.0, 2.0)
        val = np.where(k > n / 2, 4.0, 0.5)
        cfg["vol"] = np.stack([val, fld, lab]).astype(np.float32)
    return cfg


def test_label_volume_rewritten_per_voxel(engine):
    base = problems.cube60(1_000_000)
    base.update(issavedet=0, seed=99)
    base.pop("detpos")
    a = engine.run(base)["stat"]
    words = dict(base, vol=np.full((60, 60, 60), 0.005, np.float32))
    b = engine.run(words)["stat"]
    assert b["error_flags"] == 0
    # same photons, same properties: the histories coincide (up to FP contraction)
    assert abs(a["energyabs"] / a["energytot"] - b["energyabs"] / b["energytot"]) < 1e-4
    assert abs(a["n_steps"] - b["n_steps"]) <= 1e-4 * a["n_steps"]


def test_label_half_equals_label_volume(engine):
    """MEDIA_LABEL_HALF (src/mcx_core.cu:597-613): a cube of label 1 whose inclusion voxels replace
    mua by 0.0625 (exact in binary16) runs as the label volume with that inclusion as label 2."""
    base = problems.cube60(1_000_000)
    base.update(issavedet=0, seed=99)
    base.pop("detpos")
    inc = np.zeros((60, 60, 60), bool)
    inc[20:40, 20:40, 5:25] = True
    prop = np.array([[0, 0, 1, 1], [0.005, 1.0, 0.01, 1.37], [0.0625, 1.0, 0.01, 1.37]], np.float32)
    a = engine.run(dict(base, vol=np.where(inc, 2, 1).astype(np.uint8), prop=prop))["stat"]
    # inside: field 0 (mua) := 0.0625; outside: field 1 (mus) := 1.0, label 1's own value (exact in binary16)
    vol = np.stack([np.where(inc, 0.0625, 1.0), np.where(inc, 0.0, 1.0), np.ones((60, 60, 60))]).astype(np.float32)
    b = engine.run(dict(base, vol=vol, prop=prop[:2]))["stat"]
    assert b["error_flags"] == 0
    assert abs(a["energyabs"] / a["energytot"] - b["energyabs"] / b["energytot"]) < 1e-4
    assert abs(a["n_steps"] - b["n_steps"]) <= 1e-4 * a["n_steps"]


def _label_deck(prop, vol):
    cfg = problems.cube60(1_000_000)
    cfg.update(issavedet=0, seed=99, prop=np.asarray(prop, np.float32), vol=vol)
    cfg.pop("detpos")
    return cfg


def test_asgn_f2h_equals_label_volume(engine):
    """MEDIA_ASGN_F2H (src/mcx_core.cu:628-647): every voxel's mua, mus, g, n as binary16 halves in
    two words; values exact in binary16 reproduce the label run."""
    prop = [[0, 0, 1, 1], [0.0625, 1.0, 0.5, 1.375], [0.03125, 4.0, 0.75, 1.5]]
    inc = np.zeros((60, 60, 60), bool)
    inc[20:40, 20:40, 5:25] = True
    a = engine.run(_label_deck(prop, np.where(inc, 2, 1).astype(np.uint8)))["stat"]
    p = np.asarray(prop, np.float32)
    vol = np.where(inc[None], p[2][:, None, None, None], p[1][:, None, None, None]).astype(np.float32)
    b = engine.run(_label_deck(prop, vol))["stat"]
    assert engine.prepare(_label_deck(prop, vol)).c.mediabyte == 96
    assert b["error_flags"] == 0
    assert abs(a["energyabs"] / a["energytot"] - b["energyabs"] / b["energytot"]) < 1e-4
    assert abs(a["n_steps"] - b["n_steps"]) <= 1e-4 * a["n_steps"]


def test_mix_extremes(engine):
    """MEDIA_2LABEL_MIX (src/mcx_core.cu:649-666): fraction 0 is label 0 without a draw (the label
    run exactly); fraction 32767 is always label 1, drawn at every entry (the label-1 run within
    statistical error)."""
    prop = [[0, 0, 1, 1], [0.005, 1.0, 0.01, 1.37], [0.02, 4.0, 0.9, 1.37]]
    inc = np.zeros((60, 60, 60), bool)
    inc[20:40, 20:40, 5:25] = True
    ones = np.ones((60, 60, 60))
    a = engine.run(_label_deck(prop, np.where(inc, 2, 1).astype(np.uint8)))["stat"]
    lab0 = np.where(inc, 2, 1)
    mix0 = np.stack([lab0, 2 * ones, 0 * ones]).astype(np.int16)             # fraction 0: label 0 = lab0
    b = engine.run(_label_deck(prop, mix0))["stat"]
    assert b["error_flags"] == 0
    assert abs(a["energyabs"] / a["energytot"] - b["energyabs"] / b["energytot"]) < 1e-4
    mix1 = np.stack([ones, lab0, np.where(inc, 32767, 0)]).astype(np.int16)  # inclusion: always label 2
    c = engine.run(_label_deck(prop, mix1))["stat"]
    fa, fc = a["energyabs"] / a["energytot"], c["energyabs"] / c["energytot"]
    assert abs(fa - fc) <= 5 * np.sqrt(2 * fa * (1 - fa) / 1e6), (fa, fc)


@pytest.mark.parametrize("fmt,code", [("mua_float", 101), ("f2h", 100), ("asgn_byte", 103), ("as_short", 104),
                                      ("label_half", 99), ("asgn_f2h", 96), ("mix", 98)])
def test_media_format_matches_oracle(engine, oracle, fmt, code):
    ng, no = 1_000_000, 200_000
    g = engine.run(deck(fmt, 40, ng))
    s = g["stat"]
    assert engine.prepare(deck(fmt, 40, 10)).c.mediabyte == code
    assert s["error_flags"] == 0
    bal = abs(s["e_launch"] - (s["e_absdep"] + s["e_absother"] + s["e_escape"] + s["e_detect"]))
    assert bal <= 1e-5 * s["e_launch"]
    o = oracle.run(engine.prepare(deck(fmt, 40, no)), nphoton=no, seed=1234)["stat"]
    fg, fo = s["energyabs"] / s["energytot"], o["energyabs"] / o["energytot"]
    se = np.sqrt(fg * (1 - fg) / ng + fo * (1 - fo) / no)
    assert abs(fg - fo) <= 5 * se, (fmt, fg, fo)
    dg, do = s["detected"] / ng, o["detected"] / no
    assert abs(dg - do) <= 5 * np.sqrt(dg / ng + do / no) + 2.0 / no, (fmt, dg, do)
    # records keep the detector id only: per-medium columns need labels (src/mcx_utils.c:1801-1806)
    assert g["detp"].shape[0] == 1 and set(np.unique(g["detp"][0]).astype(int)) == {1}
