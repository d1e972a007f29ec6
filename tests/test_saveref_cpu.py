"""Preparation of the diffuse-reflectance output (src/mcx_utils.c:3757-3759, 1808-1818)."""

from __future__ import annotations

import pytest

from mcx_gb300 import problems


def test_saveref_needs_the_field(engine):
    pc = engine.prepare(problems.reflectance_cube(100) | {"issave2pt": 0})
    assert pc.c.issaveref == b"\x00"
    pc = engine.prepare(problems.reflectance_cube(100))
    assert pc.c.issaveref == b"\x01"


def test_exit_path_mode_needs_detection(engine):
    with pytest.raises(engine.MCXError, match="two outputs"):
        engine.prepare(problems.reflectance_cube(100) | {"issaveref": 2})


def test_exit_path_mode_settings(engine):
    pc = engine.prepare(problems.reflectance_cube(100) | {"issaveref": 2, "issavedet": 1, "maxdetphoton": 10,
                                                          "detpos": [[31.0, 31.0, 61.0, 1.0]]})
    assert pc.c.maxdetphoton == 62 ** 3 and pc.c.savedetflag == 5
