"""mcx_gb300 -- a GB300-native (sm_103a) engine for MCX's voxel Monte Carlo photon transport.

The engine is the shared library ``libmcx_gb300.so`` exporting MCX's own entry points
``mcx_run_simulation`` / ``mcx_list_gpu`` over MCX's ``Config`` layout; this package is its
pmcx-style Python front-end (``run``, ``gpuinfo``, ``version``) plus the device-resident
session used by the benchmark.

The library is loaded on first use of a name that needs it: ``mcx_gb300.problems`` (the input
decks) and ``mcx_gb300.abi`` (the struct layouts) import without it, so code that only builds
inputs -- a front-end of another engine, a test generator -- never maps the engine.
"""

from __future__ import annotations

import importlib

_API = ("MCXError", "PreparedConfig", "gpuinfo", "prepare", "run", "run_batch", "run_prepared", "version")

__all__ = ["run", "run_batch", "run_prepared", "prepare", "gpuinfo", "version", "MCXError", "PreparedConfig", "Session"]


def __getattr__(name: str):
    if name in _API:
        return getattr(importlib.import_module(".api", __name__), name)
    if name == "Session":
        return importlib.import_module(".session", __name__).Session
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
