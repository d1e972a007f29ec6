"""mcx_gb300 -- a GB300-native (sm_103a) engine for MCX's voxel Monte Carlo photon transport.

The engine is the shared library ``libmcx_gb300.so`` exporting MCX's own entry points
``mcx_run_simulation`` / ``mcx_list_gpu`` over MCX's ``Config`` layout; this package is its
pmcx-style Python front-end (``run``, ``gpuinfo``, ``version``) plus the device-resident
session used by the benchmark.
"""

from .api import MCXError, PreparedConfig, gpuinfo, prepare, run, run_batch, run_prepared, version  # noqa: F401
from .session import Session  # noqa: F401

__all__ = ["run", "run_batch", "run_prepared", "prepare", "gpuinfo", "version", "MCXError", "PreparedConfig", "Session"]
