"""Loader of libmcx_gb300.so with the C signatures of include/mcx_abi.h and include/mcx_gb300.h.

The engine has no CPU path: if the shared library is missing, importing this module raises.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import abi

LIB_PATH = Path(__file__).resolve().parent / "libmcx_gb300.so"

if not LIB_PATH.exists():
    raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                      "(the GB300 engine has no CPU fallback)")

lib = C.CDLL(str(LIB_PATH))
libc = C.CDLL(None)
libc.free.argtypes = [C.c_void_p]
libc.free.restype = None

_CFG = C.POINTER(abi.Config)

# drop-in boundary (src/mcx_core.h:200-201)
lib.mcx_run_simulation.argtypes = [_CFG, C.POINTER(abi.GPUInfo)]
lib.mcx_run_simulation.restype = None
lib.mcx_list_gpu.argtypes = [_CFG, C.POINTER(C.POINTER(abi.GPUInfo))]
lib.mcx_list_gpu.restype = C.c_int
# extensions (include/mcx_gb300.h)
lib.mcxg_run_simulation_fp64.argtypes = [_CFG, C.POINTER(abi.GPUInfo)]
lib.mcxg_run_simulation_fp64.restype = None
lib.mcxg_initcfg.argtypes = [_CFG]
lib.mcxg_initcfg.restype = None
lib.mcxg_validatecfg.argtypes = [_CFG]
lib.mcxg_validatecfg.restype = C.c_int
lib.mcxg_maskdet.argtypes = [_CFG]
lib.mcxg_maskdet.restype = None
lib.mcxg_last_error.argtypes = []
lib.mcxg_last_error.restype = C.c_char_p
lib.mcxg_last_error_id.argtypes = []
lib.mcxg_last_error_id.restype = C.c_int
lib.mcxg_clear_error.argtypes = []
lib.mcxg_clear_error.restype = None
lib.mcxg_set_error.argtypes = [C.c_int, C.c_char_p]
lib.mcxg_set_error.restype = None
lib.mcxg_get_stats.argtypes = [C.POINTER(abi.Stats)]
lib.mcxg_get_stats.restype = C.c_int
lib.mcxg_rng_test.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_float), C.c_int]
lib.mcxg_rng_test.restype = C.c_int
lib.mcxg_photon_stream.argtypes = [C.c_uint64, C.c_uint64, C.POINTER(C.c_float), C.c_int]
lib.mcxg_photon_stream.restype = C.c_int
lib.mcxg_replayinit.argtypes = [_CFG, C.POINTER(C.c_float), C.POINTER(C.c_int), C.c_int]
lib.mcxg_replayinit.restype = C.c_int
lib.mcxg_set_field_precision.argtypes = [C.c_int]
lib.mcxg_set_field_precision.restype = None
lib.mcxg_photon_shares.argtypes = [_CFG, C.POINTER(abi.GPUInfo), C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
lib.mcxg_photon_shares.restype = C.c_int
lib.mcxg_set_step_cap.argtypes = [C.c_uint]
lib.mcxg_set_step_cap.restype = None
lib.mcxg_run_batch.argtypes = [C.POINTER(C.POINTER(abi.Config)), C.c_int, C.c_int, C.POINTER(abi.Stats),
                                C.POINTER(C.c_double)]
lib.mcxg_run_batch.restype = C.c_int
lib.mcxg_run_batch_device.argtypes = [C.POINTER(C.POINTER(abi.Config)), C.c_int, C.c_int, C.POINTER(C.c_void_p),
                                       C.POINTER(abi.Stats), C.POINTER(C.c_double)]
lib.mcxg_run_batch_device.restype = C.c_int
lib.mcxg_session_create.argtypes = [_CFG, C.c_int]
lib.mcxg_session_create.restype = C.c_void_p
lib.mcxg_session_reset.argtypes = [C.c_void_p]
lib.mcxg_session_reset.restype = C.c_int
lib.mcxg_session_run.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(C.c_float)]
lib.mcxg_session_run.restype = C.c_int
lib.mcxg_session_read.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint64,
                                  C.POINTER(abi.Stats)]
lib.mcxg_session_read.restype = C.c_int64
lib.mcxg_session_destroy.argtypes = [C.c_void_p]
lib.mcxg_session_destroy.restype = None
lib.mcxg_session_autotune.argtypes = [C.c_void_p, C.c_uint64]
lib.mcxg_session_autotune.restype = C.c_int
lib.mcxg_set_launch.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
lib.mcxg_set_launch.restype = None

lib.mcxg_probe_atomic_rate.argtypes = [C.c_uint64, C.POINTER(C.c_double)]
lib.mcxg_probe_atomic_rate.restype = C.c_int
lib.mcxg_set_seeding.argtypes = [C.c_int]
lib.mcxg_set_seeding.restype = None
lib.mcxg_run_noalloc.argtypes = [_CFG, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64,
                                 C.c_int, C.c_void_p, C.POINTER(abi.Stats)]
lib.mcxg_run_noalloc.restype = C.c_int
lib.mcxg_noalloc_scratch_bytes.argtypes = []
lib.mcxg_noalloc_scratch_bytes.restype = C.c_size_t

# fluence denoiser kernels (include/mcxg_denoise.h); pointers are device addresses
_P, _I, _LL, _F = C.c_void_p, C.c_int, C.c_longlong, C.c_float
_DN = {
    "mcxg_dn_conv_fwd": [_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _I, _P],
    "mcxg_dn_conv_wgrad": [_P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _P],
    "mcxg_dn_bias_grad": [_P, _P, _LL, _I, _P],
    "mcxg_dn_pool": [_P, _P, _I, _I, _I, _I, _I, _P],
    "mcxg_dn_upcat": [_P, _P, _P, _I, _I, _I, _I, _I, _I, _P],
    "mcxg_dn_upcat_bwd": [_P, _P, _P, _I, _I, _I, _I, _I, _I, _P],
    "mcxg_dn_unpool_add": [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P],
    "mcxg_dn_head": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _LL, _F, _P],
    "mcxg_dn_pack": [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P],
    "mcxg_dn_adamw": [_P, _P, _P, _P, _P, _P, _LL, _I, _I, _I, _F, _F, _F, _F, _F, _I, _P],
}
for _name, _args in _DN.items():
    getattr(lib, _name).argtypes = _args
    getattr(lib, _name).restype = C.c_int
lib.mcxg_dn_check.argtypes = [C.c_void_p]
lib.mcxg_dn_check.restype = C.c_int
lib.mcxg_dn_last_error.argtypes = []
lib.mcxg_dn_last_error.restype = C.c_char_p

EXPORTED = [
    "mcx_run_simulation", "mcx_list_gpu", "mcxg_run_simulation_fp64", "mcxg_initcfg", "mcxg_validatecfg",
    "mcxg_maskdet", "mcxg_last_error", "mcxg_last_error_id", "mcxg_clear_error", "mcxg_set_error", "mcxg_get_stats",
    "mcxg_rng_test", "mcxg_photon_stream", "mcxg_session_create", "mcxg_session_reset", "mcxg_session_run",
    "mcxg_session_read", "mcxg_session_destroy", "mcxg_set_launch", "mcxg_run_noalloc", "mcxg_noalloc_scratch_bytes",
    "mcxg_set_seeding", "mcxg_probe_atomic_rate",
    "mcxg_session_autotune", "mcxg_run_batch", "mcxg_run_batch_device", "mcxg_replayinit", "mcxg_set_step_cap", "mcxg_dn_last_error",
    "mcxg_set_field_precision", "mcxg_photon_shares", "mcxg_dn_check",
] + list(_DN)
