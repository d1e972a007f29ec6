"""Benchmark plumbing on the CPU: the reference arm's process must not map this repository's
libraries, and both arms describe the workload with the same `config` object."""

from __future__ import annotations

import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_imports_map_no_repo_library(built):
    # what bench.py's reference arm imports to build its inputs and drive MCX's own binary
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import bench\n"
        "from mcx_gb300 import problems\n"
        "from oracle import ref_mcx\n"
        "cfg = bench.make_cfg('workload1', 1000, 7)\n"
        "js = ref_mcx._json_input(cfg, 'x', 'vol.bin')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(int('libmcx_gb300' in maps), int('libmcx_oracle' in maps))\n" % str(ROOT)
    )
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["0", "0"]


def test_package_loads_the_engine_on_first_use(built):
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import mcx_gb300\n"
        "a = 'libmcx_gb300' in open('/proc/self/maps').read()\n"
        "mcx_gb300.version\n"
        "b = 'libmcx_gb300' in open('/proc/self/maps').read()\n"
        "print(int(a), int(b))\n" % str(ROOT)
    )
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["0", "1"]


def test_both_arms_share_the_config_object():
    sys.path.insert(0, str(ROOT))
    import bench

    cfg = bench.make_cfg("workload1", 100_000_000, 200)
    c = bench.workload_config("workload1", cfg, 100_000_000, 1)
    assert c == {"workload": "workload1", "photons_per_step": 100_000_000, "volume": [60, 60, 60], "gates": 50,
                 "detectors": 4, "parallelism": "replicas1", "l2": "flushed before each timed step"}
    # the seed does not enter the description: the reference arm's steps use other seeds
    assert bench.workload_config("workload1", bench.make_cfg("workload1", 100_000_000, 5), 100_000_000, 1) == c
    c2 = bench.workload_config("workload2", bench.make_cfg("workload2", 1000, 1), 1000, 1)
    assert c2["volume"] == [256, 256, 256] and c2["detectors"] == 0 and c2["gates"] == 1
