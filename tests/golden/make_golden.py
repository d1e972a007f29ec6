"""Regenerate tests/golden/reference_goldens.json from the MCX reference tree.

Run in a checkout that has the reference project next to it:
    python tests/golden/make_golden.py /path/to/mcx
It extracts, as text, the golden values the reference's own tests assert for the transport
path and writes them with their source lines.  Nothing at test time reads the reference.
"""

from __future__ import annotations

import base64
import json
import re
import struct
import sys
import zlib
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _line_of(text: str, needle: str) -> int:
    for i, line in enumerate(text.splitlines(), 1):
        if needle in line:
            return i
    raise ValueError(f"{needle!r} not found")


def main(ref: Path) -> None:
    sh = (ref / "test" / "testmcx.sh").read_text()
    bench = (ref / "mcxlab" / "examples" / "mcx_gpu_benchmarks.m").read_text()

    # -D R test: the zlib+base64 payload of a 2x2x2 jnii file of xorshift128+ floats
    m = re.search(r"grep '(eJx[^']+)' testrng222\.jnii", sh)
    payload = m.group(1).replace("\\+", "+").replace("\\/", "/")
    raw = base64.b64decode(payload + "=" * (-len(payload) % 4))
    data = zlib.decompressobj().decompress(raw)
    floats = list(struct.unpack("<%df" % (len(data) // 4), data))

    out = {
        "rng_kat": {
            "source": f"test/testmcx.sh:{_line_of(sh, 'testrng222.jnii)')}",
            "payload": payload,
            "note": "jnii stores the 2x2x2 x 1-gate field in row-major order (z fastest); the generator "
                    "is seeded with four words (rand()<<16)|(rand()<<1)|(rand()>>14) taken from glibc rand() "
                    "before any srand() call (src/mcx_core.cu:3062-3066)",
            "values_rowmajor": floats,
        },
        "absorbed_fraction": [
            {"deck": "cube60", "nphoton": 1e6, "pattern": "17.x%", "lo": 0.17, "hi": 0.18,
             "source": f"test/testmcx.sh:{_line_of(sh, 'absorbed:.*17')}"},
            {"deck": "cube60b", "nphoton": 1e6, "pattern": "27.x%", "lo": 0.27, "hi": 0.28,
             "source": f"test/testmcx.sh:{_line_of(sh, 'cube60b -S 0')}"},
            {"deck": "cube60", "nphoton": 1e8, "value": 0.1769, "tol": 0.005,
             "source": f"mcxlab/examples/mcx_gpu_benchmarks.m:{_line_of(bench, '0.1769')}"},
            {"deck": "sphere60b", "nphoton": 1e8, "value": 0.2701, "tol": 0.005,
             "source": f"mcxlab/examples/mcx_gpu_benchmarks.m:{_line_of(bench, '0.2701')}"},
        ],
        "energy_total": {"rule": "|energytot - nphoton| <= 10",
                         "source": f"mcxlab/examples/mcx_gpu_benchmarks.m:{_line_of(bench, 'energytot - flux.stat.nphoton')}"},
        "detected": {"deck": "cube60b", "nphoton": 1e6, "pattern": "4[0-9]+ photons", "lo": 4000, "hi": 4999,
                     "source": f"test/testmcx.sh:{_line_of(sh, 'detected.*4[0-9]+ photons')}"},
        "boundary_detected": {"deck": "cube60", "bc": "______111111", "nphoton": 1e4, "pattern": "9[7-9][0-9.]+",
                              "lo": 9700, "hi": 9999,
                              "source": f"test/testmcx.sh:{_line_of(sh, '______111111')}"},
        "cyclic": {"deck": "cube60", "bc": "cccccc", "nphoton": 1e3, "pattern": "99.x%", "lo": 0.99, "hi": 1.0,
                   "source": f"test/testmcx.sh:{_line_of(sh, 'cccccc')}"},
        "reflect_bc": {"deck": "cube60", "bc": "aarraa", "isreflect": 0, "nphoton": 1e6, "pattern": "27.x%",
                       "lo": 0.27, "hi": 0.28, "source": f"test/testmcx.sh:{_line_of(sh, '-B aarraa')}"},
        # source shapes (test/testmcx.sh "test ... source" blocks): deck, overrides of its
        # Optode/Domain, the absorbed-fraction window the reference's test greps for
        "sources": [
            {"name": "planar", "deck": "cube60planar", "set": {}, "nphoton": 1e6, "pattern": "25.x%",
             "lo": 0.25, "hi": 0.26, "source": f"test/testmcx.sh:{_line_of(sh, 'cube60planar $PARAM')}"},
            {"name": "isotropic", "deck": "cube60", "set": {"srctype": "isotropic", "srcpos": [29, 29, 29]},
             "nosave": True, "nphoton": 1e6, "pattern": "88.x%", "lo": 0.88, "hi": 0.89,
             "source": f"test/testmcx.sh:{_line_of(sh, 'absorbed:.*88')}"},
            {"name": "cone", "deck": "cube60",
             "set": {"srctype": "cone", "srcparam1": [0.5, 0, 0, 0], "prop": [[0, 0, 1, 1], [0.001, 0.001, 0, 1]]},
             "nosave": True, "nphoton": 1e6, "pattern": "6.x%", "lo": 0.06, "hi": 0.07,
             "source": f"test/testmcx.sh:{_line_of(sh, 'absorbed:.*6')}"},
            {"name": "fourier", "deck": "cube60planar", "set": {"srctype": "fourier", "srcparam1": [40, 0, 0, 2]},
             "nosave": True, "nphoton": 1e6, "pattern": "25.x%", "lo": 0.25, "hi": 0.26,
             "source": f"test/testmcx.sh:{_line_of(sh, 'fourier')}"},
            {"name": "pencilarray", "deck": "cube60planar",
             "set": {"srctype": "pencilarray", "srcparam1": [40, 0, 0, 4], "srcparam2": [0, 20, 0, 2]},
             "nosave": True, "nphoton": 1e6, "pattern": "23.x%", "lo": 0.23, "hi": 0.24,
             "source": f"test/testmcx.sh:{_line_of(sh, 'pencilarray')}"},
        ],
    }
    (HERE / "reference_goldens.json").write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", HERE / "reference_goldens.json")


if __name__ == "__main__":
    import os

    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MCX_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <MCX checkout> (or set MCX_REFERENCE_ROOT)")
    main(Path(root))
