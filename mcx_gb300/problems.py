"""Input decks: MCX's built-in cube benchmarks and the engine's three plain-MC workloads.

``cube60`` / ``cube60b`` restate the built-in benchmarks of src/mcx_bench.c:47-152 (the decks the
reference's regression tests and speed contest run).  ``workload0..2`` are the homogeneous,
heterogeneous-with-detectors and large layered workloads the engine is benchmarked on; they are
synthetic and fully determined by their seed.
"""

from __future__ import annotations

import numpy as np

CUBE60_SEED = 1648335518      # RNGSeed of the cube60 decks, src/mcx_bench.c:50
CUBE60_DETECTORS = [[29.0, 19.0, 0.0, 1.0], [29.0, 39.0, 0.0, 1.0], [19.0, 29.0, 0.0, 1.0], [39.0, 29.0, 0.0, 1.0]]


def _cube60(nphoton: float, mismatch: bool, n_medium2: float) -> dict:
    return {
        "nphoton": int(nphoton),
        "seed": CUBE60_SEED,
        "vol": np.ones((60, 60, 60), dtype=np.uint8),
        "prop": np.array([[0.0, 0.0, 1.0, 1.0], [0.005, 1.0, 0.01, 1.37], [0.002, 5.0, 0.90, n_medium2]], np.float32),
        "tstart": 0.0, "tend": 5e-9, "tstep": 5e-9,
        "srcpos": [29.0, 29.0, 0.0], "srcdir": [0.0, 0.0, 1.0],
        "detpos": np.array(CUBE60_DETECTORS, np.float32),
        "issrcfrom0": 1,
        "isreflect": 1 if mismatch else 0,
        "issavedet": 1,
    }


def cube60(nphoton: float = 1e6) -> dict:
    """Homogeneous 60^3 cube, no reflection (src/mcx_bench.c:47-101)."""
    return _cube60(nphoton, False, 1.37)


def cube60b(nphoton: float = 1e6) -> dict:
    """The same cube with Fresnel reflection at the outer boundary (src/mcx_bench.c:104-152)."""
    return _cube60(nphoton, True, 1.0)


def cube60planar(nphoton: float = 1e6) -> dict:
    """The cube with reflection and a 40 x 40 planar source 10 mm in front of the z=0 face
    (src/mcx_bench.c:155-215); every photon crosses the void before it enters."""
    cfg = _cube60(nphoton, True, 1.0)
    cfg.update(srctype="planar", srcpos=[10.0, 10.0, -10.0], srcdir=[0.0, 0.0, 1.0],
               srcparam1=[40.0, 0.0, 0.0, 0.0], srcparam2=[0.0, 40.0, 0.0, 0.0])
    return cfg


def sphere60b(nphoton: float = 1e6) -> dict:
    """cube60 plus a label-2 sphere (R=15 at (30,30,30), medium 2 = (0.002, 5.0, 0.9, 1.0)) with
    reflection on: the second deck of MCX's speed benchmark (mcxlab/examples/mcx_gpu_benchmarks.m:47-87)."""
    cfg = _cube60(nphoton, True, 1.0)
    cfg["seed"] = 29012392
    sphere_labels((60, 60, 60), (30.0, 30.0, 30.0), 15.0, 2, cfg["vol"])
    return cfg


def shared_patterns(nphoton: float = 1e6) -> dict:
    """cube60's medium lit by a 40 x 40 mm pattern source of 16 x 16 pixels carrying two
    patterns at once (photon sharing, srcnum = 2): the left half of the field, and a linear ramp
    along y.  ``srcpattern`` is (srcnum, 16, 16), patterns adjacent per pixel as MCX stores them."""
    a = np.zeros((16, 16), np.float32)
    a[:8, :] = 1.0
    b = np.tile(np.linspace(0.1, 1.0, 16, dtype=np.float32)[None, :], (16, 1))
    cfg = _cube60(nphoton, False, 1.37)
    cfg.pop("detpos")
    cfg.update(issavedet=0, srctype="pattern", srcpos=[10.0, 10.0, 0.0], srcdir=[0.0, 0.0, 1.0],
               srcparam1=[40.0, 0.0, 0.0, 16.0], srcparam2=[0.0, 40.0, 0.0, 16.0], srcnum=2,
               srcpattern=np.stack([a, b]))
    return cfg


def reflectance_cube(nphoton: float = 1e6) -> dict:
    """cube60's medium inside a one-voxel void shell (62^3 grid), a pencil beam entering at the
    centre of the z = 1 face, no reflection, a 100 ns window: every photon that leaves the medium
    ends in a void voxel of the grid, where the diffuse-reflectance output (issaveref) records it."""
    vol = np.zeros((62, 62, 62), dtype=np.uint8)
    vol[1:-1, 1:-1, 1:-1] = 1
    return {
        "nphoton": int(nphoton), "seed": CUBE60_SEED, "vol": vol,
        "prop": np.array([[0.0, 0.0, 1.0, 1.0], [0.005, 1.0, 0.01, 1.37]], np.float32),
        "tstart": 0.0, "tend": 1e-7, "tstep": 1e-7,
        "srcpos": [31.0, 31.0, 1.0], "srcdir": [0.0, 0.0, 1.0], "issrcfrom0": 1,
        "isreflect": 0, "issaveref": 1,
    }


def polarized_slab(nphoton: float = 1e6) -> dict:
    """A 10 x 10 x 1.2 mm slab (100 x 100 x 12 voxels of 0.1 mm) of small polystyrene spheres in
    water with a sphere of large ones at (6, 6, 0.6) mm, lit by a horizontally polarised planar
    beam at 632.8 nm; photons leaving through z = 0 are detected with their Stokes vectors.  The
    polarised-light deck of mcxlab/examples/demo_polarized_photon.m (sphere populations
    mua (1/mm), radius (um), density (1/um^3), n_sphere, n_water)."""
    dim = (100, 100, 12)
    vol = np.ones(dim, dtype=np.uint8)
    x, y, z = np.meshgrid(*(np.arange(n) + 0.5 for n in dim), indexing="ij")
    vol[(x - 60) ** 2 + (y - 60) ** 2 + (z - 6) ** 2 < 25] = 2
    return {
        "nphoton": int(nphoton), "seed": 1648335518, "vol": vol, "unitinmm": 0.1,
        "polprop": np.array([[0.005, 0.05, 19.1142, 1.59, 1.33], [0.005, 1.0, 1.11078e-3, 1.59, 1.33]], np.float32),
        "prop": np.array([[0, 0, 1, 1], [0, 0, 1, 1], [0, 0, 1, 1]], np.float32),
        "srctype": "planar", "srcpos": [0.0, 0.0, 0.0], "srcdir": [0.0, 0.0, 1.0],
        "srcparam1": [100.0, 0.0, 0.0, 0.0], "srcparam2": [0.0, 100.0, 0.0, 0.0],
        "srciquv": [1.0, 1.0, 0.0, 0.0], "lambda": 632.8, "issrcfrom0": 1,
        "tstart": 0.0, "tend": 5e-8, "tstep": 5e-8, "isreflect": 0,
        "savedetflag": "ixvw", "bc": "cc_cc_001000", "issavedet": 1, "maxdetphoton": int(nphoton),
    }


def rotated_stokes(detp: np.ndarray, nmedia: int, unitinmm: float, mua: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Stokes vectors of detected photons in the detector frame and their weights, from records of
    (ppath x nmedia, exit position, exit direction, w0, I, Q, U, V) columns: Q and U are rotated by
    twice the azimuth of the exit direction, and the weight is w0 exp(-sum mua ppath)
    (mcxlab/examples/demo_polarized_photon.m, utils/mcxdetweight.m)."""
    pp = detp[:nmedia]
    v = detp[nmedia + 3:nmedia + 6]
    w0 = detp[nmedia + 6]
    s = detp[nmedia + 7:nmedia + 11]
    phi = np.arctan2(v[1], v[0])
    c2, s2 = np.cos(2 * phi), np.sin(2 * phi)
    st = np.stack([s[0], s[1] * c2 + s[2] * s2, -s[1] * s2 + s[2] * c2, s[3]])
    w = w0 * np.exp(-(np.asarray(mua, np.float64)[:, None] * pp).sum(0) * unitinmm)
    return st, w


def source_deck(g: dict, nphoton: float | None = None) -> dict:
    """The deck of a source-shape golden entry: its base deck with the entry's overrides."""
    cfg = {"cube60": cube60, "cube60planar": cube60planar}[g["deck"]](nphoton or g["nphoton"])
    for k, v in g["set"].items():
        cfg[k] = np.array(v, np.float32) if k == "prop" else v
    if g.get("nosave"):
        cfg.pop("detpos", None)
        cfg["issavedet"] = 0
    return cfg


def sphere_labels(dim: tuple[int, int, int], center, radius: float, tag: int, vol: np.ndarray) -> np.ndarray:
    """Rasterise a sphere: voxel centres (i + 0.5) within `radius` of `center` get `tag`
    (the rule of MCX's shape rasteriser, src/mcx_shapes.c:237-289)."""
    ii = np.arange(dim[0], dtype=np.float32)[:, None, None] + 0.5 - center[0]
    jj = np.arange(dim[1], dtype=np.float32)[None, :, None] + 0.5 - center[1]
    kk = np.arange(dim[2], dtype=np.float32)[None, None, :] + 0.5 - center[2]
    mask = ii * ii + jj * jj + kk * kk <= np.float32(radius) * np.float32(radius)
    vol[mask] = tag
    return vol


def workload0(nphoton: float = 1e6, seed: int = CUBE60_SEED) -> dict:
    """Plain MC, homogeneous 60^3 cube: medium 1 (mua 0.005, mus 1.0, g 0.01, n 1.37) in a
    background (0, 0, 1, 1); pencil at voxel (29,29,0) along +z; one 0-5 ns gate; no
    reflection; float32 flux."""
    return {
        "nphoton": int(nphoton), "seed": seed,
        "vol": np.ones((60, 60, 60), dtype=np.uint8),
        "prop": np.array([[0.0, 0.0, 1.0, 1.0], [0.005, 1.0, 0.01, 1.37]], np.float32),
        "tstart": 0.0, "tend": 5e-9, "tstep": 5e-9,
        "srcpos": [29.0, 29.0, 0.0], "srcdir": [0.0, 0.0, 1.0],
        "issrcfrom0": 1, "isreflect": 0, "issavedet": 0,
    }


def workload1(nphoton: float = 1e8, seed: int = CUBE60_SEED) -> dict:
    """Plain MC, heterogeneous: the cube plus a label-2 sphere of radius 15 voxels centred at
    (30,30,30) (mua 0.002, mus 5.0, g 0.9, n 1.37); Fresnel reflection against n=1 outside;
    50 gates of 0.1 ns; four disk detectors of radius 1 on z=0 at 5/10/15/20 mm from the
    source, saving detector id, per-medium scattering counts and partial path lengths."""
    vol = np.ones((60, 60, 60), dtype=np.uint8)
    sphere_labels((60, 60, 60), (30.0, 30.0, 30.0), 15.0, 2, vol)
    det = np.array([[29.0 + d, 29.0, 0.0, 1.0] for d in (5, 10, 15, 20)], np.float32)
    return {
        "nphoton": int(nphoton), "seed": seed, "vol": vol,
        "prop": np.array([[0.0, 0.0, 1.0, 1.0], [0.005, 1.0, 0.01, 1.37], [0.002, 5.0, 0.9, 1.37]], np.float32),
        "tstart": 0.0, "tend": 5e-9, "tstep": 1e-10,
        "srcpos": [29.0, 29.0, 0.0], "srcdir": [0.0, 0.0, 1.0],
        "detpos": det, "issrcfrom0": 1, "isreflect": 1, "issavedet": 1, "savedetflag": "dsp",
        "maxdetphoton": 2000000,
    }


LAYERED_PROPS = np.array([
    [0.0, 0.0, 1.0, 1.0],
    [0.019, 7.8, 0.89, 1.37],
    [0.016, 16.0, 0.90, 1.37],
    [0.004, 0.01, 0.90, 1.37],
    [0.020, 9.0, 0.89, 1.37],
    [0.080, 40.9, 0.84, 1.37],
], np.float32)


def layered_volume(n: int = 256, seed: int = 20251203) -> np.ndarray:
    """Five nested axis-aligned ellipsoid shells centred near the middle of an n^3 grid, label 1
    outermost to 5 innermost; semi-axes drawn from `seed`, each shell 72-88% of the previous."""
    rng = np.random.default_rng(seed)
    vol = np.zeros((n, n, n), dtype=np.uint8)
    c = np.array([n / 2.0, n / 2.0, n / 2.0]) + rng.uniform(-2.0, 2.0, 3)
    axes = np.array([0.46 * n, 0.44 * n, 0.42 * n]) * rng.uniform(0.95, 1.0, 3)
    x = np.arange(n, dtype=np.float32) + 0.5
    dx2 = (x - c[0]) ** 2
    dy2 = (x - c[1]) ** 2
    dz2 = (x - c[2]) ** 2
    for label in range(1, 6):
        a = axes.astype(np.float32)
        inside = (dx2[:, None, None] / a[0] ** 2 + dy2[None, :, None] / a[1] ** 2 + dz2[None, None, :] / a[2] ** 2) <= 1.0
        vol[inside] = label
        axes = axes * rng.uniform(0.72, 0.88, 3)
    return vol


def workload2(nphoton: float = 1e9, seed: int = CUBE60_SEED, n: int = 256) -> dict:
    """Plain MC, large layered volume: 256^3 nested ellipsoid shells (props above, n=1.37),
    pencil beam launched from outside along +z through the volume centre line, normal to the
    outer surface; one 0-5 ns gate; Fresnel reflection against n=1; float32 flux (64 MB)."""
    vol = layered_volume(n)
    return {
        "nphoton": int(nphoton), "seed": seed, "vol": vol, "prop": LAYERED_PROPS.copy(),
        "tstart": 0.0, "tend": 5e-9, "tstep": 5e-9,
        "srcpos": [n / 2.0, n / 2.0, 0.0], "srcdir": [0.0, 0.0, 1.0],
        "issrcfrom0": 1, "isreflect": 1, "issavedet": 0,
    }


WORKLOADS = {"workload0": workload0, "workload1": workload1, "workload2": workload2}


BATCH_EDGES = (32, 48, 64, 96, 128)


def batch_instances(count: int = 256, seed: int = 20251204, budget_scale: float = 1.0) -> list[dict]:
    """The batched workload: `count` independent simulations drawn from one master seed.

    Each instance: a cube of edge uniform over {32, 48, 64, 96, 128} voxels (1 mm) of medium 1
    with 1-4 random axis-aligned ellipsoids (labels 2..5, later ones overwrite earlier ones); every
    medium has mua log-uniform in [1e-3, 5e-2]/mm, mus uniform in [0.5, 20]/mm, g uniform in
    [0.7, 0.95] and n = 1.37 (background n = 1, Fresnel reflection on); a photon budget
    log-uniform in [1e6, 1e8] (times `budget_scale`); a pencil source entering the z = 0 face
    along +z at a random point of its central half; two radius-1 detectors on that face 5 and
    10 mm from the source (detector id and per-medium partial paths saved); one 0-5 ns gate."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.choice(BATCH_EDGES))
        vol = np.ones((n, n, n), dtype=np.uint8)
        nell = int(rng.integers(1, 5))
        idx = np.arange(n, dtype=np.float32) + 0.5
        for e in range(nell):
            c = rng.uniform(0.2 * n, 0.8 * n, 3)
            r = rng.uniform(0.08 * n, 0.3 * n, 3)
            X, Y, Z = np.meshgrid((idx - c[0]) / r[0], (idx - c[1]) / r[1], (idx - c[2]) / r[2], indexing="ij")
            vol[X * X + Y * Y + Z * Z <= 1.0] = 2 + e
        nmed = 1 + nell
        prop = np.zeros((nmed + 1, 4), np.float32)
        prop[0] = [0.0, 0.0, 1.0, 1.0]
        for m in range(1, nmed + 1):
            prop[m] = [np.exp(rng.uniform(np.log(1e-3), np.log(5e-2))), rng.uniform(0.5, 20.0),
                       rng.uniform(0.7, 0.95), 1.37]
        budget = float(np.exp(rng.uniform(np.log(1e6), np.log(1e8)))) * budget_scale
        sx, sy = (float(np.floor(v)) for v in rng.uniform(0.25 * n, 0.75 * n, 2))
        ang = rng.uniform(0, 2 * np.pi)
        det = [[sx + d * np.cos(ang), sy + d * np.sin(ang), 0.0, 1.0] for d in (5.0, 10.0)]
        out.append({
            "nphoton": max(1, int(budget)), "seed": int(rng.integers(1, 2**31 - 1)),
            "vol": vol, "prop": prop,
            "tstart": 0.0, "tend": 5e-9, "tstep": 5e-9,
            "srcpos": [sx, sy, 0.0], "srcdir": [0.0, 0.0, 1.0], "issrcfrom0": 1,
            "isreflect": 1, "issavedet": 1, "savedetflag": "dp", "detpos": np.array(det, np.float32),
            "maxdetphoton": max(1000, int(budget * 0.005)),
        })
    return out


def denoise_instances(count: int, edge: int, seed: int, nphoton: float = 1e6) -> list[dict]:
    """Volumes for the fluence denoiser, drawn from the batched workload's property ranges: a cube
    of `edge` voxels (1 mm) of medium 1 with 1-4 random axis-aligned ellipsoids (labels 2..5),
    every medium with mua log-uniform in [1e-3, 5e-2]/mm, mus uniform in [0.5, 20]/mm, g uniform
    in [0.7, 0.95], n = 1.37 (background n = 1, Fresnel reflection on); a pencil source entering
    the z = 0 face along +z at a random point of its central half; one 0-5 ns gate; no detectors.
    The same (count, edge, seed) gives the same volumes; `nphoton` and the per-run seed are the
    caller's to change (the training pairs reuse one volume at several photon counts)."""
    rng = np.random.default_rng(seed)
    out = []
    idx = np.arange(edge, dtype=np.float32) + 0.5
    for i in range(count):
        vol = np.ones((edge, edge, edge), dtype=np.uint8)
        nell = int(rng.integers(1, 5))
        for e in range(nell):
            c = rng.uniform(0.2 * edge, 0.8 * edge, 3)
            r = rng.uniform(0.08 * edge, 0.3 * edge, 3)
            X, Y, Z = np.meshgrid((idx - c[0]) / r[0], (idx - c[1]) / r[1], (idx - c[2]) / r[2], indexing="ij")
            vol[X * X + Y * Y + Z * Z <= 1.0] = 2 + e
        prop = np.zeros((nell + 2, 4), np.float32)
        prop[0] = [0.0, 0.0, 1.0, 1.0]
        for m in range(1, nell + 2):
            prop[m] = [np.exp(rng.uniform(np.log(1e-3), np.log(5e-2))), rng.uniform(0.5, 20.0),
                       rng.uniform(0.7, 0.95), 1.37]
        sx, sy = (float(np.floor(v)) for v in rng.uniform(0.25 * edge, 0.75 * edge, 2))
        out.append({
            "nphoton": int(nphoton), "seed": int(rng.integers(1, 2**31 - 1)), "vol": vol, "prop": prop,
            "tstart": 0.0, "tend": 5e-9, "tstep": 5e-9,
            "srcpos": [sx, sy, 0.0], "srcdir": [0.0, 0.0, 1.0], "issrcfrom0": 1,
            "isreflect": 1, "issavedet": 0,
        })
    return out
