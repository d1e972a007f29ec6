"""MC + learned denoiser: a 4-level 3D U-Net that maps low-photon fluence to high-photon fluence.

The network works on log10 fluence: its input features are the 3x3x3 neighbourhood mean of the
noisy map and the deviations of the map and of its 5x5x5 mean from it (means taken in linear
fluence, so that voxels no photon reached do not become log-space outliers), an empty-voxel flag,
the voxel's absorption and reduced scattering coefficients and the photon count
(``mcxg_dn_pack``); 3x3x3 convolutions with ReLU at 16/32/64/128 channels, 2x2x2 average
pooling, nearest upsampling with skip concatenation, and a 1x1x1 head whose output is added to
the log of the 3x3x3 mean (the network learns a correction to a box filter; at initialisation it
is nearly that filter).

Everything on the device runs on this engine's own kernels (include/mcxg_denoise.h): BF16
tensor-core implicit-GEMM convolutions forward, data and weight gradient, pooling, upsampling,
the fused head + masked-L1 loss, and AdamW on fp32 master weights.  PyTorch only owns device
memory and the stream.  Training pairs come from the engine itself (``make_pairs``): the same
volume simulated at 1e5 / 1e6 photons (inputs) and at a high photon count (target).

The MC stays the judge: ``time_to_error_batch`` reports how long plain MC needs to reach a given
median relative fluence error against a high-photon run, and how long MC + denoiser needs, with
plain MC as the fallback wherever the denoised map does not reach it; both run through
``pipeline_maps`` (the batched MC with its fields kept on the device, the network on the device,
one copy of every final map to the host).
"""

from __future__ import annotations

import math
import time
from pathlib import Path
from typing import Any

import numpy as np
import torch

from . import problems
from ._lib import lib

# (name, input channels, output channels, level): level l runs at 1/2^l of the input grid
LAYERS = [
    ("enc1a", 16, 16, 0), ("enc1b", 16, 16, 0),
    ("enc2a", 16, 32, 1), ("enc2b", 32, 32, 1),
    ("enc3a", 32, 64, 2), ("enc3b", 64, 64, 2),
    ("bota", 64, 128, 3), ("botb", 128, 128, 3),
    ("dec3a", 192, 64, 2), ("dec3b", 64, 64, 2),
    ("dec2a", 96, 32, 1), ("dec2b", 32, 32, 1),
    ("dec1a", 48, 16, 0), ("dec1b", 16, 16, 0),
]
SPEC = {name: (cin, cout, lvl) for name, cin, cout, lvl in LAYERS}
IN_CH = 16
TAPS = 27
FLUX_FLOOR = 1e-10          # log10(F + FLUX_FLOOR) is the network's fluence coordinate
VALID_FRAC = 1e-6           # voxels at or above this fraction of the reference map's maximum are scored
DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "denoiser_unet64.npz"


def init_params(seed: int = 0) -> dict[str, np.ndarray]:
    """He-normal convolution weights [cout, 27, cin], zero biases, a small random head."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, cin, cout, _ in LAYERS:
        p[name + ".w"] = (rng.standard_normal((cout, TAPS, cin)) * math.sqrt(2.0 / (TAPS * cin))).astype(np.float32)
        p[name + ".b"] = np.zeros(cout, np.float32)
    p["head.w"] = (rng.standard_normal(16) * 0.01).astype(np.float32)
    p["head.b"] = np.zeros(1, np.float32)
    return p


def load_params(path: str | Path = DEFAULT_WEIGHTS) -> dict[str, np.ndarray]:
    with np.load(path) as z:
        return {k: z[k].astype(np.float32) for k in z.files}


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _ok(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what}: {lib.mcxg_dn_last_error().decode()} ({rc})")


class UNet:
    """The denoiser on one GPU: fp32 master weights, bf16 copies (and the flipped transposed copies
    the data gradient runs on), Adam moments, gradients and cached activation buffers."""

    def __init__(self, params: dict[str, np.ndarray] | None = None, seed: int = 0, device: str = "cuda"):
        if not torch.cuda.is_available():
            raise RuntimeError("the denoiser runs on the GPU only")
        self.dev = torch.device(device)
        params = params if params is not None else init_params(seed)
        self.t: dict[str, dict[str, torch.Tensor]] = {}
        f32 = dict(dtype=torch.float32, device=self.dev)
        for name, cin, cout, _ in LAYERS:
            w = torch.from_numpy(np.ascontiguousarray(params[name + ".w"], np.float32).reshape(-1)).to(self.dev)
            b = torch.from_numpy(np.ascontiguousarray(params[name + ".b"], np.float32)).to(self.dev)
            self.t[name] = {
                "w": w, "b": b, "gw": torch.zeros_like(w), "gb": torch.zeros_like(b),
                "mw": torch.zeros_like(w), "vw": torch.zeros_like(w), "mb": torch.zeros_like(b), "vb": torch.zeros_like(b),
                "w16": torch.empty(w.numel(), dtype=torch.bfloat16, device=self.dev),
                "wt16": torch.empty(w.numel(), dtype=torch.bfloat16, device=self.dev),
            }
        hw = torch.from_numpy(np.ascontiguousarray(params["head.w"], np.float32)).to(self.dev)
        hb = torch.from_numpy(np.ascontiguousarray(params["head.b"], np.float32)).to(self.dev)
        self.t["head"] = {"w": hw, "b": hb, "gw": torch.zeros_like(hw), "gb": torch.zeros_like(hb),
                          "mw": torch.zeros_like(hw), "vw": torch.zeros_like(hw), "mb": torch.zeros_like(hb),
                          "vb": torch.zeros_like(hb)}
        self.loss_acc = torch.zeros(1, **f32)
        self.step_count = 0
        self._bufs: dict[tuple, torch.Tensor] = {}
        self.refresh_bf16()

    # -- parameters ---------------------------------------------------------------------------
    def refresh_bf16(self) -> None:
        """bf16 weights and transposed copies from the masters (an AdamW step with lr 0 and the
        gradient left untouched would do the same; this keeps the moments as they are)."""
        s = self._stream()
        for name, cin, cout, _ in LAYERS:
            t = self.t[name]
            g = t["gw"].clone()
            m1, m2 = t["mw"].clone(), t["vw"].clone()
            _ok(lib.mcxg_dn_adamw(_ptr(t["w"]), _ptr(g), _ptr(m1), _ptr(m2), _ptr(t["w16"]), _ptr(t["wt16"]),
                                  t["w"].numel(), cout, TAPS, cin, 0.0, 0.9, 0.999, 1e-8, 0.0, 1, s), "weights")

    def params(self) -> dict[str, np.ndarray]:
        p = {}
        for name, cin, cout, _ in LAYERS:
            p[name + ".w"] = self.t[name]["w"].cpu().numpy().reshape(cout, TAPS, cin)
            p[name + ".b"] = self.t[name]["b"].cpu().numpy()
        p["head.w"] = self.t["head"]["w"].cpu().numpy()
        p["head.b"] = self.t["head"]["b"].cpu().numpy()
        return p

    def grads(self) -> dict[str, np.ndarray]:
        g = {}
        for name, cin, cout, _ in LAYERS:
            g[name + ".w"] = self.t[name]["gw"].cpu().numpy().reshape(cout, TAPS, cin)
            g[name + ".b"] = self.t[name]["gb"].cpu().numpy()
        g["head.w"] = self.t["head"]["gw"].cpu().numpy()
        g["head.b"] = self.t["head"]["gb"].cpu().numpy()
        return g

    def zero_grad(self) -> None:
        for t in self.t.values():
            t["gw"].zero_()
            t["gb"].zero_()

    def save(self, path: str | Path) -> None:
        np.savez_compressed(path, **self.params())

    # -- plumbing -----------------------------------------------------------------------------
    @staticmethod
    def _stream() -> int:
        return torch.cuda.current_stream().cuda_stream

    def _buf(self, key: str, n: int, dtype=torch.bfloat16) -> torch.Tensor:
        k = (key, n, dtype)
        b = self._bufs.get(k)
        if b is None:
            b = torch.empty(n, dtype=dtype, device=self.dev)
            self._bufs[k] = b
        return b

    def _conv(self, name: str, x: torch.Tensor, y: torch.Tensor, geo: tuple, mask=None, transposed=False) -> None:
        cin, cout, _ = SPEC[name]
        t = self.t[name]
        if transposed:   # data gradient: channels swap, no bias, no ReLU, times the mask
            _ok(lib.mcxg_dn_conv_fwd(_ptr(x), _ptr(t["wt16"]), None, _ptr(mask), _ptr(y), *geo, cout, cin, TAPS, 0,
                                     self._stream()), name + " data gradient")
        else:
            _ok(lib.mcxg_dn_conv_fwd(_ptr(x), _ptr(t["w16"]), _ptr(t["b"]), None, _ptr(y), *geo, cin, cout, TAPS, 1,
                                     self._stream()), name)

    # -- forward / backward -------------------------------------------------------------------
    def pack(self, flux: torch.Tensor, labels: torch.Tensor, props: torch.Tensor, log_photons: torch.Tensor,
             d: int, h: int, w: int):
        """Input features and residual base of nvol volumes of d x h x w voxels: flux fp32
        [nvol, vox], labels uint8 [nvol, vox], props fp32 [nvol, nprop, 4], log_photons fp32
        [nvol]."""
        nvol, vox = flux.shape
        if vox != d * h * w:
            raise ValueError("flux does not hold d * h * w voxels per volume")
        x0 = self._buf("x0", nvol * vox * IN_CH)
        xres = self._buf("xres", nvol * vox, torch.float32)
        _ok(lib.mcxg_dn_pack(_ptr(flux), _ptr(labels), _ptr(props), _ptr(log_photons), _ptr(x0), _ptr(xres), nvol, d, h,
                             w, props.shape[1], self._stream()), "pack")
        return x0, xres

    def forward(self, x0: torch.Tensor, xres: torch.Tensor, nvol: int, d: int, h: int, w: int,
                out: torch.Tensor | None = None) -> dict[str, torch.Tensor]:
        """Runs the network; returns the activations (kept for ``backward``) and, when `out` is
        given, writes the predicted log10 fluence there."""
        if d % 8 or h % 8 or w % 8:
            raise ValueError("the U-Net needs grid sizes divisible by 8")
        geo = [(nvol, d >> l, h >> l, w >> l) for l in range(4)]
        vox = [nvol * (d >> l) * (h >> l) * (w >> l) for l in range(4)]
        s = self._stream()
        A: dict[str, torch.Tensor] = {"x0": x0, "xres": xres}

        def conv(name, src, dst):
            cin, cout, lvl = SPEC[name]
            A[dst] = self._buf(dst, vox[lvl] * cout)
            self._conv(name, A[src], A[dst], geo[lvl])

        def pool(src, dst, lvl, c):
            A[dst] = self._buf(dst, vox[lvl + 1] * c)
            _ok(lib.mcxg_dn_pool(_ptr(A[src]), _ptr(A[dst]), *geo[lvl], c, s), "pool")

        def upcat(low, skip, dst, lvl, c1, c2):
            A[dst] = self._buf(dst, vox[lvl] * (c1 + c2))
            _ok(lib.mcxg_dn_upcat(_ptr(A[low]), _ptr(A[skip]), _ptr(A[dst]), *geo[lvl], c1, c2, s), "upcat")

        conv("enc1a", "x0", "e1a"); conv("enc1b", "e1a", "e1"); pool("e1", "p1", 0, 16)
        conv("enc2a", "p1", "e2a"); conv("enc2b", "e2a", "e2"); pool("e2", "p2", 1, 32)
        conv("enc3a", "p2", "e3a"); conv("enc3b", "e3a", "e3"); pool("e3", "p3", 2, 64)
        conv("bota", "p3", "e4a"); conv("botb", "e4a", "e4")
        upcat("e4", "e3", "c3", 2, 128, 64)
        conv("dec3a", "c3", "d3a"); conv("dec3b", "d3a", "d3")
        upcat("d3", "e2", "c2", 1, 64, 32)
        conv("dec2a", "c2", "d2a"); conv("dec2b", "d2a", "d2")
        upcat("d2", "e1", "c1", 0, 32, 16)
        conv("dec1a", "c1", "d1a"); conv("dec1b", "d1a", "d1")
        if out is not None:
            hd = self.t["head"]
            _ok(lib.mcxg_dn_head(_ptr(A["d1"]), _ptr(xres), _ptr(hd["w"]), _ptr(hd["b"]), None, None, _ptr(out), None,
                                 None, None, None, vox[0], 0.0, s), "head")
        A["_geo"] = geo
        A["_vox"] = vox
        return A

    def backward(self, A: dict, target: torch.Tensor, valid: torch.Tensor, inv_count: float) -> None:
        """Masked L1 loss of the predicted log-fluence against `target` (weights `valid`, scaled by
        inv_count) and the gradients of every parameter, accumulated into the fp32 gradients."""
        geo, vox = A["_geo"], A["_vox"]
        s = self._stream()
        hd = self.t["head"]
        G: dict[str, torch.Tensor] = {}
        G["d1"] = self._buf("g_d1", vox[0] * 16)
        _ok(lib.mcxg_dn_head(_ptr(A["d1"]), _ptr(A["xres"]), _ptr(hd["w"]), _ptr(hd["b"]), _ptr(target), _ptr(valid),
                             None, _ptr(G["d1"]), _ptr(hd["gw"]), _ptr(hd["gb"]), _ptr(self.loss_acc), vox[0],
                             float(inv_count), s), "head backward")

        def layer(name, gout, inp, gin=None, mask=None):
            cin, cout, lvl = SPEC[name]
            t = self.t[name]
            _ok(lib.mcxg_dn_conv_wgrad(_ptr(G[gout]), _ptr(A[inp]), _ptr(t["gw"]), *geo[lvl], cin, cout, TAPS, s),
                name + " weight gradient")
            _ok(lib.mcxg_dn_bias_grad(_ptr(G[gout]), _ptr(t["gb"]), vox[lvl], cout, s), name + " bias gradient")
            if gin is not None:
                G[gin] = self._buf("g_" + gin, vox[lvl] * cin)
                self._conv(name, G[gout], G[gin], geo[lvl], mask=None if mask is None else A[mask], transposed=True)

        def upcat_bwd(gcat, low, glow, lvl, c1, c2):
            G[glow] = self._buf("g_" + glow, vox[lvl + 1] * c1)
            _ok(lib.mcxg_dn_upcat_bwd(_ptr(G[gcat]), _ptr(A[low]), _ptr(G[glow]), *geo[lvl], c1, c2, s), "upcat backward")

        def unpool(gpool, gcat, enc, genc, lvl, c1, c):
            G[genc] = self._buf("g_" + genc, vox[lvl] * c)
            _ok(lib.mcxg_dn_unpool_add(_ptr(G[gpool]), _ptr(G[gcat]), _ptr(A[enc]), _ptr(G[genc]), *geo[lvl], c1, c, s),
                "unpool")

        layer("dec1b", "d1", "d1a", "d1a", "d1a")
        layer("dec1a", "d1a", "c1", "c1", "c1")
        upcat_bwd("c1", "d2", "d2", 0, 32, 16)
        layer("dec2b", "d2", "d2a", "d2a", "d2a")
        layer("dec2a", "d2a", "c2", "c2", "c2")
        upcat_bwd("c2", "d3", "d3", 1, 64, 32)
        layer("dec3b", "d3", "d3a", "d3a", "d3a")
        layer("dec3a", "d3a", "c3", "c3", "c3")
        upcat_bwd("c3", "e4", "e4", 2, 128, 64)
        layer("botb", "e4", "e4a", "e4a", "e4a")
        layer("bota", "e4a", "p3", "p3", None)
        unpool("p3", "c3", "e3", "e3", 2, 128, 64)
        layer("enc3b", "e3", "e3a", "e3a", "e3a")
        layer("enc3a", "e3a", "p2", "p2", None)
        unpool("p2", "c2", "e2", "e2", 1, 64, 32)
        layer("enc2b", "e2", "e2a", "e2a", "e2a")
        layer("enc2a", "e2a", "p1", "p1", None)
        unpool("p1", "c1", "e1", "e1", 0, 32, 16)
        layer("enc1b", "e1", "e1a", "e1a", "e1a")
        layer("enc1a", "e1a", "x0")

    def step(self, lr: float, weight_decay: float = 1e-4, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
        """AdamW on every parameter (no decay on biases and the head); clears the gradients."""
        self.step_count += 1
        s = self._stream()
        k = self.step_count
        for name, cin, cout, _ in LAYERS:
            t = self.t[name]
            _ok(lib.mcxg_dn_adamw(_ptr(t["w"]), _ptr(t["gw"]), _ptr(t["mw"]), _ptr(t["vw"]), _ptr(t["w16"]),
                                  _ptr(t["wt16"]), t["w"].numel(), cout, TAPS, cin, lr, b1, b2, eps, weight_decay, k, s),
                name + " AdamW")
            _ok(lib.mcxg_dn_adamw(_ptr(t["b"]), _ptr(t["gb"]), _ptr(t["mb"]), _ptr(t["vb"]), None, None, cout, 0, 0, 0,
                                  lr, b1, b2, eps, 0.0, k, s), name + " bias AdamW")
        hd = self.t["head"]
        _ok(lib.mcxg_dn_adamw(_ptr(hd["w"]), _ptr(hd["gw"]), _ptr(hd["mw"]), _ptr(hd["vw"]), None, None, 16, 0, 0, 0, lr,
                              b1, b2, eps, 0.0, k, s), "head AdamW")
        _ok(lib.mcxg_dn_adamw(_ptr(hd["b"]), _ptr(hd["gb"]), _ptr(hd["mb"]), _ptr(hd["vb"]), None, None, 1, 0, 0, 0, lr,
                              b1, b2, eps, 0.0, k, s), "head AdamW")

    # -- inference ----------------------------------------------------------------------------
    def denoise(self, flux: np.ndarray | torch.Tensor, vol: np.ndarray, prop: np.ndarray, nphoton: float) -> np.ndarray:
        """Denoised fluence of one MC result: `flux` and `vol` in MCX's [x, y, z] order (first time
        gate of a [x, y, z, t] map is used), `prop` the media table.  Returns fp32 [x, y, z]."""
        f = np.asarray(flux, np.float32)
        if f.ndim == 4:
            f = f[..., 0]
        nx, ny, nz = f.shape
        fl = torch.from_numpy(np.ascontiguousarray(f.reshape(-1, order="F"))).to(self.dev)
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        ev[0].record()
        flux_out = self.denoise_device(fl, vol, prop, nphoton)
        ev[1].record()
        lf = flux_out.cpu().numpy()
        self.last_gpu_ms = ev[0].elapsed_time(ev[1])     # pack + network + exponent on the device
        return lf.reshape((nx, ny, nz), order="F")

    def labels_device(self, vol: np.ndarray) -> torch.Tensor:
        """The label volume [x, y, z] on the device as the network reads it: uint8, x fastest,
        shape (1, voxels).  A C-ordered array is uploaded as it lies and transposed on the GPU."""
        v = np.asarray(vol)
        if v.flags.c_contiguous:
            t = torch.from_numpy(v.astype(np.uint8, copy=False)).to(self.dev)
            return t.permute(2, 1, 0).contiguous().view(1, -1)
        return torch.from_numpy(np.ascontiguousarray(v.astype(np.uint8).reshape(-1, order="F"))).to(self.dev).view(1, -1)

    def denoise_device(self, flux: torch.Tensor, vol: np.ndarray, prop: np.ndarray, nphoton: float,
                       out: torch.Tensor | None = None, labels: torch.Tensor | None = None) -> torch.Tensor:
        """`denoise` on a fluence map already on the device (fp32, x fastest: the layout of
        ``run_batch(..., device_fields=...)``), stream-ordered and without a host round trip:
        returns the denoised linear fluence in the same layout (in `out` when given).  Only the
        labels (unless `labels` from ``labels_device`` is given) and the media table cross the bus."""
        nx, ny, nz = np.asarray(vol).shape[:3]
        fl = flux.reshape(1, -1)
        lab = self.labels_device(vol) if labels is None else labels
        pr = torch.from_numpy(np.ascontiguousarray(prop, np.float32)).to(self.dev).view(1, -1, 4)
        lp = torch.full((1,), math.log10(nphoton), dtype=torch.float32, device=self.dev)
        x0, xres = self.pack(fl, lab, pr, lp, nz, ny, nx)
        logf = self._buf("out", nx * ny * nz, torch.float32)
        self.forward(x0, xres, 1, nz, ny, nx, out=logf)
        # back to linear fluence on the device
        if out is None:
            out = torch.empty(nx * ny * nz, dtype=torch.float32, device=self.dev)
        torch.pow(10.0, logf, out=out)
        return torch.clamp_(out.sub_(FLUX_FLOOR), min=0.0)

    def denoise_many_device(self, flux: torch.Tensor, vols: list[np.ndarray], props: list[np.ndarray],
                            nphotons: list[float], out: torch.Tensor | None = None) -> torch.Tensor:
        """`denoise_device` on several volumes of one shape in one pass of the network: `flux`
        [n, voxels] fp32 on the device (x fastest per row), returns [n, voxels] (in `out` when
        given).  Each volume's result is the one `denoise_device` gives it: every kernel works per
        output voxel, so batching changes only how many CTAs a layer has -- the 16^3 and 32^3
        levels of one 128^3 volume fill a fraction of the SMs, n of them fill the GPU."""
        n = len(vols)
        shape = np.asarray(vols[0]).shape[:3]
        if any(np.asarray(v).shape[:3] != shape for v in vols) or flux.shape[0] != n:
            raise ValueError("denoise_many_device needs n volumes of one shape and an [n, voxels] flux")
        nx, ny, nz = shape
        vox = nx * ny * nz
        vs = [np.asarray(v) for v in vols]
        if all(v.flags.c_contiguous for v in vs):
            lab = torch.from_numpy(np.stack([v.astype(np.uint8, copy=False) for v in vs])).to(self.dev)
            lab = lab.permute(0, 3, 2, 1).contiguous().view(n, vox)
        else:
            lab = torch.cat([self.labels_device(v) for v in vs])
        nprop = max(np.asarray(p).reshape(-1, 4).shape[0] for p in props)
        pr = np.zeros((n, nprop, 4), np.float32)
        for i, p in enumerate(props):
            p = np.asarray(p, np.float32).reshape(-1, 4)
            pr[i, :p.shape[0]] = p
            pr[i, p.shape[0]:] = p[-1]             # rows no label of this volume reads
        pr = torch.from_numpy(pr).to(self.dev)
        lp = torch.tensor([math.log10(x) for x in nphotons], dtype=torch.float32, device=self.dev)
        x0, xres = self.pack(flux.reshape(n, vox), lab, pr, lp, nz, ny, nx)
        logf = self._buf("out", n * vox, torch.float32)
        self.forward(x0, xres, n, nz, ny, nx, out=logf)
        if out is None:
            out = torch.empty(n, vox, dtype=torch.float32, device=self.dev)
        torch.pow(10.0, logf.view(n, vox), out=out)
        return torch.clamp_(out.sub_(FLUX_FLOOR), min=0.0)


# -- data -------------------------------------------------------------------------------------
def median_rel_error(est: np.ndarray, ref: np.ndarray, frac: float = VALID_FRAC) -> float:
    """Median over voxels with ref >= frac * max(ref) of |est - ref| / ref."""
    est = np.asarray(est, np.float64).reshape(-1)
    ref = np.asarray(ref, np.float64).reshape(-1)
    m = ref >= frac * ref.max()
    return float(np.median(np.abs(est[m] - ref[m]) / ref[m]))


def _flat(f: np.ndarray) -> np.ndarray:
    f = np.asarray(f, np.float32)
    if f.ndim == 4:
        f = f[..., 0]
    return f.reshape(-1, order="F")


def simulate(cfgs: list[dict[str, Any]], chunk: int = 96) -> list[np.ndarray]:
    """Fluence maps (first gate, voxel order x fastest) of many simulations through the batched
    CUDA-graph runner."""
    from .api import run_batch

    out = []
    for i in range(0, len(cfgs), chunk):
        res, _ = run_batch(cfgs[i:i + chunk], streams=16)
        out += [_flat(r["flux"]) for r in res]
    return out


def make_pairs(count: int, edge: int = 64, seed: int = 1, target_photons: float = 1e8,
               input_photons: tuple[float, ...] = (1e5, 1e6, 1e7), valid_frac: float = VALID_FRAC) -> dict[str, Any]:
    """Training pairs: `count` random volumes (the batched workload's property ranges), each
    simulated at every input photon count and once at `target_photons` with independent seeds;
    voxels at or above `valid_frac` of a target's maximum are scored.  Returns device tensors:
    inputs [len(input_photons), count, vox], target log10 fluence and score weights [count, vox],
    labels, media tables, and the photon counts."""
    base = problems.denoise_instances(count, edge, seed)
    nprop = max(c["prop"].shape[0] for c in base)
    cfgs = []
    for k, n in enumerate((target_photons,) + tuple(input_photons)):
        for i, c in enumerate(base):
            cc = dict(c)
            cc["nphoton"] = int(n)
            cc["seed"] = int((c["seed"] + 7919 * (k + 1)) % (2**31 - 1)) or 1
            cfgs.append(cc)
    maps = simulate(cfgs)
    dev = torch.device("cuda")
    tgt = torch.from_numpy(np.stack(maps[:count])).to(dev)
    inputs = torch.from_numpy(np.stack(maps[count:]).reshape(len(input_photons), count, -1)).to(dev)
    props = np.zeros((count, nprop, 4), np.float32)
    for i, c in enumerate(base):
        props[i, :c["prop"].shape[0]] = c["prop"]
        props[i, c["prop"].shape[0]:] = c["prop"][-1]
    labels = torch.from_numpy(np.stack([c["vol"].reshape(-1, order="F") for c in base])).to(dev)
    ltgt = torch.log10(tgt + FLUX_FLOOR)
    valid = (tgt >= valid_frac * tgt.amax(dim=1, keepdim=True)).float()
    return {"inputs": inputs, "target": ltgt, "valid": valid, "labels": labels,
            "props": torch.from_numpy(props).to(dev), "photons": tuple(float(n) for n in input_photons),
            "edge": edge, "count": count, "target_photons": float(target_photons), "seed": seed}


def _crop(t: torch.Tensor, edge: int, crop: int, offs: list[tuple[int, int, int]]) -> torch.Tensor:
    """Per-sample crop^3 windows at offsets (z, y, x) of [n, edge^3] tensors (voxel order x
    fastest), flattened back to [n, crop^3]."""
    v = t.view(t.shape[0], edge, edge, edge)
    if crop == edge:
        return t
    return torch.stack([v[i, z:z + crop, y:y + crop, x:x + crop] for i, (z, y, x) in enumerate(offs)]).reshape(t.shape[0], -1)


def _augment(t: torch.Tensor, edge: int, flips: tuple[bool, bool, bool]) -> torch.Tensor:
    """Mirror in x and/or y and swap x with y ([count, vox] tensors, voxel order x fastest); the
    pencil enters along +z, so these leave the physics unchanged."""
    v = t.view(t.shape[0], edge, edge, edge)     # [n, z, y, x]
    if flips[0]:
        v = v.flip(3)
    if flips[1]:
        v = v.flip(2)
    if flips[2]:
        v = v.transpose(2, 3)
    return v.reshape(t.shape[0], -1).contiguous()


def train(net: UNet, data: dict[str, Any], steps: int = 1000, batch: int = 4, lr: float = 1e-3,
          seed: int = 0, log_every: int = 100, verbose: bool = True, crop: int | None = None) -> list[float]:
    """AdamW with a short warm-up and cosine decay over `steps` batches of `batch` samples, each
    a random crop^3 window (the whole volume by default) of a random volume at a random input
    photon count, randomly mirrored / swapped.  Returns the loss per log point (mean absolute
    log10 error over scored voxels)."""
    rng = np.random.default_rng(seed)
    edge, count = data["edge"], data["count"]
    crop = crop or edge
    if crop % 8 or crop > edge:
        raise ValueError("crop must be a multiple of 8 no larger than the volumes")
    lp_all = torch.tensor([math.log10(n) for n in data["photons"]], dtype=torch.float32, device=net.dev)
    losses, acc, nacc = [], 0.0, 0
    warm = max(1, steps // 20)
    for it in range(steps):
        idx = rng.choice(count, size=batch, replace=count < batch)
        lvl = rng.integers(0, len(data["photons"]), size=batch)
        flips = tuple(bool(v) for v in rng.integers(0, 2, 3))
        offs = [tuple(int(o) for o in rng.integers(0, edge - crop + 1, 3)) for _ in range(batch)]
        ii = torch.from_numpy(idx).to(net.dev)
        ll = torch.from_numpy(lvl).to(net.dev)

        def prep(t):
            return _augment(_crop(t, edge, crop, offs), crop, flips)

        flux = prep(data["inputs"][ll, ii])
        labels = prep(data["labels"][ii])
        target = prep(data["target"][ii])
        valid = prep(data["valid"][ii])
        x0, xres = net.pack(flux, labels, data["props"][ii].contiguous(), lp_all[ll].contiguous(), crop, crop, crop)
        A = net.forward(x0, xres, batch, crop, crop, crop)
        nval = float(valid.sum().item())
        net.loss_acc.zero_()
        net.backward(A, target.reshape(-1), valid.reshape(-1), 1.0 / max(nval, 1.0))
        f = min(1.0, (it + 1) / warm) * 0.5 * (1.0 + math.cos(math.pi * it / steps))
        net.step(lr * max(f, 0.02))
        acc += float(net.loss_acc.item()) / max(nval, 1.0)
        nacc += 1
        if (it + 1) % log_every == 0 or it + 1 == steps:
            losses.append(acc / nacc)
            if verbose:
                print(f"step {it + 1}: loss {acc / nacc:.4f}", flush=True)
            acc, nacc = 0.0, 0
    return losses


def evaluate_loss(net: UNet, data: dict[str, Any], batch: int = 4) -> list[float]:
    """Mean absolute log10 error over scored voxels of the whole training set, per input photon
    count, without augmentation."""
    edge, count = data["edge"], data["count"]
    out = []
    for k, n in enumerate(data["photons"]):
        num, den = 0.0, 0.0
        for i in range(0, count, batch):
            ii = torch.arange(i, min(count, i + batch), device=net.dev)
            b = ii.numel()
            lp = torch.full((b,), math.log10(n), dtype=torch.float32, device=net.dev)
            x0, xres = net.pack(data["inputs"][k][ii].contiguous(), data["labels"][ii].contiguous(),
                                data["props"][ii].contiguous(), lp, edge, edge, edge)
            o = net._buf("eval_out", b * edge ** 3, torch.float32)
            net.forward(x0, xres, b, edge, edge, edge, out=o)
            v = data["valid"][ii].reshape(-1)
            num += float(((o - data["target"][ii].reshape(-1)).abs() * v).sum())
            den += float(v.sum())
        out.append(num / max(den, 1.0))
    return out


# -- the metric -------------------------------------------------------------------------------
def pipeline_maps(cfgs: list[dict[str, Any]], budgets: list[float], seeds: list[int], net: UNet | None = None,
                  denoise: list[bool] | None = None, streams: int = 16) -> tuple[list[np.ndarray], float, float]:
    """One pass of the pipeline over many volumes, from host inputs to host maps: one batched MC
    call whose fluence maps stay on the device (``run_batch(..., device_fields=...)``), the network
    on the volumes flagged in `denoise` (one batched pass, ``UNet.denoise_many_device``, when the
    volumes share a shape), and one copy of every final map into pinned host memory.  Returns (maps, flat fp32 x fastest; MC graph time
    in s; network GPU time in s)."""
    from .api import run_batch

    V = len(cfgs)
    denoise = denoise or [False] * V
    sizes = [int(np.asarray(c["vol"]).size) for c in cfgs]
    same = len(set(sizes)) == 1
    if same:
        # one [V, voxels] block: its rows are the fields, the network takes them as one batch
        block = torch.empty(V, sizes[0], dtype=torch.float32, device="cuda")
        fields = list(block)
    else:
        fields = [torch.empty(n, dtype=torch.float32, device="cuda") for n in sizes]
    _, ms = run_batch([dict(c, nphoton=int(n), seed=k) for c, n, k in zip(cfgs, budgets, seeds)], streams=streams,
                      device_fields=fields)
    host = [torch.empty(f.numel(), dtype=torch.float32, pin_memory=True) for f in fields]
    # the network's GPU time: events around the pack + network + exponent only
    evs = []
    sel = [v for v in range(V) if denoise[v]]
    if sel and same:
        idx = torch.tensor(sel, device="cuda")
        sub = block if len(sel) == V else block.index_select(0, idx)
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        ev[0].record()
        res = net.denoise_many_device(sub, [cfgs[v]["vol"] for v in sel], [cfgs[v]["prop"] for v in sel],
                                      [budgets[v] for v in sel], out=sub if len(sel) == V else None)
        ev[1].record()
        evs.append(ev)
        if len(sel) != V:
            block.index_copy_(0, idx, res)
    elif sel:
        for v in sel:
            c = cfgs[v]
            lab = net.labels_device(c["vol"])
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record()
            net.denoise_device(fields[v], c["vol"], c["prop"], budgets[v], out=fields[v], labels=lab)
            ev[1].record()
            evs.append(ev)
    for f, h in zip(fields, host):
        h.copy_(f, non_blocking=True)
    torch.cuda.synchronize()
    net_s = sum(a.elapsed_time(b) for a, b in evs) * 1e-3
    return [h.numpy() for h in host], ms * 1e-3, net_s


def time_to_error_batch(net: UNet, cfgs: list[dict[str, Any]], judge_photons: float = 1e9,
                        targets: tuple[float, ...] = (0.05, 0.02),
                        ladder: tuple[float, ...] = (1e5, 3e5, 1e6, 3e6, 1e7, 3e7, 1e8),
                        dn_ladder: tuple[float, ...] = (1e5, 2e5, 3e5, 6e5, 1e6, 3e6, 1e7),
                        judge_check: bool = True, streams: int = 16) -> dict[str, Any]:
    """Time for each pipeline to deliver every volume of `cfgs` at a median relative fluence error
    of each target against a `judge_photons` run of that volume, with all volumes simulated
    together through the batched entry point (one CUDA graph per call, short simulations side by
    side), so a short simulation's latency -- its longest photons -- is paid once per call rather
    than once per volume.  Both pipelines run through `pipeline_maps` (host inputs to host maps).

    The errors come from ladders of budgets (every budget one batched call over all volumes).  Plain
    MC: each volume's photon count for the target is interpolated in its ladder (log-log, the
    1/sqrt(N) law past the last budget), then ONE pipeline pass runs every volume at its own count
    and is timed: on the device (graph time) and end to end (wall time of the pass).  MC +
    denoiser: each volume takes the smallest budget of `dn_ladder` whose denoised map reaches the
    target (volumes that none reaches fall back to plain MC at their plain count), then one pass
    runs them and denoises: device time = graph time + network GPU time, wall time = the pass.
    The measured errors of those final runs are returned beside the times; they are computed
    after the clock stops."""
    V = len(cfgs)
    seed = lambda c, k: int((int(c["seed"]) + 7919 * k) % (2**31 - 1)) or 1  # noqa: E731

    def batch(budgets, k, dn_flags=None):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        maps, mc_s, net_s = pipeline_maps(cfgs, budgets, [seed(c, k) for c in cfgs], net, dn_flags, streams)
        return maps, mc_s, net_s, time.perf_counter() - t0

    judges, _, _, judge_s = batch([judge_photons] * V, 1)
    judge_err = None
    if judge_check:
        j4 = batch([judge_photons / 4] * V, 2)[0]
        judge_err = [median_rel_error(a, b) / math.sqrt(5.0) for a, b in zip(j4, judges)]
    plain = []
    for i, n in enumerate(ladder):
        maps, mc_s, _, wall_s = batch([n] * V, 10 + i)
        plain.append({"photons": n, "errors": [median_rel_error(m, j) for m, j in zip(maps, judges)],
                      "s": wall_s, "kernel_s": mc_s})
    dn = []
    for i, n in enumerate(dn_ladder):
        maps, mc_s, net_s, wall_s = batch([n] * V, 30 + i, [True] * V)
        dn.append({"photons": n, "errors": [median_rel_error(m, j) for m, j in zip(maps, judges)],
                   "kernel_s": mc_s, "network_s": net_s, "s": wall_s})

    def plain_photons(v, tgt):
        lad = [{"photons": r["photons"], "error": r["errors"][v]} for r in plain]
        for a, b in zip(lad, lad[1:]):
            if a["error"] > tgt >= b["error"]:
                slope = math.log(b["error"] / a["error"]) / math.log(b["photons"] / a["photons"])
                return a["photons"] * (tgt / a["error"]) ** (1.0 / slope)
        return lad[-1]["photons"] * (lad[-1]["error"] / tgt) ** 2 if lad[-1]["error"] > tgt else lad[0]["photons"]

    per = []
    for t_i, tgt in enumerate(targets):
        n_plain = [plain_photons(v, tgt) for v in range(V)]
        maps, p_dev, _, p_wall = batch(n_plain, 60 + t_i)
        p_err = [median_rel_error(m, j) for m, j in zip(maps, judges)]
        n_dn, use_dn = [], []
        for v in range(V):
            rec = next((r for r in dn if r["errors"][v] <= tgt), None)
            use_dn.append(rec is not None)
            n_dn.append(rec["photons"] if rec else n_plain[v])
        maps, mc_s, net_s, d_wall = batch(n_dn, 80 + t_i, use_dn)
        d_err = [median_rel_error(m, j) for m, j in zip(maps, judges)]
        d_dev = mc_s + net_s
        per.append({"target": tgt, "photons_plain": n_plain, "t_plain_s": p_wall, "t_plain_device_s": p_dev,
                    "error_plain": p_err, "photons_denoised": n_dn, "denoised": use_dn, "t_denoised_s": d_wall,
                    "t_denoised_device_s": d_dev, "network_s": net_s, "error_denoised": d_err,
                    "speedup": p_wall / d_wall, "speedup_device": p_dev / d_dev})
    return {"volumes": V, "judge_photons": judge_photons, "judge_s": judge_s, "judge_error_est": judge_err,
            "plain": plain, "denoised": dn, "targets": per}


def main(argv: list[str] | None = None) -> None:
    """``python -m mcx_gb300.denoise train ...``: simulate training pairs, train, save the weights."""
    import argparse
    import json

    ap = argparse.ArgumentParser(prog="python -m mcx_gb300.denoise")
    ap.add_argument("command", choices=["train", "forward", "conv"],
                    help="train: simulate pairs, train, save; forward: time the network on one volume; "
                         "conv: run one 3x3x3 convolution --repeat times (a fixed workload for profilers)")
    ap.add_argument("--cin", type=int, default=16, help="conv: input channels")
    ap.add_argument("--cout", type=int, default=16, help="conv: output channels")
    ap.add_argument("--repeat", type=int, default=10, help="forward: timed passes")
    ap.add_argument("--count", type=int, default=64, help="training volumes")
    ap.add_argument("--edge", type=int, default=128, help="edge of the simulated training volumes")
    ap.add_argument("--crop", type=int, default=64, help="edge of the training windows")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--target-photons", type=float, default=1e8)
    ap.add_argument("--input-photons", default="1e5,1e6,1e7")
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", default=str(DEFAULT_WEIGHTS))
    a = ap.parse_args(argv)
    if a.command == "conv":
        # one convolution on random bf16 activations [1][edge]^3[cin] and weights [cout][27][cin],
        # through the same C entry point the network uses
        n = a.edge
        g = torch.Generator(device="cuda").manual_seed(a.seed)
        x = torch.randn(n ** 3 * a.cin, generator=g, device="cuda").to(torch.bfloat16)
        w = (torch.randn(a.cout * TAPS * a.cin, generator=g, device="cuda") * 0.05).to(torch.bfloat16)
        y = torch.empty(n ** 3 * a.cout, device="cuda", dtype=torch.bfloat16)
        st = torch.cuda.current_stream().cuda_stream
        for _ in range(a.repeat):
            _ok(lib.mcxg_dn_conv_fwd(x.data_ptr(), w.data_ptr(), None, None, y.data_ptr(), 1, n, n, n, a.cin, a.cout,
                                     TAPS, 1, st), "conv")
        _ok(lib.mcxg_dn_check(st), "conv")
        print(json.dumps({"cin": a.cin, "cout": a.cout, "edge": n, "launches": a.repeat}))
        return
    if a.command == "forward":
        net = UNet(load_params() if DEFAULT_WEIGHTS.exists() else None, seed=a.seed)
        n = a.edge
        g = torch.Generator(device="cuda").manual_seed(a.seed)
        x0 = torch.randn(n ** 3 * IN_CH, generator=g, device="cuda").to(torch.bfloat16)
        xr = torch.zeros(n ** 3, device="cuda")
        out = torch.empty(n ** 3, device="cuda")
        for _ in range(3):
            net.forward(x0, xr, 1, n, n, n, out=out)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(a.repeat):
            net.forward(x0, xr, 1, n, n, n, out=out)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.repeat
        flops = sum(2.0 * (n >> l) ** 3 * ci * co * TAPS for _, ci, co, l in LAYERS)
        print(json.dumps({"edge": n, "forward_ms": ms, "gflop": flops / 1e9, "tflops": flops / ms / 1e9}))
        return
    t0 = time.perf_counter()
    data = make_pairs(a.count, a.edge, a.seed, a.target_photons, tuple(float(v) for v in a.input_photons.split(",")))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    net = UNet(seed=a.seed)
    losses = train(net, data, steps=a.steps, batch=a.batch, lr=a.lr, crop=a.crop)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    net.save(a.out)
    print(json.dumps({"volumes": a.count, "edge": a.edge, "crop": a.crop, "target_photons": a.target_photons,
                      "input_photons": data["photons"], "final_loss": evaluate_loss(net, data), "steps": a.steps,
                      "batch": a.batch, "simulate_s": t1 - t0, "train_s": t2 - t1,
                      "ms_per_step": 1e3 * (t2 - t1) / a.steps, "losses": losses, "out": a.out}))


if __name__ == "__main__":
    main()
