#!/usr/bin/env python
"""Plain-MC photon-transport throughput (photons/ms) of the GB300 engine.

One step = one complete simulation of the workload's photon budget.  By default the workload is
the heterogeneous cube (label-2 sphere, Fresnel reflection, 50 time gates of 0.1 ns, four
detectors saving id / scattering counts / partial paths) at 1e8 photons.

  value     device-resident: inputs uploaded once into a session, CUDA-event time of the transport
            launches only (L2 flushed before every timed step)
  e2e       the public call a user makes, mcx_gb300.run(cfg) -> mcx_run_simulation, from host
            buffers: Config preparation, volume upload, transport, normalisation, field and
            detected-photon copy back, all inside the timed region
  --impl reference   the reference arm: MCX itself compiled from its sources for sm_103a
            (oracle/ref_mcx.py) on the same GPU when its sources are staged, else the CPU oracle

Other workloads (--workload): workload0 (homogeneous cube), workload2 (256^3 layered volume),
cube60planar (planar source), batch (256 simulations in one CUDA graph), contest (MCX's speed
contest: cube60 + cube60b + cube60planar at 1e8 photons, the score being the sum of the three
photons/ms), denoise (MC + learned denoiser against plain MC: seconds to a 5% median relative
fluence error on 128^3 volumes; --steps volumes, --judge-photons for the judge runs).

Multi-GPU (torchrun, one rank per GPU): every rank simulates its own photon range of the same
size (weak scaling, no collective in the data path); rank 0 prints.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "photons/ms (plain MC)"
WORKLOAD_PHOTONS = {"workload0": 1_000_000, "workload1": 100_000_000, "workload2": 1_000_000_000,
                    "cube60planar": 100_000_000, "batch": 0, "contest": 100_000_000, "denoise": 0}
# photons of the CPU-oracle sample per workload: about 10 s on 16 cores
CPU_SAMPLE = {"workload0": 8_000_000, "workload1": 4_000_000, "workload2": 1_000_000, "cube60planar": 6_000_000,
              "batch": 20_000, "contest": 4_000_000, "denoise": 200_000}
# MCX's speed contest (manpage/mcxcontest.1:13, mcxlab/examples/mcx_gpu_benchmarks.m:124-130): the
# built-in cube60, cube60b and cube60planar decks at 1e8 photons; the score is the sum of the three
# photons/ms figures.
CONTEST_DECKS = ("cube60", "cube60b", "cube60planar")

# Thread-level instructions per transport step (ncu smsp__inst_executed.sum x
# smsp__thread_inst_executed_per_inst_executed.ratio over the kernel's own step counter) and
# DRAM bytes of one launch (dram__bytes_read.sum + dram__bytes_write.sum), from one ncu capture
# of `bench.py --workload W --photons 20000000 --steps 1 --warmup 1`.  The DRAM bytes are the
# field's first read and its write-back: the field and labels stay in L2, so they do not grow
# with the photon count.
# workload2: `bench.py --workload workload2 --photons 2000000 --steps 1 --warmup 1 --no-cpu-baseline`,
# the timed launch (-s 7 -c 1): 5.382e10 warp instructions x 15.63 lanes over 2e6 x 1606.5 steps.
NCU_PER_STEP = {"workload0": 222.8, "workload1": 272.0, "workload2": 261.8}
NCU_DRAM_PER_LAUNCH = {"workload0": 1.63e6, "workload1": 41.59e6, "workload2": 25.97e6}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = ""

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        d["_source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0, "_source": "fallback"}


def workload_config(name: str, cfg: dict, nphoton: int, world: int) -> dict:
    """The `config` object of a single-workload line, identical in both arms: what is simulated,
    not how (launch shapes and build details ride in their own keys)."""
    gates = max(1, int((cfg["tend"] - cfg["tstart"]) / cfg["tstep"] + 0.5))
    ndet = int(np.asarray(cfg["detpos"]).reshape(-1, 4).shape[0]) if cfg.get("issavedet") and "detpos" in cfg else 0
    return {"workload": name, "photons_per_step": int(nphoton), "volume": list(np.asarray(cfg["vol"]).shape),
            "gates": gates, "detectors": ndet, "parallelism": f"replicas{world}",
            "l2": "flushed before each timed step"}


class L2Flush:
    """Writes 256 MB (> the 129 MB L2) on the device before each timed step."""

    def __init__(self):
        import torch

        self.torch = torch
        self.buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.buf.zero_()
        self.torch.cuda.synchronize()


def make_cfg(name: str, nphoton: int, seed: int):
    from mcx_gb300 import problems

    if name == "cube60planar":
        cfg = problems.cube60planar(nphoton)
        cfg["seed"] = seed
        return cfg
    return problems.WORKLOADS[name](nphoton, seed=seed)


def contest_cfg(deck: str, nphoton: int, seed: int):
    from mcx_gb300 import problems

    cfg = getattr(problems, deck)(nphoton)
    cfg["seed"] = seed
    return cfg


def contest_main(args, world, rank) -> None:
    """The speed contest: each deck timed like the single workloads (device-resident `value`,
    `e2e` through mcx_gb300.run), the line's value and e2e being the sums of the three."""
    import torch

    import mcx_gb300
    from mcx_gb300 import Session

    torch.cuda.set_device(0)
    nphoton = int(args.photons) if args.photons else WORKLOAD_PHOTONS["contest"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    per, e2e, h2d, d2h = {}, {}, 0, 0
    with Clocks(0) as clk:
        for k, deck in enumerate(CONTEST_DECKS):
            sess = Session(mcx_gb300.prepare(contest_cfg(deck, nphoton, 1648335518)))
            sess.autotune(nphoton)
            for i in range(args.warmup):
                sess.run(i * nphoton, nphoton, 1648335518)
            ms = []
            for i in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                ms.append(sess.run((args.warmup + i) * nphoton, nphoton, 1648335518))
            sess.close()
            per[deck] = nphoton * args.steps / sum(ms)
            wall = []
            for i in range(1 + args.steps):
                c = contest_cfg(deck, nphoton, 1648335518 + i)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r = mcx_gb300.run(c)
                if i:
                    wall.append((time.perf_counter() - t0) * 1e3)
                h2d += (c["vol"].size * 4 + np.asarray(c["prop"]).nbytes) * (i > 0)
                d2h += (r["flux"].nbytes + (r["detp"].nbytes if "detp" in r else 0)) * (i > 0)
            e2e[deck] = nphoton * args.steps / sum(wall)
    if rank != 0:
        return
    value = sum(per.values())
    line = {
        "metric": METRIC + ", summed over MCX's contest decks", "value": value, "unit": "photons/ms", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(nphoton / v for v in per.values()),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "contest", "decks": list(CONTEST_DECKS), "photons_per_deck": nphoton,
                   "per_deck": per, "l2": "flushed before each timed step"},
        "e2e": {"value": sum(e2e.values()), "unit": "photons/ms", "per_deck": e2e,
                "h2d_bytes_per_step": int(h2d / max(1, args.steps)), "d2h_bytes_per_step": int(d2h / max(1, args.steps))},
        "gpu_launches": 3 * args.steps,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


def batch_cfgs(scale: float, seed: int = 20251204):
    from mcx_gb300 import problems

    return problems.batch_instances(256, seed=seed, budget_scale=scale)


def batch_main(args, world, rank) -> None:
    """The batched workload: 256 simulations per step in one CUDA graph (mcxg_run_batch).
    value = all photons of the batch over the graph's CUDA-event time (volumes already on the
    device); e2e = the same over the wall time of the whole mcx_gb300.run_batch call (Config
    preparation, uploads, graph, normalisation, copies back)."""
    import torch

    import mcx_gb300

    torch.cuda.set_device(0)
    cfgs = batch_cfgs(args.batch_scale)
    total = sum(c["nphoton"] for c in cfgs)
    for _ in range(args.warmup):
        mcx_gb300.run_batch(batch_cfgs(args.batch_scale), streams=args.streams)
    graph_ms, wall_ms, h2d, d2h = [], [], 0, 0
    steps = deps = glob = 0
    with Clocks(0) as clk:
        for _ in range(args.steps):
            cs = batch_cfgs(args.batch_scale)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res, ms = mcx_gb300.run_batch(cs, streams=args.streams)
            wall_ms.append((time.perf_counter() - t0) * 1e3)
            graph_ms.append(ms)
            for r in res:
                steps += r["stat"]["n_steps"]
                deps += r["stat"]["n_deposit"]
                glob += r["stat"]["n_deposit"] - r["stat"]["n_tile_deposit"]
            h2d = sum(c["vol"].size * 4 + np.asarray(c["prop"]).nbytes + np.asarray(c["detpos"]).nbytes for c in cs)
            d2h = sum(r["flux"].nbytes + (r["detp"].nbytes if "detp" in r else 0) for r in res)
    if rank != 0:
        return
    g = sum(graph_ms)
    line = {
        "metric": METRIC, "value": total * args.steps / g, "unit": "photons/ms", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": g / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batch", "instances": len(cfgs), "photons_per_step": total,
                   "budget_scale": args.batch_scale, "streams": args.streams,
                   "l2": "inputs (256 volumes, 256 fields) larger than L2"},
        "e2e": {"value": total * args.steps / sum(wall_ms), "unit": "photons/ms", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": sum(wall_ms) / args.steps},
        "gpu_launches": len(cfgs) * args.steps,
        "clocks": clk.summary(),
    }
    # the issue roofline of single runs over the batch's own mean steps per photon (the batch runs
    # the reflecting detector variant of workload1's kernel)
    clocks = line["clocks"]
    f_clk = (clocks["sm_mhz"] or peaks().get("sm_max_mhz", 2070.0)) * 1e6
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    photons = total * args.steps
    ips = NCU_PER_STEP["workload1"]
    p_issue = sms * 4 * 32 * f_clk / (ips * steps / photons) / 1e3
    line["roofline"] = {"bound": "fp32-issue", "achieved": line["value"], "peak": p_issue, "unit": "photons/ms",
                        "frac": line["value"] / p_issue, "traffic": None, "steps_per_photon": steps / photons,
                        "deposits_per_photon": deps / photons, "global_reductions_per_photon": glob / photons,
                        "thread_inst_per_step": ips, "sm_clock_hz": f_clk,
                        "peak_source": "issue: SMs x 4 x 32 x measured SM clock over workload1's instructions per step"}
    print(json.dumps(line))


DN_METRIC = "time to 5% median rel. fluence error on 128^3 volumes, MC+denoiser vs plain MC"


def _dn_flops(d: int, h: int, w: int, nvol: int = 1) -> float:
    """Multiply-add FLOPs (2 per MAC) of one U-Net forward pass over nvol d x h x w volumes."""
    from mcx_gb300 import denoise as dn

    return sum(2.0 * nvol * (d >> l) * (h >> l) * (w >> l) * ci * co * dn.TAPS for _, ci, co, l in dn.LAYERS)


def denoise_main(args, world, rank) -> None:
    """MC + learned denoiser against plain MC on held-out 128^3 volumes of the batched workload's
    property ranges: per volume, the time to a median relative fluence error of 5% against a
    `--judge-photons` run (mcx_gb300.denoise.time_to_error_batch).  value = device time of MC +
    denoiser over all volumes (the batched transport graph + the network); e2e = wall time of the
    same pipeline through the public calls (mcx_gb300.denoise.pipeline_maps: run_batch with the
    fields kept on the device, UNet.denoise_many_device, one pinned copy back per volume) from host
    inputs to host maps; plain MC runs through the same pipeline without the network, and its
    times and the speed-ups ride along.  One step = one volume; warm-up = full denoise pipelines
    at 1e5 photons on the first volume."""
    import torch

    from mcx_gb300 import denoise as dn
    from mcx_gb300 import problems

    torch.cuda.set_device(0)
    if dn.DEFAULT_WEIGHTS.exists():
        net, weights = dn.UNet(dn.load_params()), "checkpoint " + dn.DEFAULT_WEIGHTS.name
    else:
        data = dn.make_pairs(64, 64, 1, 1e7)
        net = dn.UNet(seed=1)
        dn.train(net, data, steps=800, batch=4, lr=1e-3, verbose=False)
        weights = "trained in this run (64 volumes, 800 steps)"
    cfgs = problems.denoise_instances(args.steps, 128, seed=31337)
    import mcx_gb300

    for i in range(args.warmup):
        r = mcx_gb300.run(dict(cfgs[0], nphoton=int(1e5), seed=1000 + i))
        net.denoise(r["flux"], cfgs[0]["vol"], cfgs[0]["prop"], 1e5)
    # the network alone at 128^3: CUDA events around repeated forward passes on resident inputs
    n = 128
    x0 = torch.zeros(n ** 3 * dn.IN_CH, dtype=torch.bfloat16, device="cuda")
    xr = torch.zeros(n ** 3, device="cuda")
    out = torch.empty(n ** 3, device="cuda")
    for _ in range(3):
        net.forward(x0, xr, 1, n, n, n, out=out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(10):
        net.forward(x0, xr, 1, n, n, n, out=out)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / 10
    with Clocks(0) as clk:
        res = dn.time_to_error_batch(net, cfgs, judge_photons=args.judge_photons)
    if rank != 0:
        return
    pk = peaks()
    flops = _dn_flops(n, n, n)
    tflops = flops / (fwd_ms * 1e-3) / 1e12
    t5, t2 = res["targets"][0], res["targets"][1]
    V = len(cfgs)
    # MC inputs (the volume as MCX's 32-bit words, the media table) and the network's labels up;
    # one fp32 map per volume down
    h2d = sum(c["vol"].size * 4 + 2 * np.asarray(c["prop"]).nbytes + c["vol"].size for c in cfgs)
    d2h = sum(4 * c["vol"].size for c in cfgs)
    # the timed 5% pass: per volume the label packing, transport and merge kernels; one batched
    # network pass (pack, 14 convolutions, pools, upsampling, head) over the denoised volumes
    launches = 3 * V + (22 if any(t5["denoised"]) else 0)
    rnd = lambda x: [round(v, 5) for v in x] if isinstance(x, list) else x  # noqa: E731
    line = {
        "metric": DN_METRIC, "value": t5["t_denoised_device_s"], "unit": "s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t5["t_denoised_device_s"] / V, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 transport, bf16 network (fp32 accumulate)",
        "data": "synthetic",
        "config": {"workload": "denoise", "volumes": V, "edge": n, "judge_photons": args.judge_photons,
                   "target_error": 0.05, "weights": weights, "pipeline": "all volumes in one batched call per budget, fields kept on the device",
                   "l2": "inputs (128^3 fields and activations) larger than L2"},
        "plain_mc_s": t5["t_plain_device_s"],
        "speedup": t5["speedup_device"],
        "e2e": {"value": t5["t_denoised_s"], "unit": "s", "plain_mc_s": t5["t_plain_s"], "speedup": t5["speedup"],
                "h2d_bytes_per_step": int(h2d / V), "d2h_bytes_per_step": int(d2h / V)},
        "targets": [{k: rnd(v) for k, v in t.items()} for t in res["targets"]],
        "judge_error_est": rnd(res["judge_error_est"]),
        "ladder": [(r["photons"], rnd(r["errors"]), round(r["kernel_s"], 5)) for r in res["plain"]],
        "denoised_ladder": [(r["photons"], rnd(r["errors"]), round(r["kernel_s"], 5)) for r in res["denoised"]],
        "at_2pct": {"value": t2["t_denoised_device_s"], "plain_mc_s": t2["t_plain_device_s"],
                    "speedup": t2["speedup_device"], "e2e_speedup": t2["speedup"]},
        "roofline": {"bound": "tensor", "kernel": "U-Net forward at 128^3 (14 implicit-GEMM convolutions)",
                     "achieved": tflops, "peak": pk.get("bf16_tflops"), "unit": "TFLOP/s",
                     "frac": tflops / pk["bf16_tflops"] if pk.get("bf16_tflops") else None, "traffic": None,
                     "flops_per_launch": flops, "forward_ms": fwd_ms, "peak_source": pk["_source"]},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        # the CPU oracle's plain MC on a bounded sample of the first volume, priced at the photon
        # count plain MC needs for 5%
        import mcx_gb300
        from oracle import oracle

        sample = args.cpu_sample or 200_000
        r = oracle.run(mcx_gb300.prepare(dict(cfgs[0], nphoton=sample)), nphoton=sample, seed=77,
                       threads=os.cpu_count() or 1)
        rate = sample / r["stat"]["seconds"]
        line["cpu_baseline"] = {"value": sum(t5["photons_plain"]) / rate, "unit": "s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{sample} photons of the first volume ({r['stat']['seconds']:.1f} s), "
                                          "plain MC priced at the photon counts that reach 5%"}
    print(json.dumps(line))


def cpu_baseline(name: str, sample: int) -> dict:
    """The CPU oracle (a C++/OpenMP restatement of MCX's loop; MCX itself has no CPU path) on a
    bounded sample of the same workload, on every host core."""
    import mcx_gb300
    from oracle import oracle

    pc = mcx_gb300.prepare(make_cfg(name, sample, 4242))
    cores = os.cpu_count() or 1
    r = oracle.run(pc, nphoton=sample, seed=4242, threads=cores)
    sec = r["stat"]["seconds"]
    return {"value": sample / (sec * 1e3), "unit": "photons/ms", "cores": cores, "kind": "port",
            "sample": f"{sample} photons of {name} ({sec:.2f} s)"}


def reference_arm(args, world, rank) -> None:
    """MCX's own CUDA build on this GPU (its kernel-only photon/ms as `value`, photons over its
    mcx_run_simulation time up to normalised output as `e2e`); the CPU oracle when the reference
    sources are not staged."""
    if rank != 0:
        return
    name = args.workload
    nphoton = int(args.photons) if args.photons else WORKLOAD_PHOTONS[name]
    from oracle import ref_mcx

    base = {"impl": "reference", "metric": METRIC, "unit": "photons/ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic"}
    if name == "contest" and ref_mcx.available():
        ref_mcx.build()
        per, e2e = {}, {}
        for deck in CONTEST_DECKS:
            for i in range(args.warmup):
                ref_mcx.run(contest_cfg(deck, min(nphoton, 10_000_000), 100 + i), keep_field=False)
            runs = [ref_mcx.run(contest_cfg(deck, nphoton, 1648335518 + i), keep_field=False) for i in range(args.steps)]
            per[deck] = statistics.mean(r["speed"] for r in runs)
            e2e[deck] = nphoton / statistics.mean(r["normalized_ms"] for r in runs)
        v = sum(per.values())
        line = dict(base, metric=METRIC + ", summed over MCX's contest decks", value=v,
                    ms_per_step=sum(nphoton / x for x in per.values()),
                    config={"workload": "contest", "decks": list(CONTEST_DECKS), "photons_per_deck": nphoton,
                            "per_deck": per},
                    e2e={"value": sum(e2e.values()), "unit": "photons/ms", "per_deck": e2e, "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": 0},
                    cpu_baseline={"value": v, "unit": "photons/ms", "cores": os.cpu_count(), "kind": "reference",
                                  "sample": "the reference MCX CUDA build itself on this GPU"})
        print(json.dumps(line))
        return
    if name == "denoise" and ref_mcx.available():
        # MCX has no denoiser: its pipeline is plain MC.  The same held-out volumes, its own judge
        # run and its own photon ladder give the photon count its fluence needs for a 5% median
        # relative error, priced at its own photon rate (kernel-only and up to normalised output).
        from mcx_gb300 import problems
        from mcx_gb300.denoise import median_rel_error

        ref_mcx.build()
        cfgs = problems.denoise_instances(args.steps, 128, seed=31337)
        for i in range(args.warmup):
            ref_mcx.run(dict(cfgs[0], nphoton=100_000, seed=500 + i), keep_field=False)
        per, t_kern, t_norm, t_kern2 = [], 0.0, 0.0, 0.0
        for c in cfgs:
            judge = ref_mcx.run(dict(c, nphoton=int(args.judge_photons), seed=c["seed"] + 1))["flux"][..., 0]
            lad = []
            for k, n in enumerate((1e5, 3e5, 1e6, 3e6, 1e7, 3e7)):
                r = ref_mcx.run(dict(c, nphoton=int(n), seed=c["seed"] + 2 + k))
                lad.append((n, median_rel_error(r["flux"][..., 0], judge), r["speed"], r["normalized_ms"]))
            def photons_for(e):
                for a, b in zip(lad, lad[1:]):
                    if a[1] > e >= b[1]:
                        return a[0] * (e / a[1]) ** (np.log(b[0] / a[0]) / np.log(b[1] / a[1]))
                return lad[-1][0] * (lad[-1][1] / e) ** 2 if lad[-1][1] > e else lad[0][0]

            n_star, n_2 = photons_for(0.05), photons_for(0.02)
            big = [x for x in lad if x[0] >= 1e6 and x[2]]
            rate_k = sum(x[0] for x in big) / sum(x[0] / x[2] for x in big)           # photons per kernel ms
            rate_n = sum(x[0] for x in big) / max(1, sum(x[3] for x in big))          # photons per normalised ms
            t_kern += n_star / rate_k / 1e3
            t_norm += n_star / rate_n / 1e3
            t_kern2 += n_2 / rate_k / 1e3
            per.append({"photons_plain": n_star, "photons_plain_2pct": n_2,
                        "ladder": [(x[0], round(x[1], 4)) for x in lad], "photons_per_ms": rate_k})
        line = dict(base, metric=DN_METRIC, value=t_kern, unit="s", higher_is_better=False,
                    ms_per_step=1e3 * t_kern / args.steps,
                    config={"workload": "denoise", "volumes": args.steps, "edge": 128,
                            "judge_photons": args.judge_photons, "target_error": 0.05,
                            "note": "MCX has no denoiser: plain MC on the reference build"},
                    per_volume=per, at_2pct={"value": t_kern2},
                    e2e={"value": t_norm, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                    cpu_baseline={"value": t_kern, "unit": "s", "cores": os.cpu_count(), "kind": "reference",
                                  "sample": "the reference MCX CUDA build itself on this GPU"})
        print(json.dumps(line))
        return
    if name == "batch" and ref_mcx.available():
        # MCX has no batch mode: its front-ends run the simulations one after another.  A bounded
        # sample of the batch (the first `--ref-sample` instances) runs that way per step.
        cfgs = batch_cfgs(args.batch_scale)[: args.ref_sample]
        ref_mcx.build()
        photons = sum(c["nphoton"] for c in cfgs)
        kern, norm, wall = 0.0, 0.0, 0.0
        for _ in range(args.steps):
            for c in cfgs:
                t0 = time.perf_counter()
                r = ref_mcx.run(c, keep_field=False)
                wall += time.perf_counter() - t0
                kern += c["nphoton"] / r["speed"]
                norm += r["normalized_ms"]
        line = dict(base, value=photons * args.steps / kern, ms_per_step=kern / args.steps,
                    config={"workload": "batch", "instances": len(cfgs), "photons_per_step": photons,
                            "budget_scale": args.batch_scale, "note": "the first instances of the batch, run in sequence"},
                    e2e={"value": photons * args.steps / norm, "unit": "photons/ms", "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": 0, "ms_per_step": norm / args.steps, "process_wall_s": wall},
                    cpu_baseline={"value": photons * args.steps / kern, "unit": "photons/ms", "cores": os.cpu_count(),
                                  "kind": "reference", "sample": f"{len(cfgs)} batch instances, the MCX CUDA build"})
        print(json.dumps(line))
        return
    if ref_mcx.available():
        try:
            t0 = time.perf_counter()
            ref_mcx.build()
            build_s = time.perf_counter() - t0
            for i in range(args.warmup):
                ref_mcx.run(make_cfg(name, min(nphoton, 10_000_000), 100 + i), keep_field=False)
            flush = L2Flush()
            runs = []
            for i in range(args.steps):
                c = make_cfg(name, nphoton, 200 + i)
                flush()
                t0 = time.perf_counter()
                r = ref_mcx.run(c, keep_field=False)
                runs.append((r, time.perf_counter() - t0))
            speed = statistics.mean(r["speed"] for r, _ in runs)
            norm_ms = statistics.mean(r["normalized_ms"] for r, _ in runs)
            wall = statistics.mean(w for _, w in runs)
            line = dict(base, value=speed, ms_per_step=nphoton / speed,
                        config=workload_config(name, make_cfg(name, nphoton, 200), nphoton, world),
                        reference_build={"threads": runs[0][0]["threads"],
                                         "build": "src/mcx_core.cu -DUSE_ATOMIC -DSAVE_DETECTORS -use_fast_math -arch=sm_103a",
                                         "build_s": round(build_s, 1)},
                        e2e={"value": nphoton / norm_ms, "unit": "photons/ms", "h2d_bytes_per_step": 0,
                             "d2h_bytes_per_step": 0, "ms_per_step": norm_ms, "process_wall_s": wall},
                        absorbed=[r["absorbed"] for r, _ in runs],
                        cpu_baseline={"value": speed, "unit": "photons/ms", "cores": os.cpu_count(), "kind": "reference",
                                      "sample": "the reference MCX CUDA build itself on this GPU"})
            print(json.dumps(line))
            return
        except Exception as e:  # noqa: BLE001 -- fall back to the CPU restatement, say why
            base["reference_build_error"] = str(e)[:300]
    sample = args.cpu_sample or CPU_SAMPLE[name]
    for _ in range(args.warmup):
        cpu_baseline(name, max(1000, sample // 10))
    t0 = time.perf_counter()
    vals = [cpu_baseline(name, sample) for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    v = sample * args.steps / (wall * 1e3)
    line = dict(base, value=v, ms_per_step=wall * 1e3 / args.steps,
                config={"workload": name, "photons_per_step": sample, "note": "CPU restatement of the CUDA-only path"},
                cpu_baseline={"value": v, "unit": "photons/ms", "cores": vals[0]["cores"], "kind": "port",
                              "sample": f"{sample} photons of {name} per step"},
                e2e={"value": v, "unit": "photons/ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    print(json.dumps(line))


def roofline(name: str, value: float, world: int, st, f_clk: float, sms: int, atom_rate: float, pk: dict) -> dict:
    """The transport roofline: the slower of FP32/INT issue (every lane slot issuing a useful
    instruction) and L2 reduction throughput for the deposits, in photons/ms."""
    steps = st.n_steps / max(1, st.n_photon)
    deps = st.n_deposit / max(1, st.n_photon)
    glob = (st.n_deposit - st.n_tile_deposit) / max(1, st.n_photon)
    achieved = value / world
    ips = NCU_PER_STEP.get(name)
    p_issue = sms * 4 * 32 * f_clk / (ips * steps) / 1e3 if ips else None
    p_atom = atom_rate / max(glob, 1e-9) / 1e3 if atom_rate else None
    cands = [(p, b) for p, b in ((p_issue, "fp32-issue"), (p_atom, "l2-atomic")) if p]
    peak, bound = min(cands) if cands else (None, "fp32-issue")
    dram = NCU_DRAM_PER_LAUNCH.get(name)
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": "photons/ms",
            "frac": achieved / peak if peak else None,
            "traffic": dram,
            "traffic_unit": "DRAM bytes per launch (ncu capture of a 2e7-photon launch; independent of the photon count)",
            "p_issue": p_issue, "p_atom": p_atom, "steps_per_photon": steps, "deposits_per_photon": deps,
            "global_reductions_per_photon": glob, "thread_inst_per_step": ips, "sm_clock_hz": f_clk,
            "l2_reductions_per_s": atom_rate, "peak_source": "issue: SMs x 4 x 32 x measured SM clock; "
                                                             "atomics: measured on this GPU"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="workload1", choices=sorted(WORKLOAD_PHOTONS))
    ap.add_argument("--photons", type=float, default=0)
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-scale", type=float, default=0.1, help="photon-budget scale of the batched workload")
    ap.add_argument("--streams", type=int, default=16, help="streams of the batched workload's graph")
    ap.add_argument("--ref-sample", type=int, default=16, help="batch instances the reference arm runs")
    ap.add_argument("--no-detectors", action="store_true",
                    help="drop the deck's detectors (measures the cost of detected-photon bookkeeping)")
    ap.add_argument("--judge-photons", type=float, default=1e9, help="photons of the denoise workload's judge runs")
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.workload == "denoise" and args.impl != "reference":
        denoise_main(args, world, rank)
        return
    if args.workload == "batch" and args.impl != "reference":
        batch_main(args, world, rank)
        return
    if args.workload == "contest" and args.impl != "reference":
        contest_main(args, world, rank)
        return

    if args.impl == "reference":
        reference_arm(args, world, rank)
        return

    import ctypes as C

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import mcx_gb300
    from mcx_gb300 import Session
    from mcx_gb300._lib import lib

    name = args.workload
    nphoton = int(args.photons) if args.photons else WORKLOAD_PHOTONS[name]
    seed = 20251203
    cfg = make_cfg(name, nphoton, seed)
    if args.no_detectors:
        cfg.pop("detpos", None)
        cfg["issavedet"] = 0
    pc = mcx_gb300.prepare(cfg)
    sess = Session(pc, device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    base = rank * nphoton * (args.warmup + args.steps + 1)
    sess.autotune(nphoton)
    for i in range(args.warmup):
        sess.run(base + i * nphoton, nphoton, seed)
    sess.reset()
    kernel_ms = []
    barrier()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            kernel_ms.append(sess.run(base + (args.warmup + i) * nphoton, nphoton, seed))
        barrier()
        wall_ms = (time.perf_counter() - t0) * 1e3
    _, _, ndet, st = sess.read(with_field=False)
    sess.close()
    dev_ms = sum(kernel_ms)
    if world > 1:
        t = torch.tensor([dev_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_ms = float(t.item())
    value = nphoton * args.steps * world / dev_ms

    # end to end through the public API with host buffers
    e2e_ms = []
    h2d = d2h = 0
    for i in range(1 + args.steps):
        c = make_cfg(name, nphoton, seed + 1 + i)
        if args.no_detectors:
            c.pop("detpos", None)
            c["issavedet"] = 0
        barrier()
        t0 = time.perf_counter()
        r = mcx_gb300.run(c)
        barrier()
        if i:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
        nvox = int(np.prod(c["vol"].shape))
        h2d = nvox * 4 + np.asarray(c["prop"]).nbytes + (np.asarray(c["detpos"]).nbytes if "detpos" in c else 0)
        d2h = r["flux"].nbytes + (r["detp"].nbytes if "detp" in r else 0)
    e2e_tot = sum(e2e_ms)
    if world > 1:
        t = torch.tensor([e2e_tot], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_tot = float(t.item())
    e2e = nphoton * args.steps * world / e2e_tot

    pk = peaks()
    clocks = clk.summary()
    props = torch.cuda.get_device_properties(local)
    f_clk = (clocks["sm_mhz"] or pk.get("sm_max_mhz", 2070.0)) * 1e6
    rate = C.c_double(0.0)
    nvox = int(np.prod(cfg["vol"].shape)) * pc.ngates
    lib.mcxg_probe_atomic_rate(max(nvox, 1 << 20), C.byref(rate))
    roof = roofline(name, value, world, st, f_clk, props.multi_processor_count, rate.value, pk)

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    line = {
        "metric": METRIC, "value": value, "unit": "photons/ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(name, cfg, nphoton, world),
        "launch": {"grid": st.grid, "block": st.block, "chunk": st.chunk},
        "e2e": {"value": e2e, "unit": "photons/ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": e2e_tot / args.steps},
        "wall_ms_per_step": wall_ms / args.steps,
        "gpu_launches": args.steps,
        "detected_per_step": ndet / max(1, args.steps),
        "roofline": roof,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(name, args.cpu_sample or CPU_SAMPLE[name])
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
