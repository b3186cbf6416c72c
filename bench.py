#!/usr/bin/env python
"""bench.py — segmentNuclei throughput (Mpixel/s) on one GB300.

Workload: the batched-tile configuration — 256 synthetic H&E tiles of uneven
size (squares 512-4096 px plus ragged slide-edge tiles 4096 x r / r x 4096),
generated on the device from fixed seeds (nscale_gb300/synth_torch.py; the
reference's validation slides are not available).  One step = the full
segmentNuclei pipeline over every tile of the batch through libnsg.so, inputs
resident in HBM.  Inputs (1.9 Gpixel, 5.6 GB) are far larger than L2.

Prints ONE JSON line (rank 0).  `--impl reference` times the reference's CPU
segmentNuclei path instead: the CPU oracle (a restatement of the reference;
the reference itself needs OpenCV 2.4, which is absent) on the host cores.

Multi-GPU (torchrun): replicas — every rank runs its own batch (seeds offset
by rank), no collective on the data path; value = all ranks' pixels / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "segmentNuclei Mpixel/s on 1 GB300, batched vs per-tile; p50/p99 tile latency"
# algorithmic bytes per pixel of each pipeline stage (read each input once,
# write each output once at native width; pointwise work fused)
STAGE_BYTES = {"background": 7, "RBC": 4, "open19": 4, "reconToNuclei": 6, "fillHoles1": 2,
               "areaThreshold1": 14, "blobsGt45": 4, "fillHoles2": 2, "openBlobs": 4, "30To1000": 14,
               "dilate": 2, "distTransform": 5, "imhmin": 8, "watershed": 40, "20To1000": 14,
               "fillHolesLast": 2, "bwlabel2": 5, "bounding_box": 4, "other": 0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="nsg", choices=["nsg", "reference"])
    ap.add_argument("--tiles", type=int, default=256)
    ap.add_argument("--streams", type=int, default=8,
                    help="tiles in flight: host threads, each with its own context and CUDA stream")
    ap.add_argument("--cpu-sample-tiles", type=int, default=0, help="tiles in the CPU baseline sample (0 = cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if args.impl == "reference" else "nccl")
    return rank, world, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sms.append(float(parts[1]))
                    mx = float(parts[2])
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sms)}


def make_batch(n_tiles, seed_base, device):
    from nscale_gb300 import synth_torch
    shapes = synth_torch.batch_shapes(n_tiles)
    tiles = [synth_torch.he_tile(r, c, seed_base + i, device=device) for i, (r, c) in enumerate(shapes)]
    return tiles


def cpu_worker(args):
    """One oracle segmentNuclei (spawned process)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    tile = np.frombuffer(args[0], dtype=np.uint8).reshape(args[1], args[2], 3)
    t = time.perf_counter()
    oracle.segment_nuclei(tile)
    return time.perf_counter() - t


def cpu_throughput(tiles_np, procs):
    """Oracle segmentNuclei over `tiles_np` with `procs` spawned workers;
    returns (Mpixel/s, wall seconds)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    payload = [(t.tobytes(), t.shape[0], t.shape[1]) for t in tiles_np]
    px = sum(t.shape[0] * t.shape[1] for t in tiles_np)
    with ctx.Pool(procs) as pool:
        pool.map(cpu_worker, payload[:procs])  # warm the workers (imports, oracle build check)
        t = time.perf_counter()
        pool.map(cpu_worker, payload)
        wall = time.perf_counter() - t
    return px / wall / 1e6, wall


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path (oracle restatement) on the
    host cores, same metric and workload shapes, bounded sample per step."""
    import numpy as np
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build(ref=False)
    from nscale_gb300 import synth_torch
    cores = os.cpu_count() or 1
    shapes = synth_torch.batch_shapes(args.tiles)
    # bounded sample: `cores` tiles of the batch's size mix (the first tiles of
    # the batch order, which mixes square and edge shapes)
    n = args.cpu_sample_tiles or cores
    sample = [synth_torch.he_tile(r, c, 0x5EED0003 + i, device="cpu").numpy() for i, (r, c) in enumerate(shapes[:n])]
    px = sum(t.shape[0] * t.shape[1] for t in sample)
    vals = []
    for i in range(args.warmup + args.steps):
        v, wall = cpu_throughput(sample, min(cores, len(sample)))
        if i >= args.warmup:
            vals.append((v, wall))
    value = statistics.mean(v for v, _ in vals)
    ms = statistics.mean(w for _, w in vals) * 1e3
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mpixel/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"segmentNuclei, CPU oracle, {len(sample)} tiles of the 256-tile batch mix "
                                   f"({px / 1e6:.1f} Mpixel per step)", "tiles": len(sample),
                       "pixels_per_step": px},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mpixel/s", "cores": min(cores, len(sample)),
                             "kind": "port",
                             "sample": f"{len(sample)} tiles ({px / 1e6:.1f} Mpixel), one tile per process"},
            "e2e": {"value": round(value, 3), "unit": "Mpixel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_nsg(args, rank, world, local):
    import numpy as np
    import torch
    from nscale_gb300 import _lib
    from nscale_gb300.context import Context, ptr
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _lib.load()
    tiles = make_batch(args.tiles, 0x5EED0003 + 100003 * rank, dev)
    maxr = max(t.shape[0] for t in tiles)
    maxc = max(t.shape[1] for t in tiles)
    px = sum(t.shape[0] * t.shape[1] for t in tiles)
    params = _lib.SegParams()
    statuses = {}
    tile_ms = []

    class Worker:
        """One tile in flight: a context (workspace arena), a stream, label buffers."""

        def __init__(self):
            self.ctx = Context(maxr, maxc, local)
            self.stream = torch.cuda.Stream(device=dev)
            self.sh = C.c_void_p(self.stream.cuda_stream)
            self.labels = torch.empty(maxr * maxc, dtype=torch.int32, device=dev)
            self.host_lab = None
            self.cc = C.c_int(0)

    workers = [Worker() for _ in range(max(1, args.streams))]

    def run_tiles(fn, items, pool):
        """Hand `items` to the workers of `pool` (one host thread each) until all are done."""
        nxt = [0]
        lock = threading.Lock()
        errors = []

        def loop(w):
            try:
                with torch.cuda.stream(w.stream):
                    while True:
                        with lock:
                            i = nxt[0]
                            nxt[0] += 1
                        if i >= len(items):
                            return
                        fn(w, items[i])
            except Exception as e:  # noqa: BLE001 - re-raised on the main thread
                errors.append(e)

        ths = [threading.Thread(target=loop, args=(w,)) for w in pool]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        if errors:
            raise errors[0]

    def seg_device(w, t, record_latency=False):
        r, c = t.shape[0], t.shape[1]
        t0 = time.perf_counter()
        st = L.nsg_segment_nuclei(w.ctx.h, ptr(t), r, c, c * 3, C.byref(params), ptr(w.labels), None,
                                  C.byref(w.cc), None, w.sh)
        if st < 0:
            raise _lib.NsgError(st, w.ctx.last_error())
        if record_latency:
            w.stream.synchronize()
            tile_ms.append((time.perf_counter() - t0) * 1e3)
            statuses[st] = statuses.get(st, 0) + 1

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    main = torch.cuda.current_stream(dev)

    def timed(fn, items, n_steps):
        """CUDA-event time of n_steps passes over `items` on all workers."""
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(main)
        for w in workers:
            w.stream.wait_event(ev0)
        for _ in range(n_steps):
            run_tiles(fn, items, workers)
        for w in workers:
            main.wait_stream(w.stream)
        ev1.record(main)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1)

    for _ in range(args.warmup):
        run_tiles(seg_device, tiles, workers)
    torch.cuda.synchronize()
    for w in workers:
        L.nsg_context_set_timing(w.ctx.h, 1)
    barrier()
    launches0 = L.nsg_kernel_launches()
    with Clocks(local) as clk:
        total_ms = timed(seg_device, tiles, args.steps)
    launches = L.nsg_kernel_launches() - launches0
    barrier()
    stage_ms = [0.0] * 19
    for w in workers:
        sm = (C.c_double * 19)()
        calls = C.c_longlong(0)
        L.nsg_context_stage_times(w.ctx.h, sm, 19, C.byref(calls))
        L.nsg_context_set_timing(w.ctx.h, 0)
        for i in range(19):
            stage_ms[i] += sm[i]
    names = [L.nsg_stage_name(i).decode() for i in range(19)]
    # per-tile latency: one tile at a time on one worker (separate pass)
    run_tiles(lambda w, t: seg_device(w, t, record_latency=True), tiles, workers[:1])
    ms_step = total_ms / args.steps
    value_rank = px / (ms_step / 1e3) / 1e6
    if world > 1:
        import torch.distributed as dist
        tmax = torch.tensor([ms_step], dtype=torch.float64)
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        ms_step = float(tmax.item())
    value = world * px / (ms_step / 1e3) / 1e6

    # roofline: the stage with the most device time in the timed region
    per_stage = {names[i]: stage_ms[i] for i in range(19)}
    dom = max(per_stage, key=per_stage.get)
    dom_ms_per_step = per_stage[dom] / args.steps
    dom_bytes = STAGE_BYTES[dom] * px
    peak, peak_kind = peaks()
    achieved = dom_bytes / (dom_ms_per_step / 1e3) / 1e9 if dom_ms_per_step > 0 else 0.0

    # e2e: host (pinned) tiles through the public host entry point, labels read
    # back to pinned host memory; copies both ways inside the timed region
    e2e_tiles = tiles[: min(len(tiles), 64)]
    host_in = [t.cpu().pin_memory() for t in e2e_tiles]
    for w in workers:
        w.host_lab = torch.empty(maxr * maxc, dtype=torch.int32).pin_memory()
    e2e_px = sum(t.shape[0] * t.shape[1] for t in e2e_tiles)

    def seg_host(w, h):
        r, c = h.shape[0], h.shape[1]
        st = L.nsg_segment_nuclei_host(w.ctx.h, C.c_void_p(h.data_ptr()), r, c, C.byref(params),
                                       C.c_void_p(w.host_lab.data_ptr()), None, C.byref(w.cc), None, w.sh)
        if st < 0:
            raise _lib.NsgError(st, w.ctx.last_error())

    run_tiles(seg_host, host_in, workers)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run_tiles(seg_host, host_in, workers)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_value = world * e2e_px / e2e_s / 1e6

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        n = args.cpu_sample_tiles or cores
        sample = [t.cpu().numpy() for t in tiles[:n]]
        v, wall = cpu_throughput(sample, min(cores, len(sample)))
        spx = sum(t.shape[0] * t.shape[1] for t in sample)
        cpu = {"value": round(v, 3), "unit": "Mpixel/s", "cores": min(cores, len(sample)), "kind": "port",
               "sample": f"{len(sample)} tiles of the batch ({spx / 1e6:.1f} Mpixel), one tile per process, "
                         f"{wall:.1f} s"}

    if rank != 0:
        return
    lat = sorted(tile_ms)
    clk = clk.summary()
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mpixel/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"segmentNuclei over {len(tiles)} uneven synthetic H&E tiles "
                               f"(squares 512-4096 + ragged edge tiles), device-resident inputs",
                   "tiles": len(tiles), "pixels_per_step": px,
                   "form": f"per-tile calls, {len(workers)} tiles in flight (host threads, one context and "
                           f"stream each)",
                   "l2": "inputs larger than L2 (5.6 GB per step)", "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": round(lat[len(lat) // 2], 3), "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3)},
        "statuses": {str(k): v for k, v in statuses.items()},
        "stage_ms_per_step": {k: round(v / args.steps, 3) for k, v in per_stage.items() if v > 0},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": dom_bytes, "traffic": None},
        "e2e": {"value": round(e2e_value, 3), "unit": "Mpixel/s", "h2d_bytes_per_step": int(3 * e2e_px),
                "d2h_bytes_per_step": int(4 * e2e_px), "tiles": len(e2e_tiles)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_nsg(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
