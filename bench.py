#!/usr/bin/env python
"""bench.py — segmentNuclei throughput (Mpixel/s) on one GB300.

Workload: the batched-tile configuration — 256 synthetic H&E tiles of uneven
size (squares 512-4096 px plus ragged slide-edge tiles 4096 x r / r x 4096),
generated on the device from fixed seeds (nscale_gb300/synth_torch.py; the
reference's validation slides are not available).  One step = the full
segmentNuclei pipeline over every tile of the batch through libnsg.so's
batched entry point (nsg_segment_nuclei_batch: a pool of workers, each with
its own context and stream, keeps several tiles in flight), inputs resident in
HBM.  Inputs (1.9 Gpixel, 5.6 GB) are far larger than L2.  Also reported, on
the same tiles: plain per-tile calls on one stream (the batched speed-up),
per-stage times, the host-buffer end-to-end rate, and a parity check of the
batched labels against the oracle on the CPU-baseline sample; then the
serving form: Poisson arrivals of tiles cut from a synthetic 100000 x 80000
slide into the in-process server (nsg_server_*), swept over arrival rates,
with p50/p99 latency, throughput and shed requests per rate.

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
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# 32 hardware work queues for the tiles in flight (read when the CUDA context
# is created; nscale_gb300 sets the same default on import)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "segmentNuclei Mpixel/s on 1 GB300, batched vs per-tile; p50/p99 tile latency"
# algorithmic bytes per pixel of a tile that runs to SUCCESS: each spatial
# stage reads its inputs once and writes its outputs once at native width,
# pointwise work fused (front 7, RBC 4, open19 4, recon 6, fill 2, area-open
# 14, bwselect 4, fill 2, open 4, area-open 14, dilate 2, EDT 5, imhmin 8,
# minima 17, bwlabel 5, watershed 12, border+mask 6, area-open 14, fill 2,
# bwlabel 5)
ALG_BYTES_PER_PX = 137
# measured DRAM reads + writes per pixel of the same pipeline: ncu
# dram__bytes_read.sum + dram__bytes_write.sum summed over every kernel of
# one 4096 x 4096 tile run to SUCCESS (python -m nscale_gb300.tile_demo 4096,
# ncu --cache-control none: the caches as in a real run)
DRAM_BYTES_PER_PX = 384.7
# the dominant kernel (largest share of the batched step): the uint8 grey
# reconstruction.  The timed call is nscale's imreconstruct: init_min_u8
# (min(marker, mask) into the output) + recon_cta<uint8>.  Algorithmic bytes:
# marker, mask read once, output written once = 3 B/px.  DRAM bytes of that
# call on the 4096 x 4096 pipeline input, L2 flushed before each kernel (ncu
# --cache-control all): init_min_u8 33.6 MB + recon_cta 34.8 MB; with warm
# caches the two move 24.4 MB.
RECON_ALG_BYTES_PER_PX = 3
RECON_CALL_DRAM_BYTES = 68.4e6



def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="nsg", choices=["nsg", "reference"])
    ap.add_argument("--tiles", type=int, default=256)
    ap.add_argument("--streams", type=int, default=32,
                    help="tiles in flight: pool workers, each with its own context and CUDA stream")
    ap.add_argument("--autotune-tiles", type=int, default=96,
                    help="tiles of the batch the autotuner measures launch shapes on (0 = defaults)")
    ap.add_argument("--serve-requests", type=int, default=1000,
                    help="slide-tile requests per arrival rate in the serving sweep (0 = skip)")
    ap.add_argument("--serve-rates", default="50,100,200,500,1000,2000",
                    help="Poisson arrival rates to sweep, tiles/s (comma list)")
    ap.add_argument("--serve-distinct", type=int, default=64, help="distinct slide positions the requests visit")
    ap.add_argument("--serve-queue", type=int, default=128, help="waiting tiles before the server sheds")
    ap.add_argument("--serve-budget-gib", type=int, default=160, help="device memory the server's workers may hold")
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


def replica_rate(px_per_rank, ms_local, world, device=None):
    """Whole-job Mpixel/s of `world` replicas that each processed px_per_rank
    pixels: the job takes as long as its slowest rank (max over ranks; no
    other exchange).  Returns (Mpixel/s, ms of the slowest rank)."""
    ms = ms_local
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms_local], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return world * px_per_rank / (ms / 1e3) / 1e6, ms


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
        d = os.environ.get("NSG_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, f"nsg_clocks_{os.getpid()}.csv")

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


def labels_digest(status, labels) -> str:
    """Status and int32 label image of one tile as a short digest (parity
    check of the benchmarked tiles against the oracle's)."""
    import hashlib
    import numpy as np
    h = hashlib.sha256(str(int(status)).encode())
    h.update(np.ascontiguousarray(labels, dtype=np.int32).tobytes())
    return h.hexdigest()[:20]


def cpu_worker(args):
    """One oracle segmentNuclei (spawned process): (seconds, digest)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    tile = np.frombuffer(args[0], dtype=np.uint8).reshape(args[1], args[2], 3)
    t = time.perf_counter()
    st, lab, _, _, _ = oracle.segment_nuclei(tile)
    dt = time.perf_counter() - t
    return dt, labels_digest(st, lab)


def cpu_throughput(tiles_np, procs):
    """Oracle segmentNuclei over `tiles_np` with `procs` spawned workers;
    returns (Mpixel/s, wall seconds, per-tile digests)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    payload = [(t.tobytes(), t.shape[0], t.shape[1]) for t in tiles_np]
    px = sum(t.shape[0] * t.shape[1] for t in tiles_np)
    with ctx.Pool(procs) as pool:
        pool.map(cpu_worker, payload[:procs])  # warm the workers (imports, oracle build check)
        t = time.perf_counter()
        res = pool.map(cpu_worker, payload)
        wall = time.perf_counter() - t
    return px / wall / 1e6, wall, [d for _, d in res]


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
        v, wall, _ = cpu_throughput(sample, min(cores, len(sample)))
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
    from nscale_gb300.serving import TilePool
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _lib.load()
    tiles = make_batch(args.tiles, 0x5EED0003 + 100003 * rank, dev)
    maxr = max(t.shape[0] for t in tiles)
    maxc = max(t.shape[1] for t in tiles)
    px = sum(t.shape[0] * t.shape[1] for t in tiles)
    params = _lib.SegParams()
    main = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def event_time(fn):
        """CUDA-event time (ms) of a blocking host call: events on the main
        stream bracket the call, with the device synchronised on both sides."""
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(main)
        main.synchronize()
        fn()
        ev1.record(main)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1)

    # ---- batched form: every tile of the batch on the pool's workers --------
    tuning = None
    if args.autotune_tiles > 0:
        # launch shapes picked on calibration tiles that are not the timed
        # batch (same generator and size mix, other seeds); the choice is
        # cached per GPU and tile-size mix.  Results do not depend on it.
        from nscale_gb300.autotune import autotune
        calib = make_batch(args.autotune_tiles, 0x5EEDCA11, dev)
        tuning = autotune(calib, device=local)
        del calib
        args.streams = tuning["workers"]
    else:
        from nscale_gb300.autotune import max_workers
        args.streams = min(args.streams, max_workers(maxr, maxc, local))
    pool = TilePool(maxr, maxc, workers=max(1, args.streams), device=local)
    if tuning:
        pool.set_tuning(tuning["recon_max_ctas"], tuning["bfs_max_cluster"], tuning["recon_wl_phases"])
    labels = [torch.empty(t.shape[0] * t.shape[1], dtype=torch.int32, device=dev) for t in tiles]
    arr = (_lib.Tile * len(tiles))()
    for i, t in enumerate(tiles):
        arr[i].bgr, arr[i].rows, arr[i].cols, arr[i].row_stride_bytes = t.data_ptr(), t.shape[0], t.shape[1], 0
        arr[i].labels, arr[i].mask, arr[i].want_bbox = labels[i].data_ptr(), None, 0
    for w in range(args.warmup):
        if w == args.warmup - 1:  # per-stage times under contention, from the last warm-up pass
            pool.set_timing(True)
        pool.run(arr, params)
    batched_stages, batched_timed = pool.stage_times()
    pool.set_timing(False)
    barrier()
    launches0 = L.nsg_kernel_launches()
    with Clocks(local) as clk:
        total_ms = event_time(lambda: [pool.run(arr, params) for _ in range(args.steps)])
    launches = L.nsg_kernel_launches() - launches0
    barrier()
    statuses = {}
    for i in range(len(tiles)):
        statuses[arr[i].status] = statuses.get(arr[i].status, 0) + 1
    value, ms_step = replica_rate(px, total_ms / args.steps, world, dev)

    # ---- e2e: the same tiles from pinned host memory, labels back to pinned
    # host memory, through the same batched entry point; copies inside the
    # timed region
    host_in = [t.cpu().pin_memory() for t in tiles]
    host_lab = [torch.empty(t.shape[0] * t.shape[1], dtype=torch.int32).pin_memory() for t in tiles]
    harr = (_lib.Tile * len(host_in))()
    for i, h in enumerate(host_in):
        harr[i].bgr, harr[i].rows, harr[i].cols, harr[i].row_stride_bytes = h.data_ptr(), h.shape[0], h.shape[1], 0
        harr[i].labels, harr[i].mask, harr[i].want_bbox = host_lab[i].data_ptr(), None, 0
    pool.run(harr, params, host=True)
    e2e_steps = max(1, min(args.steps, 3))
    e2e_ms = event_time(lambda: [pool.run(harr, params, host=True) for _ in range(e2e_steps)]) / e2e_steps
    e2e_value, _ = replica_rate(px, e2e_ms, world, dev)
    pool.close()

    # ---- per-tile form: the same tiles one call at a time on one stream,
    # with per-stage CUDA-event timing (the stage table below)
    ctx = Context(maxr, maxc, local)
    stream = torch.cuda.Stream(device=dev)
    sh = C.c_void_p(stream.cuda_stream)
    lab1 = torch.empty(maxr * maxc, dtype=torch.int32, device=dev)
    cc = C.c_int(0)
    tile_ms = []

    def per_tile(record=False):
        for t in tiles:
            t0 = time.perf_counter()
            st = L.nsg_segment_nuclei(ctx.h, ptr(t), t.shape[0], t.shape[1], t.shape[1] * 3, C.byref(params),
                                      ptr(lab1), None, C.byref(cc), None, sh)
            if st < 0:
                raise _lib.NsgError(st, ctx.last_error())
            if record:
                stream.synchronize()
                tile_ms.append((time.perf_counter() - t0) * 1e3)

    with torch.cuda.stream(stream):
        per_tile()
        L.nsg_context_set_timing(ctx.h, 1)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        per_tile()
        ev1.record(stream)
        torch.cuda.synchronize()
        pt_ms = ev0.elapsed_time(ev1)
        stage_ms = (C.c_double * 32)()
        calls = C.c_longlong(0)
        n_stages = L.nsg_context_stage_times(ctx.h, stage_ms, 32, C.byref(calls))
        L.nsg_context_set_timing(ctx.h, 0)
        per_tile(record=True)  # latency of one tile alone
    names = [L.nsg_stage_name(i).decode() for i in range(n_stages)]
    per_stage = {names[i]: stage_ms[i] for i in range(n_stages)}
    pt_value = px / (pt_ms / 1e3) / 1e6
    ctx.close()

    # ---- the dominant kernel alone: recon_cta<uint8> on the 4096^2
    # pipeline input (rc_open, rc of one tile), CUDA events on the stream it
    # is launched on
    kernel = dominant_kernel(local)

    # ---- serving: Poisson arrivals of slide tiles into the server -----------
    serving = None
    if rank == 0 and args.serve_requests > 0:
        serving = serve(args, local)

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        n = args.cpu_sample_tiles or cores
        sample = [t.cpu().numpy() for t in tiles[:n]]
        v, wall, digests = cpu_throughput(sample, min(cores, len(sample)))
        spx = sum(t.shape[0] * t.shape[1] for t in sample)
        cpu = {"value": round(v, 3), "unit": "Mpixel/s", "cores": min(cores, len(sample)), "kind": "port",
               "sample": f"{len(sample)} tiles of the batch ({spx / 1e6:.1f} Mpixel), one tile per process, "
                         f"{wall:.1f} s"}
        # the batched form's labels of the same tiles (last timed pass) against the oracle's
        bad = []
        for i in range(len(sample)):
            got = labels[i].view(tiles[i].shape[0], tiles[i].shape[1]).cpu().numpy()
            if arr[i].status != 0:
                got = np.full(got.shape, -1, np.int32)
            if labels_digest(arr[i].status, got) != digests[i]:
                bad.append(i)
        parity = {"tiles": len(sample), "mismatches": len(bad), "mismatched_tiles": bad,
                  "what": "status + int32 labels of the batched run vs the oracle, per tile (SHA-256)"}

    if rank != 0:
        return
    peak, peak_kind = peaks()
    achieved = value * ALG_BYTES_PER_PX / 1e3  # Mpixel/s x B/px -> GB/s
    lat = sorted(tile_ms)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mpixel/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"segmentNuclei over {len(tiles)} uneven synthetic H&E tiles "
                               f"(squares 512-4096 + ragged edge tiles), device-resident inputs",
                   "tiles": len(tiles), "pixels_per_step": px,
                   "form": f"batched: nsg_segment_nuclei_batch, {pool_workers(args)} tiles in flight "
                           f"(one context and stream per worker)",
                   "tuning": ({k: tuning[k] for k in ("workers", "recon_max_ctas", "bfs_max_cluster",
                                                     "recon_wl_phases")}
                              | {"picked_from": len(tuning["trials"]), "calibration_tiles": tuning["calibration_tiles"],
                                 "cached": tuning.get("cached", False)}
                              if tuning else "defaults"),
                   "l2": "inputs larger than L2 (5.6 GB per step)", "parallelism": f"replicas x{world}"},
        "per_tile": {"value": round(pt_value, 3), "unit": "Mpixel/s", "tiles": len(tiles),
                     "form": "nsg_segment_nuclei one tile at a time on one stream, the same tiles",
                     "batched_speedup": round(value / world / pt_value, 2)},
        "latency_ms": {"p50": round(lat[len(lat) // 2], 3),
                       "p99": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3),
                       "max": round(lat[-1], 3), "samples": len(lat),
                       "what": "one tile alone, per-tile form (host clock, submit to stream drained)"},
        "statuses": {str(k): v for k, v in statuses.items()},
        "stage_ms_per_tile_pass": {k: round(v, 3) for k, v in per_stage.items() if v > 0},
        "stage_ms_per_tile_batched": {k: round(v / max(1, batched_timed), 3)
                                      for k, v in batched_stages.items() if v > 0},
        "roofline": {"bound": "hbm", "kernel": kernel["kernel"], "achieved": kernel["achieved"], "peak": peak,
                     "unit": "GB/s", "frac": round(kernel["achieved"] / peak, 6), "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": kernel["alg_bytes"], "ms_per_launch": kernel["ms"],
                     "traffic": kernel["traffic"], "traffic_note": kernel["traffic_note"],
                     "why": "propagation-latency bound (winding single-pixel paths through noise; the tile "
                            "queue rescans lines), not bandwidth bound"},
        "roofline_pipeline": {"bound": "hbm", "kernel": "segmentNuclei pipeline, all stages (batched)",
                              "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                              "frac": round(achieved / peak, 5), "peak_kind": peak_kind,
                              "algorithmic_bytes_per_px": ALG_BYTES_PER_PX,
                              "traffic": int(DRAM_BYTES_PER_PX * px),
                              "traffic_note": f"DRAM bytes per step: {DRAM_BYTES_PER_PX} B/px measured by ncu over "
                                              f"all kernels of one 4096x4096 tile (warm caches), x pixels per step"},
        "e2e": {"value": round(e2e_value, 3), "unit": "Mpixel/s", "h2d_bytes_per_step": int(3 * px),
                "d2h_bytes_per_step": int(4 * px), "tiles": len(tiles),
                "form": "the same tiles from pinned host memory through nsg_segment_nuclei_batch (NSG_TILE_HOST)"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if parity:
        line["parity"] = parity
    if serving:
        line["serving"] = serving
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def dominant_kernel(device):
    """recon_cta<uint8> on the reconstruction input of one 4096 x 4096 tile
    (marker = open(255 - R, disk19), mask = 255 - R): mean of 5 launches
    timed with CUDA events on the stream the kernel runs on, after 3 warm-up
    launches.  Achieved = algorithmic bytes (3 B/px) / launch time."""
    import torch
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth_torch
    img = synth_torch.he_tile(4096, 4096, 0x5EED0000, device=f"cuda:{device}")
    rc = (255 - img[..., 2]).contiguous()
    rc_open = MO.morphOpen(rc, MO.disk19().numpy())
    stream = torch.cuda.current_stream(device)  # the library launches on the caller's stream
    for _ in range(3):
        MO.imreconstruct(rc_open, rc, 8)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(5):
        MO.imreconstruct(rc_open, rc, 8)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / 5
    px = rc.numel()
    alg = RECON_ALG_BYTES_PER_PX * px
    traffic = int(RECON_CALL_DRAM_BYTES) if px == 4096 * 4096 else None
    return {"kernel": "imreconstruct<uint8> call = recon_cta<uint8> + its min(marker, mask) init "
                      "(4096x4096 pipeline input)",
            "ms": round(ms, 3), "alg_bytes": alg, "achieved": round(alg / (ms / 1e3) / 1e9, 3),
            "traffic": traffic,
            "traffic_note": ("DRAM bytes per call: ncu dram__bytes_read.sum + dram__bytes_write.sum of init_min_u8 + "
                             "recon_cta<uint8> on this 4096x4096 input, L2 flushed before each kernel (24.4 MB with "
                             "warm caches)" if traffic else "not captured")}


def pool_workers(args):
    return max(1, args.streams)


def serve(args, device):
    """Serving form on the slide workload: tile requests cut from a synthetic
    100000 x 80000 slide (4096-px tiles, ragged right / bottom edges, 20 %
    tissue-free), Poisson arrivals at each rate of --serve-rates, at least
    --serve-requests requests per rate.  The server's workers are in two size
    classes (full 4096 x 4096 tiles and edge tiles up to 4096 x 2176 / 1696 x
    4096), bought from a device-memory budget; a full queue (--serve-queue
    waiting tiles) rejects a request, which is counted as shed.  Each result
    carries the per-nucleus features of its H channel.  Latency = submit ->
    result, over the admitted requests."""
    import random
    import numpy as np
    import torch
    from nscale_gb300 import _lib
    from nscale_gb300.serving import TileServer
    from nscale_gb300.slide import SyntheticSlide
    slide = SyntheticSlide(80000, 100000, 4096, seed=0x5EED0004)
    # the distinct tile positions the request stream visits, cut from the
    # slide before the timed runs (pinned host buffers, as a tiler would hand
    # them over); requests cycle over them in a shuffled order
    rng = random.Random(0x5EED0004)
    positions = [slide.position(k) for k in range(len(slide))]
    rng.shuffle(positions)
    positions = positions[: args.serve_distinct]
    host = []
    for (i, j) in positions:
        t = slide.tile(i, j, device=f"cuda:{device}")
        host.append(t.cpu().pin_memory().numpy())
        del t
    torch.cuda.synchronize()
    L = _lib.load()
    edge = (max(slide.rows - (slide.grid[0] - 1) * 4096, slide.cols - (slide.grid[1] - 1) * 4096), 4096)
    classes = [(4096, 4096), (4096, max(edge[0], 2176))]  # full tiles; ragged edge tiles (either orientation)
    # weights ~ the share of request pixels of each class
    full = sum(1 for h in host if h.shape[0] == 4096 and h.shape[1] == 4096)
    weights = [max(1.0, full), max(1.0, len(host) - full)]
    budget = args.serve_budget_gib << 30
    srv = TileServer(0, 0, budget, queue_cap=args.serve_queue, device=device, classes=classes, weights=weights)
    workers = srv.workers
    class_workers = {f"{r}x{c}": n for (r, c), n in srv.class_workers().items()}
    # warm-up: every worker runs tiles once (first-use set-up stays out of the latencies)
    warm = min(len(host), 2 * workers)
    for h in host[:warm]:
        srv.submit(h, None, want_features=True)
    got = 0
    while got < warm:
        got += len(srv.poll(64, 100))
    runs = []
    n_req = args.serve_requests
    for rate in [float(x) for x in str(args.serve_rates).split(",") if x]:
        arrivals = random.Random(int(rate) * 7919)
        results, shed = [], 0
        t0 = time.perf_counter()
        due = t0
        for k in range(n_req):
            due += arrivals.expovariate(rate)
            while True:
                now = time.perf_counter()
                if now >= due:
                    break
                results += srv.poll(64, 0)
                time.sleep(min(0.0005, due - now))
            try:
                srv.submit(host[k % len(host)], None, want_features=True)
            except _lib.NsgError as e:
                if e.code != _lib.ERR_QUEUE_FULL:
                    raise
                shed += 1
        while len(results) < n_req - shed:
            results += srv.poll(64, 100)
        wall = time.perf_counter() - t0
        lat = sorted(r["latency_ms"] for r in results)
        st = {}
        for r in results:
            st[str(r["status"])] = st.get(str(r["status"]), 0) + 1
        done_px = sum(host[k % len(host)].shape[0] * host[k % len(host)].shape[1] for k in range(len(results)))
        nfeat = sum(len(r["features"]) for r in results if r["features"] is not None)
        runs.append({"offered_tiles_per_s": rate, "requests": n_req, "admitted": len(results), "shed": shed,
                     "achieved_tiles_per_s": round(len(results) / wall, 2),
                     "achieved_mpx_s": round(done_px / wall / 1e6, 2),
                     "p50_ms": round(lat[len(lat) // 2], 3) if lat else None,
                     "p99_ms": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3) if lat else None,
                     "statuses": st, "nuclei_with_features": nfeat})
    srv.close()
    return {"slide": f"{slide.cols}x{slide.rows} synthetic, {slide.tile_size}-px tiles "
                     f"({slide.grid[1]}x{slide.grid[0]} grid, ragged edges, {slide.tissue_free:.0%} tissue-free), "
                     f"{len(host)} distinct positions cut before the runs",
            "arrivals": "poisson", "workers": workers, "class_workers": class_workers,
            "budget_gib": args.serve_budget_gib, "queue_cap": args.serve_queue,
            "policy": "admit while fewer than queue_cap tiles wait, else shed (submit returns NSG_ERR_QUEUE_FULL); "
                      "a worker takes the oldest waiting tile of its size class first",
            "output": "per-nucleus area, perimeter, mean/std H, mean gradient",
            "runs": runs}


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
