"""Pipeline ingest benchmark (one JSON line on stdout).

Default workload (the served form against the plain one): 16 requests
drawn (seeded) from four shapes -- the 256^3 u16 cube appended frame by
frame, 2304 x 4096 u16 sensor frames (x32), 512^2 x 64 f32 stacks (x4),
1024^2 u8 frames (x256) -- LZ4 / zstd-1 alternating, every other request
with a 4-level mean pyramid, seeded synthetic data (4.8 GB per pass).
  * served: a chucky_server (include/chucky_serve.h) with a 48 GB HBM
    admission budget, up to 16 requests open at once, encoders batched
    across streams; all 16 requests queued at once;
  * plain: the same requests one at a time (max_streams 1, each stream
    encoding on its own), appended as fast as possible.
One step = one pass over the 16 requests (the request loop runs in C, one
host thread per admitted request).  `value` / `e2e`: served GB/s of input
with the inputs resident in HBM (stream-ordered device appends) / in pinned
host memory (host-to-device copies inside the timed region); the plain form
and the ratio beside them; p50 / p99 append-to-delivered latency per epoch
from a pass with Poisson arrivals (mean gap 20 ms) and Poisson appends
(mean gap 0.5 ms).
  orca_e2e: one Orca-shaped stream -- 2304 x 4096 u16 frames, chunk
    32 x 256 x 256, 5-level (t, y, x) max pyramid with dim-0 downsampling,
    zstd-1 -- appended frame by frame from pinned host memory, as a
    fraction of the pinned host-to-device link measured in the same run.
  roofline: the dominant kernel set (the LZ4 encoder on sensor chunks)
    timed alone with CUDA events (chucky_encode_chunks).

Other workloads (`--workload`): multiscale (the 256^3 u16 + f32 pair,
zstd-3), cube-lz4, sensor-zstd / sensor-lz4, batched (five rank-5 arrays).

--impl reference times the CPU oracle of the same path (the reference's CPU
algorithm restated in oracle/, LZ4-HC / zstd from the system libraries) on
all host cores, on a bounded sample of the same workload (one request of
each shape per step).

Under torchrun (N > 1) every rank runs an independent replica ("replicas
only": the path has no exchange step); value = all ranks' bytes / max time.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np

from chucky_gb300 import capi

SIDE = 256
CHUNK = 64
METRIC = ("pipeline ingest GB/s (batched vs plain, 1 GB300, bit-exact round-trip); "
          "p99 latency")


def make_cubes(seed=7):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(SIDE), np.arange(SIDE), np.arange(SIDE),
                          indexing="ij")
    u16 = (((x ^ y ^ z) * 257 + rng.integers(0, 16, size=x.shape)) % 65536).astype("<u2")
    f32 = (np.sin(0.05 * x) * np.cos(0.07 * y) * z / 256.0
           + rng.normal(0, 0.01, size=x.shape)).astype("<f4")
    return u16, f32


# Epochs per batch.  The cubes go one 64-slice epoch per batch (four
# batches per array and step: each batch's encoders overlap the next one's
# LOD, its copy to the host the next one's encoders; measured faster than
# two or four epochs per batch); the larger workloads two.
_K_ENV = os.environ.get("CHUCKY_BENCH_EPOCHS_PER_BATCH")
CUBE_EPOCHS_PER_BATCH = int(_K_ENV or "1")
EPOCHS_PER_BATCH = int(_K_ENV or "2")


def make_config(dtype, reduce):
    dims = capi.make_dims([dict(size=SIDE, chunk=CHUNK, cps=4, downsample=1, name=n)
                           for n in "zyx"])
    cfg = capi.make_config(dims, dtype=dtype, codec="zstd", level=3, reduce=reduce,
                           append_reduce="mean", max_nlod=4,
                           epochs_per_batch=CUBE_EPOCHS_PER_BATCH,
                           buffer_capacity_bytes=128 << 20)
    cfg._dims = dims
    return cfg


WORKLOAD = ("256^3 u16 (mean LOD) + 256^3 f32 (median LOD), chunk 64^3, shard "
            "4^3 chunks, 2x2x2 pyramid (3 levels), zstd-3, K=%d epochs per batch "
            "(%d batches per array), discard sink"
            % (CUBE_EPOCHS_PER_BATCH, 4 // CUBE_EPOCHS_PER_BATCH))

# Further workloads (`--workload`), each printing its own line.
SENSOR_H, SENSOR_W = 2304, 4096


def sensor_frames(nframes, dev, seed=11):
    """u16 sensor frames 2304 x 4096: Poisson(100) background plus 64 seeded
    2-D Gaussian blobs (sigma 4-20 px, peak 500-4000), clipped to 12 bits.
    Generated on the device (seeded torch generator); returns an int16
    (nframes, H, W) device tensor whose bytes are the u16 little-endian
    frames (values <= 4095)."""
    import torch
    rng = np.random.default_rng(seed)
    yy = torch.arange(SENSOR_H, device=dev, dtype=torch.float32)[:, None]
    xx = torch.arange(SENSOR_W, device=dev, dtype=torch.float32)[None, :]
    rate = torch.full((SENSOR_H, SENSOR_W), 100.0, device=dev)
    for _ in range(64):
        cy, cx = rng.uniform(0, SENSOR_H), rng.uniform(0, SENSOR_W)
        s, a = rng.uniform(4, 20), rng.uniform(500, 4000)
        rate += a * torch.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * s * s))
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    out = torch.empty((nframes, SENSOR_H, SENSOR_W), dtype=torch.int16, device=dev)
    for f0 in range(0, nframes, 16):
        n = min(16, nframes - f0)
        r = rate.expand(n, SENSOR_H, SENSOR_W).contiguous()
        out[f0:f0 + n] = torch.poisson(r, generator=g).clamp_(max=4095).to(torch.int16)
    return out


def sensor_config(codec, reduce):
    """Unbounded dim 0 (chunk 32 frames), chunk 32 x 256 x 256, shard
    32 x 2048 x 2048, (t, y, x) pyramid of 5 levels with dim-0
    downsampling."""
    dims = capi.make_dims([
        dict(size=0, chunk=32, cps=1, downsample=1, name="t"),
        dict(size=SENSOR_H, chunk=256, cps=8, downsample=1, name="y"),
        dict(size=SENSOR_W, chunk=256, cps=8, downsample=1, name="x")])
    cfg = capi.make_config(dims, dtype="u16", codec=codec, level=1, reduce=reduce,
                           append_reduce=reduce, max_nlod=5,
                           epochs_per_batch=EPOCHS_PER_BATCH,
                           buffer_capacity_bytes=128 << 20)
    cfg._dims = dims
    return cfg


def cube_lz4_config():
    dims = capi.make_dims([dict(size=SIDE, chunk=CHUNK, cps=4, name=n) for n in "zyx"])
    cfg = capi.make_config(dims, dtype="u16", codec="lz4", level=1,
                           epochs_per_batch=CUBE_EPOCHS_PER_BATCH,
                           buffer_capacity_bytes=128 << 20)
    cfg._dims = dims
    return cfg


# rank-5 (t, c, z, y, x) arrays of 3 x 128 x 512 x 512 per time point,
# t scaled per dtype so that every array holds 768 MiB
BATCHED_DTYPES = (("u8", 8, "max_sup"), ("i16", 4, "min_sup"), ("u16", 4, "max_sup"),
                  ("f16", 4, "min_sup"), ("f32", 2, "max_sup"))


def batched_config(dtype, t, reduce):
    """Chunk 1x1x32x128x128, shard 1x1x4x4x4 chunks, (z, y, x) pyramid
    (4 levels asked; the level rule of the planner gives 3), zstd-1."""
    dims = capi.make_dims([
        dict(size=t, chunk=1, cps=1, name="t"),
        dict(size=3, chunk=1, cps=1, name="c"),
        dict(size=128, chunk=32, cps=4, downsample=1, name="z"),
        dict(size=512, chunk=128, cps=4, downsample=1, name="y"),
        dict(size=512, chunk=128, cps=4, downsample=1, name="x")])
    cfg = capi.make_config(dims, dtype=dtype, codec="zstd", level=1, reduce=reduce,
                           append_reduce=reduce, max_nlod=4,
                           epochs_per_batch=EPOCHS_PER_BATCH,
                           buffer_capacity_bytes=128 << 20)
    cfg._dims = dims
    return cfg


def batched_array(dtype, t, dev, seed=13):
    """Chunk classes by a seeded hash of the chunk index: half all-zero, a
    quarter one constant value, a quarter uniform random (compressed sizes
    spread over more than 100x).  Returns the device tensor."""
    import torch
    tdt = {"u8": torch.uint8, "i16": torch.int16, "u16": torch.int16,
           "f16": torch.float16, "f32": torch.float32}[dtype]
    out = torch.zeros((t, 3, 128, 512, 512), dtype=tdt, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    rng = np.random.default_rng(seed)
    for ti in range(t):
        for ci in range(3):
            for cz in range(4):
                for cy in range(4):
                    for cx in range(4):
                        u = rng.random()
                        if u < 0.5:
                            continue
                        view = out[ti, ci, cz * 32:(cz + 1) * 32, cy * 128:(cy + 1) * 128,
                                   cx * 128:(cx + 1) * 128]
                        if u < 0.75:
                            view.fill_(int(rng.integers(1, 100)))
                        elif tdt.is_floating_point:
                            view.copy_(torch.rand(view.shape, generator=g, device=dev,
                                                  dtype=torch.float32).to(tdt))
                        else:
                            bits = 8 if tdt == torch.uint8 else 16
                            r = torch.randint(0, 1 << bits, view.shape, generator=g,
                                              device=dev, dtype=torch.int32)
                            if bits == 16:
                                r = r - (1 << 15)
                            view.copy_(r.to(tdt))
    return out


def make_workload(name, dev, frames):
    """(description, data note, dtype, [(config, pinned host bytes, device
    bytes)], encoder name) of a workload."""
    import torch

    def pair(dbuf):
        dbuf = dbuf.reshape(-1).view(torch.uint8)
        host = torch.empty(dbuf.numel(), dtype=torch.uint8, pin_memory=True)
        host.copy_(dbuf)
        return host, dbuf

    if name == "multiscale":
        u16, f32 = make_cubes()
        arrays = []
        for cube, cfg in ((u16, make_config("u16", "mean")), (f32, make_config("f32", "median"))):
            host = torch.from_numpy(cube.reshape(-1).view(np.uint8)).pin_memory()
            arrays.append((cfg, host, host.to(dev)))
        return (WORKLOAD, "synthetic (seeded xor+noise u16 cube, sin*cos f32 cube + N(0,0.01))",
                "u16+f32", arrays, "zstd encoder (find+table+block+frame)")
    if name == "cube-lz4":
        u16, _ = make_cubes()
        host = torch.from_numpy(u16.reshape(-1).view(np.uint8)).pin_memory()
        desc = ("256^3 u16, chunk 64^3, shard 4^3 chunks (one shard), no LOD, LZ4, "
                "K=%d epochs per batch, discard sink" % CUBE_EPOCHS_PER_BATCH)
        return (desc, "synthetic (seeded xor+noise u16 cube)", "u16",
                [(cube_lz4_config(), host, host.to(dev))], "lz4 encoder (find+plan+emit)")
    if name in ("sensor-zstd", "sensor-lz4"):
        codec = name.split("-")[1]
        host, dbuf = pair(sensor_frames(frames, dev))
        desc = ("%d u16 frames 2304x4096 along unbounded dim 0, chunk 32x256x256, shard "
                "32x2048x2048, (t,y,x) max pyramid (5 levels, dim-0 downsampling), %s, "
                "K=%d epochs per batch, discard sink"
                % (frames, "zstd-1" if codec == "zstd" else "LZ4", EPOCHS_PER_BATCH))
        enc = ("zstd encoder (find+table+block+frame)" if codec == "zstd"
               else "lz4 encoder (find+plan+emit)")
        return (desc, "synthetic (seeded Poisson(100) + 64 Gaussian blobs, 12-bit; "
                "generated on the device)", "u16",
                [(sensor_config(codec, "max"), host, dbuf)], enc)
    if name == "batched":
        arrays = []
        for dt, t, red in BATCHED_DTYPES:
            host, dbuf = pair(batched_array(dt, t, dev))
            arrays.append((batched_config(dt, t, red), host, dbuf))
        desc = ("5 rank-5 (t,c,z,y,x) arrays t x 3 x 128 x 512 x 512, one per dtype "
                "(u8 t=8, i16 t=4, u16 t=4, f16 t=4, f32 t=2: 768 MiB each), chunk "
                "1x1x32x128x128, shard 1x1x4x4x4 chunks, (z,y,x) max_sup/min_sup pyramid "
                "(3 levels), half the chunks zero, a quarter constant, a quarter random, "
                "zstd-1, K=%d epochs per batch, one host thread per array, discard sink"
                % EPOCHS_PER_BATCH)
        return (desc, "synthetic (seeded chunk classes: zero / constant / uniform random)",
                "u8+i16+u16+f16+f32", arrays, "zstd encoder (find+table+block+frame)")
    raise ValueError(name)


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi",
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "20", "-i",
                 os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or "0"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            # the timed region starts once samples flow
            t0 = time.time()
            while not self.samples and time.time() - t0 < 5:
                time.sleep(0.01)
            self.samples.clear()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 6:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                pass
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[2 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def max_over_ranks(values, world, device):
    """Element-wise maximum of per-rank timings over all ranks (replicas:
    the job takes as long as its slowest rank)."""
    if world <= 1:
        return list(values)
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def h2d_probe(host, devbuf, dev, reps=3):
    """GB/s of plain pinned host -> device copies of the input buffers."""
    import torch
    s = torch.cuda.Stream(device=dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        e0.record(s)
        for _ in range(reps):
            for h, d in zip(host, devbuf):
                d.copy_(h, non_blocking=True)
        e1.record(s)
    s.synchronize()
    nbytes = reps * sum(h.numel() for h in host)
    return nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9


def whole_job_gbs(bytes_per_rank_step, steps, world, ms):
    """Input GB/s of the whole job: every rank ingests its own replica."""
    return bytes_per_rank_step * steps * world / (ms * 1e-3) / 1e9


def run_ours(args, rank, world):
    import torch
    import chucky_gb300 as cg
    from chucky_gb300 import build as cgbuild

    cgbuild.build()
    lib = cg.load()
    lib.chucky_discard_sink_create.restype = C.c_void_p
    lib.chucky_discard_sink_bytes.restype = C.c_uint64
    lib.chucky_discard_sink_bytes.argtypes = [C.c_void_p]
    lib.chucky_discard_sink_destroy.argtypes = [C.c_void_p]
    lib.tile_stream_gpu_restart.argtypes = [C.c_void_p, C.c_void_p]
    lib.chucky_launch_count.restype = C.c_uint64
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)

    desc, data_note, dtype_name, arrays, enc_name = make_workload(args.workload, dev,
                                                                  args.frames)
    host = [a[1] for a in arrays]
    devbuf = [a[2] for a in arrays]
    nbytes = sum(h.numel() for h in host)
    sink = lib.chucky_discard_sink_create()
    streams = [cg.GpuStream(a[0], sink) for a in arrays]
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step(bufs):
        for s, b in zip(streams, bufs):
            if lib.tile_stream_gpu_restart(s.h, None) != 0:
                raise RuntimeError("restart failed")
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0.record()
        # one host thread per array (the C API is single-threaded per stream;
        # streams are independent, so their GPU work overlaps)
        errs = []

        def run(s, b):
            r = s.append(b.data_ptr(), b.numel())
            if r.error:
                errs.append(f"append failed {r.error}")
                return
            r = s.flush()
            if r.error:
                errs.append(f"flush failed {r.error}")

        th = [threading.Thread(target=run, args=(s, b)) for s, b in zip(streams, bufs)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errs:
            raise RuntimeError("; ".join(errs))
        t1.record()
        torch.cuda.synchronize()
        return t0.elapsed_time(t1)

    def timed(bufs, k, w):
        for _ in range(w):
            step(bufs)
        base_metrics = [s.metrics() for s in streams]
        base_sink = lib.chucky_discard_sink_bytes(sink)
        base_launch = lib.chucky_launch_count()
        times = []
        for _ in range(k):
            flush_buf.fill_(1)  # evict L2 between steps
            times.append(step(bufs))
        end_metrics = [s.metrics() for s in streams]
        sink_b = (lib.chucky_discard_sink_bytes(sink) - base_sink) / k
        launches = lib.chucky_launch_count() - base_launch
        return times, base_metrics, end_metrics, sink_b, launches

    clocks = Clocks()
    if rank == 0:
        clocks.start()
    times_dev, m0, m1, sink_b, launches = timed(devbuf, args.steps, args.warmup)
    times_host, m0h, m1h, sink_h, launches_h = timed(host, args.steps, max(1, args.warmup // 2))
    clk = clocks.stop() if rank == 0 else None
    # the host link as the e2e leg sees it: plain copies of the same pinned
    # input buffers to the device, right after the timed region (the link
    # and host memory are shared with other tenants of the machine)
    link_gbs = h2d_probe(host, devbuf, dev)

    ms_dev, ms_host = max_over_ranks([float(np.sum(times_dev)), float(np.sum(times_host))],
                                     world, dev)
    value, e2e = (whole_job_gbs(nbytes, args.steps, world, ms) for ms in (ms_dev, ms_host))

    # dominant kernel: the zstd encoder (find + block + frame launches),
    # event-timed on its own stream inside the library
    comp_ms = sum(b.compress.ms - a.compress.ms for a, b in zip(m0, m1))
    comp_in = sum(b.compress.input_bytes - a.compress.input_bytes for a, b in zip(m0, m1))
    comp_launches = sum(b.compress.count - a.compress.count for a, b in zip(m0, m1))
    per_launch_ms = comp_ms / max(1, comp_launches)
    per_launch_bytes = comp_in / max(1, comp_launches)
    # DRAM bytes (read + written) per byte of encoder input, measured by ncu
    # on one batch of the u16 cube: 54.9 MB for 19.40 MB of chunk input
    traffic_per_input_byte = 2.83 if args.workload == "multiscale" else None
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    # algorithmic bytes of one encoder launch: chunk bytes read + compressed
    # bytes written (the compressed bytes are what the sink receives)
    launches_per_step = comp_launches / args.steps
    out_per_launch = sink_b / max(1.0, launches_per_step)
    achieved = ((per_launch_bytes + out_per_launch) / (per_launch_ms * 1e-3) / 1e9
                if per_launch_ms > 0 else 0.0)
    def stage_ms(a0, a1):
        out = {}
        for name in capi.METRIC_NAMES:
            ms = sum(getattr(b, name).ms - getattr(a, name).ms for a, b in zip(a0, a1))
            if ms > 0:
                out[name] = round(ms / args.steps, 4)
        return out

    stages, stages_e2e = stage_ms(m0, m1), stage_ms(m0h, m1h)

    for s in streams:
        s.close()
    lib.chucky_discard_sink_destroy(sink)
    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_dev / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype_name,
        "data": data_note,
        "config": {"workload": desc, "input_bytes_per_step": nbytes,
                   "l2": "flushed between steps (256 MiB write)",
                   "parallelism": f"replicas x{world}",
                   "stage_ms_per_step": stages},
        "e2e": {"value": round(e2e, 3), "unit": "GB/s",
                "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": int(sink_h),
                "ms_per_step": round(ms_host / args.steps, 4),
                "stage_ms_per_step": stages_e2e,
                # pinned H2D copies of the same input buffers, measured
                # right after the timed region
                "h2d_link_gbs": round(link_gbs, 2),
                "frac_of_h2d_link": round(e2e / link_gbs, 4) if link_gbs else None},
        # delivered chunk bytes (every pyramid level) / compressed shard bytes
        "compression_ratio": round(comp_in / args.steps / max(1.0, sink_b), 4),
        "roofline": {"kernel": enc_name, "bound": "hbm",
                     "achieved": round(achieved, 2), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_src,
                     "traffic": round(traffic_per_input_byte * per_launch_bytes)
                     if traffic_per_input_byte else None,
                     "traffic_note": "bytes per launch set, scaled by input bytes "
                                     "from the u16 ncu capture"
                     if traffic_per_input_byte else "not captured for this workload",
                     "input_gbs": round(per_launch_bytes / (per_launch_ms * 1e-3) / 1e9, 2)
                     if per_launch_ms > 0 else None},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if args.cpu_baseline and args.workload == "multiscale":
        line["cpu_baseline"] = cpu_baseline(args)
    return line


# ---------------------------------------------------------------------------
# The served form against the plain one (the default line)
# ---------------------------------------------------------------------------

ORCA_FRAMES = 512
SERVED_LINK_NOTE = ("pinned host->device copies of the same input buffers, measured "
                    "right after the timed region")


def _server_pass(srv, reqs, sink, paced=False):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    srv.replay(reqs, sink, paced=paced)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def timed_passes(srv, reqs, lib, sink, steps, warmup):
    """(ms per timed pass, discarded-sink bytes per pass, launches) of
    `steps` passes after `warmup` untimed ones."""
    for _ in range(warmup):
        srv.replay(reqs, sink, paced=False)
    srv.reset_stats()
    b0 = lib.chucky_discard_sink_bytes(sink)
    l0 = lib.chucky_launch_count()
    ms = [_server_pass(srv, reqs, sink) for _ in range(steps)]
    launches = lib.chucky_launch_count() - l0
    out_bytes = (lib.chucky_discard_sink_bytes(sink) - b0) / steps
    return ms, out_bytes, launches


def orca_e2e(lib, dev, steps):
    """The Orca-shaped sensor stream (zstd-1, 5-level dim-0 max pyramid),
    512 frames from pinned host memory, appended in pieces of 32 Mi
    elements as the reference's benchmark pumps its input
    (bench/bench_util.c:673, tests/test_data.c:138-160), and frame by
    frame."""
    import torch
    import chucky_gb300 as cg
    frames = sensor_frames(ORCA_FRAMES, dev)
    dbuf = frames.reshape(-1).view(torch.uint8)
    host = torch.empty(dbuf.numel(), dtype=torch.uint8, pin_memory=True)
    host.copy_(dbuf)
    sink = lib.chucky_discard_sink_create()
    s = cg.GpuStream(sensor_config("zstd", "max"), sink)
    frame = SENSOR_H * SENSOR_W * 2

    def one(piece):
        if lib.tile_stream_gpu_restart(s.h, None) != 0:
            raise RuntimeError("restart failed")
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        base = host.data_ptr()
        for a in range(0, host.numel(), piece):
            if s.append(base + a, min(piece, host.numel() - a)).error:
                raise RuntimeError("append failed")
        if s.flush().error:
            raise RuntimeError("flush failed")
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    pump = 32 << 21  # 32 Mi u16 elements
    for _ in range(2):
        one(pump)
    ms = [one(pump) for _ in range(steps)]
    ms_frames = [one(frame) for _ in range(max(2, steps // 2))]
    link = h2d_probe([host], [dbuf], dev)
    s.close()
    lib.chucky_discard_sink_destroy(sink)
    gbs = host.numel() * len(ms) / (sum(ms) * 1e-3) / 1e9
    gbs_frames = host.numel() * len(ms_frames) / (sum(ms_frames) * 1e-3) / 1e9
    out = {"workload": "%d u16 frames 2304x4096 (seeded Poisson(100) + 64 Gaussian blobs), "
                       "chunk 32x256x256, shard 32x2048x2048, 5-level (t,y,x) max pyramid "
                       "with dim-0 downsampling, zstd-1, K=%d, pinned host memory appended "
                       "in 64 MiB pieces (32 Mi elements, the reference benchmark's pump)"
                       % (ORCA_FRAMES, EPOCHS_PER_BATCH),
           "value": round(gbs, 3), "unit": "GB/s", "steps": len(ms),
           "frame_by_frame": round(gbs_frames, 3),
           "ms_per_step": round(float(np.mean(ms)), 3),
           "h2d_link_gbs": round(link, 2), "link_note": SERVED_LINK_NOTE,
           "frac_of_h2d_link": round(gbs / link, 4) if link else None}
    del frames, dbuf, host
    torch.cuda.empty_cache()
    return out


def cube_appends(lib, dev, steps):
    """The 256^3 u16 LZ4 cube (chunk 64^3, one shard, no pyramid) through
    writer_append from host memory in three ways: 256 appends of one
    256 x 256 frame from pinned memory and from pageable memory (both go
    through the stream's pinned staging ring), and the whole cube in one
    append from pageable memory (as the reference's benchmark pumps a
    malloc'd buffer).  GB/s of input, each way timed on the device around
    whole passes."""
    import torch
    import chucky_gb300 as cg
    u16, _ = make_cubes()
    pageable = np.ascontiguousarray(u16).view(np.uint8).reshape(-1)
    pinned = torch.from_numpy(pageable.copy()).pin_memory()
    sink = lib.chucky_discard_sink_create()
    s = cg.GpuStream(cube_lz4_config(), sink)
    frame = SIDE * SIDE * 2
    out = {}
    for name, base, step in (("frames_pinned", pinned.data_ptr(), frame),
                             ("frames_pageable", pageable.ctypes.data, frame),
                             ("whole_pageable", pageable.ctypes.data, pageable.size)):
        def one():
            if lib.tile_stream_gpu_restart(s.h, None) != 0:
                raise RuntimeError("restart failed")
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for a in range(0, pageable.size, step):
                if s.append(base + a, min(step, pageable.size - a)).error:
                    raise RuntimeError("append failed")
            if s.flush().error:
                raise RuntimeError("flush failed")
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)
        for _ in range(2):
            one()
        ms = [one() for _ in range(steps)]
        out[name] = round(pageable.size * len(ms) / (sum(ms) * 1e-3) / 1e9, 3)
    s.close()
    lib.chucky_discard_sink_destroy(sink)
    out["workload"] = ("256^3 u16 (xor + noise), chunk 64^3, one shard of 4^3 chunks, no "
                       "pyramid, LZ4, K=%d; frames = 256 appends of 256 x 256" %
                       CUBE_EPOCHS_PER_BATCH)
    out["unit"] = "GB/s"
    return out


def encoder_roofline(lib, dev, codec="lz4", reps=5, n=64, level=1):
    """The encoder launch set alone on one 256 MiB batch of sensor chunks
    (64 chunks of 32 x 256 x 256 u16), CUDA events on its stream: bytes
    read + written per launch set and the chunk-input rate."""
    import torch
    f = lib.chucky_encode_chunks
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t,
                  C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    lib.chucky_encode_bound.restype = C.c_size_t
    lib.chucky_encode_bound.argtypes = [C.c_int, C.c_size_t]
    lib.chucky_encode_scratch_bytes.restype = C.c_size_t
    lib.chucky_encode_scratch_bytes.argtypes = [C.c_int, C.c_int, C.c_size_t, C.c_size_t]
    cid = capi.CODEC[codec]
    frames = sensor_frames(64, dev)  # 64 frames: 2 epochs of 9 x 16 chunk tiles
    # chunk tiles 32 x 256 x 256 of the first 64 frames, as the stream lays them out
    t = frames.reshape(2, 32, 9, 256, 16, 256).permute(0, 2, 4, 1, 3, 5).contiguous()
    chunk_bytes = 32 * 256 * 256 * 2
    chunks = t.reshape(-1).view(torch.uint8)[: n * chunk_bytes]
    pad = torch.zeros(n * chunk_bytes + 256, dtype=torch.uint8, device=dev)
    pad[: n * chunk_bytes].copy_(chunks)
    bound = lib.chucky_encode_bound(cid, chunk_bytes)
    out_stride = (bound + 15) // 16 * 16
    out = torch.empty(n * out_stride, dtype=torch.uint8, device=dev)
    sizes = torch.zeros(n, dtype=torch.int64, device=dev)
    sb = lib.chucky_encode_scratch_bytes(cid, level, chunk_bytes, n)
    scratch = torch.empty(sb, dtype=torch.uint8, device=dev)
    st = torch.cuda.Stream(device=dev)
    times = []
    for r in range(reps + 2):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        rc = f(cid, level, pad.data_ptr(), chunk_bytes, chunk_bytes, n, out.data_ptr(),
               out_stride, sizes.data_ptr(), scratch.data_ptr(), sb, st.cuda_stream)
        e1.record(st)
        st.synchronize()
        if rc:
            raise RuntimeError("chucky_encode_chunks failed")
        if r >= 2:
            times.append(e0.elapsed_time(e1))
    comp = int(sizes.sum().item())
    ms = float(np.mean(times))
    del frames, t, chunks, pad, out, scratch
    torch.cuda.empty_cache()
    return {"input_bytes": n * chunk_bytes, "output_bytes": comp, "ms": ms,
            "ratio": n * chunk_bytes / max(comp, 1),
            "input_gbs": n * chunk_bytes / (ms * 1e-3) / 1e9,
            "achieved_gbs": (n * chunk_bytes + comp) / (ms * 1e-3) / 1e9}


# DRAM bytes (read + written) per byte of chunk input of the LZ4 launch set
# (find + emit) on sensor chunks, from one ncu capture of 48 chunks of
# 32 x 256 x 256 u16 (`--single encode-lz4`)
LZ4_SENSOR_TRAFFIC_PER_INPUT_BYTE = (209.0 + 268.5 + 527.8 + 144.2) / 201.3


def _stock_codecs():
    """liblz4 / libzstd, the reference CPU path's codecs
    (src/cpu/compress.c:55-93: LZ4_compress_HC and ZSTD_compress at the
    configured level)."""
    z = C.CDLL("libzstd.so.1")
    z.ZSTD_compressBound.restype = C.c_size_t
    z.ZSTD_compressBound.argtypes = [C.c_size_t]
    z.ZSTD_compress.restype = C.c_size_t
    z.ZSTD_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int]
    z.ZSTD_isError.argtypes = [C.c_size_t]
    l4 = C.CDLL("liblz4.so.1")
    l4.LZ4_compressBound.argtypes = [C.c_int]
    l4.LZ4_compress_HC.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]

    def zstd(x, level):
        cap = z.ZSTD_compressBound(len(x))
        buf = C.create_string_buffer(cap)
        k = z.ZSTD_compress(buf, cap, x, len(x), level)
        if z.ZSTD_isError(k):
            raise RuntimeError("ZSTD_compress failed")
        return k

    def lz4hc(x, level):
        cap = l4.LZ4_compressBound(len(x))
        buf = C.create_string_buffer(cap)
        k = l4.LZ4_compress_HC(x, buf, len(x), cap, level)
        if k <= 0:
            raise RuntimeError("LZ4_compress_HC failed")
        return k
    return zstd, lz4hc


def codec_ratios(lib, dev):
    """Compressed bytes of the 256^3 cubes' level-0 chunks (64^3, the
    multiscale and cube workloads' chunking) from this library's device
    encoders and from the reference CPU path's codecs at the same level:
    zstd-3 on the u16 and f32 cubes (the multiscale workload's codec), LZ4
    at levels 1 and 2 on the u16 cube (the cube workload's codec)."""
    import torch
    f = lib.chucky_encode_chunks
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t,
                  C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    lib.chucky_encode_bound.restype = C.c_size_t
    lib.chucky_encode_bound.argtypes = [C.c_int, C.c_size_t]
    lib.chucky_encode_scratch_bytes.restype = C.c_size_t
    lib.chucky_encode_scratch_bytes.argtypes = [C.c_int, C.c_int, C.c_size_t, C.c_size_t]
    zstd, lz4hc = _stock_codecs()
    u16, f32 = make_cubes()
    n = (SIDE // CHUNK) ** 3

    def tiles(a):
        t = a.reshape(SIDE // CHUNK, CHUNK, SIDE // CHUNK, CHUNK, SIDE // CHUNK, CHUNK)
        return np.ascontiguousarray(t.transpose(0, 2, 4, 1, 3, 5)).reshape(n, -1).view(np.uint8)

    def gpu_bytes(chunks, codec, level):
        cb = chunks.shape[1]
        cid = capi.CODEC[codec]
        d_in = torch.zeros(n * cb + 256, dtype=torch.uint8, device=dev)
        d_in[: n * cb] = torch.from_numpy(chunks.reshape(-1)).to(dev)
        stride = (lib.chucky_encode_bound(cid, cb) + 15) // 16 * 16
        out = torch.empty(n * stride, dtype=torch.uint8, device=dev)
        sizes = torch.zeros(n, dtype=torch.int64, device=dev)
        sb = lib.chucky_encode_scratch_bytes(cid, level, cb, n)
        scratch = torch.empty(sb, dtype=torch.uint8, device=dev)
        st = torch.cuda.current_stream(dev)
        if f(cid, level, d_in.data_ptr(), cb, cb, n, out.data_ptr(), stride,
             sizes.data_ptr(), scratch.data_ptr(), sb, st.cuda_stream):
            raise RuntimeError("chucky_encode_chunks failed")
        torch.cuda.synchronize(dev)
        return int(sizes.sum().item())

    def entry(chunks, codec, level, cpu):
        raw = chunks.size
        g = gpu_bytes(chunks, codec, level)
        c = sum(cpu(chunks[i].tobytes(), level) for i in range(n))
        return {"level": level, "input_bytes": int(raw), "gpu_bytes": g, "cpu_bytes": int(c),
                "gpu_ratio": round(raw / g, 4), "cpu_ratio": round(raw / c, 4),
                "gpu_over_cpu_bytes": round(g / c, 4)}

    t16, t32 = tiles(u16), tiles(f32)
    z16, z32 = entry(t16, "zstd", 3, zstd), entry(t32, "zstd", 3, zstd)
    both = {k: z16[k] + z32[k] for k in ("input_bytes", "gpu_bytes", "cpu_bytes")}
    return {
        "chunks": "the 256^3 cubes' 64 level-0 chunks of 64^3 each",
        "cpu_codec": "libzstd ZSTD_compress / liblz4 LZ4_compress_HC (the reference "
                     "CPU path's codecs) at the same level",
        "multiscale_zstd3": {"u16": z16, "f32": z32,
                             "both_gpu_over_cpu_bytes": round(both["gpu_bytes"] /
                                                              both["cpu_bytes"], 4)},
        "cube_lz4": {"level1": entry(t16, "lz4", 1, lz4hc),
                     "level2": entry(t16, "lz4", 2, lz4hc)},
    }


def autotune_table(lib):
    """The encoder autotuner's choices in this process (key -> parameters)."""
    lib.chucky_autotune_enabled.restype = C.c_int
    names = {v: k for k, v in capi.CODEC.items()}
    out = []
    for e in capi.autotune_entries(lib):
        out.append({"codec": names.get(e.codec, e.codec), "level": e.level,
                    "dtype": capi.DTYPES[e.dtype], "chunk": list(e.chunk_shape[:e.rank]),
                    "strength": e.strength or "default",
                    "min_match": e.min_match or "default",
                    "sample_gbs": round(e.encode_gbs, 1), "sample_ratio": round(e.ratio, 4),
                    "candidates": e.candidates})
    return {"enabled": bool(lib.chucky_autotune_enabled()), "entries": out}


def child_leg(name, args):
    """One single-stream leg (`--single orca-e2e` / `cube-appends`) run by
    this script in a child process; its JSON result."""
    import subprocess
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--single", name,
                        "--steps", str(max(3, args.steps // 2))],
                       capture_output=True, text=True, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError(f"{name} leg failed:\n{r.stderr[-2000:]}")
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_served_bench(args, rank, world):
    import torch
    import chucky_gb300 as cg
    from chucky_gb300 import build as cgbuild, serve
    cgbuild.build()
    lib = serve._lib()
    lib.tile_stream_gpu_restart.argtypes = [C.c_void_p, C.c_void_p]
    lib.chucky_launch_count.restype = C.c_uint64
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    # the Orca-shaped and cube legs in a child process, before this one pins
    # the served form's inputs: in-process after the served legs (4.8 GB of
    # their inputs still pinned) the same Orca-shaped stream measured 35-40 %
    # slower
    orca = child_leg("orca-e2e", args) if rank == 0 else None
    cube = child_leg("cube-appends", args) if rank == 0 else None
    sink = lib.chucky_discard_sink_create()
    import dataclasses
    host_reqs = serve.c5_requests()                   # pinned host inputs
    on_dev = {}
    for r in host_reqs:                               # HBM-resident copies
        if id(r.data) not in on_dev:
            on_dev[id(r.data)] = r.data.to(dev)
    dev_reqs = [dataclasses.replace(r, data=on_dev[id(r.data)], _cfg=None)
                for r in host_reqs]
    nbytes = sum(r.buffer()[1] for r in host_reqs)

    clocks = Clocks()
    # the served form: one server (start-up: a resident stream per request),
    # device-input passes, host-input passes, then the paced latency pass
    with serve.Server(48 << 30, 16, True, autotune=args.autotune,
                      batch_deadline_ms=args.batch_deadline_ms) as srv:
        srv.prewarm(host_reqs, sink, per_request=True)
        if rank == 0:
            clocks.start()
        ms_dev, out_b, launches = timed_passes(srv, dev_reqs, lib, sink, args.steps,
                                               args.warmup)
        st_dev = srv.stats()
        ms_host, out_h, _ = timed_passes(srv, host_reqs, lib, sink, args.steps,
                                         max(1, args.warmup // 2))
        clk = clocks.stop() if rank == 0 else None
        srv.reset_stats()
        lat_ms = _server_pass(srv, host_reqs, sink, paced=True)
        lat = srv.stats()
    # the plain form: one request at a time, each stream encoding on its own
    with serve.Server(1 << 62, 1, False, autotune=args.autotune,
                      batch_deadline_ms=args.batch_deadline_ms) as psrv:
        psrv.prewarm(host_reqs, sink, per_request=False)
        pms_dev, _, _ = timed_passes(psrv, dev_reqs, lib, sink, args.steps, args.warmup)
        pms_host, _, _ = timed_passes(psrv, host_reqs, lib, sink, args.steps,
                                      max(1, args.warmup // 2))
    tune = autotune_table(lib)
    link = h2d_probe([r.data for r in host_reqs[:4]], [r.data for r in dev_reqs[:4]], dev)
    lib.chucky_discard_sink_destroy(sink)
    del dev_reqs
    torch.cuda.empty_cache()
    enc = encoder_roofline(lib, dev, "lz4")
    enc_z = encoder_roofline(lib, dev, "zstd")
    ratios = codec_ratios(lib, dev) if rank == 0 else None

    totals = max_over_ranks([float(np.sum(ms_dev)), float(np.sum(ms_host)),
                             float(np.sum(pms_dev)), float(np.sum(pms_host))], world, dev)
    value, e2e, pvalue, pe2e = (whole_job_gbs(nbytes, args.steps, world, t) for t in totals)
    if rank != 0:
        return None
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    traffic = (round(LZ4_SENSOR_TRAFFIC_PER_INPUT_BYTE * enc["input_bytes"])
               if LZ4_SENSOR_TRAFFIC_PER_INPUT_BYTE else None)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(totals[0] / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8+u16+f32",
        "data": "synthetic (seeded: Poisson(100) u16 frames, N(0,1) f32 stacks, "
                "uniform u8 frames)",
        "config": {"workload": "served form: " + serve.C5_WORKLOAD,
                   "input_bytes_per_step": nbytes,
                   "l2": "inputs larger than L2 (4.8 GB per step)",
                   "parallelism": f"replicas x{world}",
                   "served": "chucky_server, 48 GB budget, up to 16 requests open, "
                             "encoders batched across streams, all requests queued, "
                             "encoder autotuner %s, batch deadline %g ms"
                             % ("on" if args.autotune else "off", args.batch_deadline_ms),
                   "plain": "the same requests one at a time, each stream encoding on "
                            "its own (same autotuner and batch deadline)"},
        "e2e": {"value": round(e2e, 3), "unit": "GB/s",
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": int(out_h),
                "ms_per_step": round(totals[1] / args.steps, 3),
                "h2d_link_gbs": round(link, 2), "frac_of_h2d_link": round(e2e / link, 4)},
        "plain": {"value": round(pvalue, 3), "e2e": round(pe2e, 3), "unit": "GB/s"},
        "served_over_plain": {"value": round(value / pvalue, 3),
                              "e2e": round(e2e / pe2e, 3)},
        "latency": {"p50_ms": round(lat["p50_ms"], 3), "p99_ms": round(lat["p99_ms"], 3),
                    "max_ms": round(lat["max_ms"], 3), "epochs": lat["epochs"],
                    "gbs": round(lat["input_bytes"] / (lat_ms * 1e-3) / 1e9, 3),
                    "arrivals": "Poisson, mean gap 20 ms; appends Poisson, mean gap "
                                "0.5 ms; pinned host inputs",
                    "definition": "append of an epoch's last byte to the end of the "
                                  "sink writes of its batch"},
        "autotune": tune,
        "served_stats": {k: st_dev[k] for k in (
            "peak_open", "peak_resident_bytes", "streams_created", "streams_reused",
            "engine_rounds", "engine_jobs", "engine_launch_sets",
            "engine_max_jobs_per_round")},
        "compression_ratio": round(nbytes / max(1.0, out_b), 4),
        "codec_ratios": ratios,
        "orca_e2e": orca,
        "cube_appends": cube,
        "roofline": {"kernel": "lz4 encoder launch set (find+plan+emit) on 64 sensor "
                               "chunks of 32x256x256 u16, timed alone",
                     "bound": "hbm", "limiter": "compute (match finding and sequence "
                                                "emission; not bandwidth)",
                     "achieved": round(enc["achieved_gbs"], 2), "peak": peak,
                     "unit": "GB/s", "frac": round(enc["achieved_gbs"] / peak, 4),
                     "peak_source": peak_src, "traffic": traffic,
                     "traffic_note": ("ncu DRAM bytes read + written by lz4_find_k + "
                                      "lz4_emit_k per input byte, one capture on 48 "
                                      "sensor chunks, scaled to this launch set's input"
                                      if traffic else "not captured"),
                     "input_gbs": round(enc["input_gbs"], 2),
                     "ms_per_launch_set": round(enc["ms"], 4)},
        "roofline_zstd": {"kernel": "zstd encoder launch set (find+table+block+frame), "
                                    "same chunks, timed alone",
                          "achieved": round(enc_z["achieved_gbs"], 2),
                          "frac": round(enc_z["achieved_gbs"] / peak, 4),
                          "input_gbs": round(enc_z["input_gbs"], 2),
                          "ms_per_launch_set": round(enc_z["ms"], 4)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_served(args)
    return line


def cpu_request_step(req, threads):
    """One request through the oracle (the whole array in one append)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import harness as H
    lib = H.oracle()
    sink = lib.oracle_null_sink_create()
    cfg = req.config()
    cfg.max_threads = threads
    s = lib.oracle_stream_create(C.byref(cfg), sink)
    if not s:
        raise RuntimeError("oracle stream create failed")
    data = req.data.numpy() if hasattr(req.data, "numpy") else req.data
    buf = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
    t0 = time.perf_counter()
    wp = lib.oracle_stream_writer(s)
    r = wp.contents.append(wp, capi.Slice(buf.ctypes.data, buf.ctypes.data + buf.size))
    if r.error or wp.contents.flush(wp).error:
        raise RuntimeError("oracle stream failed")
    dt = time.perf_counter() - t0
    lib.oracle_stream_destroy(s)
    lib.oracle_null_sink_destroy(sink)
    return dt, buf.size


def served_sample():
    """One request of each of the four shapes (as drawn for the workload),
    with the reference's default epochs per batch (chosen from its target of
    1024 chunks per batch, src/stream/config.c:31-45) rather than the GPU
    streams' two or four."""
    import dataclasses
    from chucky_gb300 import serve
    reqs = serve.c5_requests(pinned=False)
    out, seen = [], set()
    for r in reqs:
        kind = r.name.split(":")[1]
        if kind not in seen:
            seen.add(kind)
            kw = dict(r.cfg_kwargs, epochs_per_batch=0)
            out.append(dataclasses.replace(r, cfg_kwargs=kw, _cfg=None))
    return out


def cpu_baseline_served(args):
    threads = os.cpu_count() or 1
    sample = served_sample()
    tot_t, tot_b, passes = 0.0, 0, 0
    while passes < 5 and (passes < 1 or tot_t < 10.0):
        for r in sample:
            dt, nb = cpu_request_step(r, threads)
            tot_t += dt
            tot_b += nb
        passes += 1
    return {"value": round(tot_b / tot_t / 1e9, 4), "unit": "GB/s", "cores": threads,
            "kind": "port",
            "sample": f"{passes} pass(es) over one request of each of the four shapes "
                      f"({', '.join(r.name for r in sample)}; {tot_b / passes / 1e9:.2f} GB "
                      f"per pass, {tot_t:.1f} s) through the oracle/ restatement of the "
                      "reference CPU backend (LZ4-HC / zstd from the system libraries), "
                      "epochs per batch at the reference's default"}


def run_reference_served(args, rank, world):
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    sample = served_sample()
    for _ in range(args.warmup):
        cpu_request_step(sample[-1], threads)
    tot_t, tot_b = 0.0, 0
    for _ in range(args.steps):
        for r in sample:
            dt, nb = cpu_request_step(r, threads)
            tot_t += dt
            tot_b += nb
    v = tot_b / tot_t / 1e9
    from chucky_gb300 import serve
    desc = ("served form: " + serve.C5_WORKLOAD)
    return {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(tot_t / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u8+u16+f32", "data": "synthetic",
            "config": {"workload": desc, "same_config": True,
                       "sample": "each step: one request of each of the four shapes "
                                 "(bounded CPU sample of the same workload), epochs per "
                                 "batch at the reference's default"},
            "cpu_baseline": {"value": round(v, 4), "unit": "GB/s", "cores": threads,
                             "kind": "port",
                             "sample": "one request per shape per step through the "
                                       "oracle/ restatement of the reference CPU backend"},
            "e2e": {"value": round(v, 4), "unit": "GB/s",
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def cpu_oracle_step(cube, cfg, threads):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import harness as H
    lib = H.oracle()
    sink = lib.oracle_null_sink_create()
    cfg.max_threads = threads
    s = lib.oracle_stream_create(C.byref(cfg), sink)
    if not s:
        raise RuntimeError("oracle stream create failed")
    buf = np.ascontiguousarray(cube).view(np.uint8).reshape(-1)
    t0 = time.perf_counter()
    w = lib.oracle_stream_writer(s).contents
    wp = lib.oracle_stream_writer(s)
    r = w.append(wp, capi.Slice(buf.ctypes.data, buf.ctypes.data + buf.size))
    if r.error:
        raise RuntimeError("oracle append failed")
    r = w.flush(wp)
    dt = time.perf_counter() - t0
    out = lib.oracle_null_sink_bytes(sink)
    lib.oracle_stream_destroy(s)
    lib.oracle_null_sink_destroy(sink)
    return dt, buf.size, out


def cpu_baseline(args):
    """The oracle on all host cores, whole workload, repeated for ~10 s."""
    threads = os.cpu_count() or 1
    u16, f32 = make_cubes()
    work = [(u16, make_config("u16", "mean")), (f32, make_config("f32", "median"))]
    tot_t, tot_b, passes = 0.0, 0, 0
    while passes < 30 and (passes < 1 or tot_t < 10.0):
        for cube, cfg in work:
            dt, nb, _ = cpu_oracle_step(cube, cfg, threads)
            tot_t += dt
            tot_b += nb
        passes += 1
    return {"value": round(tot_b / tot_t / 1e9, 4), "unit": "GB/s", "cores": threads,
            "kind": "port",
            "sample": f"{passes} passes over the whole workload (both 256^3 cubes, "
                      f"{tot_t:.1f} s of CPU time) through the oracle/ restatement of "
                      "the reference CPU backend, zstd-3 from the system libzstd"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    u16, _ = make_cubes()
    cfg = make_config("u16", "mean")
    for _ in range(args.warmup):
        cpu_oracle_step(u16, cfg, threads)
    tot_t, tot_b = 0.0, 0
    for _ in range(args.steps):
        dt, nb, _ = cpu_oracle_step(u16, cfg, threads)
        tot_t += dt
        tot_b += nb
    v = tot_b / tot_t / 1e9
    return {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(tot_t / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u16", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "sample": "u16 cube only (the CPU path, bounded)"},
            "cpu_baseline": {"value": round(v, 4), "unit": "GB/s", "cores": threads,
                             "kind": "port",
                             "sample": "256^3 u16 cube per step through the oracle/ "
                                       "restatement of the reference CPU backend"},
            "e2e": {"value": round(v, 4), "unit": "GB/s",
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_single(args):
    """One array's stream (the u16 or the f32 cube of the workload) for
    `--steps` untimed passes from device memory: the small case that kernel
    profiles capture.  Prints nothing but "ok"."""
    import torch
    import chucky_gb300 as cg
    lib = cg.load()
    lib.chucky_discard_sink_create.restype = C.c_void_p
    lib.chucky_discard_sink_destroy.argtypes = [C.c_void_p]
    lib.tile_stream_gpu_restart.argtypes = [C.c_void_p, C.c_void_p]
    if args.single == "served-pass":
        # one pass of the served workload (device inputs) after the server's
        # start-up and one warm-up pass: the launch-list case
        import dataclasses
        from chucky_gb300 import serve
        slib = serve._lib()
        dev = torch.device("cuda")
        host = serve.c5_requests()
        on_dev = {}
        for r in host:
            if id(r.data) not in on_dev:
                on_dev[id(r.data)] = r.data.to(dev)
        reqs = [dataclasses.replace(r, data=on_dev[id(r.data)], _cfg=None) for r in host]
        sink = slib.chucky_discard_sink_create()
        with serve.Server(48 << 30, 16, True, autotune=args.autotune,
                          batch_deadline_ms=args.batch_deadline_ms) as srv:
            srv.prewarm(reqs, sink, per_request=True)
            for _ in range(1 + args.steps):
                srv.replay(reqs, sink, paced=False)
            torch.cuda.synchronize()
        slib.chucky_discard_sink_destroy(sink)
        print("ok", flush=True)
        return
    if args.single in ("orca-e2e", "cube-appends"):
        lib.tile_stream_gpu_restart.argtypes = [C.c_void_p, C.c_void_p]
        leg = orca_e2e if args.single == "orca-e2e" else cube_appends
        print(json.dumps(leg(lib, torch.device("cuda"), args.steps)), flush=True)
        return
    if args.single in ("encode-lz4", "encode-zstd"):
        # the encoder launch set alone on a batch of sensor chunks (48 chunks
        # of 32 x 256 x 256 u16, 192 MiB: more than L2): the ncu case
        enc = encoder_roofline(lib, torch.device("cuda"), args.single.split("-")[1],
                               reps=args.steps, n=48,
                               level=1 if args.level is None else args.level)
        print("ok", round(enc["input_gbs"], 1), "GB/s ratio", round(enc["ratio"], 4),
              flush=True)
        return
    if args.single in ("u16", "f32"):
        u16, f32 = make_cubes()
        cube = u16 if args.single == "u16" else f32
        cfg = make_config(args.single, "mean" if args.single == "u16" else "median")
        buf = torch.from_numpy(cube.reshape(-1).view(np.uint8)).cuda()
    elif args.single == "cube-lz4":
        u16, _ = make_cubes()
        cfg = cube_lz4_config()
        buf = torch.from_numpy(u16.reshape(-1).view(np.uint8)).cuda()
    else:
        cfg = sensor_config(args.single.split("-")[1], "max")
        buf = sensor_frames(args.frames, torch.device("cuda")).reshape(-1).view(torch.uint8)
    sink = lib.chucky_discard_sink_create()
    s = cg.GpuStream(cfg, sink)
    for _ in range(args.steps):
        lib.tile_stream_gpu_restart(s.h, None)
        if s.append(buf.data_ptr(), buf.numel()).error or s.flush().error:
            raise RuntimeError("stream failed")
    torch.cuda.synchronize()
    s.close()
    lib.chucky_discard_sink_destroy(sink)
    print("ok", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--workload", default="served",
                    choices=["served", "multiscale", "cube-lz4", "sensor-zstd",
                             "sensor-lz4", "batched"],
                    help="served: the served form against the plain one (default); "
                         "multiscale: the 256^3 u16 + f32 pair; cube-lz4: "
                         "the 256^3 u16 cube with LZ4 and no LOD; sensor-*: 2304x4096 "
                         "u16 frames with a 5-level dim-0 pyramid; batched: five rank-5 "
                         "arrays of different dtypes with uneven chunk classes")
    ap.add_argument("--frames", type=int, default=512,
                    help="sensor frames per step (multiple of 32)")
    ap.add_argument("--single", choices=["u16", "f32", "cube-lz4", "sensor-zstd",
                                         "sensor-lz4", "encode-lz4", "encode-zstd",
                                         "served-pass", "orca-e2e", "cube-appends"],
                    help="profiling case: one array's stream, --steps passes, no timing")
    ap.add_argument("--level", type=int, default=None,
                    help="codec level of --single encode-* (default 1)")
    ap.add_argument("--batch-deadline-ms", type=float, default=10.0,
                    help="served and plain forms: a stream starts a partial batch once "
                         "its oldest epoch has waited this long (0: full batches only)")
    ap.add_argument("--autotune", type=int, default=1, choices=[0, 1],
                    help="served form: encoder autotuner on (1, default) or off (0); "
                         "the plain form of the same run uses the same choice")
    args = ap.parse_args()
    if args.single:
        return run_single(args)
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    if args.impl == "reference":
        line = (run_reference_served(args, rank, world) if args.workload == "served"
                else run_reference(args, rank, world))
    elif args.workload == "served":
        line = run_served_bench(args, rank, world)
    else:
        line = run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
