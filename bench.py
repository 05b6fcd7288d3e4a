#!/usr/bin/env python3
"""GST decode benchmark on GB300: decoded Mpix/s and DXT1 GB/s, batched vs per-image.

Headline (``value``): the batched workload -- 64 synthetic images, width and
height drawn independently from {512, 1024, 2048} (seeds 1000+i), decoded in
one device-resident call (gst_load_compressed_dxts) per step, compressed input
and DXT1 output resident in HBM.  L2 is flushed (a 256 MiB write) before every
timed step, outside the timed events.  Also reported on the same line:

* ``per_image``: the same 64 images decoded one call per image;
* ``e2e``: the same batch through the public API with host buffers --
  pinned H2D of the packed streams, decode, D2H of the DXT1 blocks, all inside
  the timed region;
* ``workloads``: the 8192x8192 texture (10 % 1-8 px checker regions), the
  plain 512x512 image (seed 0), and the rANS-only section of 2^26 Laplace(6)
  bytes (table build + decode);
* ``roofline``: HBM-bound; algorithmic bytes = GST bytes read (28 + 2048 +
  sections) + DXT1 bytes written, per decode call, over the call's kernel time;
* ``cpu_baseline``: the C oracle (a restatement of the reference's decoder)
  on the host's cores on a bounded sample of the same batch.

``--impl reference`` times the reference's CPU decode path instead (the C
oracle port, all host threads) on bounded samples of the same workload.

Multi-GPU (torchrun): every rank decodes its own replica of the batch (images
are independent; no collective); value = all ranks' pixels / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "decoded Mpix/s & DXT1 GB/s, batched vs per-image, bit-exact; p50/p99 latency"

# DRAM bytes (read + write) per launch of each kernel on the 64-image batch,
# from one `ncu --set full --clock-control none` capture of each kernel of the
# current build (ncu flushes the caches before each replay, so these are
# cold-cache bytes: the tile kernel's reads are the rANS kernel's symbols,
# which in an unprofiled launch stay in L2).
NCU_TRAFFIC_BATCHED = {
    "gst_rans_kernel": 16.78e6 + 3.28e6,
    "gst_tile_kernel": 53.90e6 + 7.27e6,
}
FLUSH_BYTES = 256 << 20


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=("gst", "reference"), default="gst")
    p.add_argument("--skip-extra", action="store_true", help="headline workload only")
    p.add_argument("--cpu-sample", type=int, default=64, help="images of the batch the CPU baseline decodes")
    p.add_argument("--only", choices=("batched", "large", "plain", "rans", "serving", "encode", "reencode"),
                   help="time one workload's decode call only (a small command for profilers)")
    p.add_argument("--rans-blocks-per-sm", type=int, default=0,
                   help="fix the rANS kernel's CTAs of 128 threads per SM (8, 12 or 16) instead of autotuning")
    p.add_argument("--persistent", type=int, default=0, choices=(0, 1),
                   help="with --rans-blocks-per-sm: 1 = the persistent single-kernel form")
    p.add_argument("--serve-seconds", type=float, default=60.0,
                   help="length of each open-loop run of the batched server (the serving config's 60 s)")
    p.add_argument("--serve-plain-seconds", type=float, default=5.0,
                   help="length of each run of the per-request plain-decode comparison (it saturates near 10k "
                        "req/s, so its 20k req/s queue only grows with the run)")
    p.add_argument("--serve-bound-budget-mib", type=int, default=48,
                   help="device budget of the extra 20k req/s run in which admission binds (0: skip it)")
    p.add_argument("--serve-rates", default="1000,5000,20000", help="Poisson arrival rates, requests/s")
    p.add_argument("--serve-class-tune", type=int, default=1,
                   help="1: tune each size class (gst_autotune_class) before the serving runs")
    p.add_argument("--serve-modes", default="batched,plain", help="serving modes to run")
    p.add_argument("--serve-verify-every", type=int, default=500,
                   help="every k-th served result stays resident until the run ends and is checked bit for bit")
    p.add_argument("--encode-hist-match", type=int, default=0, choices=(0, 1),
                   help="encoder byte counts: merge equal lanes before the atomic (1) or not (0)")
    p.add_argument("--rans-stage-words", type=int, default=1016,
                   help="staging depth with --rans-blocks-per-sm (a multiple of 8 in [520, 4352])")
    return p.parse_args()


def tune(rb, b, stream, args) -> dict:
    """The resident batch's rANS launch configuration: fixed by the command
    line, or chosen by gst_batch_autotune (outside any timed region)."""
    if args.rans_blocks_per_sm:
        rb.set_tuning(args.rans_blocks_per_sm, args.rans_stage_words, args.persistent)
        return {"blocks_per_sm": args.rans_blocks_per_sm, "stage_words": args.rans_stage_words,
                "persistent": args.persistent, "chosen_by": "command line"}
    bps, words, pers = rb.autotune(b.d_cmp, b.d_out, stream, iterations=3)
    return {"blocks_per_sm": bps, "stage_words": words, "persistent": pers, "chosen_by": "gst_batch_autotune"}


# ---------------------------------------------------------------------------
def dist_init(n_gpus: int):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="gst_clocks_", suffix=".csv")[1])

    def _lines(self) -> int:
        try:
            return len(self.path.read_text().splitlines())
        except OSError:
            return 0

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            t0 = time.time()
            while self._lines() < 1 and time.time() - t0 < 5 and self.proc.poll() is None:
                time.sleep(0.02)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            t0 = time.time()
            while self._lines() < 3 and time.time() - t0 < 3 and self.proc.poll() is None:
                time.sleep(0.05)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        rows = []
        try:
            for line in self.path.read_text().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            self.path.unlink(missing_ok=True)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# Benchmark inputs: the reference encoder's streams of the configured images
# (tests/golden/ref_streams/, made by tests/golden/make_ref_streams.py), with
# the blocks a correct decode returns computed by the checker (the oracle's
# restatement of the reference decoder) and checked against the committed
# digests.  Where the fixtures are missing, the project's own stream producer
# stands in and every line says so.
def with_expected(images, threads=None):
    import hashlib
    from concurrent.futures import ThreadPoolExecutor
    import oracle
    threads = threads or os.cpu_count() or 1
    todo = [im for im in images if im.blocks is None]

    def one(im, n=1):
        st, dec = oracle.decode(im.stream, oracle.SCAN_EXACT, nthreads=n)
        assert st == 0, f"oracle rejects a fixture stream ({im.width}x{im.height} seed {im.seed})"
        raw = np.ascontiguousarray(dec).tobytes()
        if hashlib.sha256(raw).hexdigest() != im.decoded_sha256:
            raise AssertionError(f"oracle decode of {im.width}x{im.height} seed {im.seed} differs from the "
                                 f"fixture digest")
        im.blocks = np.frombuffer(raw, np.uint64)

    big = [im for im in todo if im.pixels >= (1 << 24)]
    for im in big:
        one(im, threads)
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(one, [im for im in todo if im not in big]))
    return images


_INPUTS: dict = {}


def _cached(key, make):
    if key not in _INPUTS:
        _INPUTS[key] = make()
    return _INPUTS[key]


def bench_batch():
    from gst_gb300 import workloads
    if workloads.ref_available():
        return _cached("batch", lambda: with_expected(workloads.ref_batched())), workloads.REF_ENCODER
    return workloads.batched(64), "gst_gb300 stream producer (reference-encoded fixtures missing)"


def bench_large():
    from gst_gb300 import workloads
    if workloads.ref_available():
        return _cached("large", lambda: with_expected([workloads.ref_large()])), workloads.REF_ENCODER
    return [workloads.large()], "gst_gb300 stream producer (reference-encoded fixtures missing)"


def bench_plain():
    from gst_gb300 import workloads
    if workloads.ref_available():
        return with_expected([workloads.ref_plain()]), workloads.REF_ENCODER
    return [workloads.plain(0)], "gst_gb300 stream producer (reference-encoded fixtures missing)"


class Batch:
    """Packed, device-resident batch of GST streams with its expected output."""

    def __init__(self, images, device):
        import torch
        from gst_gb300 import decoder
        self.images = images
        self.hdrs, packed = decoder.pack_batch([im.stream for im in images])
        self.d_cmp = torch.from_numpy(packed).to(device)
        self.h_cmp = torch.from_numpy(packed).pin_memory()
        self.out_bytes = sum(h.dxt_bytes for h in self.hdrs)
        self.d_out = torch.zeros(self.out_bytes, dtype=torch.uint8, device=device)
        self.h_out = torch.empty(self.out_bytes, dtype=torch.uint8).pin_memory()
        self.pixels = sum(im.pixels for im in images)
        self.gst_bytes = sum(len(im.stream) for im in images)
        self.alg_bytes = self.gst_bytes + self.out_bytes
        # Per-image device views for the per-image path.
        self.views = []
        cmp_off, out_off = 0, 0
        for im, h in zip(images, self.hdrs):
            _, one = decoder.pack_batch([im.stream])
            self.views.append((h, torch.from_numpy(one).to(device), out_off))
            out_off += h.dxt_bytes

    def expected(self) -> np.ndarray:
        return np.concatenate([im.blocks for im in self.images])


def time_steps(fn, steps, warmup, stream, flush, ctx=None, clear=None):
    """Runs fn() warmup + steps times; returns per-step device ms (CUDA events
    on `stream`, L2 flushed before each step outside the events) and the
    per-kernel ms of each step.  `clear` (a tensor) is zeroed before every
    step outside the events, so that the output checked after the last step
    is that step's own work."""
    import torch
    kern = []
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            if clear is not None:
                clear.zero_()
            flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
        if ctx is not None:
            kern.append(ctx.kernel_times())
    return times, kern


def kernel_summary(kern_steps):
    agg = {}
    for step in kern_steps:
        for name, ms in step:
            agg.setdefault(name, []).append(ms)
    total = sum(sum(v) for v in agg.values()) or 1.0
    return {name: {"avg_ms": statistics.mean(v), "launches": len(v), "share": sum(v) / total}
            for name, v in agg.items()}


def run_only(args, local):
    """One workload's decode call, timed; for profiler command lines."""
    import torch
    from gst_gb300 import decoder, workloads
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    ctx = decoder.GPUContext(local)
    if args.rans_blocks_per_sm:
        ctx.set_option("rans_blocks_per_sm", args.rans_blocks_per_sm)
        ctx.set_option("rans_stage_words", args.rans_stage_words)
        ctx.set_option("persistent", args.persistent)
    stream = torch.cuda.Stream(device)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=device)
    if args.only == "serving":
        out = serving(ctx, args)
        ctx.close()
        return {"only": "serving", **out}
    if args.only == "encode":
        ctx.set_option("encode_hist_match", args.encode_hist_match)
        out = encode_workloads(ctx, stream, flush, device, measured_peak_hbm()[0], args.steps, args.warmup)
        out.update(dxt_workloads(ctx, stream, flush, device, measured_peak_hbm()[0], args.steps, args.warmup))
        out.update(rgb_workloads(ctx, stream, flush, device, args.steps, args.warmup))
        ctx.close()
        return {"only": "encode", **out}
    if args.only == "reencode":
        out = rgb_workloads(ctx, stream, flush, device, args.steps, args.warmup)
        ctx.close()
        return {"only": "reencode", **out}
    if args.only == "rans":
        sec = workloads.rans_section()
        if args.rans_blocks_per_sm:  # fixed configuration (profiler command lines)
            d_f = torch.from_numpy(np.frombuffer(sec.section[:512], np.uint8).copy()).to(device)
            d_b = torch.from_numpy(np.frombuffer(sec.section[512:], np.uint8).copy()).to(device)
            d_o = torch.empty(sec.symbols.size, dtype=torch.uint8, device=device)
            fn = lambda: decoder.decode_rans_groups(ctx, d_f, d_b, len(sec.section) - 512, sec.n_groups, 32, d_o, stream)  # noqa: E731
            ctx.set_profiling(True)
            _, k = time_steps(fn, args.steps, args.warmup, stream, flush, ctx, clear=d_o)
            ctx.set_profiling(False)
            t = [sum(ms for _, ms in step) for step in k]
            ok = bool(np.array_equal(d_o.cpu().numpy(), sec.symbols))
            tuning = {"blocks_per_sm": args.rans_blocks_per_sm, "stage_words": args.rans_stage_words,
                      "chosen_by": "command line"}
        else:
            t, ok, tuning = time_rans_section(ctx, sec, device, stream, flush, args.steps, args.warmup)
        units = sec.symbols.size
    else:
        imgs, _ = {"batched": bench_batch, "large": bench_large, "plain": bench_plain}[args.only]()
        b = Batch(imgs, device)
        rb = decoder.ResidentBatch(ctx, b.hdrs)
        tuning = tune(rb, b, stream, args)
        fn = lambda: rb.launch(b.d_cmp, b.d_out, stream, graph=True)  # noqa: E731
        t, _ = time_steps(fn, args.steps, args.warmup, stream, flush, clear=b.d_out)
        ok = bool(np.array_equal(b.d_out.cpu().numpy().view(np.uint64), b.expected()))
        ok = ok and decoder.sync_status(ctx, stream) == decoder.GST_OK
        units = b.pixels
        rb.close()
    ctx.close()
    line = {"only": args.only, "ms_per_call": round(statistics.mean(t), 4), "units_per_call": units,
            "bit_exact": ok, "steps": args.steps, "warmup": args.warmup, "rans_tuning": tuning}
    return line


def run_gst(args, rank, world, local):
    import torch
    from gst_gb300 import decoder, workloads

    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    t0 = time.time()
    images, encoder_name = bench_batch()
    encode_s = time.time() - t0
    batch = Batch(images, device)
    ctx = decoder.GPUContext(local)
    stream = torch.cuda.Stream(device)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=device)
    rb = decoder.ResidentBatch(ctx, batch.hdrs)
    tuning = tune(rb, batch, stream, args)

    def step_batched():  # the resident batch, replayed as a captured CUDA graph
        rb.launch(batch.d_cmp, batch.d_out, stream, graph=True)

    def step_profiled():  # the same launch sequence, direct, with events between kernels
        rb.launch(batch.d_cmp, batch.d_out, stream)

    def step_per_image():  # the plain per-image path: one gst_load_compressed_dxt call per image
        base = batch.d_out.data_ptr()
        for h, d_one, off in batch.views:
            decoder.load_compressed_dxt(ctx, h, d_one, base + off, stream)

    def step_e2e_serial():  # host buffers: pinned H2D, graph replay, D2H of the DXT1 blocks, one after another
        with torch.cuda.stream(stream):
            batch.d_cmp.copy_(batch.h_cmp, non_blocking=True)
        rb.launch(batch.d_cmp, batch.d_out, stream, graph=True)
        with torch.cuda.stream(stream):
            batch.h_out.copy_(batch.d_out, non_blocking=True)

    chunks = 8
    hdr_arr = decoder.header_array(batch.hdrs)  # the batch's headers, passed as one array per call

    def step_e2e():  # gst_batch_host_launch: pinned host in/out, copies and decodes of `chunks` runs overlapped
        rb.host_launch(batch.h_cmp, batch.h_out, chunks, stream)

    peak, peak_kind = measured_peak_hbm()
    barrier(world)
    with ClockSampler(local) as clocks:
        times, _ = time_steps(step_batched, args.steps, args.warmup, stream, flush, clear=batch.d_out)
    clock = clocks.summary()
    stream.synchronize()
    got = batch.d_out.cpu().numpy().view(np.uint64)
    bit_exact = bool(np.array_equal(got, batch.expected()))
    status = decoder.sync_status(ctx, stream)

    ctx.set_profiling(True)
    _, kern = time_steps(step_profiled, args.steps, 2, stream, flush, ctx)
    ctx.set_profiling(False)
    launches_per_step = ctx.last_launch_count()

    total_ms = max_over_ranks(sum(times), world)
    ms_per_step = total_ms / args.steps
    value = world * batch.pixels * args.steps / (total_ms / 1e3) / 1e6
    ksum = kernel_summary(kern)
    dominant = max(ksum.items(), key=lambda kv: kv[1]["share"])[0] if ksum else None

    # per-image path
    t_img, _ = time_steps(step_per_image, max(3, args.steps // 4), 2, stream, flush, clear=batch.d_out)
    per_image_ms = statistics.mean(t_img)
    got_pi = batch.d_out.cpu().numpy().view(np.uint64)
    per_image_exact = bool(np.array_equal(got_pi, batch.expected()))

    # e2e through the public API with host buffers: the batch's pipelined
    # host-to-host launch, its chunk count (1 to 8) and decode form chosen by
    # timing outside the timed steps
    forms = [(tuning["blocks_per_sm"], tuning["stage_words"], tuning["persistent"])]
    forms.append((8, 1016, 1) if not tuning["persistent"] else (12, 1016, 0))
    forms.append((0, 0, 0))  # the batch untuned: each chunk takes its size-dependent configuration
    best = None
    for form in forms:
        rb.set_tuning(*form)
        for c in (1, 2, 3, 4, 5, 6, 8):
            chunks = c
            t_c, _ = time_steps(step_e2e, 3, 2, stream, flush)
            if best is None or statistics.mean(t_c) < best[2]:
                best = (c, form, statistics.mean(t_c))
    chunks = best[0]
    rb.set_tuning(*best[1])
    batch.h_out.zero_()
    t_e2e, _ = time_steps(step_e2e, args.steps, args.warmup, stream, flush, clear=batch.h_out)
    e2e_total = max_over_ranks(sum(t_e2e), world)
    e2e_value = world * batch.pixels * args.steps / (e2e_total / 1e3) / 1e6
    stream.synchronize()
    e2e_exact = bool(np.array_equal(batch.h_out.numpy().view(np.uint64), batch.expected()))
    e2e_exact = e2e_exact and decoder.sync_status(ctx, stream) == decoder.GST_OK
    rb.set_tuning(tuning["blocks_per_sm"], tuning["stage_words"], tuning["persistent"])
    t_ser, _ = time_steps(step_e2e_serial, max(3, args.steps // 2), args.warmup, stream, flush)

    # The host link's floor for the same bytes: the step's copy in and copy
    # out alone, issued at the same time on two streams (no decode).
    d_link = torch.empty_like(batch.d_cmp)
    side = torch.cuda.Stream(device)

    def step_link():
        fork = torch.cuda.Event()
        fork.record(stream)
        side.wait_event(fork)
        with torch.cuda.stream(side):
            d_link.copy_(batch.h_cmp, non_blocking=True)
        with torch.cuda.stream(stream):
            batch.h_out.copy_(batch.d_out, non_blocking=True)
        join = torch.cuda.Event()
        join.record(side)
        stream.wait_event(join)

    t_link, _ = time_steps(step_link, max(3, args.steps // 2), args.warmup, stream, flush)
    link_ms = statistics.mean(t_link)
    del d_link

    line = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "Mpix/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8",
        "data": "synthetic",
        "config": {
            "workload": "batched: 64 synthetic images, w,h in {512,1024,2048}, seeds 1000+i, one resident-batch "
                        "graph launch per step",
            "encoder": encoder_name,
            "images": len(images),
            "pixels_per_step": batch.pixels,
            "gst_bytes_per_step": batch.gst_bytes,
            "dxt1_bytes_per_step": batch.out_bytes,
            "l2": "flushed by a 256 MiB write before each timed step (outside the timed events)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "rans_tuning": tuning,
        },
        "dxt1_gbs": round(batch.out_bytes * args.steps / (total_ms / 1e3) / 1e9 * world, 2),
        "p50_ms": round(float(np.percentile(times, 50)), 4),
        "p99_ms": round(float(np.percentile(times, 99)), 4),
        "bit_exact": bit_exact and status == 0,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clock,
        "roofline": {
            "bound": "hbm",
            "kernel": "one batch decode (graph of " + " + ".join(ksum) + ")",
            "achieved": round(batch.alg_bytes / (ms_per_step / 1e3) / 1e9, 1),
            "peak": peak,
            "unit": "GB/s",
            "frac": round(batch.alg_bytes / (ms_per_step / 1e3) / 1e9 / peak, 4),
            "peak_source": f"{peak_kind} hbm_gbs",
            "traffic": NCU_TRAFFIC_BATCHED.get(dominant),
            "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of the dominant kernel, one cold-cache "
                            "ncu capture per launch; null where no capture of that kernel was made",
            "algorithmic_bytes_per_launch": batch.alg_bytes,
            "dominant_kernel": dominant,
            "kernels": {k: {"avg_ms": round(v["avg_ms"], 4), "share": round(v["share"], 3)} for k, v in ksum.items()},
        },
        "per_image": {
            "value": round(world * batch.pixels / (per_image_ms / 1e3) / 1e6, 2),
            "unit": "Mpix/s",
            "ms_per_step": round(per_image_ms, 4),
            "calls_per_step": len(images),
            "bit_exact": per_image_exact,
        },
        "e2e": {
            "value": round(e2e_value, 2),
            "unit": "Mpix/s",
            "ms_per_step": round(e2e_total / args.steps, 4),
            "h2d_bytes_per_step": int(batch.h_cmp.numel()),
            "d2h_bytes_per_step": int(batch.out_bytes),
            "bit_exact": e2e_exact,
            "call": f"gst_batch_host_launch (one graph launch per call), {chunks} chunks, "
                    f"{'persistent' if best[1][2] else 'two-kernel'} decodes"
                    f"{' (each chunk its size-dependent configuration)' if best[1][0] == 0 else ''} "
                    f"(pinned host layout in, pinned DXT1 out)",
            "serial_ms_per_step": round(statistics.mean(t_ser), 4),
            "link_floor_ms": round(link_ms, 4),
            "link_floor_note": "the same copy in and copy out alone, concurrently, without a decode: "
                               "the host link's time for the step's bytes",
            "link_frac": round(link_ms / (e2e_total / args.steps), 3),
        },
        "input_seconds": round(encode_s, 1),
    }
    if not args.skip_extra:
        line["workloads"] = extra_workloads(ctx, stream, flush, device, peak, args)
        line["serving"] = serving(ctx, args)
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(images[: args.cpu_sample])
        if not args.skip_extra:
            line["cpu_baseline"]["encode"] = cpu_baseline_encode(images[: args.cpu_sample])
    rb.close()
    ctx.close()
    return line


def extra_workloads(ctx, stream, flush, device, peak, args):
    import torch
    from gst_gb300 import decoder, workloads
    out = {}
    steps = max(5, args.steps // 2)
    large, large_enc = bench_large()
    plain, plain_enc = bench_plain()
    runs = [("large_8192", large, large_enc), ("plain_512", plain, plain_enc),
            ("batched_64_project_encoder", workloads.batched(64),
             "gst_gb300 stream producer (secondary input: its own DXT1 compressor and palette search)")]
    for name, imgs, enc_name in runs:
        b = Batch(imgs, device)
        rb = decoder.ResidentBatch(ctx, b.hdrs)
        tuning = tune(rb, b, stream, args)
        fn = lambda b=b, rb=rb: rb.launch(b.d_cmp, b.d_out, stream, graph=True)  # noqa: E731
        t, _ = time_steps(fn, steps, 3, stream, flush, clear=b.d_out)
        ok = bool(np.array_equal(b.d_out.cpu().numpy().view(np.uint64), b.expected()))
        ok = ok and decoder.sync_status(ctx, stream) == decoder.GST_OK
        ctx.set_profiling(True)
        _, k = time_steps(lambda b=b, rb=rb: rb.launch(b.d_cmp, b.d_out, stream), 3, 1, stream, flush, ctx)
        ctx.set_profiling(False)
        ks = kernel_summary(k)
        ms = statistics.mean(t)
        out[name] = {
            "value": round(b.pixels / (ms / 1e3) / 1e6, 2), "unit": "Mpix/s",
            "ms_per_call": round(ms, 4),
            "p50_ms": round(float(np.percentile(t, 50)), 4), "p99_ms": round(float(np.percentile(t, 99)), 4),
            "dxt1_gbs": round(b.out_bytes / (ms / 1e3) / 1e9, 2),
            "hbm_frac": round(b.alg_bytes / (ms / 1e3) / 1e9 / peak, 4),
            "kernels": {kk: round(v["avg_ms"], 4) for kk, v in ks.items()},
            "gst_bytes": b.gst_bytes, "bit_exact": ok, "rans_tuning": tuning, "encoder": enc_name,
        }
        rb.close()
    out.update(encode_workloads(ctx, stream, flush, device, peak, steps, 3))
    out.update(dxt_workloads(ctx, stream, flush, device, peak, steps, 3))
    out.update(rgb_workloads(ctx, stream, flush, device, steps, 3))
    sec = workloads.rans_section()
    t, ok, rtuning = time_rans_section(ctx, sec, device, stream, flush, steps, 3)
    alg = len(sec.section) + sec.symbols.size
    out["rans_2^26"] = {
        "value": round(sec.symbols.size / (statistics.mean(t) / 1e3) / 1e9, 3), "unit": "Gsym/s",
        "ms_per_call": round(statistics.mean(t), 4),
        "gbs": round(alg / (statistics.mean(t) / 1e3) / 1e9, 1),
        "hbm_frac": round(alg / (statistics.mean(t) / 1e3) / 1e9 / peak, 4),
        "bits_per_symbol": round(8 * (len(sec.section) - 512) / sec.symbols.size, 3), "bit_exact": ok,
        "rans_tuning": rtuning,
    }
    return out


def device_symbols(ctx, stream_bytes: bytes, device):
    """A stream's decompressed-symbol buffer (Y planes, chroma planes, palette,
    index deltas; codec/decoder.cpp:441-461) on the device, through the CUDA
    rANS stage (the encoder workloads' inputs)."""
    import torch
    from gst_gb300 import decoder
    h = decoder.parse_header(stream_bytes)
    B = h.width * h.height // 16
    nsyms = (2 * B, 4 * B, h.palette_bytes, B)
    lens = (h.y_cmp_sz, h.chroma_cmp_sz, h.palette_sz, h.indices_sz)
    out = torch.empty(7 * B + h.palette_bytes, dtype=torch.uint8, device=device)
    body, at = 28 + 2048, 0
    for k in range(4):
        d_f = torch.from_numpy(np.frombuffer(stream_bytes[28 + 512 * k:28 + 512 * (k + 1)], np.uint8).copy()).to(device)
        d_b = torch.from_numpy(np.frombuffer(stream_bytes[body:body + lens[k]], np.uint8).copy()).to(device)
        decoder.decode_rans_groups(ctx, d_f, d_b, lens[k], nsyms[k] // 8192, 32, out[at:at + nsyms[k]])
        body += lens[k]
        at += nsyms[k]
    assert decoder.sync_status(ctx) == decoder.GST_OK
    return out


def encode_workloads(ctx, stream, flush, device, peak, steps, warmup):
    """The encoder stages (include/gst_encode.h): the symbol sections of the
    64-image batch and of the 8192x8192 texture encoded back into their GST
    streams, device-resident, one gst_encode_streams call per step (host plan
    + four kernels), output checked byte for byte against the streams; then
    the host-to-host call (gst_compress_symbols) on the 8192x8192 texture."""
    import torch
    from gst_gb300 import decoder, entropy, workloads
    out = {}
    for name, imgs in (("encode_batched_64", bench_batch()[0]), ("encode_large_8192", bench_large()[0])):
        syms = [device_symbols(ctx, im.stream, device) for im in imgs]
        hdrs = [decoder.parse_header(im.stream) for im in imgs]
        descs = [entropy.stream_symbols(h.width, h.height, h.palette_bytes, s) for h, s in zip(hdrs, syms)]
        descs = (entropy.StreamSymbols * len(descs))(*descs)
        cap = sum(entropy.stream_bound(h.width, h.height, h.palette_bytes) for h in hdrs)
        d_out = torch.zeros(cap, dtype=torch.uint8, device=device)
        d_offs = torch.zeros(len(imgs) + 1, dtype=torch.int64, device=device)
        fn = lambda descs=descs, d_out=d_out, d_offs=d_offs: entropy.encode_streams(ctx, descs, d_out, d_offs, stream)  # noqa: E731
        t, _ = time_steps(fn, steps, warmup, stream, flush, clear=d_out)
        ok = decoder.sync_status(ctx, stream) == decoder.GST_OK
        o = d_offs.cpu().numpy()
        host = d_out[: int(o[-1])].cpu().numpy().tobytes()
        ok = ok and all(host[o[i]:o[i + 1]] == im.stream for i, im in enumerate(imgs))
        ctx.set_profiling(True)
        _, k = time_steps(fn, 3, 1, stream, flush, ctx)
        ctx.set_profiling(False)
        ks = kernel_summary(k)
        ms = statistics.mean(t)
        n_sym = sum(int(s.numel()) for s in syms)
        comp = sum(len(im.stream) for im in imgs)
        px = sum(im.pixels for im in imgs)
        rk = ks.get("gst_enc_rans_kernel", {}).get("avg_ms", 0.0)
        out[name] = {
            "value": round(n_sym / (ms / 1e3) / 1e9, 3), "unit": "Gsym/s",
            "mpix_s": round(px / (ms / 1e3) / 1e6, 1), "ms_per_call": round(ms, 4),
            "p50_ms": round(float(np.percentile(t, 50)), 4), "p99_ms": round(float(np.percentile(t, 99)), 4),
            "symbols": n_sym, "gst_bytes": comp,
            "gbs": round((n_sym + comp) / (ms / 1e3) / 1e9, 1),
            "hbm_frac": round((n_sym + comp) / (ms / 1e3) / 1e9 / peak, 4),
            "kernels": {kk: round(v["avg_ms"], 4) for kk, v in ks.items()},
            "rans_kernel_gsym_s": round(n_sym / (rk / 1e3) / 1e9, 3) if rk else None,
            "byte_exact": bool(ok),
        }
        if name == "encode_large_8192":
            h = hdrs[0]
            host_sym = syms[0].cpu().numpy()
            entropy.compress_symbols(ctx, h.width, h.height, h.palette_bytes, host_sym)
            e2e = []
            for _ in range(5):
                t0 = time.perf_counter()
                s2 = entropy.compress_symbols(ctx, h.width, h.height, h.palette_bytes, host_sym)
                e2e.append((time.perf_counter() - t0) * 1e3)
            out[name]["e2e"] = {"ms": round(statistics.median(e2e), 3),
                                "value": round(n_sym / (statistics.median(e2e) / 1e3) / 1e9, 3), "unit": "Gsym/s",
                                "h2d_bytes": n_sym, "d2h_bytes": len(s2), "byte_exact": s2 == imgs[0].stream}
    return out


def dxt_workloads(ctx, stream, flush, device, peak, steps, warmup):
    """The whole encoder on the GPU from DXT1 blocks (include/gst_encode.h):
    per step gst_prepare_symbols (YCoCg planes, forward wavelet, run palette),
    the palette sizes read back (the host builds the entropy plan from them),
    then gst_encode_streams; output checked against the oracle-free property
    that it decodes to the given blocks.  The endpoint stages are also timed
    alone.  Inputs: the 64-image batch's and the 8192x8192 texture's blocks."""
    import torch
    from gst_gb300 import decoder, entropy, workloads
    out = {}
    for name, imgs in (("dxt_to_gst_batched_64", bench_batch()[0]), ("dxt_to_gst_large_8192", bench_large()[0])):
        bufs, prep, hdr = [], [], []
        for im in imgs:
            B = im.width * im.height // 16
            t = {"b": torch.from_numpy(im.blocks.view(np.int64).copy()).to(device),
                 "y": torch.empty(2 * B, dtype=torch.uint8, device=device),
                 "c": torch.empty(4 * B, dtype=torch.uint8, device=device),
                 "p": torch.empty(entropy.palette_capacity(im.width, im.height), dtype=torch.uint8, device=device),
                 "i": torch.empty(B, dtype=torch.uint8, device=device)}
            bufs.append(t)
            prep.append((im.width, im.height, t["b"], t["y"], t["c"], t["p"], t["i"]))
        pal = torch.zeros(len(imgs), dtype=torch.int32, device=device)
        h_pal = torch.zeros(len(imgs), dtype=torch.int32).pin_memory()
        cap = sum(entropy.stream_bound(im.width, im.height, entropy.palette_capacity(im.width, im.height)) for im in imgs)
        d_out = torch.zeros(cap, dtype=torch.uint8, device=device)
        d_offs = torch.zeros(len(imgs) + 1, dtype=torch.int64, device=device)

        prep = entropy.symbol_buffers(prep)  # descriptors built once, as a caller with fixed buffers would
        descs = (entropy.StreamSymbols * len(imgs))(*[
            entropy.StreamSymbols(im.width, im.height, 0, 0, t["y"].data_ptr(), t["c"].data_ptr(), t["p"].data_ptr(),
                                  t["i"].data_ptr()) for im, t in zip(imgs, bufs)])

        def step():
            entropy.prepare_symbols(ctx, prep, pal, stream)
            with torch.cuda.stream(stream):
                h_pal.copy_(pal, non_blocking=True)
            stream.synchronize()
            for k, v in enumerate(h_pal.tolist()):
                descs[k].palette_bytes = v
            entropy.encode_streams(ctx, descs, d_out, d_offs, stream)

        t_all, _ = time_steps(step, steps, warmup, stream, flush, clear=d_out)
        ok = decoder.sync_status(ctx, stream) == decoder.GST_OK
        o = d_offs.cpu().numpy()
        host = d_out[: int(o[-1])].cpu().numpy().tobytes()
        for k, im in enumerate(imgs[:8] if len(imgs) > 8 else imgs):
            got = decoder.decompress_dxt(ctx, host[o[k]:o[k + 1]])
            ok = ok and bool(np.array_equal(got.view(np.uint64), im.blocks))
        t_prep, _ = time_steps(lambda: entropy.prepare_symbols(ctx, prep, pal, stream), steps, warmup, stream, flush)
        ctx.set_profiling(True)
        _, k = time_steps(lambda: entropy.prepare_symbols(ctx, prep, pal, stream), 3, 1, stream, flush, ctx)
        ctx.set_profiling(False)
        ks = kernel_summary(k)
        ms, ms_prep = statistics.mean(t_all), statistics.mean(t_prep)
        px = sum(im.pixels for im in imgs)
        blk_bytes = sum(im.blocks.nbytes for im in imgs)
        out[name] = {
            "value": round(px / (ms / 1e3) / 1e6, 1), "unit": "Mpix/s", "ms_per_call": round(ms, 4),
            "endpoint_stages_ms": round(ms_prep, 4),
            "endpoint_stages_gbs": round(blk_bytes * 2 / (ms_prep / 1e3) / 1e9, 1),
            "endpoint_kernels": {kk: round(v["avg_ms"], 4) for kk, v in ks.items()},
            "dxt1_bytes": blk_bytes, "gst_bytes": int(o[-1]), "decodes_to_blocks": bool(ok),
        }
        if name == "dxt_to_gst_large_8192":
            im = imgs[0]
            entropy.compress_dxt(ctx, im.width, im.height, im.blocks)
            e2e = []
            for _ in range(5):
                t0 = time.perf_counter()
                s2 = entropy.compress_dxt(ctx, im.width, im.height, im.blocks)
                e2e.append((time.perf_counter() - t0) * 1e3)
            out[name]["e2e"] = {"ms": round(statistics.median(e2e), 3),
                                "value": round(px / (statistics.median(e2e) / 1e3) / 1e6, 1), "unit": "Mpix/s",
                                "h2d_bytes": blk_bytes, "d2h_bytes": len(s2)}
    return out


def rgb_workloads(ctx, stream, flush, device, steps, warmup):
    """The reference encoder's path from an RGB8 source and its DXT1 blocks
    (CompressDXTImage(DXTImage(w, h, rgb, dxt))), on the GPU: per step
    gst_reencode_blocks (the reference's index palette search), gst_prepare_planes
    on the searched blocks, the palette sizes read back, gst_encode_streams.
    Inputs: the 64-image batch's synthetic RGB images (same seeds and sizes)
    and their blocks from the project's block compressor.  Checked: the two
    smallest images' streams equal the C oracle's whole pipeline (restating
    the reference's), and every stream decodes to the searched blocks."""
    import torch
    from gst_gb300 import decoder, encoder, entropy, workloads
    import oracle
    dims = workloads.batched_dims(64)
    imgs = []
    for k, (w, h) in enumerate(dims):
        rgb = encoder.synth_image(w, h, 1000 + k, 0.0)
        imgs.append((w, h, rgb, encoder.compress_blocks(rgb)))
    bufs, re_descs, prep = [], [], []
    pal = torch.zeros(len(imgs), dtype=torch.int32, device=device)
    for k, (w, h, rgb, blocks) in enumerate(imgs):
        B = w * h // 16
        t = {"rgb": torch.from_numpy(rgb.reshape(-1)).to(device),
             "b": torch.from_numpy(blocks.view(np.int64).copy()).to(device),
             "o": torch.empty(B, dtype=torch.int64, device=device),
             "y": torch.empty(2 * B, dtype=torch.uint8, device=device),
             "c": torch.empty(4 * B, dtype=torch.uint8, device=device),
             "p": torch.empty(entropy.palette_capacity(w, h), dtype=torch.uint8, device=device),
             "i": torch.empty(B, dtype=torch.uint8, device=device)}
        bufs.append(t)
        re_descs.append((w, h, t["rgb"], t["b"], t["o"], t["p"], t["i"], pal[k:k + 1]))
        prep.append((w, h, t["o"], t["y"], t["c"], t["p"], t["i"]))
    re_descs = entropy.reencode_images(re_descs)
    prep = entropy.symbol_buffers(prep)
    h_pal = torch.zeros(len(imgs), dtype=torch.int32).pin_memory()
    cap = sum(entropy.stream_bound(w, h, entropy.palette_capacity(w, h)) for w, h, *_ in imgs)
    d_out = torch.zeros(cap, dtype=torch.uint8, device=device)
    d_offs = torch.zeros(len(imgs) + 1, dtype=torch.int64, device=device)
    descs = (entropy.StreamSymbols * len(imgs))(*[
        entropy.StreamSymbols(w, h, 0, 0, t["y"].data_ptr(), t["c"].data_ptr(), t["p"].data_ptr(), t["i"].data_ptr())
        for (w, h, *_), t in zip(imgs, bufs)])

    def step():
        entropy.reencode_blocks(ctx, re_descs, stream)
        entropy.prepare_planes(ctx, prep, stream)
        with torch.cuda.stream(stream):
            h_pal.copy_(pal, non_blocking=True)
        stream.synchronize()
        for k, v in enumerate(h_pal.tolist()):
            descs[k].palette_bytes = v
        entropy.encode_streams(ctx, descs, d_out, d_offs, stream)

    t_all, _ = time_steps(step, steps, warmup, stream, flush, clear=d_out)
    ok = decoder.sync_status(ctx, stream) == decoder.GST_OK
    o = d_offs.cpu().numpy()
    host = d_out[: int(o[-1])].cpu().numpy().tobytes()
    for k, t in enumerate(bufs):
        got = decoder.decompress_dxt(ctx, host[o[k]:o[k + 1]])
        ok = ok and bool(np.array_equal(got.view(np.uint64), t["o"].cpu().numpy().view(np.uint64)))
    for k in sorted(range(len(imgs)), key=lambda i: imgs[i][0] * imgs[i][1])[:2]:
        w, h, rgb, blocks = imgs[k]
        ob, op, od = oracle.reencode(w, h, rgb, blocks)
        y, c, _ = oracle.endpoint_planes(w, h, ob)
        st, want = oracle.encode_stream(w, h, op.size, y, c, op, od)
        ok = ok and st == 0 and host[o[k]:o[k + 1]] == want
    t_re, _ = time_steps(lambda: entropy.reencode_blocks(ctx, re_descs, stream), steps, warmup, stream, flush)
    ms, ms_re = statistics.mean(t_all), statistics.mean(t_re)
    # host to host: the largest image through gst_compress_rgb_dxt (RGB8 and
    # blocks copied in, the stream copied out), as a caller of CompressDXT has it
    k = max(range(len(imgs)), key=lambda i: imgs[i][0] * imgs[i][1])
    w, h, rgb, blocks = imgs[k]
    s_ref = entropy.compress_rgb_dxt(ctx, w, h, rgb, blocks)
    e2e = []
    for _ in range(5):
        t0 = time.perf_counter()
        s2 = entropy.compress_rgb_dxt(ctx, w, h, rgb, blocks)
        e2e.append((time.perf_counter() - t0) * 1e3)
    ok = ok and s2 == s_ref == host[o[k]:o[k + 1]]
    px = sum(w * h for w, h, *_ in imgs)
    nblk = px // 16
    return {"rgb_dxt_to_gst_batched_64": {
        "value": round(px / (ms / 1e3) / 1e6, 1), "unit": "Mpix/s", "ms_per_call": round(ms, 4),
        "palette_search_ms": round(ms_re, 4), "palette_search_mblocks_s": round(nblk / (ms_re / 1e3) / 1e6, 1),
        "palette_words": int(h_pal.sum().item()) // 4, "blocks": nblk, "gst_bytes": int(o[-1]),
        "matches_oracle_and_decodes_to_searched_blocks": bool(ok),
        "e2e_one_image": {"call": "gst_compress_rgb_dxt", "image": f"{w}x{h}", "ms": round(statistics.median(e2e), 3),
                          "mblocks_s": round(w * h / 16 / (statistics.median(e2e) / 1e3) / 1e6, 2),
                          "h2d_bytes": int(rgb.nbytes + blocks.nbytes), "d2h_bytes": len(s2)},
        "cpu_baseline": cpu_baseline_reencode(imgs)}}


def cpu_baseline_reencode(imgs):
    """The C oracle's Reencode restatement on all host cores, one image per
    thread (largest first): the search is sequential within an image."""
    from concurrent.futures import ThreadPoolExecutor
    import oracle
    threads = os.cpu_count() or 1
    order = sorted(imgs, key=lambda a: -a[0] * a[1])
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda a: oracle.reencode(*a), order))
    dt = time.perf_counter() - t0
    nblk = sum(w * h // 16 for w, h, *_ in imgs)
    return {"value": round(nblk / dt / 1e6, 3), "unit": "Mblocks/s", "cores": threads, "kind": "port",
            "sample": f"palette search of all {len(imgs)} images ({nblk / 1e6:.2f} M blocks), {threads} threads, "
                      f"{dt:.2f} s"}


RANS_CANDIDATES = ((16, 520), (12, 520), (12, 1016), (8, 1528), (8, 2040), (8, 2816))


def time_rans_section(ctx, sec, device, stream, flush, steps, warmup):
    """The 2^26-symbol section through gst_decode_rans_groups: the context's
    rANS launch configuration is chosen by timing each candidate (outside the
    timed steps), then the table build + decode kernel is timed with
    instrumentation events (the call also uploads a plan from the host)."""
    import torch
    from gst_gb300 import decoder
    d_f = torch.from_numpy(np.frombuffer(sec.section[:512], np.uint8).copy()).to(device)
    d_b = torch.from_numpy(np.frombuffer(sec.section[512:], np.uint8).copy()).to(device)
    d_o = torch.empty(sec.symbols.size, dtype=torch.uint8, device=device)
    fn = lambda: decoder.decode_rans_groups(ctx, d_f, d_b, len(sec.section) - 512, sec.n_groups, 32, d_o, stream)  # noqa: E731
    ctx.set_profiling(True)
    per = {c: [] for c in RANS_CANDIDATES}
    for _ in range(2):  # two rounds over the candidates, so that one slow step does not decide
        for bps, words in RANS_CANDIDATES:
            ctx.set_option("rans_blocks_per_sm", bps)
            ctx.set_option("rans_stage_words", words)
            _, k = time_steps(fn, 5, 1, stream, flush, ctx)
            per[(bps, words)] += [sum(m for _, m in step) for step in k]
    bps, words = min(per, key=lambda c: statistics.median(per[c]))
    best = (bps, words)
    ctx.set_option("rans_blocks_per_sm", best[0])
    ctx.set_option("rans_stage_words", best[1])
    _, k = time_steps(fn, steps, warmup, stream, flush, ctx, clear=d_o)
    ctx.set_profiling(False)
    ctx.set_option("auto_tuning", 1)
    t = [sum(ms for _, ms in step) for step in k]
    ok = bool(np.array_equal(d_o.cpu().numpy(), sec.symbols)) and decoder.sync_status(ctx, stream) == decoder.GST_OK
    return t, ok, {"blocks_per_sm": best[0], "stage_words": best[1], "chosen_by": "timing each candidate"}


def serving(ctx, args) -> dict:
    """Open-loop Poisson arrivals through the continuous-batching server, and
    the same arrival trace through per-request plain decodes (one image per
    launch, one launch at a time).  Sizes w, h from {512, 1024, 2048, 4096}
    with weights 0.4/0.3/0.2/0.1; a pool of pre-encoded streams; 32 GiB
    device budget; every 50th result is read back and checked."""
    from gst_gb300 import workloads
    from gst_gb300.server import DecodeServer, run_poisson
    if workloads.ref_available():
        pool = workloads.ref_serving_pool()
        with_expected([im for ims in pool.values() for im in ims])
        pool_encoder = workloads.REF_ENCODER
    else:
        pool = workloads.serving_pool(per_class=4)
        pool_encoder = "gst_gb300 stream producer (reference-encoded fixtures missing)"
    dims = workloads.SERVING_DIMS
    weights = np.array([0.4, 0.3, 0.2, 0.1])
    keys = [(w, h) for w in dims for h in dims]
    key_p = np.array([weights[dims.index(w)] * weights[dims.index(h)] for w, h in keys])
    reqs, owner = [], []
    for k, key in enumerate(keys):
        for im in pool[key]:
            reqs.append((im.stream, im.blocks))
            owner.append(k)
    by_key = {k: [i for i, o in enumerate(owner) if o == k] for k in range(len(keys))}

    def pick(rng):
        k = int(rng.choice(len(keys), p=key_p))
        return by_key[k][int(rng.integers(len(by_key[k])))]

    # The server's launches use the configuration of their size class: tune
    # each class a request mix produces on one image of it (outside the runs).
    import torch
    from gst_gb300 import decoder
    classes = []
    for w in (dims if args.serve_class_tune else []):
        im = pool[(w, w)][0]
        hdrs, packed = decoder.pack_batch([im.stream])
        d_cmp = torch.from_numpy(packed).cuda()
        d_out = torch.empty(hdrs[0].dxt_bytes, dtype=torch.uint8, device="cuda")
        classes.append(decoder.autotune_class(ctx, hdrs, d_cmp, d_out, iterations=3))
    out = {"config": {"dims": list(dims), "weights": weights.tolist(), "pool_streams": len(reqs),
                      "pool_encoder": pool_encoder,
                      "pool_streams_per_class_min": min(len(v) for v in pool.values()),
                      "device_budget_gib": 32, "seconds_per_rate": args.serve_seconds,
                      "plain_seconds_per_rate": args.serve_plain_seconds,
                      "verify_every": args.serve_verify_every,
                      "class_tuning": {f"class {c} ({w}x{w})": list(decoder.get_class_tuning(ctx, c))
                                       for c, w in zip(classes, dims)},
                      "class_tuning_note": "gst_autotune_class on one image per class: (CTAs/SM, staging words, "
                                           "persistent); the server keeps the two-kernel form"}}
    for rate in [float(r) for r in args.serve_rates.split(",") if r]:
        row = {}
        for mode, kw, secs in (("batched", dict(max_inflight=4, max_batch_images=256), args.serve_seconds),
                               ("plain", dict(max_inflight=1, max_batch_images=1), args.serve_plain_seconds)):
            if mode not in args.serve_modes.split(",") or secs <= 0:
                continue
            with DecodeServer(ctx, device_budget_bytes=32 << 30, **kw) as srv:
                run_poisson(srv, reqs, rate, 0.2, seed=7, pick=pick)  # warm-up
                res = run_poisson(srv, reqs, rate, secs, seed=int(rate),
                                  verify_every=args.serve_verify_every, pick=pick)
            row[mode] = res.summary()
        out[f"{int(rate)}_req_s"] = row
    if args.serve_bound_budget_mib > 0 and "batched" in args.serve_modes.split(","):
        # Admission under pressure: a budget small enough that requests wait
        # for the memory of earlier ones (compressed input + DXT1 output).
        # Checked results are read and released as they arrive: held outputs
        # would otherwise take the budget.
        budget = args.serve_bound_budget_mib << 20
        secs = min(10.0, args.serve_seconds)
        with DecodeServer(ctx, device_budget_bytes=budget, max_inflight=4, max_batch_images=256) as srv:
            run_poisson(srv, reqs, 20000.0, 0.2, seed=7, pick=pick, hold=False)
            res = run_poisson(srv, reqs, 20000.0, secs, seed=20001, verify_every=args.serve_verify_every // 5 or 1,
                              pick=pick, hold=False)
        out["20000_req_s_budget_bound"] = {"device_budget_mib": args.serve_bound_budget_mib, **res.summary()}
    return out


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_decode_rate(images, threads: int, passes: int, warmup: int, scan) -> tuple[float, list[float]]:
    """Mpix/s of the oracle's decode (the reference decoder's arithmetic) over
    `images`: `warmup` untimed passes, then `passes` timed ones.  With more than
    one thread the images go one per thread (largest first), and an image
    larger than 1/threads of the sample is itself decoded by all threads."""
    from concurrent.futures import ThreadPoolExecutor
    import oracle
    oracle.load()
    px = sum(im.pixels for im in images)
    order = sorted(images, key=lambda im: -im.pixels)
    big = [im for im in order if threads > 1 and im.pixels * threads > px]
    small = [im for im in order if im not in big]

    def one(im, n=1):
        st, _ = oracle.decode(im.stream, scan, nthreads=n)
        assert st == 0

    def run_pass(ex):
        for im in big:
            one(im, threads)
        if ex is None:
            for im in small:
                one(im)
        else:
            list(ex.map(one, small))

    times = []
    with ThreadPoolExecutor(threads) if threads > 1 else _null_ctx() as ex:
        for _ in range(warmup):
            run_pass(ex)
        for _ in range(passes):
            t0 = time.perf_counter()
            run_pass(ex)
            times.append(time.perf_counter() - t0)
    return px * passes / sum(times) / 1e6, times


class _null_ctx:
    def __enter__(self):
        return None

    def __exit__(self, *exc):
        return False


CPU_PASSES = 30          # timed passes of the all-core leg (each pass decodes every sample image once)
CPU_SINGLE_PASSES = 5   # timed passes of the single-thread leg, over a quarter of the sample


def cpu_single_thread(images):
    sub = images[: max(1, len(images) // 4)]
    import oracle
    v, t = cpu_decode_rate(sub, 1, CPU_SINGLE_PASSES, 1, oracle.SCAN_REFERENCE)
    px = sum(im.pixels for im in sub)
    return {"value": round(v, 2), "unit": "Mpix/s", "cores": 1,
            "sample": f"first {len(sub)} images ({px / 1e6:.1f} Mpix), 1 warm-up + {CPU_SINGLE_PASSES} timed "
                      f"passes ({statistics.mean(t):.3f} s each)"}


def cpu_baseline(images):
    """The C oracle (restating the reference's CPU decode path: rANS groups as
    ans::DecodeInterleaved, the inverse wavelet as InverseWavelet2D, the index
    scan and DXT1 assembly) on the host: an all-core leg (one image per thread)
    and a single-thread leg, each warmed up and timed over several passes."""
    import oracle
    threads = os.cpu_count() or 1
    v_all, t_all = cpu_decode_rate(images, threads, CPU_PASSES, 1, oracle.SCAN_REFERENCE)
    px = sum(im.pixels for im in images)
    return {"value": round(v_all, 2), "unit": "Mpix/s", "cores": threads, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": f"{len(images)} images of the batched workload ({px / 1e6:.1f} Mpix), oracle decode, "
                      f"{threads} threads (one image per thread), 1 warm-up + {CPU_PASSES} timed passes "
                      f"({statistics.mean(t_all):.3f} s each, {sum(t_all) * threads:.1f} thread-seconds in all)",
            "single_thread": cpu_single_thread(images)}


def cpu_baseline_encode(images):
    """The C oracle's encoder stages (restating ByteEncoder::EncodeBytes and the
    stream assembly) on all host cores, one image per thread, re-encoding the
    images' symbol sections into their streams."""
    from concurrent.futures import ThreadPoolExecutor
    import oracle
    threads = os.cpu_count() or 1
    inputs = []
    for im in images:
        w, h, pal = (int.from_bytes(im.stream[i:i + 4], "little") for i in (0, 4, 8))
        st, sym = oracle.decode_symbols(im.stream, nthreads=threads)
        assert st == 0
        inputs.append((w, h, pal, oracle.split_symbols(w, h, pal, sym)))
    n_sym = sum(7 * (w * h // 16) + pal for w, h, pal, _ in inputs)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(lambda a: oracle.encode_stream(a[0], a[1], a[2], *a[3]), inputs))
    dt = time.perf_counter() - t0
    assert all(st == 0 and s == im.stream for (st, s), im in zip(res, images))

    def from_blocks(im):  # the whole encoder from DXT1 blocks, as the GPU pipeline runs it
        y, c, _ = oracle.endpoint_planes(im.width, im.height, im.blocks)
        p, d = oracle.run_palette(im.width, im.height, im.blocks)
        return oracle.encode_stream(im.width, im.height, p.size, y, c, p, d)

    px = sum(im.pixels for im in images)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        res2 = list(ex.map(from_blocks, images))
    dt2 = time.perf_counter() - t0
    assert all(st == 0 for st, _ in res2)
    return {"value": round(n_sym / dt / 1e9, 4), "unit": "Gsym/s", "cores": threads, "kind": "port",
            "sample": f"symbol sections of the first {len(images)} images of the batched workload "
                      f"({n_sym / 1e6:.1f} M symbols), oracle encode, {threads} threads, {dt:.2f} s",
            "dxt_to_gst": {"value": round(px / dt2 / 1e6, 1), "unit": "Mpix/s", "cores": threads, "kind": "port",
                           "sample": f"the same {len(images)} images from their DXT1 blocks (endpoint planes, "
                                     f"run palette, entropy stages), {dt2:.2f} s"}}


def run_reference(args, rank, world):
    """The reference's CPU decode path (the oracle port), all host threads, on
    the same images and with the same method as the GPU arm's cpu_baseline."""
    from gst_gb300 import workloads
    import oracle
    if rank != 0:
        return None
    images, encoder_name = bench_batch()
    images = images[: args.cpu_sample]
    threads = os.cpu_count() or 1
    px = sum(im.pixels for im in images)
    value, times = cpu_decode_rate(images, threads, args.steps, max(1, min(args.warmup, 2)), oracle.SCAN_REFERENCE)
    total = sum(times)
    sample = (f"{len(images)} of the 64 batched images ({px / 1e6:.1f} Mpix) per step, oracle port of the "
              f"reference decoder, {threads} threads (one image per thread)")
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": "Mpix/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "batched: 64 synthetic images, w,h in {512,1024,2048}, seeds 1000+i",
                   "encoder": encoder_name, "sample_images": len(images)},
        "cpu_baseline": {"value": round(value, 2), "unit": "Mpix/s", "cores": threads, "kind": "port",
                         "cpu_model": cpu_model(), "sample": sample,
                         "single_thread": cpu_single_thread(images)},
        "e2e": {"value": round(value, 2), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse_args()
    rank, world, local = dist_init(args.gpus)
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.only:
        line = run_only(args, local)
    else:
        line = run_gst(args, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
