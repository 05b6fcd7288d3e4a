"""Python binding of the continuous-batching decode server (gst_server_* in
include/gst_decoder.h) and an open-loop Poisson load generator for it.

The server itself is native: a scheduler thread in libgst_gb300.so admits
requests against a device-memory budget, launches whatever is admitted as one
batch whenever a launch slot is free, and keeps every result resident on the
device until it is released.  This module only submits, polls and releases."""
from __future__ import annotations

import ctypes
import gc
import time
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np

from .decoder import (GST_E_OOM, GST_OK, GPUContext, ServerConfig, ServerResult, ServerStats, _check,
                      load_library)


class DecodeServer:
    """gst_server_create / gst_server_destroy and friends."""

    def __init__(self, ctx: GPUContext, device_budget_bytes: int = 32 << 30, host_staging_bytes: int = 1 << 30,
                 slot_scratch_bytes: int = 256 << 20, max_inflight: int = 4, max_batch_images: int = 256):
        self.ctx = ctx
        cfg = ServerConfig(device_budget_bytes, host_staging_bytes, slot_scratch_bytes, max_inflight,
                           max_batch_images)
        h = ctypes.c_void_p()
        _check(load_library().gst_server_create(ctx.handle, ctypes.byref(cfg), ctypes.byref(h)), "gst_server_create")
        self._h = h
        self._res = (ServerResult * 1024)()

    def now_ns(self) -> int:
        return int(load_library().gst_server_now_ns(self._h))

    def submit(self, stream: bytes, arrival_ns: int = 0) -> int | None:
        """Queues one GST stream; returns its id, or None if the staging is full."""
        rid = ctypes.c_uint64(0)
        st = load_library().gst_server_submit(self._h, stream, len(stream), int(arrival_ns), ctypes.byref(rid))
        if st == GST_E_OOM:
            return None
        _check(st, "gst_server_submit")
        return rid.value

    def poll(self, wait_us: int = 0) -> list[ServerResult]:
        n = ctypes.c_int(0)
        _check(load_library().gst_server_poll(self._h, self._res, len(self._res), ctypes.byref(n), int(wait_us)),
               "gst_server_poll")
        out = []
        for i in range(n.value):
            r = ServerResult()
            ctypes.pointer(r)[0] = self._res[i]
            out.append(r)
        return out

    def read(self, rid: int, nbytes: int) -> np.ndarray:
        buf = np.empty(nbytes, dtype=np.uint8)
        _check(load_library().gst_server_read(self._h, rid, buf.ctypes.data, nbytes), "gst_server_read")
        return buf

    def release(self, rid: int) -> None:
        _check(load_library().gst_server_release(self._h, rid), "gst_server_release")

    def schedule(self, pool: Sequence[bytes], choice, offsets_ns, lead_ns: int = 1_000_000):
        """gst_server_schedule: a native thread submits pool[choice[i]] at server
        time start + offsets_ns[i], where start = now + lead_ns is read after
        every array is built (so that building them makes no submission late).
        Returns (ids, start); ids (0 = refused) is filled as the thread goes (an
        id is written before its request can run) and is final after
        schedule_wait()."""
        pool = list(pool)
        pool_ptrs = np.array([ctypes.cast(ctypes.c_char_p(b), ctypes.c_void_p).value for b in pool], dtype=np.uintp)
        pool_lens = np.array([len(b) for b in pool], dtype=np.uintp)
        ch = np.asarray(choice, dtype=np.intp)
        ptrs, lens = pool_ptrs[ch], pool_lens[ch]
        ids = np.zeros(ch.size, dtype=np.uint64)
        offs = np.asarray(offsets_ns, dtype=np.uint64)
        start = self.now_ns() + int(lead_ns)
        arr = offs + np.uint64(start)
        _check(load_library().gst_server_schedule(self._h, int(ch.size), ptrs.ctypes.data, lens.ctypes.data,
                                                  arr.ctypes.data, ids.ctypes.data), "gst_server_schedule")
        # the library's thread reads these until schedule_wait(): keep them (only
        # now, so that a refused second schedule leaves the running one's alone)
        self._sched_keep = (pool, ptrs, lens, arr, ids)
        return ids, start

    def schedule_wait(self) -> tuple[int, int, int]:
        """gst_server_schedule_wait -> (submitted, refused, worst lateness ns)."""
        sub, rej, late = ctypes.c_int(), ctypes.c_int(), ctypes.c_uint64()
        st = load_library().gst_server_schedule_wait(self._h, ctypes.byref(sub), ctypes.byref(rej),
                                                     ctypes.byref(late))
        self._sched_keep = None  # the thread has ended
        _check(st, "gst_server_schedule_wait")
        return sub.value, rej.value, late.value

    def cancel(self, rid: int) -> bool:
        """Withdraws a request that has not been launched yet; False if it
        already was (it then completes normally) or the id is unknown."""
        st = load_library().gst_server_cancel(self._h, rid)
        return st == GST_OK

    def stats(self, reset: bool = False) -> dict:
        st = ServerStats()
        _check(load_library().gst_server_read_stats(self._h, ctypes.byref(st), int(reset)), "gst_server_read_stats")
        return st.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            load_library().gst_server_destroy(self._h)  # stops and joins a running schedule first
            self._h = None
            self._sched_keep = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class LoadResult:
    rate: float
    seconds: float
    submitted: int = 0
    completed: int = 0
    rejected: int = 0
    verified: int = 0
    mismatched: int = 0
    errors: int = 0
    stats: dict = field(default_factory=dict)
    latencies_us: list = field(default_factory=list)
    waits_us: list = field(default_factory=list)  # arrival -> launch (queueing, host side)
    submit_lag_max_us: float = 0.0  # worst lateness of a submit behind its scheduled arrival
    worst: dict = field(default_factory=dict)  # the slowest request's timeline

    def summary(self) -> dict:
        lat = np.asarray(self.latencies_us) if self.latencies_us else np.zeros(1)
        s = self.stats
        return {
            "rate_req_s": self.rate, "seconds": round(self.seconds, 3),
            "submitted": self.submitted, "completed": self.completed, "rejected": self.rejected,
            "throughput_req_s": round(self.completed / self.seconds, 1) if self.seconds else 0.0,
            "throughput_mpix_s": round(s.get("pixels", 0) / self.seconds / 1e6, 1) if self.seconds else 0.0,
            "p50_ms": round(float(np.percentile(lat, 50)) / 1e3, 4),
            "p90_ms": round(float(np.percentile(lat, 90)) / 1e3, 4),
            "p99_ms": round(float(np.percentile(lat, 99)) / 1e3, 4),
            "p999_ms": round(float(np.percentile(lat, 99.9)) / 1e3, 4),
            "max_ms": round(float(lat.max()) / 1e3, 4),
            "wait_p99_ms": round(float(np.percentile(np.asarray(self.waits_us or [0.0]), 99)) / 1e3, 4),
            "submit_lag_max_ms": round(self.submit_lag_max_us / 1e3, 4),
            "worst": self.worst,
            "images_per_launch": round(s.get("launched_images", 0) / max(1, s.get("launches", 0)), 2),
            "device_bytes_peak": int(s.get("device_bytes_peak", 0)),
            "verified": self.verified, "bit_exact": self.mismatched == 0 and self.errors == 0,
        }


def run_poisson(server: DecodeServer, requests: Sequence[tuple[bytes, np.ndarray | None]], rate: float,
                seconds: float, seed: int = 0, verify_every: int = 0,
                pick: Callable[[np.random.Generator], int] | None = None, native: bool = True,
                hold: bool = True) -> LoadResult:
    """Open-loop Poisson arrivals at `rate` requests/s for `seconds`.

    requests: (GST stream, expected DXT1 blocks as uint64 or None); `pick`
    chooses the next one (uniform by default).  Each request is stamped with
    its scheduled arrival time, so queueing behind a late submitter counts as
    latency.  Results are released as soon as they are polled, except every
    `verify_every`-th one, which stays on the device until the run is over and
    is then read back and compared with its expected blocks (reading during the
    run would stall the submitter).  Python's cyclic garbage collector is
    paused for the run (a full collection in a large process stalls the
    submitter for tens of milliseconds).  With `native` (the default) the
    library's own thread submits each stream at its arrival time
    (gst_server_schedule), so no stall of this process delays a submission;
    this process only polls and releases (every `verify_every`-th id is kept
    for the check).  With `hold` False (native submitter only) a checked
    result is read and compared as soon as it is polled and then released, so
    that no held output occupies the device budget (a run whose budget binds
    would otherwise stall on the held outputs)."""
    gc_on = gc.isenabled()
    gc.collect()
    gc.disable()
    try:
        if native:
            return _run_poisson_native(server, requests, rate, seconds, seed, verify_every, pick, hold)
        return _run_poisson(server, requests, rate, seconds, seed, verify_every, pick)
    finally:
        if gc_on:
            gc.enable()


def _run_poisson_native(server, requests, rate, seconds, seed, verify_every, pick, hold=True) -> LoadResult:
    rng = np.random.default_rng(seed)
    n = int(rng.poisson(rate * seconds))
    arrivals = np.sort(rng.uniform(0.0, seconds, n))
    choice = [pick(rng) if pick else int(rng.integers(len(requests))) for _ in range(n)]
    res = LoadResult(rate, seconds)
    server.poll()
    server.stats(reset=True)
    offsets = np.round(arrivals * 1e9).astype(np.uint64)
    ids, t0 = server.schedule([r[0] for r in requests], choice, offsets)
    at_last = t0 + (int(offsets[-1]) if n else 0)
    held = {}  # id -> dxt bytes, every verify_every-th id, read back after the run
    index = {}  # id -> position in the schedule (ids are written in schedule order)
    scan = 0

    def position(rid):
        nonlocal scan
        while rid not in index and scan < n:
            v = int(ids[scan])
            if v:
                index[v] = scan
            scan += 1
        return index[rid]

    def checked(r):  # every verify_every-th result: held to the end, or read now
        if not (verify_every and r.id % verify_every == 0):
            return False
        if hold:
            held[r.id] = r.dxt_bytes
            return True
        want = requests[choice[position(r.id)]][1]
        if want is not None:
            res.verified += 1
            if not np.array_equal(server.read(r.id, r.dxt_bytes).view(np.uint64), want):
                res.mismatched += 1
        server.release(r.id)
        return True

    last_done = t0
    deadline = None
    while True:
        got = server.poll(2000)
        for r in got:
            last_done = max(last_done, r.done_ns)
            res.completed += 1
            lat = (r.done_ns - r.arrival_ns) / 1e3
            res.latencies_us.append(lat)
            res.waits_us.append((r.launch_ns - r.arrival_ns) / 1e3)
            if lat > res.worst.get("latency_ms", 0.0) * 1e3:
                res.worst = {"latency_ms": round(lat / 1e3, 4), "arrival_s": round((r.arrival_ns - t0) / 1e9, 4),
                             "wait_ms": round((r.launch_ns - r.arrival_ns) / 1e6, 4),
                             "launch_to_done_ms": round((r.done_ns - r.launch_ns) / 1e6, 4)}
            if r.status != GST_OK:
                res.errors += 1
            if not checked(r):
                server.release(r.id)
        if deadline is None and server.now_ns() >= at_last:
            deadline = time.monotonic() + 60.0  # every arrival is past: drain what is left
        if deadline is not None:
            sub = int(np.count_nonzero(ids)) if n else 0
            if res.completed >= sub or time.monotonic() > deadline:
                break
    res.submitted, res.rejected, late_ns = server.schedule_wait()
    while res.completed < res.submitted:  # after the join the count is exact
        got = server.poll(100000)
        if not got:
            break
        for r in got:
            last_done = max(last_done, r.done_ns)
            res.completed += 1
            res.latencies_us.append((r.done_ns - r.arrival_ns) / 1e3)
            res.waits_us.append((r.launch_ns - r.arrival_ns) / 1e3)
            if not checked(r):
                server.release(r.id)
    res.submit_lag_max_us = late_ns / 1e3
    res.seconds = max(seconds, (last_done - t0) / 1e9)
    res.stats = server.stats()
    for rid, nbytes in held.items():
        want = requests[choice[position(rid)]][1]
        if want is not None:
            got = server.read(rid, nbytes).view(np.uint64)
            res.verified += 1
            if not np.array_equal(got, want):
                res.mismatched += 1
        server.release(rid)
    return res


def _run_poisson(server, requests, rate, seconds, seed, verify_every, pick) -> LoadResult:
    rng = np.random.default_rng(seed)
    n = int(rng.poisson(rate * seconds))
    arrivals = np.sort(rng.uniform(0.0, seconds, n))
    choice = [pick(rng) if pick else int(rng.integers(len(requests))) for _ in range(n)]
    res = LoadResult(rate, seconds)
    server.poll()
    server.stats(reset=True)
    expected = {}
    t0 = server.now_ns()
    i = 0
    outstanding = 0
    last_done = t0
    held = []  # (id, bytes, expected blocks) read back after the run

    def drain(wait_us: int) -> None:
        nonlocal outstanding, last_done
        for r in server.poll(wait_us):
            outstanding -= 1
            last_done = max(last_done, r.done_ns)
            res.completed += 1
            lat = (r.done_ns - r.arrival_ns) / 1e3
            res.latencies_us.append(lat)
            res.waits_us.append((r.launch_ns - r.arrival_ns) / 1e3)
            if lat > res.worst.get("latency_ms", 0.0) * 1e3:
                res.worst = {"latency_ms": round(lat / 1e3, 4), "arrival_s": round((r.arrival_ns - t0) / 1e9, 4),
                             "wait_ms": round((r.launch_ns - r.arrival_ns) / 1e6, 4),
                             "launch_to_done_ms": round((r.done_ns - r.launch_ns) / 1e6, 4)}
            if r.status != GST_OK:
                res.errors += 1
            want = expected.pop(r.id, None)
            if want is not None:
                held.append((r.id, r.dxt_bytes, want))
            else:
                server.release(r.id)

    while i < n:
        now = (server.now_ns() - t0) / 1e9
        while i < n and arrivals[i] <= now:
            stream, want = requests[choice[i]]
            at = t0 + int(arrivals[i] * 1e9)
            res.submit_lag_max_us = max(res.submit_lag_max_us, (server.now_ns() - at) / 1e3)
            rid = server.submit(stream, at)
            if rid is None:
                res.rejected += 1
            else:
                res.submitted += 1
                outstanding += 1
                if verify_every and want is not None and res.submitted % verify_every == 0:
                    expected[rid] = want
            i += 1
        drain(0)
        if i < n:
            gap = arrivals[i] - (server.now_ns() - t0) / 1e9
            if gap > 0.0002:
                time.sleep(min(gap - 0.0001, 0.002))
    deadline = time.monotonic() + 60.0
    while outstanding > 0 and time.monotonic() < deadline:
        drain(100000)
    res.seconds = max(seconds, (last_done - t0) / 1e9)
    res.stats = server.stats()
    for rid, nbytes, want in held:
        got = server.read(rid, nbytes).view(np.uint64)
        res.verified += 1
        if not np.array_equal(got, want):
            res.mismatched += 1
        server.release(rid)
    return res
