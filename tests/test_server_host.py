"""Host logic of the serving load generator (gst_gb300.server.run_poisson)
against a fake server, on the CPU: open-loop arrivals, latency from the
scheduled arrival time, verification and release of every result, with this
process submitting and with a submitting thread in place of the library's
(gst_server_schedule)."""
import threading
import time

import numpy as np
import pytest

from gst_gb300 import decoder
from gst_gb300.server import run_poisson


class FakeResult:
    def __init__(self, rid, arrival, done, nbytes):
        self.id, self.arrival_ns, self.done_ns, self.dxt_bytes = rid, arrival, done, nbytes
        self.status = decoder.GST_OK
        self.launch_ns = arrival


class FakeServer:
    """Completes each request 100 us after its arrival; one output is wrong."""

    def __init__(self, bad_payload=None, capacity=None):
        self._lock = threading.Lock()
        self._t0 = time.monotonic_ns()
        self.next_id = 1
        self.pending = []
        self.outputs = {}
        self.released = set()
        self.bad_payload = bad_payload
        self.capacity = capacity
        self.submitted = self.completed = 0

    def now_ns(self):
        return time.monotonic_ns() - self._t0

    def submit(self, stream, arrival_ns=0):
        with self._lock:
            if self.capacity is not None and len(self.pending) >= self.capacity:
                return None
            rid = self.next_id
            self.next_id += 1
            self.pending.append((rid, arrival_ns, stream))
            self.submitted += 1
            return rid

    def poll(self, wait_us=0):
        out = []
        with self._lock:
            pending, self.pending = self.pending, []
        for rid, arrival, stream in pending:
            payload = self.bad_payload if stream == b"bad" else np.frombuffer(stream, np.uint8).copy()
            self.outputs[rid] = payload
            out.append(FakeResult(rid, arrival, arrival + 100_000, payload.size))
        self.completed += len(out)
        if not out and wait_us:
            time.sleep(min(wait_us, 1000) / 1e6)
        return out

    def schedule(self, pool, choice, offsets_ns, lead_ns=1_000_000):
        """A thread submitting pool[choice[i]] at start + offsets_ns[i], as gst_server_schedule does."""
        streams = [pool[c] for c in choice]
        start = self.now_ns() + lead_ns
        arrival_ns = [start + int(o) for o in offsets_ns]
        self._ids = np.zeros(len(streams), np.uint64)

        def run():
            sub = rej = late = 0
            for i, (st, at) in enumerate(zip(streams, arrival_ns)):
                while self.now_ns() < int(at):
                    time.sleep(0.0001)
                late = max(late, self.now_ns() - int(at))
                rid = self.submit(st, int(at))
                if rid is None:
                    rej += 1
                else:
                    self._ids[i] = rid
                    sub += 1
            self._sched = (sub, rej, late)

        self._thread = threading.Thread(target=run)
        self._thread.start()
        return self._ids, start

    def schedule_wait(self):
        self._thread.join()
        return self._sched

    def read(self, rid, nbytes):
        return self.outputs[rid]

    def release(self, rid):
        assert rid not in self.released
        self.released.add(rid)

    def stats(self, reset=False):
        return {"pixels": 0, "launches": 1, "launched_images": self.completed, "device_bytes_peak": 0,
                "queued": len(self.pending), "submitted": self.submitted, "completed": self.completed}


def requests():
    good = [(bytes(range(i, i + 16)), np.frombuffer(bytes(range(i, i + 16)), np.uint64)) for i in range(4)]
    return good


@pytest.mark.parametrize("native", [True, False])
def test_open_loop_counts_and_latency(native):
    srv = FakeServer()
    res = run_poisson(srv, requests(), rate=4000.0, seconds=0.25, seed=5, verify_every=2, native=native)
    s = res.summary()
    assert abs(s["submitted"] - 1000) < 150  # Poisson(1000)
    assert s["completed"] == s["submitted"] and s["rejected"] == 0
    assert len(srv.released) == s["completed"]
    assert s["verified"] == s["submitted"] // 2 and s["bit_exact"]
    assert abs(s["p50_ms"] - 0.1) < 1e-6 and abs(s["p99_ms"] - 0.1) < 1e-6


@pytest.mark.parametrize("native", [True, False])
def test_mismatch_and_rejection_are_reported(native):
    reqs = requests() + [(b"bad", np.zeros(2, np.uint64))]
    srv = FakeServer(bad_payload=np.ones(16, np.uint8))
    res = run_poisson(srv, reqs, rate=2000.0, seconds=0.2, seed=6, verify_every=1,
                      pick=lambda rng: 4, native=native)
    assert res.mismatched == res.verified > 0 and not res.summary()["bit_exact"]
    srv2 = FakeServer(capacity=0)
    res2 = run_poisson(srv2, requests(), rate=2000.0, seconds=0.1, seed=7, native=native)
    assert res2.rejected > 0 and res2.submitted == 0


def test_inline_checks_release_every_result_at_once():
    """hold=False: a checked result is read, compared and released as soon as it
    is polled (a run whose device budget binds cannot wait for held outputs);
    a wrong output is still counted."""
    srv = FakeServer()
    res = run_poisson(srv, requests(), rate=4000.0, seconds=0.25, seed=8, verify_every=2, hold=False)
    s = res.summary()
    assert s["completed"] == s["submitted"] > 0 and len(srv.released) == s["completed"]
    assert s["verified"] == s["submitted"] // 2 and s["bit_exact"]
    reqs = requests() + [(b"bad", np.zeros(2, np.uint64))]
    srv = FakeServer(bad_payload=np.ones(16, np.uint8))
    res = run_poisson(srv, reqs, rate=2000.0, seconds=0.2, seed=9, verify_every=1, pick=lambda rng: 4, hold=False)
    assert res.mismatched == res.verified > 0 and len(srv.released) == res.completed
