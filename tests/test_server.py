"""The continuous-batching decode server (gst_server_*): every result in a mix
of concurrent requests equals the plain single-image decode of the same stream
alone, bit for bit; admission holds to the device budget; a malformed stream
is reported on its own request only."""
import time

import numpy as np
import pytest

import oracle
from conftest import golden_stream
from gst_gb300 import decoder, workloads
from gst_gb300.server import DecodeServer, run_poisson

pytestmark = pytest.mark.gpu

MIX_DIMS = [(512, 512), (1024, 512), (2048, 1024), (512, 2048), (1024, 1024), (2048, 2048), (4096, 1024)]


def mixed_images():
    return [workloads.encode_image(w, h, 900 + i) for i, (w, h) in enumerate(MIX_DIMS)]


def collect(srv, n, timeout=60.0):
    got = {}
    deadline = time.monotonic() + timeout
    while len(got) < n and time.monotonic() < deadline:
        for r in srv.poll(20000):
            got[r.id] = (r.status, srv.read(r.id, r.dxt_bytes) if r.status == decoder.GST_OK else None)
            srv.release(r.id)
    return got


def test_results_same_alone_and_in_mix(gpu_ctx):
    imgs = mixed_images()
    alone = [decoder.decompress_dxt(gpu_ctx, im.stream) for im in imgs]
    for a, im in zip(alone, imgs):
        assert np.array_equal(a.view(np.uint64), im.blocks)
    budget = 64 << 20
    with DecodeServer(gpu_ctx, device_budget_bytes=budget, max_inflight=3, max_batch_images=5) as srv:
        order = list(range(len(imgs))) * 6
        np.random.default_rng(3).shuffle(order)
        ids = {}
        for k, i in enumerate(order):
            rid = srv.submit(imgs[i].stream)
            assert rid is not None
            ids[rid] = i
            if k % 5 == 4:
                time.sleep(0.0005)  # later requests arrive while earlier ones are on the GPU
        got = collect(srv, len(ids))
        assert len(got) == len(ids)
        for rid, i in ids.items():
            st, out = got[rid]
            assert st == decoder.GST_OK
            assert np.array_equal(out, alone[i]), (rid, MIX_DIMS[i])
        stats = srv.stats()
        assert stats["completed"] == len(ids)
        assert stats["launches"] < len(ids)  # requests shared launches
        assert stats["device_bytes_peak"] <= budget


def test_admission_waits_for_released_memory(gpu_ctx):
    im = workloads.encode_image(2048, 2048, 950)
    need = -(-len(im.stream) // 256) * 256 + im.blocks.size * 8
    budget = 2 * need + 1024  # room for two requests, not three
    with DecodeServer(gpu_ctx, device_budget_bytes=budget, max_inflight=2, max_batch_images=4) as srv:
        ids = [srv.submit(im.stream) for _ in range(5)]
        assert None not in ids
        first = []
        deadline = time.monotonic() + 30
        while len(first) < 2 and time.monotonic() < deadline:
            first += srv.poll(20000)
        time.sleep(0.05)
        first += srv.poll(0)
        assert len(first) == 2  # outputs held: the other three wait for memory
        stats = srv.stats()
        assert stats["queued"] == 3 and stats["device_bytes_in_use"] <= budget
        outs = [srv.read(r.id, r.dxt_bytes) for r in first]
        for r in first:
            srv.release(r.id)
        rest = collect(srv, 3)
        assert len(rest) == 3
        for out in outs + [o for _, o in rest.values()]:
            assert np.array_equal(out.view(np.uint64), im.blocks)
        assert srv.stats()["device_bytes_peak"] <= budget


def test_cancel_queued_request(gpu_ctx):
    """gst_server_cancel withdraws a request that waits for device memory: its
    memory returns at once, it never completes, the rest decode bit-exactly;
    a request already launched cannot be cancelled."""
    im = workloads.encode_image(2048, 2048, 950)
    need = -(-len(im.stream) // 256) * 256 + im.blocks.size * 8
    budget = 2 * need + 1024  # room for two requests, not three
    with DecodeServer(gpu_ctx, device_budget_bytes=budget, max_inflight=2, max_batch_images=4) as srv:
        ids = [srv.submit(im.stream) for _ in range(5)]
        assert None not in ids
        first = []
        deadline = time.monotonic() + 30
        while len(first) < 2 and time.monotonic() < deadline:
            first += srv.poll(20000)
        assert len(first) == 2 and srv.stats()["queued"] == 3
        done_ids = {r.id for r in first}
        assert not srv.cancel(first[0].id)  # done: not cancellable
        queued = [i for i in ids if i not in done_ids]
        assert srv.cancel(queued[1])
        assert not srv.cancel(queued[1])  # gone
        st = srv.stats()
        assert st["queued"] == 2 and st["cancelled"] == 1
        for r in first:
            srv.release(r.id)
        rest = collect(srv, 2)
        assert set(rest) == {queued[0], queued[2]}
        for status, out in rest.values():
            assert status == decoder.GST_OK and np.array_equal(out.view(np.uint64), im.blocks)
        time.sleep(0.05)
        assert srv.poll(0) == [] and srv.stats()["completed"] == 4


def _device_detected_corruption():
    # A payload flip that passes host validation and that the oracle reports
    # as malformed (a read leaves its group or the palette).
    base = bytearray(golden_stream("synth512_s0.gst"))
    hdr = decoder.parse_header(bytes(base))
    body = 28 + 2048
    rng = np.random.default_rng(21)
    for _ in range(200):
        s = bytearray(base)
        for pos in rng.integers(body + 4 * 64, body + hdr.compressed_bytes, size=8):
            s[int(pos)] ^= int(rng.integers(1, 256))
        s = bytes(s)
        try:
            decoder.parse_header(s)
        except decoder.GstError:
            continue
        if oracle.decode(s, oracle.SCAN_EXACT)[0] != 0:
            return s
    pytest.skip("no device-detected corruption found")


def test_malformed_stream_fails_alone(gpu_ctx):
    bad = _device_detected_corruption()
    imgs = mixed_images()[:4]
    with DecodeServer(gpu_ctx, device_budget_bytes=64 << 20, max_inflight=1, max_batch_images=16) as srv:
        ids = {srv.submit(im.stream): k for k, im in enumerate(imgs)}
        bad_id = srv.submit(bad)
        ids.update({srv.submit(im.stream): k for k, im in enumerate(imgs)})
        got = collect(srv, len(ids) + 1)
        assert got[bad_id][0] == decoder.GST_E_FORMAT
        for rid, k in ids.items():
            st, out = got[rid]
            assert st == decoder.GST_OK
            assert np.array_equal(out.view(np.uint64), imgs[k].blocks)


def test_poisson_load_bit_exact(gpu_ctx):
    imgs = mixed_images()
    reqs = [(im.stream, im.blocks) for im in imgs]
    with DecodeServer(gpu_ctx, device_budget_bytes=1 << 30) as srv:
        res = run_poisson(srv, reqs, rate=2000.0, seconds=0.5, seed=1, verify_every=3)
    s = res.summary()
    assert s["completed"] == s["submitted"] > 0 and s["rejected"] == 0
    assert s["verified"] > 0 and s["bit_exact"]
    assert 0 < s["p50_ms"] <= s["p99_ms"]


def test_poisson_load_python_submitter_bit_exact(gpu_ctx):
    """The same load with this process submitting (native=False)."""
    imgs = mixed_images()
    reqs = [(im.stream, im.blocks) for im in imgs]
    with DecodeServer(gpu_ctx, device_budget_bytes=1 << 30) as srv:
        res = run_poisson(srv, reqs, rate=2000.0, seconds=0.3, seed=2, verify_every=3, native=False)
    s = res.summary()
    assert s["completed"] == s["submitted"] > 0 and s["rejected"] == 0 and s["bit_exact"]


def test_native_schedule_submits_on_time(gpu_ctx):
    """gst_server_schedule: every stream submitted at its arrival time from
    the library's thread, ids written before the requests run, results
    bit-exact; a second schedule while one runs is refused."""
    imgs = mixed_images()
    with DecodeServer(gpu_ctx, device_budget_bytes=1 << 30) as srv:
        n = 300
        pool = [im.stream for im in imgs]
        choice = [i % len(imgs) for i in range(n)]
        offsets = np.arange(n, dtype=np.uint64) * np.uint64(200_000)  # 5k req/s for 60 ms
        ids, _ = srv.schedule(pool, choice, offsets)
        with pytest.raises(Exception):
            srv.schedule(pool, choice[:1], offsets[:1])
        got = collect(srv, n)
        sub, rej, late_ns = srv.schedule_wait()
        assert sub == n and rej == 0 and len(got) == n
        assert len(set(int(x) for x in ids)) == n and 0 not in set(int(x) for x in ids)
        assert late_ns < 50_000_000  # well within the run: the thread keeps up at 5k req/s
        for i, rid in enumerate(ids):
            st, dxt = got[int(rid)]
            assert st == decoder.GST_OK
            assert np.array_equal(dxt.view(np.uint64), imgs[i % len(imgs)].blocks)
