"""gst_load_compressed_dxt_static: the one-image decode that allocates nothing.

It exists for callers that may not allocate device memory while they decode
(a frame-budgeted render or streaming thread that cannot absorb the
device-wide synchronisation of cudaMalloc/cudaFree, an engine that owns all
device memory), so its scratch is an array built into the library instead of
cudaMalloc'd memory.  These tests call it through the C ABI and check it
against the allocating entry point, gst_load_compressed_dxt, on two calls in a
row, against the reference encoder's golden blocks and the oracle, and on a
malformed payload (reported through device_status, then a clean decode).  This
file is collected last so that a run stopping at the first failure has already
run every other test."""
import ctypes
import hashlib

import numpy as np
import pytest

import oracle
from conftest import golden_stream
from gst_gb300 import decoder, workloads

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _device_layout(stream: bytes):
    hdrs, packed = decoder.pack_batch([stream])
    return hdrs[0], torch.from_numpy(packed).cuda()


def _static_decode(hdr, d_cmp, d_out, side):
    status = ctypes.c_uint32(0xFFFFFFFF)
    rc = decoder.load_library().gst_load_compressed_dxt_static(
        ctypes.byref(hdr), d_cmp.data_ptr(), d_out.data_ptr(), side.cuda_stream, ctypes.byref(status))
    return rc, status.value


def test_static_decode_matches_allocating_entry_point_twice_in_a_row():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    side = torch.cuda.Stream()
    streams = [golden_stream("test1.gst"), workloads.encode_image(2048, 1024, 77).stream]
    ctx = decoder.GPUContext(0)
    try:
        for s in streams:
            hdr, d_cmp = _device_layout(s)
            want = torch.zeros(hdr.dxt_bytes, dtype=torch.uint8, device="cuda")
            decoder.load_compressed_dxt(ctx, hdr, d_cmp, want)
            assert decoder.sync_status(ctx) == decoder.GST_OK
            want = want.cpu().numpy()
            for call in range(2):
                got = torch.full((hdr.dxt_bytes,), 0xA5, dtype=torch.uint8, device="cuda")
                torch.cuda.synchronize()
                rc, bits = _static_decode(hdr, d_cmp, got, side)
                assert rc == decoder.GST_OK, call
                assert bits == 0, call
                assert np.array_equal(got.cpu().numpy(), want), call
    finally:
        ctx.close()


def test_static_decode_matches_golden_blocks_and_oracle(golden):
    """The reference encoder's stream of its own test image decodes to the
    encoder's blocks (codec/test/codec_test.cpp:36-48), and a 2048x2048
    reference-encoded batch image to the oracle's blocks, twice each."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    side = torch.cuda.Stream()
    cases = [(golden_stream("test1.gst"), golden["streams"]["test1.gst"]["blocks_sha256"])]
    if workloads.ref_available():
        im = max(workloads.ref_batched(), key=lambda im: im.pixels)  # 2048x2048, the largest that fits
        cases.append((im.stream, im.decoded_sha256))
    for s, digest in cases:
        st, want = oracle.decode(s, oracle.SCAN_EXACT)
        assert st == 0 and hashlib.sha256(np.ascontiguousarray(want).tobytes()).hexdigest() == digest
        hdr, d_cmp = _device_layout(s)
        for call in range(2):
            got = torch.full((hdr.dxt_bytes,), 0x5A, dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            rc, bits = _static_decode(hdr, d_cmp, got, side)
            assert rc == decoder.GST_OK and bits == 0, call
            out = got.cpu().numpy()
            assert hashlib.sha256(out.tobytes()).hexdigest() == digest, call
            assert np.array_equal(out, np.ascontiguousarray(want).reshape(-1).view(np.uint8)), call


def _malformed_payload():
    # A payload flip that passes host validation and that the oracle reports
    # as malformed (a read leaves its group, or an index leaves the palette).
    base = bytearray(golden_stream("synth512_s0.gst"))
    hdr = decoder.parse_header(bytes(base))
    body = 28 + 2048
    rng = np.random.default_rng(31)
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


def test_static_decode_reports_malformed_payload_then_decodes_cleanly(golden):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    side = torch.cuda.Stream()
    bad = _malformed_payload()
    hdr, d_cmp = _device_layout(bad)
    out = torch.zeros(hdr.dxt_bytes, dtype=torch.uint8, device="cuda")
    rc, bits = _static_decode(hdr, d_cmp, out, side)
    assert rc == decoder.GST_OK and bits != 0
    # the next call starts from cleared status words and decodes exactly
    good = golden_stream("synth512_s0.gst")
    hdr, d_cmp = _device_layout(good)
    rc, bits = _static_decode(hdr, d_cmp, out, side)
    assert rc == decoder.GST_OK and bits == 0
    assert hashlib.sha256(out.cpu().numpy().tobytes()).hexdigest() == golden["streams"]["synth512_s0.gst"][
        "blocks_sha256"]


def test_static_decode_rejects_images_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    hdr = decoder.parse_header(golden_stream("test1.gst"))
    big = decoder.GenTCHeader(*hdr.as_tuple())
    big.width = big.height = 4096  # a well-formed 4096x4096 header needs ~7.4 MB of scratch
    big.y_cmp_sz, big.chroma_cmp_sz, big.indices_sz = 256 * 264, 512 * 264, 128 * 264
    d = torch.zeros(1024, dtype=torch.uint8, device="cuda")
    rc = decoder.load_library().gst_load_compressed_dxt_static(
        ctypes.byref(big), d.data_ptr(), d.data_ptr(), None, None)
    assert rc == decoder.GST_E_ARG
