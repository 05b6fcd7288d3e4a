"""The project's stream producer: byte-identical sections to the reference's
ByteEncoder, reference histogram answers, and lossless round trips through
the oracle decoder."""
import hashlib
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, as_blocks
from gst_gb300 import encoder, workloads

sys.path.insert(0, str(GOLDEN))
from make_golden import section_input  # noqa: E402


def test_sections_match_reference_byte_encoder(golden):
    # codec/entropy.cpp:174-265 + ans/histogram.cpp + ans/encode.cpp, byte for byte.
    for c in golden["sections"]:
        x = section_input(c["seed"], c["kind"], c["n_groups"])
        sec = encoder.encode_section(x)
        assert len(sec) == c["bytes"]
        assert hashlib.sha256(sec).hexdigest() == c["sha256"], c["kind"]


def test_histogram_known_answers(golden):
    for c in golden["histograms"]:
        assert encoder.normalize_frequencies(c["counts"], c["M"]).tolist() == c["expected"]
    for c in golden["tables"]:
        assert encoder.normalize_frequencies(c["F"], 2048).tolist() == c["normalized"]


def test_section_round_trip_single_symbol():
    # A one-symbol section (frequency 2048) decodes without reading any words.
    x = np.full(8192 * 2, 128, np.uint8)
    sec = encoder.encode_section(x)
    st, got = oracle.rans_decode_groups(sec[512:], np.frombuffer(sec[:512], np.uint16), 2, 32)
    assert st == 0 and np.array_equal(got, x)


@pytest.mark.parametrize("w,h,checker", [(512, 512, 0.0), (1024, 512, 0.0), (512, 1024, 0.0),
                                         (1024, 1024, 0.1), (2048, 512, 0.0)])
def test_round_trip_through_oracle(w, h, checker):
    rgb = encoder.synth_image(w, h, 42, checker)
    stream, blocks, clips = encoder.encode_rgb(rgb)
    assert clips == 0
    for mode in (oracle.SCAN_REFERENCE, oracle.SCAN_EXACT):
        st, dxt = oracle.decode(stream, mode, nthreads=4)
        assert st == 0
        assert np.array_equal(as_blocks(dxt), blocks)


def test_synth_image_is_deterministic():
    a = encoder.synth_image(512, 512, 7, 0.1)
    b = encoder.synth_image(512, 512, 7, 0.1)
    c = encoder.synth_image(512, 512, 8, 0.1)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.std() > 10


def test_batched_dims_cover_the_size_set():
    dims = workloads.batched_dims()
    assert len(dims) == 64
    assert {w for w, _ in dims} <= set(workloads.BATCH_DIMS) and {h for _, h in dims} <= set(workloads.BATCH_DIMS)
    assert len(set(dims)) > 5


def test_encode_dxt_keeps_given_blocks():
    rgb = encoder.synth_image(512, 512, 5)
    _, blocks, _ = encoder.encode_rgb(rgb)
    stream, blocks2, _ = encoder.encode_dxt(512, 512, blocks)  # exact-match palette reuse only
    assert np.array_equal(blocks, blocks2)
    st, dxt = oracle.decode(stream, oracle.SCAN_EXACT)
    assert st == 0 and np.array_equal(as_blocks(dxt), blocks)


def test_reference_encoder_stream_sizes_comparable():
    # Where the reference is built here: compare stream sizes on the same image.
    ref = oracle.load_ref()
    if ref is None:
        pytest.skip("reference CPU code not built on this machine")
    import ctypes
    rgb = encoder.synth_image(512, 512, 0)
    cap = 1 << 24
    buf = (ctypes.c_uint8 * cap)()
    blk = (ctypes.c_uint8 * (512 * 512 // 2))()
    n = ctypes.c_size_t()
    assert ref.gstref_compress_rgb(512, 512, rgb.tobytes(), buf, cap, ctypes.byref(n), blk) == 0
    mine, _, _ = encoder.encode_rgb(rgb)
    assert 0.3 < len(mine) / n.value < 1.5
