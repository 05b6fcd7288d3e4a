"""The oracle's encoder stages (ans/histogram.cpp, ans/encode.cpp,
codec/entropy.cpp, codec/encoder.cpp restated in oracle/gst_oracle.c), pinned
against the reference: its GenerateHistogram answers and ByteEncoder digests
(tests/golden/golden.json, made by the reference itself) and its encoder's
whole streams, which the oracle rebuilds byte for byte from their symbols."""
import hashlib
import sys

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, golden_stream

sys.path.insert(0, str(GOLDEN))
from make_golden import histogram_input, section_input  # noqa: E402


def test_normalize_known_answers(golden):
    # ans/histogram_test.cpp:85-103 and the tables of ans/ans_ocl_test.cpp:64-155.
    for c in golden["histograms"]:
        st, out = oracle.normalize(c["counts"], c["M"])
        assert st == 0 and out.tolist() == c["expected"]
    for c in golden["tables"]:
        st, out = oracle.normalize(c["F"], 2048)
        assert st == 0 and out.tolist() == c["normalized"]


def test_normalize_heap_order_on_ties_and_wrap(golden):
    # Equal ranks (equal counts), uint32 wrap of counts * M, corrections of
    # both signs: the heap's tie order decides which symbols move.
    assert len(golden["histogram_stress"]) >= 30
    for c in golden["histogram_stress"]:
        counts = histogram_input(c["seed"], c["kind"])
        st, out = oracle.normalize(counts, c["M"])
        assert st == 0 and out.tolist() == c["expected"], (c["seed"], c["kind"])
        assert int(out.sum()) == c["M"]


def test_normalize_rejects_what_the_reference_asserts_on():
    assert oracle.normalize([0, 0, 0], 2048)[0] != 0
    assert oracle.normalize([1, 2], 0)[0] != 0
    assert oracle.normalize([5] * 10, 8)[0] != 0  # ten symbols cannot share 8 units


def test_encode_section_matches_reference_digests(golden):
    for c in golden["sections"]:
        x = section_input(c["seed"], c["kind"], c["n_groups"])
        st, sec = oracle.encode_section(x)
        assert st == 0 and len(sec) == c["bytes"], c["kind"]
        assert hashlib.sha256(sec).hexdigest() == c["sha256"], c["kind"]


@pytest.mark.parametrize("name", ["test1.gst", "synth512_s0.gst", "synth768x512_s3.gst"])
def test_encode_stream_rebuilds_reference_streams(name):
    # codec/encoder.cpp:122-144 over the decoded symbols of a stream that the
    # reference encoder wrote gives back that stream exactly.
    s = golden_stream(name)
    w, h, pal = (int.from_bytes(s[i:i + 4], "little") for i in (0, 4, 8))
    st, sym = oracle.decode_symbols(s)
    assert st == 0
    st, again = oracle.encode_stream(w, h, pal, *oracle.split_symbols(w, h, pal, sym))
    assert st == 0 and again == s


def test_encode_section_round_trip_through_oracle_decoder():
    for seed, kind, g in ((41, "laplace6", 5), (42, "rare_group", 4), (43, "one_symbol", 1), (44, "uniform", 3)):
        x = section_input(seed, kind, g)
        st, sec = oracle.encode_section(x)
        assert st == 0
        st, got = oracle.rans_decode_groups(sec[512:], np.frombuffer(sec[:512], np.uint16), g, 32)
        assert st == 0 and np.array_equal(got, x), kind


def test_encode_section_argument_checks():
    assert oracle.encode_section(np.zeros(0, np.uint8))[0] != 0
    assert oracle.encode_section(np.zeros(8191, np.uint8))[0] != 0
    st, sec = oracle.encode_section(np.zeros(8192, np.uint8))  # only byte 0: F[0] = 2048
    assert st == 0 and np.frombuffer(sec[:4], np.uint16).tolist() == [2048, 0]


def test_normalize_matches_reference_on_random_counts():
    ref = oracle.load_ref()
    if ref is None:
        pytest.skip("reference CPU code not built on this machine")
    rng = np.random.default_rng(77)
    for t in range(400):
        counts = histogram_input(int(rng.integers(1 << 30)), ("small_values", "spike", "equal", "wrap",
                                                               "laplace", "large")[t % 6])
        M = 2048 if t % 3 else int(rng.integers(int((counts > 0).sum()) + 1, 5000))
        want = np.zeros_like(counts)
        assert ref.gstref_generate_histogram(counts.ctypes.data, counts.size, M, want.ctypes.data) == 0
        st, out = oracle.normalize(counts, M)
        assert st == 0 and np.array_equal(out, want)


@pytest.mark.parametrize("name", ["test1.gst", "synth512_s0.gst", "synth768x512_s3.gst"])
def test_endpoint_planes_rebuild_reference_sections(name):
    # codec/encoder.cpp:20-98 over the blocks a reference stream decodes to
    # gives back that stream's Y and chroma sections.
    s = golden_stream(name)
    w, h, pal = (int.from_bytes(s[i:i + 4], "little") for i in (0, 4, 8))
    st, dxt = oracle.decode(s, oracle.SCAN_EXACT)
    assert st == 0
    st, sym = oracle.decode_symbols(s)
    y, c, clips = oracle.endpoint_planes(w, h, np.frombuffer(dxt.tobytes(), np.uint64))
    B = w * h // 16
    assert clips == 0 and np.array_equal(y, sym[:2 * B]) and np.array_equal(c, sym[2 * B:6 * B])


def test_run_palette_stream_decodes_to_its_blocks():
    from gst_gb300 import encoder
    rgb = encoder.synth_image(1024, 512, 31, 0.1)
    _, blocks, clips = encoder.encode_rgb(rgb)
    assert clips == 0
    y, c, clips = oracle.endpoint_planes(1024, 512, blocks)
    pal, deltas = oracle.run_palette(1024, 512, blocks)
    assert clips == 0 and set(np.unique(deltas)) <= {128, 129} and pal.size % 8192 == 0
    st, stream = oracle.encode_stream(1024, 512, pal.size, y, c, pal, deltas)
    assert st == 0
    st, dxt = oracle.decode(stream, oracle.SCAN_EXACT)
    assert st == 0 and np.array_equal(np.frombuffer(dxt.tobytes(), np.uint64), blocks)
