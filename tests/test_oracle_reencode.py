"""The C oracle's restatement of DXTImage::Reencode (codec/dxt_image.cpp:
510-624) against the reference's own results (tests/golden/reencode.json,
made by the reference itself through oracle/ref_harness.cpp), and against the
reference live when its CPU code is built here."""
import json
import sys

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

sys.path.insert(0, str(GOLDEN))
from reencode_inputs import CASES, edit_blocks, make_rgb, unpack  # noqa: E402


@pytest.fixture(scope="module")
def fixture():
    return json.loads((GOLDEN / "reencode.json").read_text())["cases"]


def expected(c):
    pal = unpack(c["palette"], np.uint8)
    return unpack(c["blocks_out"], np.uint64), pal, unpack(c["deltas"], np.uint8)


def test_fixture_covers_the_search_paths(fixture):
    names = {c["name"] for c in fixture}
    assert names == {c["name"] for c in CASES}
    by = {c["name"]: c for c in fixture}
    B = lambda c: c["width"] * c["height"] // 16  # noqa: E731
    assert by["noise256x64_stb"]["palette_words"] > 0.9 * B(by["noise256x64_stb"])  # > 127 appends per 256 blocks
    assert by["smooth256x128_plain"]["palette_words"] < 8                            # nearly every block reuses
    assert by["flat32_stb"]["refit"] == 0
    assert all(c["refit"] > 0 for c in fixture if c["name"].startswith("synth"))
    assert sum(1 for c in fixture if "stream_sha256" in c) >= 1


def test_oracle_reencode_matches_reference_fixtures(fixture):
    for c in fixture:
        w, h = c["width"], c["height"]
        rgb = make_rgb(c)
        blocks = unpack(c["blocks_in"], np.uint64)
        want_b, want_p, want_d = expected(c)
        got_b, got_p, got_d = oracle.reencode(w, h, rgb, blocks)
        assert np.array_equal(got_b, want_b), c["name"]
        assert np.array_equal(got_p[: want_p.size], want_p), c["name"]
        assert got_p.size % 8192 == 0 and not got_p[want_p.size:].any(), c["name"]
        assert np.array_equal(got_d, want_d), c["name"]


def test_fixture_inputs_regenerate(fixture):
    """The non-stb inputs come back from their recipes (the producer's block
    compressor is deterministic on this host)."""
    from gst_gb300 import encoder
    for c in fixture:
        if c["blocks"] == "stb":
            continue
        rgb = make_rgb(c)
        blocks = edit_blocks(encoder.compress_blocks(rgb, nthreads=1), c["blocks"], c["seed"])
        assert np.array_equal(blocks, unpack(c["blocks_in"], np.uint64)), c["name"]


def test_float_constants_of_the_refit():
    """(3 - order) / 3 and order / 3 in float: the kernel uses these bit patterns."""
    assert (np.float32(2) / np.float32(3)).view(np.uint32) == 0x3F2AAAAB
    assert (np.float32(1) / np.float32(3)).view(np.uint32) == 0x3EAAAAAB


def test_refit_to_a_single_index_word_is_never_usable():
    """All 16 pixels on one index: the normal equations are singular (1/0),
    the endpoints come out of NaN or infinity as INT32_MIN -> 0 and equal,
    so the refit would swap and is skipped."""
    px = np.arange(48, dtype=np.uint8) * 5
    for word in (0x00000000, 0x55555555):
        err, ok, e1, e2 = oracle.reencode_candidate(px, word)
        assert not ok and e1 == e2 == 0


@pytest.mark.skipif(oracle.load_ref() is None, reason="reference CPU code not built here")
def test_oracle_matches_reference_live():
    ref = oracle.load_ref()
    from gst_gb300 import encoder
    sys.path.insert(0, str(GOLDEN))
    from make_reencode_golden import reference_reencode, stb_blocks
    for seed, (w, h) in enumerate([(96, 64), (128, 128), (64, 192)]):
        rgb = encoder.synth_image(w, h, 100 + seed, 0.2)
        blocks = stb_blocks(ref, w, h, rgb)
        rb, rp, rd, _ = reference_reencode(ref, w, h, rgb, blocks, False)
        ob, op, od = oracle.reencode(w, h, rgb, blocks)
        assert np.array_equal(ob, rb) and np.array_equal(op[: rp.size], rp) and np.array_equal(od, rd)


def given_error(px48: np.ndarray, blk: int) -> int:
    """The error of a DXT1 block as given (dxt_image.cpp:144-170, 266-285):
    the three-colour palette, black last, when ep1 <= ep2."""
    def rgb(v):
        r, g, b = v >> 11, (v >> 5) & 63, v & 31
        return np.array([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (b << 3) | (b >> 2)], np.int64)
    e1, e2, word = blk & 0xFFFF, (blk >> 16) & 0xFFFF, blk >> 32
    a, c = rgb(e1), rgb(e2)
    pal = [a, c, (a + c) // 2, np.zeros(3, np.int64)] if e1 <= e2 else [a, c, (2 * a + c) // 3, (a + 2 * c) // 3]
    px = px48.reshape(16, 3).astype(np.int64)
    err = sum(int(((px[i] - pal[(word >> (2 * i)) & 3]) ** 2).sum()) for i in range(16))
    return err // 48


def test_search_output_invariants(fixture):
    """On every fixture: the index deltas rebuild each block's palette index
    (prefix sums of delta - 128, starting at 0), the palette word there is the
    block's word, a block either keeps its given block or carries the refit
    of its pixels to that word with an error raise below 35, and every
    palette word is the word of a block that kept its own block."""
    for c in fixture:
        w, h = c["width"], c["height"]
        rgb = make_rgb(c)
        given = unpack(c["blocks_in"], np.uint64)
        out = unpack(c["blocks_out"], np.uint64)
        words = unpack(c["palette"], np.uint8).view(np.uint32)
        idx = np.cumsum(unpack(c["deltas"], np.uint8).astype(np.int64) - 128)
        assert idx[0] == 0 and idx.min() >= 0 and idx.max() < words.size
        assert np.array_equal(words[idx], (out >> np.uint64(32)).astype(np.uint32)), c["name"]
        bw = w // 4
        for b in np.nonzero(out != given)[0][:64]:  # a sample of the refit blocks
            by, bx = divmod(int(b), bw)
            px = rgb[4 * by:4 * by + 4, 4 * bx:4 * bx + 4].reshape(48)
            err, ok, e1, e2 = oracle.reencode_candidate(px, int(out[b] >> np.uint64(32)))
            assert ok and int(out[b]) & 0xFFFFFFFF == e1 | (e2 << 16), (c["name"], b)
            assert err - given_error(px, int(given[b])) < 35, (c["name"], b)
        first_use = {}
        for b, k in enumerate(idx):
            first_use.setdefault(int(k), b)
        for k, b in first_use.items():  # the block that appended word k kept its own block
            assert out[b] == given[b] and int(given[b] >> np.uint64(32)) == int(words[k]), (c["name"], k)
