"""The benchmark inputs made by the reference encoder (tests/golden/ref_streams/,
written by tests/golden/make_ref_streams.py): every stream matches its
manifest digest, has the configured size and seed, and decodes under the
oracle (the reference decoder's arithmetic) to the blocks whose digest the
manifest holds; where the reference's CPU code is built here, re-encoding an
image with it reproduces the committed stream byte for byte."""
import hashlib
import json
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from gst_gb300 import encoder, workloads

MANIFEST = GOLDEN / "ref_streams" / "manifest.json"
pytestmark = pytest.mark.skipif(not MANIFEST.exists(), reason="reference-encoded fixtures not present")

SHA = lambda b: hashlib.sha256(bytes(b)).hexdigest()  # noqa: E731


@pytest.fixture(scope="module")
def manifest():
    return json.loads(MANIFEST.read_text())


def test_manifest_covers_the_configs(manifest):
    ents = manifest["streams"]
    batch = sorted((e for e in ents if e["kind"] == "batched"), key=lambda e: e["seed"])
    assert [(e["width"], e["height"]) for e in batch] == workloads.batched_dims(64)
    assert [e["seed"] for e in batch] == [1000 + i for i in range(64)]
    (large,) = [e for e in ents if e["kind"] == "large"]
    assert (large["width"], large["height"], large["seed"], large["checker_frac"]) == (8192, 8192, 8192, 0.10)
    pool = workloads.ref_serving_pool()
    assert set(pool) == {(w, h) for w in workloads.SERVING_DIMS for h in workloads.SERVING_DIMS}
    assert min(len(v) for v in pool.values()) >= 4
    assert manifest["encoder"].startswith("reference gentenc path")


def test_streams_match_digests_and_decode(manifest):
    """Every stream: its digest, its header's size, and the oracle's decode
    against the committed decoded-block digest (all 93 streams, 326 Mpix)."""
    def check(e):
        s = (GOLDEN / "ref_streams" / e["name"]).read_bytes()
        assert SHA(s) == e["stream_sha256"] and len(s) == e["gst_bytes"]
        w, h = (int.from_bytes(s[i:i + 4], "little") for i in (0, 4))
        assert (w, h) == (e["width"], e["height"])
        st, dec = oracle.decode(s, oracle.SCAN_EXACT)
        assert st == 0
        assert SHA(np.ascontiguousarray(dec)) == e["decoded_sha256"], e["name"]
        return e["blocks_differing_from_encoder"]

    with ThreadPoolExecutor(8) as ex:
        wrapped = list(ex.map(check, manifest["streams"]))
    # Only the 8192^2 texture's checker regions push wavelet coefficients past
    # 8 bits; the reference decoder then returns other blocks than the
    # encoder's (the reference's own behaviour, kept).
    assert sum(wrapped) == manifest["streams"][[e["kind"] for e in manifest["streams"]].index("large")][
        "blocks_differing_from_encoder"]


def test_plain_and_rans_fixtures(manifest, golden):
    im = workloads.ref_plain()
    st, dec = oracle.decode(im.stream, oracle.SCAN_EXACT)
    assert st == 0 and SHA(np.ascontiguousarray(dec)) == im.decoded_sha256 == \
        golden["streams"]["synth512_s0.gst"]["blocks_sha256"]
    r = manifest["rans_2pow26"]
    assert r["symbols"] == 1 << 26 and r["encoder"].startswith("reference ByteEncoder")


def test_project_producer_matches_reference_rans_section():
    """The 2^26 Laplace(6) section that the rANS workload decodes is byte for
    byte the reference ByteEncoder's (digest made by the reference)."""
    sec = workloads.rans_section()
    assert SHA(sec.section) == workloads.ref_rans_digest()["section_sha256"]


def test_reference_reencodes_a_fixture(manifest):
    """Where the reference's CPU code is built: the reference encoder, run on
    the generator's image again, writes the committed stream."""
    if not oracle.build_ref():
        pytest.skip("reference sources not mounted")
    import ctypes
    ref = oracle.load_ref()
    e = min((e for e in manifest["streams"] if e["kind"] == "serving"), key=lambda e: e["width"] * e["height"])
    rgb = encoder.synth_image(e["width"], e["height"], e["seed"], e["checker_frac"])
    cap = 1 << 24
    out = (ctypes.c_uint8 * cap)()
    blocks = (ctypes.c_uint8 * (rgb.shape[0] * rgb.shape[1] // 2))()
    n = ctypes.c_size_t()
    assert ref.gstref_compress_rgb(rgb.shape[1], rgb.shape[0], rgb.tobytes(), out, cap, ctypes.byref(n), blocks) == 0
    assert SHA(bytes(out[: n.value])) == e["stream_sha256"]
    assert SHA(bytes(blocks)) == e["encoder_blocks_sha256"]
