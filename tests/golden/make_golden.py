"""Regenerates the golden fixtures in this directory from the reference itself.

Runs only where the reference sources are mounted: it builds the reference's
CPU code (oracle/build_ref.sh) and calls it through oracle/ref_harness.cpp.
Nothing here is needed at test time; the tests read the committed outputs:

* ``test1.gst``            -- the reference encoder's stream for its own test
                              image codec/test/test1.png (codec/test/codec_test.cpp:36-48);
* ``synth512_s0.gst``      -- the plain-decode workload: the 512x512 synthetic
                              image of seed 0 encoded by the reference encoder;
* ``synth768x512_s3.gst``  -- a legal size whose block count (24,576) is not a
                              power of two, where the reference's staged index
                              scan (codec/decode_indices.cl) disagrees with the
                              encoder on the last block;
* ``rans_vectors.bin`` + ``golden.json`` -- the rANS decode vectors of
  ans/ans_ocl_test.cpp:157-345 (same frequency vectors, stream counts and
  srand(0)/rand() symbol draws), the decode tables of :64-155, the histogram
  known answers of ans/histogram_test.cpp:85-103, the 4x4 inverse wavelet known
  answer of codec/test/wavelet_test.cpp:129-158, ans::GenerateHistogram on
  seeded count vectors (ties, uint32 wrap, large corrections), and SHA-256
  digests of the reference encoder's DXT1 blocks and of its ByteEncoder
  sections.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from gst_gb300 import encoder  # noqa: E402

REF_TEST_IMAGE = Path("/root/reference/codec/test/test1.png")


def sha(b) -> str:
    return hashlib.sha256(bytes(b)).hexdigest()


def ref_compress_rgb(ref, rgb):
    h, w, _ = rgb.shape
    cap = 1 << 26
    stream = (ctypes.c_uint8 * cap)()
    blocks = (ctypes.c_uint8 * (w * h // 2))()
    n = ctypes.c_size_t()
    assert ref.gstref_compress_rgb(w, h, rgb.tobytes(), stream, cap, ctypes.byref(n), blocks) == 0
    return bytes(stream[: n.value]), bytes(blocks)


def ref_compress_file(ref, path):
    cap = 1 << 26
    stream = (ctypes.c_uint8 * cap)()
    blocks = (ctypes.c_uint8 * (1 << 24))()
    n = ctypes.c_size_t()
    w = ctypes.c_int()
    h = ctypes.c_int()
    assert ref.gstref_compress_file(str(path).encode(), stream, cap, ctypes.byref(n), blocks, 1 << 24,
                                    ctypes.byref(w), ctypes.byref(h)) == 0
    return bytes(stream[: n.value]), bytes(blocks[: w.value * h.value // 2])


def ref_histogram(ref, counts, M):
    c = np.asarray(counts, dtype=np.uint32)
    out = np.zeros_like(c)
    assert ref.gstref_generate_histogram(c.ctypes.data, c.size, M, out.ctypes.data) == 0
    return [int(v) for v in out]


def ref_encode_interleaved(ref, F, symbols, streams):
    f = np.asarray(F, dtype=np.uint32)
    s = np.ascontiguousarray(symbols, dtype=np.uint8)
    cap = 1 << 20
    out = (ctypes.c_uint8 * cap)()
    n = ctypes.c_size_t()
    assert ref.gstref_encode_interleaved(f.ctypes.data, f.size, s.ctypes.data, s.size, streams, out, cap,
                                         ctypes.byref(n)) == 0
    return bytes(out[: n.value])


def ref_encode_single(ref, F, symbols):
    f = np.asarray(F, dtype=np.uint32)
    s = np.ascontiguousarray(symbols, dtype=np.uint8)
    cap = 1 << 20
    out = (ctypes.c_uint8 * cap)()
    n = ctypes.c_size_t()
    state = ctypes.c_uint32()
    assert ref.gstref_rans_encode_single(f.ctypes.data, f.size, s.ctypes.data, s.size, out, cap, ctypes.byref(n),
                                         ctypes.byref(state)) == 0
    return bytes(out[: n.value]), int(state.value)


def next4(x: int) -> int:
    return (x + 3) // 4 * 4


def main() -> None:
    if not oracle.build_ref():
        raise SystemExit("reference sources not available; cannot regenerate fixtures")
    ref = oracle.load_ref()
    gold: dict = {"streams": {}, "rans": [], "tables": [], "histograms": [], "histogram_stress": [], "sections": []}

    # --- whole streams from the reference encoder -------------------------------
    s, blocks = ref_compress_file(ref, REF_TEST_IMAGE)
    (HERE / "test1.gst").write_bytes(s)
    gold["streams"]["test1.gst"] = {"width": 512, "height": 512, "blocks_sha256": sha(blocks),
                                    "source": "codec/test/test1.png"}
    for name, (w, h, seed) in {"synth512_s0.gst": (512, 512, 0), "synth768x512_s3.gst": (768, 512, 3)}.items():
        rgb = encoder.synth_image(w, h, seed)
        s, blocks = ref_compress_rgb(ref, rgb)
        (HERE / name).write_bytes(s)
        st_ref, dec_ref = oracle.decode(s, oracle.SCAN_REFERENCE)
        bad = np.nonzero(np.frombuffer(dec_ref.tobytes(), np.uint64) != np.frombuffer(blocks, np.uint64))[0]
        gold["streams"][name] = {"width": w, "height": h, "seed": seed, "blocks_sha256": sha(blocks),
                                 "reference_scan_sha256": sha(dec_ref), "reference_scan_mismatch": [int(v) for v in bad]}

    # --- rANS vectors of ans/ans_ocl_test.cpp ---------------------------------------
    libc = ctypes.CDLL(None)
    libc.rand.restype = ctypes.c_int
    libc.srand(0)

    def gen_symbols(F, n):  # ans_ocl_test.cpp:40-62
        M = sum(F)
        out = []
        for _ in range(n):
            r = libc.rand() % M
            acc, sym = 0, 0
            for f in F:
                acc += f
                if r < acc:
                    break
                sym += 1
            out.append(sym)
        return np.asarray(out, dtype=np.uint8)

    blob = bytearray()

    def add_case(name, F, streams, groups_syms, bodies):
        nonlocal blob
        body = b"".join(bodies) if isinstance(bodies, list) else bodies
        expected = np.concatenate(groups_syms).astype(np.uint8)
        norm = ref_histogram(ref, F, 2048)
        case = {"name": name, "F": list(F), "freqs": norm, "streams": streams, "n_groups": len(groups_syms) // streams,
                "body_off": len(blob), "body_len": len(body)}
        blob += body
        case["sym_off"] = len(blob)
        case["sym_len"] = int(expected.size)
        blob += expected.tobytes()
        gold["rans"].append(case)

    # DecodeSingleStream (:157-218): one stream, layout of OpenCLDecoder::Decode(state, data).
    F1 = [12, 14, 17, 1, 1, 2, 372]
    sym1 = gen_symbols(F1, 256)
    data, state = ref_encode_single(ref, F1, sym1)
    off = next4(len(data) + 8)
    body = bytearray(off)
    body[0:4] = off.to_bytes(4, "little")
    body[off - len(data) - 4: off - 4] = data
    body[off - 4:] = state.to_bytes(4, "little")
    add_case("single_stream", F1, 1, [sym1], bytes(body))

    # DecodeInterleavedStreams (:220-275): 24 interleaved streams in one group.
    F2 = [32, 186, 54, 8, 94, 35, 13, 21, 456, 789, 33, 215, 6, 54, 987, 54, 65, 13, 2, 1]
    sym2 = [gen_symbols(F2, 256) for _ in range(24)]
    enc = ref_encode_interleaved(ref, F2, np.concatenate(sym2), 24)
    off = next4(len(enc) + 4)
    body = bytearray(off)
    body[0:4] = off.to_bytes(4, "little")
    body[off - len(enc):] = enc
    add_case("interleaved_24", F2, 24, sym2, bytes(body))

    # DecodeMultipleInterleavedStreams (:277-345): two groups of one stream.
    F3 = [65, 4, 6, 132, 135, 64, 879, 87, 456, 13, 2, 12, 33, 16, 546, 987, 98, 74, 65, 43, 21, 32, 1]
    sym3 = [gen_symbols(F3, 256) for _ in range(2)]
    regions, ends = [], []
    total = 0
    for g in range(2):
        data, state = ref_encode_single(ref, F3, sym3[g])
        sz = next4(len(data)) + 4
        reg = bytearray(sz)
        reg[sz - 4:] = state.to_bytes(4, "little")
        reg[sz - 4 - len(data): sz - 4] = data
        regions.append(bytes(reg))
        total += sz
        ends.append(total + 4 * 2)
    body = b"".join(e.to_bytes(4, "little") for e in ends) + b"".join(regions)
    add_case("multiple_groups", F3, 1, sym3, body)

    # GST-layout groups: 32 streams x 256 symbols from the reference ByteEncoder.
    rng = np.random.default_rng(11)
    lap = (np.rint(rng.laplace(0, 6, 4 * 8192)).astype(np.int64) % 256).astype(np.uint8)
    cap = 1 << 22
    buf = (ctypes.c_uint8 * cap)()
    n = ctypes.c_size_t()
    assert ref.gstref_encode_bytes(lap.tobytes(), lap.size, buf, cap, ctypes.byref(n)) == 0
    sec = bytes(buf[: n.value])
    freqs = [int(v) for v in np.frombuffer(sec[:512], dtype=np.uint16)]
    blob_case = {"name": "gst_groups_laplace6", "F": None, "freqs": freqs, "streams": 32, "n_groups": 4,
                 "body_off": len(blob), "body_len": len(sec) - 512}
    blob += sec[512:]
    blob_case["sym_off"] = len(blob)
    blob_case["sym_len"] = int(lap.size)
    blob += lap.tobytes()
    gold["rans"].append(blob_case)
    (HERE / "rans_vectors.bin").write_bytes(bytes(blob))

    # --- decode tables of ans_ocl_test.cpp:64-155 -------------------------------
    for F in ([3, 2, 1, 4, 3], [80, 300, 2, 14, 1, 1, 1, 20]):
        gold["tables"].append({"F": F, "normalized": ref_histogram(ref, F, 2048)})

    # --- histogram known answers (ans/histogram_test.cpp:85-103) ------------------
    for counts, M in (([1, 2, 3, 4, 5, 6, 7, 8, 9, 10], 256), ([1, 2, 3, 4, 5, 6, 7, 8, 9, 10], 11),
                      ([3, 2, 1, 4, 3], 2048), ([12, 14, 17, 1, 1, 2, 372], 2048)):
        gold["histograms"].append({"counts": counts, "M": M, "expected": ref_histogram(ref, counts, M)})

    # --- GenerateHistogram on count vectors with ties, uint32 wrap and large
    #     corrections: pins the heap order of the frequency correction ---------
    for seed, kind, M in HISTOGRAM_CASES:
        counts = histogram_input(seed, kind)
        gold["histogram_stress"].append({"seed": seed, "kind": kind, "M": M,
                                         "expected": ref_histogram(ref, counts, M)})

    # --- ByteEncoder sections: digests the project's encoders must reproduce ------
    for seed, kind, n_groups in SECTION_CASES:
        x = section_input(seed, kind, n_groups)
        assert ref.gstref_encode_bytes(x.tobytes(), x.size, buf, cap, ctypes.byref(n)) == 0
        gold["sections"].append({"seed": seed, "kind": kind, "n_groups": n_groups, "bytes": int(n.value),
                                 "sha256": sha(bytes(buf[: n.value]))})

    # --- 4x4 inverse wavelet known answer (codec/test/wavelet_test.cpp:129-158) ---
    gold["wavelet_4x4"] = {
        "input": [63, 64, 0, -1, 66, 60, 6, 9, 0, 2, -2, -2, 7, -18, 16, 36],
        "expected": [63, 63, 63, 63, 63, 63, 64, 63, 63, 65, 62, 64, 62, 65, 31, 69],
    }
    (HERE / "golden.json").write_text(json.dumps(gold, indent=1) + "\n")
    print("wrote", sorted(p.name for p in HERE.iterdir()))


SECTION_CASES = ((21, "laplace1", 1), (22, "laplace6", 3), (23, "laplace20", 2), (24, "uniform", 2),
                 (25, "two_symbols", 1), (26, "seven_symbols", 2), (27, "rare_tail", 3), (28, "one_symbol", 1),
                 (29, "skewed", 2), (30, "wrap255", 1), (31, "rare_group", 4), (32, "laplace6", 70))

HISTOGRAM_KINDS = ("small_values", "spike", "equal", "wrap", "laplace", "large")
HISTOGRAM_CASES = tuple((100 + i, HISTOGRAM_KINDS[i % 6], 2048 if i % 5 else 4096 - 97 * i) for i in range(36))


def section_input(seed: int, kind: str, n_groups: int) -> np.ndarray:
    """Seeded input bytes of one ByteEncoder section (shared with the tests)."""
    rng = np.random.default_rng(seed)
    n = 8192 * n_groups
    if kind.startswith("laplace"):
        b = float(kind[len("laplace"):])
        return (np.rint(rng.laplace(0, b, n)).astype(np.int64) % 256).astype(np.uint8)
    if kind == "uniform":
        return rng.integers(0, 256, n).astype(np.uint8)
    if kind == "two_symbols":
        return np.where(rng.random(n) < 0.9, 128, 131).astype(np.uint8)
    if kind == "seven_symbols":  # equal counts: the frequency correction meets ties
        return rng.choice(np.array([3, 40, 77, 128, 129, 200, 254], np.uint8), n)
    if kind == "rare_tail":  # a Laplace body plus 60 symbols that occur once or twice
        x = (np.rint(rng.laplace(0, 4, n)).astype(np.int64) % 256).astype(np.uint8)
        pos = rng.choice(n, 90, replace=False)
        x[pos] = rng.integers(60, 200, 90).astype(np.uint8)
        return x
    if kind == "one_symbol":
        return np.full(n, 77, np.uint8)
    if kind == "skewed":  # 99.9 % one byte
        return np.where(rng.random(n) < 0.999, 128, rng.integers(0, 256, n)).astype(np.uint8)
    if kind == "wrap255":  # symbols 0 and 255 both present (256 table entries)
        return (np.rint(rng.laplace(0, 2, n)).astype(np.int64) % 256).astype(np.uint8)
    if kind == "rare_group":  # one group made only of the section's rarest symbols (one word per symbol)
        x = np.full(n, 128, np.uint8)
        x[: n // 2] = (np.rint(rng.laplace(0, 1, n // 2)).astype(np.int64) % 256).astype(np.uint8)
        x[n - 8192:] = rng.integers(0, 256, 8192).astype(np.uint8)
        return x
    raise ValueError(kind)


def histogram_input(seed: int, kind: str) -> np.ndarray:
    """Seeded count vectors for the GenerateHistogram cases (shared with the tests)."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 257))
    if kind == "small_values":
        c = rng.choice([1, 2, 3, 5, 8], size=n)
    elif kind == "spike":
        c = rng.integers(0, 4, size=n)
        c[rng.integers(0, n)] = rng.integers(1, 10**6)
    elif kind == "equal":
        c = np.full(n, int(rng.integers(1, 50)))
    elif kind == "wrap":  # counts * M overflow uint32 in the reference's product
        c = rng.integers(0, 3, size=n) * int(rng.integers(2_100_000, 3_000_000))
    elif kind == "laplace":
        c = np.round(np.exp(-np.abs(np.arange(n) - n / 2) / rng.uniform(1, 30)) * rng.integers(100, 10**7))
    elif kind == "large":
        c = rng.integers(0, 5_000_000, size=n)
    else:
        raise ValueError(kind)
    c = np.asarray(c, np.int64)
    c[-1] = max(c[-1], 1)
    return c.astype(np.uint32)


if __name__ == "__main__":
    main()
