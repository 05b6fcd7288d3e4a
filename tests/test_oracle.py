"""The CPU oracle, pinned against the reference: golden streams from the
reference encoder, the reference's own test vectors, and (where it is built on
this machine) the reference's CPU rANS decoder and inverse wavelet."""
import hashlib

import numpy as np
import pytest

import oracle
from conftest import as_blocks, golden_stream

SHA = lambda b: hashlib.sha256(bytes(b)).hexdigest()  # noqa: E731


@pytest.mark.parametrize("name", ["test1.gst", "synth512_s0.gst"])
@pytest.mark.parametrize("mode", [oracle.SCAN_REFERENCE, oracle.SCAN_EXACT])
def test_golden_stream_decodes_to_encoder_blocks(golden, name, mode):
    # codec/test/codec_test.cpp:36-48: decode == the encoder's PhysicalBlocks().
    st, dxt = oracle.decode(golden_stream(name), mode)
    assert st == 0
    assert SHA(dxt) == golden["streams"][name]["blocks_sha256"]


def test_reference_scan_diverges_on_non_power_of_two_block_count(golden):
    # 768x512 = 24,576 blocks: the staged scan of codec/decode_indices.cl
    # (driven by codec/decoder.cpp:302-393) misses the last block's carry; the
    # exact prefix sum reproduces the encoder's blocks.
    g = golden["streams"]["synth768x512_s3.gst"]
    s = golden_stream("synth768x512_s3.gst")
    st, ref_scan = oracle.decode(s, oracle.SCAN_REFERENCE)
    assert st == 0 and SHA(ref_scan) == g["reference_scan_sha256"]
    assert g["reference_scan_mismatch"] == [24575]
    st, exact = oracle.decode(s, oracle.SCAN_EXACT)
    assert st == 0 and SHA(exact) == g["blocks_sha256"]
    diff = np.nonzero(as_blocks(exact) != as_blocks(ref_scan))[0]
    assert diff.tolist() == [24575]


@pytest.mark.parametrize("n", [8192 * k for k in (1, 2, 4, 8, 16, 32, 64, 128, 512)])
def test_reference_scan_equals_exact_for_power_of_two_counts(n):
    # Every benchmark size has a power-of-two block count (2^14 .. 2^22).
    if n & (n - 1):
        pytest.skip("not a power of two")
    rng = np.random.default_rng(n)
    d = rng.integers(0, 256, n).astype(np.uint8)
    assert np.array_equal(oracle.scan_indices(d, oracle.SCAN_REFERENCE), oracle.scan_indices(d, oracle.SCAN_EXACT))


def test_reference_scan_power_of_two_large():
    n = 1 << 22  # the 8192x8192 texture
    d = np.random.default_rng(3).integers(96, 160, n).astype(np.uint8)
    assert np.array_equal(oracle.scan_indices(d, oracle.SCAN_REFERENCE), oracle.scan_indices(d, oracle.SCAN_EXACT))


def test_tables_match_ans_ocl_test(golden):
    # ans/ans_ocl_test.cpp:64-155: the table is the expansion of the normalised F.
    for case in golden["tables"]:
        norm = case["normalized"]
        assert sum(norm) == 2048
        fr, cu, sy = oracle.build_table(norm)
        exp_sym = np.repeat(np.arange(len(norm)), norm)
        exp_f = np.repeat(norm, norm)
        exp_c = np.repeat(np.concatenate([[0], np.cumsum(norm)[:-1]]), norm)
        assert np.array_equal(sy, exp_sym) and np.array_equal(fr, exp_f) and np.array_equal(cu, exp_c)


def test_table_search_equals_direct_fill_on_random_tables():
    # build_table.cl's 11-step search vs the direct expansion, including tables
    # with many zero frequencies and single-symbol tables.
    rng = np.random.default_rng(0)
    for trial in range(400):
        k = int(rng.integers(1, 257))
        f = np.zeros(256, dtype=np.int64)
        pos = np.sort(rng.choice(256, size=k, replace=False))
        if trial % 3 == 0:
            cuts = np.sort(rng.choice(np.arange(1, 2048), size=k - 1, replace=False)) if k > 1 else np.array([], int)
            parts = np.diff(np.concatenate([[0], cuts, [2048]]))
        else:
            w = rng.random(k) ** 4
            parts = np.maximum(1, np.floor(w / w.sum() * 2048)).astype(np.int64)
            parts[np.argmax(parts)] += 2048 - parts.sum()
            if parts.min() < 1:
                continue
        f[pos] = parts
        assert f.sum() == 2048
        a = oracle.build_table(f)
        b = oracle.build_table(f, direct=True)
        for x, y in zip(a, b):
            assert np.array_equal(x, y), trial


def _batch_offsets(rng, n):
    offs, o = [], 0
    for _ in range(n):
        B = 8192 * int(rng.choice([2, 4, 8, 16, 32]))
        P = 8192 * int(rng.integers(1, 9))
        for sz in (2 * B, 4 * B, P, B):
            offs.append(o)
            o += sz
    return np.asarray(offs, dtype=np.uint32), o


def _search_mismatches(oo, total):
    lib = oracle.load()
    bad = []
    for wg in range(total // 8192):
        want = int(np.searchsorted(oo, wg * 8192, side="right") - 1)
        got = lib.gsto_section_search(oo.ctypes.data, oo.size, wg)
        if got != want:
            bad.append((wg, want, got))
    return bad


@pytest.mark.parametrize("n", [1, 2, 4, 8, 16, 32, 64])
def test_section_search_exact_for_power_of_two_batches(n):
    # ans_decode.cl:104-121 assigns every work-group its true section when the
    # batch has a power-of-two number of images (the 64-image workload).
    rng = np.random.default_rng(n)
    for _ in range(5):
        oo, total = _batch_offsets(rng, n)
        assert _search_mismatches(oo, total) == []


@pytest.mark.parametrize("n", [3, 12, 48])
def test_section_search_misses_last_section_otherwise(n):
    # With 4n offsets not a power of two, the search's iteration count
    # (32 - clz(4n)) is one short when it climbs to the last section: the
    # groups of the last image's index section are decoded with the palette
    # section's table and offsets.  The product builds its work list on the
    # host and has no such search.
    rng = np.random.default_rng(100 + n)
    oo, total = _batch_offsets(rng, n)
    bad = _search_mismatches(oo, total)
    last = int(oo[-1]) // 8192
    assert bad and all(want == 4 * n - 1 and got == 4 * n - 2 and wg >= last for wg, want, got in bad)


def test_wavelet_4x4_known_answer(golden):
    # codec/test/wavelet_test.cpp:129-158.
    k = golden["wavelet_4x4"]
    blk = np.asarray(k["input"], dtype=np.int32)
    oracle.load().gsto_inverse_wavelet_level(blk.ctypes.data, 4, 4)
    assert blk.tolist() == k["expected"]


def test_ycocg_to_565_is_inverse_of_forward():
    # assemble.cl:39-62 inverts codec/image_processing.cpp:10-27 on every RGB565.
    lib = oracle.load()
    for c in range(0, 65536, 7):
        r, g, b = c >> 11, (c >> 5) & 63, c & 31
        co = r - b
        t = r + b + (b >> 4)
        cg = g - t
        y = t + int(cg / 2)
        assert lib.gsto_ycocg_to_565(y, co, cg) == c


@pytest.mark.parametrize("idx", range(4))
def test_rans_vectors(golden, rans_blob, idx):
    # ans/ans_ocl_test.cpp:157-345 and GST-layout groups.
    c = golden["rans"][idx]
    body = rans_blob[c["body_off"]: c["body_off"] + c["body_len"]]
    want = np.frombuffer(rans_blob[c["sym_off"]: c["sym_off"] + c["sym_len"]], dtype=np.uint8)
    st, got = oracle.rans_decode_groups(body, c["freqs"], c["n_groups"], c["streams"])
    assert st == 0
    assert np.array_equal(got, want)


def test_malformed_streams_rejected():
    lib = oracle.load()
    s = bytearray(golden_stream("test1.gst"))
    hdr = np.zeros(7, np.uint32)
    assert lib.gsto_parse_header(bytes(s), len(s), hdr.ctypes.data) == 0
    assert lib.gsto_parse_header(bytes(s[:-4]), len(s) - 4, hdr.ctypes.data) == 2  # truncated
    bad = bytearray(s)
    bad[0:4] = (500).to_bytes(4, "little")  # width not a multiple of 128
    assert lib.gsto_parse_header(bytes(bad), len(bad), hdr.ctypes.data) == 2
    bad = bytearray(s)
    bad[28:30] = (int.from_bytes(bad[28:30], "little") + 1).to_bytes(2, "little")  # table sum 2049
    assert lib.gsto_parse_header(bytes(bad), len(bad), hdr.ctypes.data) == 2
    bad = bytearray(s)
    body = 28 + 2048
    bad[body: body + 4] = (3).to_bytes(4, "little")  # first group end before the offset table ends
    assert lib.gsto_parse_header(bytes(bad), len(bad), hdr.ctypes.data) == 2


# --- against the reference's own CPU code (only where it is built here) -------------

@pytest.fixture(scope="module")
def ref():
    lib = oracle.load_ref()
    if lib is None:
        pytest.skip("reference CPU code not built on this machine (oracle/build_ref.sh)")
    return lib


def test_rans_stage_matches_reference_decode_interleaved(ref):
    # Per group: oracle rANS == ans::DecodeInterleaved (ans/decode.cpp:240-292).
    for name in ("test1.gst", "synth512_s0.gst", "synth768x512_s3.gst"):
        s = golden_stream(name)
        st, syms = oracle.decode_symbols(s)
        assert st == 0
        hdr = np.frombuffer(s[:28], np.uint32)
        w, h, pal = int(hdr[0]), int(hdr[1]), int(hdr[2])
        B = w * h // 16
        lens = hdr[3:7].astype(np.int64)
        nsyms = [2 * B, 4 * B, pal, B]
        body = 28 + 2048
        out_off = 0
        for sec in range(4):
            F = np.frombuffer(s[28 + 512 * sec: 28 + 512 * (sec + 1)], np.uint16).astype(np.uint32)
            F = F[: int(np.nonzero(F)[0].max()) + 1]
            G = nsyms[sec] // 8192
            secb = s[body: body + int(lens[sec])]
            prev = 4 * G
            for g in range(G):
                end = int.from_bytes(secb[4 * g: 4 * g + 4], "little")
                data = secb[prev:end]
                out = np.zeros(8192, np.uint8)
                assert ref.gstref_decode_interleaved(data, len(data), 8192, F.ctypes.data, F.size, 32,
                                                     out.ctypes.data) == 0
                assert np.array_equal(out, syms[out_off + g * 8192: out_off + (g + 1) * 8192]), (name, sec, g)
                prev = end
            out_off += nsyms[sec]
            body += int(lens[sec])


def test_wavelet_matches_reference_inverse_wavelet2d(ref):
    # Per 32x32 block: oracle == InverseWavelet2D at dims 2..32 (codec/wavelet.cpp:133-155)
    # on valid coefficient data (where the reference's int16 never overflows).
    s = golden_stream("synth512_s0.gst")
    st, syms = oracle.decode_symbols(s)
    lib = oracle.load()
    for t in range(0, 96, 7):
        blk = syms[t * 1024:(t + 1) * 1024]
        mine = np.zeros(1024, np.int8)
        lib.gsto_inverse_wavelet_block(blk.ctypes.data, mine.ctypes.data)
        a = (blk.astype(np.int16) - 128).reshape(32, 32)
        for dim in (2, 4, 8, 16, 32):
            sub = np.ascontiguousarray(a[:dim, :dim])
            out = np.zeros((dim, dim), np.int16)
            ref.gstref_inverse_wavelet2d(sub.ctypes.data, out.ctypes.data, dim)
            a[:dim, :dim] = out
        assert np.array_equal(a.astype(np.int8).ravel(), mine)


def test_histogram_known_answers(ref, golden):
    for c in golden["histograms"]:
        counts = np.asarray(c["counts"], np.uint32)
        out = np.zeros_like(counts)
        assert ref.gstref_generate_histogram(counts.ctypes.data, counts.size, c["M"], out.ctypes.data) == 0
        assert out.tolist() == c["expected"]


def test_rgb_oracle_is_four_colour_dxt1_decode():
    # The RGB restatement (assemble.cl:83-129) equals a four-colour DXT1 decode
    # of the DXT1 blocks the pinned DXT path produces (valid streams keep every
    # 5:6:5 channel in range, where the two agree).
    for name in ("test1.gst", "synth768x512_s3.gst"):
        s = golden_stream(name)
        st, rgb = oracle.decode_rgb(s, oracle.SCAN_EXACT)
        st2, dxt = oracle.decode(s, oracle.SCAN_EXACT)
        assert st == st2 == 0
        w = int.from_bytes(s[0:4], "little")
        h = int.from_bytes(s[4:8], "little")
        blk = dxt.view(np.uint64)
        e0 = (blk & 0xFFFF).astype(np.int64)
        e1 = ((blk >> np.uint64(16)) & 0xFFFF).astype(np.int64)
        sel_word = (blk >> np.uint64(32)).astype(np.uint64)

        def widen(e):
            r, g, b = (e >> 11) & 31, (e >> 5) & 63, e & 31
            return np.stack([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (b << 3) | (b >> 2)], -1)

        p0, p1 = widen(e0), widen(e1)
        pal = np.stack([p0, p1, (2 * p0 + p1) // 3, (p0 + 2 * p1) // 3], 1)
        bx = w // 4
        img = np.zeros((h, w, 3), np.uint8)
        n = np.arange(blk.size)
        for pix in range(16):
            sel = ((sel_word >> np.uint64(2 * pix)) & np.uint64(3)).astype(np.int64)
            img[(n // bx) * 4 + pix // 4, (n % bx) * 4 + pix % 4] = pal[n, sel]
        assert np.array_equal(img.reshape(-1), rgb), name
