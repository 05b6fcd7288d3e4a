"""CUDA decode path vs the oracle and the golden fixtures, through the C ABI.

Bit-exact everywhere (integer and byte work).  Small cases compare against the
CPU oracle directly; full-size cases (8192x8192, the 2^26-symbol rANS section)
check the size-independent property that decoding returns exactly what the
encoder encoded, plus the oracle where it finishes in seconds."""
import hashlib

import numpy as np
import pytest

import oracle
from conftest import as_blocks, golden_stream
from gst_gb300 import decoder, encoder, workloads

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHA = lambda b: hashlib.sha256(bytes(b)).hexdigest()  # noqa: E731


def to_dev(a) -> "torch.Tensor":
    return torch.from_numpy(np.ascontiguousarray(np.frombuffer(bytes(a), dtype=np.uint8)).copy()).cuda()


def batch_decode(ctx, streams, stream=None):
    hdrs, packed = decoder.pack_batch(streams)
    d_cmp = torch.from_numpy(packed).cuda()
    total = sum(h.dxt_bytes for h in hdrs)
    d_out = torch.zeros(total, dtype=torch.uint8, device="cuda")
    decoder.load_compressed_dxts(ctx, hdrs, d_cmp, d_out, stream)
    st = decoder.sync_status(ctx, stream)
    out = d_out.cpu().numpy()
    res, off = [], 0
    for h in hdrs:
        res.append(out[off:off + h.dxt_bytes])
        off += h.dxt_bytes
    return st, res


@pytest.mark.parametrize("name", ["test1.gst", "synth512_s0.gst"])
def test_decompress_dxt_golden(gpu_ctx, golden, name):
    # codec/test/codec_test.cpp:36-48 on the GPU: DecompressDXT == PhysicalBlocks().
    out = decoder.decompress_dxt(gpu_ctx, golden_stream(name))
    assert SHA(out) == golden["streams"][name]["blocks_sha256"]
    st, ref = oracle.decode(golden_stream(name))
    assert np.array_equal(out, ref)


@pytest.mark.skipif(not workloads.ref_available(), reason="reference-encoded fixtures not present")
def test_reference_encoded_workloads(gpu_ctx):
    """The benchmark inputs as the reference encoder (gentenc's path) wrote
    them: the 64-image batch in one call (two-kernel and persistent forms),
    the 8192x8192 texture, and every serving-pool stream alone, each
    bit-exact against the digest of the reference decoder's blocks."""
    imgs = workloads.ref_batched()
    for persistent in (0, 1):
        gpu_ctx.set_option("persistent", persistent)
        try:
            st, outs = batch_decode(gpu_ctx, [im.stream for im in imgs])
        finally:
            gpu_ctx.set_option("persistent", 0)
        assert st == decoder.GST_OK
        for im, o in zip(imgs, outs):
            assert SHA(o) == im.decoded_sha256, (im.width, im.height, im.seed, persistent)
    big = workloads.ref_large()
    assert SHA(decoder.decompress_dxt(gpu_ctx, big.stream)) == big.decoded_sha256
    for ims in workloads.ref_serving_pool().values():
        for im in ims:
            assert SHA(decoder.decompress_dxt(gpu_ctx, im.stream)) == im.decoded_sha256


def test_balanced_rans_items_follow_the_tuning():
    """The 8192x8192 texture's 4331 groups fill 8 CTAs x 152 SMs with items of
    3.56 groups: at 8 CTAs per SM its plan is cut into equal items, at 12 it
    is not (2.4 groups an item), and switching the tuning re-cuts the resident
    plan; every form decodes to the reference decoder's blocks, direct, from
    the captured graph and through the host pipeline."""
    big = workloads.ref_large()
    ctx = decoder.GPUContext(0)
    try:
        hdrs, packed = decoder.pack_batch([big.stream])
        d_cmp = torch.from_numpy(packed).cuda()
        d_out = torch.empty(hdrs[0].dxt_bytes, dtype=torch.uint8, device="cuda")
        rb = decoder.ResidentBatch(ctx, hdrs)
        s = torch.cuda.Stream()
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        for bps, words in [(8, 1528), (12, 1016), (8, 1528)]:
            rb.set_tuning(bps, words, 0)
            for graph in (False, True):
                d_out.zero_()
                rb.launch(d_cmp, d_out, s, graph=graph)
                s.synchronize()
                assert decoder.sync_status(ctx, s) == decoder.GST_OK
                assert SHA(d_out.cpu().numpy()) == big.decoded_sha256, (bps, words, graph)
                # runs of 4 groups: 1083 items; balanced (8 CTAs per SM): one item
                # per place of the wave
                if bps == 8:
                    assert 1083 < rb.rans_items <= 8 * sms, rb.rans_items
                else:
                    assert rb.rans_items == 1083, rb.rans_items
        # the context's option turns the cut off: runs of 4 again, same blocks
        ctx.set_option("balance_rans_items", 0)
        d_out.zero_()
        rb.launch(d_cmp, d_out, s, graph=True)
        s.synchronize()
        assert rb.rans_items == 1083 and SHA(d_out.cpu().numpy()) == big.decoded_sha256
        ctx.set_option("balance_rans_items", 1)
        h_cmp = torch.from_numpy(packed).pin_memory()
        h_out = torch.zeros(hdrs[0].dxt_bytes, dtype=torch.uint8).pin_memory()
        rb.host_launch(h_cmp, h_out, 1, s)
        s.synchronize()
        assert SHA(h_out.numpy()) == big.decoded_sha256
        rb.close()
    finally:
        ctx.close()


EDGE_DIMS = [(512, 256), (256, 512), (128, 1024), (1024, 128), (8192, 128), (128, 8192)]


def test_smallest_and_thinnest_images(gpu_ctx):
    """The smallest images the format admits (one index group: 8192 blocks)
    and one-tile-wide or one-tile-high strips, alone, in one mixed batch, and
    as RGB8, against the oracle."""
    imgs = [workloads.encode_image(w, h, 40 + k) for k, (w, h) in enumerate(EDGE_DIMS)]
    want = []
    for im in imgs:
        st, dec = oracle.decode(im.stream, oracle.SCAN_EXACT)
        assert st == 0
        want.append(np.ascontiguousarray(dec).reshape(-1).view(np.uint8))
        assert np.array_equal(decoder.decompress_dxt(gpu_ctx, im.stream).reshape(-1), want[-1]), (im.width, im.height)
    st, outs = batch_decode(gpu_ctx, [im.stream for im in imgs])
    assert st == decoder.GST_OK
    for im, o, w in zip(imgs, outs, want):
        assert np.array_equal(o, w), (im.width, im.height)
    im = imgs[-1]
    hdrs, packed = decoder.pack_batch([im.stream])
    rgb = torch.zeros(im.width * im.height * 3, dtype=torch.uint8, device="cuda")
    decoder.load_rgb(gpu_ctx, hdrs[0], torch.from_numpy(packed).cuda(), rgb)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
    assert np.array_equal(rgb.cpu().numpy(), oracle.decode_rgb(im.stream, oracle.SCAN_EXACT)[1])


def test_16384_square_round_trip(gpu_ctx):
    """A 16384x16384 texture (16.8 M blocks, 134 MB of DXT1; four times the
    8192x8192 configuration): smooth endpoints and indices drawn from 256
    words, made into a GST stream by the GPU stream producer, decoded on the
    GPU, checked against the oracle and against the blocks it came from."""
    from gst_gb300 import entropy
    side = 16384
    n = side // 4
    rng = np.random.default_rng(16384)
    y, x = np.mgrid[0:n, 0:n].astype(np.int64)
    r = (x * 31) // n
    g = (y * 63) // n
    b = ((x + y) * 31) // (2 * n)
    ep1 = (r << 11) | (g << 5) | b
    ep2 = (np.minimum(r + 2, 31) << 11) | (np.maximum(g - 3, 0) << 5) | np.minimum(b + 1, 31)
    words = rng.integers(0, 1 << 32, 256, dtype=np.uint64)
    blocks = (ep1.astype(np.uint64) | (ep2.astype(np.uint64) << np.uint64(16)) |
              (words[rng.integers(0, 256, n * n)].reshape(n, n) << np.uint64(32))).reshape(-1)
    stream = entropy.compress_dxt(gpu_ctx, side, side, blocks)
    got = decoder.decompress_dxt(gpu_ctx, stream)
    st, want = oracle.decode(stream, oracle.SCAN_EXACT, nthreads=8)
    assert st == 0
    assert np.array_equal(got.view(np.uint64), np.ascontiguousarray(want).reshape(-1).view(np.uint64))
    assert np.array_equal(got.view(np.uint64), blocks)


def test_non_power_of_two_block_count_matches_encoder(gpu_ctx, golden):
    # The GPU computes the exact index prefix sum: it reproduces the encoder's
    # blocks, where the reference's staged scan differs in the last block.
    g = golden["streams"]["synth768x512_s3.gst"]
    out = decoder.decompress_dxt(gpu_ctx, golden_stream("synth768x512_s3.gst"))
    assert SHA(out) == g["blocks_sha256"]
    st, ref_scan = oracle.decode(golden_stream("synth768x512_s3.gst"), oracle.SCAN_REFERENCE)
    assert np.nonzero(as_blocks(out) != as_blocks(ref_scan))[0].tolist() == g["reference_scan_mismatch"]


@pytest.mark.parametrize("idx", range(4))
def test_rans_vectors(gpu_ctx, golden, rans_blob, idx):
    # ans/ans_ocl_test.cpp:157-345 (1, 24 and 32 interleaved streams).
    c = golden["rans"][idx]
    body = rans_blob[c["body_off"]: c["body_off"] + c["body_len"]]
    want = np.frombuffer(rans_blob[c["sym_off"]: c["sym_off"] + c["sym_len"]], dtype=np.uint8)
    freqs = np.zeros(256, np.uint16)
    freqs[: len(c["freqs"])] = c["freqs"]
    d_f = to_dev(freqs.tobytes())
    d_b = to_dev(body)
    d_o = torch.zeros(want.size, dtype=torch.uint8, device="cuda")
    decoder.decode_rans_groups(gpu_ctx, d_f, d_b, len(body), c["n_groups"], c["streams"], d_o)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
    assert np.array_equal(d_o.cpu().numpy(), want)


def test_batch_of_mixed_sizes_matches_oracle_and_encoder(gpu_ctx):
    imgs = [workloads.encode_image(w, h, 300 + i) for i, (w, h) in enumerate(
        [(512, 512), (1024, 512), (512, 1024), (1024, 1024), (2048, 512), (512, 2048), (512, 512)])]
    streams = [im.stream for im in imgs] + [golden_stream("test1.gst")]
    st, outs = batch_decode(gpu_ctx, streams)
    assert st == decoder.GST_OK
    for im, out in zip(imgs, outs):
        assert np.array_equal(as_blocks(out), im.blocks)
    for s, out in zip(streams, outs):
        st_o, ref = oracle.decode(s, oracle.SCAN_EXACT, nthreads=4)
        assert st_o == 0 and np.array_equal(out, ref)


def test_same_result_alone_and_in_batch(gpu_ctx):
    imgs = [workloads.encode_image(w, h, 400 + i) for i, (w, h) in enumerate([(1024, 512), (512, 512), (1024, 1024)])]
    st, together = batch_decode(gpu_ctx, [im.stream for im in imgs])
    assert st == 0
    for im, t in zip(imgs, together):
        alone = decoder.decompress_dxt(gpu_ctx, im.stream)
        assert np.array_equal(alone, t)


def test_device_resident_single_image(gpu_ctx):
    s = golden_stream("synth512_s0.gst")
    st, outs = batch_decode(gpu_ctx, [s])
    assert st == 0
    assert np.array_equal(outs[0], oracle.decode(s)[1])


def test_repeated_decodes_are_identical(gpu_ctx):
    s = workloads.encode_image(2048, 1024, 17).stream
    a = decoder.decompress_dxt(gpu_ctx, s)
    b = decoder.decompress_dxt(gpu_ctx, s)
    assert np.array_equal(a, b)


def test_single_symbol_sections(gpu_ctx):
    # A flat image: every section but the chroma/luma ones has one symbol, whose
    # frequency is 2048 (no renormalisation words at all).
    rgb = np.full((512, 512, 3), 77, np.uint8)
    stream, blocks, clips = encoder.encode_rgb(rgb)
    out = decoder.decompress_dxt(gpu_ctx, stream)
    assert np.array_equal(as_blocks(out), blocks)


def test_large_8192_round_trip(gpu_ctx):
    im = workloads.large()
    out = decoder.decompress_dxt(gpu_ctx, im.stream)
    assert np.array_equal(as_blocks(out), im.blocks)
    st, ref = oracle.decode(im.stream, oracle.SCAN_EXACT, nthreads=16)
    assert st == 0 and np.array_equal(out, ref)


def test_rans_micro_full_size(gpu_ctx):
    sec = workloads.rans_section()
    d_f = to_dev(sec.section[:512])
    d_b = to_dev(sec.section[512:])
    d_o = torch.zeros(sec.symbols.size, dtype=torch.uint8, device="cuda")
    decoder.decode_rans_groups(gpu_ctx, d_f, d_b, len(sec.section) - 512, sec.n_groups, 32, d_o)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
    assert np.array_equal(d_o.cpu().numpy(), sec.symbols)


def test_corrupted_payloads_match_oracle_and_are_flagged(gpu_ctx):
    # Byte flips inside group payloads pass header validation; the kernels keep
    # every read inside its group and the palette, and report GST_E_FORMAT when
    # a read would leave them -- exactly when the oracle does.  With GST_OK the
    # output is bit-exact; with GST_E_FORMAT it is unspecified (the reference's
    # decoder reads out of bounds there).
    base = bytearray(golden_stream("synth512_s0.gst"))
    rng = np.random.default_rng(9)
    hdr = decoder.parse_header(bytes(base))
    body = 28 + 2048
    flagged = 0
    for trial in range(12):
        s = bytearray(base)
        lo = body + 4 * 64  # past the Y section's offset table
        hi = body + hdr.compressed_bytes
        for pos in rng.integers(lo, hi, size=8):
            s[int(pos)] ^= int(rng.integers(1, 256))
        s = bytes(s)
        try:
            decoder.parse_header(s)
        except decoder.GstError:
            continue  # a flip hit an offset table: rejected on the host
        st_g, outs = batch_decode(gpu_ctx, [s])
        st_o, ref = oracle.decode(s, oracle.SCAN_EXACT)
        assert st_g == st_o, trial
        if st_g == decoder.GST_OK:
            assert np.array_equal(outs[0], ref), trial
        flagged += st_g != 0
    # The context stays usable afterwards.
    out = decoder.decompress_dxt(gpu_ctx, golden_stream("test1.gst"))
    assert np.array_equal(out, oracle.decode(golden_stream("test1.gst"))[1])


def test_device_checks_tables_and_group_offsets(gpu_ctx):
    # On the device-resident path the host holds only headers: a bad table sum
    # or group end offset is caught by the kernels, not by a fault.
    s = bytearray(golden_stream("synth512_s0.gst"))
    s[28:30] = (int.from_bytes(s[28:30], "little") + 1).to_bytes(2, "little")
    hdrs = [decoder.GenTCHeader.load_from(bytes(s))]
    packed = np.zeros(decoder.batch_layout_bytes(hdrs), np.uint8)
    packed[512:512 + 2048] = np.frombuffer(bytes(s[28:28 + 2048]), np.uint8)
    packed[512 + 2048:] = np.frombuffer(bytes(s[28 + 2048:]), np.uint8)
    d_cmp = torch.from_numpy(packed).cuda()
    d_out = torch.zeros(hdrs[0].dxt_bytes, dtype=torch.uint8, device="cuda")
    decoder.load_compressed_dxts(gpu_ctx, hdrs, d_cmp, d_out)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_E_FORMAT
    s2 = bytearray(golden_stream("synth512_s0.gst"))
    body = 28 + 2048
    s2[body + 4: body + 8] = (1 << 30).to_bytes(4, "little")
    packed[512:512 + 2048] = np.frombuffer(bytes(s2[28:28 + 2048]), np.uint8)
    packed[512 + 2048:] = np.frombuffer(bytes(s2[28 + 2048:]), np.uint8)
    d_cmp = torch.from_numpy(packed).cuda()
    decoder.load_compressed_dxts(gpu_ctx, hdrs, d_cmp, d_out)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_E_FORMAT
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK  # cleared


def test_preallocated_scratch():
    ctx = decoder.GPUContext(0)
    try:
        s = golden_stream("test1.gst")
        h = decoder.parse_header(s)
        decoder.preallocate_decompressor(ctx, decoder.required_scratch_mem(h))
        out = decoder.decompress_dxt(ctx, s)
        assert np.array_equal(out, oracle.decode(s)[1])
        big = workloads.encode_image(1024, 1024, 3).stream
        with pytest.raises(decoder.GstError) as e:
            decoder.decompress_dxt(ctx, big)
        assert e.value.status == decoder.GST_E_OOM
        decoder.free_decompressor(ctx)
        out = decoder.decompress_dxt(ctx, big)
        assert np.array_equal(out, oracle.decode(big, oracle.SCAN_EXACT)[1])
    finally:
        ctx.close()


def test_host_validation_before_launch(gpu_ctx):
    s = golden_stream("test1.gst")
    with pytest.raises(decoder.GstError) as e:
        decoder.decompress_dxt(gpu_ctx, s[:-100])
    assert e.value.status == decoder.GST_E_FORMAT


def test_stream_argument_and_launch_count(gpu_ctx):
    s = golden_stream("synth512_s0.gst")
    side = torch.cuda.Stream()
    st, outs = batch_decode(gpu_ctx, [s, s], stream=side)
    assert st == 0 and np.array_equal(outs[0], outs[1])
    assert gpu_ctx.last_launch_count() == 2


def test_resident_batch_launch_and_graph_replay(gpu_ctx):
    # A resident batch launched directly and through its captured graph, twice
    # each, gives the encoder's blocks every time (the plan re-arms itself).
    imgs = [workloads.encode_image(w, h, 600 + i) for i, (w, h) in enumerate([(1024, 512), (512, 512), (2048, 1024)])]
    hdrs, packed = decoder.pack_batch([im.stream for im in imgs])
    want = np.concatenate([im.blocks for im in imgs])
    d_cmp = torch.from_numpy(packed).cuda()
    d_out = torch.zeros(sum(h.dxt_bytes for h in hdrs), dtype=torch.uint8, device="cuda")
    b = decoder.ResidentBatch(gpu_ctx, hdrs)
    assert b.device_bytes > 0
    side = torch.cuda.Stream()
    for graph in (False, False, True, True):
        d_out.zero_()
        torch.cuda.synchronize()
        b.launch(d_cmp, d_out, side, graph=graph)
        assert decoder.sync_status(gpu_ctx, side) == decoder.GST_OK
        assert np.array_equal(d_out.cpu().numpy().view(np.uint64), want), graph
    b.close()


AUTOTUNED = [(16, 520, 0), (12, 520, 0), (12, 1016, 0), (8, 1528, 0), (8, 2040, 0), (8, 2816, 0), (8, 4352, 0),
             (8, 1016, 1), (8, 2040, 1)]
TUNINGS = AUTOTUNED + [(10, 904, 0), (12, 2816, 1)]


def test_every_tuning_decodes_identically(gpu_ctx):
    # The rANS launch configuration (CTAs per SM x staging depth) changes only
    # the time.  A high-entropy section (about 3,700 words per group, so every
    # depth re-stages) and a mixed batch decode bit-identically under each.
    sym = workloads.laplace_bytes(1 << 20, b=40.0, seed=11)
    sec = encoder.encode_section(sym)
    d_f, d_b = to_dev(sec[:512]), to_dev(sec[512:])
    d_o = torch.zeros(sym.size, dtype=torch.uint8, device="cuda")
    imgs = [workloads.encode_image(w, h, 700 + i) for i, (w, h) in enumerate([(1024, 1024), (512, 512), (2048, 512)])]
    hdrs, packed = decoder.pack_batch([im.stream for im in imgs])
    want = np.concatenate([im.blocks for im in imgs])
    d_cmp = torch.from_numpy(packed).cuda()
    d_out = torch.zeros(sum(h.dxt_bytes for h in hdrs), dtype=torch.uint8, device="cuda")
    b = decoder.ResidentBatch(gpu_ctx, hdrs)
    try:
        for bps, words, pers in TUNINGS:
            gpu_ctx.set_option("rans_blocks_per_sm", bps)
            gpu_ctx.set_option("rans_stage_words", words)
            gpu_ctx.set_option("persistent", pers)
            d_o.zero_()
            decoder.decode_rans_groups(gpu_ctx, d_f, d_b, len(sec) - 512, sym.size // 8192, 32, d_o)
            assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
            assert np.array_equal(d_o.cpu().numpy(), sym), (bps, words)
            for graph in (False, False, True, True):  # the persistent plan re-arms itself
                d_out.zero_()
                b.launch(d_cmp, d_out, graph=graph)  # untuned: follows the context
                assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
                assert np.array_equal(d_out.cpu().numpy().view(np.uint64), want), (bps, words, pers, graph)
            st, outs = batch_decode(gpu_ctx, [im.stream for im in imgs])  # per-call plans
            assert st == decoder.GST_OK
            assert np.array_equal(np.concatenate(outs).view(np.uint64), want), (bps, words, pers)
    finally:
        gpu_ctx.set_option("rans_blocks_per_sm", 12)
        gpu_ctx.set_option("rans_stage_words", 1016)
        gpu_ctx.set_option("persistent", 0)
        b.close()


def test_auto_tuning_option_restores_the_default():
    """The context's tuning options replace the size-dependent default; the
    "auto_tuning" option brings it back, and a one-image decode is exact
    under either."""
    ctx = decoder.GPUContext(0)
    try:
        im = workloads.encode_image(1024, 512, 731)
        ctx.set_option("rans_blocks_per_sm", 8)
        assert decoder.get_class_tuning(ctx, 0) == (8, 1016, 0)
        assert np.array_equal(as_blocks(decoder.decompress_dxt(ctx, im.stream)), im.blocks)
        ctx.set_option("auto_tuning", 1)
        assert decoder.get_class_tuning(ctx, 0) == (12, 1016, 0)
        assert np.array_equal(as_blocks(decoder.decompress_dxt(ctx, im.stream)), im.blocks)
        with pytest.raises(decoder.GstError) as ei:
            ctx.set_option("auto_tuning", 0)
        assert ei.value.status == decoder.GST_E_ARG
    finally:
        ctx.close()


def test_batch_autotune_and_tuning_validation(gpu_ctx):
    imgs = [workloads.encode_image(w, h, 720 + i) for i, (w, h) in enumerate([(2048, 2048), (1024, 512)])]
    hdrs, packed = decoder.pack_batch([im.stream for im in imgs])
    want = np.concatenate([im.blocks for im in imgs])
    d_cmp = torch.from_numpy(packed).cuda()
    d_out = torch.zeros(sum(h.dxt_bytes for h in hdrs), dtype=torch.uint8, device="cuda")
    b = decoder.ResidentBatch(gpu_ctx, hdrs)
    side = torch.cuda.Stream()
    tuned = b.autotune(d_cmp, d_out, side, iterations=2)
    assert tuned in AUTOTUNED
    assert decoder.sync_status(gpu_ctx, side) == decoder.GST_OK
    assert np.array_equal(d_out.cpu().numpy().view(np.uint64), want)
    # Every later launch does the whole decode: output cleared before each.
    for tuning in (None, (8, 2040, 1), (8, 1016, 1), (12, 1016, 0)):
        if tuning:
            b.set_tuning(*tuning)
        for graph in (False, True, True):
            d_out.zero_()
            torch.cuda.synchronize()
            b.launch(d_cmp, d_out, side, graph=graph)
            assert decoder.sync_status(gpu_ctx, side) == decoder.GST_OK, (tuning, graph)
            assert np.array_equal(d_out.cpu().numpy().view(np.uint64), want), (tuning, graph)
    for bad in ((12, 512, 0), (12, 1001, 0), (12, 4360, 0), (17, 1016, 0), (0, 1016, 0), (12, 1016, 2)):
        with pytest.raises(decoder.GstError) as ei:
            b.set_tuning(*bad)
        assert ei.value.status == decoder.GST_E_ARG
    with pytest.raises(decoder.GstError):
        gpu_ctx.set_option("rans_stage_words", 1004 + 1)
    with pytest.raises(decoder.GstError):
        gpu_ctx.set_option("no_such_option", 1)
    with pytest.raises(decoder.GstError):
        gpu_ctx.set_option("persistent", 2)
    b.set_tuning(0, 0)
    b.close()


def test_load_rgb_matches_oracle(gpu_ctx):
    # LoadRGB(s): assemble_rgb's pixels (codec/assemble.cl:83-129).  The oracle's
    # RGB path is checked on the CPU against a plain four-colour DXT1 decode of
    # its own DXT1 output; here the GPU's RGB output must equal it byte for byte.
    streams = [golden_stream("test1.gst"), golden_stream("synth768x512_s3.gst")] + \
        [workloads.encode_image(w, h, 800 + i).stream for i, (w, h) in enumerate([(1024, 512), (512, 1024)])]
    hdrs, packed = decoder.pack_batch(streams)
    d_cmp = torch.from_numpy(packed).cuda()
    total = sum(h.width * h.height * 3 for h in hdrs)
    d_out = torch.zeros(total, dtype=torch.uint8, device="cuda")
    decoder.load_rgbs(gpu_ctx, hdrs, d_cmp, d_out)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
    out = d_out.cpu().numpy()
    off = 0
    for s, h in zip(streams, hdrs):
        st, ref = oracle.decode_rgb(s, oracle.SCAN_EXACT)
        assert st == 0
        assert np.array_equal(out[off:off + ref.size], ref), (h.width, h.height)
        off += ref.size
    # single-image form, device-resident
    one = torch.zeros(hdrs[0].width * hdrs[0].height * 3, dtype=torch.uint8, device="cuda")
    h0, p0 = decoder.pack_batch(streams[:1])
    decoder.load_rgb(gpu_ctx, h0[0], torch.from_numpy(p0).cuda(), one)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
    assert np.array_equal(one.cpu().numpy(), oracle.decode_rgb(streams[0], oracle.SCAN_EXACT)[1])


@pytest.mark.parametrize("chunks", [1, 3, 8])
def test_load_host_dxts_pipelined(gpu_ctx, chunks):
    # Pinned host layout in, pinned host DXT1 out, chunks overlapped on three
    # streams; twice in a row (the device mirrors are reused).
    imgs = [workloads.encode_image(w, h, 840 + i) for i, (w, h) in
            enumerate([(1024, 512), (512, 512), (2048, 1024), (512, 2048), (1024, 1024)])]
    hdrs, packed = decoder.pack_batch([im.stream for im in imgs])
    want = np.concatenate([im.blocks for im in imgs])
    h_cmp = torch.from_numpy(packed).pin_memory()
    h_out = torch.zeros(sum(h.dxt_bytes for h in hdrs), dtype=torch.uint8).pin_memory()
    s = torch.cuda.Stream()
    for _ in range(2):
        h_out.zero_()
        decoder.load_host_dxts(gpu_ctx, hdrs, h_cmp, h_out, chunks, s)
        s.synchronize()
        assert decoder.sync_status(gpu_ctx, s) == decoder.GST_OK
        assert np.array_equal(h_out.numpy().view(np.uint64), want)


@pytest.mark.parametrize("chunks,persistent", [(1, 0), (3, 0), (5, 1), (6, 0), (4, None)])
def test_batch_host_launch_graph(gpu_ctx, chunks, persistent):
    # gst_batch_host_launch: the pipelined host-to-host decode replayed from a
    # captured graph; repeated calls (outputs cleared in between), a new
    # output buffer and a change of chunk count each give the right blocks.
    imgs = [workloads.encode_image(w, h, 870 + i) for i, (w, h) in
            enumerate([(512, 512), (2048, 1024), (1024, 512), (512, 2048), (1024, 1024), (512, 1024)])]
    hdrs, packed = decoder.pack_batch([im.stream for im in imgs])
    want = np.concatenate([im.blocks for im in imgs])
    rb = decoder.ResidentBatch(gpu_ctx, hdrs)
    if persistent is not None:  # None: untuned, each chunk its size-dependent configuration
        rb.set_tuning(8, 1016, persistent)
    h_cmp = torch.from_numpy(packed).pin_memory()
    outs = [torch.zeros(sum(h.dxt_bytes for h in hdrs), dtype=torch.uint8).pin_memory() for _ in range(2)]
    s = torch.cuda.Stream()
    for it, (k, c) in enumerate([(0, chunks), (0, chunks), (1, chunks), (0, 2)]):
        outs[k].zero_()
        rb.host_launch(h_cmp, outs[k], c, s)
        s.synchronize()
        assert decoder.sync_status(gpu_ctx, s) == decoder.GST_OK
        assert np.array_equal(outs[k].numpy().view(np.uint64), want), it
    rb.close()


def test_persistent_wait_times_out_and_context_survives():
    # Fault injection on the host: the persistent launch leaves out its rANS
    # items, so every tile's bounded wait runs out (1 ms here) and the call
    # reports GST_E_TIMEOUT; the context then decodes normally.
    ctx = decoder.GPUContext(0)
    try:
        im = workloads.encode_image(512, 512, 860)
        hdrs, packed = decoder.pack_batch([im.stream])
        d_cmp = torch.from_numpy(packed).cuda()
        d_out = torch.zeros(hdrs[0].dxt_bytes, dtype=torch.uint8, device="cuda")
        ctx.set_option("persistent", 1)
        ctx.set_option("persistent_wait_us", 1000)
        ctx.set_option("inject_drop_rans", 1)
        decoder.load_compressed_dxts(ctx, hdrs, d_cmp, d_out)
        assert decoder.sync_status(ctx) == decoder.GST_E_TIMEOUT
        ctx.set_option("inject_drop_rans", 0)
        decoder.load_compressed_dxts(ctx, hdrs, d_cmp, d_out)
        assert decoder.sync_status(ctx) == decoder.GST_OK
        assert np.array_equal(d_out.cpu().numpy().view(np.uint64), im.blocks)
    finally:
        ctx.close()


def test_class_tuning_applies_and_stays_bit_exact():
    # A class's configuration is used by the context's calls of that size,
    # invalid values are refused, and every configuration decodes bit-exactly.
    ctx = decoder.GPUContext(0)
    try:
        im = workloads.plain(0)
        hdrs, packed = decoder.pack_batch([im.stream])
        d_cmp = torch.from_numpy(packed).cuda()
        d_out = torch.zeros(hdrs[0].dxt_bytes, dtype=torch.uint8, device="cuda")
        c = decoder.autotune_class(ctx, hdrs, d_cmp, d_out, iterations=2)
        assert c == decoder.size_class(512 * 512 // 16) == 0
        with pytest.raises(decoder.GstError):
            decoder.set_class_tuning(ctx, 0, 12, 1001, 0)
        with pytest.raises(decoder.GstError):
            decoder.set_class_tuning(ctx, 7, 12, 1016, 0)
        for cfg in ((8, 2040, 1), (16, 520, 0), (0, 0, 0)):
            decoder.set_class_tuning(ctx, 0, *cfg)
            d_out.zero_()
            decoder.load_compressed_dxts(ctx, hdrs, d_cmp, d_out)
            assert decoder.sync_status(ctx) == decoder.GST_OK
            assert np.array_equal(d_out.cpu().numpy().view(np.uint64), im.blocks), cfg
        decoder.set_class_tuning(ctx, 0, 8, 2040, 1)
        assert decoder.get_class_tuning(ctx, 0) == (8, 2040, 1)
        ctx.set_profiling(True)
        decoder.load_compressed_dxts(ctx, hdrs, d_cmp, d_out)
        assert [n for n, _ in ctx.kernel_times()] == ["gst_persistent_kernel"]
        ctx.set_profiling(False)
    finally:
        ctx.close()


def test_class_tuning_table_persists(tmp_path, monkeypatch):
    """The per-size-class table as JSON: saved and loaded back, loaded by a new
    context from GST_TUNING_TABLE, rewritten by gst_autotune_class; malformed
    tables and tables of another GPU are refused and change nothing."""
    import json
    path = tmp_path / "tuning.json"
    ctx = decoder.GPUContext(0)
    try:
        decoder.set_class_tuning(ctx, 1, 8, 2040, 0)
        decoder.set_class_tuning(ctx, 4, 12, 1016, 1)
        decoder.save_class_tuning(ctx, path)
        table = json.loads(path.read_text())
        assert table["format"] == "gst_gb300 class tuning" and table["version"] == 1
        assert table["device"] == torch.cuda.get_device_name(0)
        assert [(c["class"], c["blocks_per_sm"], c["stage_words"], c["persistent"]) for c in table["classes"]] == \
            [(1, 8, 2040, 0), (4, 12, 1016, 1)]
        decoder.set_class_tuning(ctx, 1, 0, 0, 0)
        decoder.set_class_tuning(ctx, 4, 0, 0, 0)
        decoder.load_class_tuning(ctx, path)
        assert decoder.get_class_tuning(ctx, 1) == (8, 2040, 0) and decoder.get_class_tuning(ctx, 4) == (12, 1016, 1)
        before = [decoder.get_class_tuning(ctx, c) for c in range(7)]
        bad = dict(table, classes=[dict(table["classes"][0], stage_words=1001)])
        for text, status in ((json.dumps(bad), decoder.GST_E_FORMAT), ("{}", decoder.GST_E_FORMAT),
                             (json.dumps(dict(table, device="some other GPU")), decoder.GST_E_ARG)):
            (tmp_path / "bad.json").write_text(text)
            with pytest.raises(decoder.GstError) as ei:
                decoder.load_class_tuning(ctx, tmp_path / "bad.json")
            assert ei.value.status == status
        assert [decoder.get_class_tuning(ctx, c) for c in range(7)] == before
    finally:
        ctx.close()
    # A new context loads the named table; autotuning a class rewrites it.
    monkeypatch.setenv("GST_TUNING_TABLE", str(path))
    ctx = decoder.GPUContext(0)
    try:
        assert decoder.get_class_tuning(ctx, 1) == (8, 2040, 0)
        im = workloads.plain(0)
        hdrs, packed = decoder.pack_batch([im.stream])
        d_cmp = torch.from_numpy(packed).cuda()
        d_out = torch.zeros(hdrs[0].dxt_bytes, dtype=torch.uint8, device="cuda")
        c = decoder.autotune_class(ctx, hdrs, d_cmp, d_out, iterations=1)
        classes = {e["class"]: e for e in json.loads(path.read_text())["classes"]}
        assert set(classes) == {0, 1, 4}
        assert (classes[0]["blocks_per_sm"], classes[0]["stage_words"], classes[0]["persistent"]) == \
            decoder.get_class_tuning(ctx, c)
    finally:
        ctx.close()
