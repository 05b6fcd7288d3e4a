"""CUDA encoder stages vs the oracle and the reference's own outputs, through
the C ABI (include/gst_encode.h).  Byte-exact everywhere.

* frequency normalisation (ans::GenerateHistogram at M = 2048): the
  reference's known answers and tie / wrap cases, plus seeded count vectors
  against the oracle's heap replay;
* ByteEncoder sections: the reference's digests, and seeded sections of every
  kind and size against the oracle, many sections per launch;
* whole GST streams: the reference encoder's streams rebuilt from their
  decoded symbols; the 64-image batch and the 8192x8192 texture re-encoded to
  their own streams; GPU encode -> GPU decode gives back the symbols."""
import hashlib
import sys

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, golden_stream
from gst_gb300 import decoder, entropy, workloads

sys.path.insert(0, str(GOLDEN))
from make_golden import HISTOGRAM_KINDS, histogram_input, section_input  # noqa: E402

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHA = lambda b: hashlib.sha256(bytes(b)).hexdigest()  # noqa: E731


def dev(a: np.ndarray) -> "torch.Tensor":
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint8).copy()).cuda()


def encode_sections(ctx, xs):
    """Encodes every array of xs in one launch -> list of section bytes."""
    secs = [dev(x) for x in xs]
    cap = sum(entropy.section_bound(x.size) for x in xs)
    out = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    offs = torch.zeros(len(xs) + 1, dtype=torch.int64, device="cuda")
    entropy.encode_bytes(ctx, secs, out, offs)
    assert decoder.sync_status(ctx) == decoder.GST_OK
    o = offs.cpu().numpy()
    host = out[: int(o[-1])].cpu().numpy().tobytes()
    return [host[o[i]:o[i + 1]] for i in range(len(xs))]


def stream_symbols(stream: bytes):
    w, h, pal = (int.from_bytes(stream[i:i + 4], "little") for i in (0, 4, 8))
    st, sym = oracle.decode_symbols(stream, nthreads=8)
    assert st == 0
    return w, h, pal, sym


def encode_streams(ctx, streams):
    """Re-encodes each stream's symbols on the GPU, all in one launch."""
    bufs, imgs = [], []
    for s in streams:
        w, h, pal, sym = stream_symbols(s)
        d = dev(sym)
        bufs.append(d)
        imgs.append(entropy.stream_symbols(w, h, pal, d))
    cap = sum(entropy.stream_bound(im.width, im.height, im.palette_bytes) for im in imgs)
    out = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    offs = torch.zeros(len(imgs) + 1, dtype=torch.int64, device="cuda")
    entropy.encode_streams(ctx, imgs, out, offs)
    assert decoder.sync_status(ctx) == decoder.GST_OK
    o = offs.cpu().numpy()
    host = out[: int(o[-1])].cpu().numpy().tobytes()
    return [host[o[i]:o[i + 1]] for i in range(len(imgs))]


def test_normalize_known_answers_and_stress(gpu_ctx, golden):
    for c in golden["tables"]:
        assert entropy.normalize_frequencies(gpu_ctx, c["F"]).tolist() == c["normalized"]
    for c in golden["histograms"]:
        if c["M"] == 2048:
            assert entropy.normalize_frequencies(gpu_ctx, c["counts"]).tolist() == c["expected"]
    n = 0
    for c in golden["histogram_stress"]:
        if c["M"] != 2048:
            continue
        counts = histogram_input(c["seed"], c["kind"])
        assert entropy.normalize_frequencies(gpu_ctx, counts).tolist() == c["expected"], (c["seed"], c["kind"])
        n += 1
    assert n >= 20


def test_normalize_matches_oracle_on_seeded_counts(gpu_ctx):
    # Tie-heavy, wrapped and long-correction vectors: every path of the kernel
    # (galloping rounds, whole tie groups, the heap replay) against the oracle.
    rng = np.random.default_rng(2024)
    for t in range(600):
        counts = histogram_input(int(rng.integers(1 << 30)), HISTOGRAM_KINDS[t % len(HISTOGRAM_KINDS)])
        st, want = oracle.normalize(counts, 2048)
        assert st == 0
        got = entropy.normalize_frequencies(gpu_ctx, counts)
        assert np.array_equal(got, want), (t, counts.tolist())


def test_normalize_rejects_all_zero(gpu_ctx):
    with pytest.raises(decoder.GstError):
        entropy.normalize_frequencies(gpu_ctx, [0, 0, 0])


def test_sections_match_reference_digests_in_one_launch(gpu_ctx, golden):
    cases = golden["sections"]
    xs = [section_input(c["seed"], c["kind"], c["n_groups"]) for c in cases]
    for c, sec in zip(cases, encode_sections(gpu_ctx, xs)):
        assert len(sec) == c["bytes"] and SHA(sec) == c["sha256"], c["kind"]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_sections_match_oracle(gpu_ctx, seed):
    rng = np.random.default_rng(seed)
    kinds = ("laplace1", "laplace6", "laplace20", "uniform", "two_symbols", "seven_symbols", "rare_tail",
             "one_symbol", "skewed", "wrap255", "rare_group")
    xs = []
    for k, kind in enumerate(kinds):
        g = int(rng.integers(1, 40)) if kind != "rare_group" else 4
        xs.append(section_input(int(rng.integers(1 << 30)), kind, g))
    got = encode_sections(gpu_ctx, xs)
    for x, sec in zip(xs, got):
        st, want = oracle.encode_section(x)
        assert st == 0 and sec == want


def test_only_byte_zero_section(gpu_ctx):
    x = np.zeros(8192 * 3, np.uint8)
    (sec,) = encode_sections(gpu_ctx, [x])
    st, want = oracle.encode_section(x)
    assert st == 0 and sec == want


def test_large_wrapped_section(gpu_ctx):
    # 2^23 symbols, one byte above 2^21 times: counts * 2048 wraps in uint32
    # and the frequency correction is long.
    rng = np.random.default_rng(9)
    x = (np.rint(rng.laplace(0, 1, 1 << 23)).astype(np.int64) % 256).astype(np.uint8)
    counts = np.bincount(x, minlength=256)
    assert counts.max() >= (1 << 21)
    (sec,) = encode_sections(gpu_ctx, [x])
    st, want = oracle.encode_section(x)
    assert st == 0 and sec == want


@pytest.mark.parametrize("name", ["test1.gst", "synth512_s0.gst", "synth768x512_s3.gst"])
def test_streams_rebuild_reference_streams(gpu_ctx, name):
    s = golden_stream(name)
    (again,) = encode_streams(gpu_ctx, [s])
    assert again == s


def test_batch_of_64_streams_in_one_launch(gpu_ctx):
    streams = [im.stream for im in workloads.batched(64)]
    assert encode_streams(gpu_ctx, streams) == streams


def test_large_8192_stream(gpu_ctx):
    s = workloads.large().stream
    (again,) = encode_streams(gpu_ctx, [s])
    assert again == s


def test_compress_symbols_host_to_host(gpu_ctx):
    s = golden_stream("synth512_s0.gst")
    w, h, pal, sym = stream_symbols(s)
    assert entropy.compress_symbols(gpu_ctx, w, h, pal, sym) == s


def test_gpu_encode_then_gpu_decode(gpu_ctx):
    x = section_input(77, "laplace6", 96)
    (sec,) = encode_sections(gpu_ctx, [x])
    d_f = dev(np.frombuffer(sec[:512], np.uint8))
    d_b = dev(np.frombuffer(sec[512:], np.uint8))
    d_o = torch.zeros(x.size, dtype=torch.uint8, device="cuda")
    decoder.decode_rans_groups(gpu_ctx, d_f, d_b, len(sec) - 512, x.size // 8192, 32, d_o)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
    assert np.array_equal(d_o.cpu().numpy(), x)


def test_argument_checks(gpu_ctx):
    good = dev(section_input(5, "laplace6", 1))
    out = torch.zeros(entropy.section_bound(8192), dtype=torch.uint8, device="cuda")
    offs = torch.zeros(2, dtype=torch.int64, device="cuda")
    with pytest.raises(decoder.GstError):  # not a multiple of 8192
        entropy.encode_bytes(gpu_ctx, [good[:4096]], out, offs)
    with pytest.raises(decoder.GstError):  # misaligned symbols
        entropy.encode_bytes(gpu_ctx, [torch.zeros(8192 + 16, dtype=torch.uint8, device="cuda")[1:8193]], out, offs)
    with pytest.raises(decoder.GstError):  # output below the bound
        entropy.encode_bytes(gpu_ctx, [good], out[:1000], offs)
    assert entropy.section_bound(8191) == 0
    assert entropy.stream_bound(500, 512, 8192) == 0
    entropy.encode_bytes(gpu_ctx, [good], out, offs)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK


def test_lookback_wait_times_out_and_context_survives():
    # Fault injection on the host: group 1 never publishes its size, so every
    # later group's bounded look-back wait (1 ms here) runs out; the call
    # reports GST_E_TIMEOUT and the context then encodes normally.
    ctx = decoder.GPUContext(0)
    try:
        x = section_input(61, "laplace6", 8)
        ctx.set_option("persistent_wait_us", 1000)
        ctx.set_option("inject_encode_stall", 1)
        encode = lambda: encode_sections_raw(ctx, [x])  # noqa: E731
        encode()
        assert decoder.sync_status(ctx) == decoder.GST_E_TIMEOUT
        ctx.set_option("inject_encode_stall", 0)
        secs = encode()
        assert decoder.sync_status(ctx) == decoder.GST_OK
        st, want = oracle.encode_section(x)
        assert st == 0 and secs[0] == want
    finally:
        ctx.close()


def encode_sections_raw(ctx, xs):
    """encode_sections without the status check (the caller reads it)."""
    secs = [dev(x) for x in xs]
    cap = sum(entropy.section_bound(x.size) for x in xs)
    out = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    offs = torch.zeros(len(xs) + 1, dtype=torch.int64, device="cuda")
    entropy.encode_bytes(ctx, secs, out, offs)
    torch.cuda.synchronize()
    o = offs.cpu().numpy()
    host = out[: int(o[-1])].cpu().numpy().tobytes() if o[-1] > 0 else b""
    return [host[o[i]:o[i + 1]] for i in range(len(xs))]
