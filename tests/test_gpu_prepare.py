"""CUDA endpoint stages of the encoder (gst_prepare_symbols, gst_compress_dxt)
vs the reference's sections and the oracle, through the C ABI.  Byte-exact.

* the Y and chroma sections (RGB565 -> YCoCg667 -> five-level forward 5/3
  wavelet -> bytes) that the reference encoder wrote into its own streams are
  rebuilt from the blocks those streams decode to;
* every section of the 64-image batch (one launch) and of the 8192x8192
  texture equals the oracle's restatement, palette and index deltas included;
* DXT1 blocks -> GST stream on the GPU -> GPU decode gives the blocks back."""
import numpy as np
import pytest

import oracle
from conftest import as_blocks, golden_stream
from gst_gb300 import decoder, entropy, workloads

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def prepare(ctx, images):
    """images: [(w, h, blocks u64)] -> per image (y, chroma, palette, deltas) from one launch."""
    bufs, descs = [], []
    for w, h, blocks in images:
        B = w * h // 16
        t = {"b": torch.from_numpy(np.ascontiguousarray(blocks, np.uint64).view(np.int64).copy()).cuda(),
             "y": torch.zeros(2 * B, dtype=torch.uint8, device="cuda"),
             "c": torch.zeros(4 * B, dtype=torch.uint8, device="cuda"),
             "p": torch.full((entropy.palette_capacity(w, h),), 7, dtype=torch.uint8, device="cuda"),
             "i": torch.zeros(B, dtype=torch.uint8, device="cuda")}
        bufs.append(t)
        descs.append((w, h, t["b"], t["y"], t["c"], t["p"], t["i"]))
    pal = torch.zeros(len(images), dtype=torch.int32, device="cuda")
    entropy.prepare_symbols(ctx, descs, pal)
    assert decoder.sync_status(ctx) == decoder.GST_OK
    pb = pal.cpu().numpy()
    return [(t["y"].cpu().numpy(), t["c"].cpu().numpy(), t["p"].cpu().numpy()[: int(pb[k])], t["i"].cpu().numpy())
            for k, t in enumerate(bufs)]


def oracle_sections(w, h, blocks):
    y, c, _ = oracle.endpoint_planes(w, h, blocks)
    p, d = oracle.run_palette(w, h, blocks)
    return y, c, p, d


@pytest.mark.parametrize("name", ["test1.gst", "synth512_s0.gst", "synth768x512_s3.gst"])
def test_planes_rebuild_reference_sections(gpu_ctx, name):
    s = golden_stream(name)
    w, h = (int.from_bytes(s[i:i + 4], "little") for i in (0, 4))
    st, dxt = oracle.decode(s, oracle.SCAN_EXACT)
    st2, sym = oracle.decode_symbols(s)
    assert st == 0 and st2 == 0
    blocks = as_blocks(dxt)
    ((y, c, p, d),) = prepare(gpu_ctx, [(w, h, blocks)])
    B = w * h // 16
    assert np.array_equal(y, sym[:2 * B]) and np.array_equal(c, sym[2 * B:6 * B])
    _, _, p2, d2 = oracle_sections(w, h, blocks)
    assert np.array_equal(p, p2) and np.array_equal(d, d2)


def test_batch_of_64_matches_oracle(gpu_ctx):
    imgs = workloads.batched(64)
    got = prepare(gpu_ctx, [(im.width, im.height, im.blocks) for im in imgs])
    for im, g in zip(imgs, got):
        for a, b in zip(g, oracle_sections(im.width, im.height, im.blocks)):
            assert np.array_equal(a, b), (im.width, im.height)


def test_large_8192_matches_oracle_and_round_trips(gpu_ctx):
    im = workloads.large()
    ((y, c, p, d),) = prepare(gpu_ctx, [(im.width, im.height, im.blocks)])
    for a, b in zip((y, c, p, d), oracle_sections(im.width, im.height, im.blocks)):
        assert np.array_equal(a, b)
    s = entropy.compress_dxt(gpu_ctx, im.width, im.height, im.blocks)
    assert np.array_equal(as_blocks(decoder.decompress_dxt(gpu_ctx, s)), im.blocks)


@pytest.mark.parametrize("dims", [(512, 512), (1024, 2048), (4096, 1024)])
def test_compress_dxt_round_trip_and_matches_oracle_stream(gpu_ctx, dims):
    w, h = dims
    im = workloads.encode_image(w, h, 300 + w // 512, 0.1)
    s = entropy.compress_dxt(gpu_ctx, w, h, im.blocks)
    y, c, p, d = oracle_sections(w, h, im.blocks)
    st, want = oracle.encode_stream(w, h, p.size, y, c, p, d)
    assert st == 0 and s == want
    assert np.array_equal(as_blocks(decoder.decompress_dxt(gpu_ctx, s)), im.blocks)


def test_argument_checks(gpu_ctx):
    w, h = 512, 512
    B = w * h // 16
    blocks = torch.zeros(B, dtype=torch.int64, device="cuda")
    y = torch.zeros(2 * B + 16, dtype=torch.uint8, device="cuda")
    c = torch.zeros(4 * B, dtype=torch.uint8, device="cuda")
    p = torch.zeros(entropy.palette_capacity(w, h), dtype=torch.uint8, device="cuda")
    i = torch.zeros(B, dtype=torch.uint8, device="cuda")
    pal = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(decoder.GstError):  # misaligned Y section
        entropy.prepare_symbols(gpu_ctx, [(w, h, blocks, y[1:], c, p, i)], pal)
    with pytest.raises(decoder.GstError):  # a size the format rejects
        entropy.prepare_symbols(gpu_ctx, [(500, 512, blocks, y, c, p, i)], pal)
    assert entropy.palette_capacity(500, 512) == 0
    entropy.prepare_symbols(gpu_ctx, [(w, h, blocks, y, c, p, i)], pal)
    assert decoder.sync_status(gpu_ctx) == decoder.GST_OK
    assert int(pal.cpu()[0]) == 8192  # all-zero blocks: one palette word
