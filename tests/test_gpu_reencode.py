"""CUDA index palette search (gst_reencode_blocks, gst_compress_rgb_dxt) vs
the reference's DXTImage::Reencode and CompressDXT, through the C ABI.
Byte-exact.

* every case of tests/golden/reencode.json (made by the reference itself):
  blocks after the search, palette words and their zero padding, index
  deltas, one image per call and all images in one call;
* the reference's whole stream of a 512x256 image (stb_dxt blocks -> Reencode
  -> CompressDXT) rebuilt by gst_compress_rgb_dxt;
* larger images and a mixed batch against the C oracle's restatement, and a
  whole stream against the oracle's stages."""
import hashlib
import json
import sys

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from gst_gb300 import decoder, encoder, entropy

sys.path.insert(0, str(GOLDEN))
from reencode_inputs import make_rgb, unpack  # noqa: E402

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def fixture():
    return json.loads((GOLDEN / "reencode.json").read_text())["cases"]


def reencode(ctx, images):
    """images: [(w, h, rgb (h, w, 3) u8, blocks u64)] -> per image (blocks_out,
    padded palette, deltas) from one gst_reencode_blocks call."""
    bufs, descs = [], []
    for w, h, rgb, blocks in images:
        B = w * h // 16
        cap = (4 * B + 8191) // 8192 * 8192
        t = {"rgb": torch.from_numpy(np.ascontiguousarray(rgb, np.uint8).reshape(-1)).cuda(),
             "b": torch.from_numpy(np.ascontiguousarray(blocks, np.uint64).view(np.int64).copy()).cuda(),
             "o": torch.zeros(B, dtype=torch.int64, device="cuda"),
             "p": torch.full((cap,), 7, dtype=torch.uint8, device="cuda"),
             "d": torch.zeros(B, dtype=torch.uint8, device="cuda")}
        bufs.append(t)
        descs.append([w, h, t["rgb"], t["b"], t["o"], t["p"], t["d"]])
    pal = torch.zeros(len(images), dtype=torch.int32, device="cuda")
    for k, dsc in enumerate(descs):
        dsc.append(pal[k:k + 1])
    entropy.reencode_blocks(ctx, [tuple(x) for x in descs])
    assert decoder.sync_status(ctx) == decoder.GST_OK
    pb = pal.cpu().numpy()
    return [(t["o"].cpu().numpy().view(np.uint64), t["p"].cpu().numpy()[: int(pb[k])], t["d"].cpu().numpy())
            for k, t in enumerate(bufs)]


def check(got, want_b, want_p, want_d, name):
    b, p, d = got
    assert np.array_equal(b, want_b), name
    assert p.size == (want_p.size + 8191) // 8192 * 8192, name
    assert np.array_equal(p[: want_p.size], want_p) and not p[want_p.size:].any(), name
    assert np.array_equal(d, want_d), name


def case_inputs(c):
    return c["width"], c["height"], make_rgb(c), unpack(c["blocks_in"], np.uint64)


def test_each_reference_case(gpu_ctx, fixture):
    for c in fixture:
        (got,) = reencode(gpu_ctx, [case_inputs(c)])
        check(got, unpack(c["blocks_out"], np.uint64), unpack(c["palette"], np.uint8),
              unpack(c["deltas"], np.uint8), c["name"])


def test_all_reference_cases_in_one_call(gpu_ctx, fixture):
    outs = reencode(gpu_ctx, [case_inputs(c) for c in fixture])
    for c, got in zip(fixture, outs):
        check(got, unpack(c["blocks_out"], np.uint64), unpack(c["palette"], np.uint8),
              unpack(c["deltas"], np.uint8), c["name"])


def test_reference_stream_rebuilt(gpu_ctx, fixture):
    for c in fixture:
        if "stream_sha256" not in c:
            continue
        w, h, rgb, blocks = case_inputs(c)
        s = entropy.compress_rgb_dxt(gpu_ctx, w, h, rgb, blocks)
        assert len(s) == c["stream_len"] and hashlib.sha256(s).hexdigest() == c["stream_sha256"], c["name"]


@pytest.mark.parametrize("w,h,seed,checker", [(1024, 1024, 21, 0.0), (768, 512, 22, 0.3), (2048, 256, 23, 0.05)])
def test_large_images_vs_oracle(gpu_ctx, w, h, seed, checker):
    rgb = encoder.synth_image(w, h, seed, checker)
    blocks = encoder.compress_blocks(rgb)
    (got,) = reencode(gpu_ctx, [(w, h, rgb, blocks)])
    ob, op, od = oracle.reencode(w, h, rgb, blocks)
    n = int(np.count_nonzero(op.reshape(-1, 4).any(axis=1))) if op.size else 0
    b, p, d = got
    assert np.array_equal(b, ob) and np.array_equal(p, op) and np.array_equal(d, od)
    assert n > 0


def test_mixed_batch_vs_oracle(gpu_ctx):
    dims = [(256, 256), (64, 1024), (512, 128), (128, 128), (1024, 64), (32, 32)]
    images = []
    for k, (w, h) in enumerate(dims):
        rgb = encoder.synth_image(w, h, 40 + k, 0.1 * (k % 3))
        images.append((w, h, rgb, encoder.compress_blocks(rgb)))
    for (w, h, rgb, blocks), got in zip(images, reencode(gpu_ctx, images)):
        ob, op, od = oracle.reencode(w, h, rgb, blocks)
        check(got, ob, op, od, f"{w}x{h}")


def test_stream_vs_oracle_stages(gpu_ctx):
    w, h = 1024, 512
    rgb = encoder.synth_image(w, h, 31, 0.1)
    blocks = encoder.compress_blocks(rgb)
    s = entropy.compress_rgb_dxt(gpu_ctx, w, h, rgb, blocks)
    ob, op, od = oracle.reencode(w, h, rgb, blocks)
    y, c, _ = oracle.endpoint_planes(w, h, ob)
    st, want = oracle.encode_stream(w, h, op.size, y, c, op, od)
    assert st == 0 and s == want


def test_bad_arguments(gpu_ctx):
    w, h = 64, 64
    rgb = np.zeros((h, w, 3), np.uint8)
    blocks = np.zeros(w * h // 16, np.uint64)
    with pytest.raises(Exception):
        reencode(gpu_ctx, [(62, 64, np.zeros((64, 62, 3), np.uint8), np.zeros(15 * 16, np.uint64))])
    with pytest.raises(Exception):  # rgb and blocks must match the size
        entropy.compress_rgb_dxt(gpu_ctx, 512, 256, rgb, blocks)
    # the context still works
    (got,) = reencode(gpu_ctx, [(w, h, rgb, blocks)])
    assert got[2][0] == 128
