"""Encodes the benchmark workloads with the reference encoder itself.

Runs only where the reference sources are mounted: oracle/build_ref.sh builds
the reference's CPU encoder, and oracle/ref_harness.cpp's gstref_compress_rgb
runs the path of its ``gentenc`` tool on an RGB8 image
(codec/command_line.cpp:9-26 -> GenTC::CompressDXT(orig_fn)): the
``DXTImage`` constructor compresses every 4x4 block with stb_dxt in its
high-quality mode (CompressRGB, codec/dxt_image.cpp:362-385), searches the
index palette (DXTImage::Reencode, codec/dxt_image.cpp:510-624), and
CompressDXTImage writes the GST stream (codec/encoder.cpp:39-180).  Only the
file read is left out: the images come from this project's seeded generator
(gst_gb300.encoder.synth_image), so nothing on disk stands between the pixels
and the encoder.

Outputs, under ``ref_streams/`` beside this script (read at bench and test
time; the reference is not needed there):

* ``b{i}_{w}x{h}_s{seed}.gst`` -- the 64 batched images (w, h drawn
  independently from {512, 1024, 2048}, seeds 1000 + i);
* ``large_8192x8192_s8192_c100.gst`` -- the 8192x8192 texture with 10 % of its
  area replaced by 1-8 px checker regions;
* ``serve_{w}x{h}_s{seed}.gst`` -- serving-pool images, so that every (w, h)
  class with w, h in {512, 1024, 2048, 4096} holds at least four streams
  (classes up to 2048 also draw on the batched images);
* ``manifest.json`` -- per stream: size, seed, checker fraction, SHA-256 of the
  stream, of the encoder's own DXT1 blocks (``DXTImage::PhysicalBlocks``) and
  of the blocks the stream decodes to under the reference decoder's
  arithmetic (the oracle's restatement, pinned elsewhere against the
  reference); they differ only where a wavelet coefficient wrapped in the
  reference encoder's 8-bit planes.

The 512x512 plain image is ``synth512_s0.gst`` beside this script
(make_golden.py).  The rANS-only section (2^26 Laplace bytes) is not stored
(43 MB): the manifest keeps the SHA-256 of the reference's
ByteEncoder::EncodeBytes output for it (codec/entropy.cpp:174-265), which the
stream producer in gst_gb300 must reproduce.

Usage: python tests/golden/make_ref_streams.py [--jobs N]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
OUT = HERE / "ref_streams"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

BATCH_DIMS = (512, 1024, 2048)
SERVING_DIMS = (512, 1024, 2048, 4096)
SERVE_PER_CLASS = 4


def sha(b) -> str:
    return hashlib.sha256(bytes(b)).hexdigest()


def batched_dims(n: int = 64, seed: int = 1000) -> list[tuple[int, int]]:
    # the same draw as gst_gb300.workloads.batched_dims
    rng = np.random.default_rng(seed)
    return [(int(rng.choice(BATCH_DIMS)), int(rng.choice(BATCH_DIMS))) for _ in range(n)]


def jobs() -> list[dict]:
    out = []
    dims = batched_dims()
    for i, (w, h) in enumerate(dims):
        out.append({"name": f"b{i:02d}_{w}x{h}_s{1000 + i}.gst", "kind": "batched", "width": w, "height": h,
                    "seed": 1000 + i, "checker_frac": 0.0})
    out.append({"name": "large_8192x8192_s8192_c100.gst", "kind": "large", "width": 8192, "height": 8192,
                "seed": 8192, "checker_frac": 0.10})
    have = {}
    for w, h in dims:
        have[(w, h)] = have.get((w, h), 0) + 1
    for ci, w in enumerate(SERVING_DIMS):
        for cj, h in enumerate(SERVING_DIMS):
            for k in range(max(0, SERVE_PER_CLASS - have.get((w, h), 0))):
                seed = 6000 + 16 * (4 * ci + cj) + k
                out.append({"name": f"serve_{w}x{h}_s{seed}.gst", "kind": "serving", "width": w, "height": h,
                            "seed": seed, "checker_frac": 0.0})
    return out


def encode_one(job: dict) -> dict:
    # The reference encoder prints progress on stdout: send it to /dev/null.
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    import oracle
    from gst_gb300 import encoder
    from make_golden import ref_compress_rgb
    ref = oracle.load_ref()
    t0 = time.time()
    rgb = encoder.synth_image(job["width"], job["height"], job["seed"], job["checker_frac"])
    stream, blocks = ref_compress_rgb(ref, rgb)
    st, dec = oracle.decode(stream, oracle.SCAN_EXACT)
    assert st == 0, f"{job['name']}: the oracle rejects the reference encoder's stream ({st})"
    mism = int(np.count_nonzero(np.frombuffer(dec.tobytes(), np.uint64) != np.frombuffer(blocks, np.uint64)))
    (OUT / job["name"]).write_bytes(stream)
    return {**job, "gst_bytes": len(stream), "stream_sha256": sha(stream), "encoder_blocks_sha256": sha(blocks),
            "decoded_sha256": sha(dec), "blocks_differing_from_encoder": mism,
            "encode_seconds": round(time.time() - t0, 2)}


def rans_digest() -> dict:
    import ctypes

    import oracle
    from gst_gb300.workloads import laplace_bytes
    sym = laplace_bytes(1 << 26, 6.0, 7)
    cap = sym.size + (1 << 22)
    buf = (ctypes.c_uint8 * cap)()
    n = ctypes.c_size_t()
    assert oracle.load_ref().gstref_encode_bytes(sym.ctypes.data, sym.size, buf, cap, ctypes.byref(n)) == 0
    sec = bytes(buf[: n.value])
    return {"symbols": int(sym.size), "laplace_b": 6.0, "seed": 7, "section_bytes": len(sec),
            "section_sha256": sha(sec), "encoder": "reference ByteEncoder::EncodeBytes (codec/entropy.cpp:174-265)"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    import oracle
    if not oracle.build_ref():
        raise SystemExit("reference sources not available; cannot regenerate the streams")
    OUT.mkdir(exist_ok=True)
    todo = jobs()
    # the largest first, so that the pool's tail is short
    todo.sort(key=lambda j: -j["width"] * j["height"])
    ctx = mp.get_context("spawn")
    t0 = time.time()
    with ctx.Pool(args.jobs) as pool:
        done = pool.map(encode_one, todo, chunksize=1)
    done.sort(key=lambda j: ({"batched": 0, "large": 1, "serving": 2}[j["kind"]], j["name"]))
    manifest = {
        "encoder": "reference gentenc path: DXTImage(w, h, rgb) [stb_dxt HIGHQUAL + Reencode] + CompressDXT, "
                   "via oracle/ref_harness.cpp gstref_compress_rgb",
        "generator": "gst_gb300.encoder.synth_image(w, h, seed, checker_frac)",
        "streams": done,
        "plain": {"name": "synth512_s0.gst", "dir": "tests/golden", "width": 512, "height": 512, "seed": 0},
        "rans_2pow26": rans_digest(),
    }
    (OUT / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")
    total = sum(j["gst_bytes"] for j in done)
    print(f"{len(done)} streams, {total / 1e6:.1f} MB, {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
