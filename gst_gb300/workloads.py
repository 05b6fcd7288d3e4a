"""Seeded synthetic inputs for the five decode workloads.

No public dataset exists for this path (the reference's photo set is not
available), so every workload is made here from a seed:

* ``plain``   -- one 512x512 image, seed 0, 16,384 DXT1 blocks.
* ``rans``    -- 2^26 bytes of a discretised Laplace(0, b=6), folded into 256
                 symbols, in one section of 8192 groups (32 streams x 256).
* ``batched`` -- 64 images, width and height drawn independently from
                 {512, 1024, 2048}, seeds 1000 + i.
* ``large``   -- one 8192x8192 image with about 10 % of its area replaced by
                 1-8 px two-colour checker regions, seed 8192.
* ``serving`` -- a pool of images per (w, h) class, w and h from
                 {512, 1024, 2048, 4096} with weights 0.4/0.3/0.2/0.1.

Two producers make the streams:

* the reference encoder itself (its ``gentenc`` path: stb_dxt high-quality
  blocks, the Reencode index palette search, CompressDXT), run ahead of time by
  tests/golden/make_ref_streams.py on the same seeded images; the streams and
  SHA-256 digests of the blocks they decode to are committed under
  tests/golden/ref_streams/ (``ref_*`` functions below).  These are the
  benchmark inputs.
* this project's CPU stream producer (csrc/gst_encoder.cpp), which runs
  anywhere: its own DXT1 compressor and a palette search that keeps each
  block's endpoints, so its streams are about half the size of the
  reference's.  Tests that need streams of other sizes or seeds use it, and
  the bench reports it as a labelled secondary input.  Its streams are cached
  under gst_gb300/_cache/ (git-ignored) keyed by the encoder sources.

A fixture image carries no decoded blocks (``blocks`` is None): the checker
that compares a decode against them computes them and checks them against
``decoded_sha256``.
"""
from __future__ import annotations

import hashlib
import json
import os
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import encoder
from .build import ENCODER_SOURCES, ENCODER_HEADERS

CACHE = Path(__file__).resolve().parent / "_cache"
REF_STREAMS = Path(__file__).resolve().parent.parent / "tests" / "golden" / "ref_streams"
REF_PLAIN = Path(__file__).resolve().parent.parent / "tests" / "golden" / "synth512_s0.gst"

BATCH_DIMS = (512, 1024, 2048)
SERVING_DIMS = (512, 1024, 2048, 4096)
SERVING_WEIGHTS = (0.4, 0.3, 0.2, 0.1)


@dataclass
class EncodedImage:
    width: int
    height: int
    seed: int
    stream: bytes
    blocks: np.ndarray | None  # uint64 per DXT1 block: what a correct decode must return
    clips: int = 0      # wavelet coefficients that wrapped (their tiles are lossy)
    encoder: str = "gst_gb300 stream producer"
    decoded_sha256: str | None = None  # reference-encoded fixtures: digest of the decoded blocks

    @property
    def pixels(self) -> int:
        return self.width * self.height


def _encoder_tag() -> str:
    h = hashlib.sha256()
    for p in list(ENCODER_SOURCES) + list(ENCODER_HEADERS):
        h.update(Path(p).read_bytes())
    return h.hexdigest()[:12]


def encode_image(w: int, h: int, seed: int, checker_frac: float = 0.0, cache: bool = True,
                 nthreads: int = 0) -> EncodedImage:
    key = f"{w}x{h}_s{seed}_c{int(round(checker_frac * 1000))}_{_encoder_tag()}"
    sp, bp = CACHE / f"{key}.gst", CACHE / f"{key}.blk"
    if cache and sp.exists() and bp.exists():
        return EncodedImage(w, h, seed, sp.read_bytes(), np.fromfile(bp, dtype=np.uint64))
    rgb = encoder.synth_image(w, h, seed, checker_frac)
    stream, blocks, clips = encoder.encode_rgb(rgb, nthreads=nthreads)
    if cache:
        CACHE.mkdir(exist_ok=True)
        tmp = sp.with_suffix(f".tmp{os.getpid()}")
        tmp.write_bytes(stream)
        tmp.replace(sp)
        tmpb = bp.with_suffix(f".tmp{os.getpid()}")
        blocks.tofile(tmpb)
        tmpb.replace(bp)
    return EncodedImage(w, h, seed, stream, blocks, clips)


def plain(seed: int = 0) -> EncodedImage:
    return encode_image(512, 512, seed)


def batched_dims(n: int = 64, seed: int = 1000) -> list[tuple[int, int]]:
    rng = np.random.default_rng(seed)
    return [(int(rng.choice(BATCH_DIMS)), int(rng.choice(BATCH_DIMS))) for _ in range(n)]


def batched(n: int = 64, seed: int = 1000) -> list[EncodedImage]:
    dims = batched_dims(n, seed)
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        futs = [ex.submit(encode_image, w, h, seed + i, 0.0, True, 2) for i, (w, h) in enumerate(dims)]
        return [f.result() for f in futs]


def large(size: int = 8192, seed: int = 8192, checker_frac: float = 0.10) -> EncodedImage:
    return encode_image(size, size, seed, checker_frac)


def serving_pool(per_class: int = 4, seed: int = 5000) -> dict[tuple[int, int], list[EncodedImage]]:
    pool = {}
    jobs = []
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        for w in SERVING_DIMS:
            for h in SERVING_DIMS:
                for k in range(per_class):
                    jobs.append(((w, h), ex.submit(encode_image, w, h, seed + 97 * len(jobs), 0.0, True, 2)))
        for key, f in jobs:
            pool.setdefault(key, []).append(f.result())
    return pool


@dataclass
class RansSection:
    symbols: np.ndarray  # the decoded bytes a correct decode returns
    section: bytes       # 512-byte frequency table + body

    @property
    def n_groups(self) -> int:
        return self.symbols.size // 8192


def laplace_bytes(n: int, b: float = 6.0, seed: int = 7) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return (np.rint(rng.laplace(0.0, b, n)).astype(np.int64) % 256).astype(np.uint8)


def rans_section(n: int = 1 << 26, b: float = 6.0, seed: int = 7) -> RansSection:
    key = f"rans_{n}_b{b}_s{seed}_{_encoder_tag()}"
    sp = CACHE / f"{key}.sec"
    sym = laplace_bytes(n, b, seed)
    if sp.exists():
        return RansSection(sym, sp.read_bytes())
    sec = encoder.encode_section(sym)
    CACHE.mkdir(exist_ok=True)
    tmp = sp.with_suffix(f".tmp{os.getpid()}")
    tmp.write_bytes(sec)
    tmp.replace(sp)
    return RansSection(sym, sec)


# ---------------------------------------------------------------------------
# Streams made by the reference encoder (tests/golden/make_ref_streams.py).
REF_ENCODER = "reference gentenc (stb_dxt HIGHQUAL + Reencode + CompressDXT)"


def ref_available() -> bool:
    return (REF_STREAMS / "manifest.json").exists()


def ref_manifest() -> dict:
    p = REF_STREAMS / "manifest.json"
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: run tests/golden/make_ref_streams.py where the reference is mounted")
    return json.loads(p.read_text())


def _ref_image(entry: dict) -> EncodedImage:
    stream = (REF_STREAMS / entry["name"]).read_bytes()
    if hashlib.sha256(stream).hexdigest() != entry["stream_sha256"]:
        raise ValueError(f"{entry['name']}: stream does not match its manifest digest")
    return EncodedImage(entry["width"], entry["height"], entry["seed"], stream, None,
                        encoder=REF_ENCODER, decoded_sha256=entry["decoded_sha256"])


def ref_batched() -> list[EncodedImage]:
    """The 64 batched images (w, h in {512, 1024, 2048}, seeds 1000 + i), in
    batch order, as the reference encoder wrote them."""
    ents = [e for e in ref_manifest()["streams"] if e["kind"] == "batched"]
    ents.sort(key=lambda e: e["seed"])
    return [_ref_image(e) for e in ents]


def ref_large() -> EncodedImage:
    """The 8192x8192 texture with 10 % of its area in 1-8 px checker regions."""
    (e,) = [e for e in ref_manifest()["streams"] if e["kind"] == "large"]
    return _ref_image(e)


def ref_plain() -> EncodedImage:
    """The 512x512 image of seed 0 (tests/golden/synth512_s0.gst)."""
    m = ref_manifest()["plain"]
    gold = json.loads((REF_PLAIN.parent / "golden.json").read_text())["streams"][REF_PLAIN.name]
    return EncodedImage(m["width"], m["height"], m["seed"], REF_PLAIN.read_bytes(), None, encoder=REF_ENCODER,
                        decoded_sha256=gold["blocks_sha256"])


def ref_serving_pool() -> dict[tuple[int, int], list[EncodedImage]]:
    """Every (w, h) class, w and h in {512, 1024, 2048, 4096}: the serving
    fixtures plus the batched images of that class (at least four each)."""
    pool: dict[tuple[int, int], list[EncodedImage]] = {}
    for e in ref_manifest()["streams"]:
        if e["kind"] in ("batched", "serving"):
            pool.setdefault((e["width"], e["height"]), []).append(_ref_image(e))
    return pool


def ref_rans_digest() -> dict:
    """SHA-256 of the reference ByteEncoder's section for rans_section()'s symbols."""
    return ref_manifest()["rans_2pow26"]
