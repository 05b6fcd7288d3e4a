"""Inputs of the palette-search fixtures (reencode.json): image recipes that
regenerate the same RGB8 bytes on every host, block edits, and the packing
of stored arrays (zlib + base64)."""
from __future__ import annotations

import base64
import zlib

import numpy as np

# blocks: "stb" = the reference encoder's own stb_dxt blocks (stored in the
# fixture); otherwise the project's block compressor, then an edit:
#   "plain"      -- as compressed;
#   "modes"      -- 10 % of the blocks with endpoints swapped (three-colour
#                   mode) and 5 % with equal endpoints;
#   "degenerate" -- 30 % of the words replaced by one index for all 16 pixels
#                   (0x00000000, 0x55555555, 0xAAAAAAAA, 0xFFFFFFFF): refits
#                   to them divide by zero or by a rounding residue.
CASES = [
    dict(name="synth64_stb", width=64, height=64, image="synth", seed=1, checker=0.0, blocks="stb"),
    dict(name="synth64_modes", width=64, height=64, image="synth", seed=2, checker=0.0, blocks="modes"),
    dict(name="checker128x32_stb", width=128, height=32, image="synth", seed=3, checker=0.5, blocks="stb"),
    dict(name="noise256x64_stb", width=256, height=64, image="noise", seed=4, blocks="stb"),
    dict(name="flat32_stb", width=32, height=32, image="flat", seed=5, blocks="stb"),
    dict(name="synth64_degenerate", width=64, height=64, image="synth", seed=6, checker=0.0, blocks="degenerate"),
    dict(name="smooth256x128_plain", width=256, height=128, image="smooth", seed=7, blocks="plain"),
    dict(name="synth256_stb", width=256, height=256, image="synth", seed=8, checker=0.1, blocks="stb"),
    dict(name="synth512x256_stb", width=512, height=256, image="synth", seed=11, checker=0.1, blocks="stb",
         stream=True),
]


def make_rgb(case: dict) -> np.ndarray:
    """The case's RGB8 image, shape (h, w, 3)."""
    w, h, seed = case["width"], case["height"], case["seed"]
    kind = case["image"]
    if kind == "synth":
        from gst_gb300 import encoder
        return encoder.synth_image(w, h, seed, case.get("checker", 0.0))
    rng = np.random.default_rng(seed)
    if kind == "noise":
        return rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)
    if kind == "flat":
        return np.broadcast_to(rng.integers(0, 256, size=3, dtype=np.uint8), (h, w, 3)).copy()
    if kind == "smooth":  # slow integer gradients: long runs of reused words
        y, x = np.mgrid[0:h, 0:w]
        r = (x * 255) // max(1, w - 1)
        g = (y * 255) // max(1, h - 1)
        b = ((x + y) * 255) // max(1, w + h - 2)
        return np.stack([r, g, b], axis=-1).astype(np.uint8)
    raise ValueError(kind)


def edit_blocks(blocks: np.ndarray, kind: str, seed: int) -> np.ndarray:
    b = np.ascontiguousarray(blocks, dtype=np.uint64).copy()
    rng = np.random.default_rng(seed + 1000)
    if kind == "plain":
        return b
    lo16 = np.uint64(0xFFFF)
    e1, e2 = b & lo16, (b >> np.uint64(16)) & lo16
    word = b >> np.uint64(32)
    if kind == "modes":
        sw = rng.random(b.size) < 0.10
        eq = ~sw & (rng.random(b.size) < 0.05)
        e1n = np.where(sw, e2, e1)
        e2n = np.where(sw, e1, np.where(eq, e1, e2))
        return e1n | (e2n << np.uint64(16)) | (word << np.uint64(32))
    if kind == "degenerate":
        m = rng.random(b.size) < 0.30
        uni = np.array([0x00000000, 0x55555555, 0xAAAAAAAA, 0xFFFFFFFF], np.uint64)[rng.integers(0, 4, b.size)]
        word = np.where(m, uni, word)
        return e1 | (e2 << np.uint64(16)) | (word << np.uint64(32))
    raise ValueError(kind)


def pack(a: np.ndarray) -> str:
    return base64.b64encode(zlib.compress(np.ascontiguousarray(a).tobytes(), 9)).decode()


def unpack(s: str, dtype) -> np.ndarray:
    return np.frombuffer(zlib.decompress(base64.b64decode(s)), dtype=dtype).copy()
