"""Regenerates tests/golden/reencode.json from the reference itself.

Runs only where the reference sources are mounted: it builds the reference's
CPU code (oracle/build_ref.sh) and calls it through oracle/ref_harness.cpp.
Each case is an RGB8 image (regenerated at test time from its recipe) and
DXT1 blocks (stored: the reference encoder's own blocks from stb_dxt, or the
project's block compressor with edited blocks), with the reference's results
of DXTImage(w, h, rgb, dxt) = DXTImage::Reencode (codec/dxt_image.cpp:455-468,
510-624): the blocks after the search, the palette words and the index
deltas; and, for sizes a GST stream allows, the SHA-256 and length of
GenTC::CompressDXT of that image (codec/encoder.cpp:39-195).

Usage: python tests/golden/make_reencode_golden.py
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

sys.path.insert(0, str(HERE))
import oracle  # noqa: E402
from reencode_inputs import CASES, edit_blocks, make_rgb, pack  # noqa: E402


def stb_blocks(ref, w: int, h: int, rgb: np.ndarray) -> np.ndarray:
    out = np.zeros(w * h // 16, np.uint64)
    ref.gstref_stb_blocks(w, h, np.ascontiguousarray(rgb).ctypes.data, out.ctypes.data)
    return out


def reference_reencode(ref, w: int, h: int, rgb: np.ndarray, blocks: np.ndarray, stream: bool):
    B = w * h // 16
    out = np.zeros(B, np.uint64)
    pal = np.zeros(4 * B, np.uint8)
    d = np.zeros(B, np.uint8)
    pl, sl = ctypes.c_size_t(), ctypes.c_size_t()
    cap = 16 * B + (1 << 20)
    st = np.zeros(cap, np.uint8) if stream else None
    rc = ref.gstref_reencode(w, h, np.ascontiguousarray(rgb).ctypes.data, np.ascontiguousarray(blocks).ctypes.data,
                             out.ctypes.data, pal.ctypes.data, pal.nbytes, ctypes.byref(pl), d.ctypes.data,
                             st.ctypes.data if stream else None, cap, ctypes.byref(sl))
    if rc != 0:
        raise RuntimeError(f"gstref_reencode failed: {rc}")
    return out, pal[: pl.value], d, (bytes(st[: sl.value]) if stream else None)


def main() -> None:
    subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True)
    ref = oracle.load_ref()
    if ref is None:
        raise SystemExit("reference harness not built")
    from gst_gb300 import encoder
    cases = []
    for c in CASES:
        w, h = c["width"], c["height"]
        rgb = make_rgb(c)
        if c["blocks"] == "stb":
            blocks = stb_blocks(ref, w, h, rgb)
        else:
            blocks = edit_blocks(encoder.compress_blocks(rgb, nthreads=1), c["blocks"], c["seed"])
        out, pal, d, stream = reference_reencode(ref, w, h, rgb, blocks, c.get("stream", False))
        entry = dict(c)
        entry.update(blocks_in=pack(blocks), blocks_out=pack(out), palette=pack(pal), deltas=pack(d),
                     palette_words=int(pal.size // 4), refit=int((out != blocks).sum()))
        if stream is not None:
            entry.update(stream_sha256=hashlib.sha256(stream).hexdigest(), stream_len=len(stream))
        cases.append(entry)
        print(f"{c['name']}: {w}x{h}, palette {pal.size // 4} of {w * h // 16}, refit {entry['refit']}")
    (HERE / "reencode.json").write_text(json.dumps({"cases": cases}, indent=1) + "\n")


if __name__ == "__main__":
    main()
