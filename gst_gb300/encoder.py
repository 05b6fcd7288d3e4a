"""Python face of the project's GST stream producer (csrc/gst_encoder.cpp).

Used to make decoder inputs: synthetic images, their GST streams, and single
rANS sections for the rANS-only workload.  The section format and the rANS and
frequency-normalisation stages match the reference encoder byte for byte
(checked in tests/test_encoder.py against the reference's own ByteEncoder).
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from .build import ENCODER_LIB

_lib = None


def load_library() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    from .build import build_all
    build_all()
    if not Path(ENCODER_LIB).exists():
        raise RuntimeError(f"gst_gb300: encoder library missing at {ENCODER_LIB}")
    lib = ctypes.CDLL(str(ENCODER_LIB))
    P, S = ctypes.c_void_p, ctypes.c_size_t
    lib.gst_synth_image.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double, P]
    lib.gst_encode_rgb.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P, ctypes.POINTER(P), ctypes.POINTER(S), P,
                                   ctypes.POINTER(ctypes.c_uint64), ctypes.c_int]
    lib.gst_encode_dxt.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P, P, ctypes.POINTER(P), ctypes.POINTER(S), P,
                                   ctypes.POINTER(ctypes.c_uint64)]
    lib.gst_compress_blocks.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P, P, ctypes.c_int]
    lib.gst_encode_section.argtypes = [P, S, ctypes.POINTER(P), ctypes.POINTER(S), ctypes.c_int]
    lib.gst_normalize_frequencies.argtypes = [P, S, ctypes.c_int, P]
    lib.gst_encoder_free.argtypes = [P]
    lib.gst_encoder_free.restype = None
    _lib = lib
    return lib


def _threads(n: int) -> int:
    return n if n > 0 else (os.cpu_count() or 1)


def synth_image(w: int, h: int, seed: int, checker_frac: float = 0.0) -> np.ndarray:
    """Seeded synthetic RGB8 image, shape (h, w, 3)."""
    out = np.empty((h, w, 3), dtype=np.uint8)
    if load_library().gst_synth_image(w, h, seed, checker_frac, out.ctypes.data) != 0:
        raise ValueError("gst_synth_image failed")
    return out


def _take(ptr: ctypes.c_void_p, n: int) -> bytes:
    data = ctypes.string_at(ptr, n)
    load_library().gst_encoder_free(ptr)
    return data


def encode_rgb(rgb: np.ndarray, nthreads: int = 0) -> tuple[bytes, np.ndarray, int]:
    """RGB8 image -> (GST stream, the DXT1 blocks it encodes as uint64, clipped
    wavelet coefficients)."""
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w, _ = rgb.shape
    out = ctypes.c_void_p()
    n = ctypes.c_size_t()
    blocks = np.empty(w * h // 16, dtype=np.uint64)
    clips = ctypes.c_uint64()
    rc = load_library().gst_encode_rgb(w, h, rgb.ctypes.data, ctypes.byref(out), ctypes.byref(n),
                                       blocks.ctypes.data, ctypes.byref(clips), _threads(nthreads))
    if rc != 0:
        raise ValueError(f"gst_encode_rgb({w}x{h}) failed: {rc}")
    return _take(out, n.value), blocks, int(clips.value)


def compress_blocks(rgb: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """RGB8 image (h, w, 3) -> its DXT1 blocks (uint64, raster order) from the
    block compressor alone, before any palette search."""
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w, _ = rgb.shape
    blocks = np.empty(w * h // 16, dtype=np.uint64)
    rc = load_library().gst_compress_blocks(w, h, rgb.ctypes.data, blocks.ctypes.data, _threads(nthreads))
    if rc != 0:
        raise ValueError(f"gst_compress_blocks({w}x{h}) failed: {rc}")
    return blocks


def encode_dxt(w: int, h: int, dxt_blocks: np.ndarray, rgb: np.ndarray | None = None) -> tuple[bytes, np.ndarray, int]:
    """Given DXT1 blocks (uint64 per block, raster order) -> GST stream."""
    dxt = np.ascontiguousarray(dxt_blocks, dtype=np.uint64)
    out = ctypes.c_void_p()
    n = ctypes.c_size_t()
    blocks = np.empty(w * h // 16, dtype=np.uint64)
    clips = ctypes.c_uint64()
    rgb_ptr = None if rgb is None else np.ascontiguousarray(rgb, dtype=np.uint8).ctypes.data
    rc = load_library().gst_encode_dxt(w, h, rgb_ptr, dxt.ctypes.data, ctypes.byref(out), ctypes.byref(n),
                                       blocks.ctypes.data, ctypes.byref(clips))
    if rc != 0:
        raise ValueError(f"gst_encode_dxt({w}x{h}) failed: {rc}")
    return _take(out, n.value), blocks, int(clips.value)


def encode_section(symbols, nthreads: int = 0) -> bytes:
    """Bytes (length a multiple of 8192) -> one section in the reference's
    ByteEncoder format: 512-byte frequency table, u32 group end offsets, groups."""
    sym = np.ascontiguousarray(np.frombuffer(bytes(symbols), dtype=np.uint8) if isinstance(symbols, (bytes, bytearray))
                               else symbols, dtype=np.uint8)
    out = ctypes.c_void_p()
    n = ctypes.c_size_t()
    rc = load_library().gst_encode_section(sym.ctypes.data, sym.size, ctypes.byref(out), ctypes.byref(n),
                                           _threads(nthreads))
    if rc != 0:
        raise ValueError(f"gst_encode_section failed: {rc}")
    return _take(out, n.value)


def normalize_frequencies(counts, M: int = 2048) -> np.ndarray:
    """ans/histogram.cpp:40-121 (GenerateHistogram)."""
    c = np.ascontiguousarray(counts, dtype=np.uint32)
    out = np.empty_like(c)
    if load_library().gst_normalize_frequencies(c.ctypes.data, c.size, M, out.ctypes.data) != 0:
        raise ValueError("gst_normalize_frequencies failed")
    return out
