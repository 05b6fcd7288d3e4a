"""The GPU encoder stages (include/gst_encode.h) from Python.

Mirrors the reference's entropy-coding interfaces: ``normalize_frequencies``
is ans::ocl::NormalizeFrequencies (ans/ans_ocl_encode.cpp:6-8),
``encode_bytes`` is ByteEncoder::EncodeBytes (codec/entropy.cpp:174-265) for
many sections at once, ``encode_streams`` / ``compress_symbols`` assemble GST
streams as GenTC::CompressDXTImage does (codec/encoder.cpp:122-144);
``prepare_symbols`` / ``compress_dxt`` run its endpoint stages (YCoCg planes,
forward wavelet, an index palette) from DXT1 blocks.  Device
buffers are torch CUDA tensors (or raw pointers); everything runs through the
CUDA kernels of libgst_gb300.so, with no CPU path.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np

from .decoder import GPUContext, ReencodeImage, StreamSymbols, SymbolBuffers, _check, _ptr, _stream, load_library

SYMS_PER_GROUP = 8192


def section_bound(n_symbols: int) -> int:
    return int(load_library().gst_encode_section_bound(n_symbols))


def stream_bound(width: int, height: int, palette_bytes: int) -> int:
    return int(load_library().gst_encode_stream_bound(width, height, palette_bytes))


def normalize_frequencies(ctx: GPUContext, counts) -> np.ndarray:
    """GenerateHistogram(counts, 2048) on the GPU (blocking)."""
    c = np.ascontiguousarray(counts, dtype=np.uint32)
    out = np.zeros(c.size, dtype=np.uint32)
    _check(load_library().gst_encode_normalize(ctx.handle, c.ctypes.data, c.size, out.ctypes.data),
           "gst_encode_normalize")
    return out


def encode_bytes(ctx: GPUContext, sections: Sequence, out, offsets, stream=None) -> None:
    """Enqueues EncodeBytes for every device section (uint8, multiples of 8192)
    into `out`; `offsets` (int64, len(sections) + 1) receives the section starts
    and the total."""
    lib = load_library()
    n = len(sections)
    ptrs = (ctypes.c_void_p * n)(*[_ptr(s) for s in sections])
    sizes = (ctypes.c_size_t * n)(*[int(s.numel()) for s in sections])
    _check(lib.gst_encode_bytes(ctx.handle, n, ptrs, sizes, _ptr(out), int(out.numel()), _ptr(offsets),
                                _stream(stream)), "gst_encode_bytes")


def stream_symbols(width: int, height: int, palette_bytes: int, symbols) -> StreamSymbols:
    """The four sections of a device buffer in the decompressed-symbol layout."""
    B = width * height // 16
    base = _ptr(symbols)
    return StreamSymbols(width, height, palette_bytes, 0, base, base + 2 * B, base + 6 * B,
                         base + 6 * B + palette_bytes)


def encode_streams(ctx: GPUContext, images, out, offsets, stream=None) -> None:
    """Enqueues one GST stream per image into `out`; `offsets` (int64,
    len(images) + 1) receives the stream starts and the total.  `images`: a
    sequence of StreamSymbols or a ctypes array of them (reused as is)."""
    lib = load_library()
    arr = images if isinstance(images, ctypes.Array) else (StreamSymbols * len(images))(*images)
    _check(lib.gst_encode_streams(ctx.handle, arr, len(arr), _ptr(out), int(out.numel()), _ptr(offsets),
                                  _stream(stream)), "gst_encode_streams")


def compress_symbols(ctx: GPUContext, width: int, height: int, palette_bytes: int, symbols: np.ndarray) -> bytes:
    """Host-to-host: one GST stream from a decompressed-symbol buffer (blocking)."""
    lib = load_library()
    s = np.ascontiguousarray(symbols, dtype=np.uint8)
    cap = stream_bound(width, height, palette_bytes)
    if cap == 0:
        raise ValueError("dimensions the decoder would reject")
    out = np.zeros(cap, dtype=np.uint8)
    n = ctypes.c_size_t()
    _check(lib.gst_compress_symbols(ctx.handle, width, height, palette_bytes, s.ctypes.data, out.ctypes.data, cap,
                                    ctypes.byref(n)), "gst_compress_symbols")
    return out[: n.value].tobytes()


def palette_capacity(width: int, height: int) -> int:
    return int(load_library().gst_palette_capacity(width, height))


def symbol_buffers(images: Sequence[tuple]) -> ctypes.Array:
    """The gst_symbol_buffers array of (width, height, d_blocks, d_y, d_chroma,
    d_palette, d_indices) tuples (device tensors or pointers), for reuse."""
    return (SymbolBuffers * len(images))(*[SymbolBuffers(w, h, *(_ptr(b) for b in bufs)) for w, h, *bufs in images])


def prepare_symbols(ctx: GPUContext, images, d_palette_bytes, stream=None) -> None:
    """Enqueues the endpoint stages; images: (width, height, d_blocks, d_y,
    d_chroma, d_palette, d_indices) tuples with device buffers (uint8 / uint64
    tensors or pointers), or a symbol_buffers() array; d_palette_bytes:
    uint32/int32 device array, one per image."""
    lib = load_library()
    arr = images if isinstance(images, ctypes.Array) else symbol_buffers(images)
    _check(lib.gst_prepare_symbols(ctx.handle, arr, len(arr), _ptr(d_palette_bytes), _stream(stream)),
           "gst_prepare_symbols")


def compress_dxt(ctx: GPUContext, width: int, height: int, blocks: np.ndarray) -> bytes:
    """Host-to-host: DXT1 blocks (uint64, raster order) -> GST stream (blocking)."""
    lib = load_library()
    b = np.ascontiguousarray(blocks, dtype=np.uint64)
    cap = stream_bound(width, height, palette_capacity(width, height))
    if cap == 0:
        raise ValueError("dimensions the decoder would reject")
    out = np.zeros(cap, dtype=np.uint8)
    n = ctypes.c_size_t()
    _check(lib.gst_compress_dxt(ctx.handle, width, height, b.ctypes.data, out.ctypes.data, cap, ctypes.byref(n)),
           "gst_compress_dxt")
    return out[: n.value].tobytes()


def prepare_planes(ctx: GPUContext, images, stream=None) -> None:
    """Enqueues the Y and chroma sections only (gst_prepare_planes); images as
    for prepare_symbols (d_palette and d_indices are not used)."""
    lib = load_library()
    arr = images if isinstance(images, ctypes.Array) else symbol_buffers(images)
    _check(lib.gst_prepare_planes(ctx.handle, arr, len(arr), _stream(stream)), "gst_prepare_planes")


def reencode_images(images: Sequence[tuple]) -> ctypes.Array:
    """The gst_reencode_image array of (width, height, d_rgb, d_blocks,
    d_blocks_out, d_palette, d_indices, d_palette_bytes) tuples, for reuse."""
    return (ReencodeImage * len(images))(*[ReencodeImage(w, h, *(_ptr(b) for b in bufs)) for w, h, *bufs in images])


def reencode_blocks(ctx: GPUContext, images, stream=None) -> None:
    """Enqueues the reference's index palette search (gst_reencode_blocks) for
    every image: tuples as for reencode_images, or such an array."""
    lib = load_library()
    arr = images if isinstance(images, ctypes.Array) else reencode_images(images)
    _check(lib.gst_reencode_blocks(ctx.handle, arr, len(arr), _stream(stream)), "gst_reencode_blocks")


def compress_rgb_dxt(ctx: GPUContext, width: int, height: int, rgb: np.ndarray, blocks: np.ndarray) -> bytes:
    """Host-to-host: RGB8 source (h, w, 3) and its DXT1 blocks -> the GST
    stream of the reference's CompressDXTImage(DXTImage(w, h, rgb, dxt))."""
    lib = load_library()
    px = np.ascontiguousarray(rgb, dtype=np.uint8)
    b = np.ascontiguousarray(blocks, dtype=np.uint64)
    if px.size != width * height * 3 or b.size != width * height // 16:
        raise ValueError("rgb and blocks must match width x height")
    cap = stream_bound(width, height, palette_capacity(width, height))
    if cap == 0:
        raise ValueError("dimensions the decoder would reject")
    out = np.zeros(cap, dtype=np.uint8)
    n = ctypes.c_size_t()
    _check(lib.gst_compress_rgb_dxt(ctx.handle, width, height, px.ctypes.data, b.ctypes.data, out.ctypes.data, cap,
                                    ctypes.byref(n)), "gst_compress_rgb_dxt")
    return out[: n.value].tobytes()
