"""CPU oracle for the GST decode path -- TEST INFRASTRUCTURE ONLY.

``load()`` compiles and loads gst_oracle.c (a plain-C restatement of the
reference's OpenCL decoder, see gst_oracle.h).  ``load_ref()`` loads the
reference's own CPU code compiled from its sources by build_ref.sh, when it has
been built on this machine (it needs the reference sources, which only exist
where the reference is mounted).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SRC = HERE / "gst_oracle.c"
ORACLE_HDR = HERE / "gst_oracle.h"
ORACLE_LIB = HERE / "libgst_oracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libgstref.so"

SCAN_REFERENCE, SCAN_EXACT = 0, 1

_lib = None
_ref = None


def build(force: bool = False) -> Path:
    if force or not ORACLE_LIB.exists() or ORACLE_LIB.stat().st_mtime < max(
            ORACLE_SRC.stat().st_mtime, ORACLE_HDR.stat().st_mtime):
        subprocess.run([os.environ.get("CC", "gcc"), "-std=c11", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-pthread",
                        str(ORACLE_SRC), "-o", str(ORACLE_LIB), "-lm"], check=True)
    return ORACLE_LIB


def build_ref() -> bool:
    """Runs build_ref.sh (a no-op where the reference sources are absent)."""
    subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True)
    return REF_LIB.exists()


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(str(ORACLE_LIB))
        P, S, I, U32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint32
        lib.gsto_parse_header.argtypes = [P, S, P]
        lib.gsto_build_table.argtypes = [P, P, P, P]
        lib.gsto_build_table_direct.argtypes = [P, P, P, P]
        lib.gsto_rans_decode_group.argtypes = [P, S, U32, P, P, P, I, S, P]
        lib.gsto_inverse_wavelet_block.argtypes = [P, P]
        lib.gsto_inverse_wavelet_level.argtypes = [P, I, I]
        lib.gsto_scan_indices.argtypes = [P, U32, P, I]
        lib.gsto_ycocg_to_565.argtypes = [I, I, I]
        lib.gsto_ycocg_to_565.restype = ctypes.c_uint16
        lib.gsto_decode.argtypes = [P, S, P, S, I, I]
        lib.gsto_decode_rgb.argtypes = [P, S, P, S, I, I]
        lib.gsto_decode_symbols.argtypes = [P, S, P, S, I]
        lib.gsto_section_search.argtypes = [P, U32, U32]
        lib.gsto_normalize.argtypes = [P, I, I, P]
        lib.gsto_encode_section.argtypes = [P, S, P, S, ctypes.POINTER(S)]
        lib.gsto_encode_section_bound.argtypes = [S]
        lib.gsto_encode_section_bound.restype = S
        lib.gsto_encode_stream.argtypes = [U32, U32, U32, P, P, P, P, P, S, ctypes.POINTER(S)]
        lib.gsto_endpoint_planes.argtypes = [U32, U32, P, P, P]
        lib.gsto_endpoint_planes.restype = ctypes.c_uint64
        lib.gsto_run_palette.argtypes = [U32, U32, P, P, S, P]
        lib.gsto_run_palette.restype = U32
        lib.gsto_reencode.argtypes = [U32, U32, P, P, P, P, S, P]
        lib.gsto_reencode.restype = U32
        lib.gsto_reencode_candidate.argtypes = [P, U32, P, P, P]
        lib.gsto_section_search.restype = U32
        _lib = lib
    return _lib


def load_ref():
    """The reference's CPU code (oracle/_ref/libgstref.so) or None if not built here."""
    global _ref
    if _ref is None and REF_LIB.exists():
        lib = ctypes.CDLL(str(REF_LIB))
        P, S, I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
        lib.gstref_compress_rgb.argtypes = [I, I, P, P, S, ctypes.POINTER(S), P]
        lib.gstref_compress_file.argtypes = [ctypes.c_char_p, P, S, ctypes.POINTER(S), P, S,
                                             ctypes.POINTER(I), ctypes.POINTER(I)]
        lib.gstref_encode_bytes.argtypes = [P, S, P, S, ctypes.POINTER(S)]
        lib.gstref_decode_interleaved.argtypes = [P, S, S, P, S, S, P]
        lib.gstref_generate_histogram.argtypes = [P, S, I, P]
        lib.gstref_inverse_wavelet2d.argtypes = [P, P, S]
        lib.gstref_inverse_wavelet2d.restype = None
        lib.gstref_rans_encode_single.argtypes = [P, S, P, S, P, S, ctypes.POINTER(S), ctypes.POINTER(ctypes.c_uint32)]
        lib.gstref_encode_interleaved.argtypes = [P, S, P, S, S, P, S, ctypes.POINTER(S)]
        lib.gstref_reencode.argtypes = [I, I, P, P, P, P, S, ctypes.POINTER(S), P, P, S, ctypes.POINTER(S)]
        lib.gstref_stb_blocks.argtypes = [I, I, P, P]
        lib.gstref_stb_blocks.restype = None
        _ref = lib
    return _ref


def decode(stream: bytes, scan_mode: int = SCAN_REFERENCE, nthreads: int = 1) -> tuple[int, np.ndarray]:
    """Whole decode of one GST stream -> (status, DXT1 bytes)."""
    lib = load()
    w = int.from_bytes(stream[0:4], "little")
    h = int.from_bytes(stream[4:8], "little")
    out = np.zeros(max(w * h // 2, 8), dtype=np.uint8)
    st = lib.gsto_decode(stream, len(stream), out.ctypes.data, out.nbytes, scan_mode, nthreads)
    return int(st), out[: w * h // 2]


def decode_rgb(stream: bytes, scan_mode: int = SCAN_REFERENCE, nthreads: int = 1) -> tuple[int, np.ndarray]:
    """Whole decode of one GST stream to RGB8 (assemble_rgb) -> (status, W*H*3 bytes)."""
    lib = load()
    w = int.from_bytes(stream[0:4], "little")
    h = int.from_bytes(stream[4:8], "little")
    out = np.zeros(max(w * h * 3, 8), dtype=np.uint8)
    st = lib.gsto_decode_rgb(stream, len(stream), out.ctypes.data, out.nbytes, scan_mode, nthreads)
    return int(st), out[: w * h * 3]


def decode_symbols(stream: bytes, nthreads: int = 1) -> tuple[int, np.ndarray]:
    """rANS stage only -> (status, the reference's decompressed-symbol buffer)."""
    lib = load()
    w = int.from_bytes(stream[0:4], "little")
    h = int.from_bytes(stream[4:8], "little")
    pal = int.from_bytes(stream[8:12], "little")
    out = np.zeros(7 * (w * h // 16) + pal, dtype=np.uint8)
    st = lib.gsto_decode_symbols(stream, len(stream), out.ctypes.data, out.nbytes, nthreads)
    return int(st), out


def build_table(freqs, direct: bool = False):
    """Decode table from 256 u16 frequencies -> (freq, cum, sym) arrays of 2048."""
    lib = load()
    f = np.zeros(256, dtype=np.uint16)
    src = np.asarray(freqs, dtype=np.uint16)
    f[: src.size] = src
    fr = np.zeros(2048, np.uint16)
    cu = np.zeros(2048, np.uint16)
    sy = np.zeros(2048, np.uint8)
    (lib.gsto_build_table_direct if direct else lib.gsto_build_table)(
        f.ctypes.data, fr.ctypes.data, cu.ctypes.data, sy.ctypes.data)
    return fr, cu, sy


def rans_decode_groups(body: bytes, freqs, n_groups: int, streams: int) -> tuple[int, np.ndarray]:
    """ans_decode.cl over every group of a section body -> (status, symbols)."""
    lib = load()
    fr, cu, sy = build_table(freqs)
    out = np.zeros(n_groups * streams * 256, dtype=np.uint8)
    status = 0
    for g in range(n_groups):
        lo = 4 * n_groups if g == 0 else int.from_bytes(body[4 * (g - 1): 4 * g], "little")
        st = lib.gsto_rans_decode_group(body, len(body), g, fr.ctypes.data, cu.ctypes.data, sy.ctypes.data,
                                        streams, lo, out[g * streams * 256:].ctypes.data)
        status = status or int(st)
    return status, out


def scan_indices(deltas: np.ndarray, mode: int) -> np.ndarray:
    lib = load()
    d = np.ascontiguousarray(deltas, dtype=np.uint8)
    out = np.zeros(d.size, dtype=np.int32)
    lib.gsto_scan_indices(d.ctypes.data, d.size, out.ctypes.data, mode)
    return out


def normalize(counts, M: int = 2048) -> tuple[int, np.ndarray]:
    """ans::GenerateHistogram restated -> (status, normalized frequencies)."""
    lib = load()
    c = np.ascontiguousarray(counts, dtype=np.uint32)
    out = np.zeros(max(c.size, 1), dtype=np.uint32)
    st = lib.gsto_normalize(c.ctypes.data, c.size, M, out.ctypes.data)
    return int(st), out[: c.size]


def encode_section(symbols: np.ndarray) -> tuple[int, bytes]:
    """ByteEncoder::EncodeBytes restated -> (status, section bytes)."""
    lib = load()
    x = np.ascontiguousarray(symbols, dtype=np.uint8)
    cap = int(lib.gsto_encode_section_bound(x.size))
    out = np.zeros(max(cap, 1), dtype=np.uint8)
    n = ctypes.c_size_t()
    st = lib.gsto_encode_section(x.ctypes.data, x.size, out.ctypes.data, cap, ctypes.byref(n))
    return int(st), out[: n.value].tobytes()


def split_symbols(width: int, height: int, palette_bytes: int, symbols: np.ndarray):
    """The decompressed-symbol buffer (decoder.cpp:441-461 layout) as its four sections."""
    B = width * height // 16
    s = np.ascontiguousarray(symbols, dtype=np.uint8)
    return s[: 2 * B], s[2 * B: 6 * B], s[6 * B: 6 * B + palette_bytes], s[6 * B + palette_bytes: 7 * B + palette_bytes]


def encode_stream(width: int, height: int, palette_bytes: int, y, chroma, palette, indices) -> tuple[int, bytes]:
    """codec/encoder.cpp:122-144 restated: a GST stream from its four symbol sections."""
    lib = load()
    secs = [np.ascontiguousarray(a, dtype=np.uint8) for a in (y, chroma, palette, indices)]
    cap = 28 + sum(int(lib.gsto_encode_section_bound(a.size)) for a in secs)
    out = np.zeros(cap, dtype=np.uint8)
    n = ctypes.c_size_t()
    st = lib.gsto_encode_stream(width, height, palette_bytes, *(a.ctypes.data for a in secs), out.ctypes.data, cap,
                                ctypes.byref(n))
    return int(st), out[: n.value].tobytes()


def endpoint_planes(width: int, height: int, blocks: np.ndarray) -> tuple[np.ndarray, np.ndarray, int]:
    """The encoder's endpoint stages restated -> (Y section, chroma section, clipped coefficients)."""
    lib = load()
    blk = np.ascontiguousarray(blocks, dtype=np.uint64)
    B = width * height // 16
    y = np.zeros(2 * B, np.uint8)
    c = np.zeros(4 * B, np.uint8)
    clips = lib.gsto_endpoint_planes(width, height, blk.ctypes.data, y.ctypes.data, c.ctypes.data)
    return y, c, int(clips)


def reencode(width: int, height: int, rgb: np.ndarray, blocks: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """DXTImage::Reencode restated -> (blocks after the search, padded palette bytes, index deltas)."""
    lib = load()
    px = np.ascontiguousarray(rgb, dtype=np.uint8).reshape(-1)
    blk = np.ascontiguousarray(blocks, dtype=np.uint64)
    B = width * height // 16
    assert px.size == width * height * 3 and blk.size == B
    cap = (4 * B + 8191) // 8192 * 8192
    pal = np.zeros(cap, np.uint8)
    d = np.zeros(B, np.uint8)
    out = np.zeros(B, np.uint64)
    n = lib.gsto_reencode(width, height, px.ctypes.data, blk.ctypes.data, out.ctypes.data, pal.ctypes.data, cap,
                          d.ctypes.data)
    return out, pal[:n], d


def reencode_candidate(px48: np.ndarray, word: int) -> tuple[int, bool, int, int]:
    """One refit of the Reencode search -> (error, ok, ep1, ep2)."""
    lib = load()
    px = np.ascontiguousarray(px48, dtype=np.uint8).reshape(48)
    ok = ctypes.c_int()
    e1, e2 = ctypes.c_uint16(), ctypes.c_uint16()
    err = lib.gsto_reencode_candidate(px.ctypes.data, word, ctypes.byref(ok), ctypes.byref(e1), ctypes.byref(e2))
    return int(err), bool(ok.value), e1.value, e2.value


def run_palette(width: int, height: int, blocks: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The GPU pipeline's run palette restated -> (padded palette bytes, index deltas)."""
    lib = load()
    blk = np.ascontiguousarray(blocks, dtype=np.uint64)
    B = width * height // 16
    cap = (4 * B + 8191) // 8192 * 8192
    pal = np.zeros(cap, np.uint8)
    d = np.zeros(B, np.uint8)
    n = lib.gsto_run_palette(width, height, blk.ctypes.data, pal.ctypes.data, cap, d.ctypes.data)
    return pal[:n], d
