"""The reference's decoder API (codec/decoder.h, namespace GenTC) over the C ABI.

Names, argument meaning and error behaviour mirror ``GenTC``:

=====================================  ==========================================
reference                              here
=====================================  ==========================================
``gpu::GPUContext::InitializeOpenCL``  :class:`GPUContext` (a CUDA device)
``GenTCHeader`` / ``LoadFrom``         :class:`GenTCHeader` / ``load_from``
``InitializeDecoder``                  :func:`initialize_decoder`
``DecompressDXT``                      :func:`decompress_dxt`
``LoadCompressedDXT(s)``               :func:`load_compressed_dxt(s)`
``RequiredScratchMem``                 :func:`required_scratch_mem`
``PreallocateDecompressor``            :func:`preallocate_decompressor`
``FreeDecompressor``                   :func:`free_decompressor`
=====================================  ==========================================

Device buffers are passed as integers or objects with ``data_ptr()`` (torch
tensors); streams as ``None``, an integer ``cudaStream_t`` or an object with a
``cuda_stream`` attribute (``torch.cuda.Stream``).  The library is the in-tree
``libgst_gb300.so``; if it is missing the calls raise -- there is no fallback.
"""
from __future__ import annotations

import ctypes
from pathlib import Path
from typing import Iterable, Sequence

import numpy as np

from .build import DECODER_LIB

GST_OK, GST_E_ARG, GST_E_FORMAT, GST_E_OOM, GST_E_CUDA, GST_E_TIMEOUT = range(6)
STATUS_NAMES = {
    GST_OK: "GST_OK", GST_E_ARG: "GST_E_ARG", GST_E_FORMAT: "GST_E_FORMAT",
    GST_E_OOM: "GST_E_OOM", GST_E_CUDA: "GST_E_CUDA", GST_E_TIMEOUT: "GST_E_TIMEOUT",
}

# Every symbol include/gst_decoder.h declares.
EXPORTED_SYMBOLS = (
    "gst_init", "gst_destroy", "gst_initialize_decoder", "gst_parse_header",
    "gst_required_scratch", "gst_preallocate", "gst_free_decompressor",
    "gst_decompress_dxt", "gst_load_compressed_dxt", "gst_load_compressed_dxts", "gst_load_rgb", "gst_load_rgbs",
    "gst_load_host_dxts",
    "gst_batch_layout_bytes", "gst_pack_batch", "gst_decode_rans_groups",
    "gst_batch_create", "gst_batch_destroy", "gst_batch_device_bytes", "gst_batch_rans_items",
    "gst_batch_launch", "gst_batch_graph_launch", "gst_batch_host_launch", "gst_batch_autotune", "gst_size_class",
    "gst_set_class_tuning", "gst_get_class_tuning", "gst_autotune_class", "gst_save_class_tuning",
    "gst_load_class_tuning", "gst_batch_set_tuning", "gst_load_compressed_dxt_static",
    "gst_sync_status", "gst_last_launch_count", "gst_set_profiling", "gst_kernel_times", "gst_set_option",
    "gst_status_string",
    "gst_server_create", "gst_server_destroy", "gst_server_now_ns", "gst_server_submit", "gst_server_poll",
    "gst_server_read", "gst_server_release", "gst_server_cancel", "gst_server_read_stats", "gst_server_schedule",
    "gst_server_schedule_wait",
    # include/gst_encode.h
    "gst_encode_section_bound", "gst_encode_stream_bound", "gst_encode_bytes", "gst_encode_streams",
    "gst_compress_symbols", "gst_encode_normalize", "gst_palette_capacity", "gst_prepare_symbols",
    "gst_compress_dxt", "gst_prepare_planes", "gst_reencode_blocks", "gst_compress_rgb_dxt",
)


class GstError(RuntimeError):
    """A C-ABI call returned a status other than GST_OK."""

    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)}")


class ServerConfig(ctypes.Structure):
    """gst_server_config."""
    _fields_ = [("device_budget_bytes", ctypes.c_size_t), ("host_staging_bytes", ctypes.c_size_t),
                ("slot_scratch_bytes", ctypes.c_size_t), ("max_inflight", ctypes.c_int),
                ("max_batch_images", ctypes.c_int)]


class ServerResult(ctypes.Structure):
    """gst_server_result."""
    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_int), ("d_dxt", ctypes.c_void_p),
                ("dxt_bytes", ctypes.c_size_t), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("arrival_ns", ctypes.c_uint64), ("launch_ns", ctypes.c_uint64), ("done_ns", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    """gst_server_stats."""
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "rejected", "launches", "launched_images",
                                                "pixels", "queued")] + \
               [("device_bytes_in_use", ctypes.c_size_t), ("device_bytes_peak", ctypes.c_size_t)] + \
               [(n, ctypes.c_double) for n in ("seconds", "latency_mean_us", "latency_p50_us", "latency_p99_us",
                                                "latency_max_us")] + \
               [("cancelled", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class StreamSymbols(ctypes.Structure):
    """gst_stream_symbols: the four symbol sections of one image (device pointers)."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("palette_bytes", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("d_y", ctypes.c_void_p), ("d_chroma", ctypes.c_void_p),
                ("d_palette", ctypes.c_void_p), ("d_indices", ctypes.c_void_p)]


class SymbolBuffers(ctypes.Structure):
    """gst_symbol_buffers: one image's DXT1 blocks in, its four sections out (device pointers)."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("d_blocks", ctypes.c_void_p),
                ("d_y", ctypes.c_void_p), ("d_chroma", ctypes.c_void_p), ("d_palette", ctypes.c_void_p),
                ("d_indices", ctypes.c_void_p)]


class ReencodeImage(ctypes.Structure):
    """gst_reencode_image: one image's RGB8 source and DXT1 blocks in; the
    searched blocks, palette, index deltas and palette size out (device pointers)."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("d_rgb", ctypes.c_void_p),
                ("d_blocks", ctypes.c_void_p), ("d_blocks_out", ctypes.c_void_p), ("d_palette", ctypes.c_void_p),
                ("d_indices", ctypes.c_void_p), ("d_palette_bytes", ctypes.c_void_p)]


class GenTCHeader(ctypes.Structure):
    """codec/codec_base.h:9-20 -- seven little-endian u32 words."""

    _fields_ = [(name, ctypes.c_uint32) for name in (
        "width", "height", "palette_bytes", "y_cmp_sz", "chroma_cmp_sz", "palette_sz", "indices_sz")]

    @classmethod
    def load_from(cls, buf: bytes) -> "GenTCHeader":
        """codec/codec_base.cpp:18-25, without validation (see :func:`parse_header`)."""
        if len(buf) < 28:
            raise GstError(GST_E_FORMAT, "GenTCHeader.load_from")
        return cls.from_buffer_copy(bytes(buf[:28]))

    @property
    def num_blocks(self) -> int:
        return (self.width // 4) * (self.height // 4)

    @property
    def dxt_bytes(self) -> int:
        return self.num_blocks * 8

    @property
    def compressed_bytes(self) -> int:
        return self.y_cmp_sz + self.chroma_cmp_sz + self.palette_sz + self.indices_sz

    def as_tuple(self):
        return tuple(getattr(self, f) for f, _ in self._fields_)


_lib = None


def load_library() -> ctypes.CDLL:
    """Loads libgst_gb300.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    from .build import build_all
    build_all()
    if not Path(DECODER_LIB).exists():
        raise RuntimeError(f"gst_gb300: CUDA decoder library missing at {DECODER_LIB}")
    lib = ctypes.CDLL(str(DECODER_LIB))
    P, S, U32, I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int
    HP = ctypes.POINTER(GenTCHeader)
    sig = {
        "gst_init": (I, [I, ctypes.POINTER(P)]),
        "gst_destroy": (None, [P]),
        "gst_initialize_decoder": (I, [P]),
        "gst_parse_header": (I, [P, S, HP]),
        "gst_required_scratch": (S, [HP]),
        "gst_preallocate": (I, [P, S]),
        "gst_free_decompressor": (I, [P]),
        "gst_decompress_dxt": (I, [P, P, S, P, S]),
        "gst_load_compressed_dxt": (I, [P, HP, P, P, P]),
        "gst_load_compressed_dxts": (I, [P, HP, I, P, P, P]),
        "gst_load_rgb": (I, [P, HP, P, P, P]),
        "gst_load_host_dxts": (I, [P, HP, I, P, P, I, P]),
        "gst_load_rgbs": (I, [P, HP, I, P, P, P]),
        "gst_batch_layout_bytes": (S, [HP, I]),
        "gst_pack_batch": (I, [ctypes.POINTER(P), ctypes.POINTER(S), I, P, S]),
        "gst_decode_rans_groups": (I, [P, P, P, U32, U32, U32, P, P]),
        "gst_batch_create": (I, [P, HP, I, ctypes.POINTER(P)]),
        "gst_batch_destroy": (None, [P]),
        "gst_batch_device_bytes": (S, [P]),
        "gst_batch_rans_items": (I, [P]),
        "gst_batch_launch": (I, [P, P, P, P]),
        "gst_batch_autotune": (I, [P, P, P, P, I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]),
        "gst_batch_set_tuning": (I, [P, I, I, I]),
        "gst_batch_graph_launch": (I, [P, P, P, P]),
        "gst_batch_host_launch": (I, [P, P, P, I, P]),
        "gst_size_class": (I, [ctypes.c_uint64]),
        "gst_set_class_tuning": (I, [P, I, I, I, I]),
        "gst_get_class_tuning": (I, [P, I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]),
        "gst_autotune_class": (I, [P, HP, I, P, P, P, I, ctypes.POINTER(I)]),
        "gst_save_class_tuning": (I, [P, ctypes.c_char_p]),
        "gst_load_class_tuning": (I, [P, ctypes.c_char_p]),
        "gst_load_compressed_dxt_static": (I, [HP, P, P, P, ctypes.POINTER(U32)]),
        "gst_sync_status": (I, [P, P]),
        "gst_last_launch_count": (I, [P]),
        "gst_set_profiling": (I, [P, I]),
        "gst_set_option": (I, [P, ctypes.c_char_p, I]),
        "gst_kernel_times": (I, [P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_char_p), I]),
        "gst_status_string": (ctypes.c_char_p, [I]),
        "gst_server_create": (I, [P, ctypes.POINTER(ServerConfig), ctypes.POINTER(P)]),
        "gst_server_destroy": (None, [P]),
        "gst_server_now_ns": (ctypes.c_uint64, [P]),
        "gst_server_submit": (I, [P, P, S, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
        "gst_server_poll": (I, [P, ctypes.POINTER(ServerResult), I, ctypes.POINTER(I), I]),
        "gst_server_read": (I, [P, ctypes.c_uint64, P, S]),
        "gst_server_release": (I, [P, ctypes.c_uint64]),
        "gst_server_cancel": (I, [P, ctypes.c_uint64]),
        "gst_server_read_stats": (I, [P, ctypes.POINTER(ServerStats), I]),
        "gst_server_schedule": (I, [P, I, P, P, P, P]),
        "gst_server_schedule_wait": (I, [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(ctypes.c_uint64)]),
        "gst_encode_section_bound": (S, [S]),
        "gst_encode_stream_bound": (S, [U32, U32, U32]),
        "gst_encode_bytes": (I, [P, I, ctypes.POINTER(P), ctypes.POINTER(S), P, S, P, P]),
        "gst_encode_streams": (I, [P, ctypes.POINTER(StreamSymbols), I, P, S, P, P]),
        "gst_compress_symbols": (I, [P, U32, U32, U32, P, P, S, ctypes.POINTER(S)]),
        "gst_encode_normalize": (I, [P, P, I, P]),
        "gst_palette_capacity": (S, [U32, U32]),
        "gst_prepare_symbols": (I, [P, ctypes.POINTER(SymbolBuffers), I, P, P]),
        "gst_compress_dxt": (I, [P, U32, U32, P, P, S, ctypes.POINTER(S)]),
        "gst_prepare_planes": (I, [P, ctypes.POINTER(SymbolBuffers), I, P]),
        "gst_reencode_blocks": (I, [P, ctypes.POINTER(ReencodeImage), I, P]),
        "gst_compress_rgb_dxt": (I, [P, U32, U32, P, P, P, S, ctypes.POINTER(S)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status: int, what: str) -> None:
    if status != GST_OK:
        raise GstError(status, what)


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if hasattr(x, "__cuda_array_interface__"):
        return int(x.__cuda_array_interface__["data"][0])
    raise TypeError(f"cannot take a device pointer from {type(x)!r}")


def _stream(s) -> int:
    if s is None:
        return 0
    if isinstance(s, int):
        return s
    if hasattr(s, "cuda_stream"):
        return int(s.cuda_stream)
    raise TypeError(f"cannot take a CUDA stream from {type(s)!r}")


def _as_bytes(data) -> bytes:
    if isinstance(data, (bytes, bytearray, memoryview)):
        return bytes(data)
    return np.ascontiguousarray(data, dtype=np.uint8).tobytes()


class GPUContext:
    """One CUDA device and its decoder context (gpu::GPUContext, gpu/gpu.h:35-176)."""

    def __init__(self, device: int = 0):
        lib = load_library()
        h = ctypes.c_void_p()
        _check(lib.gst_init(device, ctypes.byref(h)), "gst_init")
        self._h = h
        self.device = device

    @property
    def handle(self) -> ctypes.c_void_p:
        if self._h is None:
            raise GstError(GST_E_ARG, "GPUContext is closed")
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            load_library().gst_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_launch_count(self) -> int:
        return int(load_library().gst_last_launch_count(self.handle))

    def set_option(self, name: str, value: int) -> None:
        """gst_set_option: a tuning knob ("rans_blocks_per_sm", "rans_stage_words")."""
        _check(load_library().gst_set_option(self.handle, name.encode(), int(value)), "gst_set_option")

    def set_profiling(self, enable: bool) -> None:
        _check(load_library().gst_set_profiling(self.handle, int(enable)), "gst_set_profiling")

    def kernel_times(self) -> list[tuple[str, float]]:
        """(kernel name, milliseconds) of each kernel of the last decode call."""
        ms = (ctypes.c_float * 8)()
        names = (ctypes.c_char_p * 8)()
        n = load_library().gst_kernel_times(self.handle, ms, names, 8)
        return [(names[i].decode(), float(ms[i])) for i in range(n)]


class ResidentBatch:
    """A resident batch (gst_batch_*): plan uploaded once, own scratch; each
    launch enqueues kernels only.  ``graph=True`` replays a captured CUDA graph."""

    def __init__(self, ctx: GPUContext, hdrs: Sequence[GenTCHeader]):
        arr = (GenTCHeader * len(hdrs))(*hdrs)
        h = ctypes.c_void_p()
        _check(load_library().gst_batch_create(ctx.handle, arr, len(hdrs), ctypes.byref(h)), "gst_batch_create")
        self._h = h
        self.ctx = ctx
        self.hdrs = list(hdrs)

    @property
    def device_bytes(self) -> int:
        return int(load_library().gst_batch_device_bytes(self._h))

    @property
    def rans_items(self) -> int:
        """gst_batch_rans_items: rANS CTAs of the next two-kernel launch."""
        return int(load_library().gst_batch_rans_items(self._h))

    def launch(self, cmp_data, output, stream=None, graph: bool = False) -> None:
        fn = load_library().gst_batch_graph_launch if graph else load_library().gst_batch_launch
        _check(fn(self._h, _ptr(cmp_data), _ptr(output), _stream(stream)), "gst_batch_launch")

    def host_launch(self, h_cmp, h_out, chunks: int = 0, stream=None) -> None:
        """gst_batch_host_launch: pinned host layout in, pinned DXT1 out, the
        pipelined copies and decodes replayed from a captured graph."""
        _check(load_library().gst_batch_host_launch(self._h, _ptr(h_cmp), _ptr(h_out), int(chunks), _stream(stream)),
               "gst_batch_host_launch")

    def autotune(self, cmp_data, output, stream=None, iterations: int = 3) -> tuple[int, int, int]:
        """gst_batch_autotune: times each launch configuration on this batch
        and keeps the fastest; returns (blocks_per_sm, stage_words, persistent)."""
        bps, words, pers = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        _check(load_library().gst_batch_autotune(self._h, _ptr(cmp_data), _ptr(output), _stream(stream),
                                                 int(iterations), ctypes.byref(bps), ctypes.byref(words),
                                                 ctypes.byref(pers)),
               "gst_batch_autotune")
        return bps.value, words.value, pers.value

    def set_tuning(self, blocks_per_sm: int, stage_words: int, persistent: int = 0) -> None:
        """gst_batch_set_tuning; (0, 0) returns to the context's configuration."""
        _check(load_library().gst_batch_set_tuning(self._h, int(blocks_per_sm), int(stage_words), int(persistent)),
               "gst_batch_set_tuning")

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            load_library().gst_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def parse_header(data) -> GenTCHeader:
    """GenTCHeader::LoadFrom plus validation of the whole stream (raises GstError)."""
    buf = _as_bytes(data)
    hdr = GenTCHeader()
    _check(load_library().gst_parse_header(buf, len(buf), ctypes.byref(hdr)), "gst_parse_header")
    return hdr


def initialize_decoder(ctx: GPUContext) -> bool:
    """codec/decoder.cpp:558-591: True if the device can run the kernels."""
    return load_library().gst_initialize_decoder(ctx.handle) == GST_OK


def decompress_dxt(ctx: GPUContext, cmp_data) -> np.ndarray:
    """codec/decoder.cpp:525-532: GST bytes -> DXT1 bytes (w*h/2, uint8), blocking."""
    buf = _as_bytes(cmp_data)
    hdr = GenTCHeader.load_from(buf)
    out = np.empty(hdr.dxt_bytes, dtype=np.uint8)
    _check(load_library().gst_decompress_dxt(ctx.handle, buf, len(buf), out.ctypes.data, out.nbytes),
           "gst_decompress_dxt")
    return out


def load_compressed_dxts(ctx: GPUContext, hdrs: Sequence[GenTCHeader], cmp_data, output, stream=None) -> None:
    """codec/decoder.cpp:540-544: device-resident batch decode, enqueued on `stream`."""
    arr = (GenTCHeader * len(hdrs))(*hdrs)
    _check(load_library().gst_load_compressed_dxts(ctx.handle, arr, len(hdrs), _ptr(cmp_data), _ptr(output),
                                                   _stream(stream)), "gst_load_compressed_dxts")


def header_array(hdrs: Sequence[GenTCHeader]) -> ctypes.Array:
    """The gst_header array of a batch, for calls that reuse it."""
    return (GenTCHeader * len(hdrs))(*hdrs)


def load_host_dxts(ctx: GPUContext, hdrs, h_cmp, h_out, chunks: int = 0, stream=None) -> None:
    """gst_load_host_dxts: pinned host layout in, pinned host DXT1 out, with the
    copies in, decodes and copies out of `chunks` runs of images overlapped.
    `hdrs`: GenTCHeader sequence or a header_array()."""
    arr = hdrs if isinstance(hdrs, ctypes.Array) else header_array(hdrs)
    _check(load_library().gst_load_host_dxts(ctx.handle, arr, len(hdrs), _ptr(h_cmp), _ptr(h_out), int(chunks),
                                             _stream(stream)), "gst_load_host_dxts")


def load_rgbs(ctx: GPUContext, hdrs: Sequence[GenTCHeader], cmp_data, output, stream=None) -> None:
    """LoadRGBs (codec/decoder.cpp:552-556): the decode as RGB8, w*h*3 bytes per image."""
    arr = (GenTCHeader * len(hdrs))(*hdrs)
    _check(load_library().gst_load_rgbs(ctx.handle, arr, len(hdrs), _ptr(cmp_data), _ptr(output), _stream(stream)),
           "gst_load_rgbs")


def load_rgb(ctx: GPUContext, hdr: GenTCHeader, cmp_data, output, stream=None) -> None:
    """LoadRGB (codec/decoder.cpp:546-550)."""
    _check(load_library().gst_load_rgb(ctx.handle, ctypes.byref(hdr), _ptr(cmp_data), _ptr(output),
                                       _stream(stream)), "gst_load_rgb")


def load_compressed_dxt(ctx: GPUContext, hdr: GenTCHeader, cmp_data, output, stream=None) -> None:
    """codec/decoder.cpp:534-538."""
    _check(load_library().gst_load_compressed_dxt(ctx.handle, ctypes.byref(hdr), _ptr(cmp_data), _ptr(output),
                                                  _stream(stream)), "gst_load_compressed_dxt")


def decode_rans_groups(ctx: GPUContext, freqs, body, body_bytes: int, n_groups: int, streams_per_group: int,
                       output, stream=None) -> None:
    """rANS stage alone (ans::ocl::OpenCLDecoder::Decode, ans/ans_ocl.h:26-72)."""
    _check(load_library().gst_decode_rans_groups(ctx.handle, _ptr(freqs), _ptr(body), body_bytes, n_groups,
                                                 streams_per_group, _ptr(output), _stream(stream)),
           "gst_decode_rans_groups")


def sync_status(ctx: GPUContext, stream=None) -> int:
    """Waits for `stream`; GST_OK or the device-side status of the last decode."""
    return int(load_library().gst_sync_status(ctx.handle, _stream(stream)))


def required_scratch_mem(hdr: GenTCHeader) -> int:
    """codec/decoder.cpp:41-47 (this decoder's own requirement)."""
    return int(load_library().gst_required_scratch(ctypes.byref(hdr)))


def preallocate_decompressor(ctx: GPUContext, req_sz: int) -> None:
    """codec/decoder.cpp:478-481."""
    _check(load_library().gst_preallocate(ctx.handle, req_sz), "gst_preallocate")


def free_decompressor(ctx: GPUContext) -> None:
    """codec/decoder.cpp:483-485."""
    _check(load_library().gst_free_decompressor(ctx.handle), "gst_free_decompressor")


def batch_layout_bytes(hdrs: Sequence[GenTCHeader]) -> int:
    arr = (GenTCHeader * len(hdrs))(*hdrs)
    return int(load_library().gst_batch_layout_bytes(arr, len(hdrs)))


def pack_batch(streams: Iterable[bytes]) -> tuple[list[GenTCHeader], np.ndarray]:
    """Writes the reference's device layout for a batch of complete GST streams
    (offsets page, 4N frequency tables, sections; demo/photos_sf.cpp:753-791)."""
    bufs = [_as_bytes(s) for s in streams]
    hdrs = [parse_header(b) for b in bufs]
    n = len(bufs)
    out = np.zeros(batch_layout_bytes(hdrs), dtype=np.uint8)
    keep = [ctypes.create_string_buffer(b, len(b)) for b in bufs]
    ptrs = (ctypes.c_void_p * n)(*[ctypes.addressof(k) for k in keep])
    lens = (ctypes.c_size_t * n)(*[len(b) for b in bufs])
    _check(load_library().gst_pack_batch(ptrs, lens, n, out.ctypes.data, out.nbytes), "gst_pack_batch")
    return hdrs, out


def blocks_u64(dxt_bytes: np.ndarray) -> np.ndarray:
    """View DXT1 output bytes as one u64 per block (PhysicalDXTBlock::dxt_block)."""
    return np.ascontiguousarray(dxt_bytes).view(np.uint64)


def size_class(blocks: int) -> int:
    """gst_size_class: the size class of a launch of `blocks` DXT1 blocks."""
    return int(load_library().gst_size_class(blocks))


def set_class_tuning(ctx: GPUContext, size_class_index: int, blocks_per_sm: int, stage_words: int,
                     persistent: int = 0) -> None:
    _check(load_library().gst_set_class_tuning(ctx.handle, size_class_index, blocks_per_sm, stage_words, persistent),
           "gst_set_class_tuning")


def save_class_tuning(ctx: GPUContext, path) -> None:
    """gst_save_class_tuning: the classes that are set, as a JSON table."""
    _check(load_library().gst_save_class_tuning(ctx.handle, str(path).encode()), "gst_save_class_tuning")


def load_class_tuning(ctx: GPUContext, path) -> None:
    """gst_load_class_tuning: replaces the context's class table with the file's."""
    _check(load_library().gst_load_class_tuning(ctx.handle, str(path).encode()), "gst_load_class_tuning")


def get_class_tuning(ctx: GPUContext, size_class_index: int) -> tuple[int, int, int]:
    """gst_get_class_tuning -> (blocks_per_sm, stage_words, persistent)."""
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(load_library().gst_get_class_tuning(ctx.handle, size_class_index, ctypes.byref(a), ctypes.byref(b),
                                               ctypes.byref(c)), "gst_get_class_tuning")
    return a.value, b.value, c.value


def autotune_class(ctx: GPUContext, hdrs: Sequence[GenTCHeader], cmp_data, output, stream=None,
                   iterations: int = 3) -> int:
    """gst_autotune_class: tunes on a representative batch; returns its size class."""
    arr = (GenTCHeader * len(hdrs))(*hdrs)
    c = ctypes.c_int(-1)
    _check(load_library().gst_autotune_class(ctx.handle, arr, len(hdrs), _ptr(cmp_data), _ptr(output),
                                             _stream(stream), int(iterations), ctypes.byref(c)),
           "gst_autotune_class")
    return c.value
