"""The C ABI library: it loads, exports every symbol include/gst_decoder.h and
include/gst_encode.h declare, and its host-side logic (stream validation, batch layout, error
reporting without a GPU) behaves as documented.  No kernel runs here."""
import ctypes
import re

import numpy as np
import pytest

from conftest import ROOT, golden_stream
from gst_gb300 import decoder
from gst_gb300.decoder import GST_E_ARG, GST_E_CUDA, GST_E_FORMAT, GST_OK


def header_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        names |= set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(gst_\w+)\s*\(", h.read_text(), re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = decoder.load_library()
    names = header_functions()
    assert len(names) >= 16
    assert set(names) == set(decoder.EXPORTED_SYMBOLS)
    for n in names:
        assert hasattr(lib, n), n


def test_build_targets_sm103a_only():
    from gst_gb300 import build
    cmd = build.decoder_cmd()
    assert "arch=compute_103a,code=sm_103a" in cmd and cmd.count("-gencode") == 1


@pytest.mark.parametrize("name", ["test1.gst", "synth512_s0.gst", "synth768x512_s3.gst"])
def test_parse_header_accepts_golden(name):
    s = golden_stream(name)
    h = decoder.parse_header(s)
    assert h.width * h.height // 2 == h.dxt_bytes
    assert 28 + 2048 + h.compressed_bytes == len(s)


def mutate(s: bytes, off: int, val: int, width: int = 4) -> bytes:
    b = bytearray(s)
    b[off:off + width] = val.to_bytes(width, "little")
    return bytes(b)


def test_parse_header_rejects_malformed():
    s = golden_stream("test1.gst")
    cases = {
        "truncated": s[:-4],
        "empty": b"",
        "width": mutate(s, 0, 500),
        "height_zero": mutate(s, 4, 0),
        "area": mutate(mutate(s, 0, 384), 4, 128),  # 384*128 not a multiple of 131072
        "palette_zero": mutate(s, 8, 0),
        "palette_unaligned": mutate(s, 8, 8196),
        "section_unaligned": mutate(s, 12, int.from_bytes(s[12:16], "little") + 2),
        "table_sum": mutate(s, 28, int.from_bytes(s[28:30], "little") + 1, 2),
        "group_end_small": mutate(s, 28 + 2048, 3),
        "group_end_past_section": mutate(s, 28 + 2048, 1 << 30),
    }
    for why, bad in cases.items():
        with pytest.raises(decoder.GstError) as e:
            decoder.parse_header(bad)
        assert e.value.status == GST_E_FORMAT, why


def test_pack_batch_layout():
    # demo/photos_sf.cpp:753-791: offsets page, 4N tables, sections.
    streams = [golden_stream("test1.gst"), golden_stream("synth768x512_s3.gst")]
    hdrs, buf = decoder.pack_batch(streams)
    assert buf.size == decoder.batch_layout_bytes(hdrs)
    page = 512
    offs = buf[:page].view(np.uint32)
    B0 = 512 * 512 // 16
    B1 = 768 * 512 // 16
    assert offs[:4].tolist() == [0, 2 * B0, 6 * B0, 6 * B0 + hdrs[0].palette_bytes]
    assert offs[4] == 7 * B0 + hdrs[0].palette_bytes
    assert offs[8:12].tolist()[0] == 0 and offs[9] == hdrs[0].y_cmp_sz
    assert offs[12] == hdrs[0].compressed_bytes
    assert bytes(buf[page:page + 2048]) == streams[0][28:28 + 2048]
    assert bytes(buf[page + 2048:page + 4096]) == streams[1][28:28 + 2048]
    body = page + 4096
    assert bytes(buf[body:body + hdrs[0].compressed_bytes]) == streams[0][28 + 2048:]
    assert bytes(buf[body + hdrs[0].compressed_bytes:]) == streams[1][28 + 2048:]
    del B1


def test_required_scratch_positive_and_monotone():
    h = decoder.parse_header(golden_stream("test1.gst"))
    small = decoder.required_scratch_mem(h)
    h2 = decoder.GenTCHeader(*h.as_tuple())
    h2.width *= 2
    h2.y_cmp_sz *= 2
    h2.chroma_cmp_sz *= 2
    h2.indices_sz *= 2
    assert small >= 7 * 16384 + h.palette_bytes
    assert decoder.required_scratch_mem(h2) > small
    bad = decoder.GenTCHeader(*h.as_tuple())
    bad.width = 100
    assert decoder.required_scratch_mem(bad) == 0


def test_init_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = decoder.load_library()
    h = ctypes.c_void_p()
    assert lib.gst_init(0, ctypes.byref(h)) == GST_E_CUDA
    assert lib.gst_load_compressed_dxts(None, None, 0, None, None, None) == GST_E_ARG
    assert lib.gst_decompress_dxt(None, None, 0, None, 0) == GST_E_ARG
    assert lib.gst_batch_rans_items(None) == 0 and lib.gst_batch_device_bytes(None) == 0
    assert lib.gst_status_string(GST_OK) == b"ok"


def test_size_classes():
    # class 0 up to 2^14 blocks (one 512x512 image), each class 4x larger, 7 classes
    cases = {1: 0, 1 << 14: 0, (1 << 14) + 1: 1, 1 << 16: 1, 1 << 18: 2, (1 << 18) + 1: 3, 1 << 20: 3,
             1 << 22: 4, 1 << 24: 5, 1 << 26: 6, 1 << 40: 6}
    for blocks, c in cases.items():
        assert decoder.size_class(blocks) == c, blocks
