"""gst_gb300 -- GST (GPU-decodable Supercompressed Textures) decoding on GB300.

GST stream -> DXT1 blocks with hand-written sm_103a kernels behind a C ABI
(include/gst_decoder.h).  ``decoder`` mirrors the reference's GenTC decoder
API; ``encoder`` and ``workloads`` make inputs; ``serving`` runs the
continuous-batching loop.
"""
from .decoder import (  # noqa: F401
    GenTCHeader, GPUContext, GstError, decompress_dxt, free_decompressor, initialize_decoder,
    load_compressed_dxt, load_compressed_dxts, pack_batch, parse_header, preallocate_decompressor,
    required_scratch_mem, sync_status,
)
