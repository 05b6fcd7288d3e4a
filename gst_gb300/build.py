"""Builds the native parts in-tree.

* ``gst_gb300/libgst_gb300.so`` -- the CUDA decoder (sm_103a kernels + C ABI),
  compiled by nvcc with ``-gencode arch=compute_103a,code=sm_103a``.
* ``gst_gb300/libgst_encoder.so`` -- the host-side GST stream producer.

Both are plain shared libraries loaded with ctypes; nothing links PyTorch.
The builds run in parallel and are skipped when the library is newer than its
sources.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]

DECODER_LIB = PKG / "libgst_gb300.so"
ENCODER_LIB = PKG / "libgst_encoder.so"

DECODER_SOURCES = [CSRC / "gst_kernels.cu", CSRC / "gst_encode.cu", CSRC / "gst_prepare.cu", CSRC / "gst_reencode.cu",
                   CSRC / "gst_api.cpp",
                   CSRC / "gst_encode_api.cpp", CSRC / "gst_server.cpp"]
DECODER_HEADERS = [CSRC / "gst_plan.h", CSRC / "gst_encode_plan.h", CSRC / "gst_host.h", INCLUDE / "gst_decoder.h",
                   INCLUDE / "gst_encode.h"]
ENCODER_SOURCES = [CSRC / "gst_encoder.cpp"]
ENCODER_HEADERS = [CSRC / "gst_encoder.h"]
OBJ_DIR = PKG / "_build"


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build gst_gb300")
    return cand


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def compile_cmd(src: Path) -> list[str]:
    """nvcc command that compiles one source of the decoder library to an object."""
    return [
        nvcc_path(), *ARCH_FLAGS, "-lineinfo", "-O3", "-std=c++17",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread",
        f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(OBJ_DIR / (src.name + ".o")),
    ]


def decoder_cmd() -> list[str]:
    return compile_cmd(DECODER_SOURCES[0])


def link_cmd() -> list[str]:
    return [nvcc_path(), *ARCH_FLAGS, "-shared", *(str(OBJ_DIR / (s.name + ".o")) for s in DECODER_SOURCES),
            "-o", str(DECODER_LIB), "-lpthread"]


def encoder_cmd() -> list[str]:
    return [
        os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off",
        "-shared", "-fPIC", "-pthread",
        *map(str, ENCODER_SOURCES), "-o", str(ENCODER_LIB),
    ]


def _run_parallel(jobs, verbose: bool) -> None:
    procs = []
    for name, cmd in jobs:
        if verbose:
            print("[gst_gb300 build]", " ".join(cmd))
        procs.append((name, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for name, cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"{name} build failed ({' '.join(cmd)}):\n{out.decode(errors='replace')}")
    if errors:
        raise RuntimeError("\n".join(errors))


def build_all(force: bool = False, verbose: bool = False) -> None:
    """Compiles the decoder library's sources in parallel (with the host
    encoder library), then links the decoder library."""
    OBJ_DIR.mkdir(exist_ok=True)
    jobs = []
    for src in DECODER_SOURCES:
        if force or _stale(OBJ_DIR / (src.name + ".o"), [src] + DECODER_HEADERS):
            jobs.append((src.name, compile_cmd(src)))
    if force or _stale(ENCODER_LIB, ENCODER_SOURCES + ENCODER_HEADERS):
        jobs.append(("encoder", encoder_cmd()))
    _run_parallel(jobs, verbose)
    objs = [OBJ_DIR / (s.name + ".o") for s in DECODER_SOURCES]
    if force or _stale(DECODER_LIB, objs):
        _run_parallel([("link", link_cmd())], verbose)


if __name__ == "__main__":
    build_all(force=True, verbose=True)
