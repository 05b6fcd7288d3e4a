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

DECODER_SOURCES = [CSRC / "gst_kernels.cu", CSRC / "gst_api.cpp", CSRC / "gst_server.cpp"]
DECODER_HEADERS = [CSRC / "gst_plan.h", CSRC / "gst_host.h", INCLUDE / "gst_decoder.h"]
ENCODER_SOURCES = [CSRC / "gst_encoder.cpp"]
ENCODER_HEADERS = [CSRC / "gst_encoder.h"]


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


def decoder_cmd() -> list[str]:
    return [
        nvcc_path(), *ARCH_FLAGS, "-lineinfo", "-O3", "-std=c++17",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread", "-shared",
        f"-I{INCLUDE}", f"-I{CSRC}",
        *map(str, DECODER_SOURCES), "-o", str(DECODER_LIB), "-lpthread",
    ]


def encoder_cmd() -> list[str]:
    return [
        os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off",
        "-shared", "-fPIC", "-pthread",
        *map(str, ENCODER_SOURCES), "-o", str(ENCODER_LIB),
    ]


def build_all(force: bool = False, verbose: bool = False) -> None:
    jobs = []
    if force or _stale(DECODER_LIB, DECODER_SOURCES + DECODER_HEADERS):
        jobs.append(("decoder", decoder_cmd()))
    if force or _stale(ENCODER_LIB, ENCODER_SOURCES + ENCODER_HEADERS):
        jobs.append(("encoder", encoder_cmd()))
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


if __name__ == "__main__":
    build_all(force=True, verbose=True)
