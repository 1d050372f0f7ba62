"""Build libneuronephys.so (CUDA kernels + C ABI) for sm_103a with nvcc.

The translation units are compiled in parallel into ``_build/`` and linked
into ``neuronephys_clean_gb300/lib/libneuronephys.so``.  A rebuild happens
only when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = ROOT / "_build"
LIB = PKG / "lib" / "libneuronephys.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")

SOURCES = ["nn_api.cu", "nn_ref.cu", "nn_pcg.cu", "nn_cg.cu", "nn_sim.cu", "nn_conv.cu", "nn_unet.cu", "nn_probe.cu", "nn_io.cu", "nn_bpcg.cu", "nn_cortex.cu", "nn_mg.cu",
           "nn_step.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
          "-I", str(INCLUDE), "-I", str(CSRC)]


def _deps() -> list[Path]:
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def lib_path() -> Path:
    return LIB


def needs_build() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not needs_build():
        return LIB
    BUILD.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)

    def compile_one(src: str) -> str:
        obj = BUILD / (Path(src).stem + ".o")
        _run([NVCC, *ARCH, *CFLAGS, "-c", str(CSRC / src), "-o", str(obj)])
        return str(obj)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    _run([NVCC, *ARCH, "-shared", "-o", str(tmp), *objs])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
