"""Build recipe for the test oracle (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``oracle.c`` into
  ``oracle/liboracle.so`` (gcc, OpenMP, no FP contraction).
* ``build_ref()`` compiles the reference's own host-side connectivity code
  (``src/network_factory.cu`` and ``src/defines.cu``, read where they lie in
  the reference checkout) together with the include shims in
  ``oracle/refshim/`` into ``oracle/_ref/ref_netgen``.  It needs the reference
  checkout (``NN_REFERENCE_ROOT``, default the mounted reference path) and is a
  no-op when that is absent (e.g. on the GPU machine, which only uses the
  committed golden vectors).

Nothing in the product package imports this module.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_ROOT = Path(os.environ.get("NN_REFERENCE_ROOT", "/root/reference"))
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def oracle_lib_path() -> Path:
    return HERE / "liboracle.so"


def build_oracle(force: bool = False) -> Path:
    out = oracle_lib_path()
    src = [HERE / "oracle.c", HERE / "oracle.h"]
    if not force and out.exists() and all(out.stat().st_mtime >= s.stat().st_mtime for s in src):
        return out
    tmp = out.with_suffix(".so.tmp")
    _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
          str(HERE / "oracle.c"), "-o", str(tmp), "-lm"])
    os.replace(tmp, out)
    return out


def ref_netgen_path() -> Path:
    return HERE / "_ref" / "ref_netgen"


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference's network factory (host code) as an oracle."""
    src_dir = REF_ROOT / "src"
    if not (src_dir / "network_factory.cu").exists():
        return None
    out = ref_netgen_path()
    if out.exists() and not force:
        return out
    outdir = out.parent
    outdir.mkdir(parents=True, exist_ok=True)
    flags = ["-std=c++17", "-O1", "-w",
             "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP",
             "-I", str(HERE / "refshim"),
             "-I", str(CUDA_HOME / "include" / "cccl"),
             "-I", str(CUDA_HOME / "include"),
             "-I", str(REF_ROOT / "ann" / "include"),
             "-I", str(src_dir)]
    objs = []
    for name, path in [("network_factory", src_dir / "network_factory.cu"),
                       ("defines", src_dir / "defines.cu"),
                       ("host_stubs", HERE / "refshim" / "host_stubs.cpp"),
                       ("ref_netgen", HERE / "refshim" / "ref_netgen.cpp")]:
        obj = outdir / f"{name}.o"
        _run(["g++", *flags, "-x", "c++", "-c", str(path), "-o", str(obj)])
        objs.append(str(obj))
    _run(["g++", *objs, "-o", str(out)])
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
