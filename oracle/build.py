"""Build recipe for the test oracle (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``oracle.c`` into
  ``oracle/liboracle.so`` (gcc, OpenMP, no FP contraction).
* ``build_ref()`` compiles the reference's own host-side connectivity code
  (``src/network_factory.cu`` and ``src/defines.cu``, read where they lie in
  the reference checkout) together with the include shims in
  ``oracle/refshim/`` into ``oracle/_ref/ref_netgen``.
* ``build_ref_kernels()`` compiles the reference's own CUDA kernels
  (``src/ephys.cu``: ``Leapfrog_HH``, ``init_random``; ``src/coupling.cu``:
  ``signal_spikes_kernel``, ``signal_spikes_kernel_chunked``,
  ``merge_kernel``; and the whole-brain ``src_wholebrain/ephys.cu`` and
  ``src_wholebrain/coupling.cu``) for sm_103a into device-only cubins
  ``oracle/_ref/ref_{ephys,coupling,wb_ephys,wb_coupling}.cubin``.  The
  only shims are the HDF5 stub above and ``thrust::identity``, which CCCL 3
  removed (used by ``src/coupling.cu:125,160``).  A cubin carries no host code,
  so the files built here also run on a GPU host of another architecture.
* ``build_refkern()`` compiles ``refkern.c``, the driver-API harness that
  loads those cubins and launches the kernels as the reference's host code
  does, into ``oracle/librefkern.so``.

The two reference builds need the reference checkout: ``NN_REFERENCE_ROOT``,
or else a directory ``reference`` beside the repository.  They are no-ops
where it is absent (a GPU host, which uses the files built where the checkout
is and the committed golden vectors).

Nothing in the product package imports this module.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_ROOT = Path(os.environ.get("NN_REFERENCE_ROOT", str(HERE.parent.parent / "reference")))
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


# cubin name -> (reference directory, source file)
REF_KERNEL_SOURCES = {"ephys": ("src", "ephys.cu"), "coupling": ("src", "coupling.cu"),
                      "wb_ephys": ("src_wholebrain", "ephys.cu"), "wb_coupling": ("src_wholebrain", "coupling.cu")}


def ref_cubin_path(name: str) -> Path:
    return HERE / "_ref" / f"ref_{name}.cubin"


def build_ref_kernels(force: bool = False) -> list[Path] | None:
    """Compile the reference's ephys and coupling kernels into cubins."""
    srcs = {name: REF_ROOT / d / f for name, (d, f) in REF_KERNEL_SOURCES.items()}
    if not all(p.exists() for p in srcs.values()):
        return None
    outs = [ref_cubin_path(n) for n in srcs]
    if not force and all(o.exists() for o in outs):
        return outs
    outs[0].parent.mkdir(parents=True, exist_ok=True)
    for (name, src), out in zip(srcs.items(), outs):
        tmp = out.with_suffix(".cubin.tmp")
        _run([str(CUDA_HOME / "bin" / "nvcc"), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
              "-std=c++17", "--expt-extended-lambda", "-w",
              "-I", str(HERE / "refshim"), "-I", str(src.parent),
              "-include", str(HERE / "refshim" / "thrust_identity.h"),
              str(src), "-o", str(tmp)])
        os.replace(tmp, out)
    return outs


def refkern_lib_path() -> Path:
    return HERE / "librefkern.so"


def build_refkern(force: bool = False) -> Path:
    """Compile the driver-API harness of the reference kernels."""
    out = refkern_lib_path()
    src = HERE / "refkern.c"
    if not force and out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    tmp = out.with_suffix(".so.tmp")
    _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fvisibility=hidden", str(src),
          "-I", str(CUDA_HOME / "include"), "-L", str(CUDA_HOME / "lib64" / "stubs"), "-lcuda", "-o", str(tmp)])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
    print(build_ref_kernels(force=True))
    print(build_refkern(force=True))
