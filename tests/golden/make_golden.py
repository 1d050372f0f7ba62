"""Regenerate the golden vectors of the reference's own connectivity code.

Builds ``oracle/_ref/ref_netgen`` from the reference sources (see
``oracle/build.py``), runs it, and stores its outputs:

* ``ref_netgen_A.npz`` -- full arrays of the hh_benchmark pattern at N=1000
  (UniformRandomNetwork(8) then (2) from the shared unseeded engine, their CSR
  and in-degree Tcount).
* ``ref_netgen_B.json`` -- SHA-256 digests (and array lengths) of the chunked
  adjacency list at N = NCHUNKS * N_PER_CHUNK = 14638 with Ncouple = 3.

Run from the repository root: ``python tests/golden/make_golden.py``.
This needs the reference checkout; the committed outputs are what the tests
read.
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.build import build_ref  # noqa: E402

HERE = Path(__file__).resolve().parent


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    exe = build_ref(force=True)
    if exe is None:
        raise SystemExit("reference checkout not found")
    with tempfile.TemporaryDirectory() as td:
        subprocess.run([str(exe), td], check=True, capture_output=True)
        t = Path(td)
        rd = lambda name, dt: np.fromfile(t / name, dtype=dt)  # noqa: E731
        np.savez_compressed(
            HERE / "ref_netgen_A.npz",
            e_indices=rd("A_e_indices.i32", np.int32),
            e_offsets=rd("A_e_offsets.i32", np.int32),
            e_tcount=rd("A_e_tcount.f32", np.float32),
            i_indices=rd("A_i_indices.i32", np.int32),
            i_offsets=rd("A_i_offsets.i32", np.int32),
            i_tcount=rd("A_i_tcount.f32", np.float32),
        )
        b = {}
        for name, dt in [("B_indices.i32", np.int32), ("B_offsets.i32", np.int32),
                         ("B_tcount.f32", np.float32),
                         ("B_chunk0_indices.i32", np.int32), ("B_chunk0_offsets.i32", np.int32),
                         ("B_chunk1_indices.i32", np.int32), ("B_chunk1_offsets.i32", np.int32)]:
            a = rd(name, dt)
            b[name] = {"len": int(a.size), "sha256": sha(a), "head": a[:16].tolist()}
        (HERE / "ref_netgen_B.json").write_text(json.dumps(b, indent=1) + "\n")
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
