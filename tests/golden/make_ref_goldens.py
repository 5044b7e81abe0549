#!/usr/bin/env python3
"""Writes tests/golden/ref_dynamics.npz: the read-outs of the cases in
ref_cases.py computed by the reference's own dynamics code.

The reference build (oracle/_ref/libnsdg_ref.so) is made by
`make -C oracle ref REF=<reference source tree>` from the reference's
unmodified sources and the project's Eigen subset; this script builds it
first when the reference sources are found ($NSDG_REFERENCE or the recipe's
default), then runs every case and stores its read-outs, with the case
definitions, in one compressed file.  It runs the reference single-threaded
(see OMP_NUM_THREADS below).

    NSDG_REFERENCE=<reference source tree> python tests/golden/make_ref_goldens.py
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

# One OpenMP thread: the reference's SSH gradient (CGDynamicsKernel.cpp:211-219)
# advances a counter shared by the threads of a parallel loop, so with more
# than one thread its CG2 node values (and every result of a case with a
# non-zero sea-surface height) vary from run to run; single-threaded they are
# deterministic.  The other cases are the same with any thread count.
os.environ["OMP_NUM_THREADS"] = "1"

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

from oracle import pyref  # noqa: E402
import ref_cases  # noqa: E402

OUT = HERE / "ref_dynamics.npz"


def main() -> None:
    if pyref.build() is None or not pyref.available():
        sys.exit("the reference build is missing and the reference sources were not found "
                 "(set NSDG_REFERENCE)")
    arrays = {}
    for name, case in ref_cases.CASES.items():
        t0 = time.time()
        k = pyref.RefKernel(case["rheology"], case["dg"], case["alpha"], ref_cases.beta(case), case["sub"])
        ref_cases.run(k, case)
        for key, a in ref_cases.readouts(k, case).items():
            arrays[f"{name}/{key}"] = np.asarray(a, dtype=np.float64)
        k.close()
        print(f"{name}: {time.time() - t0:.1f} s", flush=True)
    arrays["cases"] = np.array(json.dumps(ref_cases.CASES))
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
