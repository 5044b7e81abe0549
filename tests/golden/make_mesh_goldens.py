"""Generate tests/golden/mesh_25km_NH.json from the reference's mesh fixture.

The reference's ParametricMesh test (dynamics/test/ParametricMesh_test.cpp)
reads dynamics/test/25km_NH.smesh, a 154 x 121 grid of 25 km cells over the
Arctic with a land mask and the closed (Dirichlet) element sides listed in
the file, and checks that the lists derived from the mask
(ParametricMesh::dirichletFromMask + dirichletFromEdge + sortDirichlet,
dynamics/src/ParametricMesh.cpp:228-272) equal the file's.  This script keeps
what that check needs: the grid size and spacing, the mask (packed bits, row
0 first, element index i + nx*j) and the file's four Dirichlet lists.

The smesh format (ParametricMesh::readmesh, ParametricMesh.cpp:8-175):
"ParametricMesh 2.0", nx ny, (nx+1)(ny+1) vertex pairs, "landmask" ne and ne
flags, "dirichlet" nd and nd pairs (element, side), "periodic" np ...

Run from the repository root, where the reference tree is readable:
    python tests/golden/make_mesh_goldens.py [path/to/25km_NH.smesh]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

MESH = "dynamics/test/25km_NH.smesh"  # within the reference source tree
OUT = Path(__file__).resolve().parent / "mesh_25km_NH.json"


def parse_smesh(path: str) -> dict:
    tok = Path(path).read_text().split()
    if tok[0] != "ParametricMesh" or tok[1] != "2.0":
        raise ValueError("not a ParametricMesh 2.0 file")
    nx, ny = int(tok[2]), int(tok[3])
    i = 4
    nn = (nx + 1) * (ny + 1)
    v = np.array(tok[i:i + 2 * nn], dtype=np.float64).reshape(nn, 2)
    i += 2 * nn
    if tok[i] != "landmask":
        raise ValueError("landmask section expected")
    ne = int(tok[i + 1])
    i += 2
    if ne != nx * ny:
        raise ValueError("landmask size")
    mask = np.array(tok[i:i + ne], dtype=np.int64)
    i += ne
    if tok[i] != "dirichlet":
        raise ValueError("dirichlet section expected")
    nd = int(tok[i + 1])
    i += 2
    dirichlet: list[list[int]] = [[], [], [], []]
    for k in range(nd):
        dirichlet[int(tok[i + 2 * k + 1])].append(int(tok[i + 2 * k]))
    i += 2 * nd
    if tok[i] != "periodic":
        raise ValueError("periodic section expected")
    return dict(nx=nx, ny=ny, vertices=v, mask=mask, dirichlet=dirichlet, periodic=int(tok[i + 1]))


def _default_path() -> str:
    """$NSDG_REFERENCE, else the location the oracle build recipe uses."""
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent.parent))
    from oracle import pyref
    root = pyref.reference_root()
    if root is None:
        sys.exit("give the .smesh path as the argument or the reference source tree in NSDG_REFERENCE")
    return str(root / MESH)


def main(path: str | None = None) -> None:
    path = path or _default_path()
    m = parse_smesh(path)
    nx, ny, v = m["nx"], m["ny"], m["vertices"]
    dx, dy = float(v[1, 0] - v[0, 0]), float(v[nx + 1, 1] - v[0, 1])
    ix, iy = np.arange(v.shape[0]) % (nx + 1), np.arange(v.shape[0]) // (nx + 1)
    uniform = bool(np.array_equal(v[:, 0], ix * dx) and np.array_equal(v[:, 1], iy * dy))
    if not uniform:
        raise ValueError("the fixture's grid is expected to be uniform")
    out = {
        "source": "dynamics/test/25km_NH.smesh (read by dynamics/test/ParametricMesh_test.cpp)",
        "nx": nx, "ny": ny, "dx": dx, "dy": dy, "uniform_grid": uniform,
        "mask_bits_hex": np.packbits(m["mask"].astype(np.uint8)).tobytes().hex(),
        "mask_ice_count": int(m["mask"].sum()),
        "dirichlet": m["dirichlet"],
        "periodic_segments": m["periodic"],
    }
    OUT.write_text(json.dumps(out, separators=(",", ":")) + "\n")
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main(*sys.argv[1:])
