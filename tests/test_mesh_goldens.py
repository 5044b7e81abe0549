"""Closed (Dirichlet) element sides derived from a land mask, pinned on the
reference's 25 km Arctic mesh (dynamics/test/25km_NH.smesh as
dynamics/test/ParametricMesh_test.cpp reads it; fixture made by
tests/golden/make_mesh_goldens.py).

The reference test checks that ParametricMesh::dirichletFromMask +
dirichletFromEdge + sortDirichlet on the file's mask give exactly the lists
stored in the file.  Here: the fixture against that test's own known answers,
then the oracle's and the library's mask-derived lists against the stored
lists (exact), and the two against each other on seeded random masks."""
import json
from pathlib import Path

import numpy as np
import pytest

from nextsimdg_gb300._lib import NSDG_ERR_SIZE_MISMATCH

GOLDEN = Path(__file__).resolve().parent / "golden" / "mesh_25km_NH.json"


@pytest.fixture(scope="module")
def mesh():
    g = json.loads(GOLDEN.read_text())
    n = g["nx"] * g["ny"]
    bits = np.unpackbits(np.frombuffer(bytes.fromhex(g["mask_bits_hex"]), dtype=np.uint8))[:n]
    g["mask"] = bits.astype(np.float64)
    return g


def test_fixture_matches_the_reference_known_answers(mesh):
    """ParametricMesh_test.cpp:30-33 (sizes, spacing), 45-84 (mask values,
    first closed elements, list lengths, no periodic segments)."""
    nx, ny = mesh["nx"], mesh["ny"]
    assert (nx, ny) == (154, 121)
    assert mesh["dx"] == 25000.0 and mesh["dy"] == 25000.0 and mesh["uniform_grid"]
    lm = mesh["mask"]
    assert int(lm.sum()) == mesh["mask_ice_count"]
    assert not lm[0] and not lm[4] and lm[5] and lm[nx - 1] and not lm[(ny - 1) * nx]
    d = mesh["dirichlet"]
    assert d[0][0] == 5 and d[3][0] == 5  # element 5 closed on sides 0 and 3
    assert d[1][0] == 7 and d[2][0] == 48
    assert [len(x) for x in d] == [369, 384, 369, 384]
    assert mesh["periodic_segments"] == 0
    assert all(x == sorted(x) for x in d)


def test_oracle_dirichlet_from_mask_equals_the_file(mesh, oracle):
    got = oracle.mesh_dirichlet(mesh["nx"], mesh["ny"], mesh["mask"])
    for s in range(4):
        np.testing.assert_array_equal(got[s], mesh["dirichlet"][s], err_msg=f"side {s}")


def test_library_dirichlet_from_mask_equals_the_file(mesh, nsdg_lib):
    from nextsimdg_gb300.dynamics import mesh_dirichlet
    got = mesh_dirichlet(mesh["mask"], mesh["nx"], mesh["ny"])
    for s in range(4):
        np.testing.assert_array_equal(got[s], mesh["dirichlet"][s], err_msg=f"side {s}")


@pytest.mark.parametrize("seed,nx,ny,p", [(0, 1, 1, 1.0), (1, 7, 5, 0.7), (2, 16, 16, 0.9), (3, 33, 9, 0.5),
                                          (4, 5, 40, 0.97), (5, 12, 12, 0.0)])
def test_library_and_oracle_agree_on_random_masks(oracle, nsdg_lib, seed, nx, ny, p):
    """Ragged masks, single rows and columns, all land and all ice; values
    other than 0 and 1 count as land (the mask == 1.0 rule of
    ParametricMesh::landmaskFromModelArray)."""
    from nextsimdg_gb300.dynamics import mesh_dirichlet
    rng = np.random.default_rng(seed)
    mask = (rng.random(nx * ny) < p).astype(np.float64)
    mask[rng.random(nx * ny) < 0.05] = 0.5
    a = mesh_dirichlet(mask, nx, ny)
    b = oracle.mesh_dirichlet(nx, ny, mask)
    for s in range(4):
        np.testing.assert_array_equal(a[s], b[s], err_msg=f"side {s}")


def test_library_reports_short_capacity(nsdg_lib):
    from ctypes import c_size_t
    counts = (c_size_t * 4)()
    ids = np.empty(3, dtype=np.uint64)
    mask = np.ones(4)
    st = nsdg_lib.nsdg_mesh_dirichlet(2, 2, mask.ctypes.data, counts, ids.ctypes.data, ids.size)
    assert st == NSDG_ERR_SIZE_MISMATCH
    assert list(counts) == [2, 2, 2, 2]
    from nextsimdg_gb300.dynamics import mesh_dirichlet
    with pytest.raises(ValueError):
        mesh_dirichlet(np.ones(3), 2, 2)
