"""nsdg_mean_value_noalloc: the FP64 mesh integral (Tools::MeanValue) for
callers that cannot allocate device memory.

Such callers — a host model whose own pool allocator owns the GPU memory, or a
time-critical loop that may not pay cudaMalloc's implicit synchronisation —
pass device pointers to the field and the quadrature weights and get the
integral written to a device pointer; the reduction's scratch is a fixed
file-scope device array inside the library.  The test checks it against the
allocating entry point (nsdg_transport_mean_value) on two calls in a row,
with different fields, so a stale scratch would show, and directly against
the CPU oracle's MeanValue of the same field on the same mesh.  This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jacobian_weights(verts, nx, ny):
    """J*w at the 3x3 Gauss points of each element, SoA [9][N] (bilinear map)."""
    g = 0.5 + np.array([-np.sqrt(3 / 20), 0.0, np.sqrt(3 / 20)])
    w1 = np.array([5 / 18, 8 / 18, 5 / 18])
    V = verts.reshape(ny + 1, nx + 1, 2)
    c00, c10 = V[:-1, :-1].reshape(-1, 2), V[:-1, 1:].reshape(-1, 2)
    c01, c11 = V[1:, :-1].reshape(-1, 2), V[1:, 1:].reshape(-1, 2)
    out = np.empty((9, nx * ny))
    for q in range(9):
        x, y = g[q % 3], g[q // 3]
        dxi = (c10 - c00) * (1 - y) + (c11 - c01) * y
        deta = (c01 - c00) * (1 - x) + (c11 - c10) * x
        J = dxi[:, 0] * deta[:, 1] - dxi[:, 1] * deta[:, 0]
        out[q] = J * (w1[q % 3] * w1[q // 3])
    return out


def test_noalloc_mean_value_matches_allocating_entry_point(gpu, oracle):
    torch = pytest.importorskip("torch")
    from nextsimdg_gb300.dynamics import DGTransport

    lib = gpu
    fn = lib.nsdg_mean_value_noalloc
    nx, ny, dg = 300, 211, 6
    verts, dirichlet, _ = oracle.rectangle_mesh(4.0e5, 3.0e5, nx, ny, 0.03)
    t = DGTransport(dg, nx, ny, verts, dirichlet, [])
    jw = torch.tensor(_jacobian_weights(verts, nx, ny), dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(7)
    fields = [rng.standard_normal((nx * ny, dg)), 2.0 + rng.random((nx * ny, dg))]
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    dev_fields = [torch.tensor(f.T.copy(), dtype=torch.float64, device="cuda") for f in fields]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for i, d in enumerate(dev_fields):  # two calls in a row, sharing the scratch
        st = fn(dg, nx * ny, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(jw.data_ptr()),
                ctypes.c_void_p(out.data_ptr() + 8 * i), stream)
        assert st == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    o = oracle.OracleTransport(dg, nx, ny, verts, dirichlet)
    for i, f in enumerate(fields):
        want = t.meanValue(f)
        assert got[i] == pytest.approx(want, rel=1e-12, abs=1e-12 * abs(want) + 1e-300)
        # the oracle's Tools::MeanValue (Tools.hpp:24-50) of the same field
        want_oracle = o.meanValue(f)
        assert got[i] == pytest.approx(want_oracle, rel=1e-12, abs=1e-12 * abs(want_oracle) + 1e-300)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    too_big = (1 << 24) + 1
    assert lib.nsdg_mean_value_noalloc(6, too_big, p, p, p, None) == 3  # NSDG_ERR_SIZE_MISMATCH
    assert lib.nsdg_mean_value_noalloc(5, 10, p, p, p, None) == 1       # NSDG_ERR_BAD_ARG
