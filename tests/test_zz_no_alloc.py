"""plb_conservation_static: the conservation sums for callers that cannot
allocate device memory (an application that owns all device memory up front,
a process under a hard memory quota, an allocator that must see every
allocation).  It works on the caller's own device arrays and keeps its block
partials in a fixed array inside the library, so it allocates nothing.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.  The checks compare the new
entry point with the existing plb_conservation on the same state, within the
tolerance the other conservation tests use, on two calls in a row."""
import numpy as np
import pytest

from cases import CASES

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-12, 1e-13


def _static_sums(torch, lib, q, n_interior, solid, pad=37):
    """Copies the interior populations into a device array with q planes
    (plane stride ncells + pad) and runs the static entry point twice."""
    nz, ny, nx, _ = n_interior.shape
    ncells = nz * ny * nx
    plane = ncells + pad
    flat = np.zeros((q, plane), np.float32)
    flat[:, :ncells] = n_interior.reshape(ncells, q).T
    dev = torch.from_numpy(flat).to("cuda")
    sol = torch.from_numpy(np.ascontiguousarray(solid.reshape(-1).astype(np.uint8))).to("cuda")
    outs = []
    for _ in range(2):
        out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.plb_conservation_static(q, dev.data_ptr(), ncells, plane, sol.data_ptr(), out.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
        assert rc == 0, lib.plb_last_error().decode()
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy())
    return outs


def test_static_matches_plb_conservation_reference_semantics():
    torch = pytest.importorskip("torch")
    from plbpd_gb300 import capi
    lib = capi.lib()
    cfg = CASES["d3q19_xy_periodic"]
    with capi.Solve.create(**cfg, semantics=capi.SEMANTICS_REFERENCE, arith=capi.ARITH_REFERENCE) as s:
        s.initialize()
        for _ in range(2):
            s.step(7)
            want = s.conservation()
            n = s.get(capi.FIELD_N)[1:-1, 1:-1, 1:-1]
            solid = np.zeros(n.shape[:3], bool)
            solid[0] = solid[-1] = True          # the up/down wall layers
            for got in _static_sums(torch, lib, s.q, n, solid):
                np.testing.assert_allclose(got, want, rtol=RTOL, atol=ATOL)


def test_static_matches_plb_conservation_many_blocks():
    """24,000 cells: several 4,096-cell blocks and a ragged last block."""
    torch = pytest.importorskip("torch")
    from plbpd_gb300 import capi
    lib = capi.lib()
    periodic = {f: "periodic" for f in capi.FACES}
    with capi.Solve.create("D3Q19", 40, 30, 20, 0.05, u0=(0.02, -0.01, 0.0), face_type=periodic,
                           semantics=capi.SEMANTICS_NATIVE, arith=capi.ARITH_FP32) as s:
        s.initialize()
        for _ in range(2):
            s.step(5)
            n = s.get(capi.FIELD_N)[1:-1, 1:-1, 1:-1]
            want = s.conservation()
            solid = np.zeros(n.shape[:3], bool)
            for got in _static_sums(torch, lib, s.q, n, solid):
                np.testing.assert_allclose(got, want, rtol=RTOL, atol=ATOL)


def test_static_rejects_more_cells_than_its_scratch_holds():
    torch = pytest.importorskip("torch")
    from plbpd_gb300 import capi
    lib = capi.lib()
    dev = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    too_many = 16_777_216 + 1
    rc = lib.plb_conservation_static(19, dev.data_ptr(), too_many, too_many, None, out.data_ptr(), None)
    assert rc == capi.EINVAL
    assert "static scratch limit" in lib.plb_last_error().decode()
