"""sed_op_apply_noalloc: the matvec for callers that may not allocate device
memory while they work (a host whose pool owns the device memory, a serving
loop that cannot take cudaMalloc's device-wide synchronisation, a fixed memory
budget after set-up).  The set-up here (catalog, sector, operator, the test's
own input and output buffers) allocates as usual; the entry point under test
allocates nothing and keeps its work vectors in a fixed device array.

It is called through the C ABI on device buffers and must give the same vector
as the allocating entry point sed_op_apply, within the FP64 matvec tolerance of
the other parity tests, on two consecutive calls with different inputs (the
second call must not see the first call's leftovers)."""
import ctypes as C

import numpy as np
import pytest

from cases import case_by_name, x_random

pytestmark = pytest.mark.gpu


def _op(case, sector, precision="fp64"):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    cat = A.build_symmetry_orbit_catalog(n_filled=case.spec.n_filled, symmetry_group=case.group(),
                                         particle_statistics=statistics_from_name(case.statistics))
    basis = A.build_symmetry_sector_basis(cat, case.irreps()[sector])
    return A.MatrixFreeHamiltonian(basis, case.bilinear1(), case.density1(), precision=precision)


@pytest.mark.parametrize("name,sector,precision", [("checkerboard3x2_f_flux", 1, "fp64"),
                                                   ("ring16", 0, "fp64"),
                                                   ("hubbard2x3", 2, "mixed")])
def test_noalloc_apply_matches_allocating_apply(name, sector, precision):
    import torch

    from realspace_exactdiagonalization_gb300 import _lib

    lib = _lib.load()
    H = _op(case_by_name(name), sector, precision)
    n = H.n
    tol = 1e-11  # the FP64 matvec tolerance of the parity tests (both entry points run the same kernels)
    for call, seed in enumerate((11, 12)):
        x = x_random(n, seed=seed)
        y_ref = H(x)
        xd = torch.from_numpy(x.view(np.float64).copy()).cuda()
        yd = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        st = lib.sed_op_apply_noalloc(H.handle, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), n)
        assert st == 0, lib.sed_last_error()
        torch.cuda.synchronize()
        y = yd.cpu().numpy().view(np.complex128)
        scale = max(1.0, np.abs(y_ref).max())
        assert np.abs(y - y_ref).max() <= tol * scale, (name, call)


def test_noalloc_rejects_sectors_above_the_scratch_limit():
    """A catalog with more orbits than the fixed scratch holds is refused with
    SED_ERR_LIMIT and a clear message, before any device work."""
    import torch

    from cases import Case
    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300 import lattice as L

    lib = _lib.load()
    H = _op(Case("heisenberg28", L.heisenberg_ring(28)), 0)  # 1432860 orbits
    assert H.info()["n_orbits"] > (1 << 20)
    xd = torch.zeros(2 * H.n, dtype=torch.float64, device="cuda")
    yd = torch.zeros(2 * H.n, dtype=torch.float64, device="cuda")
    st = lib.sed_op_apply_noalloc(H.handle, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), H.n)
    assert st == _lib.SED_ERR_LIMIT
    assert b"1048576" in lib.sed_last_error()
