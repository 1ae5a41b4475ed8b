"""sed_op_apply_noalloc: the matvec for callers that may not allocate device
memory while they work (a host whose pool owns the device memory, a serving
loop that cannot take cudaMalloc's device-wide synchronisation, a fixed memory
budget after set-up).  The set-up here (catalog, sector, operator, the test's
own input and output buffers) allocates as usual; the entry point under test
allocates nothing and keeps its work vectors in a fixed device array.

It is called through the C ABI on device buffers, first thing on a freshly
built operator (so it cannot borrow work vectors or a tuned launch shape that
an earlier allocating call left behind), and must give the same vector as the
allocating entry point sed_op_apply on a second, independent operator, within
the FP64 matvec tolerance of the other parity tests, on two consecutive calls
with different inputs (the second call must not see the first call's
leftovers).  A second test checks that a hundred calls leave the device's free
memory unchanged."""
import ctypes as C

import numpy as np
import pytest

from cases import case_by_name, x_random

pytestmark = pytest.mark.gpu


def _op(case, sector, precision="fp64"):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    cat = A.build_symmetry_orbit_catalog(n_filled=case.spec.n_filled, species=case.spec.species,
                                         symmetry_group=case.group(),
                                         particle_statistics=statistics_from_name(case.statistics))
    basis = A.build_symmetry_sector_basis(cat, case.irreps()[sector])
    return A.MatrixFreeHamiltonian(basis, case.bilinear1(), case.density1(), precision=precision)


def _free_bytes(lib):
    free = C.c_int64(0)
    st = lib.sed_device_info(None, None, C.byref(free), None)
    assert st == 0, lib.sed_last_error()
    return free.value


@pytest.mark.parametrize("name,sector,precision", [("checkerboard3x2_f_flux", 1, "fp64"),
                                                   ("ring16", 0, "fp64"),
                                                   ("hubbard2x3", 2, "mixed")])
def test_noalloc_apply_matches_allocating_apply(name, sector, precision):
    import torch

    from realspace_exactdiagonalization_gb300 import _lib

    lib = _lib.load()
    case = case_by_name(name)
    H = _op(case, sector, precision)       # used only through the no-alloc entry point
    H_ref = _op(case, sector, precision)   # an independent operator for the reference
    n = H.n
    tol = 1e-11  # the FP64 matvec tolerance of the parity tests (both entry points run the same kernels)
    xs = [x_random(n, seed=s) for s in (11, 12)]
    outs = []
    for x in xs:
        xd = torch.from_numpy(x.view(np.float64).copy()).cuda()
        yd = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        st = lib.sed_op_apply_noalloc(H.handle, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), n)
        assert st == 0, lib.sed_last_error()
        torch.cuda.synchronize()
        outs.append(yd.cpu().numpy().view(np.complex128).copy())
    for call, (x, y) in enumerate(zip(xs, outs)):
        y_ref = H_ref(x)
        scale = max(1.0, np.abs(y_ref).max())
        assert np.abs(y - y_ref).max() <= tol * scale, (name, call)


def test_noalloc_allocates_no_device_memory():
    """A hundred calls on a 400,000-orbit sector (each of the allocating path's
    work vectors would take 6.4 MB) leave the device's free memory and the
    torch allocator's bytes unchanged.  One call first loads the kernels the
    entry point launches (module loading may take device memory once)."""
    import torch

    from cases import Case
    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300 import lattice as L

    lib = _lib.load()
    H = _op(Case("heisenberg26", L.heisenberg_ring(26)), 0)
    assert 300_000 < H.info()["n_orbits"] <= (1 << 20)
    n = H.n
    xd = torch.from_numpy(x_random(n, seed=3).view(np.float64).copy()).cuda()
    yd = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert lib.sed_op_apply_noalloc(H.handle, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), n) == 0
    torch.cuda.synchronize()
    first = yd.clone()
    free0 = _free_bytes(lib)
    torch_bytes0 = torch.cuda.memory_allocated()
    for _ in range(100):
        st = lib.sed_op_apply_noalloc(H.handle, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), n)
        assert st == 0, lib.sed_last_error()
    torch.cuda.synchronize()
    assert _free_bytes(lib) == free0
    assert torch.cuda.memory_allocated() == torch_bytes0
    assert torch.equal(yd, first)  # same input, same launch shape: the same bits


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
