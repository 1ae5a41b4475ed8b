"""The C ABI library loads, exports every declared entry point, and rejects
malformed inputs on the host (no GPU needed for any call here)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "sed_capi.h")).read()
    return sorted(set(re.findall(r"^(?:int|void|const char\*)\s+(sed_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from realspace_exactdiagonalization_gb300 import _lib, build_lib

    build_lib.build()
    return _lib.load()


def test_every_declared_symbol_is_exported_and_bound(lib):
    from realspace_exactdiagonalization_gb300 import _lib

    names = declared_functions()
    assert len(names) >= 25
    bound = {n for n, _, _ in _lib.SIGNATURES}
    for n in names:
        assert hasattr(lib, n), f"{n} missing from libsed_gb300.so"
        assert n in bound, f"{n} has no ctypes signature"


def test_version_and_error_string(lib):
    assert lib.sed_api_version() == 1
    assert isinstance(lib.sed_last_error(), bytes)


def _group(lib, perm, phase=None, identity=0, stats=0):
    perm = np.ascontiguousarray(perm, dtype=np.int32)
    n_ops, n_site = perm.shape
    if phase is None:
        phase = np.ones((n_ops, n_site), dtype=np.complex128)
    phase = np.ascontiguousarray(phase, dtype=np.complex128)
    h = C.c_void_p()
    st = lib.sed_group_create(n_site, n_ops, perm.ctypes.data_as(C.c_void_p), phase.ctypes.data_as(C.c_void_p),
                              identity, stats, C.byref(h))
    return st, h


def test_group_validation(lib):
    from realspace_exactdiagonalization_gb300 import _lib

    ring = np.array([[(i + d) % 6 for i in range(6)] for d in range(6)])
    st, h = _group(lib, ring)
    assert st == _lib.SED_OK
    inv = np.zeros(6, dtype=np.int32)
    assert lib.sed_group_inverse(h, inv.ctypes.data_as(C.c_void_p)) == 0
    assert list(inv) == [0, 5, 4, 3, 2, 1]
    lib.sed_group_destroy(h)
    st, _ = _group(lib, [[0, 0, 1]])  # not a permutation
    assert st == _lib.SED_ERR_ARG and b"permute" in lib.sed_last_error()
    st, _ = _group(lib, [[1, 0, 2], [0, 1, 2]])  # identity index 0 is not the identity
    assert st == _lib.SED_ERR_ARG and b"Identity" in lib.sed_last_error()
    st, _ = _group(lib, np.tile(np.arange(64), (1, 1)))
    assert st == _lib.SED_ERR_LIMIT
    # phases that do not close under inversion (SRE:109-117 raises)
    ph = np.ones((2, 2), dtype=np.complex128)
    ph[1] = [1j, 1j]
    st, _ = _group(lib, [[0, 1], [1, 0]], ph)
    assert st == _lib.SED_ERR_ARG and b"inversion" in lib.sed_last_error()


def test_terms_validation(lib):
    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300 import lattice as L

    spec = L.checkerboard(3, 2, n_filled=4)
    for th in [(0.0, 0.0), (0.23, 0.17)]:
        G = L.build_translation_group(spec.lattice, th)
        st, g = _group(lib, G.perm0(), G.phases(), 0, 1)
        assert st == 0
        terms = spec.bilinear_terms(th)
        ij = np.ascontiguousarray([[i - 1, j - 1] for (i, j, _) in terms], dtype=np.int32)
        t = np.ascontiguousarray([v for (_, _, v) in terms], dtype=np.complex128)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        assert lib.sed_terms_validate(g, len(t), vp(ij), vp(t)) == 0, lib.sed_last_error()
        bad = t.copy()
        bad[0] *= 1.5  # breaks Hermiticity and translation invariance
        assert lib.sed_terms_validate(g, len(t), vp(ij), vp(bad)) == _lib.SED_ERR_NOT_HERMITIAN
        # the validator's term table is reused across calls: a rejected list
        # leaves no residue behind
        assert lib.sed_terms_validate(g, len(t), vp(ij), vp(t)) == 0, lib.sed_last_error()
        if th != (0.0, 0.0):
            # twist phases applied without the matching group gauge
            G0 = L.build_translation_group(spec.lattice, (0.0, 0.0))
            st, g0 = _group(lib, G0.perm0(), G0.phases(), 0, 1)
            assert lib.sed_terms_validate(g0, len(t), vp(ij), vp(t)) == _lib.SED_ERR_NOT_HERMITIAN
            lib.sed_group_destroy(g0)
        diag = ij.copy()
        diag[0] = [2, 2]
        assert lib.sed_terms_validate(g, len(t), vp(diag), vp(t)) == _lib.SED_ERR_ARG
        lib.sed_group_destroy(g)


def test_python_api_fails_loudly_without_library(monkeypatch, tmp_path):
    from realspace_exactdiagonalization_gb300 import _lib

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load()
