"""ctypes wrapper around liboracle.so, the CPU restatement of the reference.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check in
__graft_entry__.py and by bench.py's CPU-baseline / reference arm.  The product
package never imports this module.

All arrays crossing this wrapper are numpy arrays; sites are 0-based here.
See sed_oracle.cpp for the reference functions each entry point restates.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

FIELD_REPS, FIELD_STAB_ORDER, FIELD_STAB_PTR, FIELD_STAB_G, FIELD_STAB_PHASE = 0, 1, 2, 3, 4
FIELD_REP_RANK, FIELD_REP_SYM, FIELD_REP_AMP = 5, 6, 7


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile."""
    src = os.path.join(_HERE, "sed_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        p, i32, i64, u64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double
        L.or_last_error.restype = C.c_char_p
        L.or_binom.restype = i64
        L.or_binom.argtypes = [i32, i32]
        L.or_rank.restype = i64
        L.or_rank.argtypes = [u64]
        L.or_gosper_next.restype = u64
        L.or_gosper_next.argtypes = [u64]
        L.or_lin_table.restype = i32
        L.or_lin_table.argtypes = [i32, i32, p, p]
        L.or_lin_index.restype = i64
        L.or_lin_index.argtypes = [u64, p, p, i32]
        L.or_apply_op.argtypes = [i32, p, p, i32, u64, p, p]
        L.or_inverse_ops.restype = i32
        L.or_inverse_ops.argtypes = [i32, i32, p, p, i32, i32, p]
        L.or_catalog_build.restype = p
        L.or_catalog_build.argtypes = [i32, i32, p, p, i32, i32, i32]
        L.or_catalog_update_phases.restype = i32
        L.or_catalog_update_phases.argtypes = [p, p]
        L.or_catalog_free.argtypes = [p]
        for f in ("or_catalog_n_states", "or_catalog_n_orbits", "or_catalog_n_stab"):
            getattr(L, f).restype = i64
            getattr(L, f).argtypes = [p]
        L.or_catalog_get.restype = i32
        L.or_catalog_get.argtypes = [p, i32, p]
        L.or_sector_build.restype = p
        L.or_sector_build.argtypes = [p, p, dbl]
        L.or_sector_free.argtypes = [p]
        L.or_sector_dim.restype = i64
        L.or_sector_dim.argtypes = [p]
        L.or_sector_get.argtypes = [p, p, p, p]
        L.or_project.restype = i32
        L.or_project.argtypes = [p, u64, i32, p, p]
        L.or_sector_expand_fock.restype = i32
        L.or_sector_expand_fock.argtypes = [p, p, dbl, p, p]
        L.or_canonical.argtypes = [p, u64, p, p, p]
        L.or_op_create.restype = p
        L.or_op_create.argtypes = [p, i32, p, p, i32, p, p]
        L.or_op_free.argtypes = [p]
        L.or_op_build_table.restype = i64
        L.or_op_build_table.argtypes = [p]
        L.or_op_get_table.argtypes = [p, p, p, p, p]
        L.or_op_apply.argtypes = [p, p, p, i32, i32]
        L.or_op_matrix_coo_count.restype = i64
        L.or_op_matrix_coo_count.argtypes = [p]
        L.or_op_matrix_coo.argtypes = [p, p, p, p]
        L.or_op_solve.restype = i32
        L.or_op_solve.argtypes = [p, i32, dbl, i32, i32, u64, i32, p, p, p, p, p]
        L.or_max_threads.restype = i32
        L.or_group_create.restype = p
        L.or_group_create.argtypes = [i32, i32, p, p, i32, i32]
        L.or_group_free.argtypes = [p]
        L.or_group_state_entry.argtypes = [p, u64, p, p, p, p]
        L.or_group_compatible.restype = i32
        L.or_group_compatible.argtypes = [p, p, u64, dbl]
        L.or_group_column.restype = i64
        L.or_group_column.argtypes = [p, p, i32, p, p, i32, p, p, u64, dbl, p, p, p, i64]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _err():
    return lib().or_last_error().decode()


def binom(n: int, k: int) -> int:
    return int(lib().or_binom(n, k))


def rank(m: int) -> int:
    return int(lib().or_rank(C.c_uint64(m)))


def gosper_next(x: int) -> int:
    return int(lib().or_gosper_next(C.c_uint64(x)))


def lin_table(n_site: int, n_filled: int):
    nr = n_site // 2
    nl = n_site - nr
    left = np.zeros(1 << nl, dtype=np.int64)
    right = np.zeros(1 << nr, dtype=np.int64)
    lib().or_lin_table(n_site, n_filled, _ptr(left), _ptr(right))
    return left, right, nr


def lin_index(m: int, left, right, n_right: int) -> int:
    return int(lib().or_lin_index(C.c_uint64(m), _ptr(left), _ptr(right), n_right))


def apply_op(perm0: np.ndarray, phase: np.ndarray, stats: int, m: int):
    perm0 = np.ascontiguousarray(perm0, dtype=np.int32)
    ph = np.ascontiguousarray(phase, dtype=np.complex128)
    out = np.zeros(1, dtype=np.uint64)
    amp = np.zeros(1, dtype=np.complex128)
    lib().or_apply_op(len(perm0), _ptr(perm0), _ptr(ph), stats, C.c_uint64(m), _ptr(out), _ptr(amp))
    return int(out[0]), complex(amp[0])


class Catalog:
    """Oracle orbit catalog (build_symmetry_orbit_catalog, SRE:371-487)."""

    def __init__(self, perm0: np.ndarray, phase: np.ndarray, identity0: int, stats: int, n_filled: int):
        self.perm0 = np.ascontiguousarray(perm0, dtype=np.int32)
        self.phase = np.ascontiguousarray(phase, dtype=np.complex128)
        n_ops, n_site = self.perm0.shape
        self.n_ops, self.n_site, self.stats, self.n_filled = n_ops, n_site, stats, n_filled
        self.h = lib().or_catalog_build(n_site, n_ops, _ptr(self.perm0), _ptr(self.phase), identity0, stats,
                                        n_filled)
        if not self.h:
            raise ValueError(_err())

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_catalog_free(self.h)
            self.h = None

    @property
    def n_states(self) -> int:
        return int(lib().or_catalog_n_states(self.h))

    @property
    def n_orbits(self) -> int:
        return int(lib().or_catalog_n_orbits(self.h))

    def get(self, field: int) -> np.ndarray:
        n_orb, n_st, n_stab = self.n_orbits, self.n_states, int(lib().or_catalog_n_stab(self.h))
        shape_dtype = {
            FIELD_REPS: (n_orb, np.uint64), FIELD_STAB_ORDER: (n_orb, np.int32), FIELD_STAB_PTR: (n_orb + 1, np.int64),
            FIELD_STAB_G: (n_stab, np.int32), FIELD_STAB_PHASE: (n_stab, np.complex128),
            FIELD_REP_RANK: (n_st, np.int32), FIELD_REP_SYM: (n_st, np.int32), FIELD_REP_AMP: (n_st, np.complex128),
        }[field]
        out = np.zeros(shape_dtype[0], dtype=shape_dtype[1])
        if lib().or_catalog_get(self.h, field, _ptr(out)) != 0:
            raise ValueError(_err())
        return out

    def update_phases(self, phase: np.ndarray) -> None:
        self.phase = np.ascontiguousarray(phase, dtype=np.complex128)
        if lib().or_catalog_update_phases(self.h, _ptr(self.phase)) != 0:
            raise ValueError(_err())

    def canonical(self, m: int):
        r = np.zeros(1, dtype=np.uint64)
        g = np.zeros(1, dtype=np.int32)
        a = np.zeros(1, dtype=np.complex128)
        lib().or_canonical(self.h, C.c_uint64(m), _ptr(r), _ptr(g), _ptr(a))
        return int(r[0]), int(g[0]), complex(a[0])


class Sector:
    """Oracle sector basis (build_symmetry_sector_basis, SRE:544-556)."""

    def __init__(self, cat: Catalog, chi: np.ndarray, atol: float = 1e-12):
        self.cat = cat
        self.chi = np.ascontiguousarray(chi, dtype=np.complex128)
        self.h = lib().or_sector_build(cat.h, _ptr(self.chi), atol)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_sector_free(self.h)
            self.h = None

    @property
    def dim(self) -> int:
        return int(lib().or_sector_dim(self.h))

    def arrays(self):
        n = self.dim
        reps = np.zeros(n, dtype=np.uint64)
        stab = np.zeros(n, dtype=np.int32)
        orb = np.zeros(n, dtype=np.int32)
        lib().or_sector_get(self.h, _ptr(reps), _ptr(stab), _ptr(orb))
        return reps, stab, orb

    def expand_fock(self, c: np.ndarray, atol: float = 1e-12) -> np.ndarray:
        """_expand_sector_state_to_fock_amplitudes (observables/entanglement_spectrum.jl:46-79)
        as a dense complex128 vector over the fixed-filling states in colex-rank order."""
        c = np.ascontiguousarray(c, dtype=np.complex128)
        out = np.zeros(self.cat.n_states, dtype=np.complex128)
        n2 = np.zeros(1)
        if lib().or_sector_expand_fock(self.h, _ptr(c), atol, _ptr(out), _ptr(n2)) != 0:
            raise RuntimeError(_err())
        return out

    def project(self, m: int, mode: int = 0):
        row = np.zeros(1, dtype=np.int64)
        coeff = np.zeros(1, dtype=np.complex128)
        if lib().or_project(self.h, C.c_uint64(m), mode, _ptr(row), _ptr(coeff)) == 0:
            return None
        return int(row[0]), complex(coeff[0])


class Op:
    """Oracle Hamiltonian on a sector (SRE:680-963)."""

    def __init__(self, sec: Sector, bilinear, density):
        self.sec = sec
        self.bij = np.ascontiguousarray([[i, j] for (i, j, _) in bilinear], dtype=np.int32).reshape(-1, 2)
        self.bt = np.ascontiguousarray([t for (_, _, t) in bilinear], dtype=np.complex128)
        self.dij = np.ascontiguousarray([[i, j] for (i, j, _) in density], dtype=np.int32).reshape(-1, 2)
        self.dv = np.ascontiguousarray([v for (_, _, v) in density], dtype=np.complex128)
        self.h = lib().or_op_create(sec.h, len(self.bt), _ptr(self.bij), _ptr(self.bt), len(self.dv),
                                    _ptr(self.dij), _ptr(self.dv))

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_op_free(self.h)
            self.h = None

    @property
    def dim(self) -> int:
        return self.sec.dim

    def projection_table(self):
        nnz = int(lib().or_op_build_table(self.h))
        row = np.zeros(nnz, dtype=np.int64)
        col = np.zeros(nnz, dtype=np.int64)
        vals = np.zeros(nnz, dtype=np.complex128)
        diag = np.zeros(self.dim, dtype=np.complex128)
        lib().or_op_get_table(self.h, _ptr(row), _ptr(col), _ptr(vals), _ptr(diag))
        return row, col, vals, diag

    def apply(self, x: np.ndarray, mode: int = 0, nthreads: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.dim, dtype=np.complex128)
        lib().or_op_apply(self.h, _ptr(x), _ptr(y), mode, nthreads)
        return y

    def matrix_coo(self):
        n = int(lib().or_op_matrix_coo_count(self.h))
        I = np.zeros(n, dtype=np.int64)
        J = np.zeros(n, dtype=np.int64)
        V = np.zeros(n, dtype=np.complex128)
        lib().or_op_matrix_coo(self.h, _ptr(I), _ptr(J), _ptr(V))
        return I, J, V

    def dense(self) -> np.ndarray:
        I, J, V = self.matrix_coo()
        H = np.zeros((self.dim, self.dim), dtype=np.complex128)
        np.add.at(H, (I, J), V)
        return H

    def solve(self, nev: int, tol: float = 1e-10, maxiter: int = 300, krylovdim: int = 30, seed: int = 1,
              nthreads: int = 0, want_vectors: bool = False):
        n = self.dim
        ev = np.zeros(nev, dtype=np.float64)
        vecs = np.zeros((nev, n), dtype=np.complex128) if want_vectors else None
        nr = np.zeros(1, dtype=np.int32)
        nm = np.zeros(1, dtype=np.int32)
        res = np.zeros(nev, dtype=np.float64)
        st = lib().or_op_solve(self.h, nev, tol, maxiter, krylovdim, C.c_uint64(seed), nthreads, _ptr(ev),
                               _ptr(vecs) if vecs is not None else None, _ptr(nr), _ptr(nm), _ptr(res))
        return {"status": int(st), "evals": ev, "evecs": vecs, "restarts": int(nr[0]), "matvecs": int(nm[0]),
                "residuals": res}


class Group:
    """Catalog-free oracle for sectors too large for an in-memory catalog:
    table entries, compatibility and matrix columns for single masks, computed
    straight from the group (SRE:371-487, 534-542, 627-632, 843-866)."""

    def __init__(self, perm0: np.ndarray, phase: np.ndarray, identity0: int, stats: int):
        self.perm0 = np.ascontiguousarray(perm0, dtype=np.int32)
        self.phase = np.ascontiguousarray(phase, dtype=np.complex128)
        n_ops, n_site = self.perm0.shape
        self.h = lib().or_group_create(n_site, n_ops, _ptr(self.perm0), _ptr(self.phase), identity0, stats)
        if not self.h:
            raise ValueError(_err())

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_group_free(self.h)
            self.h = None

    def state_entry(self, m: int):
        """(representative, stabilizer order, rep_sym (1-based), rep_amp) of basis state m."""
        r = np.zeros(1, dtype=np.uint64)
        st = np.zeros(1, dtype=np.int32)
        sym = np.zeros(1, dtype=np.int32)
        amp = np.zeros(1, dtype=np.complex128)
        lib().or_group_state_entry(self.h, C.c_uint64(int(m)), _ptr(r), _ptr(st), _ptr(sym), _ptr(amp))
        return int(r[0]), int(st[0]), int(sym[0]), complex(amp[0])

    def compatible(self, chi: np.ndarray, rep: int, atol: float = 1e-12) -> bool:
        chi = np.ascontiguousarray(chi, dtype=np.complex128)
        return bool(lib().or_group_compatible(self.h, _ptr(chi), C.c_uint64(int(rep)), atol))

    def column(self, chi: np.ndarray, bilinear, density, rep_c: int, atol: float = 1e-12):
        """Column rep_c of the sector matrix: (diagonal, [(target rep, element), ...])."""
        chi = np.ascontiguousarray(chi, dtype=np.complex128)
        bij = np.ascontiguousarray([[i, j] for (i, j, _) in bilinear], dtype=np.int32).reshape(-1, 2)
        bt = np.ascontiguousarray([t for (_, _, t) in bilinear], dtype=np.complex128)
        dij = np.ascontiguousarray([[i, j] for (i, j, _) in density], dtype=np.int32).reshape(-1, 2)
        dv = np.ascontiguousarray([v for (_, _, v) in density], dtype=np.complex128)
        cap = max(len(bt), 1)
        tr = np.zeros(cap, dtype=np.uint64)
        el = np.zeros(cap, dtype=np.complex128)
        dg = np.zeros(1, dtype=np.complex128)
        n = lib().or_group_column(self.h, _ptr(chi), len(bt), _ptr(bij), _ptr(bt), len(dv), _ptr(dij), _ptr(dv),
                                  C.c_uint64(int(rep_c)), atol, _ptr(dg), _ptr(tr), _ptr(el), cap)
        if n < 0:
            raise RuntimeError("column buffer too small")
        return complex(dg[0]), list(zip(tr[:n].tolist(), el[:n].tolist()))


def max_threads() -> int:
    return int(lib().or_max_threads())
