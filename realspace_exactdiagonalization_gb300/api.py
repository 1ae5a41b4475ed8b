"""Reference-facing API: the Julia package's hot-path types and functions,
backed by the GPU library.

Names, argument meaning and error behaviour follow
src/symmetry_resolved_ed.jl (SRE) of RealSpace_ExactDiagonalization v0.1.0;
Julia's mutating ``f!`` becomes ``f_``.  Site indices in term lists and
permutations are 1-based, as in the reference; the C ABI underneath is 0-based.
Every compute call goes to libsed_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import check, ptr
from .groups import (Bosonic, Fermionic, Finite_Symmetry_Group, OneDim_Irrep, Particle_Statistics,
                     Symmetry_Operation, build_identity_group, build_identity_irrep_list, group_order)

__all__ = [
    "Bosonic", "Fermionic", "Symmetry_Operation", "Finite_Symmetry_Group", "OneDim_Irrep", "group_order",
    "build_identity_group", "build_identity_irrep_list", "Real_Space_Second_Quantized_Model",
    "Symmetry_Orbit_Catalog", "build_symmetry_orbit_catalog", "update_orbit_stabilizer_phases_",
    "expand_sector_state_to_fock", "_expand_sector_state_to_fock_amplitudes", "colex_unrank",
    "Symmetry_Sector_Basis", "build_symmetry_sector_basis", "CanonicalMap", "populate_canonical_map_",
    "MatrixFreeHamiltonian", "apply_hamiltonian_", "hamiltonian_linear_operator", "diagonalize_block_matrixfree",
    "DeviceGroup",
]


@dataclass
class Real_Space_Second_Quantized_Model:
    """Mirror of ``Real_Space_Second_Quantized_Model{T}`` (src/second_quantized_model.jl:19-26).
    ``bilinear_terms`` are ``(i, j, t)``: t moves a particle from site i to site j."""

    params: Dict[str, Any]
    lattice: Any
    tb_model: Any
    particle_statistics: Particle_Statistics
    bilinear_terms: List[Tuple[int, int, complex]]
    density_density_terms: List[Tuple[int, int, complex]]


def update_second_quantized_model_with_twisted_phases_(model: Real_Space_Second_Quantized_Model,
                                                       twisted_phases_over_2pi: Sequence[float]):
    """src/second_quantized_model.jl:39-53: regenerate the bilinear terms with a twist."""
    from .lattice import generate_bilinear_terms

    if len(twisted_phases_over_2pi) != model.lattice.dim:
        raise ValueError(f"twisted_phases_over_2π must have length {model.lattice.dim}.")
    model.bilinear_terms = generate_bilinear_terms(model.tb_model, twisted_phases_over_2pi)
    model.lattice.twisted_phases_over_2pi = list(twisted_phases_over_2pi)
    return model


# ------------------------------------------------------------------- handles
class _Handle:
    _destroy = ""

    def __init__(self, h: C.c_void_p):
        self._h = h

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                getattr(_lib.load(), self._destroy)(h)
            except Exception:
                pass
            self._h = None


class DeviceGroup(_Handle):
    """A Finite_Symmetry_Group uploaded to the library (with its statistics)."""

    _destroy = "sed_group_destroy"

    def __init__(self, G: Finite_Symmetry_Group, stats: Particle_Statistics):
        lib = _lib.load()
        perm = np.ascontiguousarray(G.perm0(), dtype=np.int32)
        ph = np.ascontiguousarray(G.phases(), dtype=np.complex128)
        h = C.c_void_p()
        check(lib.sed_group_create(G.n_site, len(G), ptr(perm), ptr(ph), G.identity_idx - 1, stats.code,
                                   C.byref(h)))
        super().__init__(h)
        self.group = G
        self.stats = stats

    def inverse(self) -> np.ndarray:
        inv = np.zeros(len(self.group), dtype=np.int32)
        check(_lib.load().sed_group_inverse(self._h, ptr(inv)))
        return inv


class Symmetry_Orbit_Catalog(_Handle):
    """SRE:305-327.  The tables live on the device; the reference's fields are
    read back lazily, in the reference's layout (1-based indices)."""

    _destroy = "sed_catalog_destroy"

    def __init__(self, h, dgroup: DeviceGroup, n_filled: int, species=None):
        super().__init__(h)
        self._dgroup = dgroup
        self.symmetry_group = dgroup.group
        self.particle_statistics = dgroup.stats
        self.n_filled = n_filled
        # (n_split, n_lo, n_hi) for a two-species catalog, else None
        self.species = tuple(species) if species else None
        ns, no, nst = C.c_int64(), C.c_int64(), C.c_int64()
        check(_lib.load().sed_catalog_info(h, C.byref(ns), C.byref(no), C.byref(nst)))
        self.n_states, self.n_orbits, self.n_stab_total = ns.value, no.value, nst.value
        self._cache: Dict[int, np.ndarray] = {}

    def _get(self, field: int) -> np.ndarray:
        if field not in self._cache:
            n, dt = {
                _lib.FIELD_REPS: (self.n_orbits, np.uint64), _lib.FIELD_STAB_ORDER: (self.n_orbits, np.int32),
                _lib.FIELD_STAB_PTR: (self.n_orbits + 1, np.int64), _lib.FIELD_STAB_G: (self.n_stab_total, np.int32),
                _lib.FIELD_STAB_PHASE: (self.n_stab_total, np.complex128),
                _lib.FIELD_REP_RANK: (self.n_states, np.int32), _lib.FIELD_REP_SYM: (self.n_states, np.int32),
                _lib.FIELD_REP_AMP: (self.n_states, np.complex128),
            }[field]
            out = np.zeros(n, dtype=dt)
            check(_lib.load().sed_catalog_get(self._h, field, ptr(out), out.nbytes))
            self._cache[field] = out
        return self._cache[field]

    @property
    def representative_mask_list(self) -> np.ndarray:
        return self._get(_lib.FIELD_REPS)

    @property
    def stabilizer_order_list(self) -> np.ndarray:
        return self._get(_lib.FIELD_STAB_ORDER)

    @property
    def stabilizer_g_indices_list(self) -> List[np.ndarray]:
        p, g = self._get(_lib.FIELD_STAB_PTR), self._get(_lib.FIELD_STAB_G)
        return [g[p[i]:p[i + 1]] for i in range(self.n_orbits)]

    @property
    def stabilizer_phases_list(self) -> List[np.ndarray]:
        p, v = self._get(_lib.FIELD_STAB_PTR), self._get(_lib.FIELD_STAB_PHASE)
        return [v[p[i]:p[i + 1]] for i in range(self.n_orbits)]

    @property
    def rep_rank_table(self) -> np.ndarray:
        return self._get(_lib.FIELD_REP_RANK)

    @property
    def rep_sym_table(self) -> np.ndarray:
        return self._get(_lib.FIELD_REP_SYM)

    @property
    def rep_amp_table(self) -> np.ndarray:
        return self._get(_lib.FIELD_REP_AMP)

    def lookup(self, masks) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(rep_rank, rep_sym, rep_amp) at the given masks, 1-based like the
        whole tables, without reading the tables back."""
        m = np.ascontiguousarray(masks, dtype=np.uint64)
        rk = np.zeros(m.size, dtype=np.int32)
        sy = np.zeros(m.size, dtype=np.int32)
        am = np.zeros(m.size, dtype=np.complex128)
        check(_lib.load().sed_catalog_lookup(self._h, m.size, ptr(m), ptr(rk), ptr(sy), ptr(am)))
        return rk, sy, am


def build_symmetry_orbit_catalog(*, second_quantized_model=None, n_filled: int,
                                 symmetry_group: Finite_Symmetry_Group,
                                 particle_statistics: Particle_Statistics,
                                 species=None) -> Symmetry_Orbit_Catalog:
    """SRE:371-487, on the device.

    ``species=(n_split, n_lo, n_hi)`` (an extension: the reference fixes only
    the total particle number) restricts the catalog to n_lo particles on
    sites 1..n_split and n_hi on the rest, e.g. one (N_up, N_down) block of a
    Hubbard model whose up spins sit on the first half of the modes; n_filled
    must then equal n_lo + n_hi."""
    if second_quantized_model is not None and second_quantized_model.lattice.n_site != symmetry_group.n_site:
        raise ValueError("the group and the model act on different numbers of sites")
    if not 0 <= n_filled <= symmetry_group.n_site:
        raise ValueError("n_filled must be in [0, n_site]")
    dg = DeviceGroup(symmetry_group, particle_statistics)
    h = C.c_void_p()
    if species:
        n_split, n_lo, n_hi = species
        if n_lo + n_hi != n_filled:
            raise ValueError("n_filled must equal n_lo + n_hi of the species")
        check(_lib.load().sed_catalog_build_species(dg.handle, n_split, n_lo, n_hi, C.byref(h)))
    else:
        check(_lib.load().sed_catalog_build(dg.handle, n_filled, C.byref(h)))
    return Symmetry_Orbit_Catalog(h, dg, n_filled, species)


def update_orbit_stabilizer_phases_(catalog: Symmetry_Orbit_Catalog, new_group: Finite_Symmetry_Group,
                                    particle_statistics: Particle_Statistics) -> Symmetry_Orbit_Catalog:
    """SRE:338-369: adopt a twisted copy of the group without re-enumeration."""
    if new_group is catalog.symmetry_group:
        return catalog
    dg = DeviceGroup(new_group, particle_statistics)
    check(_lib.load().sed_catalog_update_phases(catalog.handle, dg.handle))
    catalog._dgroup = dg
    catalog.symmetry_group = new_group
    catalog._cache.clear()
    return catalog


class Symmetry_Sector_Basis(_Handle):
    """SRE:522-528: orbits compatible with a 1D irrep, in catalog order."""

    _destroy = "sed_sector_destroy"

    def __init__(self, h, catalog: Symmetry_Orbit_Catalog, irrep: OneDim_Irrep, dim: int):
        super().__init__(h)
        self.catalog = catalog
        self.irrep = irrep
        self.symmetry_group = catalog.symmetry_group
        self.dim = dim
        self._arrays = None
        self._map = None

    def _load(self):
        if self._arrays is None:
            reps = np.zeros(self.dim, dtype=np.uint64)
            stab = np.zeros(self.dim, dtype=np.int32)
            orb = np.zeros(self.dim, dtype=np.int32)
            check(_lib.load().sed_sector_get(self._h, ptr(reps), ptr(stab), ptr(orb)))
            self._arrays = (reps, stab, orb)
        return self._arrays

    @property
    def representative_mask_list(self) -> np.ndarray:
        return self._load()[0]

    @property
    def stabilizer_order_list(self) -> np.ndarray:
        return self._load()[1]

    @property
    def orbit_index_list(self) -> np.ndarray:
        return self._load()[2]

    def project(self, masks) -> Tuple[np.ndarray, np.ndarray]:
        """project_to_sector (SRE:627-632) for many masks: (1-based rows, 0 when
        the orbit is outside the sector; coefficients)."""
        m = np.ascontiguousarray(masks, dtype=np.uint64)
        rows = np.zeros(len(m), dtype=np.int64)
        coeff = np.zeros(len(m), dtype=np.complex128)
        check(_lib.load().sed_sector_project(self._h, len(m), ptr(m), ptr(rows), ptr(coeff)))
        return rows + 1, coeff

    @property
    def representative_mask_to_mask_idx_map(self) -> Dict[int, int]:
        if self._map is None:
            self._map = {int(m): i + 1 for i, m in enumerate(self.representative_mask_list)}
        return self._map


def build_symmetry_sector_basis(catalog: Symmetry_Orbit_Catalog, irrep: OneDim_Irrep,
                                atol: float = 1e-12, group: Optional[Finite_Symmetry_Group] = None
                                ) -> Symmetry_Sector_Basis:
    """SRE:544-556.  With ``group`` (a twisted copy of the catalog's group,
    same permutations) the sector uses that group's phases without changing
    the catalog: update_orbit_stabilizer_phases! + build_symmetry_sector_basis
    in one step, safe to run for several twists at once."""
    chi = np.ascontiguousarray(irrep.array(), dtype=np.complex128)
    if len(chi) != group_order(catalog.symmetry_group):
        raise ValueError("the irrep needs one value per group element")
    h, dim = C.c_void_p(), C.c_int64()
    if group is None:
        check(_lib.load().sed_sector_build(catalog.handle, ptr(chi), float(atol), C.byref(h), C.byref(dim)))
    else:
        dg = DeviceGroup(group, catalog.particle_statistics)
        check(_lib.load().sed_sector_build_group(catalog.handle, dg.handle, ptr(chi), float(atol), C.byref(h),
                                                 C.byref(dim)))
    basis = Symmetry_Sector_Basis(h, catalog, irrep, dim.value)
    if group is not None:
        basis.symmetry_group = group
    return basis


def expand_sector_state_to_fock(c: np.ndarray, basis: "Symmetry_Sector_Basis", atol: float = 1e-12) -> np.ndarray:
    """_expand_sector_state_to_fock_amplitudes (observables/entanglement_spectrum.jl:46-79)
    on the device, as a dense complex128 vector over the fixed-filling Fock
    states in colex-rank order (ascending masks); dropped amplitudes are 0."""
    c = np.ascontiguousarray(c, dtype=np.complex128)
    if c.shape != (basis.dim,):
        raise ValueError(f"expected {basis.dim} sector coefficients")
    out = np.zeros(basis.catalog.n_states, dtype=np.complex128)
    n2 = C.c_double()
    check(_lib.load().sed_sector_expand_fock(basis.handle, ptr(c), basis.dim, float(atol), ptr(out),
                                             basis.catalog.n_states, 0, C.byref(n2)))
    return out


def colex_unrank(ranks: np.ndarray, n_site: int, n_filled: int) -> np.ndarray:
    """Masks of the given colex ranks (the r-th k-subset in ascending order)."""
    from math import comb

    r = np.asarray(ranks, dtype=np.int64).copy()
    m = np.zeros(r.shape, dtype=np.uint64)
    b = np.full(r.shape, n_site - 1, dtype=np.int64)
    table = np.array([[comb(n, j) for j in range(n_filled + 1)] for n in range(n_site + 1)], dtype=np.int64)
    for j in range(n_filled, 0, -1):
        while True:
            big = (b >= j) & (table[np.maximum(b, 0), j] > r)
            if not big.any():
                break
            b = np.where(big, b - 1, b)
        m |= np.left_shift(np.uint64(1), b.astype(np.uint64))
        r -= table[b, j]
        b -= 1
    return m


def catalog_state_masks(catalog: "Symmetry_Orbit_Catalog", ranks: np.ndarray) -> np.ndarray:
    """Masks of the catalog's basis states of the given ranks: colex k-subsets,
    or for a two-species catalog rank = rank_hi * binom(n_split, n_lo) +
    rank_lo (both ascending-mask orders)."""
    from math import comb

    n_site = catalog.symmetry_group.n_site
    if not catalog.species:
        return colex_unrank(ranks, n_site, catalog.n_filled)
    n_split, n_lo, n_hi = catalog.species
    r = np.asarray(ranks, dtype=np.int64)
    lo = colex_unrank(r % comb(n_split, n_lo), n_split, n_lo)
    hi = colex_unrank(r // comb(n_split, n_lo), n_site - n_split, n_hi)
    return lo | np.left_shift(hi, np.uint64(n_split))


def _expand_sector_state_to_fock_amplitudes(c: np.ndarray, basis: "Symmetry_Sector_Basis",
                                            particle_statistics=None, atol: float = 1e-12) -> Dict[int, complex]:
    """The reference's Dict{Mask, ComplexF64} form of expand_sector_state_to_fock."""
    dense = expand_sector_state_to_fock(c, basis, atol)
    nz = np.nonzero(dense)[0]
    masks = catalog_state_masks(basis.catalog, nz)
    return {int(mk): complex(a) for mk, a in zip(masks, dense[nz])}


@dataclass
class CanonicalMap:
    """SRE:577-581.  The representative tables are already on the device."""

    symmetry_group: Finite_Symmetry_Group
    particle_statistics: Particle_Statistics
    catalog: Symmetry_Orbit_Catalog


def populate_canonical_map_(cmap: CanonicalMap, basis, bilinear_terms) -> CanonicalMap:
    """SRE:605-608: a no-op kept for API compatibility, as in the reference."""
    return cmap


def _terms_arrays(terms, n_site: int, what: str):
    n = len(terms)
    ij = np.zeros((n, 2), dtype=np.int32)
    v = np.zeros(n, dtype=np.complex128)
    for k, (i, j, t) in enumerate(terms):
        if not (1 <= int(i) <= n_site and 1 <= int(j) <= n_site):
            raise ValueError(f"{what} term {k} has a site index outside 1:{n_site}")
        ij[k] = (int(i) - 1, int(j) - 1)
        v[k] = complex(t)
    return ij, v


class MatrixFreeHamiltonian(_Handle):
    """SRE:767-791 / hamiltonian_linear_operator SRE:891-897: ``H(x) -> y``.

    ``precision="fp64"`` is the plain drop-in (complex128 matvec);
    ``"mixed"`` runs the matvec in complex64 and solves with FP64 Lanczos and
    an FP64 Rayleigh-Ritz polish."""

    _destroy = "sed_op_destroy"

    def __init__(self, basis: Symmetry_Sector_Basis, bilinear_terms, density_terms, cmap: Optional[CanonicalMap] = None,
                 precision: str = "fp64"):
        self.basis = basis
        n_site = basis.symmetry_group.n_site
        self.bilinear_terms = [(int(i), int(j), complex(t)) for (i, j, t) in bilinear_terms]
        self.density_terms = [(int(i), int(j), complex(v)) for (i, j, v) in density_terms]
        bij, bt = _terms_arrays(self.bilinear_terms, n_site, "bilinear")
        dij, dv = _terms_arrays(self.density_terms, n_site, "density")
        prec = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[precision]
        h = C.c_void_p()
        check(_lib.load().sed_op_create(basis.handle, len(bt), ptr(bij), ptr(bt), len(dv), ptr(dij), ptr(dv), prec,
                                        C.byref(h)))
        super().__init__(h)
        self.precision = precision
        self.n = basis.dim

    def __call__(self, x: np.ndarray) -> np.ndarray:
        y = np.empty(self.n, dtype=np.complex128)
        return self.apply(x, y)

    def apply(self, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.complex128)
        if x.shape != (self.n,) or y.shape != (self.n,) or y.dtype != np.complex128:
            raise ValueError(f"x and y must be complex128 vectors of length {self.n}")
        check(_lib.load().sed_op_apply(self._h, ptr(x), ptr(y), self.n, 0))
        return y

    def info(self):
        d, no, hops = C.c_int64(), C.c_int64(), C.c_int64()
        check(_lib.load().sed_op_info(self._h, C.byref(d), C.byref(no), C.byref(hops)))
        return {"dim": d.value, "n_orbits": no.value, "hops": hops.value}

    HOP_TABLE_OFF, HOP_TABLE_AUTO, HOP_TABLE_NOW = 0, 1, 2

    def set_apply_shape(self, threads_per_row: int = 0, threads_per_block: int = 0) -> None:
        """Pin the gather matvec's launch shape ((0, 0): let the autotuner choose)."""
        check(_lib.load().sed_op_set_apply_shape(self._h, int(threads_per_row), int(threads_per_block)))

    def apply_shape(self, complex64: bool = False) -> tuple:
        """(threads per row, threads per block) of the gather matvec; (0, 0) before the first gather."""
        t, b = C.c_int(0), C.c_int(0)
        check(_lib.load().sed_op_apply_shape(self._h, int(bool(complex64)), C.byref(t), C.byref(b)))
        return t.value, b.value

    def set_priority(self, high: bool) -> None:
        """Scheduling priority of this operator's stream when several solves
        share the GPU (sed_op_set_priority): high-priority kernels are
        scheduled before the queued kernels of low-priority solves."""
        check(_lib.load().sed_op_set_priority(self._h, 1 if high else 0))

    def set_sm_limit(self, n_sm: int) -> None:
        """Size this operator's kernel grids for n_sm SMs (0: the whole
        device; sed_op_set_sm_limit), for a server that keeps other work
        resident on the remaining SMs.  Results do not change."""
        check(_lib.load().sed_op_set_sm_limit(self._h, int(n_sm)))

    def set_hop_table(self, mode: int) -> None:
        """The stored form of this operator's matvec (8 bytes per hop): 0 off,
        1 built at the first solve when it fits (default), 2 built now."""
        check(_lib.load().sed_op_set_hop_table(self._h, int(mode)))

    def hop_table_info(self) -> dict:
        built, rec, nb = C.c_int32(), C.c_int64(), C.c_int64()
        check(_lib.load().sed_op_hop_table_info(self._h, C.byref(built), C.byref(rec), C.byref(nb)))
        return {"built": bool(built.value), "records": rec.value, "bytes": nb.value}

    def solve(self, nev: int, tol: float = 1e-10, maxiter: int = 300, krylovdim: int = 30, seed: int = 0x5EED0000,
              want_vectors: bool = True):
        ev = np.zeros(max(nev, 1), dtype=np.float64)
        k = min(nev, self.n)
        vecs = np.zeros((k, self.n), dtype=np.complex128) if (want_vectors and k > 0) else None
        info = _lib.sed_solve_info()
        st = _lib.load().sed_solve(self._h, nev, float(tol), int(maxiter), int(krylovdim), C.c_uint64(seed), ptr(ev),
                                   ptr(vecs), C.byref(info))
        check(st)
        return ev[:k], (vecs.T.copy() if vecs is not None else None), info


def apply_hamiltonian_(y: np.ndarray, x: np.ndarray, basis: Symmetry_Sector_Basis, bilinear_terms, density_terms,
                       cmap: Optional[CanonicalMap] = None) -> np.ndarray:
    """SRE:804-878: y = H x on the device (builds a transient operator)."""
    if len(y) != len(x):
        raise ValueError("length(y) == n")
    H = MatrixFreeHamiltonian(basis, bilinear_terms, density_terms, cmap)
    return H.apply(x, y)


def hamiltonian_linear_operator(basis: Symmetry_Sector_Basis, bilinear_terms, density_terms,
                                cmap: Optional[CanonicalMap] = None, precision: str = "fp64"):
    """SRE:891-897: ``(H_op, n)``."""
    H = MatrixFreeHamiltonian(basis, bilinear_terms, density_terms, cmap, precision=precision)
    return H, basis.dim


def diagonalize_block_matrixfree(H_op: MatrixFreeHamiltonian, n: int, nev: int = 5, tol: float = 1e-10,
                                 maxiter: int = 300, krylovdim: int = 30, seed: int = 0x5EED0000):
    """SRE:998-1030: lowest ``nev`` eigenpairs, ``(vals, vecs)`` with
    ``vecs[:, i]`` the i-th eigenvector.  Raises SEDError (status
    SED_ERR_NOT_CONVERGED) where the reference raises "Lanczos did not
    converge".  Only device operators are accepted: there is no CPU path."""
    if n == 0:
        return np.zeros(0), np.zeros((0, 0), dtype=np.complex128)
    if not isinstance(H_op, MatrixFreeHamiltonian):
        raise TypeError("diagonalize_block_matrixfree needs a device MatrixFreeHamiltonian")
    if H_op.n != n:
        raise ValueError("n must equal the operator dimension")
    vals, vecs, _ = H_op.solve(nev, tol=tol, maxiter=maxiter, krylovdim=krylovdim, seed=seed)
    return vals, vecs
