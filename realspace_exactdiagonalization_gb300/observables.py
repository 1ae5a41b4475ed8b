"""Flux-torus observables: the many-body charge pump and Chern number.

Restates the reference's ``observables/charge_pump.jl`` and
``observables/many_body_chern_number.jl`` over this package's device solves:

* ``many_body_position_phases`` (charge_pump.jl:17-33) -- the per-site
  phases of Resta's periodic position operator;
* ``position_operator_matrix`` (charge_pump.jl:47-91) -- that operator
  projected between two symmetry sectors, evaluated on the device
  (``sed_position_operator``);
* ``subspace_overlap_matrix`` / ``unit_det_link``
  (many_body_chern_number.jl:46-80) -- overlaps of Fock-expanded states, on
  the device (``sed_fock_overlaps``), and the unit determinant link;
* ``flux_point_states`` (many_body_chern_number.jl:82-131 and the selection
  step of charge_pump.jl:288-303) -- every momentum sector solved at one flux,
  the globally lowest ``manifold_size`` states selected and their isolation
  gap checked;
* ``many_body_chern_number`` (many_body_chern_number.jl:166-257) and
  ``flux_charge_pump`` (charge_pump.jl:228-386), without the reference's
  checkpoint files and figures.

Sector eigenpairs come from ``MatrixFreeHamiltonian.solve`` (the reference's
dense branch for sectors up to 500 states, Lanczos above), Fock expansions from
``expand_sector_state_to_fock``.  Errors follow the reference's: a closed
manifold gap, a singular Berry link or a singular projected position operator
raises ``ValueError``.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from . import api as A
from . import lattice as L
from ._lib import check
from .groups import statistics_from_name


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------ position operator
def many_body_position_phases(lattice: L.Real_Space_Lattice, direction: int,
                              include_sublattice: bool = True) -> np.ndarray:
    """exp(2 pi i x_{j, d}) for every site j (charge_pump.jl:17-33): x is the
    crystal coordinate of the site's cell along ``direction`` (1-based), plus
    the sublattice offset, over the sample length along that direction."""
    if not 1 <= direction <= lattice.dim:
        raise ValueError(f"direction must be in 1:{lattice.dim}.")
    Ld = float(lattice.sample_size[direction - 1])
    ph = np.empty(lattice.n_site, dtype=np.complex128)
    for i, (cell, sub) in enumerate(lattice.site_list):
        x = float(cell[direction - 1])
        if include_sublattice:
            x += float(lattice.sub_crys(sub)[direction - 1])
        ph[i] = np.exp(2j * math.pi * x / Ld)
    return ph


def position_operator_matrix(basis_to: A.Symmetry_Sector_Basis, basis_from: A.Symmetry_Sector_Basis,
                             site_phases: np.ndarray):
    """<chi_to|U_d|chi_from> (charge_pump.jl:47-91) as a scipy CSC matrix of
    shape (dim_to, dim_from); evaluated on the device."""
    import scipy.sparse as sp

    if basis_to.catalog is not basis_from.catalog:
        raise ValueError("both sectors must come from the same orbit catalog")
    n = basis_from.dim
    ph = np.ascontiguousarray(site_phases, dtype=np.complex128)
    if ph.shape != (basis_from.catalog.symmetry_group.n_site,):
        raise ValueError("one site phase per site")
    rows = np.zeros(max(n, 1), dtype=np.int64)
    vals = np.zeros(max(n, 1), dtype=np.complex128)
    if n:
        check(_lib.load().sed_position_operator(basis_to.handle, basis_from.handle, _ptr(ph), _ptr(rows),
                                                _ptr(vals)))
    keep = rows[:n] >= 0
    cols = np.nonzero(keep)[0]
    return sp.csc_matrix((vals[:n][keep], (rows[:n][keep], cols)), shape=(basis_to.dim, n))


# ------------------------------------------------------------------ overlaps
def subspace_overlap_matrix(states_a: Sequence[np.ndarray], states_b: Sequence[np.ndarray]) -> np.ndarray:
    """M_ij = <a_i|b_j> of dense Fock-amplitude vectors
    (many_body_chern_number.jl:46-71); evaluated on the device."""
    if len(states_a) != len(states_b):
        raise ValueError("Chern link compares subspaces of different dimensions.")
    a = np.ascontiguousarray(np.stack([np.asarray(s, dtype=np.complex128) for s in states_a]))
    b = np.ascontiguousarray(np.stack([np.asarray(s, dtype=np.complex128) for s in states_b]))
    if a.shape[1] != b.shape[1]:
        raise ValueError("states over different Fock spaces")
    m = np.zeros((a.shape[0], b.shape[0]), dtype=np.complex128)
    check(_lib.load().sed_fock_overlaps(_ptr(a), a.shape[0], _ptr(b), b.shape[0], a.shape[1], 0, _ptr(m)))
    return m


def unit_det_link(states_a, states_b, det_atol: float = 1e-10) -> Tuple[complex, float]:
    """det of the overlap matrix, as a unit phase and its modulus
    (many_body_chern_number.jl:73-80)."""
    z = np.linalg.det(subspace_overlap_matrix(states_a, states_b))
    if abs(z) <= det_atol:
        raise ValueError(f"Singular Berry link (|det|={abs(z)}); refine the grid or select an isolated manifold.")
    return z / abs(z), abs(z)


# ---------------------------------------------------------- one flux point
class FluxPoint:
    """The selected manifold at one flux: energies, (sector, level) labels, the
    sector bases and eigenvectors, and the states' dense Fock amplitudes."""

    def __init__(self):
        self.energies: List[float] = []
        self.labels: List[Tuple[Tuple[int, int], int]] = []
        self.vectors: List[np.ndarray] = []
        self.bases: Dict[Tuple[int, int], A.Symmetry_Sector_Basis] = {}
        self.gap = 0.0
        self.states: List[np.ndarray] = []


def flux_point_states(spec: L.ModelSpec, flux: Sequence[float], manifold_size: int,
                      catalog: Optional[A.Symmetry_Orbit_Catalog] = None, want_fock: bool = True,
                      tol: float = 1e-10) -> FluxPoint:
    """Solve every momentum sector at ``flux`` for manifold_size + 1 levels,
    select the globally lowest ``manifold_size`` states and check the gap
    above them (many_body_chern_number.jl:82-131; charge_pump.jl:288-303)."""
    flux = tuple(float(f) for f in flux)
    G = L.build_translation_group(spec.lattice, flux)
    if catalog is None:
        catalog = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                                 particle_statistics=statistics_from_name(spec.statistics))
    terms = spec.bilinear_terms(flux)
    cands = []
    vecs: Dict[Tuple[int, int], np.ndarray] = {}
    bases: Dict[Tuple[int, int], A.Symmetry_Sector_Basis] = {}
    for irr in L.build_translation_irrep_list(G, spec.lattice):
        basis = A.build_symmetry_sector_basis(catalog, irr, group=G)
        if basis.dim == 0:
            continue
        H = A.MatrixFreeHamiltonian(basis, terms, spec.density_terms)
        vals, v, _ = H.solve(manifold_size + 1, tol=tol, want_vectors=True)
        label = tuple(int(x) for x in irr.label)
        bases[label] = basis
        vecs[label] = v
        for lev, e in enumerate(vals):
            cands.append((float(e), label, lev))
    cands.sort(key=lambda c: c[0])
    if len(cands) <= manifold_size:
        raise ValueError("Need a state above the selected manifold to check its gap.")
    pt = FluxPoint()
    pt.gap = cands[manifold_size][0] - cands[manifold_size - 1][0]
    if not pt.gap > 1e-9:
        raise ValueError(f"Low-energy manifold is not isolated at flux {list(flux)} (gap={pt.gap}).")
    pt.bases = bases
    for e, label, lev in cands[:manifold_size]:
        pt.energies.append(e)
        pt.labels.append((label, lev + 1))
        v = vecs[label][:, lev]
        pt.vectors.append(v)
        if want_fock:
            pt.states.append(A.expand_sector_state_to_fock(v, bases[label]))
    return pt


def flux_points_batched(spec: L.ModelSpec, fluxes: Sequence[Sequence[float]], manifold_size: int,
                        catalog: A.Symmetry_Orbit_Catalog, want_fock: bool = True, tol: float = 1e-10,
                        precision: str = "fp64") -> List[FluxPoint]:
    """flux_point_states for many fluxes at once: every (flux, momentum)
    sector of the list is solved in one persistent batched launch, which
    returns eigenvalues and eigenvectors (the reference solves them one at a
    time, many_body_chern_number.jl:193-210, charge_pump.jl:288-303); each
    point then selects its globally lowest manifold_size states and checks the
    gap above them as flux_point_states does."""
    from .batched import BatchedSectorSolver, flux_scan_requests

    nev = manifold_size + 1
    if nev > 6:
        raise ValueError("the batched path solves at most 6 levels per sector (manifold_size <= 5)")
    fluxes = [tuple(float(f) for f in fl) for fl in fluxes]
    reqs = flux_scan_requests(spec, fluxes)
    pairs = [(i, j) for (i, j, _) in spec.bilinear_terms()]
    solver = BatchedSectorSolver(catalog, pairs, spec.density_terms, precision=precision, nev=nev,
                                 max_requests=len(reqs))
    out = solver.run(reqs, tol=tol, want_vectors=True)
    bad = np.nonzero(out["status"] != 0)[0]
    if bad.size:
        raise RuntimeError(f"batched solve did not converge for requests {bad.tolist()}")
    n_k = len(reqs) // len(fluxes)
    pts = []
    for f, flux in enumerate(fluxes):
        cands = []
        bases: Dict[Tuple[int, int], A.Symmetry_Sector_Basis] = {}
        vecs: Dict[Tuple[int, int], np.ndarray] = {}
        for q in range(f * n_k, (f + 1) * n_k):
            r = reqs[q]
            if out["dims"][q] == 0:
                continue
            label = tuple(int(x) for x in r.irrep.label)
            basis = A.build_symmetry_sector_basis(catalog, r.irrep, group=r.group)
            if basis.dim != out["dims"][q]:
                raise RuntimeError("batched sector dimension differs from the sector basis")
            bases[label] = basis
            vecs[label] = out["evecs"][q]
            for lev in range(vecs[label].shape[1]):
                cands.append((float(out["evals"][q, lev]), label, lev))
        cands.sort(key=lambda c: c[0])
        if len(cands) <= manifold_size:
            raise ValueError("Need a state above the selected manifold to check its gap.")
        pt = FluxPoint()
        pt.gap = cands[manifold_size][0] - cands[manifold_size - 1][0]
        if not pt.gap > 1e-9:
            raise ValueError(f"Low-energy manifold is not isolated at flux {list(flux)} (gap={pt.gap}).")
        pt.bases = bases
        for e, label, lev in cands[:manifold_size]:
            pt.energies.append(e)
            pt.labels.append((label, lev + 1))
            v = vecs[label][:, lev]
            pt.vectors.append(v)
            if want_fock:
                pt.states.append(A.expand_sector_state_to_fock(v, bases[label]))
        pts.append(pt)
    return pts


# ------------------------------------------------------------ Chern number
def many_body_chern_number(spec: L.ModelSpec, manifold_size: int, flux_grid_size=(5, 5),
                           det_atol: float = 1e-10, solver: str = "batch") -> dict:
    """Fukui-Hatsugai-Suzuki Chern number of the globally lowest
    ``manifold_size`` states over the flux torus
    (many_body_chern_number.jl:166-257): U(1) links are the phases of the
    overlap-matrix determinants between neighbouring flux points, the
    curvature is the plaquette phase, and C = sum / 2 pi.  solver="batch"
    solves the whole grid's sectors in one batched launch (FP64);
    solver="single" one sector at a time."""
    if isinstance(flux_grid_size, int):
        nx = ny = int(flux_grid_size)
    else:
        nx, ny = int(flux_grid_size[0]), int(flux_grid_size[1])
    if nx < 2 or ny < 2:
        raise ValueError("flux_grid_size must be at least 2 in both directions.")
    if manifold_size <= 0:
        raise ValueError("manifold_size must be positive.")
    G0 = L.build_translation_group(spec.lattice)
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G0,
                                         particle_statistics=statistics_from_name(spec.statistics))
    fx = [ix / nx for ix in range(nx)]
    fy = [iy / ny for iy in range(ny)]
    if solver == "batch" and manifold_size + 1 <= 6:
        flat = flux_points_batched(spec, [(fx[ix], fy[iy]) for ix in range(nx) for iy in range(ny)],
                                   manifold_size, cat)
        pts = [[flat[ix * ny + iy] for iy in range(ny)] for ix in range(nx)]
    else:
        pts = [[flux_point_states(spec, (fx[ix], fy[iy]), manifold_size, catalog=cat) for iy in range(ny)]
               for ix in range(nx)]
    Ux = np.zeros((nx, ny), dtype=np.complex128)
    Uy = np.zeros((nx, ny), dtype=np.complex128)
    dx = np.zeros((nx, ny))
    dy = np.zeros((nx, ny))
    for ix in range(nx):
        for iy in range(ny):
            ixp, iyp = (ix + 1) % nx, (iy + 1) % ny
            Ux[ix, iy], dx[ix, iy] = unit_det_link(pts[ix][iy].states, pts[ixp][iy].states, det_atol)
            Uy[ix, iy], dy[ix, iy] = unit_det_link(pts[ix][iy].states, pts[ix][iyp].states, det_atol)
    curv = np.zeros((nx, ny))
    for ix in range(nx):
        for iy in range(ny):
            ixp, iyp = (ix + 1) % nx, (iy + 1) % ny
            curv[ix, iy] = np.angle(Ux[ix, iy] * Uy[ixp, iy] * np.conj(Ux[ix, iyp]) * np.conj(Uy[ix, iy]))
    gaps = np.array([[pts[ix][iy].gap for iy in range(ny)] for ix in range(nx)])
    c = float(curv.sum() / (2 * math.pi))
    return {"chern_number": c, "rounded_chern": int(round(c)), "manifold_size": manifold_size,
            "berry_curvature": curv, "gaps": gaps, "min_gap": float(gaps.min()),
            "min_link_det": float(min(dx.min(), dy.min())), "link_det_abs_x": dx, "link_det_abs_y": dy,
            "flux_x": fx, "flux_y": fy, "flux_grid_size": (nx, ny),
            "selected_states": [[pts[ix][iy].labels for iy in range(ny)] for ix in range(nx)],
            "energies": [[pts[ix][iy].energies for iy in range(ny)] for ix in range(nx)]}


# --------------------------------------------------------------- charge pump
def _best_phase_permutation(raw: np.ndarray, prev: np.ndarray) -> List[int]:
    """Brute-force assignment of the new phases to the previous branches that
    minimises sum (d - round(d))^2 (charge_pump.jl:123-155)."""
    nb = len(prev)
    best, best_cost = list(range(nb)), math.inf
    used = [False] * nb
    cur = [0] * nb

    def visit(depth: int, cost: float):
        nonlocal best, best_cost
        if depth == nb:
            if cost < best_cost:
                best_cost = cost
                best = list(cur)
            return
        for j in range(nb):
            if used[j]:
                continue
            d = raw[j] - prev[depth]
            d -= round(d)
            nxt = cost + d * d
            if nxt >= best_cost:
                continue
            used[j] = True
            cur[depth] = j
            visit(depth + 1, nxt)
            used[j] = False

    visit(0, 0.0)
    return best


def _tracked_phase_branches(raw_phases: np.ndarray) -> np.ndarray:
    """Unwrap phase branches along the flux path (charge_pump.jl:100-121)."""
    n_theta, nb = raw_phases.shape
    tracked = np.zeros_like(raw_phases)
    order0 = np.argsort(raw_phases[0], kind="stable")
    tracked[0] = raw_phases[0, order0]
    prev = tracked[0].copy()
    for it in range(1, n_theta):
        perm = _best_phase_permutation(raw_phases[it], prev)
        for b in range(nb):
            phi = raw_phases[it, perm[b]]
            tracked[it, b] = phi + round(prev[b] - phi)
        prev = tracked[it].copy()
    return tracked


def flux_charge_pump(spec: L.ModelSpec, manifold_size: int, flux_direction: int = 1,
                     polarization_direction: Optional[int] = None,
                     twisted_phases_over_2pi_list: Optional[Sequence[float]] = None,
                     polarization_atol: float = 1e-10, include_sublattice: bool = True,
                     solver: str = "batch") -> dict:
    """Many-body charge pump (charge_pump.jl:228-386): at every flux along
    ``flux_direction`` the globally lowest ``manifold_size`` states are
    selected, Resta's position operator along ``polarization_direction`` is
    projected into them, and the phases of its eigenvalues are unwrapped along
    the path; the pumped charges are the end-to-start differences."""
    lat = spec.lattice
    dim = lat.dim
    if polarization_direction is None:  # _default_polarization_direction
        polarization_direction = flux_direction if dim == 1 else (flux_direction % dim) + 1
    if not 1 <= flux_direction <= dim or not 1 <= polarization_direction <= dim:
        raise ValueError(f"directions must be in 1:{dim}.")
    if manifold_size <= 0:
        raise ValueError("manifold_size must be positive.")
    fluxes = list(twisted_phases_over_2pi_list) if twisted_phases_over_2pi_list is not None else \
        list(np.linspace(0.0, 1.0, 9))
    G0 = L.build_translation_group(lat)
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G0,
                                         particle_statistics=statistics_from_name(spec.statistics))
    site_phases = many_body_position_phases(lat, polarization_direction, include_sublattice)
    gaps, min_sv, selected = [], [], []
    pol_eigs = np.zeros((len(fluxes), manifold_size), dtype=np.complex128)
    path = []
    for th in fluxes:
        flux = [0.0] * dim
        flux[flux_direction - 1] = float(th)
        path.append(flux)
    if solver == "batch" and manifold_size + 1 <= 6:  # the whole flux path in one batched launch
        batched = flux_points_batched(spec, path, manifold_size, cat, want_fock=False)
    for it, th in enumerate(fluxes):
        if solver == "batch" and manifold_size + 1 <= 6:
            pt = batched[it]
        else:
            pt = flux_point_states(spec, path[it], manifold_size, catalog=cat, want_fock=False)
        gaps.append(pt.gap)
        selected.append(list(pt.labels))
        blocks = {}
        P = np.zeros((manifold_size, manifold_size), dtype=np.complex128)
        for r, (lt, _) in enumerate(pt.labels):
            for c, (lf, _) in enumerate(pt.labels):
                key = (lt, lf)
                if key not in blocks:
                    blocks[key] = position_operator_matrix(pt.bases[lt], pt.bases[lf], site_phases)
                P[r, c] = np.vdot(pt.vectors[r], blocks[key] @ pt.vectors[c])
        sv = float(np.linalg.svd(P, compute_uv=False).min())
        min_sv.append(sv)
        if not sv > polarization_atol:
            raise ValueError(f"Projected Resta operator is singular at flux index {it + 1}; "
                             "polarization is undefined.")
        ev = np.linalg.eigvals(P)
        pol_eigs[it] = ev[np.argsort(np.angle(ev), kind="stable")]
    raw = np.angle(pol_eigs) / (2 * math.pi)
    pol = _tracked_phase_branches(raw)
    traj = pol - pol[0:1, :]
    return {"twisted_phases_over_2pi_list": fluxes, "flux_direction": flux_direction,
            "polarization_direction": polarization_direction, "manifold_size": manifold_size,
            "selected_states": selected, "gaps": gaps, "min_gap": float(min(gaps)),
            "min_position_singular_values": min_sv, "polarization_eigenvalues": pol_eigs,
            "polarizations": pol, "pumped_charge_trajectories": traj, "pumped_charges": traj[-1].copy(),
            "include_sublattice": include_sublattice}
