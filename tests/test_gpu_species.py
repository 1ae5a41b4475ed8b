"""Two-species catalogs: the (N_up, N_down) blocks of the Hubbard model.

The reference fixes only the total particle number (SRE:1460-1466), so its
Hubbard catalog holds every S^z at once.  sed_catalog_build_species keeps one
(N_up, N_down) block.  Its tables must equal the reference's total-particle
tables restricted to the masks of that block, bit for bit: the same
representatives in the same (ascending) order, the same stabilizers, the same
rep_sym / rep_amp entries per mask, and REP_RANK pointing to the same orbit
(renumbered within the block).  Hopping conserves each species, so the sector
Hamiltonian is the restriction of the oracle's block-diagonal sector matrix,
and the ground energies of the half-filled S^z = 0 blocks equal the stored
energies of the reference's benchmark (the ground state has S = 0).
"""
import json
import os

import numpy as np
import pytest

from cases import Case, assert_lanczos_spectrum, x_random

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")))


def _cases():
    from realspace_exactdiagonalization_gb300 import lattice as L

    # split at 8 (chunk-aligned) and at 6 (a rank-table chunk straddles the
    # species boundary); empty and full species blocks as edge cases
    return [
        Case("hubbard2x4_4u4d_flux", L.hubbard_square(2, 4, n_up=4, n_dn=4), theta=(0.3, 0.1)),
        Case("hubbard2x4_3u5d", L.hubbard_square(2, 4, n_up=3, n_dn=5)),
        Case("hubbard3x2_3u3d_flux", L.hubbard_square(3, 2, n_up=3, n_dn=3), theta=(0.23, 0.17)),
        Case("hubbard3x2_0u3d", L.hubbard_square(3, 2, n_up=0, n_dn=3)),
        Case("hubbard3x2_6u2d", L.hubbard_square(3, 2, n_up=6, n_dn=2)),
    ]


CASES = {c.name: c for c in _cases()}


def _restriction(oracle, case):
    """The oracle's total-particle catalog and the block's orbits in it."""
    G = case.group()
    n_split, n_lo, _ = case.spec.species
    oc = oracle.Catalog(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code, case.spec.n_filled)
    reps = oc.get(oracle.FIELD_REPS)
    low = reps & np.uint64((1 << n_split) - 1)
    keep = np.array([bin(int(m)).count("1") == n_lo for m in low], dtype=bool)
    return oc, keep


def _device_catalog(case):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    return A.build_symmetry_orbit_catalog(n_filled=case.spec.n_filled, species=case.spec.species,
                                          symmetry_group=case.group(),
                                          particle_statistics=statistics_from_name(case.statistics))


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64) if a.dtype == np.complex128 else a


@pytest.mark.parametrize("name", list(CASES))
def test_species_catalog_equals_restricted_reference_catalog(oracle, name):
    import realspace_exactdiagonalization_gb300.api as A
    from math import comb

    case = CASES[name]
    n_split, n_lo, n_hi = case.spec.species
    oc, keep = _restriction(oracle, case)
    dc = _device_catalog(case)
    n_site = case.spec.lattice.n_site
    assert dc.n_states == comb(n_split, n_lo) * comb(n_site - n_split, n_hi)
    assert dc.n_orbits == int(keep.sum())
    np.testing.assert_array_equal(dc.representative_mask_list, oc.get(oracle.FIELD_REPS)[keep])
    np.testing.assert_array_equal(dc.stabilizer_order_list, oc.get(oracle.FIELD_STAB_ORDER)[keep])
    optr, og, oph = oc.get(oracle.FIELD_STAB_PTR), oc.get(oracle.FIELD_STAB_G), oc.get(oracle.FIELD_STAB_PHASE)
    sel = np.concatenate([np.arange(optr[o], optr[o + 1]) for o in np.nonzero(keep)[0]] or [np.zeros(0, int)])
    np.testing.assert_array_equal(dc._get(3), og[sel])
    np.testing.assert_array_equal(_bits(dc._get(4)), _bits(oph[sel]))
    # per basis state: the block's masks in rank order are ascending masks
    masks = A.catalog_state_masks(dc, np.arange(dc.n_states))
    assert (np.diff(masks.astype(np.int64)) > 0).all()
    oranks = np.array([oracle.rank(int(m)) for m in masks], dtype=np.int64)
    renumber = np.full(keep.size + 1, -1, dtype=np.int64)
    renumber[1:][keep] = np.arange(1, int(keep.sum()) + 1)
    np.testing.assert_array_equal(dc.rep_rank_table, renumber[oc.get(oracle.FIELD_REP_RANK)[oranks]])
    np.testing.assert_array_equal(dc.rep_sym_table, oc.get(oracle.FIELD_REP_SYM)[oranks])
    np.testing.assert_array_equal(_bits(dc.rep_amp_table), _bits(oc.get(oracle.FIELD_REP_AMP)[oranks]))


@pytest.mark.parametrize("name", list(CASES))
def test_species_sectors_matvec_and_spectra(oracle, name):
    """Every momentum sector: the block's sector rows equal the oracle's sector
    restricted to the block; the matvec equals the oracle's block-diagonal
    sector matrix restricted to the block (1e-11 FP64, 3e-6 complex64); the
    lowest eigenvalues equal a dense diagonalisation of that block."""
    import realspace_exactdiagonalization_gb300.api as A

    case = CASES[name]
    oc, keep = _restriction(oracle, case)
    dc = _device_catalog(case)
    for k, irr in enumerate(case.irreps()):
        osec = oracle.Sector(oc, irr.array())
        oreps, ostab, oorb = osec.arrays()
        rows = keep[oorb]
        dsec = A.build_symmetry_sector_basis(dc, irr)
        assert dsec.dim == int(rows.sum()), (name, k)
        np.testing.assert_array_equal(dsec.representative_mask_list, oreps[rows])
        np.testing.assert_array_equal(dsec.stabilizer_order_list, ostab[rows])
        if dsec.dim == 0:
            continue
        op = oracle.Op(osec, case.bilinear0(), case.density0())
        Hfull = op.dense()
        Hb = Hfull[np.ix_(rows, rows)]
        # hopping conserves each species: no element couples the block to the rest
        assert np.abs(Hfull[np.ix_(rows, ~rows)]).max(initial=0.0) == 0.0
        ref = np.linalg.eigvalsh(Hb)
        for precision, tol in (("fp64", 1e-11), ("mixed", 3e-6)):
            H = A.MatrixFreeHamiltonian(dsec, case.bilinear1(), case.density1(), precision=precision)
            x = x_random(dsec.dim, seed=k)
            y_ref = Hb @ x
            scale = max(1.0, np.abs(y_ref).max())
            assert np.abs(H(x) - y_ref).max() <= tol * scale, (name, k, precision)
            nev = min(3, dsec.dim)
            vals, _, _ = H.solve(nev, tol=1e-10)
            if dsec.dim <= 500:
                np.testing.assert_allclose(vals, ref[:nev], atol=1e-9 * max(1.0, abs(ref[0])), rtol=0)
            else:
                assert abs(vals[0] - ref[0]) <= 1e-9 * max(1.0, abs(ref[0])), (name, k, precision)


@pytest.mark.parametrize("label,shape,n_half", [("2\u00d74", (2, 4), 4), ("3\u00d74", (3, 4), 6)])
def test_species_half_filling_energy_matches_stored_reference_energy(label, shape, n_half):
    """benchmark_raw.csv: Hubbard k=(0,0) ground energies of the reference's
    total-particle catalogs at half filling.  The S = 0 ground state lies in the
    N_up = N_down block, which gives the same energy (FP64, 1e-10)."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300 import lattice as L

    rows = [r for r in GOLDEN["benchmark_raw"] if r["model"] == "Hubbard_Fermion" and r["label"] == label
            and r["mode"] == "matrix"]
    assert rows, label
    e_ref = rows[0]["energy"]
    spec = L.hubbard_square(*shape, n_up=n_half, n_dn=n_half)
    G = L.build_translation_group(spec.lattice)
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                         particle_statistics=A.Fermionic())
    irr = L.build_translation_irrep_list(G, spec.lattice)[0]
    basis = A.build_symmetry_sector_basis(cat, irr)
    assert basis.dim < rows[0]["sector_dim"]  # one S^z block of the reference's sector
    H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms(), spec.density_terms)
    vals, _, _ = H.solve(1, tol=1e-10)
    assert abs(vals[0] - e_ref) <= 1e-10 * max(1.0, abs(e_ref)), (vals[0], e_ref)


def test_species_rejections():
    """A group that maps one species onto the other, and a hop between the
    species, are refused with the library's messages."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300 import lattice as L
    from realspace_exactdiagonalization_gb300.groups import Finite_Symmetry_Group, Symmetry_Operation

    spec = L.hubbard_square(2, 2, n_up=1, n_dn=1)
    n = spec.lattice.n_site
    swap = list(range(n // 2 + 1, n + 1)) + list(range(1, n // 2 + 1))  # up <-> down
    G = Finite_Symmetry_Group("spin flip", [Symmetry_Operation("id", list(range(1, n + 1))),
                                            Symmetry_Operation("swap", swap)])
    with pytest.raises(_lib.SEDError, match="species"):
        A.build_symmetry_orbit_catalog(n_filled=2, species=spec.species, symmetry_group=G,
                                       particle_statistics=A.Fermionic())
    G = L.build_translation_group(spec.lattice)
    cat = A.build_symmetry_orbit_catalog(n_filled=2, species=spec.species, symmetry_group=G,
                                         particle_statistics=A.Fermionic())
    basis = A.build_symmetry_sector_basis(cat, L.build_translation_irrep_list(G, spec.lattice)[0])
    cross = [(i + 1, i + 1 + n // 2, 0.5) for i in range(n // 2)] + [(i + 1 + n // 2, i + 1, 0.5)
                                                                       for i in range(n // 2)]
    with pytest.raises(_lib.SEDError, match="species"):
        A.MatrixFreeHamiltonian(basis, cross, [])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("name", ["hubbard2x4_4u4d_flux", "hubbard3x2_3u3d_flux"])
def test_species_blocks_through_the_batch(oracle, name, precision):
    """A two-species catalog through the batched solver (its site-gauge hop
    table, bank-ordered records): every (momentum, twist) request gives the
    block's sector dimension and the spectrum of the oracle's sector matrix
    restricted to the block (Lanczos semantics, 1e-9)."""
    from realspace_exactdiagonalization_gb300.batched import BatchedSectorSolver, flux_scan_requests

    case = CASES[name]
    twists = [(0.0, 0.0), (0.3, 0.1), (0.5, 0.75)]
    reqs = flux_scan_requests(case.spec, twists)
    pairs = [(i, j) for (i, j, _) in case.spec.bilinear_terms()]
    solver = BatchedSectorSolver(_device_catalog(case), pairs, case.spec.density_terms, precision=precision, nev=3,
                                 max_requests=64)
    out = solver.run(reqs)
    assert (out["status"] == 0).all()
    assert solver.last_stats()["hop_table"]
    nk = len(reqs) // len(twists)
    for b in range(len(reqs)):
        tcase = Case(name, case.spec, theta=twists[b // nk])
        oc, keep = _restriction(oracle, tcase)
        osec = oracle.Sector(oc, tcase.irreps()[b % nk].array())
        _, _, oorb = osec.arrays()
        rows = keep[oorb]
        assert out["dims"][b] == int(rows.sum()), (name, b)
        if not rows.any():
            continue
        Hb = oracle.Op(osec, tcase.bilinear0(), tcase.density0()).dense()[np.ix_(rows, rows)]
        ref = np.linalg.eigvalsh(Hb)
        k = min(3, int(rows.sum()))
        assert_lanczos_spectrum(out["evals"][b, :k], ref, 1e-9 * max(1.0, abs(ref[0])), msg=f"{name} {b}")
