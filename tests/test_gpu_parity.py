"""Device parity against the CPU oracle (restatement of the reference).

Integer and bitmask tables must match bit for bit; amplitude tables too (both
sides use separately rounded complex products in the reference's order);
matvecs within 1e-11 relative; eigenvalues within 1e-10 of a dense
diagonalisation of the oracle's matrix-mode sector block.
"""
import numpy as np
import pytest

from cases import assert_lanczos_spectrum, case_by_name, oracle_objects, small_cases, x_ramp, x_random

pytestmark = pytest.mark.gpu

CASES = [c.name for c in small_cases()]


def _device(case, sector=None, precision="fp64"):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    st = statistics_from_name(case.statistics)
    G = case.group()
    cat = A.build_symmetry_orbit_catalog(n_filled=case.spec.n_filled, species=case.spec.species, symmetry_group=G, particle_statistics=st)
    if sector is None:
        return cat
    basis = A.build_symmetry_sector_basis(cat, case.irreps()[sector])
    H = A.MatrixFreeHamiltonian(basis, case.bilinear1(), case.density1(), None, precision=precision)
    return cat, basis, H


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64) if a.dtype == np.complex128 else a


@pytest.mark.parametrize("name", CASES)
def test_catalog_tables_bit_exact(oracle, name):
    case = case_by_name(name)
    G = case.group()
    oc = oracle.Catalog(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code, case.spec.n_filled)
    dc = _device(case)
    assert dc.n_states == oc.n_states
    assert dc.n_orbits == oc.n_orbits
    np.testing.assert_array_equal(dc.representative_mask_list, oc.get(oracle.FIELD_REPS))
    np.testing.assert_array_equal(dc.stabilizer_order_list, oc.get(oracle.FIELD_STAB_ORDER))
    np.testing.assert_array_equal(dc._get(2), oc.get(oracle.FIELD_STAB_PTR))
    np.testing.assert_array_equal(dc._get(3), oc.get(oracle.FIELD_STAB_G))
    np.testing.assert_array_equal(bits(dc._get(4)), bits(oc.get(oracle.FIELD_STAB_PHASE)))
    np.testing.assert_array_equal(dc.rep_rank_table, oc.get(oracle.FIELD_REP_RANK))
    np.testing.assert_array_equal(dc.rep_sym_table, oc.get(oracle.FIELD_REP_SYM))
    np.testing.assert_array_equal(bits(dc.rep_amp_table), bits(oc.get(oracle.FIELD_REP_AMP)))


@pytest.mark.parametrize("name", CASES)
def test_sector_bases_bit_exact(oracle, name):
    import realspace_exactdiagonalization_gb300.api as A

    case = case_by_name(name)
    G = case.group()
    oc = oracle.Catalog(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code, case.spec.n_filled)
    dc = _device(case)
    for irr in case.irreps():
        osec = oracle.Sector(oc, irr.array())
        dsec = A.build_symmetry_sector_basis(dc, irr)
        reps, stab, orb = osec.arrays()
        assert dsec.dim == osec.dim, irr.label
        np.testing.assert_array_equal(dsec.representative_mask_list, reps)
        np.testing.assert_array_equal(dsec.stabilizer_order_list, stab)
        np.testing.assert_array_equal(dsec.orbit_index_list, orb)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_matvec_matches_oracle(oracle, name, precision):
    case = case_by_name(name)
    for k in range(len(case.irreps())):
        _, _, op = oracle_objects(oracle, case, k)
        if op.dim == 0:
            continue
        _, _, H = _device(case, k, precision)
        for x in (x_ramp(op.dim), x_random(op.dim, seed=k)):
            y_tab = op.apply(x, mode=0)
            y_fly = op.apply(x, mode=1)
            y = H(x)
            scale = max(1.0, np.abs(y_tab).max())
            tol = 1e-11 if precision == "fp64" else 3e-6
            assert np.abs(y_tab - y_fly).max() <= 1e-11 * scale
            assert np.abs(y - y_tab).max() <= tol * scale, (name, k, precision)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hop_table_matvec_matches_oracle(oracle, name, precision):
    """The operator's stored hop table (8 bytes per hop, the compressed
    projection table of SRE:680-765) gives the same matvec as the oracle and,
    to rounding, as the on-the-fly gather."""
    case = case_by_name(name)
    for k in range(len(case.irreps())):
        _, _, op = oracle_objects(oracle, case, k)
        if op.dim == 0:
            continue
        _, _, H = _device(case, k, precision)
        x = x_random(op.dim, seed=100 + k)
        y_fly = H(x)
        H.set_hop_table(H.HOP_TABLE_NOW)
        info = H.hop_table_info()
        assert info["built"] and info["records"] >= H.info()["hops"]
        y = H(x)
        y_ref = op.apply(x, mode=0)
        scale = max(1.0, np.abs(y_ref).max())
        tol = 1e-11 if precision == "fp64" else 3e-6
        assert np.abs(y - y_ref).max() <= tol * scale, (name, k, precision)
        assert np.abs(y - y_fly).max() <= (1e-13 if precision == "fp64" else 1e-6) * scale, (name, k, precision)
        H.set_hop_table(H.HOP_TABLE_OFF)
        assert not H.hop_table_info()["built"]


@pytest.mark.parametrize("name", CASES)
def test_eigenvalues_match_dense(oracle, name):
    """Sectors up to 500 take the reference's dense branch (SRE:1004-1017):
    exactly the lowest nev eigenvalues with multiplicity.  Larger sectors take
    Lanczos: see assert_lanczos_spectrum."""
    case = case_by_name(name)
    for k in range(len(case.irreps())):
        _, _, op = oracle_objects(oracle, case, k)
        if op.dim == 0:
            continue
        Hd = op.dense()
        assert np.abs(Hd - Hd.conj().T).max() < 1e-11
        ref = np.linalg.eigvalsh(Hd)
        nev = min(4, op.dim)
        for precision in ("fp64", "mixed"):
            _, _, H = _device(case, k, precision)
            vals, vecs, info = H.solve(nev, tol=1e-10)
            tol = 1e-9 * max(1.0, abs(ref[0]))
            if op.dim <= 500:
                np.testing.assert_allclose(vals, ref[:nev], atol=tol, rtol=0, err_msg=f"{name} k={k} {precision}")
            else:
                assert_lanczos_spectrum(vals, ref, tol, f"{name} k={k} {precision}")
            for i in range(len(vals)):
                r = Hd @ vecs[:, i] - vals[i] * vecs[:, i]
                bound = 1e-7 if (precision == "fp64" or op.dim <= 500) else 1e-4
                assert np.linalg.norm(r) < bound * max(1.0, abs(vals[i])), (name, k, precision, i)


def test_ring16_k0_lowest_four_eigenvalues_within_1e12(oracle):
    """Plain method on the 16-site ring of hard-core bosons (t = 1, V = 2,
    8 particles, k = 0, 810 representatives): the sector and its tables are
    bit-exact (test_catalog_tables_bit_exact, test_sector_bases_bit_exact), and
    the FP64 device Lanczos (810 > 500 rows, so not the dense branch) gives the
    lowest four eigenvalues within 1e-12 (absolute) of a dense diagonalisation
    of the oracle's matrix-mode block, from a seeded Gaussian start vector.
    These four levels are non-degenerate, so the Lanczos and the reference's
    matrix mode list the same values."""
    case = case_by_name("ring16")
    _, _, op = oracle_objects(oracle, case, 0)
    assert op.dim == 810
    ref = np.linalg.eigvalsh(op.dense())
    assert np.min(np.diff(ref[:5])) > 1e-3  # no degenerate copies among them
    for seed in (0, 1, 12345):
        _, _, H = _device(case, 0, "fp64")
        vals, vecs, info = H.solve(4, tol=1e-10, seed=seed)
        assert np.abs(vals - ref[:4]).max() <= 1e-12, (seed, vals - ref[:4])
        assert info.n_restarts >= 0 and info.converged == 4


def test_lanczos_odd_orbit_count(oracle):
    """A catalog with an odd orbit count: a ring of 16 sites with 7 particles
    at a twist, 715 orbits, every sector above the dense branch's 500 rows.
    The mixed solve's vector kernels take element pairs plus the last element
    alone; both precisions give the oracle's lowest eigenvalues."""
    from cases import Case
    from realspace_exactdiagonalization_gb300 import lattice as L

    case = Case("ring16_7", L.ring_xxz(16, 1.0, 2.0, n_filled=7), theta=(0.21, 0.0))
    for k in (0, 3):
        _, _, op = oracle_objects(oracle, case, k)
        ref = np.linalg.eigvalsh(op.dense())
        for precision in ("fp64", "mixed"):
            cat, basis, H = _device(case, k, precision)
            assert cat.n_orbits == 715 and basis.dim > 500
            vals, vecs, _ = H.solve(3, tol=1e-10)
            assert_lanczos_spectrum(vals, ref, 1e-9 * max(1.0, abs(ref[0])), f"k={k} {precision}")
            for i in range(len(vals)):
                r = op.dense() @ vecs[:, i] - vals[i] * vecs[:, i]
                assert np.linalg.norm(r) < (1e-7 if precision == "fp64" else 1e-4) * max(1.0, abs(vals[i]))


def test_mixed_solve_without_hop_table(oracle):
    """The mixed solve with the operator's hop table switched off: each
    matvec is the on-the-fly gather with an FP64 output, converted to the
    complex64 work vector.  Same lowest eigenvalues as the oracle."""
    from cases import Case
    from realspace_exactdiagonalization_gb300 import lattice as L

    case = Case("ring16_7", L.ring_xxz(16, 1.0, 2.0, n_filled=7), theta=(0.21, 0.0))
    for k in (1, 5):
        _, _, op = oracle_objects(oracle, case, k)
        ref = np.linalg.eigvalsh(op.dense())
        _, basis, H = _device(case, k, "mixed")
        H.set_hop_table(H.HOP_TABLE_OFF)
        vals, _, _ = H.solve(3, tol=1e-10)
        assert not H.hop_table_info()["built"]
        assert_lanczos_spectrum(vals, ref, 1e-9 * max(1.0, abs(ref[0])), f"k={k}")


def test_sector_union_equals_full_spectrum(oracle):
    """flux_regression.jl:46 on the device: the union of the device sector
    spectra equals the identity-group (full Fock) spectrum at a twisted flux."""
    case = case_by_name("checkerboard3x2_f_flux")
    G = case.group()
    from realspace_exactdiagonalization_gb300.groups import build_identity_group

    Gid = build_identity_group(G.n_site)
    ocat = oracle.Catalog(Gid.perm0(), Gid.phases(), 0, case.stats_code, case.spec.n_filled)
    osec = oracle.Sector(ocat, np.array([1.0 + 0j]))
    full = np.linalg.eigvalsh(oracle.Op(osec, case.bilinear0(), case.density0()).dense())
    allv = []
    for k in range(len(case.irreps())):
        _, basis, H = _device(case, k)
        n = basis.dim
        M = np.zeros((n, n), dtype=np.complex128)
        for j in range(n):
            e = np.zeros(n, dtype=np.complex128)
            e[j] = 1.0
            M[:, j] = H(e)
        assert np.abs(M - M.conj().T).max() < 1e-11
        allv.extend(np.linalg.eigvalsh(M))
    np.testing.assert_allclose(np.sort(allv), full, atol=1e-10)


def test_golden_haldane3x4_ground_energy():
    """The config-4 model at zero flux, sector k=(0,0): the reference's stored
    E0 = -14.301456146831118 (benchmark_raw.csv:20-21), tolerance 1e-11 (FP64)
    and |dE|/|E| <= 1e-9 (mixed precision)."""
    from cases import Case
    from realspace_exactdiagonalization_gb300 import lattice as L

    case = Case("haldane3x4", L.haldane_honeycomb(3, 4))
    for precision, tol in (("fp64", 1e-11), ("mixed", 14.3 * 1e-9)):
        _, basis, H = _device(case, 0, precision)
        assert basis.dim == 11240
        vals, _, info = H.solve(4, tol=1e-10)
        assert abs(vals[0] - (-14.301456146831118)) <= tol, (precision, vals[0], info.max_residual)


@pytest.mark.parametrize("name", ["checkerboard3x2_f_flux", "checkerboard3x2_b_flux", "hubbard2x3"])
def test_project_to_sector_bit_exact(oracle, name):
    """project_to_sector (SRE:627-632) for every basis state, every sector:
    same row and bit-identical coefficient as the oracle's table path, which
    itself equals the O(|G|) path (flux_regression.jl:36-44)."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.groups import build_identity_group

    case = case_by_name(name)
    G = case.group()
    Gid = build_identity_group(G.n_site)
    masks = oracle.Catalog(Gid.perm0(), Gid.phases(), 0, case.stats_code, case.spec.n_filled).get(oracle.FIELD_REPS)
    oc = oracle.Catalog(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code, case.spec.n_filled)
    dc = _device(case)
    for irr in case.irreps():
        osec = oracle.Sector(oc, irr.array())
        rows, coeff = A.build_symmetry_sector_basis(dc, irr).project(masks)
        for m, r, c in zip(masks, rows, coeff):
            ref = osec.project(int(m), 0)
            if ref is None:
                assert r == 0
            else:
                assert r == ref[0] + 1
                assert np.array([c]).view(np.uint64).tolist() == np.array([ref[1]]).view(np.uint64).tolist()


def test_flux_refresh_matches_fresh_build(oracle):
    """update_orbit_stabilizer_phases! (SRE:338-369): a catalog built at zero
    flux and refreshed to a twisted group equals one built at that twist."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    case = case_by_name("checkerboard3x2_f_flux")
    spec = case.spec
    st = statistics_from_name(case.statistics)
    from realspace_exactdiagonalization_gb300 import lattice as L

    G0 = L.build_translation_group(spec.lattice, (0.0, 0.0))
    Gt = case.group()
    dc = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G0, particle_statistics=st)
    A.update_orbit_stabilizer_phases_(dc, Gt, st)
    oc = oracle.Catalog(G0.perm0(), G0.phases(), 0, case.stats_code, spec.n_filled)
    oc.update_phases(Gt.phases())
    fresh = oracle.Catalog(Gt.perm0(), Gt.phases(), 0, case.stats_code, spec.n_filled)
    for f in (oracle.FIELD_STAB_PHASE, oracle.FIELD_REP_SYM, oracle.FIELD_REP_AMP):
        np.testing.assert_array_equal(bits(oc.get(f)), bits(fresh.get(f)))
        np.testing.assert_array_equal(bits(dc._get(f)), bits(fresh.get(f)))
    for k, irr in enumerate(case.irreps()):
        dsec = A.build_symmetry_sector_basis(dc, irr)
        osec = oracle.Sector(fresh, irr.array())
        assert dsec.dim == osec.dim
        H = A.MatrixFreeHamiltonian(dsec, case.bilinear1(), case.density1())
        op = oracle.Op(osec, case.bilinear0(), case.density0())
        x = x_random(osec.dim, seed=k)
        assert np.abs(H(x) - op.apply(x)).max() < 1e-11 * max(1, np.abs(op.apply(x)).max())


SHAPES = [(1, 512), (1, 256), (2, 512), (2, 256), (4, 512), (4, 256), (8, 512), (8, 256)]


@pytest.mark.parametrize("name", ["checkerboard3x2_f_flux", "hubbard2x4_flux", "ring16"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gather_launch_shapes_match_oracle(oracle, name, precision):
    """Every launch shape of the matrix-free gather (threads per row x threads
    per block) gives the oracle's matvec; the autotuner's choice is one of
    them."""
    case = case_by_name(name)
    for k in (0, 1):
        _, _, op = oracle_objects(oracle, case, k)
        if op.dim == 0:
            continue
        _, _, H = _device(case, k, precision)
        H.set_hop_table(H.HOP_TABLE_OFF)
        x = x_random(op.dim, seed=7 + k)
        ref = op.apply(x, mode=0)
        scale = max(1.0, np.abs(ref).max())
        tol = 1e-11 if precision == "fp64" else 3e-6
        y = H(x)  # autotuned
        assert H.apply_shape(precision == "mixed") in SHAPES
        assert np.abs(y - ref).max() <= tol * scale
        for tpr, block in SHAPES:
            H.set_apply_shape(tpr, block)
            y = H(x)
            assert H.apply_shape(precision == "mixed") == (tpr, block)
            assert np.abs(y - ref).max() <= tol * scale, (name, k, precision, tpr, block)
        H.set_apply_shape(0, 0)


@pytest.mark.parametrize("spec_name,n_filled", [("ring16", 0), ("ring16", 16), ("checkerboard3x2_f_flux", 0),
                                                ("checkerboard3x2_f_flux", 12), ("checkerboard3x2_b_flux", 12)])
def test_empty_and_full_fillings(oracle, spec_name, n_filled):
    """n_filled = 0 or n_site, the reference's special case (SRE:410-431: one
    orbit whose stabilizer is the whole group): the catalog tables bit for bit,
    every momentum sector's basis (the one orbit belongs to the sectors whose
    characters match its stabilizer phases -- at flux, the product of the
    twist phases over all sites), and in each non-empty sector the matvec and
    the single eigenvalue against the oracle."""
    import dataclasses

    import realspace_exactdiagonalization_gb300.api as A

    base = case_by_name(spec_name)
    case = dataclasses.replace(base, name=f"{spec_name}_n{n_filled}",
                               spec=dataclasses.replace(base.spec, n_filled=n_filled))
    G = case.group()
    oc = oracle.Catalog(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code, n_filled)
    dc = _device(case)
    assert dc.n_states == oc.n_states == 1 and dc.n_orbits == oc.n_orbits == 1
    np.testing.assert_array_equal(dc.representative_mask_list, oc.get(oracle.FIELD_REPS))
    np.testing.assert_array_equal(dc.stabilizer_order_list, oc.get(oracle.FIELD_STAB_ORDER))
    np.testing.assert_array_equal(dc._get(3), oc.get(oracle.FIELD_STAB_G))
    np.testing.assert_array_equal(bits(dc._get(4)), bits(oc.get(oracle.FIELD_STAB_PHASE)))
    np.testing.assert_array_equal(dc.rep_rank_table, oc.get(oracle.FIELD_REP_RANK))
    np.testing.assert_array_equal(dc.rep_sym_table, oc.get(oracle.FIELD_REP_SYM))
    np.testing.assert_array_equal(bits(dc.rep_amp_table), bits(oc.get(oracle.FIELD_REP_AMP)))
    nonempty = 0
    for k, irr in enumerate(case.irreps()):
        osec = oracle.Sector(oc, irr.array())
        dsec = A.build_symmetry_sector_basis(dc, irr)
        assert dsec.dim == osec.dim, (case.name, k)
        if osec.dim == 0:
            continue
        nonempty += 1
        np.testing.assert_array_equal(dsec.representative_mask_list, osec.arrays()[0])
        op = oracle.Op(osec, case.bilinear0(), case.density0())
        H = A.MatrixFreeHamiltonian(dsec, case.bilinear1(), case.density1(), None, precision="fp64")
        x = np.array([0.6 - 0.8j])
        y_ref = op.apply(x, mode=0)
        assert abs(H(x)[0] - y_ref[0]) <= 1e-12 * max(1.0, abs(y_ref[0])), (case.name, k)
        vals, _, _ = H.solve(1, tol=1e-10, seed=1, want_vectors=False)
        e = np.linalg.eigvalsh(op.dense())[0]
        assert abs(vals[0] - e) <= 1e-12 * max(1.0, abs(e)), (case.name, k)
    assert nonempty >= 1
    # the same one-orbit catalog through the batched solver (a hop table
    # without records), mixed precision, every momentum at two twists
    from realspace_exactdiagonalization_gb300.batched import BatchedSectorSolver, flux_scan_requests

    twists = [(0.0, 0.0), (0.3, 0.1)]
    reqs = flux_scan_requests(case.spec, twists)
    pairs = [(i, j) for (i, j, _) in case.spec.bilinear_terms()]
    solver = BatchedSectorSolver(dc, pairs, case.spec.density_terms, precision="mixed", nev=1, max_requests=64)
    out = solver.run(reqs)
    assert (out["status"] == 0).all()
    nk = len(reqs) // len(twists)
    for b in range(len(reqs)):
        tcase = dataclasses.replace(case, theta=twists[b // nk])
        _, osec, op = oracle_objects(oracle, tcase, b % nk)
        assert out["dims"][b] == osec.dim, (case.name, b)
        if osec.dim:
            e = np.linalg.eigvalsh(op.dense())[0]
            assert abs(out["evals"][b, 0] - e) <= 1e-10 * max(1.0, abs(e)), (case.name, b)
        else:
            assert np.isnan(out["evals"][b, 0])


def test_mixed_solve_on_an_odd_large_catalog():
    """A mixed-precision solve whose catalog is large enough for the staged
    (bulk-copy) dot sweeps and has an odd orbit count, so the last element of
    every vector sits alone in its pair: ring29 with 13 hard-core bosons
    (C(29,13)/29 = 2,340,135 orbits), momentum 0.  The lowest eigenvalues agree
    with the FP64 solve within the mixed path's 1e-9 relative."""
    import realspace_exactdiagonalization_gb300.api as A
    import realspace_exactdiagonalization_gb300.lattice as L

    spec = L.ring_xxz(29, 1.0, 2.0, n_filled=13)
    G = L.build_translation_group(spec.lattice)
    cat = A.build_symmetry_orbit_catalog(n_filled=13, symmetry_group=G, particle_statistics=A.Bosonic())
    assert cat.n_orbits == 2340135 and cat.n_orbits % 2 == 1
    basis = A.build_symmetry_sector_basis(cat, L.build_translation_irrep_list(G, spec.lattice)[0])
    vals = {}
    for prec in ("fp64", "mixed"):
        H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms(), spec.density_terms, precision=prec)
        vals[prec], _, info = H.solve(3, tol=1e-10, want_vectors=False)
        del H
    np.testing.assert_allclose(vals["mixed"], vals["fp64"], rtol=1e-9, atol=0)
