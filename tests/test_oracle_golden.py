"""Pin the CPU oracle against the reference's own stored answers.

Golden values come from tests/golden/reference_golden.json, extracted from the
reference's benchmark CSV and design notebook by tests/golden/make_golden.py.
"""
import json
import os

import numpy as np
import pytest

from cases import case_by_name, oracle_objects, x_ramp, x_random
from realspace_exactdiagonalization_gb300 import lattice as L

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")))


def test_colex_rank_table(oracle):
    """doc/design.ipynb cell 22: colex ranks of the six 2-subsets of 4 sites."""
    for mask, r in GOLD["colex_rank_n4_k2"]:
        assert oracle.rank(mask) == r
    assert oracle.rank(0b1010) == GOLD["rank_0b1010"]


def test_gosper_enumerates_colex_order(oracle):
    x = 0b111
    for r in range(oracle.binom(12, 3)):
        assert oracle.rank(x) == r
        x = oracle.gosper_next(x)


def test_lin_table_matches_rank(oracle):
    """doc/design.ipynb cell 24: LinTable == rank over C(12,3); worked example."""
    g = GOLD["lin_table_12_3"]
    left, right, nr = oracle.lin_table(12, 3)
    assert (len(left), len(right), nr) == (g["left_len"], g["right_len"], g["n_right"])
    x, mism = 0b111, 0
    for _ in range(oracle.binom(12, 3)):
        mism += oracle.lin_index(x, left, right, nr) != oracle.rank(x)
        x = oracle.gosper_next(x)
    assert mism == g["mismatches_over_220"]
    l4, r4, n4 = oracle.lin_table(4, 2)
    assert oracle.lin_index(0b1010, l4, r4, n4) == g["lin_index_0b1010_n4k2"]


def test_haldane_2x3_counts(oracle):
    """doc/design.ipynb cells 26/43: orbits, sector dim, nnz(H), projection entries."""
    import scipy.sparse as sp

    g = GOLD["haldane_2x3"]
    cat, sec, op = oracle_objects(oracle, case_by_name("haldane2x3"), 0)
    assert cat.n_orbits == g["n_orbits"] and cat.n_states == g["full_basis"]
    assert int((cat.get(oracle.FIELD_REP_RANK) == 0).sum()) == g["rep_rank_unset"]
    assert sec.dim == g["sector_dim"]
    row, col, vals, diag = op.projection_table()
    assert len(row) == g["projection_entries"]
    I, J, V = op.matrix_coo()
    H = sp.coo_matrix((V, (I, J)), shape=(sec.dim, sec.dim)).tocsr()
    H.sum_duplicates()
    H.eliminate_zeros()
    assert H.nnz == g["nnz_H"]


BUILDERS = {
    "Heisenberg": lambda lab: L.heisenberg_ring(int(lab.split("=")[1])),
    "Haldane_Boson": lambda lab: L.haldane_honeycomb(*map(int, lab.split("×"))),
    "Hubbard_Fermion": lambda lab: L.hubbard_square(*map(int, lab.split("×"))),
}


def _rows(max_full):
    seen, out = set(), []
    for r in GOLD["benchmark_raw"]:
        key = (r["model"], r["label"])
        if r["mode"] != "matrix" or key in seen or r["full_dim"] > max_full:
            continue
        seen.add(key)
        out.append(r)
    return out


@pytest.mark.parametrize("row", _rows(200_000), ids=lambda r: f"{r['model']}-{r['label']}")
def test_benchmark_rows(oracle, row):
    """benchmark_raw.csv: orbit count, k=(0,0) sector dim and ground energy."""
    from cases import Case

    spec = BUILDERS[row["model"]](row["label"])
    case = Case(row["model"], spec)
    assert spec.lattice.n_site == row["n_site"] and spec.n_filled == row["n_filled"]
    cat, sec, op = oracle_objects(oracle, case, 0)
    assert cat.n_states == row["full_dim"]
    assert cat.n_orbits == row["n_orbits"]
    assert len(case.group()) == row["n_group"]
    assert sec.dim == row["sector_dim"]
    if sec.dim <= 2000:
        e0 = np.linalg.eigvalsh(op.dense())[0]
    else:
        r = op.solve(1, tol=1e-10, seed=3)
        assert r["status"] == 0
        e0 = r["evals"][0]
    assert abs(e0 - row["energy"]) < 1e-10, (e0, row["energy"])


def test_table_and_onthefly_modes_agree(oracle):
    """The two reference matvec spellings (SRE:731-765 vs 804-878) agree."""
    case = case_by_name("checkerboard3x2_f_flux")
    for k in range(len(case.irreps())):
        _, _, op = oracle_objects(oracle, case, k)
        for x in (x_ramp(op.dim), x_random(op.dim)):
            a, b = op.apply(x, mode=0), op.apply(x, mode=1)
            assert np.abs(a - b).max() <= 1e-11 * max(1.0, np.abs(a).max())
            np.testing.assert_allclose(op.dense() @ x, a, atol=1e-10)


def test_projection_table_vs_fallback(oracle):
    """flux_regression.jl:36-44: project_to_sector == project_to_unnormalized_sector."""
    case = case_by_name("checkerboard3x2_f_flux")
    G = case.group()
    from realspace_exactdiagonalization_gb300.groups import build_identity_group

    Gid = build_identity_group(G.n_site)
    full = oracle.Catalog(Gid.perm0(), Gid.phases(), 0, case.stats_code, case.spec.n_filled)
    masks = full.get(oracle.FIELD_REPS)
    for k in range(len(case.irreps())):
        _, sec, _ = oracle_objects(oracle, case, k)
        for m in masks:
            a, z = sec.project(int(m), 0), sec.project(int(m), 1)
            assert (a is None) == (z is None)
            if a is not None:
                assert a[0] == z[0] and abs(a[1] - z[1]) < 1e-11


def _expand(sec, stats, G, chi, c):
    """_expand_sector_state_to_fock_amplitudes (observables/entanglement_spectrum.jl:46-79)."""
    import oracle as O

    reps, stab, _ = sec.arrays()
    amps = {}
    nG = len(G)
    perm0, ph = G.perm0(), G.phases()
    for col, rep in enumerate(reps):
        if abs(c[col]) <= 1e-12:
            continue
        pref = c[col] / np.sqrt(nG * stab[col])
        for g in range(nG):
            s, a = O.apply_op(perm0[g], ph[g], stats, int(rep))
            amps[s] = amps.get(s, 0) + pref * np.conj(chi[g]) * a
    amps = {k: v for k, v in amps.items() if abs(v) > 1e-12}
    nrm = np.sqrt(sum(abs(v) ** 2 for v in amps.values()))
    return {k: v / nrm for k, v in amps.items()}


@pytest.mark.parametrize("name", ["checkerboard3x2_f_flux", "checkerboard3x2_b_flux", "checkerboard3x2_f_flux1"])
def test_sector_block_equals_projected_full_block(oracle, name):
    """flux_regression.jl:28-31,46: H = H', B'B = I, H = B' H_full B, and the
    union of sector spectra equals the identity-group spectrum."""
    case = case_by_name(name)
    G = case.group()
    from realspace_exactdiagonalization_gb300.groups import build_identity_group

    Gid = build_identity_group(G.n_site)
    fcat = oracle.Catalog(Gid.perm0(), Gid.phases(), 0, case.stats_code, case.spec.n_filled)
    fsec = oracle.Sector(fcat, np.array([1.0 + 0j]))
    Hf = oracle.Op(fsec, case.bilinear0(), case.density0()).dense()
    freps = fsec.arrays()[0]
    fidx = {int(m): i for i, m in enumerate(freps)}
    allv = []
    for k, irr in enumerate(case.irreps()):
        _, sec, op = oracle_objects(oracle, case, k)
        n = sec.dim
        if n == 0:
            continue
        H = op.dense()
        B = np.zeros((len(freps), n), dtype=np.complex128)
        for j in range(n):
            v = np.zeros(n, dtype=np.complex128)
            v[j] = 1
            for m, a in _expand(sec, case.stats_code, G, irr.array(), v).items():
                B[fidx[m], j] = a
        assert np.abs(H - H.conj().T).max() < 1e-11
        assert np.abs(B.conj().T @ B - np.eye(n)).max() < 1e-11
        assert np.abs(H - B.conj().T @ Hf @ B).max() < 1e-11
        allv.extend(np.linalg.eigvalsh(H))
    np.testing.assert_allclose(np.sort(allv), np.linalg.eigvalsh(Hf), atol=1e-10)
