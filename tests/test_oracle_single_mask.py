"""The oracle's single-mask layer, pinned to its catalog layer.

Sectors at the configured sizes (48 sites, 1.6e7 orbits; 32 modes, 8.2e6
orbits) are too large for the oracle's in-memory catalog, so their GPU parity
tests sample: table entries of random masks (oracle.Group.state_entry), sector
rows of the matrix (oracle.Group.column) and the sector dimension from the
projector trace (cases.character_dimension).  Here each of those is checked
against the catalog-based oracle, which is itself pinned to the reference's
stored answers (test_oracle_golden.py), on every small case.
"""
from math import comb

import numpy as np
import pytest

from cases import Case, character_dimension, oracle_objects, small_cases
from realspace_exactdiagonalization_gb300 import lattice as L
from realspace_exactdiagonalization_gb300.api import colex_unrank


def _all_cases():
    return small_cases() + [Case("hubbard2x4_3u4d_flux", L.hubbard_square(2, 4, n_up=3, n_dn=4), theta=(0.3, 0.1))]


@pytest.mark.parametrize("case", _all_cases(), ids=lambda c: c.name)
def test_state_entries_equal_catalog_tables(oracle, case):
    G = case.group()
    cat = oracle.Catalog(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code, case.spec.n_filled)
    og = oracle.Group(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code)
    reps, order = cat.get(oracle.FIELD_REPS), cat.get(oracle.FIELD_STAB_ORDER)
    rr, rs, ra = cat.get(oracle.FIELD_REP_RANK), cat.get(oracle.FIELD_REP_SYM), cat.get(oracle.FIELD_REP_AMP)
    masks = colex_unrank(np.arange(cat.n_states), G.n_site, case.spec.n_filled)
    step = max(1, cat.n_states // 3000)
    for r in range(0, cat.n_states, step):
        rep, stab, sym, amp = og.state_entry(int(masks[r]))
        assert rep == reps[rr[r] - 1] and stab == order[rr[r] - 1], (case.name, r)
        assert sym == rs[r], (case.name, r)
        assert np.array([amp]).view(np.uint64).tolist() == ra[r:r + 1].view(np.uint64).tolist(), (case.name, r)


@pytest.mark.parametrize("case", _all_cases()[:6], ids=lambda c: c.name)
def test_columns_give_the_matrix_rows(oracle, case):
    """Row r of the sector matrix from column r and Hermiticity (H_rc =
    conj(H_cr), which the reference's own regression test checks, H = H'):
    y_r = diag_r x_r + sum over the hops of rep_r of conj(H_cr) x_c."""
    G = case.group()
    og = oracle.Group(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code)
    for k in range(min(3, len(case.irreps()))):
        _, sec, op = oracle_objects(oracle, case, k)
        if sec.dim == 0:
            continue
        reps, _, _ = sec.arrays()
        Hd = op.dense()
        chi = case.irreps()[k].array()
        for r in range(0, sec.dim, max(1, sec.dim // 60)):
            dg, col = og.column(chi, case.bilinear0(), case.density0(), int(reps[r]))
            row = np.zeros(sec.dim, dtype=np.complex128)
            row[r] += dg
            for t, e in col:
                i = int(np.searchsorted(reps, np.uint64(t)))
                assert reps[i] == t
                row[i] += np.conj(e)
            assert np.abs(row - Hd[r]).max() <= 1e-13 * max(1.0, np.abs(Hd).max()), (case.name, k, r)


@pytest.mark.parametrize("case", _all_cases(), ids=lambda c: c.name)
def test_character_dimension_equals_sector_dimension(oracle, case):
    G = case.group()
    sp = case.spec.species
    n_states = comb(sp[0], sp[1]) * comb(G.n_site - sp[0], sp[2]) if sp else comb(G.n_site, case.spec.n_filled)
    for k, irr in enumerate(case.irreps()):
        _, sec, _ = oracle_objects(oracle, case, k)
        reps, _, _ = sec.arrays()
        if sp:
            low = reps & np.uint64((1 << sp[0]) - 1)
            dim = sum(1 for m in low if bin(int(m)).count("1") == sp[1])
        else:
            dim = sec.dim
        assert character_dimension(oracle, G, case.stats_code, irr.array(), case.spec.n_filled, sp,
                                   n_states) == dim, (case.name, k)
