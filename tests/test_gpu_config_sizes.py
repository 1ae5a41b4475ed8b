"""Parity at the configured sizes, where the oracle cannot hold a catalog.

* Checkerboard 4x6 spinless fermions (48 sites; NN |t| = 1 with e^{+-i pi/4}
  by plaquette arrow, NNN +-0.3, NNNN -0.2, V = 1), 8 particles, k = (0, 0):
  C(48, 8) = 3.8e8 basis states, about 1.6e7 sector rows.
* Hubbard 4x4 (t = 1, U = 8) as 32 modes, up spin at bit i and down spin at
  bit i + 16, in the N_up = N_down = 7 block, k = (pi, 0): 1.3e8 basis states,
  about 8.2e6 sector rows.

Checked on the GPU catalog, sector and operator, against the oracle's
single-mask layer (pinned in test_oracle_single_mask.py):
* table entries (rep_rank -> representative, stabilizer order, rep_sym,
  rep_amp) of 10,000 random basis states, bit for bit;
* the representative list strictly ascending, the orbit count and the sector
  dimension equal to the group-theoretic counts (projector traces over the
  fixed masks of each element), sampled sector rows compatible, and sampled
  compatible orbits present;
* 400 sampled rows of H x for a random x within 1e-11 of the largest |y|;
* the lowest eigenvalues of the FP64 and mixed-precision solves within 1e-9
  relative of each other (the mixed path's promise; no dense oracle exists at
  this size).
"""
from math import comb

import numpy as np
import pytest

from cases import character_dimension

pytestmark = pytest.mark.gpu

N_TABLE_SAMPLES = 10_000
N_ROW_SAMPLES = 400


def _config(name):
    from realspace_exactdiagonalization_gb300 import lattice as L

    if name == "checkerboard4x6_np8_k00":
        return L.checkerboard(4, 6, n_filled=8), 0, 3
    spec = L.hubbard_square(4, 4, n_up=7, n_dn=7)
    return spec, 2 * 4 + 0, 1  # momentum label (2, 0) = (pi, 0)


def _random_masks(rng, spec, n):
    """n random basis states with the catalog's particle number(s)."""
    N = spec.lattice.n_site
    out = np.zeros(n, dtype=np.uint64)
    for i in range(n):
        if spec.species:
            L_, a, b = spec.species
            lo = rng.choice(L_, a, replace=False)
            hi = L_ + rng.choice(N - L_, b, replace=False)
            sites = np.concatenate([lo, hi])
        else:
            sites = rng.choice(N, spec.n_filled, replace=False)
        out[i] = sum(1 << int(s) for s in sites)
    return out


@pytest.mark.parametrize("name", ["checkerboard4x6_np8_k00", "hubbard4x4_7u7d_kpi0"])
def test_configured_size_tables_rows_and_spectrum(oracle, name):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300 import lattice as L

    spec, k, nev = _config(name)
    G = L.build_translation_group(spec.lattice)
    irr = L.build_translation_irrep_list(G, spec.lattice)[k]
    stats = 1
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                         particle_statistics=A.Fermionic())
    N = spec.lattice.n_site
    sp = spec.species
    n_states = comb(sp[0], sp[1]) * comb(N - sp[0], sp[2]) if sp else comb(N, spec.n_filled)
    assert cat.n_states == n_states
    og = oracle.Group(G.perm0(), G.phases(), G.identity_idx - 1, stats)

    # --- representatives and orbit count
    reps = cat.representative_mask_list
    stab = cat.stabilizer_order_list
    assert (np.diff(reps.astype(np.uint64)) > 0).all() if reps.size > 1 else True
    trivial = np.ones(len(G.operations), dtype=np.complex128)
    # orbits: projector trace of the trivial irrep in the phase-free action
    from realspace_exactdiagonalization_gb300.groups import Finite_Symmetry_Group, Symmetry_Operation

    G_plain = Finite_Symmetry_Group("plain", [Symmetry_Operation(op.label, op.perm) for op in G.operations],
                                    G.identity_idx)
    assert cat.n_orbits == character_dimension(oracle, G_plain, 0, trivial, spec.n_filled, sp, n_states)

    # --- table entries of random basis states, bit for bit
    rng = np.random.default_rng(20261204)
    masks = _random_masks(rng, spec, N_TABLE_SAMPLES)
    rk, sy, am = cat.lookup(masks)
    for i, m in enumerate(masks):
        rep, st, sym, amp = og.state_entry(int(m))
        assert rk[i] >= 1 and reps[rk[i] - 1] == rep and stab[rk[i] - 1] == st, (name, int(m))
        assert sy[i] == sym, (name, int(m))
        assert np.array([amp]).view(np.uint64).tolist() == am[i:i + 1].view(np.uint64).tolist(), (name, int(m))

    # --- the sector
    basis = A.build_symmetry_sector_basis(cat, irr)
    assert basis.dim == character_dimension(oracle, G, stats, irr.array(), spec.n_filled, sp, n_states)
    srows = basis.representative_mask_list
    chi = irr.array()
    for r in rng.choice(basis.dim, 2000, replace=False):
        assert og.compatible(chi, int(srows[r])), (name, r)
    for m in masks[:2000]:
        rep = og.state_entry(int(m))[0]
        i = int(np.searchsorted(srows, np.uint64(rep)))
        found = i < basis.dim and srows[i] == rep
        assert found == og.compatible(chi, rep), (name, rep)

    # --- sampled rows of the matvec (FP64)
    H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms(), spec.density_terms, precision="fp64")
    x = rng.standard_normal(basis.dim) + 1j * rng.standard_normal(basis.dim)
    y = H(x)
    scale = np.abs(y).max()
    bil = [(i - 1, j - 1, t) for (i, j, t) in spec.bilinear_terms()]
    den = [(i - 1, j - 1, v) for (i, j, v) in spec.density_terms]
    for r in rng.choice(basis.dim, N_ROW_SAMPLES, replace=False):
        dg, col = og.column(chi, bil, den, int(srows[r]))
        yr = dg * x[r]
        for t, e in col:
            c = int(np.searchsorted(srows, np.uint64(t)))
            assert srows[c] == t
            yr += np.conj(e) * x[c]
        assert abs(yr - y[r]) <= 1e-11 * scale, (name, r, yr, y[r])
    del y, x

    # --- lowest eigenvalues: FP64 against mixed precision
    vals64, _, _ = H.solve(nev, tol=1e-10, want_vectors=False)
    del H
    Hm = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms(), spec.density_terms, precision="mixed")
    valsm, _, info = Hm.solve(nev, tol=1e-10, want_vectors=False)
    np.testing.assert_allclose(valsm, vals64, rtol=1e-9, atol=0, err_msg=name)


def test_flux_scan_768_mixed_against_fp64():
    """Config 4 at its stated size: the 768 sectors of the Haldane 3x4 flux
    scan (12 momenta x 8 x 8 twists, about 11,200 rows each) in one mixed
    launch and one FP64 launch.  Every sector's ground energy agrees within
    the mixed path's 1e-9 relative, every request converges, and the zero-twist
    k = (0, 0) sector gives the reference's stored E0 = -14.301456146831118
    (benchmark_raw.csv:20-21) within 1e-11 in FP64."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300 import lattice as L
    from realspace_exactdiagonalization_gb300.batched import BatchedSectorSolver, flux_scan_requests

    spec = L.haldane_honeycomb(3, 4)
    twists = [(a / 8, b / 8) for a in range(8) for b in range(8)]
    reqs = flux_scan_requests(spec, twists)
    assert len(reqs) == 768
    G = L.build_translation_group(spec.lattice)
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, symmetry_group=G, particle_statistics=A.Bosonic())
    pairs = [(i, j) for (i, j, _) in spec.bilinear_terms()]
    out = {}
    for prec in ("mixed", "fp64"):
        s = BatchedSectorSolver(cat, pairs, spec.density_terms, precision=prec, nev=4, max_requests=768)
        out[prec] = s.run(reqs)
        assert (out[prec]["status"] == 0).all()
    np.testing.assert_array_equal(out["mixed"]["dims"], out["fp64"]["dims"])
    assert out["fp64"]["dims"].min() > 11000
    e_mixed, e_fp64 = out["mixed"]["evals"][:, 0], out["fp64"]["evals"][:, 0]
    np.testing.assert_allclose(e_mixed, e_fp64, rtol=1e-9, atol=0)
    assert abs(e_fp64[0] - (-14.301456146831118)) <= 1e-11 * 14.3
