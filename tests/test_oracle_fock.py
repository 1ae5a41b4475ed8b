"""The oracle's _expand_sector_state_to_fock_amplitudes (observables/
entanglement_spectrum.jl:46-79), pinned at the physics level: a sector
eigenvector expanded to Fock amplitudes is a unit eigenvector of the
full-basis Hamiltonian (identity group) with the same eigenvalue."""
import numpy as np
import pytest

from cases import case_by_name, oracle_objects
from realspace_exactdiagonalization_gb300.groups import build_identity_group


@pytest.mark.parametrize("name,k", [("checkerboard3x2_f_flux", 1), ("checkerboard3x2_b_flux", 2),
                                    ("hubbard2x3", 0), ("haldane2x3", 4)])
def test_expanded_eigenvector_is_full_basis_eigenvector(oracle, name, k):
    case = case_by_name(name)
    cat, sec, op = oracle_objects(oracle, case, k)
    vals, vecs = np.linalg.eigh(op.dense())
    f = sec.expand_fock(vecs[:, 0])
    assert abs(np.linalg.norm(f) - 1.0) < 1e-12
    Gi = build_identity_group(case.spec.lattice.n_site)
    cati = oracle.Catalog(Gi.perm0(), Gi.phases(), Gi.identity_idx - 1, case.stats_code, case.spec.n_filled)
    opi = oracle.Op(oracle.Sector(cati, np.ones(1, complex)), case.bilinear0(), case.density0())
    r = opi.dense() @ f - vals[0] * f
    assert np.linalg.norm(r) < 1e-11


def test_expand_rejects_zero_state(oracle):
    case = case_by_name("checkerboard3x2_f_flux0")
    _, sec, _ = oracle_objects(oracle, case, 0)
    with pytest.raises(RuntimeError, match="near-zero norm"):
        sec.expand_fock(np.zeros(sec.dim, complex))
