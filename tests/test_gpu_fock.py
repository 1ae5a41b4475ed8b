"""Device Fock expansion (sed_sector_expand_fock) against the oracle's
restatement of _expand_sector_state_to_fock_amplitudes
(observables/entanglement_spectrum.jl:46-79): same amplitudes on the same
sector vector, the Dict form's keys, and the reference's error."""
import numpy as np
import pytest

from cases import case_by_name, oracle_objects

pytestmark = pytest.mark.gpu


def _device_basis(case, k):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    cat = A.build_symmetry_orbit_catalog(n_filled=case.spec.n_filled, species=case.spec.species, symmetry_group=case.group(),
                                         particle_statistics=statistics_from_name(case.statistics))
    return A.build_symmetry_sector_basis(cat, case.irreps()[k])


@pytest.mark.parametrize("name,k", [("ring16", 0), ("checkerboard3x2_f_flux", 1), ("checkerboard3x2_b_flux", 2),
                                    ("hubbard2x4_flux", 3), ("haldane2x3", 4)])
def test_fock_expansion_matches_oracle(oracle, name, k):
    import realspace_exactdiagonalization_gb300.api as A

    case = case_by_name(name)
    _, sec, op = oracle_objects(oracle, case, k)
    basis = _device_basis(case, k)
    assert basis.dim == sec.dim
    vals, vecs = np.linalg.eigh(op.dense())
    for c in (vecs[:, 0], vecs[:, 1] + 0.5j * vecs[:, 2]):
        ref = sec.expand_fock(c)
        got = A.expand_sector_state_to_fock(c, basis)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13)
    d = A._expand_sector_state_to_fock_amplitudes(vecs[:, 0], basis)
    ref = sec.expand_fock(vecs[:, 0])
    nz = np.nonzero(ref)[0]
    assert len(d) == len(nz)
    assert all(oracle.rank(m) in set(nz.tolist()) for m in list(d)[:50])


def test_fock_expansion_rejects_zero_state():
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300._lib import SEDError

    basis = _device_basis(case_by_name("checkerboard3x2_f_flux0"), 0)
    with pytest.raises(SEDError, match="near-zero norm"):
        A.expand_sector_state_to_fock(np.zeros(basis.dim, complex), basis)
