"""Device flux-torus observables against the oracle and the reference's stored
answers: the projected position operator and the Fock-space overlaps, then
the full Chern number and charge pump of the bosonic Haldane 2x3 model
(doc/charge_pump.ipynb cells 5 and 7)."""

import numpy as np
import pytest

from cases import Case, case_by_name, oracle_objects
from realspace_exactdiagonalization_gb300 import lattice as L
from test_oracle_observables import CHERN_MIN_GAP, CHERN_MIN_LINK_DET, PUMP_MIN_GAP

pytestmark = pytest.mark.gpu


def _device_sector(case: Case, sector: int, catalog=None):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    G = case.group()
    if catalog is None:
        catalog = A.build_symmetry_orbit_catalog(n_filled=case.spec.n_filled, species=case.spec.species, symmetry_group=G,
                                                 particle_statistics=statistics_from_name(case.statistics))
    return catalog, A.build_symmetry_sector_basis(catalog, case.irreps()[sector], group=G)


@pytest.mark.parametrize("name", ["haldane2x3", "checkerboard3x2_f_flux", "hubbard2x4_flux"])
def test_position_operator_matches_oracle(oracle, name):
    import observables_oracle as OB
    from realspace_exactdiagonalization_gb300.observables import many_body_position_phases, position_operator_matrix

    case = case_by_name(name)
    lat = case.spec.lattice
    nk = len(case.irreps())
    G = case.group()
    cat = None
    for d in (1, 2):
        ph = many_body_position_phases(lat, d)
        for k_to, k_from in [(0, 0), (1 % nk, 0), (0, (nk - 1) % nk), (2 % nk, 1 % nk)]:
            cat, b_to = _device_sector(case, k_to, cat)
            _, b_from = _device_sector(case, k_from, cat)
            U = position_operator_matrix(b_to, b_from, ph).toarray()
            _, s_to, _ = oracle_objects(oracle, case, k_to)
            _, s_from, _ = oracle_objects(oracle, case, k_from)
            ref = OB.position_operator_matrix(s_to.arrays()[0], s_from.arrays()[0], G.perm0(),
                                              case.irreps()[k_to].array(), case.irreps()[k_from].array(), ph)
            assert U.shape == ref.shape
            np.testing.assert_allclose(U, ref, atol=1e-13, rtol=0, err_msg=f"{name} d={d} {k_to}<-{k_from}")


def test_fock_overlaps_match_numpy():
    from realspace_exactdiagonalization_gb300.observables import subspace_overlap_matrix

    rng = np.random.default_rng(3)
    for n in (1, 220, 70001):
        a = [rng.standard_normal(n) + 1j * rng.standard_normal(n) for _ in range(3)]
        b = [rng.standard_normal(n) + 1j * rng.standard_normal(n) for _ in range(3)]
        M = subspace_overlap_matrix(a, b)
        ref = np.array([[np.vdot(x, y) for y in b] for x in a])
        np.testing.assert_allclose(M, ref, rtol=1e-12, atol=1e-12 * n)


@pytest.mark.parametrize("solver", ["batch", "single"])
def test_chern_number_haldane2x3(solver):
    """The 5x5 flux grid's 150 sector solves in one batched launch (eigenvalues
    and eigenvectors), or one sector at a time: the same Chern number, gap and
    link determinant as the reference notebook."""
    from realspace_exactdiagonalization_gb300.observables import many_body_chern_number

    res = many_body_chern_number(L.haldane_honeycomb(2, 3), manifold_size=2, flux_grid_size=(5, 5), solver=solver)
    assert abs(res["chern_number"] - 1.0) <= 1e-8 and res["rounded_chern"] == 1
    assert abs(res["min_gap"] - CHERN_MIN_GAP) <= 1e-9
    assert abs(res["min_link_det"] - CHERN_MIN_LINK_DET) <= 1e-9


@pytest.mark.parametrize("solver", ["batch", "single"])
def test_charge_pump_haldane2x3(solver):
    from realspace_exactdiagonalization_gb300.observables import flux_charge_pump

    res = flux_charge_pump(L.haldane_honeycomb(2, 3), manifold_size=2, flux_direction=1,
                           polarization_direction=2, twisted_phases_over_2pi_list=[k / 16 for k in range(17)],
                           solver=solver)
    np.testing.assert_allclose(res["pumped_charges"], [0.5, 0.5], atol=1e-8)
    assert abs(res["min_gap"] - PUMP_MIN_GAP) <= 1e-9
    assert min(res["min_position_singular_values"]) > 1e-10
