"""The oracle's flux-torus observables pinned to the reference's stored
answers (doc/charge_pump.ipynb, cells 5 and 7): for the bosonic Haldane FCI
model on 2x3 cells (3 hard-core bosons on 12 sites) the two-state manifold has
Chern number 1 over a 5x5 flux grid, and the Resta pump along y under x-flux
(17 points over one cycle) moves charge 1/2 on each branch.  The notebook also
prints the minimum manifold gaps and the minimum link determinant, which pin
the twisted spectra and the Fock-space overlaps themselves."""
import math

import numpy as np

from realspace_exactdiagonalization_gb300 import lattice as L

# doc/charge_pump.ipynb outputs
CHERN_MIN_GAP = 0.29557407915615386
CHERN_MIN_LINK_DET = 0.6583441079398972
PUMP_MIN_GAP = 0.36256914952301766


def haldane_inputs(spec):
    lat = spec.lattice

    def point_inputs(flux):
        G = L.build_translation_group(lat, tuple(flux))
        irreps = [(tuple(int(x) for x in irr.label), irr.array()) for irr in L.build_translation_irrep_list(G, lat)]
        bil0 = [(i - 1, j - 1, t) for (i, j, t) in spec.bilinear_terms(tuple(flux))]
        den0 = [(i - 1, j - 1, v) for (i, j, v) in spec.density_terms]
        return G.perm0(), G.phases(), G.identity_idx - 1, 0, spec.n_filled, irreps, bil0, den0

    return point_inputs


def resta_phases(lat, direction):
    """charge_pump.jl:17-33 with the sublattice offsets."""
    Ld = lat.sample_size[direction - 1]
    return np.array([np.exp(2j * math.pi * (cell[direction - 1] + lat.sub_crys(sub)[direction - 1]) / Ld)
                     for (cell, sub) in lat.site_list])


def test_oracle_chern_number_haldane2x3(oracle):
    import observables_oracle as OB

    spec = L.haldane_honeycomb(2, 3)
    res = OB.chern_number(oracle, haldane_inputs(spec), manifold_size=2, nx=5, ny=5)
    assert abs(res["chern_number"] - 1.0) <= 1e-8
    assert abs(res["min_gap"] - CHERN_MIN_GAP) <= 1e-9
    assert abs(res["min_link_det"] - CHERN_MIN_LINK_DET) <= 1e-9


def test_oracle_charge_pump_haldane2x3(oracle):
    import observables_oracle as OB

    spec = L.haldane_honeycomb(2, 3)
    fluxes = [k / 16 for k in range(17)]
    res = OB.charge_pump(oracle, haldane_inputs(spec), resta_phases(spec.lattice, 2), fluxes, manifold_size=2)
    np.testing.assert_allclose(res["pumped_charges"], [0.5, 0.5], atol=1e-8)
    assert abs(res["min_gap"] - PUMP_MIN_GAP) <= 1e-9
    assert min(res["min_position_singular_values"]) > 1e-10


def test_oracle_phase_branch_tracking():
    """_tracked_phase_branches / _best_phase_permutation on a hand-made path:
    two branches that cross and wrap are followed continuously."""
    import observables_oracle as OB

    raw = np.array([[-0.45, 0.10], [0.12, -0.40], [-0.35, 0.20], [0.30, 0.49], [-0.48, 0.40]])
    tr = OB.tracked_phase_branches(raw)
    np.testing.assert_allclose(tr[:, 0], [-0.45, -0.40, -0.35, -0.51, -0.48])
    np.testing.assert_allclose(tr[:, 1], [0.10, 0.12, 0.20, 0.30, 0.40])
