"""Batched persistent-kernel solves against dense oracle spectra, and the
alone-versus-in-the-mix property of the batch path."""
import numpy as np
import pytest

from cases import Case, oracle_objects
from realspace_exactdiagonalization_gb300 import lattice as L

pytestmark = pytest.mark.gpu

TWISTS = [(0.0, 0.0), (0.23, 0.17), (0.5, 0.0), (0.75, 0.5)]


def _solver(spec, precision, nev=4, max_requests=256):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.batched import BatchedSectorSolver
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    G = L.build_translation_group(spec.lattice)
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, symmetry_group=G,
                                         particle_statistics=statistics_from_name(spec.statistics))
    pairs = [(i, j) for (i, j, _) in spec.bilinear_terms()]
    return BatchedSectorSolver(cat, pairs, spec.density_terms, precision=precision, nev=nev,
                               max_requests=max_requests)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("model", ["checkerboard3x2_f", "checkerboard3x2_b", "haldane2x4"])
def test_batch_matches_dense(oracle, model, precision):
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = {"checkerboard3x2_f": lambda: L.checkerboard(3, 2, n_filled=4),
            "checkerboard3x2_b": lambda: L.checkerboard(3, 2, n_filled=4, statistics="bosonic"),
            "haldane2x4": lambda: L.haldane_honeycomb(2, 4)}[model]()
    reqs = flux_scan_requests(spec, TWISTS)
    out = _solver(spec, precision).run(reqs)
    assert (out["status"] == 0).all()
    nG = len(reqs) // len(TWISTS)
    for b, r in enumerate(reqs):
        th = TWISTS[b // nG]
        case = Case(model, spec, theta=th)
        _, sec, op = oracle_objects(oracle, case, b % nG)
        assert out["dims"][b] == sec.dim
        if sec.dim == 0:
            continue
        ref = np.linalg.eigvalsh(op.dense())
        k = min(4, sec.dim)
        tol = 1e-9 * max(1.0, abs(ref[0]))
        np.testing.assert_allclose(out["evals"][b, :k], ref[:k], atol=tol, rtol=0, err_msg=f"{model} {b} {th}")


def test_batch_alone_equals_in_mix():
    """A request's result does not depend on the other requests of the launch."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.haldane_honeycomb(2, 4)
    reqs = flux_scan_requests(spec, TWISTS)
    solver = _solver(spec, "mixed")
    mix = solver.run(reqs)
    for b in (0, 5, len(reqs) - 1):
        alone = solver.run([reqs[b]])
        assert np.array_equal(alone["evals"][0], mix["evals"][b])
        assert alone["dims"][0] == mix["dims"][b]


def test_batch_config4_sample_golden():
    """Haldane 3x4 bosons (the flux-scan batch model): the zero-twist k=(0,0)
    request reproduces the reference's stored E0 = -14.301456146831118
    (benchmark_raw.csv:20-21) within |dE|/|E| <= 1e-9, in the batch path."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.haldane_honeycomb(3, 4)
    reqs = flux_scan_requests(spec, [(0.0, 0.0), (0.5, 0.25)])
    out = _solver(spec, "mixed", max_requests=64).run(reqs)
    assert (out["status"] == 0).all()
    assert out["dims"][0] == 11240
    assert abs(out["evals"][0, 0] - (-14.301456146831118)) <= 14.3 * 1e-9
