"""The served path: a mixed request stream through the continuous-batching
scheduler (batched kernel lanes + concurrent device-wide solves) against the
oracle's dense spectra, and each request alone against its result in the mix
(within the mixed path's |dE|/|E| <= 1e-9)."""
import numpy as np
import pytest

from cases import Case, oracle_objects
from realspace_exactdiagonalization_gb300 import lattice as L

pytestmark = pytest.mark.gpu


def _families():
    return {"checkerboard3x2": L.checkerboard(3, 2, n_filled=4),
            "haldane2x4": L.haldane_honeycomb(2, 4),
            "ring16": L.ring_xxz(16, 1.0, 2.0)}


def test_served_mix_matches_oracle_and_alone(oracle):
    from realspace_exactdiagonalization_gb300.serving import SectorServer, random_requests

    fams = _families()
    reqs = random_requests(fams, 36, rate=0.0, seed=7, nev=1)
    # ring16 (810 orbits) takes the device-wide route, the others the batched kernel
    srv = SectorServer(fams, budget_bytes=8e9, batch_lanes=2, large_workers=2, small_max_orbits=300)
    assert srv.families["ring16"].route == "large" and srv.families["haldane2x4"].route == "batch"
    done = sorted(srv.serve(reqs), key=lambda r: r.rid)
    assert len(done) == len(reqs) and all(r.status == 0 for r in done)
    for r in done:
        case = Case(r.family, fams[r.family], theta=r.twist)
        _, sec, op = oracle_objects(oracle, case, r.k_index)
        assert r.dim == sec.dim
        if sec.dim == 0:
            continue
        e0 = np.linalg.eigvalsh(op.dense())[0]
        assert abs(r.evals[0] - e0) <= 1e-9 * max(1.0, abs(e0)), (r.rid, r.family, r.route)
    # alone: a fresh server answers each of a few requests on its own
    for r in done[:: 7]:
        srv1 = SectorServer({r.family: fams[r.family]}, budget_bytes=8e9, batch_lanes=1, large_workers=1,
                            small_max_orbits=300)
        q = random_requests(fams, 36, rate=0.0, seed=7, nev=1)[r.rid]
        alone = srv1.serve([q])[0]
        assert alone.dim == r.dim
        # the mixed path's stated tolerance, |dE|/|E| <= 1e-9
        assert np.all(np.abs(alone.evals - r.evals) <= 1e-9 * np.maximum(1.0, np.abs(r.evals))), \
            (r.rid, r.family, alone.evals, r.evals)
