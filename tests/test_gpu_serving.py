"""The served path: a mixed request stream through the continuous-batching
scheduler (batched kernel lanes, a mid-size lane, concurrent device-wide
solves) against the oracle's dense spectra, and each request alone against
its result in the mix (within the mixed path's |dE|/|E| <= 1e-9)."""
import numpy as np
import pytest

from cases import Case, oracle_objects
from realspace_exactdiagonalization_gb300 import lattice as L

pytestmark = pytest.mark.gpu


def _families():
    return {"checkerboard3x2": L.checkerboard(3, 2, n_filled=4),
            "haldane2x4": L.haldane_honeycomb(2, 4),
            "ring16": L.ring_xxz(16, 1.0, 2.0)}


@pytest.mark.parametrize("ring_route", ["large", "medium"])
def test_served_mix_matches_oracle_and_alone(oracle, ring_route):
    from realspace_exactdiagonalization_gb300.serving import SectorServer, random_requests

    fams = _families()
    reqs = random_requests(fams, 36, rate=0.0, seed=7, nev=1)
    # ring16 (810 orbits) takes the device-wide route, or the batched kernel's
    # mid-size lane with its matvec input in global memory; the others take
    # the batched kernel's shared lanes
    medium = 1000 if ring_route == "medium" else 0
    srv = SectorServer(fams, budget_bytes=8e9, batch_lanes=2, large_workers=2, small_max_orbits=300,
                       medium_max_orbits=medium)
    assert srv.families["ring16"].route == ring_route and srv.families["haldane2x4"].route == "batch"
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
                            small_max_orbits=300, medium_max_orbits=medium)
        q = random_requests(fams, 36, rate=0.0, seed=7, nev=1)[r.rid]
        alone = srv1.serve([q])[0]
        assert alone.dim == r.dim
        # the mixed path's stated tolerance, |dE|/|E| <= 1e-9
        assert np.all(np.abs(alone.evals - r.evals) <= 1e-9 * np.maximum(1.0, np.abs(r.evals))), \
            (r.rid, r.family, alone.evals, r.evals)


def test_warm_up_leaves_no_tuning_to_requests():
    """The server's warm-up runs every batched family's lanes once at setup,
    so the launch autotuner's trial launches (and the hop-table builds) are
    behind it: no served batch runs the autotuner."""
    from realspace_exactdiagonalization_gb300.serving import SectorServer, random_requests

    fams = _families()
    srv = SectorServer(fams, budget_bytes=8e9, batch_lanes=2, large_workers=1, small_max_orbits=300)
    batch = [f for f in srv.families.values() if f.route == "batch"]
    assert batch
    before = {(f.name, i): s.shape()["tune_runs"] for f in batch for i, s in enumerate(f.solvers)}
    assert all(s.shape()["krylovdim"] > 0 for f in batch for s in f.solvers)
    done = srv.serve(random_requests(fams, 24, rate=0.0, seed=11, nev=1))
    assert all(r.status == 0 for r in done)
    after = {(f.name, i): s.shape()["tune_runs"] for f in batch for i, s in enumerate(f.solvers)}
    assert after == before


def test_op_priority_keeps_results():
    """sed_op_set_priority moves the operator to a stream of the device's
    greatest (or least) priority; the solve gives the same bits, and a
    priority other than 0 or 1 is refused."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300 import _lib

    spec = L.ring_xxz(16, 1.0, 2.0)
    G = L.build_translation_group(spec.lattice, (0.2, 0.0))
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                         particle_statistics=A.Bosonic())
    basis = A.build_symmetry_sector_basis(cat, L.build_translation_irrep_list(G, spec.lattice)[3], group=G)
    H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms((0.2, 0.0)), spec.density_terms, precision="mixed")
    a, _, _ = H.solve(2, want_vectors=False)
    H.set_priority(True)
    b, _, _ = H.solve(2, want_vectors=False)
    H.set_priority(False)
    c, _, _ = H.solve(2, want_vectors=False)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
    with pytest.raises(_lib.SEDError):
        _lib.check(_lib.load().sed_op_set_priority(H.handle, 2))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_op_sm_limit_keeps_results(oracle, precision):
    """sed_op_set_sm_limit sizes the operator's grids for fewer SMs; the
    reduction partitions change, so the eigenvalues agree within the path's
    tolerance (and with the oracle), and a negative limit is refused."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300 import _lib

    spec = L.ring_xxz(16, 1.0, 2.0)
    G = L.build_translation_group(spec.lattice, (0.2, 0.0))
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                         particle_statistics=A.Bosonic())
    irr = L.build_translation_irrep_list(G, spec.lattice)[3]
    basis = A.build_symmetry_sector_basis(cat, irr, group=G)
    vals = {}
    for sms in (0, 16, 1):
        H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms((0.2, 0.0)), spec.density_terms, precision=precision)
        H.set_sm_limit(sms)
        vals[sms], _, _ = H.solve(2, want_vectors=False)
    _, sec, op = oracle_objects(oracle, Case("ring16", spec, theta=(0.2, 0.0)), 3)
    ref = np.linalg.eigvalsh(op.dense())
    for sms, v in vals.items():
        np.testing.assert_allclose(v, vals[0], rtol=1e-9, atol=1e-12, err_msg=f"sm_limit={sms}")
        np.testing.assert_allclose(v, ref[:2], rtol=1e-9, atol=1e-12, err_msg=f"sm_limit={sms}")
    with pytest.raises(_lib.SEDError):
        _lib.check(_lib.load().sed_op_set_sm_limit(H.handle, -1))


def test_concurrent_table_builds_from_two_threads():
    """Catalog expansions and operator hop tables stage per-catalog rank
    tables of different sizes in shared memory; their kernels' shared-memory
    opt-in is shared by every host thread.  Two threads building catalogs,
    sectors and hop tables of two fillings (different rank-table sizes) over
    and over must all succeed and give the same ground energies each time."""
    import threading

    import realspace_exactdiagonalization_gb300.api as A

    def work(n_filled, out, errs):
        try:
            spec = L.hubbard_square(2, 4, n_filled=n_filled)
            G = L.build_translation_group(spec.lattice, (0.3, 0.1))
            irr = L.build_translation_irrep_list(G, spec.lattice)[1]
            for _ in range(12):
                cat = A.build_symmetry_orbit_catalog(n_filled=n_filled, symmetry_group=G,
                                                     particle_statistics=A.Fermionic())
                basis = A.build_symmetry_sector_basis(cat, irr, group=G)
                H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms((0.3, 0.1)), spec.density_terms,
                                            precision="mixed")
                H.set_hop_table(2)
                vals, _, _ = H.solve(1, want_vectors=False)
                out.append(float(vals[0]))
                del H
        except Exception as e:  # reported to the main thread
            errs.append(repr(e))

    outs, errs = {5: [], 8: []}, []
    ts = [threading.Thread(target=work, args=(nf, outs[nf], errs)) for nf in (5, 8)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs, errs
    for nf, vals in outs.items():
        assert len(vals) == 12 and len(set(vals)) == 1, (nf, vals)


def test_native_server_matches_oracle(oracle):
    """The native server (sed_server_* in the C ABI; C++ host threads driving
    the batch lanes and the device-wide solves) answers a mixed stream with
    the oracle's ground energies (1e-9) and the sector dimensions; misuse is
    refused with SED_ERR_ARG."""
    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300.serving import NativeSectorServer, random_requests

    fams = _families()
    reqs = random_requests(fams, 36, rate=0.0, seed=7, nev=1)
    srv = NativeSectorServer(fams, budget_bytes=8e9, batch_lanes=2, large_workers=2, small_max_orbits=300)
    try:
        done = sorted(srv.serve(reqs), key=lambda r: r.rid)
        assert len(done) == len(reqs) and all(r.status == 0 for r in done), [r.error for r in done if r.status]
        for r in done:
            case = Case(r.family, fams[r.family], theta=r.twist)
            _, sec, op = oracle_objects(oracle, case, r.k_index)
            assert r.dim == sec.dim
            if sec.dim == 0:
                assert np.isnan(r.evals[0])
                continue
            e0 = np.linalg.eigvalsh(op.dense())[0]
            assert abs(r.evals[0] - e0) <= 1e-9 * max(1.0, abs(e0)), (r.rid, r.family)
        st = srv.stats()
        assert st["done"] == len(reqs) and st["pending"] == 0 and st["resident_bytes"] > 0
        bad = random_requests(fams, 1, rate=0.0, seed=8, nev=2)[0]  # nev above the families' nev_max (1)
        with pytest.raises(_lib.SEDError) as e:
            srv.submit(bad)
        assert e.value.code == _lib.SED_ERR_ARG
    finally:
        srv.close()


def test_served_mix_through_device_resident_loops(oracle):
    """ring_blocks > 0: the batched families are answered by device-resident
    request loops (sed_batch_ring_*), each request submitted straight into its
    family's ring; the answers are the oracle's ground energies (1e-9)."""
    from realspace_exactdiagonalization_gb300.serving import SectorServer, random_requests

    fams = _families()
    reqs = random_requests(fams, 36, rate=0.0, seed=9, nev=1)
    srv = SectorServer(fams, budget_bytes=8e9, batch_lanes=2, large_workers=2, small_max_orbits=300,
                       ring_blocks=8, ring_idle_ms=50)
    done = sorted(srv.serve(reqs), key=lambda r: r.rid)
    assert len(done) == len(reqs) and all(r.status == 0 for r in done), [r.error for r in done if r.status]
    assert {r.route for r in done if srv.families[r.family].route == "batch"} == {"ring"}
    for r in done:
        _, sec, op = oracle_objects(oracle, Case(r.family, fams[r.family], theta=r.twist), r.k_index)
        assert r.dim == sec.dim
        if sec.dim:
            e0 = np.linalg.eigvalsh(op.dense())[0]
            assert abs(r.evals[0] - e0) <= 1e-9 * max(1.0, abs(e0)), (r.rid, r.family, r.route)


def test_native_server_refusals():
    """The native server's refusals: an unknown ticket, sed_server_next on an
    idle server (SED_ERR_TIMEOUT), a family registered after the first
    request (SED_ERR_ARG), and an unknown family."""
    import ctypes as C

    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300.serving import NativeSectorServer, random_requests

    fams = {"haldane2x4": L.haldane_honeycomb(2, 4)}
    srv = NativeSectorServer(fams, budget_bytes=4e9, batch_lanes=1, large_workers=1, small_max_orbits=300)
    lib = _lib.load()
    try:
        ev = np.zeros(1)
        st, dim, t = C.c_int32(0), C.c_int64(0), C.c_int64(0)
        assert lib.sed_server_wait(srv._h, 12345, 0, ev.ctypes.data, C.byref(st), C.byref(dim)) == _lib.SED_ERR_ARG
        assert lib.sed_server_next(srv._h, 0, C.byref(t), ev.ctypes.data, C.byref(st), C.byref(dim)) == \
            _lib.SED_ERR_TIMEOUT
        r = random_requests(fams, 1, rate=0.0, seed=3, nev=1)[0]
        ticket = srv.submit(r)
        srv.wait(ticket, r)
        assert r.status == 0 and r.dim > 0
        cat = srv.catalogs["haldane2x4"]
        bij = np.zeros(2, dtype=np.int32)
        bt = np.zeros(1, dtype=np.complex128)
        fid = C.c_int32(-1)
        assert lib.sed_server_add_family(srv._h, cat.handle, 0, bij.ctypes.data, bt.ctypes.data, 0, None, None, 1,
                                         C.byref(fid)) == _lib.SED_ERR_ARG
        chi = np.ones(16, dtype=np.complex128)
        assert lib.sed_server_submit(srv._h, 7, chi.ctypes.data, chi.ctypes.data, chi.ctypes.data, 1, 1,
                                     C.byref(t)) == _lib.SED_ERR_ARG
    finally:
        srv.close()


def test_native_server_one_collector_per_ticket():
    """Two threads waiting on one ticket at once (sed_server_wait from both):
    exactly one receives the answer, the other SED_ERR_ARG; the server stays
    usable."""
    import ctypes as C
    import threading

    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300.serving import NativeSectorServer, random_requests

    fams = {"haldane2x4": L.haldane_honeycomb(2, 4)}
    srv = NativeSectorServer(fams, budget_bytes=4e9, batch_lanes=1, large_workers=1, small_max_orbits=300)
    lib = _lib.load()
    try:
        for seed in range(3):
            r = random_requests(fams, 1, rate=0.0, seed=20 + seed, nev=1)[0]
            ticket = srv.submit(r)
            rcs, evs = [None, None], [np.zeros(1), np.zeros(1)]

            def waiter(i):
                st, dim = C.c_int32(0), C.c_int64(0)
                rcs[i] = lib.sed_server_wait(srv._h, ticket, 60_000, evs[i].ctypes.data, C.byref(st), C.byref(dim))

            th = [threading.Thread(target=waiter, args=(i,)) for i in range(2)]
            for t in th:
                t.start()
            for t in th:
                t.join()
            assert sorted(rcs) == [0, _lib.SED_ERR_ARG], rcs
            assert np.isfinite(evs[rcs.index(0)][0])
        r = random_requests(fams, 1, rate=0.0, seed=30, nev=1)[0]
        srv.wait(srv.submit(r), r)
        assert r.status == 0
    finally:
        srv.close()
