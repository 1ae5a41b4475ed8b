"""Batched persistent-kernel solves against dense oracle spectra, and the
alone-versus-in-the-mix property of the batch path."""
import numpy as np
import pytest

from cases import Case, assert_lanczos_spectrum, oracle_objects
from realspace_exactdiagonalization_gb300 import lattice as L

pytestmark = pytest.mark.gpu

TWISTS = [(0.0, 0.0), (0.23, 0.17), (0.5, 0.0), (0.75, 0.5)]


def _assert_oracle_spectra(oracle, model, spec, twists, out, tol=1e-9):
    """Every request of a flux-scan run against the oracle's dense spectrum
    (Lanczos semantics: an exactly degenerate level may be listed fewer times
    than its multiplicity, so two runs that differ only in rounding may list
    different copies; their lowest levels agree)."""
    nk = len(out["dims"]) // len(twists)
    for b in range(len(out["dims"])):
        case = Case(model, spec, theta=twists[b // nk])
        _, sec, op = oracle_objects(oracle, case, b % nk)
        assert out["dims"][b] == sec.dim
        if sec.dim == 0:
            continue
        ref = np.linalg.eigvalsh(op.dense())
        k = min(out["evals"].shape[1], sec.dim)
        assert_lanczos_spectrum(out["evals"][b, :k], ref, tol * max(1.0, abs(ref[0])), msg=f"{model} {b}")


def _solver(spec, precision, nev=4, max_requests=256):
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.batched import BatchedSectorSolver
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    G = L.build_translation_group(spec.lattice)
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                         particle_statistics=statistics_from_name(spec.statistics))
    pairs = [(i, j) for (i, j, _) in spec.bilinear_terms()]
    return BatchedSectorSolver(cat, pairs, spec.density_terms, precision=precision, nev=nev,
                               max_requests=max_requests)


@pytest.mark.parametrize("hop_table", [True, False], ids=["table", "on_the_fly"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("model", ["checkerboard3x2_f", "checkerboard3x2_b", "haldane2x4", "ring16"])
def test_batch_matches_dense(oracle, model, precision, hop_table):
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = {"checkerboard3x2_f": lambda: L.checkerboard(3, 2, n_filled=4),
            "checkerboard3x2_b": lambda: L.checkerboard(3, 2, n_filled=4, statistics="bosonic"),
            "haldane2x4": lambda: L.haldane_honeycomb(2, 4),
            # a one-dimensional ring (twist along x only) with density terms
            "ring16": lambda: L.ring_xxz(16, 1.0, 2.0)}[model]()
    reqs = flux_scan_requests(spec, TWISTS)
    solver = _solver(spec, precision)
    solver.set_hop_table(hop_table)
    out = solver.run(reqs)
    assert solver.last_stats()["hop_table"] == hop_table
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
        # the batch is a single-vector Krylov method at every size (the ring at
        # twist 0.5 has exactly degenerate levels)
        assert_lanczos_spectrum(out["evals"][b, :k], ref, tol, msg=f"{model} {b} {th}")


@pytest.mark.parametrize("fresh", [False, True], ids=["same_solver", "fresh_solver"])
def test_batch_alone_equals_in_mix(fresh):
    """A request's result is the same alone and in the mix, within the mixed
    path's 1e-9 relative tolerance: the other requests of a launch change only
    the hop table's phase-class partition (fresh solver), never the sector or
    its matrix.  Repeating a launch reproduces it bit for bit."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.haldane_honeycomb(2, 4)
    reqs = flux_scan_requests(spec, TWISTS)
    solver = _solver(spec, "mixed")
    mix = solver.run(reqs)
    again = solver.run(reqs)
    assert np.array_equal(again["evals"], mix["evals"])
    for b in (0, 5, 9, len(reqs) - 1):
        alone = (_solver(spec, "mixed") if fresh else solver).run([reqs[b]])
        assert alone["dims"][0] == mix["dims"][b]
        e0, e1 = alone["evals"][0], mix["evals"][b]
        ok = ~np.isnan(e1)
        np.testing.assert_allclose(e0[ok], e1[ok], rtol=1e-9, atol=1e-12)


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


def test_hop_table_fermion_flux_matches_on_the_fly(oracle):
    """The hop table carries the Jordan-Wigner / permutation signs and the
    twist-phase class counts of every hop: spinless fermions under a flux grid
    give the oracle's spectra through the table as through the on-the-fly
    matvec (FP64 batch, 1e-9).  Every level of these 80-row sectors at a
    twist is exactly two-fold degenerate; the batch always runs Lanczos (no
    dense branch), so each path lists a level at most as often as its
    multiplicity, and which copies rounding reveals depends on the summation
    order (Lanczos semantics, cases.assert_lanczos_spectrum)."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.checkerboard(3, 2, n_filled=4)
    twists = [(a / 4, b / 4) for a in range(4) for b in range(4)]
    reqs = flux_scan_requests(spec, twists)
    s_tab = _solver(spec, "fp64")
    s_fly = _solver(spec, "fp64")
    s_fly.set_hop_table(False)
    a = s_tab.run(reqs)
    st = s_tab.last_stats()
    assert st["hop_table"] and st["hop_records"] > 0
    b = s_fly.run(reqs)
    assert not s_fly.last_stats()["hop_table"]
    assert np.array_equal(a["dims"], b["dims"])
    assert (a["status"] == 0).all() and (b["status"] == 0).all()
    nk = len(reqs) // len(twists)
    for r in range(len(reqs)):
        if a["dims"][r] == 0:
            continue
        case = Case("checkerboard3x2_f", spec, theta=twists[r // nk])
        _, sec, op = oracle_objects(oracle, case, r % nk)
        assert sec.dim == a["dims"][r]
        ref = np.linalg.eigvalsh(op.dense())
        for name, out in (("table", a), ("on the fly", b)):
            assert_lanczos_spectrum(out["evals"][r], ref, 1e-9, f"{name} request {r}")


def test_batch_rejects_a_bad_request_in_a_large_batch():
    """Every request's term list is validated before the launch (on several
    host threads for a large batch): one non-Hermitian request among 96 fails
    the whole call with SED_ERR_NOT_HERMITIAN, and the solver stays usable."""
    import dataclasses

    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.checkerboard(3, 2, n_filled=4)
    twists = [(a / 4, b / 4) for a in range(4) for b in range(4)]
    reqs = flux_scan_requests(spec, twists)
    assert len(reqs) == 96
    solver = _solver(spec, "mixed", max_requests=128)
    bad = list(reqs)
    amps = list(bad[70].amplitudes)
    amps[0] *= 1.5
    bad[70] = dataclasses.replace(bad[70], amplitudes=amps)
    with pytest.raises(_lib.SEDError) as e:
        solver.run(bad)
    assert e.value.code == _lib.SED_ERR_NOT_HERMITIAN
    out = solver.run(reqs[:8])
    assert (out["status"] == 0).all()


def test_batch_launch_is_a_replayed_graph():
    """The batch launch is captured as a CUDA graph on its first run and
    replayed while the launch configuration repeats; a replay gives the same
    bits as the captured run, and a different configuration is captured anew."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.checkerboard(3, 2, n_filled=4)
    reqs = flux_scan_requests(spec, TWISTS[:2])
    solver = _solver(spec, "mixed")
    a = solver.run(reqs)
    st = solver.last_stats()
    assert (st["graph_captures"], st["graph_replays"]) == (1, 0)
    b = solver.run(reqs)
    st = solver.last_stats()
    assert (st["graph_captures"], st["graph_replays"]) == (1, 1)
    np.testing.assert_array_equal(a["evals"], b["evals"])
    solver.run(reqs[:5])
    st = solver.last_stats()
    assert st["graph_captures"] == 2
    # on the legacy default stream (which cannot itself be captured) the
    # graph is still captured, replayed, and gives the same bits
    solver.set_stream(0)
    np.testing.assert_array_equal(solver.run(reqs)["evals"], a["evals"])
    np.testing.assert_array_equal(solver.run(reqs)["evals"], a["evals"])
    st = solver.last_stats()
    assert (st["graph_captures"], st["graph_replays"]) == (3, 2)


def test_batch_x_in_global_memory_matches_shared():
    """The mixed kernel with its matvec input in global memory (the layout of
    sectors too large for shared memory) gives the shared-memory layout's
    results on the same requests."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.haldane_honeycomb(2, 4)
    reqs = flux_scan_requests(spec, TWISTS)
    solver = _solver(spec, "mixed")
    a = solver.run(reqs)
    solver.set_x_in_shared_memory(False)
    b = solver.run(reqs)
    assert (a["status"] == 0).all() and (b["status"] == 0).all()
    np.testing.assert_allclose(b["evals"], a["evals"], rtol=0, atol=1e-12 * np.nanmax(np.abs(a["evals"])))
    solver.set_x_in_shared_memory(True)
    np.testing.assert_array_equal(solver.run(reqs)["evals"], a["evals"])


def test_batch_sector_too_large_for_shared_memory():
    """A ring of 22 sites at half filling (32,066 orbits: its complex64 x does
    not fit in shared memory) through the batched kernel, against device-wide
    FP64 solves of the same sectors."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.ring_xxz(22, 1.0, 2.0)
    reqs = flux_scan_requests(spec, [(0.0, 0.0), (0.3, 0.0)])[::5]
    solver = _solver(spec, "mixed", nev=2)
    out = solver.run(reqs)
    assert (out["status"] == 0).all()
    cat = solver.catalog
    for b, r in enumerate(reqs):
        basis = A.build_symmetry_sector_basis(cat, r.irrep, group=r.group)
        H = A.MatrixFreeHamiltonian(basis, [(i, j, t) for (i, j, _), t in zip(spec.bilinear_terms(), r.amplitudes)],
                                    spec.density_terms)
        ref, _, _ = H.solve(2, tol=1e-10, want_vectors=False)
        assert abs(out["evals"][b, 0] - ref[0]) <= 1e-9 * max(1.0, abs(ref[0])), (b, out["evals"][b], ref)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("model", ["haldane2x4", "checkerboard3x2_f"])
def test_site_gauge_matches_phase_classes(oracle, model, precision):
    """Flux-twisted translation groups have a site gauge, so flux-scan runs
    take the sign-only hop table (site_gauge in last_stats).  The same run
    with phase-class records (gauge off) solves the same sectors: the lowest
    levels agree within the path's tolerance (1e-9 relative mixed, 1e-11
    FP64), and both runs give the oracle's spectra."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = {"haldane2x4": lambda: L.haldane_honeycomb(2, 4),
            "checkerboard3x2_f": lambda: L.checkerboard(3, 2, n_filled=4)}[model]()
    reqs = flux_scan_requests(spec, TWISTS)
    solver = _solver(spec, precision)
    on = solver.run(reqs)
    st_on = solver.last_stats()
    assert st_on["hop_table"] and st_on["site_gauge"]
    solver.set_site_gauge(False)
    off = solver.run(reqs)
    st_off = solver.last_stats()
    assert st_off["hop_table"] and not st_off["site_gauge"]
    assert (on["status"] == 0).all() and (off["status"] == 0).all()
    np.testing.assert_array_equal(on["dims"], off["dims"])
    ok = off["dims"] > 0
    tol = 1e-9 if precision == "mixed" else 1e-11
    np.testing.assert_allclose(on["evals"][ok, 0], off["evals"][ok, 0], rtol=tol, atol=1e-12)
    _assert_oracle_spectra(oracle, model, spec, TWISTS, on)
    _assert_oracle_spectra(oracle, model, spec, TWISTS, off)
    solver.set_site_gauge(True)
    again = solver.run(reqs)
    assert solver.last_stats()["site_gauge"]
    np.testing.assert_array_equal(again["evals"], on["evals"])


@pytest.mark.parametrize("gauge", [True, False])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("model", ["haldane2x4", "checkerboard3x2_f"])
def test_bank_ordered_records_solve_the_same_sectors(oracle, monkeypatch, model, precision, gauge):
    """The hop table's records are reordered within each row so that a warp's
    shared-memory gathers fall into different bank groups
    (SED_BATCH_BANK_ORDER=0 keeps the fill order).  Only the summation order
    of a row changes: both orders give the same sectors and eigenvalues within
    the path's tolerance (1e-9 relative mixed, 1e-11 FP64), in site-gauge and
    in phase-class mode: the same lowest levels, and the oracle's spectra in
    both."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = {"haldane2x4": lambda: L.haldane_honeycomb(2, 4),
            "checkerboard3x2_f": lambda: L.checkerboard(3, 2, n_filled=4)}[model]()
    reqs = flux_scan_requests(spec, TWISTS)
    out = {}
    for order in ("1", "0"):
        monkeypatch.setenv("SED_BATCH_BANK_ORDER", order)
        solver = _solver(spec, precision)
        solver.set_site_gauge(gauge)
        out[order] = solver.run(reqs)
        st = solver.last_stats()
        assert st["hop_table"] and st["site_gauge"] == gauge
        assert (out[order]["status"] == 0).all()
    np.testing.assert_array_equal(out["1"]["dims"], out["0"]["dims"])
    ok = out["0"]["dims"] > 0
    tol = 1e-9 if precision == "mixed" else 1e-11
    np.testing.assert_allclose(out["1"]["evals"][ok, 0], out["0"]["evals"][ok, 0], rtol=tol, atol=1e-12)
    for order in ("1", "0"):
        _assert_oracle_spectra(oracle, model, spec, TWISTS, out[order])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("model", ["haldane2x4", "checkerboard3x2_f"])
def test_batch_eigenvectors(oracle, model, precision):
    """sed_batch_run_vectors: every request's eigenvectors in sector-row
    order, in the gauge of its own twisted group.  Each is a unit eigenvector
    of the oracle's sector matrix for its eigenvalue (residual 1e-8 |E| FP64,
    1e-5 |E| mixed), and it spans the same eigenvector as the single-sector
    solve of that sector (|<v_batch, v_single>| = 1 for isolated levels)."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = {"haldane2x4": lambda: L.haldane_honeycomb(2, 4),
            "checkerboard3x2_f": lambda: L.checkerboard(3, 2, n_filled=4)}[model]()
    reqs = flux_scan_requests(spec, TWISTS)
    solver = _solver(spec, precision, nev=3)
    out = solver.run(reqs, want_vectors=True)
    assert (out["status"] == 0).all()
    nG = len(reqs) // len(TWISTS)
    rtol = 1e-8 if precision == "fp64" else 1e-5
    for b, r in enumerate(reqs):
        th = TWISTS[b // nG]
        case = Case(model, spec, theta=th)
        _, sec, op = oracle_objects(oracle, case, b % nG)
        if sec.dim == 0:
            continue
        Hd = op.dense()
        ref = np.linalg.eigvalsh(Hd)
        V = out["evecs"][b]
        assert V.shape == (sec.dim, min(3, sec.dim))
        for i in range(V.shape[1]):
            v, e = V[:, i], out["evals"][b, i]
            assert abs(np.linalg.norm(v) - 1.0) <= 1e-9, (b, i)
            assert np.linalg.norm(Hd @ v - e * v) <= rtol * max(1.0, abs(e)), (model, b, i, precision)
        # against the single-sector solve of the same sector, for levels
        # isolated from their neighbours
        if b % 5 == 0:
            cat = solver.catalog
            basis = A.build_symmetry_sector_basis(cat, r.irrep, group=r.group)
            H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms(th), spec.density_terms)
            _, vs, _ = H.solve(V.shape[1], tol=1e-10)
            for i in range(V.shape[1]):
                lo = ref[i - 1] if i > 0 else -np.inf
                hi = ref[i + 1] if i + 1 < len(ref) else np.inf
                if min(ref[i] - lo, hi - ref[i]) > 1e-6:
                    assert abs(abs(np.vdot(vs[:, i], V[:, i])) - 1.0) <= 1e-6, (model, b, i, precision)


def test_batch_launch_autotuner(oracle):
    """The first run of a catalog shape sweeps the candidate launch shapes
    (threads per row 1 and 2 of the table matvec; Krylov dimensions 20, 24,
    28) on one wave of its requests and keeps the fastest; a second solver of
    the same shape reuses it without a sweep.  Every pinned shape solves the
    same sectors to the oracle's dense spectrum, and its lowest levels agree
    with the tuned one within the mixed path's 1e-9."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.haldane_honeycomb(2, 4, tp=0.55)
    reqs = flux_scan_requests(spec, TWISTS[:2])
    s1 = _solver(spec, "mixed", nev=5)  # nev 5: a shape key no other test tunes first
    tuned = s1.run(reqs)
    sh = s1.shape()
    assert sh["tune_runs"] == 1 and sh["threads_per_row"] in (1, 2) and sh["krylovdim"] in (20, 24, 28)
    s2 = _solver(spec, "mixed", nev=5)
    s2.run(reqs)
    assert s2.shape()["tune_runs"] == 0 and s2.shape()["krylovdim"] == sh["krylovdim"]
    nG = len(reqs) // 2
    for m, tpr in ((20, 1), (24, 2), (28, 2)):
        s2.set_shape(m, tpr)
        out = s2.run(reqs)
        assert s2.shape()["krylovdim"] == m and s2.shape()["threads_per_row"] == tpr
        assert (out["status"] == 0).all()
        ok = out["dims"] > 0
        np.testing.assert_allclose(out["evals"][ok, 0], tuned["evals"][ok, 0], rtol=1e-9, atol=1e-12)
        for b in range(len(reqs)):
            _, sec, op = oracle_objects(oracle, Case("haldane2x4_tp", spec, theta=TWISTS[b // nG]), b % nG)
            if sec.dim == 0:
                continue
            ref = np.linalg.eigvalsh(op.dense())
            assert_lanczos_spectrum(out["evals"][b, :min(5, sec.dim)], ref, 1e-9 * max(1.0, abs(ref[0])))
    s2.set_shape(0, 0)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_device_resident_request_loop(oracle, precision):
    """The device-resident loop (sed_batch_ring_*): requests submitted one at
    a time to a running persistent launch give the batch run's eigenvalues
    (same seeds; within the path's tolerance) and the oracle's spectra; a
    full ring refuses a submit until a ticket is collected; blocks that stay
    idle leave and the next submit relaunches; a batch run is refused while
    the ring runs."""
    import time

    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.haldane_honeycomb(2, 4)
    reqs = flux_scan_requests(spec, TWISTS)
    ref = _solver(spec, precision).run(reqs)
    solver = _solver(spec, precision)
    solver.ring_start(capacity=16, n_blocks=8, idle_ms=50)
    try:
        with pytest.raises(_lib.SEDError):
            solver.run(reqs[:2])
        got = np.full_like(ref["evals"], np.nan)
        dims = np.zeros(len(reqs), dtype=np.int64)
        pending = []
        for i, r in enumerate(reqs):
            while True:
                try:
                    pending.append((i, solver.ring_submit(r)))
                    break
                except _lib.SEDError as e:
                    assert e.code == _lib.SED_ERR_LIMIT and len(pending) == 16
                    j, t = pending.pop(0)
                    ev, st, dims[j] = solver.ring_wait(t)
                    assert st == 0
                    got[j] = ev
        for j, t in pending:
            ev, st, dims[j] = solver.ring_wait(t)
            assert st == 0
            got[j] = ev
        np.testing.assert_array_equal(dims, ref["dims"])
        ok = ref["dims"] > 0
        tol = 1e-9 if precision == "mixed" else 1e-11
        np.testing.assert_allclose(got[ok, 0], ref["evals"][ok, 0], rtol=tol, atol=1e-12)
        _assert_oracle_spectra(oracle, "haldane2x4", spec, TWISTS, {"dims": dims, "evals": got})
        launches = solver.ring_info()["launches"]
        time.sleep(0.5)  # longer than idle_ms: the blocks leave
        assert not solver.ring_info()["running"]
        t = solver.ring_submit(reqs[3])
        ev, st, _ = solver.ring_wait(t)
        assert st == 0 and solver.ring_info()["launches"] > launches
        np.testing.assert_allclose(ev[0], ref["evals"][3, 0], rtol=tol, atol=1e-12)
    finally:
        solver.ring_stop()
    out = solver.run(reqs[:4])  # the object runs batches again after the ring
    assert (out["status"] == 0).all()


def test_ring_calls_from_several_threads():
    """The ring calls are thread-safe among themselves: two threads waiting on
    one ticket get the answer once (the other: "already collected"); a stop
    while another thread waits ends that wait with an error, or with the
    answer if it came first; a ticket of a stopped ring is refused after a
    restart; the restarted ring answers as before."""
    import threading

    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.haldane_honeycomb(2, 4)
    reqs = flux_scan_requests(spec, TWISTS)
    ref = _solver(spec, "mixed").run(reqs[:8])
    solver = _solver(spec, "mixed")
    solver.ring_start(capacity=16, n_blocks=8, idle_ms=50)
    try:
        for i in range(3):
            t = solver.ring_submit(reqs[i])
            got, errs = [], []

            def waiter():
                try:
                    got.append(solver.ring_wait(t, timeout_ms=60_000))
                except _lib.SEDError as e:
                    errs.append(str(e))

            th = [threading.Thread(target=waiter) for _ in range(2)]
            for x in th:
                x.start()
            for x in th:
                x.join()
            assert len(got) == 1 and len(errs) == 1 and "collected" in errs[0], (got, errs)
            ev, st, dim = got[0]
            assert st == 0 and dim == ref["dims"][i]
            if dim:
                np.testing.assert_allclose(ev[0], ref["evals"][i, 0], rtol=1e-9, atol=1e-12)
        t = solver.ring_submit(reqs[3])
        got, errs = [], []

        def waiter2():
            try:
                got.append(solver.ring_wait(t, timeout_ms=60_000))
            except _lib.SEDError as e:
                errs.append(str(e))

        w = threading.Thread(target=waiter2)
        w.start()
        solver.ring_stop()
        w.join()
        assert len(got) + len(errs) == 1
        if errs:
            assert "stopped" in errs[0] or "not running" in errs[0], errs
        else:
            assert got[0][1] == 0
        solver.ring_start(capacity=16, n_blocks=8, idle_ms=50)
        with pytest.raises(_lib.SEDError):
            solver.ring_wait(t + 5, timeout_ms=0)
        ev, st, dim = solver.ring_wait(solver.ring_submit(reqs[4]))
        assert st == 0 and dim == ref["dims"][4]
        if dim:
            np.testing.assert_allclose(ev[0], ref["evals"][4, 0], rtol=1e-9, atol=1e-12)
    finally:
        solver.ring_stop()


@pytest.mark.parametrize("statistics", ["fermionic", "bosonic"])
def test_flux_period_one(oracle, statistics):
    """A whole flux quantum changes nothing but the momentum labels
    (flux_regression.jl:53-60, global energies at twist 0 and 1 equal): the
    batch at twists (0, 0) and (1, 0) gives the same multiset of sector
    dimensions and of sector ground energies (1e-10), and every request at
    twist (0.23, 0) in between the oracle's spectrum."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.checkerboard(3, 2, n_filled=4, statistics=statistics)
    twists = [(0.0, 0.0), (0.23, 0.0), (1.0, 0.0)]
    out = _solver(spec, "mixed").run(flux_scan_requests(spec, twists))
    assert (out["status"] == 0).all()
    _assert_oracle_spectra(oracle, f"checkerboard3x2_{statistics}", spec, twists, out)
    nk = len(out["dims"]) // len(twists)
    d0, d1 = out["dims"][:nk], out["dims"][2 * nk:]
    np.testing.assert_array_equal(np.sort(d0), np.sort(d1))
    e0 = np.sort(out["evals"][:nk, 0][d0 > 0])
    e1 = np.sort(out["evals"][2 * nk:, 0][d1 > 0])
    np.testing.assert_allclose(e1, e0, rtol=0, atol=1e-10 * max(1.0, np.abs(e0).max()))
    assert np.abs(out["evals"][nk:2 * nk, 0][out["dims"][nk:2 * nk] > 0].min() - e0.min()) > 1e-6  # the twist matters


def test_gauge_only_phase_table_when_shared_memory_is_tight():
    """Checkerboard 4x4 with Np = 5 (12,586 orbits): its complex64 x fills so
    much shared memory that the full phase-id table (2048 entries) does not
    fit beside it.  The batch then keeps gauge mode's three entries (+1, -1,
    zero), so flux-scan runs still take the site-gauge hop table, and give the
    on-the-fly matvec's lowest levels (1e-9)."""
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.checkerboard(4, 4, n_filled=5)
    reqs = flux_scan_requests(spec, [(0.0, 0.0), (0.3, 0.7)])
    tab = _solver(spec, "mixed", max_requests=64)
    out = tab.run(reqs)
    st = tab.last_stats()
    assert st["hop_table"] and st["site_gauge"]
    fly = _solver(spec, "mixed", max_requests=64)
    fly.set_hop_table(False)
    ref = fly.run(reqs)
    assert not fly.last_stats()["hop_table"]
    assert (out["status"] == 0).all() and (ref["status"] == 0).all()
    np.testing.assert_array_equal(out["dims"], ref["dims"])
    ok = ref["dims"] > 0
    np.testing.assert_allclose(out["evals"][ok, 0], ref["evals"][ok, 0], rtol=1e-9, atol=1e-12)
