"""Host-side arithmetic behind reported numbers (no GPU): the roofline's
Lanczos byte count follows the thick-restart schedule the kernels run, and the
served scheduler's device-memory estimate covers what a device-wide mixed
solve allocates, and the served scheduler's ring route handles a full ring and
a refused request."""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))

import bench  # noqa: E402
from realspace_exactdiagonalization_gb300.serving import solver_footprint  # noqa: E402


def _schedule_bytes(nmv, dim, m, keep, n_polish, elem):
    """The thick-restart schedule walked step by step: the first cycle grows
    the basis 1..m, every later one keep+1..m; each step streams three
    vectors and reads the k basis vectors its dots sweep; each completed
    cycle ends in a rotation of m vectors into keep."""
    steps = max(nmv - n_polish, 0)
    k, total, restarts, open_cycle = 0, 0, 0, False
    for _ in range(steps):
        k += 1
        open_cycle = True
        total += 3 + k
        if k == m:
            restarts += 1
            k = keep
            open_cycle = False
    if open_cycle:  # a partial cycle, first or last, also ends in a rotation
        restarts += 1
    return float((total + restarts * (m + keep)) * dim * elem)


def test_lanczos_bytes_follows_the_restart_schedule():
    for nmv in (0, 5, 6, 7, 30, 31, 160, 163, 301):
        for m, keep in ((24, 8), (24, 15), (30, 5)):
            for elem in (8, 16):
                got = bench.lanczos_bytes(nmv, 11240, m=m, keep=keep, n_polish=6, elem=elem)
                assert got == _schedule_bytes(nmv, 11240, m, keep, 6, elem), (nmv, m, keep, elem)


def test_lanczos_bytes_scale_with_element_size():
    assert bench.lanczos_bytes(160, 1000, elem=16) == 2 * bench.lanczos_bytes(160, 1000, elem=8)


def test_solver_footprint_covers_the_allocations():
    """The device-wide mixed solve of nev requested pairs allocates, with
    nw = nev + 2 and m = max(30, 2 nw + 1) (sed_lanczos.cu): two complex64
    buffers of max(m + 1, 3 nw + 1) vectors plus one work vector, all padded
    to 64 elements, and 5 nw FP64 vectors plus two FP64 matvec inputs."""
    for n in (1000, 112_720, 14_113_596):
        for nev in (1, 3):
            nw = nev + 2
            m = max(30, 2 * nw + 1)
            ldc = (n + 63) // 64 * 64
            alloc = (2 * max(m + 1, 3 * nw + 1) + 1) * ldc * 8 + (5 * nw) * n * 16 + 2 * ldc * 16
            assert solver_footprint(n, nev) >= alloc, (n, nev)
            assert solver_footprint(n, nev + 1) > solver_footprint(n, nev)


def test_ring_route_waits_for_a_slot_and_reports_refusals_per_request():
    """SectorServer.submit on a family served by a device-resident ring: a full
    ring (SED_ERR_LIMIT) is a wait for the collector, not a failure; any other
    refusal is reported on the request itself (status, NaN evals, message), as
    the other routes report theirs, and the stream goes on.  Host logic only:
    the ring is a fake."""
    import queue
    import threading
    import time
    from types import SimpleNamespace

    import numpy as np

    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300.serving import Request, SectorServer

    class FakeRing:
        def __init__(self, outcomes):
            self.outcomes = list(outcomes)  # SED_* codes to raise, then tickets
            self.calls = 0

        def ring_submit(self, req):
            self.calls += 1
            o = self.outcomes.pop(0)
            if isinstance(o, int) and o < 0:
                raise _lib.SEDError(-o, f"refused with {-o}")
            return o

    srv = object.__new__(SectorServer)  # no catalogs or device state: only the submit path
    srv._t0 = time.perf_counter()
    srv._lock = threading.Condition()
    srv._done = []
    srv._request_arrays = lambda fam, reqs: [None for _ in reqs]
    ring = FakeRing([-_lib.SED_ERR_LIMIT, -_lib.SED_ERR_LIMIT, 7, -_lib.SED_ERR_ARG, 8])
    srv.families = {"ring20": SimpleNamespace(name="ring20", solvers=[ring])}
    srv._ring_q = {"ring20": queue.Queue()}

    r1 = Request(rid=1, family="ring20", k_index=0, twist=(0.0, 0.0))
    srv.submit(r1)  # two full-ring refusals, then ticket 7
    assert ring.calls == 3 and srv._ring_q["ring20"].get_nowait() == (7, r1) and not srv._done
    r2 = Request(rid=2, family="ring20", k_index=0, twist=(0.0, 0.0), nev=2)
    srv.submit(r2)  # refused outright: reported on the request
    assert srv._done == [r2] and r2.status == _lib.SED_ERR_ARG and r2.route == "ring"
    assert np.isnan(r2.evals).all() and len(r2.evals) == 2 and "refused" in r2.error
    assert srv._ring_q["ring20"].empty()
    r3 = Request(rid=3, family="ring20", k_index=0, twist=(0.0, 0.0))
    srv.submit(r3)  # the stream goes on
    assert srv._ring_q["ring20"].get_nowait() == (8, r3)
