"""Host-side arithmetic behind reported numbers (no GPU): the roofline's
Lanczos byte count follows the thick-restart schedule the kernels run, and the
served scheduler's device-memory estimate covers what a device-wide mixed
solve allocates."""
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
