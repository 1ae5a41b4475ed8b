"""Batched sector solves: many (momentum, flux twist) sectors of one model in
one persistent device launch (C ABI ``sed_batch_*``).

This replaces the reference's sequential scans over sectors and twists
(``_ed_scan_sectors!`` src/symmetry_resolved_ed.jl:1199-1256, the flux branch
of ``ed_scan!`` :1320-1355, ``many_body_chern_number`` grids), each of which
calls ``diagonalize_block_matrixfree`` once per sector.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from . import _lib
from ._lib import check, ptr
from .api import Symmetry_Orbit_Catalog
from .groups import Finite_Symmetry_Group, OneDim_Irrep


@dataclass
class SectorRequest:
    """One sector solve: momentum irrep, (twisted) group, hop amplitudes, seed."""

    irrep: OneDim_Irrep
    group: Finite_Symmetry_Group
    amplitudes: Sequence[complex]
    seed: int = 0x5EED0000


class BatchedSectorSolver:
    """Persistent-kernel solver for many small sectors that share a catalog.

    ``bilinear_pairs`` is the fixed 1-based (i, j) list; every request supplies
    the amplitude of each pair (twisted boundary phases change amplitudes, not
    the pair list).  ``precision="mixed"`` runs complex64 matvecs with FP64
    Lanczos and an FP64 Rayleigh-Ritz polish; ``"fp64"`` is all FP64.
    ``krylovdim=0`` lets the launch autotuner choose the Krylov dimension
    (with the matvec's threads per row); a positive value fixes it.

    Every sector is solved by Lanczos, whatever its size (the reference and
    ``MatrixFreeHamiltonian.solve`` take a dense solve up to 500 rows), so an
    exactly degenerate level may be listed fewer times than its multiplicity,
    as in the reference's KrylovKit branch."""

    def __init__(self, catalog: Symmetry_Orbit_Catalog, bilinear_pairs, density_terms, precision: str = "mixed",
                 nev: int = 4, krylovdim: int = 0, max_requests: int = 1024):
        self.catalog = catalog
        n_site = catalog.symmetry_group.n_site
        self.pairs = [(int(i), int(j)) for (i, j) in bilinear_pairs]
        bij = np.ascontiguousarray([[i - 1, j - 1] for (i, j) in self.pairs], dtype=np.int32).reshape(-1, 2)
        if bij.size and (bij.min() < 0 or bij.max() >= n_site):
            raise ValueError(f"bilinear site index outside 1:{n_site}")
        dij = np.ascontiguousarray([[int(i) - 1, int(j) - 1] for (i, j, _) in density_terms], dtype=np.int32)
        dv = np.ascontiguousarray([complex(v) for (_, _, v) in density_terms], dtype=np.complex128)
        prec = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[precision]
        h = C.c_void_p()
        check(_lib.load().sed_batch_create(catalog.handle, len(self.pairs), ptr(bij), len(dv),
                                           ptr(dij.reshape(-1, 2)) if len(dv) else None,
                                           ptr(dv) if len(dv) else None, prec, nev, krylovdim, max_requests,
                                           C.byref(h)))
        self._h = h
        self.nev = nev
        self.max_requests = max_requests
        self.precision = precision
        self._bij = bij

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().sed_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def info(self):
        sm, nb, fp = C.c_int64(), C.c_int64(), C.c_int64()
        check(_lib.load().sed_batch_info(self._h, C.byref(sm), C.byref(nb), C.byref(fp)))
        return {"smem_bytes": sm.value, "blocks": nb.value, "footprint_bytes": fp.value}

    def pack(self, requests: Sequence[SectorRequest]):
        G0 = self.catalog.symmetry_group
        n = len(requests)
        chi = np.zeros((n, len(G0)), dtype=np.complex128)
        ph = np.zeros((n, len(G0), G0.n_site), dtype=np.complex128)
        amp = np.zeros((n, max(len(self.pairs), 1)), dtype=np.complex128)
        seeds = np.zeros(n, dtype=np.uint64)
        for b, r in enumerate(requests):
            if not r.group.same_permutations(G0):
                raise ValueError("every request's group must have the catalog's permutations")
            if len(r.amplitudes) != len(self.pairs):
                raise ValueError("one amplitude per bilinear pair")
            chi[b] = r.irrep.array()
            ph[b] = r.group.phases()
            amp[b, :len(self.pairs)] = np.asarray(r.amplitudes, dtype=np.complex128)
            seeds[b] = r.seed
        return chi, ph, amp, seeds

    def run_packed(self, chi, ph, amp, seeds, tol: float = 1e-10, maxiter: int = 300, want_vectors: bool = False):
        n = len(seeds)
        self._last_n = n
        if n > self.max_requests:
            raise ValueError("more requests than max_requests")
        ev = np.zeros((n, self.nev), dtype=np.float64)
        st = np.zeros(n, dtype=np.int32)
        dims = np.zeros(n, dtype=np.int64)
        delta = np.zeros(n, dtype=np.float64)
        nmv = np.zeros(n, dtype=np.int32)
        out = {"evals": ev, "status": st, "dims": dims, "delta_polish": delta, "matvecs": nmv}
        if not want_vectors:
            check(_lib.load().sed_batch_run(self._h, n, ptr(chi), ptr(ph), ptr(amp), ptr(seeds), float(tol),
                                            int(maxiter), ptr(ev), ptr(st), ptr(dims), ptr(delta), ptr(nmv)))
            return out
        ld = max(int(self.catalog.n_orbits), 1)
        vec = np.zeros((n, self.nev, ld), dtype=np.complex128)
        check(_lib.load().sed_batch_run_vectors(self._h, n, ptr(chi), ptr(ph), ptr(amp), ptr(seeds), float(tol),
                                                int(maxiter), ptr(ev), ptr(st), ptr(dims), ptr(delta), ptr(nmv),
                                                ptr(vec), ld))
        # request b: vecs[:, i] is its i-th eigenvector in sector-row order
        out["evecs"] = [vec[b, :min(self.nev, int(dims[b])), :int(dims[b])].T.copy() for b in range(n)]
        return out

    def last_stats(self):
        """Hops of one matvec and device start/end clocks (ns) of the last run's requests."""
        n = getattr(self, "_last_n", 0)
        hops = np.zeros(n, dtype=np.int64)
        t0 = np.zeros(n, dtype=np.int64)
        t1 = np.zeros(n, dtype=np.int64)
        check(_lib.load().sed_batch_last_stats(self._h, ptr(hops), ptr(t0), ptr(t1)))
        nf, tab, nrec = C.c_int32(0), C.c_int32(0), C.c_int64(0)
        check(_lib.load().sed_batch_last_info(self._h, C.byref(nf), C.byref(tab), C.byref(nrec)))
        caps, reps = C.c_int32(0), C.c_int32(0)
        check(_lib.load().sed_batch_graph_info(self._h, C.byref(caps), C.byref(reps)))
        gauge = C.c_int32(0)
        check(_lib.load().sed_batch_last_gauge(self._h, C.byref(gauge)))
        return {"hops": hops, "t_start_ns": t0, "t_end_ns": t1, "fp64_fallbacks": int(nf.value),
                "hop_table": bool(tab.value), "hop_records": int(nrec.value), "site_gauge": bool(gauge.value),
                "graph_captures": int(caps.value), "graph_replays": int(reps.value)}

    def set_x_in_shared_memory(self, enable: bool) -> None:
        """Keep the complex64 matvec input in shared memory (default when it
        fits) or in global memory (the layout of sectors too large for it)."""
        check(_lib.load().sed_batch_set_x_in_shared_memory(self._h, int(bool(enable))))

    def set_shape(self, krylovdim: int = 0, threads_per_row: int = 0) -> None:
        """Pin the launch shape, or (0, 0) to let the autotuner choose."""
        check(_lib.load().sed_batch_set_shape(self._h, int(krylovdim), int(threads_per_row)))

    def shape(self):
        """(krylovdim, threads_per_row) of the last run and the number of
        autotuner sweeps this solver ran."""
        m, t, n = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        check(_lib.load().sed_batch_shape(self._h, C.byref(m), C.byref(t), C.byref(n)))
        return {"krylovdim": m.value, "threads_per_row": t.value, "tune_runs": n.value}

    def set_site_gauge(self, enable: bool) -> None:
        """Solve runs whose requests all have a site gauge (the flux-twisted
        translation groups do) in that gauge, with sign-only hop records
        (default), or always with phase-class records."""
        check(_lib.load().sed_batch_set_site_gauge(self._h, int(bool(enable))))

    def set_hop_table(self, enable: bool) -> None:
        """Stream the shared hop table (default) or derive every hop on the fly."""
        check(_lib.load().sed_batch_set_hop_table(self._h, int(bool(enable))))

    def run_device(self, n: int, d_chi: int, d_phase: int, d_amp: int, d_seeds: int, d_evals: int, d_status: int,
                   d_dims: int, d_delta: int, d_nmv: int, tol: float = 1e-10, maxiter: int = 300) -> None:
        """Asynchronous launch on device-resident buffers (raw device pointers)."""
        self._last_n = n
        vp = C.c_void_p
        check(_lib.load().sed_batch_run_device(self._h, n, vp(d_chi), vp(d_phase), vp(d_amp), vp(d_seeds),
                                               float(tol), int(maxiter), vp(d_evals), vp(d_status), vp(d_dims),
                                               vp(d_delta), vp(d_nmv)))

    # ---------------------------------------------------- device-resident loop
    def ring_start(self, capacity: int = 1024, n_blocks: int = 152, idle_ms: int = 100) -> None:
        """Start the device-resident request loop (sed_batch_ring_start): one
        persistent launch whose blocks claim requests from a ring as they are
        submitted; a block idle for idle_ms leaves, and the next submit or wait
        relaunches.  Needs a site gauge for every request (flux-twisted
        translation groups have one)."""
        check(_lib.load().sed_batch_ring_start(self._h, int(capacity), int(n_blocks), int(idle_ms)))

    def ring_submit(self, r: SectorRequest) -> int:
        chi, ph, amp, seeds = self.pack([r])
        t = C.c_int64(0)
        check(_lib.load().sed_batch_ring_submit(self._h, chi.ctypes.data, ph.ctypes.data, amp.ctypes.data,
                                                int(seeds[0]), C.byref(t)))
        return t.value

    def ring_wait(self, ticket: int, timeout_ms: int = 600_000):
        """(evals, status, dim) of a ticket; raises SEDError (SED_ERR_TIMEOUT)
        when it has not finished within timeout_ms."""
        ev = np.zeros(self.nev, dtype=np.float64)
        st, dim = C.c_int32(0), C.c_int64(0)
        check(_lib.load().sed_batch_ring_wait(self._h, int(ticket), int(timeout_ms), ev.ctypes.data, C.byref(st),
                                              C.byref(dim)))
        return ev, st.value, dim.value

    def ring_info(self) -> dict:
        n, nb, run = C.c_int64(0), C.c_int32(0), C.c_int32(0)
        check(_lib.load().sed_batch_ring_info(self._h, C.byref(n), C.byref(nb), C.byref(run)))
        return {"launches": n.value, "blocks": nb.value, "running": bool(run.value)}

    def ring_stop(self) -> None:
        check(_lib.load().sed_batch_ring_stop(self._h))

    def set_stream(self, stream_ptr: int) -> None:
        check(_lib.load().sed_batch_set_stream(self._h, C.c_void_p(stream_ptr)))

    def run(self, requests: Sequence[SectorRequest], tol: float = 1e-10, maxiter: int = 300,
            want_vectors: bool = False):
        """Solve the requests in one launch.  With want_vectors, out["evecs"][b]
        holds request b's eigenvectors as columns (sector-row order, the
        reference's (vals, vecs) layout, SRE:1124)."""
        return self.run_packed(*self.pack(requests), tol=tol, maxiter=maxiter, want_vectors=want_vectors)


def flux_scan_requests(spec, twists: Sequence[Sequence[float]], seed0: int = 0x5EED0000) -> List[SectorRequest]:
    """All momentum sectors x the given twists of a lattice model (the batch
    of the reference's flux scans), with seeds 0x5EED0000 + request index."""
    from .lattice import build_translation_group, build_translation_irrep_list

    reqs = []
    pairs = [(i, j) for (i, j, _) in spec.bilinear_terms((0.0, 0.0))]
    for th in twists:
        G = build_translation_group(spec.lattice, th)
        terms = spec.bilinear_terms(th)
        assert [(i, j) for (i, j, _) in terms] == pairs
        amps = [t for (_, _, t) in terms]
        for irr in build_translation_irrep_list(G, spec.lattice):
            reqs.append(SectorRequest(irr, G, amps, seed0 + len(reqs)))
    return reqs
