"""Served ground-state requests with continuous batching.

A request is one sector solve: (model family, momentum, flux twist, nev).  The
reference answers such streams one sector at a time
(``ed_scan_at_irrep_matrixfree!``, src/symmetry_resolved_ed.jl:1092-1128, inside
the loops of ``_ed_scan_sectors!`` :1199-1256 and ``ed_scan!`` :1320-1355).
Here a scheduler keeps the GPU busy with many requests at once:

* every model family has one device catalog, built once and kept resident;
  a request only brings its momentum, its twisted group phases and its hop
  amplitudes;
* small sectors go to the persistent batched kernel (``sed_batch_run``); two
  lanes alternate, so requests that arrive while one batch runs start in the
  next launch as soon as a lane frees, overlapping the batch in flight;
* mid-size sectors go to the same batched kernel with its matvec input in
  global memory, on a lane of their own, so they neither wait behind the
  device-wide solves' kernels nor delay the small sectors' lanes;
* large sectors go to device-wide solves (``sed_solve``), several at once on
  their own streams, each admitted only while the reserved device memory of
  the solves in flight plus its own footprint stays within the budget;
* every library call releases the Python GIL, so the lanes and workers drive
  the GPU concurrently from one process.
A request's result depends only on its own inputs and seed: the same request
gives the same eigenvalues alone and in any mix.

:class:`NativeSectorServer` runs the same scheduling in the library itself
(``sed_server_*``: C++ threads behind the C ABI, the entry points a Julia
service would call).  With ``ring_blocks > 0`` the batched families are
answered by device-resident request loops (``sed_batch_ring_*``) instead of
batch lanes.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import api as A
from . import lattice as L
from .batched import BatchedSectorSolver
from .groups import statistics_from_name

# sectors whose catalog has at most SMALL_MAX_ORBITS orbits are solved by the
# batched kernel, one thread block each (its complex64 matvec input fits in
# shared memory), on the shared batch lanes; larger sectors take concurrent
# device-wide solves.  Sectors up to medium_max_orbits can instead take the
# batched kernel with that input in global memory, on lanes of their own.
# That route is off by default (MEDIUM_MAX_ORBITS = 0): in the served mix its
# thread blocks, each holding an SM for about a second per batch, slowed the
# other routes more than they relieved the device-wide one.
SMALL_MAX_ORBITS = 16384
MEDIUM_MAX_ORBITS = 0
# device-wide solves of catalogs below this size run on high-priority streams:
# their short host-synchronised steps then go ahead of the larger solves'
# queued kernels instead of waiting behind them
PRIORITY_MAX_ORBITS = 2_000_000
# mid-size catalogs keep their batch workspace (the per-block Lanczos basis)
# to MEDIUM_MAX_BATCH concurrent requests per lane
MEDIUM_MAX_BATCH = 48


@dataclass
class Family:
    name: str
    spec: L.ModelSpec
    catalog: A.Symmetry_Orbit_Catalog
    pairs: List[tuple]
    route: str  # "batch" | "medium" | "large"
    solvers: List[BatchedSectorSolver] = field(default_factory=list)

    @property
    def n_orbits(self) -> int:
        return self.catalog.n_orbits


@dataclass
class Request:
    rid: int
    family: str
    k_index: int
    twist: tuple
    nev: int = 1
    seed: int = 0
    arrival: float = 0.0
    # results
    evals: Optional[np.ndarray] = None
    status: int = -1
    dim: int = -1
    t_start: float = 0.0
    t_end: float = 0.0
    delta_polish: float = 0.0
    route: str = ""
    error: str = ""  # the library's message when status != 0


def config5_families(hubbard_blocks: bool = True) -> Dict[str, L.ModelSpec]:
    """The served mix: hard-core boson rings (t=1, V=2) at half filling, checkerboard
    fermions at 1/3 lower-band filling (4x4: Np=5, since 16/3 is not an integer),
    and spinful Hubbard (t=1, U=8) with N_up = N_down = 5 or 6: by default in its
    (N_up, N_down) block (a two-species catalog); with hubbard_blocks=False as
    the reference encodes it, a fixed total particle number 2 N_up over all
    S^z."""
    fam = {}
    for n in (20, 24, 28):
        fam[f"ring{n}"] = L.ring_xxz(n, 1.0, 2.0)
    fam["checkerboard3x4"] = L.checkerboard(3, 4, n_filled=4)
    fam["checkerboard4x4"] = L.checkerboard(4, 4, n_filled=5)
    for (l1, l2) in ((3, 4), (4, 4)):
        for nh in (5, 6):
            fam[f"hubbard{l1}x{l2}_{nh}+{nh}"] = (L.hubbard_square(l1, l2, n_up=nh, n_dn=nh) if hubbard_blocks
                                                  else L.hubbard_square(l1, l2, n_filled=2 * nh))
    return fam


def random_requests(families: Dict[str, L.ModelSpec], n: int, rate: float, seed: int = 20261203,
                    nev: int = 1) -> List[Request]:
    """A seeded Poisson stream: uniformly drawn (family, momentum, twist),
    exponential inter-arrival times with the given rate (requests/s)."""
    rng = np.random.default_rng(seed)
    names = sorted(families)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate) if rate > 0 else 0.0
        name = names[rng.integers(len(names))]
        spec = families[name]
        nk = spec.lattice.sample_size[0] * spec.lattice.sample_size[1]
        tw = (float(rng.random()), float(rng.random()) if spec.lattice.sample_size[1] > 1 else 0.0)
        out.append(Request(i, name, int(rng.integers(nk)), tw, nev, 0x5EED0000 + i, t))
    return out


def solver_footprint(n_orbits: int, nev: int, krylovdim: int = 30) -> int:
    """Device bytes one device-wide mixed solve holds: the complex64 Lanczos
    basis, restart buffer and work vector (8 B per element, padded to 64
    elements), the FP64 polish block and matvec inputs (16 B per element),
    and the operator's per-orbit tables."""
    nw = nev + 2
    m = max(krylovdim, 2 * nw + 1)
    slots8 = 2 * max(m + 1, 3 * nw + 1) + 1
    slots16 = 5 * nw + 2
    padded = (n_orbits + 63) // 64 * 64
    return int(slots8 * padded * 8 + slots16 * padded * 16 + n_orbits * 17 + (64 << 20))


class SectorServer:
    def __init__(self, families: Dict[str, L.ModelSpec], budget_bytes: float = 160e9, batch_lanes: int = 2,
                 large_workers: int = 3, max_batch: int = 512, small_max_orbits: int = SMALL_MAX_ORBITS,
                 precision: str = "mixed", tol: float = 1e-10, nev: int = 1,
                 medium_max_orbits: int = MEDIUM_MAX_ORBITS, medium_lanes: int = 1,
                 priority_max_orbits: int = PRIORITY_MAX_ORBITS, warm_up: bool = True,
                 medium_max_batch: int = MEDIUM_MAX_BATCH, large_sm_limit: int = 0, ring_blocks: int = 0,
                 ring_idle_ms: int = 2, large_krylovdim: int = 24):
        self.budget = float(budget_bytes)
        # device-wide solves size their grids for this many SMs (0: all); the
        # mid-size lane's persistent blocks (at most medium_max_batch of them,
        # one SM each) keep the rest
        self.large_sm_limit = int(large_sm_limit)
        # ring_blocks > 0: each batched family runs a device-resident request
        # loop (sed_batch_ring_*) on up to that many SMs instead of batch
        # lanes; requests go straight into its ring
        self.ring_blocks = int(ring_blocks)
        # Krylov dimension of the device-wide solves: 24 answered the served
        # mix's one-eigenvalue requests 3.5 % faster than the library's 30
        self.large_krylovdim = int(large_krylovdim)
        self.ring_idle_ms = int(ring_idle_ms)
        self.priority_max_orbits = priority_max_orbits
        self.precision = precision
        self.tol = tol
        self.max_batch = max_batch
        self.families: Dict[str, Family] = {}
        self.resident = 0
        for name, spec in families.items():
            G = L.build_translation_group(spec.lattice)
            cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                                 particle_statistics=statistics_from_name(spec.statistics))
            pairs = [(i, j) for (i, j, _) in spec.bilinear_terms()]
            if cat.n_orbits <= small_max_orbits:
                route = "batch"
            elif cat.n_orbits <= medium_max_orbits and medium_lanes > 0:
                route = "medium"
            else:
                route = "large"
            fam = Family(name, spec, cat, pairs, route)
            self.resident += cat.n_states * 8 + cat.n_orbits * 9
            if route != "large":
                cap = max_batch if route == "batch" else min(max_batch, medium_max_batch)
                n_solvers = batch_lanes if route == "batch" else medium_lanes
                if route == "batch" and self.ring_blocks > 0:
                    n_solvers = 1
                for _ in range(n_solvers):
                    s = BatchedSectorSolver(cat, pairs, spec.density_terms, precision=precision, nev=nev,
                                            max_requests=cap)
                    fam.solvers.append(s)
                    self.resident += s.info()["footprint_bytes"]
            self.families[name] = fam
        if self.resident > self.budget:
            raise MemoryError(f"resident catalogs and batch workspaces ({self.resident / 1e9:.1f} GB) exceed the budget")
        self.n_lanes = batch_lanes
        self.n_medium = medium_lanes if any(f.route == "medium" for f in self.families.values()) else 0
        self.n_large = large_workers
        self._lock = threading.Condition()
        self._pending: Dict[str, List[Request]] = {"batch": [], "medium": [], "large": []}
        self._reserved = 0.0
        self._done: List[Request] = []
        self._closed = False
        self._t0 = 0.0
        self._threads: List[threading.Thread] = []
        self.peak_reserved = 0.0
        if warm_up:
            self.warm_up()
        self._ring_q: Dict[str, "queue.Queue"] = {}
        if self.ring_blocks > 0:
            for fam in self.families.values():
                if fam.route == "batch":
                    fam.solvers[0].ring_start(capacity=1024, n_blocks=self.ring_blocks, idle_ms=self.ring_idle_ms)
                    self._ring_q[fam.name] = queue.Queue()

    def warm_up(self, max_wave: int = 152) -> None:
        """Before any request arrives, run one wave of every batched family's
        own sectors (its momenta at a few twists) through each of its lanes:
        every lane builds its hop table, and the first run of the catalog
        shape lets the launch autotuner pick the batch's launch shape (its
        trial launches take a few seconds per family).  Served requests then
        wait for neither.  Results of the warm-up are discarded."""
        for fam in self.families.values():
            if fam.route == "large":
                continue
            lat = fam.spec.lattice
            nk = lat.sample_size[0] * lat.sample_size[1]
            n = min(max_wave, fam.solvers[0].max_requests, int(fam.solvers[0].info()["blocks"]))
            twists = [(0.0, 0.0), (0.5, 0.25 if lat.sample_size[1] > 1 else 0.0),
                      (0.25, 0.75 if lat.sample_size[1] > 1 else 0.0), (0.75, 0.5 if lat.sample_size[1] > 1 else 0.0)]
            reqs = [Request(-1 - i, fam.name, i % nk, twists[(i // nk) % len(twists)], 1, 0x5EED0000 + i)
                    for i in range(n)]
            arrays = self._request_arrays(fam, reqs)
            for solver in fam.solvers:
                solver.run(arrays, tol=self.tol)

    # ------------------------------------------------------------ workers
    def _now(self) -> float:
        return time.perf_counter() - self._t0

    def _request_arrays(self, fam: Family, reqs: Sequence[Request]):
        from .batched import SectorRequest

        srs = []
        for r in reqs:
            G = L.build_translation_group(fam.spec.lattice, r.twist)
            irr = L.build_translation_irrep_list(G, fam.spec.lattice)[r.k_index]
            amps = [t for (_, _, t) in fam.spec.bilinear_terms(r.twist)]
            srs.append(SectorRequest(irr, G, amps, r.seed))
        return srs

    def _batch_lane(self, route: str, lane: int):
        pending = self._pending[route]
        while True:
            with self._lock:
                while not pending and not self._closed:
                    self._lock.wait()
                if not pending and self._closed:
                    return
                fam_name = pending[0].family  # oldest request decides the family
                cap = self.families[fam_name].solvers[lane % len(self.families[fam_name].solvers)].max_requests
                take = [r for r in pending if r.family == fam_name][:cap]
                for r in take:
                    pending.remove(r)
            fam = self.families[fam_name]
            t_start = self._now()
            solver = fam.solvers[lane % len(fam.solvers)]
            out = solver.run(self._request_arrays(fam, take), tol=self.tol)
            t_end = self._now()
            with self._lock:
                for i, r in enumerate(take):
                    r.evals = out["evals"][i, : r.nev].copy()
                    r.status = int(out["status"][i])
                    r.dim = int(out["dims"][i])
                    r.delta_polish = float(out["delta_polish"][i])
                    r.t_start, r.t_end, r.route = t_start, t_end, route
                    self._done.append(r)
                self._lock.notify_all()

    def _ring_collector(self, fam_name: str):
        """Collect a family's ring tickets in submission order."""
        fam = self.families[fam_name]
        q = self._ring_q[fam_name]
        while True:
            item = q.get()
            if item is None:
                return
            ticket, r = item
            try:
                ev, st, dim = fam.solvers[0].ring_wait(ticket)
                r.evals, r.status, r.dim = ev[: r.nev].copy(), st, dim
            except A._lib.SEDError as e:
                r.status, r.evals, r.error = e.code, np.full(r.nev, np.nan), str(e)
            t_end = self._now()
            with self._lock:
                r.t_start, r.t_end, r.route = r.arrival, t_end, "ring"
                self._done.append(r)
                self._lock.notify_all()

    def _large_worker(self):
        pending = self._pending["large"]
        while True:
            with self._lock:
                while True:
                    if pending:
                        r = pending[0]
                        need = solver_footprint(self.families[r.family].n_orbits, r.nev)
                        if self._reserved + need <= self.budget - self.resident or self._reserved == 0:
                            pending.pop(0)
                            self._reserved += need
                            self.peak_reserved = max(self.peak_reserved, self._reserved)
                            break
                    elif self._closed:
                        return
                    self._lock.wait()
            fam = self.families[r.family]
            t_start = self._now()
            try:
                G = L.build_translation_group(fam.spec.lattice, r.twist)
                irr = L.build_translation_irrep_list(G, fam.spec.lattice)[r.k_index]
                basis = A.build_symmetry_sector_basis(fam.catalog, irr, group=G)
                if basis.dim == 0:
                    vals, status, delta = np.full(r.nev, np.nan), 0, 0.0
                else:
                    H = A.MatrixFreeHamiltonian(basis, fam.spec.bilinear_terms(r.twist), fam.spec.density_terms,
                                                precision=self.precision)
                    if fam.n_orbits <= self.priority_max_orbits:
                        H.set_priority(True)
                    if self.large_sm_limit > 0:
                        H.set_sm_limit(self.large_sm_limit)
                    vals, _, info = H.solve(r.nev, tol=self.tol, seed=r.seed, krylovdim=self.large_krylovdim,
                                            want_vectors=False)
                    status, delta = 0, info.max_delta_polish
                    del H
                r.evals, r.status, r.dim, r.delta_polish = np.asarray(vals), status, basis.dim, delta
            except A._lib.SEDError as e:  # reported per request, never silently dropped
                r.status, r.evals, r.error = e.code, np.full(r.nev, np.nan), str(e)
            r.t_start, r.t_end, r.route = t_start, self._now(), "large"
            with self._lock:
                self._reserved -= need
                self._done.append(r)
                self._lock.notify_all()

    # --------------------------------------------------------------- API
    def start(self):
        self._t0 = time.perf_counter()
        self._closed = False
        self._threads = [threading.Thread(target=self._batch_lane, args=("batch", i), daemon=True)
                         for i in range(self.n_lanes)]
        self._threads += [threading.Thread(target=self._batch_lane, args=("medium", i), daemon=True)
                          for i in range(self.n_medium)]
        self._threads += [threading.Thread(target=self._large_worker, daemon=True) for _ in range(self.n_large)]
        self._ring_threads = [threading.Thread(target=self._ring_collector, args=(name,), daemon=True)
                              for name in self._ring_q]
        for t in self._threads + self._ring_threads:
            t.start()

    def submit(self, r: Request) -> None:
        fam = self.families[r.family]
        if fam.name in self._ring_q:  # straight into the family's device-resident loop
            r.arrival = self._now()
            req = self._request_arrays(fam, [r])[0]
            while True:
                try:
                    ticket = fam.solvers[0].ring_submit(req)
                    break
                except A._lib.SEDError as e:
                    if e.code == A._lib.SED_ERR_LIMIT:
                        # every slot awaits collection: the collector, which
                        # takes the tickets in order, frees the oldest soon
                        time.sleep(1e-4)
                        continue
                    with self._lock:  # refused: reported on the request, like the other routes
                        r.status, r.evals, r.error = e.code, np.full(r.nev, np.nan), str(e)
                        r.t_start, r.t_end, r.route = r.arrival, self._now(), "ring"
                        self._done.append(r)
                        self._lock.notify_all()
                    return
            self._ring_q[fam.name].put((ticket, r))
            return
        with self._lock:
            r.arrival = self._now()
            self._pending[fam.route].append(r)
            self._lock.notify_all()

    def close(self) -> List[Request]:
        with self._lock:
            self._closed = True
            self._lock.notify_all()
        for q in self._ring_q.values():
            q.put(None)
        for t in self._threads + getattr(self, "_ring_threads", []):
            t.join()
        for name in self._ring_q:
            self.families[name].solvers[0].ring_stop()
        self._ring_q = {}
        return list(self._done)

    def serve(self, requests: Sequence[Request], time_scale: float = 1.0) -> List[Request]:
        """Replay a request stream: each request is submitted at its arrival
        time (scaled), and the call returns when every request is answered."""
        self.start()
        for r in sorted(requests, key=lambda q: q.arrival):
            delay = r.arrival * time_scale - self._now()
            if delay > 0:
                time.sleep(delay)
            self.submit(r)
        return self.close()


def latency_stats(done: Sequence[Request]) -> dict:
    lat = np.array([r.t_end - r.arrival for r in done])
    span = max(r.t_end for r in done) - min(r.arrival for r in done)
    return {"n": len(done), "solves_per_s": len(done) / span if span > 0 else float("nan"),
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "span_s": span}


class NativeSectorServer:
    """The same continuous batching, run by the library's native server
    (``sed_server_*`` in the C ABI): host threads in C++ drive the batch lanes
    and the device-wide solves, and Python only submits and collects.  Model
    families come from lattice specs as for :class:`SectorServer`; requests are
    the same :class:`Request` objects."""

    def __init__(self, families: Dict[str, L.ModelSpec], budget_bytes: float = 160e9, batch_lanes: int = 2,
                 large_workers: int = 3, small_max_orbits: int = SMALL_MAX_ORBITS, precision: str = "mixed",
                 tol: float = 1e-10, nev_max: int = 1):
        import ctypes as C

        self._C = C
        lib = A._lib.load()
        prec = {"fp64": A._lib.PREC_FP64, "mixed": A._lib.PREC_MIXED}[precision]
        h = C.c_void_p()
        A._lib.check(lib.sed_server_create(float(budget_bytes), int(batch_lanes), int(large_workers),
                                           int(small_max_orbits), prec, float(tol), C.byref(h)))
        self._h = h
        self.specs = dict(families)
        self.catalogs: Dict[str, A.Symmetry_Orbit_Catalog] = {}
        self.family_id: Dict[str, int] = {}
        for name, spec in families.items():
            G = L.build_translation_group(spec.lattice)
            cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                                 particle_statistics=statistics_from_name(spec.statistics))
            terms = spec.bilinear_terms()
            bij = np.ascontiguousarray([[i - 1, j - 1] for (i, j, _) in terms], dtype=np.int32)
            bt = np.ascontiguousarray([complex(t) for (_, _, t) in terms], dtype=np.complex128)
            dij = np.ascontiguousarray([[int(i) - 1, int(j) - 1] for (i, j, _) in spec.density_terms], dtype=np.int32)
            dv = np.ascontiguousarray([complex(v) for (_, _, v) in spec.density_terms], dtype=np.complex128)
            fid = C.c_int32(-1)
            A._lib.check(lib.sed_server_add_family(self._h, cat.handle, len(terms), bij.ctypes.data, bt.ctypes.data,
                                                   len(dv), dij.ctypes.data if len(dv) else None,
                                                   dv.ctypes.data if len(dv) else None, int(nev_max), C.byref(fid)))
            self.catalogs[name] = cat
            self.family_id[name] = fid.value
        self._t0 = time.perf_counter()

    def _now(self) -> float:
        return time.perf_counter() - self._t0

    def submit(self, r: Request) -> int:
        spec = self.specs[r.family]
        G = L.build_translation_group(spec.lattice, r.twist)
        irr = L.build_translation_irrep_list(G, spec.lattice)[r.k_index]
        chi = np.ascontiguousarray(irr.array(), dtype=np.complex128)
        ph = np.ascontiguousarray(G.phases(), dtype=np.complex128)
        amp = np.ascontiguousarray([t for (_, _, t) in spec.bilinear_terms(r.twist)], dtype=np.complex128)
        t = self._C.c_int64(0)
        A._lib.check(A._lib.load().sed_server_submit(self._h, self.family_id[r.family], chi.ctypes.data,
                                                     ph.ctypes.data, amp.ctypes.data, int(r.seed), int(r.nev),
                                                     self._C.byref(t)))
        r.arrival = self._now()
        return t.value

    def wait(self, ticket: int, r: Request, timeout_ms: int = 600_000) -> Request:
        ev = np.zeros(r.nev, dtype=np.float64)
        st, dim = self._C.c_int32(0), self._C.c_int64(0)
        rc = A._lib.load().sed_server_wait(self._h, int(ticket), int(timeout_ms), ev.ctypes.data,
                                           self._C.byref(st), self._C.byref(dim))
        A._lib.check(rc)
        r.evals, r.status, r.dim, r.t_end = ev, st.value, dim.value, self._now()
        if st.value != 0:
            r.error = A._lib.load().sed_last_error().decode()
        r.route = "native"
        return r

    def serve(self, requests: Sequence[Request], time_scale: float = 1.0) -> List[Request]:
        """Replay a stream: each request submitted at its arrival time (scaled);
        a collector thread takes the requests as they finish (sed_server_next,
        completion order) and stamps each when it is handed over."""
        self._t0 = time.perf_counter()
        by_ticket: Dict[int, Request] = {}
        done: List[Request] = []
        lock = threading.Lock()
        total = len(requests)
        nev_max = max((r.nev for r in requests), default=1)

        def collect():
            C = self._C
            ev = np.zeros(nev_max, dtype=np.float64)
            t, st, dim = C.c_int64(0), C.c_int32(0), C.c_int64(0)
            lib = A._lib.load()
            while len(done) < total:
                rc = lib.sed_server_next(self._h, 200, C.byref(t), ev.ctypes.data, C.byref(st), C.byref(dim))
                if rc == A._lib.SED_ERR_TIMEOUT:
                    continue
                A._lib.check(rc)
                with lock:
                    r = by_ticket.pop(t.value)
                r.evals, r.status, r.dim, r.t_end = ev[: r.nev].copy(), st.value, dim.value, self._now()
                if st.value != 0:
                    r.error = lib.sed_last_error().decode()
                r.route = "native"
                done.append(r)

        th = threading.Thread(target=collect, daemon=True)
        th.start()
        for r in sorted(requests, key=lambda x: x.arrival):
            arr = r.arrival * time_scale
            delay = arr - self._now()
            if delay > 0:
                time.sleep(delay)
            with lock:
                tk = self.submit(r)  # stamps the arrival
                by_ticket[tk] = r
        th.join()
        return done

    def stats(self) -> dict:
        C = self._C
        nd, npend, peak, res = C.c_int64(0), C.c_int64(0), C.c_double(0), C.c_double(0)
        A._lib.check(A._lib.load().sed_server_stats(self._h, C.byref(nd), C.byref(npend), C.byref(peak),
                                                    C.byref(res)))
        return {"done": nd.value, "pending": npend.value, "peak_reserved_bytes": peak.value,
                "resident_bytes": res.value}

    def close(self) -> None:
        if self._h:
            A._lib.load().sed_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
