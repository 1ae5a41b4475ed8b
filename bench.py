"""Benchmark: sector solves/s for the flux-scan batch, versus the plain FP64 drop-in.

Workload (default "flux_scan_haldane3x4"): hard-core bosons on a 3x4 Haldane
honeycomb (24 sites, t=1, t'=0.6 e^{+-i0.4pi}, t''=-0.58), Np=6; every one of
the 12 momentum sectors at each of an 8x8 grid of flux twists
(theta/2pi in {0, 1/8, ..., 7/8}^2): 768 sector solves of dimension ~1.1e4,
lowest 4 eigenvalues each.  One step = the whole 768-solve batch.
  value : solves/s of the batched mixed-precision path (complex64 matvec, FP64
          Lanczos + polish) with inputs resident in HBM, CUDA events;
  e2e   : the same through the C ABI with host buffers (H2D of the request
          parameters and D2H of the results inside the timed region);
and beside them the plain FP64 drop-in (sed_solve on one sector at a time, the
reference's call pattern), the FP64 batched path, |dE|/|E| of the mixed results
against FP64, p50/p99 request latency, the kernel roofline and clocks.

``--impl reference`` times the CPU restatement of the reference's matrix-free
path (projection table + threaded _apply_table! + Lanczos, oracle/) on the host
cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from typing import Optional

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sector solves/s (flux-scan batch), mixed precision at |dE|/|E|<=1e-9"
UNIT = "solves/s"
WORKLOAD = "flux_scan_haldane3x4"


def workload_requests(grid: int = 8):
    from realspace_exactdiagonalization_gb300 import lattice as L
    from realspace_exactdiagonalization_gb300.batched import flux_scan_requests

    spec = L.haldane_honeycomb(3, 4)
    twists = [(a / grid, b / grid) for a in range(grid) for b in range(grid)]
    return spec, twists, flux_scan_requests(spec, twists)


def config(n_req, extra=None, grid=8):
    c = {"workload": WORKLOAD, "model": "haldane_honeycomb_3x4_hardcore_bosons", "n_site": 24, "n_particles": 6,
         "sectors_per_step": n_req, "momenta": 12, "twist_grid": f"{grid}x{grid}", "nev": 4, "tol": 1e-10,
         "l2": "flushed between timed steps (256 MiB write)"}
    if extra:
        c.update(extra)
    return c


def lanczos_bytes(nmv: int, dim: int, m: int = 24, keep: int = 8, n_polish: int = 6, elem: int = 8) -> float:
    """Algorithmic bytes of the Lanczos vector work of one batched solve with
    ``nmv`` matvecs on a sector of dimension ``dim``, ``elem`` bytes per vector
    element (8: the mixed kernel's complex64 basis; 16: the FP64 kernel's
    double-float basis): each iteration streams three vectors (the matvec's
    output, and the normalisation's read of it and write of the new basis
    vector) and reads the k basis vectors the reorthogonalisation's dot
    products sweep; each restart rotates m vectors into ``keep``.  k follows the
    thick-restart schedule: 1..m in the first cycle, keep+1..m after each
    restart.  The n_polish FP64-class matvecs of the final check are not
    iterations."""
    steps = max(nmv - n_polish, 0)
    first = min(steps, m)
    ksum = first * (first + 1) // 2
    rest = steps - first
    cyc = m - keep
    full, part = divmod(rest, cyc)
    ksum += full * sum(range(keep + 1, m + 1)) + sum(range(keep + 1, keep + 1 + part))
    # every cycle ends in a rotation, a partial one (first or last) included
    restarts = (1 if steps > 0 else 0) + full + (1 if part else 0)
    return float((3 * steps + ksum + restarts * (m + keep)) * dim * elem)


def profiled_traffic_per_sector():
    """DRAM bytes (read + write) per sector of one k_batch launch, read from the
    committed ncu capture summary of the 192-sector case (the capture scales
    with the sector count)."""
    path = os.path.join(ROOT, "profiles", "k_batch_flux_scan_haldane3x4.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_sector:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


# ------------------------------------------------------------------ clocks
class ClockSampler:
    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        j = json.load(open(p))
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------ reference arm
def run_reference(args, rank):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    if rank != 0:
        return
    O.build()
    spec, twists, reqs = workload_requests()
    cores = O.max_threads()
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    st = statistics_from_name(spec.statistics).code
    G0 = reqs[0].group
    cat = O.Catalog(G0.perm0(), G0.phases(), 0, st, spec.n_filled)
    per_step = max(1, args.ref_sample)
    # each step: a bounded sample of the batch, spread over twists and momenta
    order = [(i * 97) % len(reqs) for i in range(len(reqs))]
    pos = 0

    def step():
        nonlocal pos
        n = 0
        for _ in range(per_step):
            b = order[pos % len(order)]
            pos += 1
            r = reqs[b]
            cat.update_phases(r.group.phases())
            sec = O.Sector(cat, r.irrep.array())
            if sec.dim == 0:
                continue
            terms = [(i - 1, j - 1, t) for (i, j), t in zip(
                [(i, j) for (i, j, _) in spec.bilinear_terms()], r.amplitudes)]
            op = O.Op(sec, terms, [(i - 1, j - 1, v) for (i, j, v) in spec.density_terms])
            res = op.solve(4, tol=1e-10, maxiter=300, krylovdim=30, seed=r.seed)
            assert res["status"] == 0
            n += 1
        return n

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    done = 0
    for _ in range(args.steps):
        done += step()
    dt = time.perf_counter() - t0
    v = done / dt
    sample = f"{per_step} of the {len(reqs)} sector solves per step (spread over twists and momenta); " \
             f"projection-table build + threaded table apply + thick-restart Lanczos, catalog excluded"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (generated lattice model)", "config": config(len(reqs), {"sample": sample}),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(n_solves=4):
    """CPU restatement of the reference on the host cores, bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    spec, twists, reqs = workload_requests()
    G0 = reqs[0].group
    cat = O.Catalog(G0.perm0(), G0.phases(), 0, 0, spec.n_filled)
    pairs = [(i, j) for (i, j, _) in spec.bilinear_terms()]
    t0 = time.perf_counter()
    done = 0
    evals = {}
    for b in [(i * 97) % len(reqs) for i in range(n_solves)]:
        r = reqs[b]
        cat.update_phases(r.group.phases())
        sec = O.Sector(cat, r.irrep.array())
        op = O.Op(sec, [(i - 1, j - 1, t) for (i, j), t in zip(pairs, r.amplitudes)], [])
        res = op.solve(4, tol=1e-10, maxiter=300, krylovdim=30, seed=r.seed)
        evals[b] = res["evals"]
        done += 1
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
            "sample": f"{n_solves} of the {len(reqs)} sector solves (CPU restatement of the reference's matrix-free "
                      f"path: projection table + threaded table apply + Lanczos)"}, evals


# ------------------------------------------------------------------ our arm
def run_ours(args, rank, world):
    import torch

    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300.batched import BatchedSectorSolver

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    spec, twists, reqs = workload_requests(args.twist_grid)
    n = len(reqs)
    G0 = reqs[0].group
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G0,
                                         particle_statistics=A.Bosonic())
    pairs = [(i, j) for (i, j, _) in spec.bilinear_terms()]
    solver = BatchedSectorSolver(cat, pairs, spec.density_terms, precision="mixed", nev=4, max_requests=n)
    stream = torch.cuda.current_stream()
    solver.set_stream(stream.cuda_stream)
    chi, ph, amp, seeds = solver.pack(reqs)
    # device-resident inputs and outputs
    d = {k: torch.from_numpy(v.view(np.float64) if v.dtype == np.complex128 else v.view(np.int64)).cuda()
         for k, v in (("chi", chi), ("ph", ph), ("amp", amp), ("seeds", seeds))}
    out = {"ev": torch.zeros(n * 4, dtype=torch.float64, device="cuda"),
           "st": torch.zeros(n, dtype=torch.int32, device="cuda"),
           "dims": torch.zeros(n, dtype=torch.int64, device="cuda"),
           "delta": torch.zeros(n, dtype=torch.float64, device="cuda"),
           "nmv": torch.zeros(n, dtype=torch.int32, device="cuda")}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        solver.run_device(n, d["chi"].data_ptr(), d["ph"].data_ptr(), d["amp"].data_ptr(), d["seeds"].data_ptr(),
                          out["ev"].data_ptr(), out["st"].data_ptr(), out["dims"].data_ptr(),
                          out["delta"].data_ptr(), out["nmv"].data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(dev) as clk:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            times.append((e0, e1))
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in times]
    tot_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([tot_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot_ms = float(t.item())
    value = world * n * args.steps / (tot_ms / 1e3)
    st = out["st"].cpu().numpy()
    ev_mixed = out["ev"].cpu().numpy().reshape(n, 4)
    dims = out["dims"].cpu().numpy()
    nmv = out["nmv"].cpu().numpy()
    stats = solver.last_stats()
    lat_ms = (stats["t_end_ns"] - stats["t_start_ns"].min()) / 1e6
    if rank != 0:
        return
    assert (st == 0).all(), "unconverged requests in the batch"

    # --- roofline of the batch kernel: algorithmic bytes of its matvecs and
    # of its Lanczos vector work (per H|psi>: D*(8+4+2s) + hops*(4+1+4+s); per
    # Lanczos iteration: (3+k)*D*8; per restart: (m+keep)*D*8)
    s = 8  # complex64 matvec input
    b_mv = dims * (8 + 4 + 2 * s) + stats["hops"] * (4 + 1 + 4 + s)
    bytes_mv = float((nmv * b_mv).sum())
    # the mixed kernel keeps nev + 2 = 8 Ritz vectors (nev = 4 requested + 2 spare)
    bytes_lz = float(sum(lanczos_bytes(int(k), int(d), keep=8, elem=8) for k, d in zip(nmv, dims)))
    bytes_launch = bytes_mv + bytes_lz
    t_launch = tot_ms / args.steps / 1e3
    achieved = bytes_launch / t_launch / 1e9
    peak, peak_kind = measured_peak()

    # --- end to end through the C ABI with host buffers
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = solver.run_packed(chi, ph, amp, seeds)
    e2e_s = (time.perf_counter() - t0) / args.steps
    h2d = chi.nbytes + ph.nbytes + amp.nbytes + seeds.nbytes
    d2h = n * (4 * 8 + 4 + 8 + 8 + 4)

    # --- FP64 batched path and |dE|/|E| of the mixed results
    solver64 = BatchedSectorSolver(cat, pairs, spec.density_terms, precision="fp64", nev=4, max_requests=n)
    solver64.run_packed(chi, ph, amp, seeds)  # first run of this shape: the launch autotuner's sweep
    t0 = time.perf_counter()
    r64 = solver64.run_packed(chi, ph, amp, seeds)
    fp64_batch_s = time.perf_counter() - t0
    shape64 = solver64.shape()
    ev64 = r64["evals"]
    rel = np.abs(ev_mixed - ev64) / np.maximum(np.abs(ev64), 1e-300)
    max_rel = float(np.nanmax(rel))

    # --- plain FP64 drop-in: one sector at a time through sed_solve (sample)
    n_plain = args.plain_sample
    idx = [(i * 97) % n for i in range(n_plain)]
    t0 = time.perf_counter()
    plain_ev, plain_svc = {}, []
    for b in idx:
        t1 = time.perf_counter()
        rq = reqs[b]
        A.update_orbit_stabilizer_phases_(cat, rq.group, A.Bosonic())
        basis = A.build_symmetry_sector_basis(cat, rq.irrep)
        H = A.MatrixFreeHamiltonian(basis, [(i, j, t) for (i, j), t in zip(pairs, rq.amplitudes)],
                                    spec.density_terms)
        vals, _, info = H.solve(4, tol=1e-10, seed=rq.seed, want_vectors=False)
        plain_ev[b] = vals
        plain_svc.append(time.perf_counter() - t1)
    plain = None
    if n_plain:
        plain_s = (time.perf_counter() - t0) / n_plain
        svc = np.array(plain_svc)
        max_rel_plain = max(float(np.max(np.abs(ev_mixed[b] - plain_ev[b]) / np.abs(plain_ev[b]))) for b in idx)
        # the whole batch arrives at once; one solve at a time, request i waits
        # for the i solves before it: latencies modelled from the sample's
        # measured service times (the served stream below measures both arms)
        q = np.cumsum(np.resize(svc, n))
        plain = {"solves_per_s": 1.0 / plain_s, "sample": n_plain,
                 "service_ms_p50": float(np.percentile(svc, 50) * 1e3),
                 "service_ms_p99": float(np.percentile(svc, 99) * 1e3),
                 "queue_p50_ms_modelled": float(np.percentile(q, 50) * 1e3),
                 "queue_p99_ms_modelled": float(np.percentile(q, 99) * 1e3),
                 "max_rel_dE_mixed_vs_plain": max_rel_plain}

    cpu = None
    if not args.no_cpu:
        cpu, cpu_ev = cpu_baseline_sample(args.cpu_sample)
        cpu["max_rel_dE_vs_gpu_fp64"] = max(float(np.max(np.abs(cpu_ev[b] - ev64[b]) / np.abs(ev64[b])))
                                           for b in cpu_ev)

    clocks = clk.summary()
    extras = {}
    if not args.no_extras and world == 1:
        # the other configurations, measured after the timed region: the large
        # single-sector kernels and solves (configs 2 and 3) and a short served
        # stream (config 5) with both arms' latencies measured
        del solver64
        torch.cuda.empty_cache()
        kernels = {}
        for cfg in (config2_spec, config3_spec):
            spec2, sec2, name2 = cfg()
            kernels[name2] = large_sector_report(spec2, sec2, name2, steps=5, nev=3 if cfg is config2_spec else 1,
                                                 krylovdim=30)
            torch.cuda.empty_cache()
        extras["kernels"] = kernels
        extras["served"] = served_report(args.extras_served_n, 50.0, args.large_workers)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 matvec / f64 Lanczos", "data": "synthetic (generated lattice model, seeded start vectors)",
        "config": config(n, {"parallelism": f"replicas x{world}" if world > 1 else "single GPU"}, args.twist_grid),
        "e2e": {"value": n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (lambda t: t * n if t else None)(profiled_traffic_per_sector()),
                     "traffic_source": "from the committed ncu profile (profiles/k_batch_flux_scan_haldane3x4.md): "
                                       "dram__bytes_read.sum + dram__bytes_write.sum of one 192-sector k_batch launch, "
                                       "scaled by sectors; not measured in this run",
                     "peak_kind": peak_kind, "kernel": "k_batch (persistent batched Lanczos)",
                     "bytes_per_launch": bytes_launch, "matvec_bytes_per_launch": bytes_mv,
                     "lanczos_bytes_per_launch": bytes_lz, "frac_matvec_bytes_only": bytes_mv / t_launch / 1e9 / peak,
                     # the DRAM side: the profiled traffic over this run's launch time.  The
                     # algorithmic bytes above include the gathers that shared memory and L2
                     # serve, so `frac` can pass 1 while DRAM stays far below its peak
                     "traffic_gbs": (lambda t: t * n / t_launch / 1e9 if t else None)(profiled_traffic_per_sector()),
                     "traffic_frac": (lambda t: t * n / t_launch / 1e9 / peak if t else None)(
                         profiled_traffic_per_sector()),
                     "note": "algorithmic bytes of one launch: every matvec D*(8+4+2s)+hops*(4+1+4+s) (s=8), plus "
                             "every Lanczos iteration's (3+k)*D*8 (three complex64 vector streams and the "
                             "reorthogonalisation's read of the k basis vectors) and every restart's "
                             "(m+keep)*D*8 rotation, k following the thick-restart schedule m=24, keep=8"},
        "cpu_baseline": cpu,
        # one k_batch launch per step, plus the FP64 re-solve launch when a
        # request's polish missed its target (inputs are identical every step)
        "gpu_launches": args.steps * (1 + (stats["fp64_fallbacks"] > 0)),
        "fp64_fallbacks_per_step": stats["fp64_fallbacks"],
        "launch_shape": solver.shape(), "site_gauge": stats["site_gauge"],
        "clocks": clocks,
        "plain_fp64_dropin": plain,
        "fp64_batched": {"solves_per_s": n / fp64_batch_s, "launch_shape": shape64},
        "speedup_vs_plain_fp64": value / plain["solves_per_s"] if plain else None,
        "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99))},
        "max_rel_dE_mixed_vs_fp64": max_rel,
        "dims": {"min": int(dims.min()), "max": int(dims.max())},
        "matvecs_per_solve": float(nmv.mean()),
        "wall_s_timed": t_wall,
        **extras,
    }
    print(json.dumps(line), flush=True)


def large_sector_report(spec, sector: int, name: str, steps: int, nev: int, krylovdim: int,
                        precisions=("fp64", "mixed"), solve: bool = True):
    """One large sector: the device catalog and sector builds, the H|psi>
    kernels -- the matrix-free gather and the stored hop table -- in FP64 and
    complex64 (CUDA-event medians over ``steps`` launches, L2 flushed between
    them; GB/s of the algorithmic bytes D*(8+4+2s) + hops*(4+1+4+s) against the
    measured HBM peak), and the FP64 and mixed-precision solves."""
    import ctypes as C

    import torch

    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300 import _lib
    from realspace_exactdiagonalization_gb300 import lattice as L
    from realspace_exactdiagonalization_gb300.groups import statistics_from_name

    G = L.build_translation_group(spec.lattice)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cat = A.build_symmetry_orbit_catalog(n_filled=spec.n_filled, species=spec.species, symmetry_group=G,
                                         particle_statistics=statistics_from_name(spec.statistics))
    t_cat = time.perf_counter() - t0
    irr = L.build_translation_irrep_list(G, spec.lattice)[sector]
    t0 = time.perf_counter()
    basis = A.build_symmetry_sector_basis(cat, irr)
    t_sec = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    res = {}
    peak, peak_kind = measured_peak()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for prec in precisions:
        H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms(), spec.density_terms, precision=prec)
        info = H.info()
        _lib.check(_lib.load().sed_op_set_stream(H.handle, C.c_void_p(stream.cuda_stream)))
        n_orb = info["n_orbits"]
        s = 16 if prec == "fp64" else 8
        xs = torch.randn(n_orb * 2, dtype=torch.float64 if prec == "fp64" else torch.float32, device="cuda")
        y = torch.empty(n_orb * 2, dtype=torch.float64, device="cuda")

        def time_matvec():
            for _ in range(2):
                _lib.check(_lib.load().sed_op_apply_orbit(H.handle, C.c_void_p(xs.data_ptr()),
                                                          C.c_void_p(y.data_ptr())))
            torch.cuda.synchronize()
            ms = []
            for _ in range(steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                _lib.check(_lib.load().sed_op_apply_orbit(H.handle, C.c_void_p(xs.data_ptr()),
                                                          C.c_void_p(y.data_ptr())))
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            return statistics.median(ms) / 1e3

        # the matrix-free gather (every hop re-derived from the representative)
        H.set_hop_table(H.HOP_TABLE_OFF)
        t_fly = time_matvec()
        b_alg = info["dim"] * (8 + 4 + 2 * s) + info["hops"] * (4 + 1 + 4 + s)
        r = {"k_apply": {"matvec_ms": 1e3 * t_fly, "bytes_alg": b_alg, "achieved_gbs": b_alg / t_fly / 1e9,
                         "frac": b_alg / t_fly / 1e9 / peak,
                         "shape_threads_per_row_block": list(H.apply_shape(prec == "mixed"))},
             "hops": info["hops"]}
        # the stored hop table (8 bytes per hop, streamed)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            H.set_hop_table(H.HOP_TABLE_NOW)
            t_build = time.perf_counter() - t0
            tinfo = H.hop_table_info()
            t_tab = time_matvec()
            # bytes the table matvec must move: records, x gathers, row reads and writes
            b_tab = tinfo["records"] * 8 + info["hops"] * s + info["dim"] * (16 + 4 + 1 + s + 16)
            r["k_apply_tab"] = {"matvec_ms": 1e3 * t_tab, "build_s": t_build, "table_gb": tinfo["bytes"] / 1e9,
                                "records": tinfo["records"], "padding": tinfo["records"] / max(info["hops"], 1) - 1,
                                "achieved_gbs": b_alg / t_tab / 1e9, "frac": b_alg / t_tab / 1e9 / peak,
                                "table_bytes": b_tab, "achieved_gbs_table_bytes": b_tab / t_tab / 1e9,
                                "frac_table_bytes": b_tab / t_tab / 1e9 / peak, "speedup_vs_gather": t_fly / t_tab}
        except _lib.SEDError as e:
            r["k_apply_tab"] = {"unavailable": str(e)}
        if solve:
            t0 = time.perf_counter()
            vals, _, sinfo = H.solve(nev, tol=1e-10, krylovdim=krylovdim, want_vectors=False)
            r.update({"solve_s": time.perf_counter() - t0, "evals": [float(v) for v in vals],
                      "nev": nev, "krylovdim": krylovdim, "restarts": sinfo.n_restarts,
                      "matvecs": sinfo.n_matvec, "matvecs_fp64": sinfo.n_matvec_fp64,
                      "max_residual": sinfo.max_residual, "delta_polish": sinfo.max_delta_polish,
                      "solve_uses_hop_table": H.hop_table_info()["built"]})
        res[prec] = r
        del H, xs, y
        torch.cuda.synchronize()
    if "evals" in res.get("fp64", {}) and "evals" in res.get("mixed", {}):
        e64, em = np.array(res["fp64"]["evals"]), np.array(res["mixed"]["evals"])
        res["max_rel_dE_mixed_vs_fp64"] = float(np.max(np.abs(em - e64) / np.abs(e64)))
        res["mixed_speedup_vs_fp64_solve"] = res["fp64"]["solve_s"] / res["mixed"]["solve_s"]
    return {"workload": name, "n_states": cat.n_states, "n_orbits": cat.n_orbits, "dim": basis.dim,
            "catalog_build_s": t_cat, "sector_build_s": t_sec, "peak_gbs": peak, "peak_kind": peak_kind, **res}


def config2_spec():
    """Checkerboard 4x6 spinless fermions (48 sites; NN |t| = 1 with
    e^{+-i pi/4}, NNN +-0.3, NNNN -0.2, V = 1), 8 particles, momentum (0, 0)."""
    from realspace_exactdiagonalization_gb300 import lattice as L

    return L.checkerboard(4, 6, n_filled=8), 0, "checkerboard4x6_np8_k(0,0)"


def config3_spec():
    """Hubbard 4x4 (t = 1, U = 8) as 32 modes, up spin at bit i and down spin
    at bit i + 16, N_up = N_down = 7, momentum (pi, 0) = label (2, 0)."""
    from realspace_exactdiagonalization_gb300 import lattice as L

    return L.hubbard_square(4, 4, n_up=7, n_dn=7), 2 * 4 + 0, "hubbard4x4_7u7d_k(pi,0)"


def run_large(args):
    import torch

    from realspace_exactdiagonalization_gb300 import lattice as L

    torch.cuda.set_device(0)
    L1, L2, npart = args.large_shape
    if args.large_model == "hubbard":
        spec, sector, name = config3_spec()
        if (L1, L2, npart) != (4, 6, 8):  # a shape other than the default: N_up = N_down = npart / 2
            spec = L.hubbard_square(L1, L2, n_up=npart // 2, n_dn=npart - npart // 2)
            sector = (L1 // 2) * L2
            name = f"hubbard{L1}x{L2}_{npart // 2}u{npart - npart // 2}d_k(pi,0)"
    else:
        spec = L.checkerboard(L1, L2, n_filled=npart)
        sector, name = 0, f"checkerboard{L1}x{L2}_np{npart}_k(0,0)"
    precs = ("fp64", "mixed") if args.large_precision == "both" else (args.large_precision,)
    line = large_sector_report(spec, sector, name, args.steps, args.large_nev, args.krylovdim, precs,
                               solve=not args.no_solve)
    print(json.dumps(line), flush=True)


def fifo_latencies(arrivals, service):
    """One server answering requests in arrival order: request i starts when
    it has arrived and request i-1 is done."""
    t, out = 0.0, []
    for a, sv in zip(arrivals, service):
        t = max(t, a) + sv
        out.append(t - a)
    return np.asarray(out), t


def served_report(n_req: int, rate: float, large_workers: int = 3, plain_all: bool = True, plain_per_family: int = 2,
                  seed: int = 20261203, partition: Optional[dict] = None, native: bool = False):
    """Config 5: a seeded Poisson stream of ground-state requests drawn
    uniformly from rings N in {20, 24, 28}, checkerboard 3x4 / 4x4 and Hubbard
    3x4 / 4x4 with N_up = N_down in {5, 6} (two-species blocks), random momentum
    and twist, nev = 1; served with continuous batching under a 160 GB device
    budget.  Against it, the plain FP64 drop-in answers the same requests one
    at a time: every request's FP64 solve is timed (plain_all), and the same
    arrival times are replayed through a first-in-first-out single server with
    those service times; or, for long streams, per-family means of a sample of
    plain_per_family requests stand in for the service times (stated in the
    result).  native: the same stream through the library's native server
    (sed_server_*, C++ host threads) instead of the Python scheduler."""
    import realspace_exactdiagonalization_gb300.api as A
    from realspace_exactdiagonalization_gb300 import lattice as L
    from realspace_exactdiagonalization_gb300.serving import (SMALL_MAX_ORBITS, NativeSectorServer, SectorServer,
                                                              config5_families, latency_stats, random_requests)

    fams = config5_families()
    t0 = time.perf_counter()
    if native:
        srv = NativeSectorServer(fams, budget_bytes=160e9, batch_lanes=2, large_workers=large_workers)
        fam_of = {n: (srv.specs[n], srv.catalogs[n],
                      "batch" if srv.catalogs[n].n_orbits <= SMALL_MAX_ORBITS else "large") for n in fams}
    else:
        srv = SectorServer(fams, budget_bytes=160e9, batch_lanes=2, large_workers=large_workers, **(partition or {}))
        fam_of = {n: (f.spec, f.catalog, f.route) for n, f in srv.families.items()}
    t_setup = time.perf_counter() - t0
    reqs = random_requests(fams, n_req, rate=rate, seed=seed)
    done = sorted(srv.serve(reqs), key=lambda r: r.rid)
    st = latency_stats(done)
    errors = {r.rid: f"{r.family}: {r.error or r.status}" for r in done if r.status != 0}

    def plain_solve(r):
        spec, catalog, _ = fam_of[r.family]
        G = L.build_translation_group(spec.lattice, r.twist)
        irr = L.build_translation_irrep_list(G, spec.lattice)[r.k_index]
        t1 = time.perf_counter()
        basis = A.build_symmetry_sector_basis(catalog, irr, group=G)
        e = float("nan")
        if basis.dim:
            H = A.MatrixFreeHamiltonian(basis, spec.bilinear_terms(r.twist), spec.density_terms)
            vals, _, _ = H.solve(r.nev, tol=1e-10, seed=r.seed, want_vectors=False)
            e = float(vals[0])
            del H
        return time.perf_counter() - t1, e

    plain_ev, service = {}, {}
    if plain_all:
        for r in done:
            service[r.rid], plain_ev[r.rid] = plain_solve(r)
        kind = "measured: every request's FP64 solve timed, FIFO replay of the stream's arrival times"
    else:
        per = {}
        for name in sorted(fams):
            for r in [q for q in done if q.family == name][:plain_per_family]:
                sv, plain_ev[r.rid] = plain_solve(r)
                per.setdefault(name, []).append(sv)
        for r in done:
            service[r.rid] = float(np.mean(per[r.family]))
        kind = (f"modelled: FIFO replay with per-family mean FP64 service times of {plain_per_family} measured "
                f"requests per family")
    arr = np.array([r.arrival for r in done])
    sv = np.array([service[r.rid] for r in done])
    order = np.argsort(arr, kind="stable")
    lat, t_last = fifo_latencies(arr[order], sv[order])
    plain = {"solves_per_s": len(done) / (t_last - arr.min()), "p50_ms": float(np.percentile(lat, 50) * 1e3),
             "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_service_s": float(sv.mean()), "latencies": kind}
    rel = [abs(done[i].evals[0] - e) / abs(e) for i, e in plain_ev.items() if np.isfinite(e)]
    per_fam = {}
    for name in sorted(fams):
        mine = [r for r in done if r.family == name]
        _, catalog, route = fam_of[name]
        per_fam[name] = {"route": route, "n_orbits": catalog.n_orbits, "served": len(mine),
                         "plain_fp64_service_s": float(np.mean([service[r.rid] for r in mine])) if mine else None,
                         "mean_latency_s": float(np.mean([r.t_end - r.arrival for r in mine])) if mine else None}
        if not native:  # the Python scheduler stamps when a request's solve starts
            per_fam[name]["mean_service_s"] = float(np.mean([r.t_end - r.t_start for r in mine])) if mine else None
            per_fam[name]["mean_wait_s"] = float(np.mean([r.t_start - r.arrival for r in mine])) if mine else None
    return {"workload": "served_config5", "requests": len(done), "rate_per_s": rate, "seed": seed,
            "served": st, "plain_fp64_one_at_a_time": plain,
            "speedup_solves_per_s": st["solves_per_s"] / plain["solves_per_s"],
            "p50_ratio_plain_over_served": plain["p50_ms"] / st["p50_ms"],
            "p99_ratio_plain_over_served": plain["p99_ms"] / st["p99_ms"],
            "unconverged": [r.rid for r in done if r.status != 0], "errors": errors, "setup_s": t_setup,
            "server": "native" if native else "python",
            "peak_reserved_gb": (srv.stats()["peak_reserved_bytes"] if native else srv.peak_reserved) / 1e9,
            "resident_gb": (srv.stats()["resident_bytes"] if native else srv.resident) / 1e9,
            "max_rel_dE_vs_plain_fp64": float(max(rel)) if rel else None, "families": per_fam}


def run_served(args):
    import torch

    torch.cuda.set_device(0)
    part = {}
    if args.served_medium_orbits is not None:
        part["medium_max_orbits"] = args.served_medium_orbits
    if args.served_medium_batch is not None:
        part["medium_max_batch"] = args.served_medium_batch
    if args.served_large_sms:
        part["large_sm_limit"] = args.served_large_sms
    if args.served_ring_blocks:
        part["ring_blocks"] = args.served_ring_blocks
        part["ring_idle_ms"] = args.served_ring_idle_ms
    if args.served_large_krylovdim:
        part["large_krylovdim"] = args.served_large_krylovdim
    line = served_report(args.served_n, args.served_rate, args.large_workers, plain_all=not args.plain_sampled,
                         plain_per_family=args.plain_per_family, partition=part, native=args.served_native)
    line["partition"] = part
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-sample", type=int, default=24)
    ap.add_argument("--cpu-sample", type=int, default=6)
    ap.add_argument("--ref-sample", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--twist-grid", type=int, default=8,
                    help="flux-scan batch: twist grid G (12 G^2 sectors per step; 8 = the 768-sector batch)")
    ap.add_argument("--workload", default="flux_scan", choices=["flux_scan", "large", "served"])
    ap.add_argument("--served-n", type=int, default=300)
    ap.add_argument("--served-rate", type=float, default=50.0)
    ap.add_argument("--large-workers", type=int, default=3)
    ap.add_argument("--plain-per-family", type=int, default=2)
    ap.add_argument("--plain-sampled", action="store_true",
                    help="served workload: model the plain FP64 arm from per-family samples instead of timing "
                         "every request (long streams)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the config-2/3 kernel and solve report and the short served stream")
    ap.add_argument("--extras-served-n", type=int, default=200)
    ap.add_argument("--served-medium-orbits", type=int, default=None,
                    help="served: catalogs up to this many orbits take the mid-size batch lane")
    ap.add_argument("--served-medium-batch", type=int, default=None,
                    help="served: requests (so SMs) of one mid-size batch launch")
    ap.add_argument("--served-large-krylovdim", type=int, default=0,
                    help="served: Krylov dimension of the device-wide solves (0: the server's default)")
    ap.add_argument("--served-ring-blocks", type=int, default=0,
                    help="served: batched families run a device-resident request loop on up to this many SMs")
    ap.add_argument("--served-ring-idle-ms", type=int, default=2,
                    help="served: idle time after which a device-resident loop's blocks leave")
    ap.add_argument("--served-native", action="store_true",
                    help="served: use the library's native server (sed_server_*) instead of the Python scheduler")
    ap.add_argument("--served-large-sms", type=int, default=0,
                    help="served: SMs the device-wide solves size their grids for (0: all)")
    ap.add_argument("--large-shape", type=int, nargs=3, default=[4, 6, 8], metavar=("L1", "L2", "NP"))
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--large-nev", type=int, default=3, help="eigenpairs of the large-sector solve")
    ap.add_argument("--krylovdim", type=int, default=30, help="Krylov dimension of the large-sector solve")
    ap.add_argument("--large-model", default="checkerboard", choices=["checkerboard", "hubbard"])
    ap.add_argument("--large-precision", default="both", choices=["both", "fp64", "mixed"],
                    help="which precisions the large-sector workload measures")
    args = ap.parse_args()
    if args.workload == "large":
        run_large(args)
        return
    if args.workload == "served":
        run_served(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
