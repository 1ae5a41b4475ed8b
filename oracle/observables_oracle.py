"""CPU restatement of the reference's flux-torus observables.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the device
path; the product package never imports this module.

Follows, in plain numpy and Python loops (small systems only):
* _position_phase_for_mask and _position_operator_matrix
  (observables/charge_pump.jl:36-91);
* _fock_amplitude_overlap / _subspace_overlap_matrix / _unit_det_link
  (observables/many_body_chern_number.jl:46-80), on dense Fock vectors;
* _tracked_phase_branches / _best_phase_permutation
  (observables/charge_pump.jl:100-155);
* the manifold selection of _flux_point_states_for_chern
  (many_body_chern_number.jl:82-131), with each sector diagonalised densely by
  the oracle (the reference's mode=:matrix);
* many_body_chern_number (many_body_chern_number.jl:166-257) and the
  polarisation part of flux_charge_pump (charge_pump.jl:288-353).

Callers supply the model through ``point_inputs(flux)``, which returns the
oracle group arrays and term lists for one flux (generated by the tests from
the package's lattice module, which is input generation, not the checked
path).
"""
from __future__ import annotations

import math

import numpy as np


def position_phase_for_mask(m: int, site_phases: np.ndarray) -> complex:
    z = complex(1.0, 0.0)
    while m:
        lsb = m & -m
        z *= site_phases[lsb.bit_length() - 1]
        m ^= lsb
    return z


def apply_perm(m: int, perm0) -> int:
    r = 0
    i = 0
    while m:
        if m & 1:
            r |= 1 << int(perm0[i])
        m >>= 1
        i += 1
    return r


def position_operator_matrix(reps_to, reps_from, perm0: np.ndarray, chi_to: np.ndarray, chi_from: np.ndarray,
                             site_phases: np.ndarray) -> np.ndarray:
    """Dense (dim_to x dim_from) <chi_to|U|chi_from> (charge_pump.jl:47-91)."""
    index_to = {int(r): i for i, r in enumerate(reps_to)}
    nG = perm0.shape[0]
    M = np.zeros((len(reps_to), len(reps_from)), dtype=np.complex128)
    for col, rep in enumerate(reps_from):
        row = index_to.get(int(rep))
        if row is None:
            continue
        elem = 0j
        for g in range(nG):
            shifted = apply_perm(int(rep), perm0[g])
            elem += chi_to[g] * np.conj(chi_from[g]) * position_phase_for_mask(shifted, site_phases)
        elem *= 1.0 / nG
        if abs(elem) > 1e-13:
            M[row, col] = elem
    return M


def subspace_overlap_matrix(states_a, states_b) -> np.ndarray:
    n = len(states_a)
    if len(states_b) != n:
        raise ValueError("Chern link compares subspaces of different dimensions.")
    M = np.zeros((n, n), dtype=np.complex128)
    for i in range(n):
        for j in range(n):
            M[i, j] = np.vdot(states_a[i], states_b[j])
    return M


def unit_det_link(states_a, states_b, det_atol: float = 1e-10):
    z = np.linalg.det(subspace_overlap_matrix(states_a, states_b))
    if abs(z) <= det_atol:
        raise ValueError("Singular Berry link")
    return z / abs(z), abs(z)


def best_phase_permutation(raw, prev):
    nb = len(prev)
    best = [list(range(nb)), math.inf]
    for perm in _perms(nb):
        cost = 0.0
        for depth, j in enumerate(perm):
            d = raw[j] - prev[depth]
            d -= round(d)
            cost += d * d
        if cost < best[1]:
            best = [list(perm), cost]
    return best[0]


def _perms(n):
    # lexicographic, so that ties resolve like the reference's depth-first
    # search (the first minimum found is kept)
    import itertools

    return itertools.permutations(range(n))


def tracked_phase_branches(raw: np.ndarray) -> np.ndarray:
    nt, nb = raw.shape
    out = np.zeros_like(raw)
    order = np.argsort(raw[0], kind="stable")
    out[0] = raw[0, order]
    prev = out[0].copy()
    for t in range(1, nt):
        p = best_phase_permutation(raw[t], prev)
        for b in range(nb):
            phi = raw[t, p[b]]
            out[t, b] = phi + round(prev[b] - phi)
        prev = out[t].copy()
    return out


def flux_point(O, point_inputs, flux, manifold_size: int, atol: float = 1e-12):
    """Every sector solved densely at one flux; the globally lowest
    ``manifold_size`` states, their gap, sector objects and Fock vectors."""
    perm0, phases, identity0, stats, n_filled, irreps, bil0, den0 = point_inputs(flux)
    cat = O.Catalog(perm0, phases, identity0, stats, n_filled)
    cands, secs = [], {}
    for label, chi in irreps:
        sec = O.Sector(cat, chi)
        if sec.dim == 0:
            continue
        op = O.Op(sec, bil0, den0)
        w, v = np.linalg.eigh(op.dense())
        secs[label] = (sec, chi, v)
        for lev in range(min(manifold_size + 1, len(w))):
            cands.append((float(w[lev]), label, lev))
    cands.sort(key=lambda c: c[0])
    gap = cands[manifold_size][0] - cands[manifold_size - 1][0]
    if not gap > 1e-9:
        raise ValueError("manifold is not isolated")
    sel = cands[:manifold_size]
    states = [secs[label][0].expand_fock(secs[label][2][:, lev], atol) for _, label, lev in sel]
    return {"cat": cat, "secs": secs, "sel": sel, "gap": gap, "states": states, "perm0": perm0}


def chern_number(O, point_inputs, manifold_size: int, nx: int, ny: int):
    pts = [[flux_point(O, point_inputs, (ix / nx, iy / ny), manifold_size) for iy in range(ny)] for ix in range(nx)]
    Ux = np.zeros((nx, ny), dtype=np.complex128)
    Uy = np.zeros((nx, ny), dtype=np.complex128)
    dets = []
    for ix in range(nx):
        for iy in range(ny):
            ixp, iyp = (ix + 1) % nx, (iy + 1) % ny
            Ux[ix, iy], a = unit_det_link(pts[ix][iy]["states"], pts[ixp][iy]["states"])
            Uy[ix, iy], b = unit_det_link(pts[ix][iy]["states"], pts[ix][iyp]["states"])
            dets += [a, b]
    curv = np.zeros((nx, ny))
    for ix in range(nx):
        for iy in range(ny):
            ixp, iyp = (ix + 1) % nx, (iy + 1) % ny
            curv[ix, iy] = np.angle(Ux[ix, iy] * Uy[ixp, iy] * np.conj(Ux[ix, iyp]) * np.conj(Uy[ix, iy]))
    return {"chern_number": float(curv.sum() / (2 * math.pi)),
            "min_gap": min(p["gap"] for row in pts for p in row), "min_link_det": float(min(dets)),
            "berry_curvature": curv}


def charge_pump(O, point_inputs, site_phases: np.ndarray, fluxes, manifold_size: int):
    pol = np.zeros((len(fluxes), manifold_size), dtype=np.complex128)
    gaps, min_sv, Ps = [], [], []
    for t, th in enumerate(fluxes):
        pt = flux_point(O, point_inputs, (float(th), 0.0), manifold_size)
        gaps.append(pt["gap"])
        P = np.zeros((manifold_size, manifold_size), dtype=np.complex128)
        for r, (_, lt, levt) in enumerate(pt["sel"]):
            sec_t, chi_t, v_t = pt["secs"][lt]
            reps_t = sec_t.arrays()[0]
            for c, (_, lf, levf) in enumerate(pt["sel"]):
                sec_f, chi_f, v_f = pt["secs"][lf]
                U = position_operator_matrix(reps_t, sec_f.arrays()[0], pt["perm0"], chi_t, chi_f, site_phases)
                P[r, c] = np.vdot(v_t[:, levt], U @ v_f[:, levf])
        Ps.append(P)
        min_sv.append(float(np.linalg.svd(P, compute_uv=False).min()))
        ev = np.linalg.eigvals(P)
        pol[t] = ev[np.argsort(np.angle(ev), kind="stable")]
    raw = np.angle(pol) / (2 * math.pi)
    tr = tracked_phase_branches(raw)
    traj = tr - tr[0:1]
    return {"pumped_charges": traj[-1].copy(), "min_gap": float(min(gaps)), "min_position_singular_values": min_sv,
            "projected": Ps}
