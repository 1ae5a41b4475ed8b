"""Model cases shared by the tests.

Each case is a (model, n_filled, twist) triple built with the package's own
lattice generator; the oracle and the device library are fed the same group
and term arrays.  Sizes are chosen so the CPU oracle finishes in seconds.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from realspace_exactdiagonalization_gb300 import lattice as L
from realspace_exactdiagonalization_gb300.groups import statistics_from_name


@dataclass
class Case:
    name: str
    spec: L.ModelSpec
    theta: Tuple[float, float] = (0.0, 0.0)
    stats_override: str = ""

    @property
    def statistics(self) -> str:
        return self.stats_override or self.spec.statistics

    @property
    def stats_code(self) -> int:
        return statistics_from_name(self.statistics).code

    def group(self):
        return L.build_translation_group(self.spec.lattice, self.theta)

    def irreps(self):
        return L.build_translation_irrep_list(self.group(), self.spec.lattice)

    def bilinear0(self):
        """0-based (i, j, t) for the oracle."""
        return [(i - 1, j - 1, t) for (i, j, t) in self.spec.bilinear_terms(self.theta)]

    def density0(self):
        return [(i - 1, j - 1, v) for (i, j, v) in self.spec.density_terms]

    def bilinear1(self):
        return list(self.spec.bilinear_terms(self.theta))

    def density1(self):
        return list(self.spec.density_terms)


def small_cases() -> List[Case]:
    return [
        Case("ring16", L.ring_xxz(16, 1.0, 2.0)),
        Case("heisenberg18", L.heisenberg_ring(18)),
        Case("haldane2x3", L.haldane_honeycomb(2, 3)),
        Case("hubbard2x3", L.hubbard_square(2, 3)),
        Case("checkerboard3x2_f_flux0", L.checkerboard(3, 2, n_filled=4)),
        Case("checkerboard3x2_f_flux", L.checkerboard(3, 2, n_filled=4), theta=(0.23, 0.17)),
        Case("checkerboard3x2_f_flux1", L.checkerboard(3, 2, n_filled=4), theta=(1.0, 0.0)),
        Case("checkerboard3x2_b_flux", L.checkerboard(3, 2, n_filled=4), theta=(0.23, 0.17),
             stats_override="bosonic"),
        Case("hubbard2x4_flux", L.hubbard_square(2, 4, n_filled=5), theta=(0.3, 0.1)),
    ]


def case_by_name(name: str) -> Case:
    for c in small_cases():
        if c.name == name:
            return c
    raise KeyError(name)


def oracle_objects(O, case: Case, sector: int):
    G = case.group()
    cat = O.Catalog(G.perm0(), G.phases(), G.identity_idx - 1, case.stats_code, case.spec.n_filled)
    sec = O.Sector(cat, case.irreps()[sector].array())
    op = O.Op(sec, case.bilinear0(), case.density0())
    return cat, sec, op


def x_ramp(n: int) -> np.ndarray:
    """x = 1:n .+ im, the probe vector of the reference's flux_regression.jl:32-34."""
    return np.arange(1, n + 1, dtype=np.float64) + 1j


def x_random(n: int, seed: int = 7) -> np.ndarray:
    r = np.random.default_rng(seed)
    return r.standard_normal(n) + 1j * r.standard_normal(n)


def assert_lanczos_spectrum(vals, ref, tol, msg=""):
    """Lanczos semantics (the reference's KrylovKit branch, n > 500): every
    returned value is an eigenvalue; the distinct returned values are exactly
    the lowest distinct eigenvalues (none skipped), each copy at most as often
    as its multiplicity.  A single-vector Krylov method may return an exactly
    degenerate level fewer times than its multiplicity."""
    distinct, mult = [], []
    for e in ref:
        if distinct and abs(e - distinct[-1]) <= 1e-8 * max(1.0, abs(e)):
            mult[-1] += 1
        else:
            distinct.append(e)
            mult.append(1)
    got = []
    for v in vals:
        i = int(np.argmin([abs(v - d) for d in distinct]))
        assert abs(v - distinct[i]) <= tol, (msg, v, distinct[:6])
        got.append(i)
    assert got == sorted(got), msg
    assert sorted(set(got)) == list(range(len(set(got)))), (msg, got)
    for i in set(got):
        assert got.count(i) <= mult[i], (msg, got, mult[:6])


def _cycles(perm0_row):
    seen, cycles = set(), []
    for s in range(len(perm0_row)):
        if s in seen:
            continue
        c, t = [], s
        while t not in seen:
            seen.add(t)
            c.append(t)
            t = int(perm0_row[t])
        cycles.append(c)
    return cycles


def fixed_masks(perm0_row, n_filled, species=None):
    """Masks with the catalog's particle numbers that the permutation maps to
    themselves: unions of whole cycles (each cycle stays inside one species
    when the group preserves the species)."""
    cycles = _cycles(perm0_row)
    if species:
        n_split, n_lo, n_hi = species
        want = (n_lo, n_hi)
        weight = [(len(c) if c[0] < n_split else 0, len(c) if c[0] >= n_split else 0) for c in cycles]
    else:
        want = (n_filled, 0)
        weight = [(len(c), 0) for c in cycles]
    out = []

    def rec(i, a, b, m):
        if a == want[0] and b == want[1]:
            out.append(m)
            return
        if i == len(cycles) or a > want[0] or b > want[1]:
            return
        rec(i + 1, a, b, m)
        bits = 0
        for s in cycles[i]:
            bits |= 1 << s
        rec(i + 1, a + weight[i][0], b + weight[i][1], m | bits)

    rec(0, 0, 0, 0)
    return out


def character_dimension(oracle, group, stats_code, chi, n_filled, species=None, n_states=None):
    """Sector dimension from the trace of the projector onto the irrep chi,
    (1/|G|) sum_g conj(chi(g)) sum_{m : g(m) = m} alpha_g(m), over the fixed
    masks of each element only: a check of the sector basis (one row per
    compatible orbit, SRE:534-556) that needs no enumeration of the basis.  The
    identity's trace is the number of basis states, ``n_states``."""
    perm0, phases = group.perm0(), group.phases()
    tot = 0j
    for g in range(len(perm0)):
        if g == group.identity_idx - 1:
            tr = complex(n_states)
        else:
            tr = 0j
            for m in fixed_masks(perm0[g], n_filled, species):
                img, a = oracle.apply_op(perm0[g], phases[g], stats_code, m)
                assert img == m
                tr += a
        tot += np.conj(chi[g]) * tr
    d = tot / len(perm0)
    assert abs(d.imag) < 1e-6 and abs(d.real - round(d.real)) < 1e-6, d
    return int(round(d.real))
