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
