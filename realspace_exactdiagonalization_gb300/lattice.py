"""Synthetic real-space lattices, hopping lists and translation groups.

The reference builds its models with the external TightBinding package
(`initialize_real_space_lattice`, `add_hopping_term!`, `generate_bilinear_terms`),
which is not vendored with it.  This module restates the behaviour the
reference relies on, in plain Python, so that the model shapes the reference
benchmarks (ring, Haldane honeycomb, checkerboard, spinful square Hubbard) can
be generated without it:

* a representative bond ``((cell_a, sub_a), (cell_b, sub_b)) => t`` added with
  ``is_hermitian=True`` is translated over every unit cell of the periodic
  sample, and its Hermitian partner is added with ``conj(t)``;
* bonds that land on the same ordered site pair with the same winding are
  **summed**; bonds on the same pair with different windings stay separate
  terms (their twist phases differ).  This is the semantics that reproduces
  the reference's stored numbers for samples with a side of length 2, where a
  bond and the partner of a translated bond coincide (tests/test_oracle_golden.py
  pins it against the Haldane 2x3 projection-table size and the Hubbard 2xL
  ground energies of ``benchmark/benchmark_data/benchmark_raw.csv``);
* twisted boundary phases follow the reference's docstring
  (``src/second_quantized_model.jl:29-37``): the hop from site ``i`` to site
  ``j`` is multiplied by ``exp(i 2 pi theta_d w_d)`` where ``w_d`` is the
  number of times the bond wraps the periodic boundary in direction ``d``;
* ``build_translation_group`` restates ``src/symmetry_resolved_ed.jl:1374-1405``
  (operations ordered ``dx`` outer, ``dy`` inner; the site phase is
  ``cis(2 pi theta . (cell - shifted_cell) / L)``), and
  ``build_translation_irrep_list`` restates ``:1415-1430``.

Sites are numbered cell-major then sublattice-minor (``x`` outer, ``y`` inner)
unless a builder says otherwise.  Spectra do not depend on the numbering, and
the orbit catalog is compared against the oracle on the same generated input.
Site indices in this module are 1-based, as in the reference API.
"""
from __future__ import annotations

import cmath
import math
from dataclasses import dataclass, field
from typing import Dict, List, Sequence, Tuple

Cell = Tuple[int, int]
SiteKey = Tuple[Cell, int]


@dataclass
class Real_Space_Lattice:
    """Minimal restatement of ``TightBinding.Real_Space_Lattice``."""

    sample_size: Tuple[int, int]
    n_sub: int
    site_list: List[SiteKey]
    site_to_index_map: Dict[SiteKey, int]
    pbc_indicator: Tuple[bool, bool] = (True, True)
    name: str = ""
    twisted_phases_over_2pi: List[float] = field(default_factory=lambda: [0.0, 0.0])
    # crystal coordinates of the sublattice sites inside a cell (``sub_crys_list``)
    sub_crys_list: List[Tuple[float, float]] = field(default_factory=list)

    def sub_crys(self, sub: int) -> Tuple[float, float]:
        """Offset of sublattice ``sub`` (1-based); zero when none was given."""
        return tuple(self.sub_crys_list[sub - 1]) if self.sub_crys_list else (0.0, 0.0)

    @property
    def n_site(self) -> int:
        return len(self.site_list)

    @property
    def dim(self) -> int:
        return 2


def initialize_real_space_lattice(sample_size: Sequence[int], n_sub: int, name: str = "",
                                  order: str = "cell_major",
                                  pbc_indicator: Sequence[bool] = (True, True),
                                  sub_crys_list: Sequence[Sequence[float]] = ()) -> Real_Space_Lattice:
    """Number the sites of an ``L1 x L2`` sample with ``n_sub`` sublattices.

    ``order="cell_major"``: index = (x*L2 + y)*n_sub + sub; ``"sub_major"``:
    index = sub*L1*L2 + x*L2 + y (used for the spinful Hubbard encoding with
    the up spin at bit i and the down spin at bit i + L1*L2).
    """
    L1, L2 = int(sample_size[0]), int(sample_size[1])
    sites: List[SiteKey] = []
    if order == "cell_major":
        for x in range(L1):
            for y in range(L2):
                for s in range(1, n_sub + 1):
                    sites.append(((x, y), s))
    elif order == "sub_major":
        for s in range(1, n_sub + 1):
            for x in range(L1):
                for y in range(L2):
                    sites.append(((x, y), s))
    else:
        raise ValueError(f"unknown site order {order!r}")
    idx = {key: i + 1 for i, key in enumerate(sites)}
    if sub_crys_list and len(sub_crys_list) != n_sub:
        raise ValueError("sub_crys_list needs one offset per sublattice")
    return Real_Space_Lattice((L1, L2), n_sub, sites, idx, tuple(bool(b) for b in pbc_indicator), name,
                              sub_crys_list=[tuple(float(v) for v in c) for c in sub_crys_list])


@dataclass
class TightBindingModel:
    """Bond list of a translation-invariant hopping model (``Real_Space_TightBinding_Model``)."""

    lattice: Real_Space_Lattice
    # ordered site pair (1-based from, to) -> [amplitude, winding (w1, w2)]
    full_hopping_map: Dict[Tuple[int, int], list] = field(default_factory=dict)

    def _insert(self, i: int, j: int, t: complex, w: Tuple[int, int]) -> None:
        key = (i, j)
        if key in self.full_hopping_map:
            entry = self.full_hopping_map[key]
            if tuple(entry[1]) != tuple(w):
                # Two bonds with different windings on the same site pair: the
                # twist phase would differ per bond, so keep them separate.
                self.full_hopping_map[(i, j, len(self.full_hopping_map))] = [t, w]
                return
            entry[0] += t
        else:
            self.full_hopping_map[key] = [t, w]


def add_hopping_term(tb: TightBindingModel, bond: Tuple[Tuple[Sequence[int], int], Tuple[Sequence[int], int]],
                     t: complex, is_hermitian: bool = True) -> None:
    """Translate a representative bond over every cell (``add_hopping_term!``)."""
    lat = tb.lattice
    L1, L2 = lat.sample_size
    (ca, sa), (cb, sb) = bond
    for x in range(L1):
        for y in range(L2):
            ax, ay = x + ca[0], y + ca[1]
            bx, by = x + cb[0], y + cb[1]
            # windings of each end relative to the folded sample
            wa = (ax // L1, ay // L2)
            wb = (bx // L1, by // L2)
            if (not lat.pbc_indicator[0] and (wa[0] or wb[0])) or (not lat.pbc_indicator[1] and (wa[1] or wb[1])):
                continue
            i = lat.site_to_index_map[((ax % L1, ay % L2), sa)]
            j = lat.site_to_index_map[((bx % L1, by % L2), sb)]
            w = (wb[0] - wa[0], wb[1] - wa[1])
            tb._insert(i, j, complex(t), w)
            if is_hermitian:
                tb._insert(j, i, complex(t).conjugate(), (-w[0], -w[1]))


def generate_bilinear_terms(tb: TightBindingModel, twisted_phases_over_2pi: Sequence[float] = (0.0, 0.0)
                            ) -> List[Tuple[int, int, complex]]:
    """Bilinear terms ``(i, j, t)`` with the twist phase ``exp(i 2 pi theta . w)``."""
    th = [float(v) for v in twisted_phases_over_2pi] + [0.0] * (2 - len(twisted_phases_over_2pi))
    out = []
    for key, (t, w) in tb.full_hopping_map.items():
        i, j = key[0], key[1]
        ph = w[0] * th[0] + w[1] * th[1]
        amp = t if ph == 0.0 else t * cmath.exp(2j * math.pi * ph)
        if amp != 0:
            out.append((i, j, complex(amp)))
    return out


# --------------------------------------------------------------------- groups
def build_translation_group(lattice: Real_Space_Lattice, theta: Sequence[float] = ()):
    """Flux-aware translation group Z_L1 x Z_L2 (reference SRE:1374-1405)."""
    from .groups import Finite_Symmetry_Group, Symmetry_Operation

    L1, L2 = lattice.sample_size
    if len(theta) == 0:
        th = list(lattice.twisted_phases_over_2pi) if lattice.twisted_phases_over_2pi else [0.0, 0.0]
    else:
        if len(theta) != lattice.dim:
            raise ValueError(f"theta must have length {lattice.dim}.")
        th = [float(v) for v in theta]
    ops = []
    for dx in range(L1):
        for dy in range(L2):
            perm = [0] * lattice.n_site
            phases = [0j] * lattice.n_site
            for i, (cell, sub) in enumerate(lattice.site_list):
                sx, sy = (cell[0] + dx) % L1, (cell[1] + dy) % L2
                perm[i] = lattice.site_to_index_map[((sx, sy), sub)]
                arg = th[0] * ((cell[0] - sx) / L1) + th[1] * ((cell[1] - sy) / L2)
                phases[i] = complex(math.cos(2 * math.pi * arg), math.sin(2 * math.pi * arg))
            ops.append(Symmetry_Operation((dx, dy), perm, perm_phases=phases))
    return Finite_Symmetry_Group("translations", ops, identity_idx=1)


def build_translation_irrep_list(G, lattice: Real_Space_Lattice):
    """Momentum irreps chi(g) = cis(2 pi (k1 dx / L1 + k2 dy / L2)) (SRE:1415-1430)."""
    from .groups import OneDim_Irrep

    L1, L2 = lattice.sample_size
    if G.name != "translations" or len(G.operations) != L1 * L2:
        raise ValueError("expected the translation group of this lattice")
    out = []
    for k1 in range(L1):
        for k2 in range(L2):
            vals = []
            for op in G.operations:
                dx, dy = op.label
                a = 2 * math.pi * (k1 * dx / L1 + k2 * dy / L2)
                vals.append(complex(math.cos(a), math.sin(a)))
            out.append(OneDim_Irrep((k1, k2), vals))
    return out


# ------------------------------------------------------------------ models
@dataclass
class ModelSpec:
    """A second-quantized model plus its translation-symmetry data."""

    name: str
    lattice: Real_Space_Lattice
    tb: TightBindingModel
    statistics: str  # "bosonic" | "fermionic"
    density_terms: List[Tuple[int, int, complex]]
    n_filled: int
    # (n_split, n_lo, n_hi): two separately conserved species, n_lo particles
    # on the first n_split modes and n_hi on the rest (None: only the total
    # particle number is fixed, as in the reference)
    species: Tuple[int, int, int] | None = None

    def bilinear_terms(self, theta: Sequence[float] = (0.0, 0.0)) -> List[Tuple[int, int, complex]]:
        return generate_bilinear_terms(self.tb, theta)


def ring_xxz(N: int, t: float = 1.0, V: float = 2.0, n_filled: int | None = None) -> ModelSpec:
    """Hard-core bosons on an N-site ring: -t sum (b+_i b_i+1 + h.c.) + V sum n_i n_i+1."""
    lat = initialize_real_space_lattice((N, 1), 1, f"ring{N}", pbc_indicator=(True, False))
    tb = TightBindingModel(lat)
    add_hopping_term(tb, (((0, 0), 1), ((1, 0), 1)), -t)
    den = [(lat.site_to_index_map[((x, 0), 1)], lat.site_to_index_map[(((x + 1) % N, 0), 1)], complex(V))
           for x in range(N)]
    return ModelSpec(f"ring{N}", lat, tb, "bosonic", den, N // 2 if n_filled is None else n_filled)


def heisenberg_ring(N: int, J: float = 1.0) -> ModelSpec:
    """S=1/2 Heisenberg ring as hard-core bosons (reference benchmark/benchmark.jl:67-111)."""
    lat = initialize_real_space_lattice((N, 1), 1, f"heisenberg{N}", pbc_indicator=(True, False))
    tb = TightBindingModel(lat)
    add_hopping_term(tb, (((0, 0), 1), ((1, 0), 1)), J / 2)
    den = []
    for x in range(N):
        den.append((lat.site_to_index_map[((x, 0), 1)], lat.site_to_index_map[(((x + 1) % N, 0), 1)], complex(J)))
    for x in range(N):
        i = lat.site_to_index_map[((x, 0), 1)]
        den.append((i, i, complex(-J / 2)))
    return ModelSpec(f"heisenberg{N}", lat, tb, "bosonic", den, N // 2)


def haldane_honeycomb(L1: int, L2: int, t: float = 1.0, tp: float = 0.6, tpp: float = -0.58,
                      phi_over_2pi: float = 0.2, n_filled: int | None = None) -> ModelSpec:
    """Haldane honeycomb hard-core bosons (reference benchmark/benchmark.jl:114-152)."""
    lat = initialize_real_space_lattice((L1, L2), 2, f"haldane{L1}x{L2}", sub_crys_list=[(0.0, 0.0), (1 / 3, 1 / 3)])
    tb = TightBindingModel(lat)
    s = 2 * math.pi * phi_over_2pi
    e = cmath.exp(1j * s)
    ec = cmath.exp(-1j * s)
    add_hopping_term(tb, (((0, 0), 1), ((0, 0), 2)), -t)
    add_hopping_term(tb, (((0, 0), 1), ((0, -1), 2)), -t)
    add_hopping_term(tb, (((0, 0), 1), ((-1, 0), 2)), -t)
    add_hopping_term(tb, (((0, 0), 1), ((1, 0), 1)), -tp * e)
    add_hopping_term(tb, (((0, 0), 1), ((0, 1), 1)), -tp * ec)
    add_hopping_term(tb, (((0, 0), 1), ((-1, 1), 1)), -tp * e)
    add_hopping_term(tb, (((0, 0), 2), ((1, 0), 2)), -tp * ec)
    add_hopping_term(tb, (((0, 0), 2), ((0, 1), 2)), -tp * e)
    add_hopping_term(tb, (((0, 0), 2), ((-1, 1), 2)), -tp * ec)
    add_hopping_term(tb, (((0, 0), 2), ((1, 1), 1)), -tpp)
    add_hopping_term(tb, (((1, 0), 1), ((0, 1), 2)), -tpp)
    add_hopping_term(tb, (((1, 0), 2), ((0, 1), 1)), -tpp)
    nf = (L1 * L2) // 2 if n_filled is None else n_filled
    return ModelSpec(f"haldane{L1}x{L2}", lat, tb, "bosonic", [], nf)


def checkerboard(L1: int, L2: int, t: float = 1.0, tp1: float = 0.3, tp2: float = -0.3, tpp: float = -0.2,
                 phi_over_2pi: float = 1 / 8, V1: float = 1.0, V2: float = 0.0, V3: float = 0.0,
                 n_filled: int | None = None, statistics: str = "fermionic") -> ModelSpec:
    """Checkerboard spinless fermions with staggered flux (reference
    phase_exploration/src/model.jl:1-71, bond list and density rules)."""
    lat = initialize_real_space_lattice((L1, L2), 2, f"checkerboard{L1}x{L2}", sub_crys_list=[(0.5, 0.0), (0.0, 0.5)])
    tb = TightBindingModel(lat)
    ph = 2 * math.pi * phi_over_2pi
    add_hopping_term(tb, (((0, 0), 1), ((0, 0), 2)), -t * cmath.exp(-1j * ph))
    add_hopping_term(tb, (((0, 0), 1), ((1, 0), 2)), -t * cmath.exp(1j * ph))
    add_hopping_term(tb, (((0, 0), 2), ((0, 1), 1)), -t * cmath.exp(-1j * ph))
    add_hopping_term(tb, (((1, 0), 2), ((0, 1), 1)), -t * cmath.exp(1j * ph))
    add_hopping_term(tb, (((0, 0), 1), ((1, 0), 1)), -tp1)
    add_hopping_term(tb, (((0, 0), 1), ((0, 1), 1)), -tp2)
    add_hopping_term(tb, (((0, 0), 2), ((1, 0), 2)), -tp2)
    add_hopping_term(tb, (((0, 0), 2), ((0, 1), 2)), -tp1)
    add_hopping_term(tb, (((0, 0), 1), ((1, 1), 1)), -tpp)
    add_hopping_term(tb, (((0, 0), 2), ((1, 1), 2)), -tpp)
    add_hopping_term(tb, (((1, 0), 2), ((0, 1), 2)), -tpp)
    add_hopping_term(tb, (((0, 1), 1), ((1, 0), 1)), -tpp)
    den = []
    for i_from, (cf, sf) in enumerate(lat.site_list, start=1):
        for i_to, (ct, st) in enumerate(lat.site_list, start=1):
            if i_from == i_to:
                continue
            sh = ((ct[0] - cf[0]) % L1, (ct[1] - cf[1]) % L2)
            if V1 != 0 and sf == 1 and st == 2 and sh in ((0, 0), (1, 0), (0, L2 - 1), (1, L2 - 1)):
                den.append((i_from, i_to, complex(V1)))
            if V2 != 0 and sf == st and sh in ((1, 0), (0, 1)):
                den.append((i_from, i_to, complex(V2)))
            if V3 != 0 and sf == st and sh in ((1, 1), (1, L2 - 1)):
                den.append((i_from, i_to, complex(V3)))
    nf = (2 * L1 * L2) // 6 if n_filled is None else n_filled
    return ModelSpec(f"checkerboard{L1}x{L2}", lat, tb, statistics, den, nf)


def hubbard_square(L1: int, L2: int, t: float = 1.0, U: float = 8.0, n_filled: int | None = None,
                   order: str = "sub_major", n_up: int | None = None, n_dn: int | None = None) -> ModelSpec:
    """Spinful Fermi-Hubbard on an L1 x L2 square torus as 2*L1*L2 fermionic
    modes (sublattice 1 = up, 2 = down; reference benchmark/benchmark.jl:155-219).
    ``order="sub_major"`` puts the up spin of cell i at bit i and the down spin
    at bit i + L1*L2.  The particle number is fixed over all S^z, as in the
    reference (its default is half filling, N = L1*L2).  With ``n_up`` and
    ``n_dn`` (sub_major order only) the model carries the two-species block
    (N_up, N_down) instead: species = (L1*L2, n_up, n_dn)."""
    lat = initialize_real_space_lattice((L1, L2), 2, f"hubbard{L1}x{L2}", order=order)
    spinless = initialize_real_space_lattice((L1, L2), 1, "square")
    tb1 = TightBindingModel(spinless)
    add_hopping_term(tb1, (((0, 0), 1), ((1, 0), 1)), -t)
    add_hopping_term(tb1, (((0, 0), 1), ((0, 1), 1)), -t)
    tb = TightBindingModel(lat)
    cell_of = {v: k[0] for k, v in spinless.site_to_index_map.items()}
    for key, (amp, w) in tb1.full_hopping_map.items():
        cf, ct = cell_of[key[0]], cell_of[key[1]]
        for s in (1, 2):
            tb._insert(lat.site_to_index_map[(cf, s)], lat.site_to_index_map[(ct, s)], amp, tuple(w))
    den = []
    for y in range(L2):
        for x in range(L1):
            den.append((lat.site_to_index_map[((x, y), 1)], lat.site_to_index_map[((x, y), 2)], complex(U)))
    if (n_up is None) != (n_dn is None):
        raise ValueError("give both n_up and n_dn, or neither")
    if n_up is not None:
        if order != "sub_major":
            raise ValueError("the (N_up, N_down) block needs the sub_major mode order")
        if n_filled is not None and n_filled != n_up + n_dn:
            raise ValueError("n_filled must equal n_up + n_dn")
        return ModelSpec(f"hubbard{L1}x{L2}_{n_up}u{n_dn}d", lat, tb, "fermionic", den, n_up + n_dn,
                         (L1 * L2, n_up, n_dn))
    nf = L1 * L2 if n_filled is None else n_filled
    return ModelSpec(f"hubbard{L1}x{L2}", lat, tb, "fermionic", den, nf)
