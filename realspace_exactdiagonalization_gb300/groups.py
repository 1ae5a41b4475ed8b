"""Symmetry operations, finite groups and one-dimensional irreps.

Host-side mirror of the reference types ``Symmetry_Operation``
(src/symmetry_resolved_ed.jl:62-79), ``Finite_Symmetry_Group`` (:90-104) and
``OneDim_Irrep`` (:501-506).  Permutations are 1-based, as in the reference;
``perm0()`` gives the 0-based array the C ABI takes.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, List, Optional, Sequence

import numpy as np


class Particle_Statistics:
    code = -1


class Bosonic(Particle_Statistics):
    """Hard-core bosons (reference src/second_quantized_model.jl:1-4)."""

    code = 0

    def __eq__(self, other):
        return isinstance(other, Bosonic)

    def __hash__(self):
        return 0

    def __repr__(self):
        return "Bosonic()"


class Fermionic(Particle_Statistics):
    """Spinless fermions (reference src/second_quantized_model.jl:1-4)."""

    code = 1

    def __eq__(self, other):
        return isinstance(other, Fermionic)

    def __hash__(self):
        return 1

    def __repr__(self):
        return "Fermionic()"


def statistics_from_name(name: str) -> Particle_Statistics:
    return Fermionic() if name.lower().startswith("ferm") else Bosonic()


@dataclass
class Symmetry_Operation:
    """One group element: ``U_g b+_i U_g^-1 = eta_g(i) b+_perm[i]`` (SRE:62-79)."""

    label: Any
    perm: List[int]
    perm_phases: Optional[List[complex]] = None

    def __post_init__(self):
        self.perm = [int(p) for p in self.perm]
        if self.perm_phases is None:
            self.perm_phases = [1.0 + 0.0j] * len(self.perm)
        else:
            self.perm_phases = [complex(v) for v in self.perm_phases]
        if len(self.perm_phases) != len(self.perm):
            raise ValueError("perm_phases must have one entry per site")


class Finite_Symmetry_Group:
    """A finite group of symmetry operations (SRE:90-104)."""

    def __init__(self, name: str, operations: Sequence[Symmetry_Operation], identity_idx: int = 1):
        if not operations:
            raise ValueError("a group needs at least one operation")
        n_site = len(operations[0].perm)
        for op in operations:
            if len(op.perm) != n_site or len(op.perm_phases) != n_site:
                raise ValueError("all operations must act on the same number of sites")
        if operations[identity_idx - 1].perm != list(range(1, n_site + 1)):
            raise ValueError("Identity must have trivial permutation")
        self.name = name
        self.n_site = n_site
        self.operations = list(operations)
        self.identity_idx = int(identity_idx)

    def __len__(self):
        return len(self.operations)

    def perm0(self) -> np.ndarray:
        """(n_ops, n_site) int32 array of 0-based targets."""
        return np.asarray([[p - 1 for p in op.perm] for op in self.operations], dtype=np.int32)

    def phases(self) -> np.ndarray:
        """(n_ops, n_site) complex128 array of per-site phases."""
        return np.asarray([op.perm_phases for op in self.operations], dtype=np.complex128)

    def same_permutations(self, other: "Finite_Symmetry_Group") -> bool:
        return len(self) == len(other) and all(a.perm == b.perm for a, b in zip(self.operations, other.operations))


def group_order(G: Finite_Symmetry_Group) -> int:
    return len(G.operations)


def build_identity_group(n_site: int) -> Finite_Symmetry_Group:
    """The trivial group (SRE:1362-1365)."""
    return Finite_Symmetry_Group("identity", [Symmetry_Operation("identity", list(range(1, n_site + 1)))], 1)


@dataclass
class OneDim_Irrep:
    """chi(g) for every group element (SRE:501-506)."""

    label: Any
    values: List[complex]

    def __post_init__(self):
        self.values = [complex(v) for v in self.values]

    def array(self) -> np.ndarray:
        return np.asarray(self.values, dtype=np.complex128)


def build_identity_irrep_list() -> List[OneDim_Irrep]:
    return [OneDim_Irrep("identity", [1.0 + 0.0j])]
