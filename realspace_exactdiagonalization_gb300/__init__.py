"""GB300-native symmetry-sector exact diagonalization.

Drop-in for the matrix-free hot path of the Julia package
RealSpace_ExactDiagonalization: device construction of the orbit catalog and
sector basis, the sector H|psi> gather kernel, and the Lanczos solve around it,
all behind the C ABI of libsed_gb300.so (include/sed_capi.h).  Importing the
package does not load the CUDA library; the first compute call does, and
raises if it has not been built.
"""
from .api import *  # noqa: F401,F403
from .api import __all__ as _api_all
from .lattice import build_translation_group, build_translation_irrep_list  # noqa: F401
from .observables import (flux_charge_pump, many_body_chern_number,  # noqa: F401
                          many_body_position_phases, position_operator_matrix)

__all__ = list(_api_all) + ["build_translation_group", "build_translation_irrep_list", "flux_charge_pump",
                            "many_body_chern_number", "many_body_position_phases", "position_operator_matrix"]
