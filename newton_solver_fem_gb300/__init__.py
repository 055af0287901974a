"""GB300 (sm_103a) implementation of SolverFEM's per-substep hot path.

Public names follow the reference package (``newton_solver_fem/__init__.py``):
``SolverFEM`` (alias ``SolverLinearFEM``), ``FEMBuilder`` and ``LinearFEMData``,
plus the minimal ``Model`` / ``State`` / ``Control`` / ``Contacts`` containers the solver reads.
The numerical work runs in ``libfemgb300.so`` (``include/fem_gb300.h``).
"""

from .builder import (Contacts, Control, FEMBuilder, HashGrid, LinearFEMData, Model, State, hex_gauss_data,
                      model_from_arrays, triangle_rest_data)
from .prepared_step import PreparedFEMStep
from .solver import BsrMatrix, SolverFEM, SolverLinearFEM

__all__ = [
    "BsrMatrix",
    "Contacts",
    "Control",
    "FEMBuilder",
    "HashGrid",
    "LinearFEMData",
    "Model",
    "PreparedFEMStep",
    "SolverFEM",
    "SolverLinearFEM",
    "State",
    "hex_gauss_data",
    "model_from_arrays",
    "triangle_rest_data",
]
