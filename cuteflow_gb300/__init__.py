"""GB300-native CuteFlow time step: FP64 St-Venant finite volumes on unstructured triangles.

``Solver`` drives the sm_103a step through the C ABI of include/cuteflow_gb300.h;
``cases`` builds seeded synthetic inputs in the reference's mesh-table format.
"""
from . import _abi, cases  # noqa: F401
from .solver import Batch, CFError, Solver, StepInfo, load  # noqa: F401
