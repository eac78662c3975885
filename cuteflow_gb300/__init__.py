"""GB300-native CuteFlow time step: FP64 St-Venant finite volumes on unstructured triangles.

``Solver`` drives the sm_103a step through the C ABI of include/cuteflow_gb300.h;
``Batch`` steps many independent simulations together; ``adjoint.Adjoint`` and
``adjoint.gauge_run`` give Manning and initial-state gradients by the discrete adjoint;
``cases`` builds seeded synthetic inputs in the reference's mesh-table format.
"""
from . import _abi, cases  # noqa: F401
from .solver import Batch, CFError, Solver, StepInfo, load  # noqa: F401
from .adjoint import Adjoint, gauge_run  # noqa: F401,E402
