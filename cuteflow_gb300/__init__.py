"""GB300-native CuteFlow time step: FP64 St-Venant finite volumes on unstructured triangles."""
from . import _abi, cases  # noqa: F401
