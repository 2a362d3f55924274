"""GB300-native SlakoNet electronic-structure path (sm_103a CUDA kernels behind a C ABI)."""
from .model import (Geometry, MultiElementSkfParameterOptimizer, SkfParameterOptimizer, properties_dict,  # noqa: F401
                    reduce_time_reversal)
from .engine import Engine, TableSet, plan_batch  # noqa: F401
from .pdos import compute_atom_projected_dos  # noqa: F401

__all__ = ["Geometry", "MultiElementSkfParameterOptimizer", "SkfParameterOptimizer", "Engine", "TableSet",
           "plan_batch", "properties_dict", "compute_atom_projected_dos", "reduce_time_reversal"]
