"""pytreegrav_gb300 -- a GB300-native (sm_103a) Barnes-Hut gravity engine behind pytreegrav's API.

    from pytreegrav_gb300 import Accel, Potential, AccelTarget, PotentialTarget, TidalTensor, \
        TidalTensorTarget, ConstructTree, Field, ColumnDensity, DensityCorrFunc, VelocityCorrFunc, \
        VelocityStructFunc

The compute path is libpytreegrav_gb300.so (hand-written CUDA, C ABI in include/pytreegrav_gb300.h),
built in-tree by ``python -m pytreegrav_gb300.build``.
"""

from .frontend import (Accel, AccelTarget, ColumnDensity, ConstructTree, DensityCorrFunc, Field, Potential,
                       PotentialTarget, TidalTensor, TidalTensorTarget, VelocityCorrFunc, VelocityStructFunc,
                       checkTreeQuadrupoles, valueTestMethod, warn_if_coincident_positions)
from .tree import Octree, TargetSet, bruteforce, morton_order

__all__ = [
    "Accel", "AccelTarget", "ColumnDensity", "ConstructTree", "DensityCorrFunc", "Field", "Potential",
    "PotentialTarget", "TidalTensor", "TidalTensorTarget", "VelocityCorrFunc", "VelocityStructFunc", "checkTreeQuadrupoles", "valueTestMethod", "warn_if_coincident_positions", "Octree",
    "TargetSet", "bruteforce", "morton_order",
]
