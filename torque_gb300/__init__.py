"""torque_gb300: GB300-native block-sparse tensor contraction (sm_103a).

The compute path is libtorque_gb300.so (hand-written CUDA behind a C ABI,
include/torque_gb300.h); this package is its Python binding and the host-side
helpers (charge-sector constructors, synthetic workloads, the PEPS-norm driver,
the cost model's data and proposal logic).
"""
from ._lib import TorqueError, load  # noqa: F401
from .block_sparse import Batch, BlockSparseTensor, ContractionPlan, contract_blocks  # noqa: F401
from .dense import DenseTensor, SparseTensor  # noqa: F401
from .sectors import BlockList, Leg, charge_blocks  # noqa: F401

__all__ = ["BlockSparseTensor", "ContractionPlan", "Batch", "contract_blocks", "DenseTensor",
           "SparseTensor",
           "TorqueError", "Leg", "BlockList", "charge_blocks", "load"]
