"""GB300-native differentiable iso-surface extraction (DiffMC / DiffDMC).

Drop-in for the reference package's public API (diso/__init__.py):

    from diso_gb300 import DiffMC, DiffDMC
    verts, faces = DiffMC(dtype=torch.float32)(sdf, deform, isovalue=0.0, normalize=True)
    verts, faces = DiffDMC(dtype=torch.float32)(sdf, deform, isovalue=0.0, return_quads=False, normalize=True)

The compute path is hand-written sm_103a CUDA behind the C ABI of
include/diso_gb300.h; there is no CPU path.
"""
from .batch import BatchPlan, DiffDMCBatch, DiffMCBatch, extract_batch  # noqa: F401
from .bricks import BrickGrid, extract_bricks  # noqa: F401
from .extraction import DiffDMC, DiffMC, extract  # noqa: F401
from .fields import SphereUnion, extract_field  # noqa: F401
from .neural import MLPField, extract_mlp  # noqa: F401
from . import tune  # noqa: F401

__all__ = ["DiffMC", "DiffDMC", "extract", "DiffMCBatch", "DiffDMCBatch", "extract_batch", "BatchPlan", "SphereUnion",
           "extract_field", "BrickGrid", "extract_bricks", "MLPField", "extract_mlp", "tune"]
__version__ = "0.1.0"
