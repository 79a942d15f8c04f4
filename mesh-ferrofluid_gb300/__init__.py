"""mesh-ferrofluid_gb300 -- GB300 (sm_103a) implementation of the GeCao/Mesh-Ferrofluid
boundary-element hot path: RWG method-of-moments assembly / excitation / solve and the
3D Laplace single- and double-layer Galerkin operators.

The directory name contains a hyphen, so import it with
``importlib.import_module("mesh-ferrofluid_gb300")``; the package also registers itself as
``mesh_ferrofluid_gb300`` in ``sys.modules``.

Public surface (mirrors the reference's ``src.mesh_BEM`` / ``src.utils`` entry points):
``MeshBEMSolver3d``, ``MeshMOMZmatKernel``, ``MeshMOMRhsKernel``,
``MeshMOMInterpolateJsKernel``, the op module ``mesh_MOM_3d``,
``double_integration_on_panels_3d``, the layer classes and the utilities of ``utils``;
``ray_query.RayQueryApp`` replaces the Vulkan ray-query plugin.
The compute path is libmeshbem_gb300.so (``build.py``); nothing falls back to the CPU.
"""
import sys as _sys

_sys.modules.setdefault("mesh_ferrofluid_gb300", _sys.modules[__name__])

from . import batch, layers, learned, mesh_io, meshes, mesh_MOM_3d, ray_query, roofline, utils  # noqa: E402
from ._lib import MeshBEMError, load as load_library  # noqa: E402
from .kernel_functions import (  # noqa: E402
    MeshMOMInterpolateJsKernel,
    MeshMOMRhsKernel,
    MeshMOMZmatKernel,
)
from .layers import (  # noqa: E402
    DoubleLayer3d,
    HyperSingularLayer3d,
    RhsLayer3d,
    SingleLayer3d,
    double_integration_on_panels_3d,
)
from .mesh_BEM_solver_3d import MeshBEMSolver3d  # noqa: E402
from .mesh_pressure import MeshPressure  # noqa: E402
from .ray_query import RayQueryApp  # noqa: E402
from .utils import (  # noqa: E402
    BEMType,
    BoundaryType,
    LayerType,
    Logger,
    OrderType,
    PanelRelationType,
    VertexType,
)

__all__ = [
    "MeshBEMSolver3d", "MeshMOMZmatKernel", "MeshMOMRhsKernel", "MeshMOMInterpolateJsKernel",
    "mesh_MOM_3d", "double_integration_on_panels_3d", "SingleLayer3d", "DoubleLayer3d",
    "RhsLayer3d", "BEMType", "BoundaryType", "LayerType", "OrderType", "PanelRelationType",
    "Logger", "MeshBEMError", "load_library", "meshes", "utils", "ray_query", "RayQueryApp",
    "HyperSingularLayer3d", "MeshPressure", "VertexType", "layers",
]
