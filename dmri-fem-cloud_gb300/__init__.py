"""GB300 Bloch-Torrey finite-element engine (drop-in for the solve path of
van-dang/DMRI-FEM-Cloud).

The package directory name contains hyphens, so import it with
``importlib.import_module("dmri-fem-cloud_gb300")``.  Compute runs in
``libbtgpu.so`` (hand-written sm_103a CUDA behind a C ABI, ``include/btgpu.h``);
this package holds the host side: the ctypes binding (``_native``), the
reference-named API (``api``), time profiles (``sequences``), synthetic
geometries (``meshgen``) and the build recipe (``build``).
"""

from . import _native, sequences, meshgen, meshfiles  # noqa: F401
from .api import (  # noqa: F401
    Mesh, KrylovSolver, MRI_parameters, MyDomain, MRI_simulation, PostProcessing, simulate, project_cell_values,
)
from ._native import Context, BtError, PRECISION_FP64, PRECISION_MIXED, solve_multi, adjoint_multi  # noqa: F401


def build(force=False, verbose=False):
    """Compile libbtgpu.so for sm_103a in-tree."""
    from .build import build as _b
    return _b(force=force, verbose=verbose)
