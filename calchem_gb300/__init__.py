"""calchem_gb300: CalChem's DFT exchange-correlation grid quadrature on one GB300 (sm_103a).

The compute lives in the in-tree native library ``_lib/libcalchem_xc.so`` (C ABI
in ``include/calchem_xc.h``); this package is the host-side mirror of CalChem's
Rust call surface (``RksVxcEngine``, ``UksVxcEngine``, ``MolecularGrid``,
``BasisSet``, ``XcFunctional``).
"""

from .basis import BasisSet
from .grid import GridLevel, MolecularGrid
from .molecule import ANGSTROM_TO_BOHR, Atom, Molecule
from . import autotune
from .vxc import (FP64, MIXED, FxcKernel, GpuVxcGrid, RksVxcEngine, UksVxcEngine, VxcGroup, eval_closed_shell_gpu,
                  evaluate_vxc_rks, evaluate_vxc_uks, is_cuda_available, plan_points, xc_nuclear_gradient,
                  xc_nuclear_gradient_with_gpu)
from .xc import XcFunctional

__all__ = [
    "ANGSTROM_TO_BOHR", "Atom", "Molecule", "BasisSet", "GridLevel", "MolecularGrid", "XcFunctional",
    "RksVxcEngine", "UksVxcEngine", "VxcGroup", "FxcKernel", "GpuVxcGrid", "evaluate_vxc_rks", "evaluate_vxc_uks", "is_cuda_available",
    "xc_nuclear_gradient", "xc_nuclear_gradient_with_gpu", "eval_closed_shell_gpu", "plan_points", "FP64", "MIXED",
]
