"""GB300 (sm_103a) implementation of Amaru's mechanical hot path, Python host side.

The package mirrors Amaru.jl's user API for solid mechanics (Block/Mesh,
FEModel, MechSolid + LinearElastic/VonMises/DruckerPrager, NodeBC/SurfaceBC/
EdgeBC/BodyC, MechAnalysis, DynAnalysis, ModalAnalysis,
addstage, solve) over the C ABI of
libamaru_gpu.so, where element integration, assembly, the constitutive
update, the loads and the staged Newton loop with its linear solver run.
"""
from ._lib import (AmrError, HEX8, HEX20, LIN2, LIN3, QUAD4, QUAD8, QUAD9, TET4, TET10, TRI3, TRI6,  # noqa: F401
                   SOLVER_AMG, SOLVER_AMG_FP64, SOLVER_FP64, SOLVER_MIXED, lib)
from . import coupled  # noqa: F401
from .args import ArgumentError  # noqa: F401
from .expr import evaluate  # noqa: F401
from .mesh import Block, Mesh  # noqa: F401
from .model import (BatchAnalysis, BodyC, DruckerPrager, DynAnalysis, EdgeBC, ElemBC, FaceBC, FEModel,  # noqa: F401
                    LinearElastic, MechAnalysis, MechContext, MechSolid, ModalAnalysis, NodeBC, SurfaceBC,
                    VonMises)
