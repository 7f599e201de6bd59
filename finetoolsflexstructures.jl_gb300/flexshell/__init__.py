"""flexshell: GB300-native element assembly for the shell hot path of
FinEtoolsFlexStructures.jl (T3FF, Q4RS and their layered variants), the
deterministic CSR assembly and the explicit central-difference step.

The compute path is libflexshell.so (CUDA, sm_103a) behind the C ABI of
include/flexshell.h; this package is its host-side mirror of the reference
interface.
"""
from . import _abi, mesh, materials
from ._abi import FS_FP64, FS_MIXED, FS_MIXED_COMP
from .femm import (CSysCartesian, CSysCylindrical, CSysSpherical,
                   FEMMShellQ4RS, FEMMShellQ4RSComp, FEMMShellT3FF, FEMMShellT3FFComp,
                   NodalField, SysmatAssemblerFFBlock, SysmatAssemblerSparse,
                   SysmatAssemblerSparseCSRSymm, SysmatAssemblerSparseDiag,
                   SysmatAssemblerSparseSymm, ShellBatch)
from .beam import FEMMCorotBeam
from .eigen import ShiftInvert, eigs
from .explicit import CentralDifference, cd_loop
from .loads import (FEMMBase, ForceIntensity, GaussRule, IntegDomain, SysvecAssembler,
                    SysvecAssemblerFBlock, TriRule, distribloads)
from ._lib import Context, FlexShellError, laminate
