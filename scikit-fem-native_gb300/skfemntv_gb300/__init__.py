"""skfemntv_gb300 -- GB300-native finite-element assembly, a drop-in for the
matrix-assembly path of scikit-fem-native (``skfemntv``).

Same public names for the hot path: ``MeshTet``, ``MeshTet2``,
``ElementTetP1``, ``ElementTetP2``, ``ElementVector``, ``Basis``,
``BilinearForm``, ``LinearForm``, ``asm`` (+ ``dot``, ``ddot``, ``grad``,
``mul``, ``div``, ``sym_grad``), ``AffineTetN1Basis``, ``TetN1Assembler``,
the runtime controls and the memory preflight.  Assembly runs in hand-written
CUDA kernels for sm_103a reached through the C ABI in
``include/skfem_gb300.h``.
"""
from .adjoint import P1Energy
from .assembly import (AssemblyGraph, LinearFormDiagnostics, NativeBilinearForm, NativeCrossBilinearForm,
                       NativeLinearForm)
from .basis import Basis, GeometryDiagnostics
from .element import ElementTetP1, ElementTetP2, ElementVector
from .errors import UnsupportedNativeForm
from .forms import BilinearForm, LinearForm, asm, ddot, div, dot, grad, inner, mul, sym_grad
from .hyperelastic import EnergySurrogate, NeoHookean
from .hcurl import (AffineTetN1Basis, HcurlTetGeometryDiagnostics, OrientedEdgeDofMap, OrientedEdgeTopology,
                    TetN1Assembler, TetN1LinearAssembler, build_oriented_edge_dof_map, build_oriented_edge_topology,
                    estimate_tet_n1_assembly_memory)
from .mesh import MeshTet, MeshTet2
from .preflight import (AssemblyMemoryBudgetError, AssemblyMemoryEstimate, enforce_memory_budget,
                        estimate_bilinear_memory, format_bytes)
from .runtime import (BACKEND, CAPABILITIES, available_num_threads, get_num_threads, has_capability,
                      set_num_threads, thread_limit)

__version__ = "0.1.0"

__all__ = [
    "AssemblyGraph", "LinearFormDiagnostics", "NativeBilinearForm", "NativeCrossBilinearForm", "NativeLinearForm",
    "AffineTetN1Basis", "AssemblyMemoryBudgetError", "AssemblyMemoryEstimate", "BACKEND", "Basis",
    "BilinearForm", "CAPABILITIES", "ElementTetP1", "ElementTetP2", "ElementVector", "GeometryDiagnostics",
    "HcurlTetGeometryDiagnostics", "LinearForm", "OrientedEdgeDofMap", "OrientedEdgeTopology",
    "build_oriented_edge_dof_map", "build_oriented_edge_topology", "EnergySurrogate", "MeshTet", "MeshTet2", "NeoHookean", "P1Energy", "TetN1Assembler", "TetN1LinearAssembler",
    "UnsupportedNativeForm", "asm", "available_num_threads", "ddot", "div", "dot", "enforce_memory_budget",
    "estimate_bilinear_memory", "estimate_tet_n1_assembly_memory", "format_bytes", "get_num_threads",
    "grad", "has_capability", "inner", "mul", "set_num_threads", "sym_grad", "thread_limit",
]
