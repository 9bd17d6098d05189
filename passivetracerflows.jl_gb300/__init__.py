"""GB300-native TracerAdvectionDiffusion time step with the PassiveTracerFlows.jl API.

``import`` name: the directory is ``passivetracerflows.jl_gb300`` (mirroring the
Julia package name), so it is loaded under the module name ``ptf_gb300`` by
:func:`__graft_entry__.load_package` (or any ``importlib`` spec loader).

Everything numerical runs in ``libptf.so`` (hand-written sm_103a CUDA, C ABI in
``include/ptf.h``); this package holds the host-side mirror of the reference's
user API, as PassiveTracerFlows.jl re-exports ``TracerAdvectionDiffusion``
(``src/PassiveTracerFlows.jl:1-13``).
"""
from . import traceradvectiondiffusion as TracerAdvectionDiffusion
from .traceradvectiondiffusion import (CPU, GPU, Problem, OneDAdvectingFlow, ThreeDAdvectingFlow,
                                       TwoDAdvectingFlow, ThreeDGrid, TwoDGrid, OneDGrid, gridpoints, noflow, set_c,
                                       stepforward, updatevars, MultiLayerQGFlow, MultiLayerTracerProblem)
from ._lib import LIB_PATH, load as load_library
from .batched import BatchedProblem, Server, SolveSpec
from .output import Output, get_concentration, get_sol, jldopen, saveoutput, saveproblem

__all__ = ["TracerAdvectionDiffusion", "CPU", "GPU", "Problem", "OneDAdvectingFlow", "TwoDAdvectingFlow",
           "ThreeDAdvectingFlow", "OneDGrid", "TwoDGrid", "ThreeDGrid", "gridpoints", "noflow", "set_c", "stepforward",
           "updatevars", "LIB_PATH", "load_library", "BatchedProblem", "Server", "SolveSpec", "MultiLayerQGFlow",
           "MultiLayerTracerProblem", "Output", "saveproblem", "saveoutput", "jldopen", "get_sol",
           "get_concentration"]
