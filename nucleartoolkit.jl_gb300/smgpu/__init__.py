"""smgpu — GB300-native valence shell-model eigensolver (NuclearToolkit.jl
`main_sm` path) behind the C ABI of libsmgpu.so."""
from ._lib import FP64, MIXED, MIXED_DF, SmgpuError, library_path, load
from .shellmodel import BatchProblem, MultiSampleProblem, ShellModelProblem, l2_read_bandwidth, main_sm
from .transit import eval_moment, transit_main
from .ec import prep_ec, solve_ec

__all__ = ["FP64", "MIXED", "MIXED_DF", "SmgpuError", "ShellModelProblem", "MultiSampleProblem", "BatchProblem", "main_sm", "l2_read_bandwidth",
           "eval_moment", "transit_main", "prep_ec", "solve_ec", "load", "library_path"]
