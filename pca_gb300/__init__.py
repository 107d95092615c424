"""pca_gb300 -- GB300-native exhaustive superoptimizer for the PCA-16 ISA.

The engine is native (include/pca_gb300.h, pca_gb300/csrc/); this package is
its Python host side: the ctypes mirror of the reference's libpca interface
(`pcalib.PCALib`), the GPU engine wrapper (`pcalib.Engine`) and the seeded
task generators of the benchmark workloads (`taskgen`).
"""
from .pcalib import (PCALib, Engine, EngineError, TaskSpec, SearchCtx, SearchState, Solution,
                     make_task, load_library, OEP_NONE, OEP_EXACT, OEP_EXACT_LIVE)

__all__ = ["PCALib", "Engine", "EngineError", "TaskSpec", "SearchCtx", "SearchState", "Solution",
           "make_task", "load_library", "OEP_NONE", "OEP_EXACT", "OEP_EXACT_LIVE"]
