"""GB300-native exact map-folding counting engine.

Lunnon's backtracking DFS over leaves and sym_fold's symmetry-reduced case
counting, as sm_103a kernels behind a C ABI (include/mapfold.h); this package
is the Python mirror of that ABI plus the chunk-sweep driver.
"""
from .api import (  # noqa: F401
    BatchConfig,
    EngineError,
    LunnonBatch,
    LunnonPlan,
    RunStats,
    SymGraph,
    SymPlan,
    count_cases_batched_device,
    count_cases_device,
    gpu_folding,
    lunnon_batch_count,
    pack_case_buffer,
    solve_cases,
    sym_edges,
    sym_fold,
    sym_sort_order,
    sym_workspace_bytes,
)

__version__ = "0.1.0"
