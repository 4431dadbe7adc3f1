"""sphadjoint_gb300: the forward + hand-written-adjoint WCSPH step of SPHAdjoint
(hanafsky/SPHAdjoint), rebuilt as sm_103a CUDA kernels behind a C ABI
(include/sphadjoint_gb300.h). This package is the Python mirror of the
reference's Julia API over that ABI."""
from .api import (  # noqa: F401
    AdjointWorkspace,
    CellList,
    NeighborList,
    Batch,
    BatchField,
    BatchWorkspace,
    DesignField,
    batch_backward,
    SPHParams,
    State,
    Tape,
    backward,
    TUNED_KERNELS,
    autotune_in_solve,
    backward_seeded,
    capture,
    Graph,
    build,
    build_neighbors,
    group_lanes,
    kinetic_energy_right_half,
    launch_count,
    reset,
    set_group_lanes,
    set_density_form,
    set_launch_overlap,
    set_step_graphs,
    step_graphs,
    step_graph_counts,
    density_form,
    simulate,
    step,
    synchronize,
    target_objective,
    tape_plan,
)
from ._lib import SPHError, CapacityError, ArgumentError, load  # noqa: F401

__version__ = "0.1.0"
