"""seismic_engine — the GB300 (sm_103a) implementation of the hot path of
13262233692/03-seismic-tomography-compute behind the reference's own Python
module name and API (src/cpp/pybind/bindings.cpp:13-301), extended with the
fused GPU shot, RTM, gradient and tomography-solve entry points.

All compute runs in libseismic_gb300.so (CUDA, sm_103a) through its C ABI
(include/seismic_gb300.h); there is no CPU fallback.
"""
from ._lib import SeismicError, load as load_library, lib_path  # noqa: F401
from .wave import (  # noqa: F401
    FaultStats, FaultTolerance, GridParams, HealthStatus, PropagationResult, SolverConfig, StepResult, WaveEquationSolver,
    WaveField, field_layout, rtm_shot, rtm_shot_checkpointed, rtm_shot_host, shot_adjoint, shot_forward,
    shot_forward_host,
)
from .sparse import CSRMatrix, SparseOps, compute_fd_stencil, normal_cg_device, normal_pcg_stencil_device  # noqa: F401
from .fields import check_field_health, clamp_field_safe, repair_field_nan  # noqa: F401
from .config import (  # noqa: F401
    InversionConfig, ModelConfig, TomographyConfig, load_config,
)
from .rtm import RTMConfig, RTMEngine, RTMImageCondition, SliceAxis, SliceSpec  # noqa: F401
from .rays import SampledRays  # noqa: F401
from .terrain import BathymetryPoint, TerrainBoundary, generate_bathymetry  # noqa: F401
from .slices import (  # noqa: F401
    CapturedSlice, MmapSnapshotWriter, MmapStats, SliceStream, capture_slice_frames, deserialize_slice,
)
from . import workloads  # noqa: F401

__version__ = "1.2.0+gb300"
