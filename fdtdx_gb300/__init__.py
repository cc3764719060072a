"""GB300-native (sm_103a) FDTD time-stepping with fdtdx's API.

The public names mirror ``fdtdx`` (``run_fdtd``, ``reversible_fdtd``,
``checkpointed_fdtd``, ``place_objects``, ``apply_params``, ``ArrayContainer``,
``ObjectContainer``, ``SimulationConfig``, the objects).  The time loop runs in
``libfdtd_gb300.so`` (C ABI in ``include/fdtd_gb300.h``); there is no CPU path.
"""

from fdtdx_gb300.config import (
    DtypeConversion,
    GradientConfig,
    LinearReconstructEveryK,
    Recorder,
    SimulationConfig,
    UniformGrid,
)
from fdtdx_gb300.constants import wavelength_to_period
from fdtdx_gb300.container import ArrayContainer, FieldState, ObjectContainer, ParameterContainer, RecordingState
from fdtdx_gb300.dispersion import DispersionModel, DrudePole, LorentzPole
from fdtdx_gb300.core import (
    GaussianPulseProfile,
    GaussianWindow,
    OnOffSwitch,
    SingleFrequencyProfile,
    TukeyWindow,
    WaveCharacter,
)
from fdtdx_gb300.adjoint import reversible_fdtd
from fdtdx_gb300.batch import SimulationBatch, run_fdtd_batch
from fdtdx_gb300.fdtd import checkpointed_fdtd, run_fdtd
from fdtdx_gb300.initialization import apply_params, place_objects
from fdtdx_gb300.objects import (
    BlochBoundary,
    BoundaryConfig,
    Device,
    EnergyDetector,
    FieldDetector,
    GaussianPlaneSource,
    Material,
    PerfectElectricConductor,
    PerfectlyMatchedLayer,
    PerfectMagneticConductor,
    PeriodicBoundary,
    PhasorDetector,
    PhasorPoyntingFluxDetector,
    PointDipoleSource,
    PoyntingFluxDetector,
    SimulationVolume,
    UniformMaterialObject,
    UniformPlaneSource,
    boundary_objects_from_config,
)


__all__ = [
    "ArrayContainer",
    "BlochBoundary",
    "BoundaryConfig",
    "Device",
    "DispersionModel",
    "DrudePole",
    "DtypeConversion",
    "LinearReconstructEveryK",
    "LorentzPole",
    "EnergyDetector",
    "FieldDetector",
    "FieldState",
    "GaussianPlaneSource",
    "GaussianPulseProfile",
    "GaussianWindow",
    "GradientConfig",
    "Material",
    "ObjectContainer",
    "OnOffSwitch",
    "ParameterContainer",
    "PerfectElectricConductor",
    "PerfectlyMatchedLayer",
    "PerfectMagneticConductor",
    "PeriodicBoundary",
    "PhasorDetector",
    "PhasorPoyntingFluxDetector",
    "PointDipoleSource",
    "PoyntingFluxDetector",
    "Recorder",
    "RecordingState",
    "SimulationConfig",
    "SimulationVolume",
    "SingleFrequencyProfile",
    "TukeyWindow",
    "UniformGrid",
    "UniformMaterialObject",
    "UniformPlaneSource",
    "WaveCharacter",
    "apply_params",
    "boundary_objects_from_config",
    "checkpointed_fdtd",
    "place_objects",
    "reversible_fdtd",
    "run_fdtd",
    "run_fdtd_batch",
    "SimulationBatch",
    "wavelength_to_period",
]
