"""Simulation objects: volume, materials, boundaries, sources and detectors.

Each class keeps the user-facing field names of its fdtdx counterpart so that a
scene written for fdtdx reads the same here:

* ``SimulationVolume``, ``UniformMaterialObject``   fdtdx/objects/static_material/static.py
* ``PerfectlyMatchedLayer``                         fdtdx/objects/boundaries/perfectly_matched_layer.py:12-275
* ``PerfectElectricConductor`` / ``PerfectMagneticConductor``  fdtdx/objects/boundaries/pec.py, pmc.py
* ``PeriodicBoundary``, ``BlochBoundary``           fdtdx/objects/boundaries/bloch.py (the kernels run
  a zero Bloch vector, i.e. a periodic boundary; a non-zero one needs complex fields)
* ``PointDipoleSource`` (axis-aligned or tilted)    fdtdx/objects/sources/dipole.py:51-277
* ``GaussianPlaneSource`` / ``UniformPlaneSource``  fdtdx/objects/sources/linear_polarization.py:414-482
* ``FieldDetector``, ``PhasorDetector``, ``PoyntingFluxDetector``,
  ``PhasorPoyntingFluxDetector``, ``EnergyDetector``  fdtdx/objects/detectors/*.py

Placement is explicit: every object carries a ``grid_slice_tuple``
``((x0, x1), (y0, y1), (z0, z1))`` in cells (the reference's constraint solver is
host-side setup and is not part of the time-stepping path).  Derived per-object
data that the kernels need (PML coefficient vectors, plane-source incident
profiles and Yee time offsets, per-step tables) is computed on the host in
``fdtdx_gb300.engine``.
"""

from __future__ import annotations

import cmath
import math
from dataclasses import dataclass, field
from typing import Literal, Sequence

import numpy as np

from fdtdx_gb300 import constants
from fdtdx_gb300.core import (
    GaussianPulseProfile,
    OnOffSwitch,
    SingleFrequencyProfile,
    TemporalProfile,
    TemporalWindow,
    WaveCharacter,
)

SliceTuple3D = tuple[tuple[int, int], tuple[int, int], tuple[int, int]]
COMPONENTS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def _normalize_slice_tuple(st) -> SliceTuple3D:
    out = tuple((int(a), int(b)) for a, b in st)
    if len(out) != 3 or any(b <= a for a, b in out):
        raise ValueError(f"invalid grid slice {st}")
    return out  # type: ignore[return-value]


@dataclass(eq=False)
class SimulationObject:
    """Base object: a name and a placed grid slice."""

    name: str | None = None
    grid_slice_tuple: SliceTuple3D | None = None

    def place_on_grid(self, grid_slice_tuple, config=None, key=None):
        del config, key
        self.grid_slice_tuple = _normalize_slice_tuple(grid_slice_tuple)
        return self

    @property
    def grid_slice(self) -> tuple[slice, slice, slice]:
        assert self.grid_slice_tuple is not None, f"object {self.name} is not placed"
        return tuple(slice(a, b) for a, b in self.grid_slice_tuple)  # type: ignore[return-value]

    @property
    def grid_shape(self) -> tuple[int, int, int]:
        assert self.grid_slice_tuple is not None, f"object {self.name} is not placed"
        return tuple(b - a for a, b in self.grid_slice_tuple)  # type: ignore[return-value]


@dataclass(eq=False)
class SimulationVolume(SimulationObject):
    """The whole grid.  ``grid_shape`` is given in cells."""

    shape: tuple[int, int, int] = (1, 1, 1)
    material: "Material | None" = None

    def __post_init__(self):
        self.grid_slice_tuple = tuple((0, int(n)) for n in self.shape)  # type: ignore[assignment]
        if self.name is None:
            self.name = "volume"


def _to9(v) -> tuple[float, ...]:
    """Scalar, 3-tuple (diagonal) or 9-tuple material value -> 9-tuple, fdtdx/materials.py convention."""
    if isinstance(v, (int, float)):
        return (float(v), 0.0, 0.0, 0.0, float(v), 0.0, 0.0, 0.0, float(v))
    v = tuple(float(x) for x in v)
    if len(v) == 3:
        return (v[0], 0.0, 0.0, 0.0, v[1], 0.0, 0.0, 0.0, v[2])
    if len(v) == 9:
        return v
    raise ValueError(f"invalid material tensor {v}")


@dataclass(frozen=True)
class Material:
    """Relative permittivity/permeability and conductivities (scalar, diagonal 3-tuple or 3x3 9-tuple)."""

    permittivity: tuple[float, ...] | float = 1.0
    permeability: tuple[float, ...] | float = 1.0
    electric_conductivity: tuple[float, ...] | float = 0.0
    magnetic_conductivity: tuple[float, ...] | float = 0.0
    #: optional ``DispersionModel``; ``permittivity`` is then eps_infinity (fdtdx/materials.py:138-142)
    dispersion: object | None = None

    def __post_init__(self):
        for f in ("permittivity", "permeability", "electric_conductivity", "magnetic_conductivity"):
            object.__setattr__(self, f, _to9(getattr(self, f)))

    @staticmethod
    def _iso(t) -> bool:
        return t[1:4] == (0.0, 0.0, 0.0) and t[5:8] == (0.0, 0.0, 0.0) and t[0] == t[4] == t[8]

    @staticmethod
    def _diag(t) -> bool:
        return t[1:4] == (0.0, 0.0, 0.0) and t[5:8] == (0.0, 0.0, 0.0)

    @property
    def is_isotropic_permittivity(self) -> bool:
        return self._iso(self.permittivity)

    @property
    def is_diagonal_permittivity(self) -> bool:
        return self._diag(self.permittivity)

    @property
    def is_isotropic_permeability(self) -> bool:
        return self._iso(self.permeability)

    @property
    def is_diagonal_permeability(self) -> bool:
        return self._diag(self.permeability)

    @property
    def is_dispersive(self) -> bool:
        return self.dispersion is not None and self.dispersion.num_poles > 0

    @property
    def is_magnetic(self) -> bool:
        return self.permeability != _to9(1.0)

    @property
    def is_electrically_conductive(self) -> bool:
        return any(x != 0.0 for x in self.electric_conductivity)  # type: ignore[union-attr]

    @property
    def is_magnetically_conductive(self) -> bool:
        return any(x != 0.0 for x in self.magnetic_conductivity)  # type: ignore[union-attr]


@dataclass(eq=False)
class UniformMaterialObject(SimulationObject):
    """An axis-aligned box of one material.  Painted in ``placement_order`` (stable)."""

    material: Material = field(default_factory=Material)
    placement_order: int = 0


@dataclass(eq=False)
class Device(SimulationObject):
    """Design region whose per-voxel parameters in [0, 1] map linearly between two permittivities.

    Restates the continuous branch of ``apply_params`` (fdtdx/fdtd/initialization.py:404-417):
    eps = eps_lo + p * (eps_hi - eps_lo), written as inv_eps = 1 / eps.
    """

    permittivity_low: float = 1.0
    permittivity_high: float = 1.0
    placement_order: int = 1_000_000


# --------------------------------------------------------------------------------------------
# boundaries
# --------------------------------------------------------------------------------------------


@dataclass(eq=False)
class BaseBoundary(SimulationObject):
    axis: int = 0
    direction: Literal["+", "-"] = "-"

    @property
    def descriptive_name(self) -> str:
        return f"{'min' if self.direction == '-' else 'max'}_{'xyz'[self.axis]}"

    @property
    def uses_wrap_padding(self) -> bool:
        return False

    def interface_slice_tuple(self) -> SliceTuple3D:
        """The slab's innermost cell layer (fdtdx/objects/boundaries/boundary.py:126-132)."""
        st = list(self.grid_slice_tuple)  # type: ignore[arg-type]
        lo, hi = st[self.axis]
        st[self.axis] = (lo, lo + 1) if self.direction == "+" else (hi - 1, hi)
        return tuple(st)  # type: ignore[return-value]


@dataclass(eq=False)
class PerfectlyMatchedLayer(BaseBoundary):
    """CPML slab.  ``None`` parameters take the reference defaults (perfectly_matched_layer.py:69-110)."""

    alpha_start: float | None = None
    alpha_end: float | None = None
    alpha_order: float | None = None
    kappa_start: float | None = None
    kappa_end: float | None = None
    kappa_order: float | None = None
    sigma_start: float | None = None
    sigma_end: float | None = None
    sigma_order: float | None = None

    def __post_init__(self):
        if self.alpha_start is None:
            self.alpha_start = 0.01 * 2 * math.pi * constants.c / 1.55e-6 * constants.eps0
        if self.alpha_end is None:
            self.alpha_end = 0.0
        if self.alpha_order is None:
            self.alpha_order = 1.0
        if self.kappa_start is None:
            self.kappa_start = 1.0
        if self.kappa_end is None:
            self.kappa_end = 1.0
        if self.kappa_order is None:
            self.kappa_order = 3.0
        if self.sigma_start is None:
            self.sigma_start = 0.0
        if self.sigma_order is None:
            self.sigma_order = 3.0

    @property
    def thickness(self) -> int:
        return self.grid_shape[self.axis]

    @property
    def kappa_is_one(self) -> bool:
        return self.kappa_start == 1.0 and self.kappa_end == 1.0

    def coefficients(self, spacing: float, dt: float) -> dict[str, np.ndarray]:
        """1-D CPML coefficient vectors along the slab axis (index 0 = lowest grid index).

        Restates ``place_on_grid`` and ``_compute_pml_profile``
        (perfectly_matched_layer.py:97-136, 231-275): graded profiles at the E and
        H depths, b = exp(-dt/eps0 (sigma/kappa + alpha)), a = (b - 1) sigma /
        (sigma + alpha kappa) / kappa with NaN -> 0.  Evaluated in float64 and
        returned as float32 (the reference evaluates in the config dtype).
        """
        L = self.thickness
        sigma_end = self.sigma_end
        if sigma_end is None:
            sigma_end = -(self.sigma_order + 1) * math.log(1e-6) / (2 * constants.eta0 * L * spacing)
        if self.direction == "-":
            dE = np.arange(L - 1, -1, -1, dtype=np.float64)
            dH = np.append(np.arange(L - 1.5, -0.5, -1, dtype=np.float64), 0.0)
        else:
            dE = np.insert(np.arange(0.5, L - 0.5, 1, dtype=np.float64), 0, 0.0)
            dH = np.arange(0, L, 1, dtype=np.float64)

        def prof(v0, v1, order, d):
            return v0 + (v1 - v0) * np.power(d / L, order)

        out = {}
        for tag, d in (("E", dE), ("H", dH)):
            sigma = prof(self.sigma_start, sigma_end, self.sigma_order, d)
            kappa = prof(self.kappa_start, self.kappa_end, self.kappa_order, d)
            alpha = prof(self.alpha_start, self.alpha_end, self.alpha_order, d)
            b = np.expm1(-dt / constants.eps0 * (sigma / kappa + alpha)) + 1.0
            with np.errstate(invalid="ignore", divide="ignore"):
                a = np.nan_to_num((b - 1.0) * sigma / (sigma + alpha * kappa) / kappa, nan=0.0)
            out[f"a_{tag}"] = a.astype(np.float32)
            out[f"b_{tag}"] = b.astype(np.float32)
            out[f"inv_kappa_{tag}"] = (1.0 / kappa).astype(np.float32)
        out["sigma_end"] = np.float64(sigma_end)
        return out


@dataclass(eq=False)
class PerfectElectricConductor(BaseBoundary):
    """Zeroes the tangential E components on the face layer after every E update."""

    @property
    def tangential_components(self) -> tuple[int, int]:
        return ((1, 2), (0, 2), (0, 1))[self.axis]


@dataclass(eq=False)
class PerfectMagneticConductor(BaseBoundary):
    """Zeroes the tangential H components on the face layer after every H update."""

    @property
    def tangential_components(self) -> tuple[int, int]:
        return ((1, 2), (0, 2), (0, 1))[self.axis]


@dataclass(eq=False)
class PeriodicBoundary(BaseBoundary):
    """Wrap halo along the axis (a Bloch boundary with zero Bloch vector)."""

    @property
    def uses_wrap_padding(self) -> bool:
        return True

    @property
    def needs_complex_fields(self) -> bool:
        return False


@dataclass(eq=False)
class BlochBoundary(PeriodicBoundary):
    """Wrap halo whose ghost layers carry the Bloch phase F(x + L) = F(x) exp(i k L)
    (fdtdx/objects/boundaries/bloch.py:13-155): the '+' ghost layer is multiplied by
    exp(i k L), the '-' one by its conjugate, k the vector's component along the axis.  A zero
    component is a plain periodic boundary; a non-zero one needs complex fields."""

    bloch_vector: tuple[float, float, float] = (0.0, 0.0, 0.0)

    @property
    def needs_complex_fields(self) -> bool:
        return self.bloch_vector[self.axis] != 0.0

    def get_bloch_phase(self, volume_shape, resolution: float) -> complex:
        """exp(i k L), L = the volume's extent along the axis (uniform grid)."""
        return cmath.exp(1j * self.bloch_vector[self.axis] * volume_shape[self.axis] * resolution)


@dataclass
class BoundaryConfig:
    """Per-face boundary types and PML thicknesses (fdtdx/objects/boundaries/initialization.py:16-160)."""

    boundary_type_minx: str = "pml"
    boundary_type_maxx: str = "pml"
    boundary_type_miny: str = "pml"
    boundary_type_maxy: str = "pml"
    boundary_type_minz: str = "pml"
    boundary_type_maxz: str = "pml"
    thickness_grid_minx: int = 10
    thickness_grid_maxx: int = 10
    thickness_grid_miny: int = 10
    thickness_grid_maxy: int = 10
    thickness_grid_minz: int = 10
    thickness_grid_maxz: int = 10
    pml_kwargs: dict = field(default_factory=dict)
    bloch_vector: tuple[float, float, float] = (0.0, 0.0, 0.0)

    @classmethod
    def from_uniform_bound(cls, thickness: int = 10, boundary_type: str = "pml", override_types: dict | None = None,
                           bloch_vector: tuple[float, float, float] = (0.0, 0.0, 0.0), **pml_kwargs) -> "BoundaryConfig":
        """One type and thickness on every face, ``override_types`` ({"min_x": "bloch", ...})
        replacing the type of single faces (initialization.py:444-553)."""
        override_types = {} if override_types is None else override_types
        kw = {}
        for side in ("minx", "maxx", "miny", "maxy", "minz", "maxz"):
            kw[f"boundary_type_{side}"] = override_types.get(f"{side[:3]}_{side[3]}", boundary_type)
            kw[f"thickness_grid_{side}"] = thickness
        return cls(**kw, pml_kwargs=dict(pml_kwargs), bloch_vector=tuple(float(k) for k in bloch_vector))


def boundary_objects_from_config(config: BoundaryConfig, volume: SimulationVolume) -> dict[str, BaseBoundary]:
    """Create and place the six boundary objects on the volume faces (initialization.py:554-663)."""
    out: dict[str, BaseBoundary] = {}
    shape = volume.grid_shape
    for kind in ("min_x", "max_x", "min_y", "max_y", "min_z", "max_z"):
        side, ax = kind.split("_")
        axis = "xyz".index(ax)
        direction = "-" if side == "min" else "+"
        btype = getattr(config, f"boundary_type_{side}{ax}")
        thick = getattr(config, f"thickness_grid_{side}{ax}") if btype == "pml" else 1
        st = [(0, n) for n in shape]
        st[axis] = (0, thick) if direction == "-" else (shape[axis] - thick, shape[axis])
        if btype == "pml":
            obj: BaseBoundary = PerfectlyMatchedLayer(name=kind, axis=axis, direction=direction, **config.pml_kwargs)
        elif btype == "periodic":
            obj = PeriodicBoundary(name=kind, axis=axis, direction=direction)
        elif btype == "bloch":
            obj = BlochBoundary(name=kind, axis=axis, direction=direction, bloch_vector=config.bloch_vector)
        elif btype == "pec":
            obj = PerfectElectricConductor(name=kind, axis=axis, direction=direction)
        elif btype == "pmc":
            obj = PerfectMagneticConductor(name=kind, axis=axis, direction=direction)
        else:
            raise ValueError(f"Unknown boundary type '{btype}' for '{kind}'.")
        obj.place_on_grid(tuple(st))
        out[kind] = obj
    return out


# --------------------------------------------------------------------------------------------
# sources
# --------------------------------------------------------------------------------------------


def tilt_vector(vector, azimuth: float, elevation: float, axes: tuple[int, int, int]) -> np.ndarray:
    """Tilt a vector by azimuth / elevation (radians) in the frame ``axes`` = (horizontal,
    vertical, propagation) (fdtdx/core/linalg.py:90-160).

    The frame's tilted rows are u = (cos az, 0, sin az) (the horizontal axis turned about the
    vertical one), v = (0, cos el, sin el) (the vertical axis turned about the horizontal one)
    and w = u x v / |u x v|.  The vector's frame coordinates go through those rows and back to
    the global axes, and the result is rescaled to the input's norm: u and v are not orthogonal
    when both angles are set, so the map is not a rotation and the rescaling is part of it.
    """
    vec = np.asarray(vector, dtype=np.float64)
    frame = np.eye(3)[list(axes)]  # rows: global -> frame coordinates
    ca, sa, ce, se = math.cos(azimuth), math.sin(azimuth), math.cos(elevation), math.sin(elevation)
    u = np.array([ca, 0.0, sa])
    v = np.array([0.0, ce, se])
    w = np.cross(u, v)
    w = w / np.linalg.norm(w)
    out = frame.T @ (np.stack([u, v, w]) @ (frame @ vec))
    return out / np.linalg.norm(out) * np.linalg.norm(vec)


@dataclass(eq=False)
class Source(SimulationObject):
    wave_character: WaveCharacter = field(default_factory=lambda: WaveCharacter(wavelength=1.55e-6))
    temporal_profile: TemporalProfile = field(default_factory=SingleFrequencyProfile)
    static_amplitude_factor: float = 1.0
    switch: OnOffSwitch = field(default_factory=OnOffSwitch)


@dataclass(eq=False)
class PointDipoleSource(Source):
    """Soft point dipole: E[i] += -c * amp * s(t) * inv_eps[i] * p[i] at one cell for the unit
    orientation p (dipole.py:195-277); axis-aligned (p = e_polarization) unless tilted by
    ``azimuth_angle`` / ``elevation_angle`` (degrees)."""

    polarization: int = 2
    azimuth_angle: float = 0.0
    elevation_angle: float = 0.0
    source_type: Literal["electric", "magnetic"] = "electric"
    amplitude: float = 1.0

    def __post_init__(self):
        if self.source_type not in ("electric", "magnetic"):
            raise ValueError(f"source_type must be electric or magnetic, got {self.source_type}")
        if self.polarization not in (0, 1, 2):
            raise ValueError(f"polarization must be 0, 1, or 2, got {self.polarization}")

    @property
    def is_tilted(self) -> bool:
        return self.azimuth_angle != 0.0 or self.elevation_angle != 0.0

    @property
    def orientation(self) -> np.ndarray:
        """Unit orientation: e_polarization tilted in the frame (p+1, p+2, p) (dipole.py:130-148)."""
        base = np.zeros(3)
        base[self.polarization] = 1.0
        if not self.is_tilted:
            return base
        p = self.polarization
        return tilt_vector(base, math.radians(self.azimuth_angle), math.radians(self.elevation_angle),
                           ((p + 1) % 3, (p + 2) % 3, p))


@dataclass(eq=False)
class LinearlyPolarizedPlaneSource(Source):
    """TFSF plane source: injection on a single plane normal to the propagation axis (tfsf.py:413-806)."""

    direction: Literal["+", "-"] = "+"
    fixed_E_polarization_vector: tuple[float, float, float] | None = None
    fixed_H_polarization_vector: tuple[float, float, float] | None = None
    normalize_by_energy: bool = True
    azimuth_angle: float = 0.0
    elevation_angle: float = 0.0
    max_angle_random_offset: float = 0.0
    max_vertical_offset: float = 0.0
    max_horizontal_offset: float = 0.0

    def __post_init__(self):
        if self.max_angle_random_offset:
            raise NotImplementedError("random plane-source angle offsets are not supported")
        if self.max_vertical_offset or self.max_horizontal_offset:
            raise NotImplementedError("random plane-source offsets are not supported")

    @property
    def propagation_axis(self) -> int:
        return self.grid_shape.index(1)

    @property
    def horizontal_axis(self) -> int:
        return (self.propagation_axis + 1) % 3

    @property
    def vertical_axis(self) -> int:
        return (self.propagation_axis + 2) % 3

    @property
    def is_tilted(self) -> bool:
        return self.azimuth_angle != 0.0 or self.elevation_angle != 0.0

    def polarization_vectors(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """E/H polarization unit vectors and wave vector (fdtdx/core/misc.py:471-553, core/linalg.py:7-47),
        all three tilted by the azimuth / elevation angles in the frame (horizontal, vertical,
        propagation) when the source is tilted."""
        k = np.zeros(3)
        k[self.propagation_axis] = 1.0 if self.direction == "+" else -1.0
        e = None if self.fixed_E_polarization_vector is None else np.asarray(self.fixed_E_polarization_vector, float)
        h = None if self.fixed_H_polarization_vector is None else np.asarray(self.fixed_H_polarization_vector, float)
        if h is not None:
            h = h / np.linalg.norm(h)
        if e is not None:
            e = e / np.linalg.norm(e)
        if e is None:
            if h is None:
                raise Exception("Need to specify either E or H polarization")
            e = np.cross(h, k)
        if h is None:
            h = np.cross(k, e)
        if self.is_tilted:
            axes = (self.horizontal_axis, self.vertical_axis, self.propagation_axis)
            az, el = math.radians(self.azimuth_angle), math.radians(self.elevation_angle)
            e, h, k = (tilt_vector(x, az, el, axes) for x in (e, h, k))
        return e, h, k

    def amplitude_raw_hv(self, spacing: float) -> np.ndarray:
        raise NotImplementedError


@dataclass(eq=False)
class GaussianPlaneSource(LinearlyPolarizedPlaneSource):
    """Truncated Gaussian spot of ``radius`` (m) and relative ``std`` (linear_polarization.py:414-468)."""

    radius: float = 1e-6
    std: float = 1 / 3

    def amplitude_raw_hv(self, spacing: float) -> np.ndarray:
        W = self.grid_shape[self.horizontal_axis]
        H = self.grid_shape[self.vertical_axis]
        center = np.array([0.5 * (W - 1), 0.5 * (H - 1)])
        r = self.radius / spacing
        w, h = np.meshgrid(np.arange(W), np.arange(H), indexing="ij")
        d2 = ((w - center[0]) / r) ** 2 + ((h - center[1]) / r) ** 2
        prof = np.where(d2 < 1, np.exp(-0.5 * d2 / self.std**2), 0.0)
        return prof / prof.sum()


@dataclass(eq=False)
class UniformPlaneSource(LinearlyPolarizedPlaneSource):
    """Constant amplitude over the plane (linear_polarization.py:471-482)."""

    amplitude: float = 1.0

    def amplitude_raw_hv(self, spacing: float) -> np.ndarray:
        return self.amplitude * np.ones(
            (self.grid_shape[self.horizontal_axis], self.grid_shape[self.vertical_axis]), dtype=np.float64
        )


# --------------------------------------------------------------------------------------------
# detectors
# --------------------------------------------------------------------------------------------


@dataclass(eq=False)
class Detector(SimulationObject):
    dtype: object = None
    exact_interpolation: bool = True
    inverse: bool = False
    switch: OnOffSwitch = field(default_factory=OnOffSwitch)
    plot: bool = False

    def on_list(self, config) -> list[bool]:
        return self.switch.calculate_on_list(config.time_steps_total, config.time_step_duration)

    def num_time_steps_recorded(self, config) -> int:
        return int(sum(self.on_list(config)))

    @property
    def needs_E(self) -> bool:
        return any(c.startswith("E") for c in self.recorded_components)

    @property
    def needs_H(self) -> bool:
        return any(c.startswith("H") for c in self.recorded_components)

    @property
    def recorded_components(self) -> tuple[str, ...]:
        return COMPONENTS


@dataclass(eq=False)
class FieldDetector(Detector):
    """Time-domain field samples: state["fields"][t_on] = EH (field.py:10-63)."""

    reduce_volume: bool = False
    components: Sequence[str] = COMPONENTS

    @property
    def recorded_components(self) -> tuple[str, ...]:
        return tuple(c for c in COMPONENTS if c in self.components)


@dataclass(eq=False)
class EnergyDetector(Detector):
    """Electromagnetic energy density 0.5 (eps |E|^2 + mu |H|^2) per cell or volume sum (energy.py)."""

    reduce_volume: bool = False
    as_slices: bool = False

    def __post_init__(self):
        if self.as_slices:
            raise NotImplementedError("EnergyDetector(as_slices=True) is not supported")


@dataclass(eq=False)
class PhasorDetector(Detector):
    """Running DFT of the co-located fields at the given wave characters (phasor.py:20-235)."""

    wave_characters: Sequence[WaveCharacter] = field(default_factory=tuple)
    reduce_volume: bool = False
    components: Sequence[str] = COMPONENTS
    scaling_mode: Literal["continuous", "pulse"] = "continuous"
    dft_subsample: int | Literal["auto"] = 1
    apodization: TemporalWindow | None = None

    def __post_init__(self):
        if self.apodization is not None and not isinstance(self.apodization, TemporalWindow):
            raise Exception(f"apodization must be a TemporalWindow, got {type(self.apodization).__name__}. "
                            "Source temporal profiles are not valid windows.")

    @property
    def recorded_components(self) -> tuple[str, ...]:
        return tuple(c for c in COMPONENTS if c in self.components)

    def resolve_dft_stride(self, config) -> int:
        sub = self.dft_subsample
        if isinstance(sub, str):
            if sub != "auto":
                raise Exception(f"Invalid dft_subsample: {sub!r}")
            dt = float(config.time_step_duration)
            f_max = max((abs(float(wc.get_frequency())) for wc in self.wave_characters), default=0.0)
            if f_max <= 0.0 or dt <= 0.0:
                return 1
            return max(1, math.floor(1.0 / (12 * f_max * dt)))
        return max(1, int(sub))

    def on_list(self, config) -> list[bool]:
        base = self.switch.calculate_on_list(config.time_steps_total, config.time_step_duration)
        stride = self.resolve_dft_stride(config)
        if stride <= 1:
            return base
        active = [t for t, on in enumerate(base) if on]
        kept = [False] * len(base)
        for t in active[::stride]:
            kept[t] = True
        return kept


@dataclass(eq=False)
class PoyntingFluxDetector(Detector):
    """Instantaneous Poynting flux through a plane (poynting_flux.py:74-195)."""

    direction: Literal["+", "-"] = "+"
    reduce_volume: bool = True
    fixed_propagation_axis: int | None = None
    keep_all_components: bool = False

    @property
    def propagation_axis(self) -> int:
        if self.fixed_propagation_axis is not None:
            return self.fixed_propagation_axis
        if sum(a == 1 for a in self.grid_shape) != 1:
            raise Exception(f"Invalid poynting flux detector shape: {self.grid_shape}")
        return self.grid_shape.index(1)


@dataclass(eq=False)
class PhasorPoyntingFluxDetector(PhasorDetector):
    """Phasors of all six components on a plane; the time-averaged flux is formed after the run."""

    direction: Literal["+", "-"] = "+"
    fixed_propagation_axis: int | None = None
    keep_all_components: bool = False

    def __post_init__(self):
        super().__post_init__()
        self.components = COMPONENTS
        self.reduce_volume = False

    @property
    def propagation_axis(self) -> int:
        if self.fixed_propagation_axis is not None:
            return self.fixed_propagation_axis
        if sum(a == 1 for a in self.grid_shape) != 1:
            raise Exception(f"Invalid poynting flux detector shape: {self.grid_shape}")
        return self.grid_shape.index(1)

    def compute_poynting_flux(self, state, spacing: float):
        """0.5 Re(E x conj H) . n dA summed over the plane, per frequency (poynting_flux.py:361-387)."""
        import torch

        ph = state["phasor"][0]  # (F, 6, *grid_shape)
        E, H = ph[:, :3], ph[:, 3:].conj()
        S = torch.stack(
            [
                E[:, 1] * H[:, 2] - E[:, 2] * H[:, 1],
                E[:, 2] * H[:, 0] - E[:, 0] * H[:, 2],
                E[:, 0] * H[:, 1] - E[:, 1] * H[:, 0],
            ],
            dim=1,
        ).real
        if self.direction == "-":
            S = -S
        area = spacing * spacing
        if self.keep_all_components:
            flux = (S * area).sum(dim=(2, 3, 4))
        else:
            flux = (S[:, self.propagation_axis] * area).sum(dim=(1, 2, 3))
        if self.scaling_mode == "continuous":
            flux = 0.5 * flux
        return flux


__all__ = [
    "SimulationObject",
    "SimulationVolume",
    "Material",
    "UniformMaterialObject",
    "Device",
    "BaseBoundary",
    "PerfectlyMatchedLayer",
    "PerfectElectricConductor",
    "PerfectMagneticConductor",
    "PeriodicBoundary",
    "BlochBoundary",
    "BoundaryConfig",
    "boundary_objects_from_config",
    "Source",
    "PointDipoleSource",
    "LinearlyPolarizedPlaneSource",
    "GaussianPlaneSource",
    "UniformPlaneSource",
    "Detector",
    "FieldDetector",
    "EnergyDetector",
    "PhasorDetector",
    "PoyntingFluxDetector",
    "PhasorPoyntingFluxDetector",
    "GaussianPulseProfile",
    "SingleFrequencyProfile",
]
