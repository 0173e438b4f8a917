"""Scene authoring: the reference's problem description, as plain data.

Mirrors the Rust types a caller of the reference builds a run from —
``Axis``/``Extent``/``Grid``/``Refinement`` (src/grid.rs), ``Material`` and
``MaterialTable`` (src/material.rs), ``Boundary`` (src/boundary.rs),
``Waveform``/``Source`` (src/source.rs), ``Shape``/``Scene`` with its presets
(src/scene.rs) — and flattens them into the C ABI's ``dp_scene_desc``.

All arithmetic a preset performs is done in float32, in the reference's
order, so a preset built here describes exactly the scene the Rust one does.
Grid quantities that need the resolved (possibly graded) spacing come from
the library's host-only ``dp_grid_resolve`` (``use_grid_resolver`` swaps in
another implementation of the same query).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field, replace
from enum import IntEnum
from typing import Sequence

import numpy as np

from . import _abi

f32 = np.float32
SPEED_OF_LIGHT = f32(299792458.0)          # src/grid.rs:42
VACUUM_PERMEABILITY = f32(1.2566371e-6)    # src/grid.rs:44
VACUUM_PERMITTIVITY = f32(8.854188e-12)    # src/grid.rs:46
COURANT_LIMIT = f32(0.57735026)            # src/grid.rs:411
PRESET_CELL_SIZE = f32(1e-3)               # src/scene.rs:16


def _round_half_away(v: np.float32) -> np.float32:
    """f32::round: halves away from zero (numpy rounds halves to even)."""
    r = np.floor(np.abs(v))
    if np.abs(v) - r >= f32(0.5):
        r = r + f32(1.0)
    return f32(np.copysign(r, v))


class Axis(IntEnum):
    X = 0
    Y = 1
    Z = 2

    def next(self) -> "Axis":
        return Axis((self + 1) % 3)

    def prev(self) -> "Axis":
        return Axis((self + 2) % 3)


@dataclass(frozen=True)
class Extent:
    x: int
    y: int
    z: int

    @staticmethod
    def cube(side: int) -> "Extent":
        return Extent(side, side, side)

    def as_array(self) -> tuple[int, int, int]:
        return (self.x, self.y, self.z)

    def total(self) -> int:
        return self.x * self.y * self.z

    def index(self, coord: Sequence[int]) -> int:
        return (coord[2] * self.y + coord[1]) * self.x + coord[0]


@dataclass(frozen=True)
class Refinement:
    """src/grid.rs:313-336."""
    center: tuple[float, float, float]
    size: tuple[float, float, float]
    cell_size: float

    @staticmethod
    def across(axis: Axis, offset: float, size: float, cell_size: float) -> "Refinement":
        center = [0.0, 0.0, 0.0]
        extent = [0.0, 0.0, 0.0]
        center[int(axis)] = offset
        extent[int(axis)] = size
        return Refinement(tuple(center), tuple(extent), cell_size)


class LibraryGridResolver:
    """Grid::build and the grid queries through the library's host-only
    dp_grid_resolve / dp_grid_map (no device is touched)."""

    @staticmethod
    def resolve(spec: _abi.dp_grid_spec, out: _abi.dp_grid_info) -> None:
        _abi.check(_abi.lib().dp_grid_resolve(C.byref(spec), C.byref(out)))

    @staticmethod
    def map(spec: _abi.dp_grid_spec, op: int, src, dst) -> None:
        _abi.check(_abi.lib().dp_grid_map(C.byref(spec), op, src, dst))


_grid_resolver = LibraryGridResolver


def use_grid_resolver(resolver) -> object:
    """Sets what resolves grid recipes (an object with ``resolve(spec, out)``
    and ``map(spec, op, src, dst)`` filling the ABI structs) and returns the
    previous one.  The library's own is the default; a process that must not
    load the CUDA library at all (a CPU-only baseline) installs another that
    computes the same values."""
    global _grid_resolver
    previous, _grid_resolver = _grid_resolver, resolver
    return previous


@dataclass
class Grid:
    """The recipe of a Grid (GridSpec, src/grid.rs:381-392); resolved lazily."""
    base_extent: Extent
    cell_size: float
    courant: float = 0.5
    refinements: list[Refinement] = field(default_factory=list)
    max_ratio: float = 1.15

    @staticmethod
    def new(extent: Extent, cell_size: float) -> "Grid":
        return Grid(extent, float(f32(cell_size)))

    @staticmethod
    def extent_for(size: Sequence[float], resolution: float) -> Extent:
        cells = [int(max(_round_half_away(f32(m) * f32(resolution)), f32(2.0))) for m in size]
        return Extent(*cells)

    @staticmethod
    def for_size(size: Sequence[float], resolution: float) -> "Grid":
        return Grid.new(Grid.extent_for(size, resolution), float(f32(1.0) / f32(resolution)))

    @staticmethod
    def graded(size: Sequence[float], resolution: float, refinements: list[Refinement],
               max_ratio: float = 1.15) -> "Grid":
        return Grid(Grid.extent_for(size, resolution), float(f32(1.0) / f32(resolution)), 0.5,
                    list(refinements), max_ratio)

    def with_resolution(self, resolution: float) -> "Grid":
        return Grid(Grid.extent_for(self.size(), resolution), float(f32(1.0) / f32(resolution)), self.courant,
                    list(self.refinements), self.max_ratio)

    def is_uniform(self) -> bool:
        return not self.refinements

    # -- flattening -----------------------------------------------------------
    def spec(self) -> tuple[_abi.dp_grid_spec, object]:
        refs = (_abi.dp_refinement * max(1, len(self.refinements)))()
        for i, r in enumerate(self.refinements):
            refs[i] = _abi.dp_refinement(_abi.F3(*r.center), _abi.F3(*r.size), r.cell_size)
        spec = _abi.dp_grid_spec(_abi.U3(*self.base_extent.as_array()), self.cell_size, self.courant,
                                 self.max_ratio, len(self.refinements),
                                 C.cast(refs, C.POINTER(_abi.dp_refinement)))
        return spec, refs

    def info(self) -> _abi.dp_grid_info:
        spec, keep = self.spec()
        out = _abi.dp_grid_info()
        _grid_resolver.resolve(spec, out)
        del keep
        return out

    def _map(self, op: int, values: Sequence[float]) -> tuple[float, float, float]:
        spec, keep = self.spec()
        src = _abi.F3(*values)
        dst = _abi.F3()
        _grid_resolver.map(spec, op, src, dst)
        del keep
        return (dst[0], dst[1], dst[2])

    # -- queries of the resolved grid (src/grid.rs:521-745) --------------------
    @property
    def extent(self) -> Extent:
        return Extent(*self.info().extent)

    def size(self) -> tuple[float, float, float]:
        return tuple(self.info().size)

    def time_step(self) -> float:
        return self.info().time_step

    def coarsest(self) -> float:
        return self.info().coarsest

    def finest(self) -> float:
        return self.info().finest

    def worst_ratio(self) -> float:
        return self.info().worst_ratio

    def reference_cell_size(self) -> float:
        return self.info().reference_cell_size

    def frequency_for_resolution(self, cells: float) -> float:
        """src/grid.rs:742-744."""
        return float(SPEED_OF_LIGHT / (f32(cells) * f32(self.coarsest())))

    def cells_per_wavelength(self, frequency: float, refractive_index: float = 1.0) -> float:
        return float(SPEED_OF_LIGHT / (f32(refractive_index) * f32(frequency) * f32(self.coarsest())))

    def to_cell(self, position: Sequence[float]) -> tuple[float, float, float]:
        return self._map(_abi.DP_MAP_TO_CELL, position)

    def to_position(self, cell: Sequence[float]) -> tuple[float, float, float]:
        return self._map(_abi.DP_MAP_TO_POSITION, cell)

    def cell_containing(self, position: Sequence[float]) -> tuple[int, int, int]:
        return tuple(int(v) for v in self._map(_abi.DP_MAP_CELL_CONTAINING, position))

    def cell_center(self, coord: Sequence[int]) -> tuple[float, float, float]:
        return self._map(_abi.DP_MAP_CELL_CENTER, [float(c) for c in coord])


@dataclass(frozen=True)
class Material:
    """src/material.rs:29-123."""
    relative_permittivity: float = 1.0
    relative_permeability: float = 1.0
    conductivity: float = 0.0
    magnetic_loss: float = 0.0

    @staticmethod
    def dielectric(relative_permittivity: float) -> "Material":
        return Material(float(f32(relative_permittivity)))

    @staticmethod
    def refractive(index: float) -> "Material":
        return Material.dielectric(float(f32(index) * f32(index)))

    @staticmethod
    def matched_lossy(relative_permittivity: float, conductivity: float) -> "Material":
        er, s = f32(relative_permittivity), f32(conductivity)
        return Material(float(er), 1.0, float(s), float(s * VACUUM_PERMEABILITY / (VACUUM_PERMITTIVITY * er)))

    def refractive_index(self) -> float:
        return float(np.sqrt(f32(self.relative_permittivity) * f32(self.relative_permeability)))

    def _key(self) -> tuple:
        return tuple(float(f32(v)) for v in (self.relative_permittivity, self.relative_permeability,
                                              self.conductivity, self.magnetic_loss))


Material.VACUUM = Material()
Material.PERFECT_CONDUCTOR = Material(1.0, 1.0, math.inf, 0.0)


class MaterialTable:
    """src/material.rs:166-223: index 0 is vacuum; duplicates merge."""
    VACUUM = 0

    def __init__(self) -> None:
        self.materials: list[Material] = [Material.VACUUM]

    def push(self, material: Material) -> int:
        key = material._key()
        for i, m in enumerate(self.materials):
            if m._key() == key:
                return i
        self.materials.append(material)
        return len(self.materials) - 1

    def get(self, index: int) -> Material:
        return self.materials[index]

    def __len__(self) -> int:
        return len(self.materials)

    def copy(self) -> "MaterialTable":
        t = MaterialTable()
        t.materials = list(self.materials)
        return t

    def peak_refractive_index(self) -> float:
        return max([1.0] + [m.refractive_index() for m in self.materials if math.isfinite(m.conductivity)])


@dataclass(frozen=True)
class Boundary:
    """src/boundary.rs:53-80."""
    kind: int
    thickness: int = 0
    target_reflection: float = 1.0

    @staticmethod
    def absorbing(thickness: int = 10, target_reflection: float = 1e-6) -> "Boundary":
        return Boundary(_abi.DP_BOUNDARY_ABSORBING, thickness, target_reflection)


Boundary.PEC = Boundary(_abi.DP_BOUNDARY_PEC, 0, 1.0)
Boundary.DEFAULT = Boundary.absorbing(10, 1e-6)


@dataclass(frozen=True)
class Waveform:
    """src/source.rs:31-127."""
    kind: int
    frequency: float
    duration_cycles: float = 0.0
    ramp_cycles: float = 0.0
    delay: float = 0.0

    @staticmethod
    def ricker(peak_frequency: float) -> "Waveform":
        f = f32(peak_frequency)
        return Waveform(_abi.DP_WAVE_RICKER, float(f), delay=float(f32(1.4) / f))

    @staticmethod
    def ricker_at(peak_frequency: float, delay: float) -> "Waveform":
        return Waveform(_abi.DP_WAVE_RICKER, float(f32(peak_frequency)), delay=float(f32(delay)))

    @staticmethod
    def gaussian_pulse(center_frequency: float, duration_cycles: float) -> "Waveform":
        f, d = f32(center_frequency), f32(duration_cycles)
        return Waveform(_abi.DP_WAVE_GAUSSIAN_PULSE, float(f), duration_cycles=float(d),
                        delay=float(f32(2.0) * d / f))

    @staticmethod
    def continuous_wave(frequency: float, ramp_cycles: float) -> "Waveform":
        return Waveform(_abi.DP_WAVE_CONTINUOUS, float(f32(frequency)), ramp_cycles=float(f32(ramp_cycles)))

    def dominant_frequency(self) -> float:
        return self.frequency

    def to_c(self) -> _abi.dp_waveform:
        return _abi.dp_waveform(self.kind, self.frequency, self.duration_cycles, self.ramp_cycles, self.delay)


@dataclass(frozen=True)
class Source:
    """src/source.rs:136-272."""
    shape: int
    polarization: Axis
    waveform: Waveform
    amplitude: float = 1.0
    at: tuple[float, float, float] = (0.0, 0.0, 0.0)
    velocity: tuple[float, float, float] = (0.0, 0.0, 0.0)
    axis: Axis = Axis.X
    offset: float = 0.0
    waist: float = 0.0
    box_low: tuple[float, float, float] = (0.0, 0.0, 0.0)
    box_high: tuple[float, float, float] = (0.0, 0.0, 0.0)

    @staticmethod
    def point(at: Sequence[float], polarization: Axis, waveform: Waveform) -> "Source":
        return Source(_abi.DP_SOURCE_POINT, polarization, waveform, at=tuple(at))

    @staticmethod
    def point_moving(at: Sequence[float], velocity: Sequence[float], polarization: Axis,
                     waveform: Waveform) -> "Source":
        return Source(_abi.DP_SOURCE_POINT, polarization, waveform, at=tuple(at), velocity=tuple(velocity))

    @staticmethod
    def sheet(axis: Axis, offset: float, waist: float, polarization: Axis, waveform: Waveform) -> "Source":
        return Source(_abi.DP_SOURCE_SHEET, polarization, waveform, axis=axis, offset=offset, waist=waist)

    @staticmethod
    def plane_wave(axis: Axis, offset: float, polarization: Axis, waveform: Waveform) -> "Source":
        return Source(_abi.DP_SOURCE_PLANE_WAVE, polarization, waveform, axis=axis, offset=offset)

    @staticmethod
    def plane_wave_box(axis: Axis, low: Sequence[float], high: Sequence[float], polarization: Axis,
                       waveform: Waveform) -> "Source":
        """A plane wave travelling toward +axis through the total-field box
        whose corner cells contain `low` and `high` (metres from the domain
        centre); outside the box every side sees the scattered field alone.
        An extension: the reference's plane wave spans the whole cross-section
        (src/source.rs:162-181)."""
        return Source(_abi.DP_SOURCE_PLANE_WAVE_BOX, polarization, waveform, axis=axis,
                      box_low=tuple(low), box_high=tuple(high))

    def with_amplitude(self, amplitude: float) -> "Source":
        return replace(self, amplitude=amplitude)

    def to_c(self) -> _abi.dp_source:
        return _abi.dp_source(self.shape, int(self.polarization), _abi.F3(*self.at), _abi.F3(*self.velocity),
                              int(self.axis), self.offset, self.waist, self.amplitude, self.waveform.to_c(),
                              _abi.F3(*self.box_low), _abi.F3(*self.box_high))


@dataclass(frozen=True)
class Shape:
    """src/scene.rs:32-56."""
    kind: int
    material: int
    center: tuple[float, float, float] = (0.0, 0.0, 0.0)
    size: tuple[float, float, float] = (0.0, 0.0, 0.0)
    radius: float = 0.0
    axis: Axis = Axis.X
    offset: float = 0.0
    thickness: float = 0.0

    @staticmethod
    def block(center: Sequence[float], size: Sequence[float], material: int) -> "Shape":
        return Shape(_abi.DP_SHAPE_BLOCK, material, center=tuple(center), size=tuple(size))

    @staticmethod
    def sphere(center: Sequence[float], radius: float, material: int) -> "Shape":
        return Shape(_abi.DP_SHAPE_SPHERE, material, center=tuple(center), radius=radius)

    @staticmethod
    def slab(axis: Axis, offset: float, thickness: float, material: int) -> "Shape":
        return Shape(_abi.DP_SHAPE_SLAB, material, axis=axis, offset=offset, thickness=thickness)

    def to_c(self) -> _abi.dp_shape:
        return _abi.dp_shape(self.kind, self.material, _abi.F3(*self.center), _abi.F3(*self.size), self.radius,
                             int(self.axis), self.offset, self.thickness)


@dataclass
class Scene:
    """src/scene.rs:116-457."""
    grid: Grid
    boundary: Boundary = Boundary.DEFAULT
    materials: MaterialTable = field(default_factory=MaterialTable)
    shapes: list[Shape] = field(default_factory=list)
    sources: list[Source] = field(default_factory=list)

    @staticmethod
    def on_grid(grid: Grid) -> "Scene":
        return Scene(grid)

    @staticmethod
    def empty(extent: Extent, cell_size: float) -> "Scene":
        return Scene(Grid.new(extent, cell_size))

    @staticmethod
    def sized(size: Sequence[float], resolution: float) -> "Scene":
        return Scene(Grid.for_size(size, resolution))

    def with_boundary(self, boundary: Boundary) -> "Scene":
        self.boundary = boundary
        return self

    def with_source(self, source: Source) -> "Scene":
        self.sources.append(source)
        return self

    def with_shape(self, shape: Shape) -> "Scene":
        self.shapes.append(shape)
        return self

    def with_resolution(self, resolution: float) -> "Scene":
        return Scene(self.grid.with_resolution(resolution), self.boundary, self.materials.copy(),
                     list(self.shapes), list(self.sources))

    def is_reversible(self) -> bool:
        return self.boundary == Boundary.PEC and all(
            m.conductivity == 0.0 and m.magnetic_loss == 0.0 for m in self.materials.materials)

    # -- presets (src/scene.rs:376-456) ------------------------------------------
    @staticmethod
    def photon(extent: Extent) -> "Scene":
        grid = Grid.new(extent, PRESET_CELL_SIZE)
        size = [f32(s) for s in grid.size()]
        frequency = grid.frequency_for_resolution(16.0)
        source = Source.sheet(Axis.X, float(f32(-0.3) * size[0]), float(f32(0.25) * min(size[1], size[2])),
                              Axis.Z, Waveform.gaussian_pulse(frequency, 2.0))
        return Scene(grid, Boundary.DEFAULT, MaterialTable(), [], [source])

    @staticmethod
    def cavity(extent: Extent) -> "Scene":
        return Scene.cavity_on(Grid.new(extent, PRESET_CELL_SIZE))

    @staticmethod
    def cavity_on(grid: Grid) -> "Scene":
        size = [f32(s) for s in grid.size()]
        frequency = grid.frequency_for_resolution(16.0)
        source = Source.point([float(-size[0] / f32(6.0)), 0.0, 0.0], Axis.Z, Waveform.ricker(frequency))
        return Scene(grid, Boundary.PEC, MaterialTable(), [], [source])

    @staticmethod
    def slab(extent: Extent, refractive_index: float) -> "Scene":
        scene = Scene.photon(extent)
        size = [f32(s) for s in scene.grid.size()]
        material = scene.materials.push(Material.refractive(refractive_index))
        scene.shapes.append(Shape.slab(Axis.X, float(size[0] / f32(8.0)), float(size[0] / f32(4.0)), material))
        frequency = scene.grid.frequency_for_resolution(float(f32(16.0) * f32(refractive_index)))
        scene.sources = [replace(s, waveform=Waveform.gaussian_pulse(frequency, 2.0)) for s in scene.sources]
        return scene

    # -- flattening ---------------------------------------------------------------
    def desc(self) -> tuple[_abi.dp_scene_desc, list]:
        """The C description, plus the ctypes arrays it points into (keep alive)."""
        spec, refs = self.grid.spec()
        mats = (_abi.dp_material * len(self.materials))(
            *[_abi.dp_material(m.relative_permittivity, m.relative_permeability, m.conductivity, m.magnetic_loss)
              for m in self.materials.materials])
        shapes = (_abi.dp_shape * max(1, len(self.shapes)))(*[s.to_c() for s in self.shapes])
        sources = (_abi.dp_source * max(1, len(self.sources)))(*[s.to_c() for s in self.sources])
        b = _abi.dp_boundary(self.boundary.kind, self.boundary.thickness, self.boundary.target_reflection)
        d = _abi.dp_scene_desc(spec, b, len(self.materials), C.cast(mats, C.POINTER(_abi.dp_material)),
                               len(self.shapes), C.cast(shapes, C.POINTER(_abi.dp_shape)),
                               len(self.sources), C.cast(sources, C.POINTER(_abi.dp_source)))
        return d, [refs, mats, shapes, sources]
