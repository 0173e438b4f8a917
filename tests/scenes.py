"""The reference's parity scenes (tests/parity.rs:124-289) and a few more,
rebuilt through the Python scene model."""
from __future__ import annotations

import math

from diaphane_gb300 import (Axis, Boundary, Extent, Grid, Material, Refinement, Scene, Shape, Source, Waveform)


def photon():  # tests/parity.rs:124-134
    return Scene.photon(Extent(96, 40, 36)), 150


def cavity():  # tests/parity.rs:136-141
    return Scene.cavity(Extent(40, 36, 32)), 500


def materials():  # tests/parity.rs:143-183
    scene = Scene.empty(Extent(44, 40, 40), 1e-3)
    frequency = scene.grid.frequency_for_resolution(24.0)
    glass = scene.materials.push(Material.refractive(1.5))
    lossy = scene.materials.push(Material.matched_lossy(2.0, 0.05))
    metal = scene.materials.push(Material.PERFECT_CONDUCTOR)
    scene.shapes.append(Shape.slab(Axis.X, 6e-3, 8e-3, glass))
    scene.shapes.append(Shape.sphere((-8e-3, 0.0, 0.0), 5e-3, lossy))
    scene.shapes.append(Shape.block((14e-3, 0.0, 0.0), (4e-3, 12e-3, 12e-3), metal))
    scene.sources.append(Source.point((-10e-3, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    return scene, 200


def several_sources():  # tests/parity.rs:185-219
    scene = Scene.empty(Extent.cube(40), 1e-3).with_boundary(Boundary.absorbing(8, 1e-6))
    frequency = scene.grid.frequency_for_resolution(20.0)
    scene.sources.append(Source.point((0.0, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    scene.sources.append(Source.point((0.0, 0.0, 0.0), Axis.X, Waveform.ricker(frequency)).with_amplitude(-0.5))
    scene.sources.append(Source.sheet(Axis.Y, -8e-3, 6e-3, Axis.Z, Waveform.gaussian_pulse(frequency, 3.0)))
    scene.sources.append(Source.point_moving((-6e-3, 2e-3, 0.0), (2.7e8, 0.0, 0.0), Axis.Z,
                                             Waveform.ricker(frequency)))
    return scene, 250


def graded():  # tests/parity.rs:221-265
    grid = Grid.graded((48e-3, 40e-3, 36e-3), 1e3, [Refinement.across(Axis.X, 6e-3, 8e-3, 0.25e-3),
                                                     Refinement.across(Axis.Y, -4e-3, 6e-3, 0.5e-3)])
    scene = Scene.on_grid(grid).with_boundary(Boundary.absorbing(8, 1e-6))
    frequency = scene.grid.frequency_for_resolution(24.0)
    glass = scene.materials.push(Material.refractive(1.5))
    scene.shapes.append(Shape.slab(Axis.X, 6e-3, 2e-3, glass))
    scene.sources.append(Source.point((0.0, -4e-3, 0.0), Axis.Z, Waveform.ricker(frequency)))
    return scene, 280


def graded_aligned():
    """The graded case on a 47 mm domain: 80 cells along x, so the fused
    kernel (which needs nx % 4 == 0 for its TMA row stride) covers it too."""
    grid = Grid.graded((47e-3, 40e-3, 36e-3), 1e3, [Refinement.across(Axis.X, 6e-3, 8e-3, 0.25e-3),
                                                     Refinement.across(Axis.Y, -4e-3, 6e-3, 0.5e-3)])
    scene = Scene.on_grid(grid).with_boundary(Boundary.absorbing(8, 1e-6))
    frequency = scene.grid.frequency_for_resolution(24.0)
    glass = scene.materials.push(Material.refractive(1.5))
    scene.shapes.append(Shape.slab(Axis.X, 6e-3, 2e-3, glass))
    scene.sources.append(Source.point((0.0, -4e-3, 0.0), Axis.Z, Waveform.ricker(frequency)))
    return scene, 280


def plane_wave():  # tests/parity.rs:267-289
    scene = Scene.empty(Extent(96, 36, 36), 1e-3)
    frequency = scene.grid.frequency_for_resolution(20.0)
    glass = scene.materials.push(Material.refractive(1.5))
    scene.shapes.append(Shape.sphere((8e-3, 0.0, 0.0), 6e-3, glass))
    scene.sources.append(Source.plane_wave(Axis.X, -0.020, Axis.Z, Waveform.gaussian_pulse(frequency, 3.0)))
    return scene, 350


def reversible():  # tests/parity.rs:291-311
    scene = Scene.empty(Extent(40, 36, 36), 1e-3).with_boundary(Boundary.PEC)
    frequency = scene.grid.frequency_for_resolution(24.0)
    glass = scene.materials.push(Material.refractive(2.0))
    scene.shapes.append(Shape.sphere((4e-3, 0.0, 0.0), 6e-3, glass))
    scene.sources.append(Source.point((-12e-3, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    return scene


def free_flight(side: int = 80):
    """Uniform 80³ at 1 mm, Courant 0.99/√3, 10-cell absorber, Ez point source
    at the centre, Gaussian-modulated sinusoid at 30 GHz with 50% bandwidth
    read as a 15 GHz amplitude-spectrum FWHM: time FWHM = 4 ln2/(π·15 GHz)
    = 58.8 ps = 1.765 carrier cycles."""
    scene = Scene.empty(Extent.cube(side), 1e-3)
    scene.grid.courant = 0.99 / math.sqrt(3.0)
    cycles = 4.0 * math.log(2.0) / (math.pi * 15e9) * 30e9
    scene.sources.append(Source.point((0.0, 0.0, 0.0), Axis.Z, Waveform.gaussian_pulse(30e9, cycles)))
    return scene


def box_wave():
    """A total-field box (an extension of the reference's plane wave) 14 cells
    in from every wall of a 60×48×44 absorbing grid, x-travelling and
    z-polarized, with a dielectric sphere and a conductor inside it: the wave
    crosses the box, the scatterers' field leaves it on every side."""
    scene = Scene.empty(Extent(60, 48, 44), 1e-3)
    frequency = scene.grid.frequency_for_resolution(10.0)
    n = (60, 48, 44)

    def metres(axis: int, cell: int) -> float:
        return (cell + 0.5) * 1e-3 - n[axis] * 1e-3 / 2.0

    glass = scene.materials.push(Material.refractive(1.5))
    metal = scene.materials.push(Material.PERFECT_CONDUCTOR)
    scene.shapes.append(Shape.sphere((-3e-3, 1e-3, 0.0), 6e-3, glass))
    scene.shapes.append(Shape.sphere((8e-3, -4e-3, 2e-3), 3e-3, metal))
    low = tuple(metres(a, 14) for a in range(3))
    high = tuple(metres(a, n[a] - 15) for a in range(3))
    scene.sources.append(Source.plane_wave_box(Axis.X, low, high, Axis.Z, Waveform.gaussian_pulse(frequency, 3.0)))
    return scene, 220


def has_box(scene) -> bool:
    from diaphane_gb300 import _abi
    return any(s.shape == _abi.DP_SOURCE_PLANE_WAVE_BOX for s in scene.sources)


PARITY_CASES = {
    "photon": photon,
    "cavity": cavity,
    "materials": materials,
    "several_sources": several_sources,
    "graded": graded,
    "graded_aligned": graded_aligned,
    "plane_wave": plane_wave,
    "box_wave": box_wave,
}
