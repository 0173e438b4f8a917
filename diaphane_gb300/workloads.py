"""Seeded synthetic scenes for the benchmark workloads.

There is no public dataset behind these: each is a scene generated from a
seed with the sizes and value ranges the workload names, using SplitMix64 so
the same seed gives the same scene on any machine.
"""
from __future__ import annotations

import math

from .scene import Axis, Boundary, Extent, Grid, Material, Refinement, Scene, Shape, Source, Waveform, f32

MASK = (1 << 64) - 1


class SplitMix64:
    """Steele, Lea and Flood's SplitMix64 generator."""

    def __init__(self, seed: int):
        self.state = seed & MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


HETEROGENEOUS_SEED = 0x5EED_0002


def heterogeneous(side: int = 512, spheres: int = 200, seed: int = HETEROGENEOUS_SEED) -> Scene:
    """Heterogeneous scatterers on a uniform side³ grid at 1 mm.

    * 10-cell absorbing layer (R0 = 1e-6).
    * A total-field box 16 cells inside the absorber on every side (faces at
      cells 26 and side-27; fewer cells on grids too small for that) through
      which an x-travelling, z-polarized plane wave passes; outside it every
      side sees the scattered field alone.  Gaussian pulse, 3 cycles, at the
      frequency whose wavelength is 10 cells.
    * `spheres` dielectric spheres, radius uniform in [4, 24] cells, εr
      uniform in [1, 4], centres uniform over the box's interior, kept two
      cells clear of its faces (which must lie in vacuum).  Each sphere is
      its own material.
    * One perfectly conducting sphere of radius 40 cells at the centre.
    * One lossy slab, Material::matched_lossy(2, σ), 16 cells thick across x
      at 3/4 of the domain and spanning the box's cross-section two cells
      short of its faces, with σ chosen so the electric half-step loss
      σ·Δt/(2ε0εr) is 0.02; matched magnetic loss keeps it reflectionless.
    Painted in that order: spheres, then the conductor, then the slab.
    """
    rng = SplitMix64(seed)
    cell = f32(1e-3)
    scene = Scene.empty(Extent.cube(side), float(cell))
    grid = scene.grid
    half = side * float(cell) / 2.0
    absorber = 10
    inset = min(16, max(2, (side - 2 * absorber) // 6))
    lo = max(1, min(absorber + inset, side // 2 - 3))  # the box's faces, in cells
    hi = side - 1 - lo
    largest = max(1.0, min(24.0, (hi - lo) / 2.0 - 3.0))

    def position(c: float) -> float:
        return float(f32(c) * cell - f32(half))

    for _ in range(spheres):
        r = min(rng.uniform(4.0, 24.0), largest)
        eps = rng.uniform(1.0, 4.0)
        c_lo, c_hi = lo + 2 + r, hi - 2 - r
        cx, cy, cz = rng.uniform(c_lo, c_hi), rng.uniform(c_lo, c_hi), rng.uniform(c_lo, c_hi)
        m = scene.materials.push(Material.dielectric(eps))
        scene.shapes.append(Shape.sphere((position(cx), position(cy), position(cz)), float(f32(r) * cell), m))

    pec = scene.materials.push(Material.PERFECT_CONDUCTOR)
    scene.shapes.append(Shape.sphere((0.0, 0.0, 0.0), float(f32(min(40.0, largest)) * cell), pec))

    dt = grid.time_step()
    eps_slab = 2.0
    sigma = 0.02 * 2.0 * 8.854188e-12 * eps_slab / dt
    lossy = scene.materials.push(Material.matched_lossy(eps_slab, sigma))
    thickness = max(1, min(16, (hi - lo) // 4))
    slab_x = min(0.75 * side, hi - 2 - thickness / 2.0)
    across = float(f32(max(1, hi - lo - 4)) * cell)
    scene.shapes.append(Shape.block((position(slab_x), 0.0, 0.0), (float(f32(thickness) * cell), across, across),
                                    lossy))

    frequency = grid.frequency_for_resolution(10.0)
    low, high = (position(lo + 0.5),) * 3, (position(hi + 0.5),) * 3
    scene.sources.append(Source.plane_wave_box(Axis.X, low, high, Axis.Z, Waveform.gaussian_pulse(frequency, 3.0)))
    return scene


def free_flight(side: int = 80) -> Scene:
    """Uniform side³ at 1 mm, vacuum, Courant 0.99/√3, 10-cell absorber, Ez
    point source at the centre: Gaussian-modulated sinusoid at 30 GHz with
    50% bandwidth, read as an amplitude-spectrum FWHM of 15 GHz, which is a
    time-envelope FWHM of 4·ln2/(π·15 GHz) = 58.8 ps = 1.765 carrier cycles."""
    scene = Scene.empty(Extent.cube(side), 1e-3)
    scene.grid.courant = float(f32(0.99) / f32(math.sqrt(3.0)))
    cycles = 4.0 * math.log(2.0) / (math.pi * 15e9) * 30e9
    scene.sources.append(Source.point((0.0, 0.0, 0.0), Axis.Z, Waveform.gaussian_pulse(30e9, cycles)))
    return scene


def graded_stack(open_boundary: bool = True) -> Scene:
    """640×256×256 graded layered stack: x graded at cap 1.15 from 1 mm down
    to 0.1 mm across an 8 mm band, y and z uniform at 1 mm; six quarter-wave
    pairs of n = 1.5 and n = 2.3 fill the band (λ0 = 4·8 mm/(6·(1/1.5... see
    below)); a sheet source at λ0 in vacuum launches into it."""
    grid = Grid.graded((0.549, 0.256, 0.256), 1000.0, [Refinement.across(Axis.X, 0.0, 0.008, 1e-4)], 1.15)
    scene = Scene.on_grid(grid)
    if not open_boundary:
        scene.boundary = Boundary.PEC
    # Quarter-wave pair: d1 = λ0/(4·1.5), d2 = λ0/(4·2.3); six pairs fill
    # 8 mm, so λ0 = 8 mm·4/(6·(1/1.5 + 1/2.3)) = 4.84 mm (f0 = 61.9 GHz).
    n1, n2 = 1.5, 2.3
    lam0 = 0.008 * 4.0 / (6.0 * (1.0 / n1 + 1.0 / n2))
    d1, d2 = lam0 / (4 * n1), lam0 / (4 * n2)
    m1 = scene.materials.push(Material.refractive(n1))
    m2 = scene.materials.push(Material.refractive(n2))
    x = -0.004
    for _ in range(6):
        scene.shapes.append(Shape.slab(Axis.X, x + d1 / 2, d1, m1))
        x += d1
        scene.shapes.append(Shape.slab(Axis.X, x + d2 / 2, d2, m2))
        x += d2
    f0 = 299792458.0 / lam0
    scene.sources.append(Source.sheet(Axis.X, -0.15, 0.06, Axis.Z, Waveform.gaussian_pulse(f0, 3.0)))
    return scene


def mixed_scene(seed: int, lo: int = 32, hi: int = 160, steps: int = 1000) -> Scene:
    """One scene of the mixed-size batch: each axis log-uniform in [lo, hi]
    cells at 1 mm, 10-cell absorber, up to 8 seeded dielectric spheres (εr in
    [1, 4]), a perfectly conducting sphere with probability 1/2, and one
    source — a point dipole or, with probability 1/2, an x-travelling plane
    wave — at 10 cells per wavelength."""
    rng = SplitMix64(seed)
    n = [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(3)]
    cell = f32(1e-3)
    scene = Scene.empty(Extent(*n), float(cell))
    half = [f32(v) * cell / f32(2.0) for v in n]
    margin = 12  # clear of the absorber (and of the plane-wave rows)

    def inside(axis: int, radius: float) -> float:
        lo_c, hi_c = margin + radius, n[axis] - margin - radius
        c = rng.uniform(lo_c, hi_c) if hi_c > lo_c else n[axis] / 2.0
        return float(f32(c) * cell - half[axis])

    for _ in range(int(rng.uniform(0, 9))):
        r = rng.uniform(2.0, max(2.5, min(n) / 8.0))
        m = scene.materials.push(Material.dielectric(rng.uniform(1.0, 4.0)))
        scene.shapes.append(Shape.sphere((inside(0, r + 16), inside(1, r), inside(2, r)), float(f32(r) * cell), m))
    if rng.uniform(0, 1) < 0.5:
        r = max(2.0, min(n) / 10.0)
        pec = scene.materials.push(Material.PERFECT_CONDUCTOR)
        scene.shapes.append(Shape.sphere((inside(0, r + 16), inside(1, r), inside(2, r)), float(f32(r) * cell), pec))
    frequency = scene.grid.frequency_for_resolution(10.0)
    if rng.uniform(0, 1) < 0.5:
        scene.sources.append(Source.point((inside(0, 4), inside(1, 4), inside(2, 4)), Axis.Z,
                                          Waveform.gaussian_pulse(frequency, 3.0)))
    else:
        scene.sources.append(Source.plane_wave(Axis.X, float(f32(13.5) * cell - half[0]), Axis.Z,
                                               Waveform.gaussian_pulse(frequency, 3.0)))
    return scene


def graded_cavity() -> Scene:
    """192³ graded conducting box: 175.5 × 192 × 192 mm at 1 mm, x graded at
    cap 1.15 down to 0.4 mm across an 8 mm band at the centre (192 cells
    along x), perfectly conducting walls, a Ricker point source at 16 cells
    per wavelength a sixth of the box from the centre (Scene::cavity_on)."""
    grid = Grid.graded((0.1755, 0.192, 0.192), 1000.0, [Refinement.across(Axis.X, 0.0, 0.008, 4e-4)], 1.15)
    return Scene.cavity_on(grid)
