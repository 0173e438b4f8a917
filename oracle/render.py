"""ORACLE — test infrastructure only.

A CPU restatement, in numpy float32, of the reference viewer's volume
renderer: the ray-march and shading of examples/common/shaders/volume.wgsl
(cell_of :101-113, densities :124-132, diverging :145-154, signed_log
:161-166, intersect_box :169-180, edge_glow :184-193, main_fs :214-339,
ribbons :351-388, emission :402-416, scrub_bar :440-479, background :481-486,
measure_peak :493-515) and its host-side control in examples/common/render.rs
(update_scale :281-325, params :327-382, reference_path :480-488) and
examples/common/camera.rs (Camera::basis).  Only the tests use it, to check
the CUDA renderer; nothing in the product imports it.

Arithmetic follows the CUDA kernel's operation order in float32; the host
trigonometry (camera) goes through the C library's sinf/cosf/tanf, as the
product's host code does.  Transcendentals inside the shading (exp, log, pow)
are numpy's, which may differ from CUDA's by an ulp, so images are compared
channel by channel within one 8-bit step.
"""
from __future__ import annotations

import ctypes
import ctypes.util
from dataclasses import dataclass, field

import numpy as np

F = np.float32
_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _name in ("sinf", "cosf", "tanf", "sqrtf"):
    getattr(_libm, _name).restype = ctypes.c_float
    getattr(_libm, _name).argtypes = [ctypes.c_float]

ENERGY, ELECTRIC, MAGNETIC, MAGNITUDE, FIELDS, GRID, RIBBONS, INTENSITY = range(8)
ELECTRIC_TINT = np.array([1.0, 0.45, 0.15], F)
MAGNETIC_TINT = np.array([0.20, 0.65, 1.0], F)
GRID_TINT = np.array([0.16, 0.19, 0.26], F)
INTENSITY_TINT = np.array([1.0, 0.8, 0.45], F)


@dataclass
class View:
    yaw: float = 0.9
    pitch: float = 0.45
    distance: float = 1.9
    fov: float = 0.8
    mode: int = FIELDS
    gain: float = 1.0
    log_strength: float = 6.0
    scrub: bool = False
    played: float = 0.0
    window_start: float = 0.0


@dataclass
class Exposure:
    """The renderer's running state (Renderer::scale, ::components)."""
    scale: float = 0.0
    components: list = field(default_factory=lambda: [2, 1])


def measure_peak(e, h, intensity, accumulated):
    """Eight slots: max of the larger energy density, max |E_c|, max |H_c|,
    max averaged intensity.  e, h: (3, cells) float32."""
    se = (F(0) + e[0] * e[0]) + e[1] * e[1]
    se = se + e[2] * e[2]
    sh = (F(0) + h[0] * h[0]) + h[1] * h[1]
    sh = sh + h[2] * h[2]
    slots = np.zeros(8, F)
    slots[0] = np.max(np.maximum(F(0.5) * se, F(0.5) * sh))
    for c in range(3):
        slots[1 + c] = np.max(np.abs(e[c]))
        slots[4 + c] = np.max(np.abs(h[c]))
    slots[7] = np.max(intensity / F(max(accumulated, 1)))
    return np.maximum(slots, F(0))


def update_scale(state: Exposure, slots, advanced: bool, mode: int) -> None:
    if not advanced:
        return
    measured = F(slots[7] if mode == INTENSITY else slots[0])

    def dominant(offset):
        best = -1
        for a in range(3):
            v = slots[offset + a]
            if not np.isfinite(v):
                continue
            if best < 0 or not v < slots[offset + best]:
                best = a
        return max(best, 0)

    electric, magnetic = dominant(1), dominant(4)
    if magnetic == electric:
        magnetic = (electric + 1) % 3
    state.components = [electric, magnetic]
    if not np.isfinite(measured) or measured <= 0:
        return
    if state.scale == 0:
        state.scale = F(measured)
        return
    rate = F(0.4) if measured > state.scale else F(0.02)
    state.scale = F(F(state.scale) + rate * (measured - F(state.scale)))


def camera_basis(view: View, box, aspect):
    box = [F(b) for b in box]
    center = [F(0.5) * b for b in box]
    radius = max(max(box[0], box[1]), box[2])
    sp, cp = F(_libm.sinf(view.pitch)), F(_libm.cosf(view.pitch))
    sy, cy = F(_libm.sinf(view.yaw)), F(_libm.cosf(view.yaw))
    away = [cp * sy, sp, cp * cy]
    position = [center[a] + away[a] * F(view.distance) * radius for a in range(3)]
    forward = [-away[a] for a in range(3)]
    world_up = [F(0), F(1), F(0)]
    r = [forward[1] * world_up[2] - forward[2] * world_up[1], forward[2] * world_up[0] - forward[0] * world_up[2],
         forward[0] * world_up[1] - forward[1] * world_up[0]]
    norm = F(_libm.sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]))
    r = [c / norm for c in r]
    u = [r[1] * forward[2] - r[2] * forward[1], r[2] * forward[0] - r[0] * forward[2],
         r[0] * forward[1] - r[1] * forward[0]]
    tangent = F(_libm.tanf(F(0.5) * F(view.fov)))
    right = [r[a] * tangent * F(aspect) for a in range(3)]
    up = [u[a] * tangent for a in range(3)]
    return position, right, up, forward


def _mix(a, b, t):
    return a * (F(1) - t) + b * t


def _smooth(lo, hi, x):
    t = np.clip((x - F(lo)) / (F(hi) - F(lo)), F(0), F(1))
    return t * t * (F(3) - F(2) * t)


def _sign(v):
    return np.where(v > 0, F(1), np.where(v < 0, F(-1), F(0))).astype(F)


def _signed_log(value, strength):
    if strength <= 0:
        return value
    return _sign(value) * np.log(F(1) + F(strength) * np.abs(value)) / np.log(F(1) + F(strength))


def _srgb8(linear):
    c = np.clip(linear, F(0), F(1))
    s = np.where(c <= F(0.0031308), F(12.92) * c, F(1.055) * np.power(c, F(1.0) / F(2.4)) - F(0.055))
    return np.rint(s.astype(F) * F(255)).astype(np.uint8)


def render(e, h, intensity, extent, lookup, samples, box, view: View, state: Exposure, accumulated, width, height):
    """RGBA8 image (height, width, 4); e, h: (3, cells) dense float32."""
    nx, ny, nz = extent
    box = np.array(box, F)
    aspect = F(width) / F(max(height, 1))
    origin, right, up, forward = camera_basis(view, box, aspect)
    reference = max(F(state.scale), F(np.finfo(F).tiny))
    signed_modes = (ELECTRIC, MAGNETIC, RIBBONS, FIELDS)
    exposure = (F(view.gain) / F(_libm.sqrtf(F(2) * reference)) if view.mode in signed_modes
                else F(view.gain) / reference)
    inverse_path = F(1) / max(max(max(box[0], box[1]), box[2]) / F(3), F(1))
    ce, ch = state.components
    px, py = np.meshgrid(np.arange(width, dtype=F), np.arange(height, dtype=F))
    sx = ((px + F(0.5)) / F(width) * F(2) - F(1)).ravel()
    sy = (F(1) - (py + F(0.5)) / F(height) * F(2)).ravel()
    d = np.stack([F(forward[a]) + sx * F(right[a]) + sy * F(up[a]) for a in range(3)])
    norm = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    d = d / norm
    o = np.array(origin, F)
    shade_sky = F(0.5) + F(0.5) * sy
    sky = np.stack([_mix(F(lo), F(hi), shade_sky) for lo, hi in ((0.02, 0.05), (0.02, 0.05), (0.03, 0.07))])
    near = np.full(sx.shape, -np.finfo(F).max, F)
    far = np.full(sx.shape, np.finfo(F).max, F)
    with np.errstate(divide="ignore", invalid="ignore"):
        for a in range(3):
            inv = F(1) / d[a]
            lo = (F(0) - o[a]) * inv
            hi = (box[a] - o[a]) * inv
            near = np.fmax(near, np.fmin(lo, hi))
            far = np.fmin(far, np.fmax(lo, hi))
    enter = np.fmax(near, F(0))
    hit = far > enter
    march = F(1)
    mode = view.mode
    signed_view = mode in (ELECTRIC, MAGNETIC, FIELDS)
    glow = np.zeros((3, sx.size), F)
    ex = np.zeros(sx.size, F)
    ey = np.zeros(sx.size, F)
    distance = enter + F(0.5) * march
    cells = nx * ny * nz
    ext = np.array([nx, ny, nz])
    for _ in range(4096):
        active = hit & (distance < far)
        if not active.any():
            break
        idx = np.nonzero(active)[0]
        point = o[:, None] + d[:, idx] * distance[idx]
        frac = np.empty_like(point)
        for a in range(3):
            fraction = np.clip(point[a] / box[a], F(0), F(1))
            position = fraction * F(samples - 1)
            low = position.astype(np.uint32)
            high = np.minimum(low + 1, samples - 1)
            section = lookup[a * samples:(a + 1) * samples]
            frac[a] = _mix(section[low], section[high], position - low.astype(F))
        coord = np.minimum(np.fmax(frac, F(0)).astype(np.uint32), (ext - 1)[:, None].astype(np.uint32))
        base = (coord[2].astype(np.int64) * ny + coord[1]) * nx + coord[0]
        if mode == RIBBONS:
            extf = ext.astype(F)
            middle = F(0.5) * extf
            travel = 3 - ce - ch
            probe = np.repeat(middle.astype(np.uint32)[:, None], idx.size, axis=1)
            probe[travel] = np.minimum(np.fmax(frac[travel], F(0)).astype(np.uint32), ext[travel] - 1)
            pb = (probe[2].astype(np.int64) * ny + probe[1]) * nx + probe[0]
            electric = e[ce][pb] * exposure
            magnetic = h[ch][pb] * exposure
            reach = F(0.33) * extf[ce]
            thick = F(0.015) * extf[ce]
            from_e = frac[ce] - middle[ce]
            from_h = frac[ch] - middle[ch]
            lit = np.zeros((3, idx.size), F)
            m1 = (np.abs(from_h) < thick) & (from_e * electric > 0) & (np.abs(from_e) < np.abs(electric) * reach)
            m2 = (np.abs(from_e) < thick) & (from_h * magnetic > 0) & (np.abs(from_h) < np.abs(magnetic) * reach)
            m3 = (np.abs(from_e) < thick) & (np.abs(from_h) < thick)
            lit = lit + np.where(m1, ELECTRIC_TINT[:, None], F(0))
            lit = lit + np.where(m2, MAGNETIC_TINT[:, None], F(0))
            lit = lit + np.where(m3, F(0.10), F(0))
            glow[:, idx] = glow[:, idx] + lit
        elif mode == GRID:
            edge = np.abs(frac - np.rint(frac))
            nearest = np.fmin(np.fmin(edge[0], edge[1]), edge[2])
            glow[:, idx] = glow[:, idx] + GRID_TINT[:, None] * _smooth(0.08, 0.0, nearest)
        elif signed_view:
            electric = e[ce][base]
            magnetic = h[ch][base]
            if mode == FIELDS:
                vx, vy = electric * exposure, magnetic * exposure
            else:
                vx = (magnetic if mode == MAGNETIC else electric) * exposure
                vy = np.zeros_like(vx)
            ex[idx] = np.where(np.abs(vx) > np.abs(ex[idx]), vx, ex[idx])
            ey[idx] = np.where(np.abs(vy) > np.abs(ey[idx]), vy, ey[idx])
        else:
            if mode == INTENSITY:
                avg = intensity[base] / F(max(accumulated, 1))
                em = INTENSITY_TINT[:, None] * _signed_log(avg * exposure, view.log_strength)
            else:
                se = (F(0) + e[0][base] * e[0][base]) + e[1][base] * e[1][base]
                se = se + e[2][base] * e[2][base]
                sh = (F(0) + h[0][base] * h[0][base]) + h[1][base] * h[1][base]
                sh = sh + h[2][base] * h[2][base]
                we = F(0.5) * se * exposure
                wh = F(0.5) * sh * exposure
                if mode == MAGNITUDE:
                    m = _signed_log(we + wh, view.log_strength)
                    em = np.stack([m, m, m])
                else:
                    em = (ELECTRIC_TINT[:, None] * _signed_log(we, view.log_strength) +
                          MAGNETIC_TINT[:, None] * _signed_log(wh, view.log_strength))
            glow[:, idx] = glow[:, idx] + em
        distance[idx] = distance[idx] + march
    # Rim.
    p = o[:, None] + d * far
    dist = np.fmin(p, box[:, None] - p) / box[:, None]
    lo = np.fmin(np.fmin(dist[0], dist[1]), dist[2])
    hi = np.fmax(np.fmax(dist[0], dist[1]), dist[2])
    middle = dist[0] + dist[1] + dist[2] - lo - hi
    rim = np.array([0.16, 0.18, 0.22], F)[:, None] * _smooth(0.01, 0.0, middle)
    if mode == FIELDS:
        e_s, h_s = _signed_log(ex, view.log_strength), _signed_log(ey, view.log_strength)
        lit = ELECTRIC_TINT[:, None] * np.abs(e_s) + MAGNETIC_TINT[:, None] * np.abs(h_s)
        shade = np.stack([F(0.5) + F(0.5) * (_sign(e_s) * np.abs(e_s)), np.full_like(e_s, F(0.5) + F(0.5) * F(0)),
                          F(0.5) + F(0.5) * (_sign(h_s) * np.abs(h_s))])
        length = np.sqrt(lit[0] * lit[0] + lit[1] * lit[1] + lit[2] * lit[2])
        fieldc = (sky * np.exp(-length) + lit * shade) + rim
    elif signed_view:
        scaled = _signed_log(ex, view.log_strength)
        opacity = np.fmin(np.abs(scaled), F(1))
        neutral = np.array([0.05, 0.05, 0.07], F)[:, None]
        cold = np.array([0.25, 0.48, 1.0], F)[:, None]
        hot = np.array([1.0, 0.30, 0.18], F)[:, None]
        div = np.where(scaled < 0, _mix(neutral, cold, opacity), _mix(neutral, hot, opacity))
        fieldc = (div * opacity + sky * (F(1) - opacity)) + rim
    else:
        glow = glow * (march * inverse_path)
        fade = np.exp(-glow)
        fieldc = ((F(1) - fade) + sky * fade) + rim
    colour = np.where(hit, fieldc, sky)
    # Scrub bar.
    if view.scrub:
        height_bar = F(0.045)
        from_bottom = F(0.5) * (sy + F(1))
        position = F(0.5) * (sx + F(1))
        bar = np.repeat(np.array([0.12, 0.13, 0.16], F)[:, None], sx.size, axis=1)
        bar = np.where(position >= F(view.window_start), np.array([0.22, 0.30, 0.40], F)[:, None], bar)
        bar = np.where(position <= F(view.played), np.array([0.35, 0.62, 0.95], F)[:, None], bar)
        bar = np.where(np.abs(position - F(view.played)) < F(0.0025), np.array([1.0, 0.85, 0.45], F)[:, None], bar)
        softness = _smooth(height_bar, height_bar * F(0.6), from_bottom)
        alpha = np.where(from_bottom > height_bar, F(0), F(0.55) + F(0.45) * softness)
        colour = _mix(colour, bar, alpha)
    else:
        colour = _mix(colour, np.zeros_like(colour), F(0))
    out = np.empty((sx.size, 4), np.uint8)
    for c in range(3):
        out[:, c] = _srgb8(colour[c].astype(F))
    out[:, 3] = 255
    return out.reshape(height, width, 4)
