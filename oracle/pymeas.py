"""CPU restatement of the measurement-grid generation -- TEST INFRASTRUCTURE ONLY (the checker,
never the product).  numpy float32 operations in the order of the GPU kernels
(dynamic-occupancy-grid-map_gb300/csrc/k_meas.cu), which restate the reference's
  * inverse_sensor_model / combine_masses (dogm/demo/simulator/mapping/kernel/
    measurement_grid.cu:14-71, clamp :79-82),
  * the triangle fan of generateCircleSegmentVertices (opengl/renderer.cpp:11-31) drawn over a
    grid_size^2 viewport, the fragment shader's uv = (1 - s / (t + 1e-10), t)
    (opengl/shader.cpp:22-35), a bilinear fetch with border (0, 0) (opengl/texture.cpp:11-38)
    and the row flip of cartesianGridToMeasurementGridKernel (measurement_grid.cu:115-132).
Given the same polar grid the warp is bit-exact with the GPU; the inverse sensor model differs
only through exp (numpy's float32 exp against CUDA's expf, a few ulp)."""
from __future__ import annotations

import math

import numpy as np

F = np.float32
EPS = F(0.00001)


def polar_ism(ranges: np.ndarray, bins: int, resolution: float, sigma: float) -> np.ndarray:
    """(bins, beams, 2) float32 {occ, free} of one scan, clamped to [eps, 1 - eps]."""
    z = np.asarray(ranges, F)
    beams = z.size
    i = np.arange(bins, dtype=np.int64)[:, None]
    res, sg = F(resolution), F(sigma)
    free = F(0.15) + (i.astype(F) * (F(1.0) - F(0.15))) / F(bins)
    free = np.broadcast_to(free, (bins, beams)).astype(F)
    finite = np.isfinite(z)[None, :]
    zz = np.where(np.isfinite(z), z, F(0)).astype(F)
    r = (zz / res).astype(np.int64)[None, :]
    diff = (i - r).astype(F) * res
    e = ((F(-0.5) * diff) * diff) / (sg * sg)
    occ = F(0.95) * np.exp(e.astype(F)).astype(F)
    inside = i <= r
    o = np.where(inside, np.where(occ > free, occ, F(0)), np.where(occ > F(0.5), occ, F(0)))
    f = np.where(inside, np.where(occ > free, F(0), F(1) - free), F(0))
    o = np.where(finite, o, F(0))
    f = np.where(finite, f, F(1) - free)
    o = np.maximum(EPS, np.minimum(F(1) - EPS, o.astype(F)))
    f = np.maximum(EPS, np.minimum(F(1) - EPS, f.astype(F)))
    return np.stack([o, f], -1).astype(F)


def combine(prior: np.ndarray, m: np.ndarray) -> np.ndarray:
    """Dempster's rule for {occ, free} (combine_masses)."""
    po, pf, mo, mf = prior[..., 0], prior[..., 1], m[..., 0], m[..., 1]
    unk = (F(1) - po) - pf
    m_unk = (F(1) - mo) - mf
    K = pf * mo + po * mf
    den = F(1) - K
    occ = ((po * m_unk + unk * mo) + po * mo) / den
    fre = ((pf * m_unk + unk * mf) + pf * mf) / den
    return np.stack([occ, fre], -1).astype(F)


def fan_vertices(max_range: float, fov: float, grid_length: float, gs: int) -> dict:
    """The fan in window coordinates x 256 (renderer.cpp:11-31 with cos/sin in float)."""
    fov = F(fov)
    half = fov / F(2)
    start, end = F(90) - half, F(90) + half
    radius = F(2.0) * (F(max_range) / F(grid_length))
    half_gs = F(gs) / F(2)

    def snap(ndc):
        return int(math.floor(float((F(ndc) + F(1)) * half_gs) * 256.0 + 0.5))  # llround for x >= 0

    xs, ys, ss = [snap(0.0)], [snap(-1.0)], [F(0)]
    angle = int(start)
    while angle <= end:
        rad = F(angle * math.pi / F(180.0))
        xv, yv = np.cos(rad, dtype=F), np.sin(rad, dtype=F)
        xs.append(snap(F(0) + radius * xv))
        ys.append(snap(F(-1) + radius * yv))
        ss.append((F(angle) - start) / fov)
        angle += 1
    return {"x256": np.array(xs, np.int64), "y256": np.array(ys, np.int64), "s": np.array(ss, F),
            "first_angle": int(start)}


def _edge(ax, ay, bx, by, px, py):
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax)


def _owns(e, ax, ay, bx, by):
    return (e > 0) | ((e == 0) & ((by < ay) | ((by == ay) & (bx < ax))))


def warp(polar: np.ndarray, gs: int, fan: dict) -> np.ndarray:
    """(gs*gs, 4) float32 measurement cells {free, occ, likelihood, p_A} from the polar grid."""
    bins, beams = polar.shape[0], polar.shape[1]
    vx, vy, sv, a0 = fan["x256"], fan["y256"], fan["s"], fan["first_angle"]
    nv = vx.size
    y, x = np.divmod(np.arange(gs * gs, dtype=np.int64), gs)
    px, py = 256 * x + 128, 256 * y + 128
    cx, cy = vx[0], vy[0]
    ang = np.degrees(np.arctan2((py - cy).astype(np.float64), (px - cx).astype(np.float64)))
    k0 = np.floor(ang).astype(np.int64) - a0 + 1
    chosen = np.full(gs * gs, -1, np.int64)
    for d in (-1, 0, 1):
        tri = k0 + d
        valid = (tri >= 1) & (tri <= nv - 2) & (chosen < 0)
        t = np.clip(tri, 1, nv - 2)
        ax, ay, bx, by = vx[t], vy[t], vx[t + 1], vy[t + 1]
        ok = (_owns(_edge(ax, ay, bx, by, px, py), ax, ay, bx, by) & _owns(_edge(bx, by, cx, cy, px, py), bx, by, cx, cy)
              & _owns(_edge(cx, cy, ax, ay, px, py), cx, cy, ax, ay))
        chosen = np.where(valid & ok, t, chosen)
    cov = chosen >= 0
    t = np.where(cov, chosen, 1)
    ax, ay, bx, by = vx[t], vy[t], vx[t + 1], vy[t + 1]
    area = _edge(cx, cy, ax, ay, bx, by).astype(F)
    la = _edge(bx, by, cx, cy, px, py).astype(F) / area
    lb = _edge(cx, cy, ax, ay, px, py).astype(F) / area
    tt = (la + lb).astype(F)
    s = (la * sv[t] + lb * sv[t + 1]).astype(F)
    u = F(1) - s / (tt + F(1e-10))
    v = tt
    xs = u * F(beams) - F(0.5)
    ys = v * F(bins) - F(0.5)
    fx, fy = np.floor(xs), np.floor(ys)
    a, b = (xs - fx).astype(F), (ys - fy).astype(F)
    i0, j0 = fx.astype(np.int64), fy.astype(np.int64)

    def tex(i, j):
        inside = (i >= 0) & (i < beams) & (j >= 0) & (j < bins)
        return np.where(inside[:, None], polar[np.clip(j, 0, bins - 1), np.clip(i, 0, beams - 1)], F(0))

    t00, t10, t01, t11 = tex(i0, j0), tex(i0 + 1, j0), tex(i0, j0 + 1), tex(i0 + 1, j0 + 1)
    w00 = (F(1) - a) * (F(1) - b)
    w10 = a * (F(1) - b)
    w01 = (F(1) - a) * b
    w11 = a * b
    val = ((w00[:, None] * t00 + w10[:, None] * t10) + w01[:, None] * t01) + w11[:, None] * t11
    val = np.where(cov[:, None], val, F(0)).astype(F)
    out = np.zeros((gs * gs, 4), F)
    row = (gs - 1 - y) * gs + x
    out[row, 0] = val[:, 1]  # free = green
    out[row, 1] = val[:, 0]  # occ = red
    out[:, 2] = 1
    out[:, 3] = 1
    return out


def dynamic_cells(cells: np.ndarray, gs: int, min_occ: float, min_vel: float) -> dict:
    """computeCellsWithVelocity (dogm/demo/utils/image_creation.cpp:24-66) in the GPU's FP32
    order: pignistic occupancy, v^T Sigma^-1 v by the closed-form 2 x 2 inverse (0 when
    singular), kept cells in row-major order."""
    occ_m, free_m = cells["occ_mass"].astype(F), cells["free_mass"].astype(F)
    occ = occ_m + F(0.5) * ((F(1) - occ_m) - free_m)
    vx, vy, c = cells["var_x_vel"].astype(F), cells["var_y_vel"].astype(F), cells["covar_xy_vel"].astype(F)
    mx, my = cells["mean_x_vel"].astype(F), cells["mean_y_vel"].astype(F)
    det = vx * vy - c * c
    q = (vy * (mx * mx) - F(2) * (c * (mx * my))) + vx * (my * my)
    with np.errstate(divide="ignore", invalid="ignore"):
        m = np.where(det != 0, q / np.where(det != 0, det, F(1)), F(0)).astype(F)
    keep = (occ >= F(min_occ)) & (m >= F(min_vel))
    idx = np.flatnonzero(keep)
    return {"index": idx.astype(np.int32), "occupancy": occ[idx], "mahalanobis": m[idx],
            "x": (idx % gs).astype(F), "y": (idx // gs).astype(F)}
