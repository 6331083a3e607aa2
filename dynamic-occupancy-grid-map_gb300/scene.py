"""Seeded synthetic scenes and measurement grids for the DOGM update.

The reference feeds updateGrid from a lidar simulator and an OpenGL polar-to-cartesian
renderer (dogm/demo/simulator, laser_to_meas_grid.cu:25-70).  Neither is part of the update,
and no graphics stack is available, so the measurement grids here come from a numpy model
with the workload shapes of the benchmark configurations: rectangular moving obstacles, a
360-degree lidar at the grid centre with Gaussian range noise, and an inverse sensor model
that puts occupied mass 0.7 at the hit cell and free mass 0.4 before it.  Masses are clamped
to [1e-5, 1 - 1e-5] like the reference's inverse sensor model (measurement_grid.cu:81-82);
likelihood and p_A are 1 (measurement_grid.cu:129-130).
"""
from __future__ import annotations

import numpy as np

FILTER = dict(persistence_prob=0.99, stddev_process_noise_position=0.1, stddev_process_noise_velocity=2.0,
              birth_prob=0.02, stddev_velocity=30.0, init_max_velocity=12.0, freespace_discount=0.01)

# Workloads: "small" is the reference's CPU-runnable case (50 m at 0.2 m), "large" the
# 2M-particle / 1.44M-cell grid the headline metric is quoted on, "precision" the 2048^2 grid.
CONFIGS = {
    "small": dict(size=50.0, resolution=0.2, particle_count=300_000, new_born_particle_count=30_000, frames=20,
                  vehicles=10, pedestrians=0, beams=1080, ego_speed=0.0, yaw_rate=0.0, range_noise=0.05),
    "large": dict(size=120.0, resolution=0.1, particle_count=2_000_000, new_born_particle_count=200_000, frames=50,
                  vehicles=40, pedestrians=30, beams=2160, ego_speed=10.0, yaw_rate=None, range_noise=0.05),
    "precision": dict(size=204.8, resolution=0.1, particle_count=8_000_000, new_born_particle_count=800_000,
                      frames=30, vehicles=120, pedestrians=60, beams=4096, ego_speed=10.0, yaw_rate=None,
                      range_noise=0.05),
}

DT = 0.1
OCC_HIT = 0.7
FREE_BEFORE = 0.4
EPS = 1e-5


def grid_size(cfg: dict) -> int:
    return int(np.float32(cfg["size"]) / np.float32(cfg["resolution"]))


def params_dict(cfg: dict) -> dict:
    d = dict(size=cfg["size"], resolution=cfg["resolution"], particle_count=cfg["particle_count"],
             new_born_particle_count=cfg["new_born_particle_count"])
    d.update(FILTER)
    return d


class Scene:
    """Objects and ego motion in world coordinates; the grid is ego-centred."""

    def __init__(self, cfg: dict, seed: int = 0):
        self.cfg = cfg
        rng = np.random.default_rng(seed)
        self.rng = rng
        size, res = float(cfg["size"]), float(cfg["resolution"])
        self.gs = grid_size(cfg)
        n_v, n_p = int(cfg["vehicles"]), int(cfg["pedestrians"])
        n = n_v + n_p
        half = size / 2.0
        # spawn uniformly in the initial grid, away from the sensor
        pos = rng.uniform(-half * 0.9, half * 0.9, size=(n, 2))
        near = np.hypot(pos[:, 0], pos[:, 1]) < 3.0
        pos[near] += np.sign(pos[near] + 1e-3) * 4.0
        self.pos0 = pos
        self.heading = rng.uniform(-np.pi, np.pi, size=n)
        speed = np.concatenate([rng.uniform(0.0, 15.0, n_v), rng.uniform(0.0, 2.0, n_p)])
        self.vel = speed[:, None] * np.stack([np.cos(self.heading), np.sin(self.heading)], axis=1)
        self.half_len = np.concatenate([np.full(n_v, 2.25), np.full(n_p, 0.25)])
        self.half_wid = np.concatenate([np.full(n_v, 1.0), np.full(n_p, 0.25)])
        yr = cfg.get("yaw_rate")
        self.yaw_rate = float(rng.uniform(-0.2, 0.2)) if yr is None else float(yr)
        self.ego_speed = float(cfg["ego_speed"])
        self.beams = int(cfg["beams"])
        self.max_range = half * np.sqrt(2.0)
        # polar coordinates of the cell centres relative to the sensor (grid centre).  Cell
        # indices run against the world axes: the reference moves the grid content by
        # +int(d / resolution) cells when the ego moves by +d (dogm.cu:177-178 with
        # ego_motion_compensation.cu:20,40), so a static world point keeps its cell only
        # if index = (half - world offset) / resolution.
        c = half - (np.arange(self.gs, dtype=np.float64) + 0.5) * res
        cx, cy = np.meshgrid(c, c)  # row = y, column = x -> index x + gs * y
        self.cell_r = np.hypot(cx, cy).ravel()
        ang = np.mod(np.arctan2(cy, cx).ravel(), 2 * np.pi)
        self.cell_beam = (np.floor(ang / (2 * np.pi) * self.beams + 0.5).astype(np.int64)) % self.beams
        self.band = res * 0.5 * np.sqrt(2.0)
        th = 2 * np.pi * np.arange(self.beams) / self.beams
        self.beam_dir = np.stack([np.cos(th), np.sin(th)], axis=1)

    def ego_pose(self, k: int) -> tuple[float, float, float]:
        """Ego pose at frame k (constant speed and yaw rate), world frame."""
        if self.yaw_rate == 0.0:
            return self.ego_speed * DT * k, 0.0, 0.0
        x = y = psi = 0.0
        for _ in range(k):
            x += self.ego_speed * np.cos(psi) * DT
            y += self.ego_speed * np.sin(psi) * DT
            psi += self.yaw_rate * DT
        return x, y, psi

    def ranges(self, k: int, ego: tuple[float, float]) -> tuple[np.ndarray, np.ndarray]:
        t = k * DT
        centre = self.pos0 + self.vel * t - np.asarray(ego)[None, :]
        cos_h, sin_h = np.cos(self.heading), np.sin(self.heading)
        ax = np.stack([cos_h, sin_h], 1)
        ay = np.stack([-sin_h, cos_h], 1)
        corners = []
        for sx, sy in ((1, 1), (-1, 1), (-1, -1), (1, -1)):
            corners.append(centre + sx * self.half_len[:, None] * ax + sy * self.half_wid[:, None] * ay)
        a = np.concatenate([corners[i] for i in range(4)], 0)
        b = np.concatenate([corners[(i + 1) % 4] for i in range(4)], 0)
        e = b - a  # (S, 2)
        d = self.beam_dir  # (R, 2)
        denom = d[:, None, 0] * e[None, :, 1] - d[:, None, 1] * e[None, :, 0]
        with np.errstate(divide="ignore", invalid="ignore"):
            tt = (a[None, :, 0] * e[None, :, 1] - a[None, :, 1] * e[None, :, 0]) / denom
            ss = (a[None, :, 0] * d[:, None, 1] - a[None, :, 1] * d[:, None, 0]) / denom
        ok = (np.abs(denom) > 1e-12) & (tt > 0) & (ss >= 0) & (ss <= 1)
        tt = np.where(ok, tt, np.inf)
        r = tt.min(axis=1)
        hit = np.isfinite(r) & (r < self.max_range)
        r = np.where(hit, r + self.rng.normal(0.0, self.cfg["range_noise"], size=r.shape), self.max_range)
        return np.maximum(r, 0.0), hit

    def frame(self, k: int) -> tuple[np.ndarray, float, float, float]:
        """Measurement grid (grid_size^2 x {free, occ, likelihood, p_A}, float32) and ego pose."""
        ex, ey, psi = self.ego_pose(k)
        r, hit = self.ranges(k, (ex, ey))
        rb = r[self.cell_beam]
        hb = hit[self.cell_beam]
        free = np.where(self.cell_r < rb - self.band, FREE_BEFORE, 0.0)
        occ = np.where(hb & (np.abs(self.cell_r - rb) <= self.band), OCC_HIT, 0.0)
        free = np.where(occ > 0, 0.0, free)
        m = np.empty((self.gs * self.gs, 4), np.float32)
        m[:, 0] = np.clip(free, EPS, 1.0 - EPS)
        m[:, 1] = np.clip(occ, EPS, 1.0 - EPS)
        m[:, 2] = 1.0
        m[:, 3] = 1.0
        return m, float(ex), float(ey), float(psi)


def random_measurements(gs: int, seed: int, occ_fraction: float = 0.02) -> np.ndarray:
    """Unstructured measurement grid for small parity cases: random occupied and free cells."""
    rng = np.random.default_rng(seed)
    c = gs * gs
    m = np.zeros((c, 4), np.float32)
    u = rng.random(c)
    occ = u < occ_fraction
    fre = (u >= occ_fraction) & (u < 0.5)
    m[occ, 1] = rng.uniform(0.3, 0.95, occ.sum()).astype(np.float32)
    m[fre, 0] = rng.uniform(0.1, 0.8, fre.sum()).astype(np.float32)
    m[:, 0] = np.clip(m[:, 0], EPS, 1 - EPS)
    m[:, 1] = np.clip(m[:, 1], EPS, 1 - EPS)
    m[:, 2] = 1.0
    m[:, 3] = 1.0
    return m


def stream_configs(n: int, seed: int = 0, side_min: int = 128, side_max: int = 1024,
                   density: float = 0.004) -> list[dict]:
    """Uneven sensor streams for the batched and serving workloads: square grids with a side
    drawn log-uniform in [side_min, side_max] cells at a resolution U(0.1, 0.2) m, 1.5
    persistent particles per cell and 10 % newborns, and a static sensor among obstacles at
    `density` per square metre (the small workload's scene: 2 x 4.5 m vehicles at U(0, 15) m/s,
    1080 beams).  The size is chosen so that int(float(size) / float(resolution)) is the side."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        side = int(round(np.exp(rng.uniform(np.log(side_min), np.log(side_max)))))
        res = float(np.float32(rng.uniform(0.1, 0.2)))
        size = float(np.float32(side * res))
        while int(np.float32(size) / np.float32(res)) < side:
            size = float(np.nextafter(np.float32(size), np.float32(np.inf)))
        while int(np.float32(size) / np.float32(res)) > side:
            size = float(np.nextafter(np.float32(size), np.float32(0)))
        cells = side * side
        n_part = int(1.5 * cells)
        area = (side * res) ** 2
        out.append(dict(size=size, resolution=res, particle_count=n_part, new_born_particle_count=n_part // 10,
                        frames=2, vehicles=max(1, int(round(density * area))), pedestrians=0, beams=1080,
                        ego_speed=0.0, yaw_rate=0.0, range_noise=0.05))
    return out
