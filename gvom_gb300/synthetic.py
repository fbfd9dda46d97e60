"""Seeded synthetic lidar scenes: the workload generator for tests and benchmarks.

The reference publishes no dataset (its numbers come from live RELLIS vehicle
runs, README.md:16-17), so every measured or parity-checked scan here is made
by this module from fixed seeds:

* terrain: a sum of 6 sinusoids (amplitude U[0, 0.5] m, wavelength U[2, 20] m,
  uniform direction and phase), 5 axis-aligned flat-topped boxes 0.3-1.5 m
  tall (footprint sides U[0.5, 3] m) and 2 rectangular ditches 0.5 m deep
  (length U[2, 6] m, width U[0.5, 1.5] m);
* lidar: ``beams x columns`` rays, elevation evenly spread over
  [-22.5 deg, 22.5 deg], azimuth evenly spaced, mounted 1.0 m above the ground
  under the vehicle, Gaussian range noise sigma = 0.02 m, 60 m maximum range;
  a ray with no return inside 60 m is emitted at 60 m so the point count is
  fixed;
* points are returned in the sensor frame together with the sensor->world
  4x4 transform and the sensor origin (the ``ego_position`` the mapper gets);
* trajectory: 0.4 m per scan, yaw step U[-3 deg, 3 deg];
* optional world-fixed vegetation (uniform 0-1.5 m above ground, a given
  density per m^2) appended when inside the map footprint, optional whole-beam
  dropout and an optional world offset (to stress far-from-origin precision).

Seeds: terrain 0, range noise 1, trajectory 2, dropout 3, arrivals 4.

Ray casting runs in torch (float64) on whatever device is given, so large
scans are generated on the GPU in milliseconds and small test scans on CPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

SEED_TERRAIN = 0
SEED_NOISE = 1
SEED_TRAJECTORY = 2
SEED_DROPOUT = 3
SEED_ARRIVALS = 4


@dataclass
class Terrain:
    """World-fixed heightfield: sinusoids + boxes (raise) + ditches (lower)."""

    amp: np.ndarray
    kx: np.ndarray
    ky: np.ndarray
    phase: np.ndarray
    boxes: np.ndarray  # (n, 5): x0, x1, y0, y1, top_z
    ditches: np.ndarray  # (n, 4): x0, x1, y0, y1
    ditch_depth: float = 0.5
    offset: tuple = (0.0, 0.0, 0.0)

    @staticmethod
    def make(seed: int = SEED_TERRAIN, extent: float = 40.0, n_sin: int = 6,
             n_boxes: int = 5, n_ditches: int = 2, path_len: float = 40.0,
             offset=(0.0, 0.0, 0.0), keepout: float = 3.0) -> "Terrain":
        rng = np.random.default_rng(seed)
        amp = rng.uniform(0.0, 0.5, n_sin)
        lam = rng.uniform(2.0, 20.0, n_sin)
        th = rng.uniform(0.0, 2 * np.pi, n_sin)
        phase = rng.uniform(0.0, 2 * np.pi, n_sin)
        kx = 2 * np.pi / lam * np.cos(th)
        ky = 2 * np.pi / lam * np.sin(th)
        t = Terrain(amp, kx, ky, phase, np.zeros((0, 5)), np.zeros((0, 4)),
                    offset=tuple(float(v) for v in offset))
        boxes = []
        for _ in range(n_boxes):
            # Place obstacles beside the path (x in [-extent/4, path_len + extent/4]),
            # at least `keepout` metres off the path centre line (y = 0).
            cx = rng.uniform(-extent / 4, path_len + extent / 4)
            cy = rng.uniform(keepout, extent / 2) * rng.choice([-1.0, 1.0])
            sx, sy = rng.uniform(0.5, 3.0, 2)
            h = rng.uniform(0.3, 1.5)
            top = float(t._sin_height_np(cx, cy)) + h
            boxes.append((cx - sx / 2, cx + sx / 2, cy - sy / 2, cy + sy / 2, top))
        ditches = []
        for _ in range(n_ditches):
            cx = rng.uniform(0.0, path_len)
            cy = rng.uniform(keepout, extent / 2) * rng.choice([-1.0, 1.0])
            length = rng.uniform(2.0, 6.0)
            width = rng.uniform(0.5, 1.5)
            if rng.uniform() < 0.5:
                sx, sy = length, width
            else:
                sx, sy = width, length
            ditches.append((cx - sx / 2, cx + sx / 2, cy - sy / 2, cy + sy / 2))
        t.boxes = np.array(boxes, dtype=np.float64).reshape(-1, 5)
        t.ditches = np.array(ditches, dtype=np.float64).reshape(-1, 4)
        return t

    def _sin_height_np(self, x, y):
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        h = np.zeros(np.broadcast(x, y).shape)
        for a, kx, ky, ph in zip(self.amp, self.kx, self.ky, self.phase):
            h = h + a * np.sin(kx * x + ky * y + ph)
        return h

    def height(self, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
        """Surface height at local (offset-free) coordinates, float64 tensors."""
        h = torch.zeros_like(x)
        for a, kx, ky, ph in zip(self.amp, self.kx, self.ky, self.phase):
            h = h + float(a) * torch.sin(float(kx) * x + float(ky) * y + float(ph))
        for x0, x1, y0, y1 in self.ditches:
            m = (x >= x0) & (x <= x1) & (y >= y0) & (y <= y1)
            h = torch.where(m, h - self.ditch_depth, h)
        for x0, x1, y0, y1, top in self.boxes:
            m = (x >= x0) & (x <= x1) & (y >= y0) & (y <= y1)
            h = torch.where(m, torch.clamp(h, min=float(top)), h)
        return h


@dataclass
class Lidar:
    beams: int = 32
    columns: int = 512
    el_min_deg: float = -22.5
    el_max_deg: float = 22.5
    max_range: float = 60.0
    noise_sigma: float = 0.02
    mount_height: float = 1.0
    # mounting on the vehicle: offset in the vehicle frame (m), yaw and pitch (deg)
    mount_x: float = 0.0
    mount_y: float = 0.0
    mount_yaw_deg: float = 0.0
    mount_pitch_deg: float = 0.0

    @property
    def n_points(self) -> int:
        return self.beams * self.columns

    def directions(self) -> np.ndarray:
        """Unit ray directions in the sensor frame, beam-major (row = beam)."""
        el = np.deg2rad(np.linspace(self.el_min_deg, self.el_max_deg, self.beams))
        az = np.arange(self.columns) * (2 * np.pi / self.columns)
        el, az = np.meshgrid(el, az, indexing="ij")
        d = np.stack([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)], -1)
        return d.reshape(-1, 3)


@dataclass
class Pose:
    x: float
    y: float
    yaw: float


def make_trajectory(n_scans: int, step: float = 0.4, yaw_step_deg: float = 3.0,
                    seed: int = SEED_TRAJECTORY) -> list[Pose]:
    rng = np.random.default_rng(seed)
    poses = []
    x = y = yaw = 0.0
    for _ in range(n_scans):
        poses.append(Pose(x, y, yaw))
        yaw += math.radians(rng.uniform(-yaw_step_deg, yaw_step_deg))
        x += step * math.cos(yaw)
        y += step * math.sin(yaw)
    return poses


@dataclass
class Vegetation:
    """World-fixed soft-obstacle points: `density` per m^2, 0-1.5 m above ground."""

    xyz: np.ndarray  # (n, 3) local (offset-free) world coordinates

    @staticmethod
    def make(terrain: Terrain, x_range, y_range, density: float = 20.0,
             max_height: float = 1.5, seed: int = SEED_TERRAIN + 100) -> "Vegetation":
        rng = np.random.default_rng(seed)
        area = (x_range[1] - x_range[0]) * (y_range[1] - y_range[0])
        n = int(round(area * density))
        x = rng.uniform(x_range[0], x_range[1], n)
        y = rng.uniform(y_range[0], y_range[1], n)
        g = terrain.height(torch.from_numpy(x), torch.from_numpy(y)).numpy()
        z = g + rng.uniform(0.0, max_height, n)
        return Vegetation(np.stack([x, y, z], -1))


@dataclass
class Scan:
    points: np.ndarray  # (N, 3) sensor frame, float32
    transform: np.ndarray  # (4, 4) sensor -> world
    ego: tuple  # sensor origin in world coordinates (float64)
    n_lidar: int = 0
    n_veg: int = 0
    meta: dict = field(default_factory=dict)


def _pose_matrix(pose: Pose, z: float, offset, lidar: "Lidar | None" = None) -> np.ndarray:
    c, s = math.cos(pose.yaw), math.sin(pose.yaw)
    T = np.eye(4)
    T[:3, :3] = [[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]]
    T[:3, 3] = [pose.x + offset[0], pose.y + offset[1], z + offset[2]]
    if lidar is not None and (lidar.mount_x or lidar.mount_y or lidar.mount_yaw_deg or lidar.mount_pitch_deg):
        my, mp = math.radians(lidar.mount_yaw_deg), math.radians(lidar.mount_pitch_deg)
        Rz = np.array([[math.cos(my), -math.sin(my), 0.0], [math.sin(my), math.cos(my), 0.0], [0.0, 0.0, 1.0]])
        Ry = np.array([[math.cos(mp), 0.0, math.sin(mp)], [0.0, 1.0, 0.0], [-math.sin(mp), 0.0, math.cos(mp)]])
        T[:3, 3] += T[:3, :3] @ np.array([lidar.mount_x, lidar.mount_y, 0.0])
        T[:3, :3] = T[:3, :3] @ Rz @ Ry
    return T


def cast_rays(terrain: Terrain, origin: np.ndarray, dirs: np.ndarray, max_range: float,
              device="cpu", coarse: float = 0.2, refine_iters: int = 14,
              chunk: int = 16384, dtype=None) -> np.ndarray:
    """First intersection range of each ray with the surface (max_range if none).

    Runs in float64 on CPU; on a GPU it defaults to float32 (coordinates are
    local, offset-free, so float32 resolves ~1e-5 m)."""
    if dtype is None:
        dtype = torch.float64 if str(device) == "cpu" else torch.float32
    o = torch.tensor(origin, dtype=dtype, device=device)
    d_all = torch.as_tensor(dirs, dtype=dtype, device=device)
    ts = torch.arange(coarse, max_range + 1e-9, coarse, dtype=dtype, device=device)
    out = torch.full((d_all.shape[0],), max_range, dtype=dtype, device=device)
    for s in range(0, d_all.shape[0], chunk):
        d = d_all[s:s + chunk]
        p = o[None, None, :] + ts[None, :, None] * d[:, None, :]
        below = p[..., 2] < terrain.height(p[..., 0], p[..., 1])
        hit_any = below.any(dim=1)
        first = torch.argmax(below.to(torch.int8), dim=1)
        hi = ts[first]
        lo = torch.where(first > 0, ts[(first - 1).clamp(min=0)], torch.zeros_like(hi))
        for _ in range(refine_iters):
            mid = 0.5 * (lo + hi)
            pm = o[None, :] + mid[:, None] * d
            b = pm[:, 2] < terrain.height(pm[:, 0], pm[:, 1])
            hi = torch.where(b, mid, hi)
            lo = torch.where(b, lo, mid)
        r = torch.where(hit_any, hi, torch.full_like(hi, max_range))
        out[s:s + chunk] = r
    return out.cpu().double().numpy()


def make_scan(terrain: Terrain, lidar: Lidar, pose: Pose, scan_index: int = 0,
              vegetation: Vegetation | None = None, footprint: float | None = None,
              dropout: float = 0.0, transform_dtype=np.float32, device="cpu",
              noise_seed: int = SEED_NOISE, dropout_seed: int = SEED_DROPOUT) -> Scan:
    """One lidar scan at `pose`; see the module docstring for the model."""
    off = terrain.offset
    g = float(terrain.height(torch.tensor([pose.x], dtype=torch.float64),
                             torch.tensor([pose.y], dtype=torch.float64))[0])
    z_sensor = g + lidar.mount_height
    T = _pose_matrix(pose, z_sensor, off, lidar)
    R = T[:3, :3]
    d_s = lidar.directions()
    keep = np.ones(d_s.shape[0], dtype=bool)
    if dropout > 0.0:
        rng_d = np.random.default_rng([dropout_seed, scan_index])
        beam_drop = rng_d.uniform(size=lidar.beams) < dropout
        keep = np.repeat(~beam_drop, lidar.columns)
    d_s = d_s[keep]
    d_w = d_s @ R.T
    origin_local = np.array([pose.x, pose.y, z_sensor])
    if lidar.mount_x or lidar.mount_y:
        origin_local = T[:3, 3] - np.asarray(off, dtype=np.float64)
    r = cast_rays(terrain, origin_local, d_w, lidar.max_range, device=device)
    rng_n = np.random.default_rng([noise_seed, scan_index])
    r = r + rng_n.normal(0.0, lidar.noise_sigma, r.shape)
    r = np.clip(r, 0.05, None)  # zero-range points are never emitted
    pts = r[:, None] * d_s
    n_lidar = pts.shape[0]
    n_veg = 0
    if vegetation is not None and footprint is not None:
        v = vegetation.xyz
        m = (np.abs(v[:, 0] - pose.x) < footprint / 2) & (np.abs(v[:, 1] - pose.y) < footprint / 2)
        vw = v[m] - origin_local[None, :]
        vs = vw @ R  # world -> sensor: R^T (p - t)
        pts = np.concatenate([pts, vs], 0)
        n_veg = vs.shape[0]
    ego = (float(T[0, 3]), float(T[1, 3]), float(T[2, 3]))
    return Scan(pts.astype(np.float32), T.astype(transform_dtype), ego, n_lidar, n_veg,
                meta={"pose": pose, "scan_index": scan_index})


# ---------------------------------------------------------------------------
# Named workloads (grid parameters + scene recipe)
# ---------------------------------------------------------------------------

LAUNCH_THRESHOLDS = dict(
    min_distance=1.0, positive_obstacle_threshold=0.5, negative_obstacle_threshold=0.5,
    slope_obsacle_threshold=0.3, robot_height=2.0, robot_radius=4.0,
    ground_to_lidar_height=1.0, xy_eigen_dist=1, z_eigen_dist=1)


@dataclass
class Workload:
    name: str
    res: float
    xy_size: int
    z_size: int
    buffer_size: int
    beams: int
    columns: int
    n_scans: int = 1
    veg_density: float = 0.0
    offset: tuple = (0.0, 0.0, 0.0)
    transform_dtype: type = np.float32

    def gvom_args(self):
        t = LAUNCH_THRESHOLDS
        return (self.res, self.res, self.xy_size, self.z_size, self.buffer_size,
                t["min_distance"], t["positive_obstacle_threshold"],
                t["negative_obstacle_threshold"], t["slope_obsacle_threshold"],
                t["robot_height"], t["robot_radius"], t["ground_to_lidar_height"],
                t["xy_eigen_dist"], t["z_eigen_dist"])

    @property
    def voxels(self) -> int:
        return self.xy_size * self.xy_size * self.z_size


WORKLOADS = {
    # one 32x512 scan, 0.2 m voxels, 128x128x32, buffer 2 (CPU-runnable case)
    "small_32x512": Workload("small_32x512", 0.2, 128, 32, 2, 32, 512),
    # OS1-64 shape + vegetation (20 points/m^2), 0.15 m, 256x256x64, buffer 4, 100-scan path
    "os1_64_veg": Workload("os1_64_veg", 0.15, 256, 64, 4, 64, 1024, n_scans=100, veg_density=20.0),
    # OS1-128x2048, 0.1 m, 512x512x96, buffer 8, world offset 1e4 m
    "os1_128_far": Workload("os1_128_far", 0.1, 512, 96, 8, 128, 2048, offset=(1.0e4, 0.0, 0.0)),
}


def scene_for(w: Workload, path_len: float | None = None):
    """Terrain (+ vegetation) covering the workload's trajectory and map footprint."""
    if path_len is None:
        path_len = max(1, w.n_scans) * 0.4
    extent = w.xy_size * w.res
    terrain = Terrain.make(SEED_TERRAIN, extent=extent, path_len=path_len, offset=w.offset)
    veg = None
    if w.veg_density > 0.0:
        veg = Vegetation.make(terrain, (-extent / 2 - 1, path_len + extent / 2 + 1),
                              (-path_len / 2 - extent / 2 - 1, path_len / 2 + extent / 2 + 1),
                              density=w.veg_density)
    return terrain, veg


def make_workload_scans(w: Workload, n: int | None = None, device="cpu", dropout: float = 0.0):
    n = w.n_scans if n is None else n
    # the scene of the workload's own n_scans; longer runs extend it along the path
    terrain, veg = scene_for(w, None if n <= w.n_scans else n * 0.4)
    lidar = Lidar(beams=w.beams, columns=w.columns)
    poses = make_trajectory(n)
    return [make_scan(terrain, lidar, p, i, vegetation=veg, footprint=w.xy_size * w.res,
                      dropout=dropout, transform_dtype=w.transform_dtype, device=device)
            for i, p in enumerate(poses)]


# ---------------------------------------------------------------------------
# Batched form: several sensors per vehicle, every step's scans in one launch
# ---------------------------------------------------------------------------

# four mountings: front, rear, left, right (offset m, yaw deg, pitch deg)
MOUNTS = ((0.6, 0.0, 0.0, -5.0), (-0.6, 0.0, 180.0, -5.0), (0.0, 0.4, 90.0, -10.0), (0.0, -0.4, -90.0, -10.0))


@dataclass
class Sensor:
    beams: int
    columns: int
    dropout: float  # probability that a whole beam is missing in a scan
    mount: int      # index into MOUNTS


@dataclass
class BatchedWorkload:
    name: str
    res: float
    xy_size: int
    z_size: int
    buffer_size: int
    sensors: tuple
    n_steps: int = 24
    transform_dtype: type = np.float32

    def gvom_args(self):
        return Workload(self.name, self.res, self.xy_size, self.z_size, self.buffer_size, 0, 0).gvom_args()

    @property
    def voxels(self) -> int:
        return self.xy_size * self.xy_size * self.z_size

    def lidar(self, k: int) -> Lidar:
        sn = self.sensors[k]
        mx, my, yaw, pitch = MOUNTS[sn.mount]
        return Lidar(beams=sn.beams, columns=sn.columns, mount_x=mx, mount_y=my, mount_yaw_deg=yaw,
                     mount_pitch_deg=pitch)


BATCHED = {
    # 8 sensors of 16,384-262,144 points (before 0-60 % beam dropout) on 4 mountings;
    # 0.15 m voxels, 256 x 256 x 64, buffer 16 (two steps of 8 scans)
    "batched_8": BatchedWorkload("batched_8", 0.15, 256, 64, 16, (
        Sensor(32, 512, 0.0, 0), Sensor(64, 512, 0.1, 1), Sensor(64, 1024, 0.2, 2), Sensor(128, 1024, 0.3, 3),
        Sensor(64, 2048, 0.4, 0), Sensor(128, 2048, 0.6, 1), Sensor(32, 1024, 0.5, 2), Sensor(128, 512, 0.15, 3))),
}


def make_batched_steps(w: BatchedWorkload, n_steps: int | None = None, device="cpu") -> list:
    """`n_steps` steps along the seeded trajectory, each a list of one scan per
    sensor (sensor k's beam dropout re-drawn per step from seed 3)."""
    n_steps = w.n_steps if n_steps is None else n_steps
    extent = w.xy_size * w.res
    terrain = Terrain.make(SEED_TERRAIN, extent=extent, path_len=max(1, n_steps) * 0.4)
    poses = make_trajectory(n_steps)
    steps = []
    for i, p in enumerate(poses):
        scans = []
        for k, sn in enumerate(w.sensors):
            scans.append(make_scan(terrain, w.lidar(k), p, i * len(w.sensors) + k, dropout=sn.dropout,
                                   transform_dtype=w.transform_dtype, device=device))
        steps.append(scans)
    return steps
