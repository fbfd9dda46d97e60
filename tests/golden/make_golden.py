"""Generate the golden fixtures in tests/golden/ by running the REFERENCE mapper.

Runs the reference's own scripts/gvom.py, unchanged, from the reference
checkout named by $GVOM_REFERENCE (required) on the host through
the sequential numba stand-in in oracle/numba_shim, for a set of small scenes,
and writes each scene's inputs and the reference's outputs and internal state
(in canonical voxel order) to tests/golden/<scene>.npz.

The fixtures pin the C oracle: tests/test_oracle_golden.py checks that the
oracle reproduces every array here.  This script needs the reference checkout,
so it runs only in the build container; its outputs are committed.

    python tests/golden/make_golden.py [scene ...]
"""
from __future__ import annotations

import importlib.util
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle", "numba_shim"))
sys.path.insert(1, REPO)

import numba  # noqa: E402  (the stand-in)
from numba import cuda as shim_cuda  # noqa: E402

from oracle.canonical import canonical_map  # noqa: E402

REF = os.environ.get("GVOM_REFERENCE")
if not REF:
    raise SystemExit("set GVOM_REFERENCE to the reference checkout (the directory holding scripts/gvom.py)")


def load_reference():
    path = os.path.join(REF, "scripts", "gvom.py")
    spec = importlib.util.spec_from_file_location("gvom_reference", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.math = numba.math_proxy  # compiled-Numba typing of math.sqrt / math.floor
    return mod


# ---------------------------------------------------------------------------
# scenes: (params, ops); ops = [("P", points, ego, T or None), ("C",), ...]
# ---------------------------------------------------------------------------

def kat_params(X=16, Z=8, B=2, res=1.0, robot_radius=0.5, min_distance=0.5):
    return (res, res, X, Z, B, min_distance, 0.5, 0.5, 0.3, 2.0, robot_radius, 1.0, 1, 1)


def P(points, ego, T=None, dtype=np.float32):
    return ("P", np.asarray(points, dtype=dtype).reshape(-1, 3), tuple(float(v) for v in ego), T)


def scene_kat_rays():
    """Axis-aligned rays in 6 directions, a diagonal with a 3-way tie, a ray leaving the grid."""
    ego = (0.5, 0.5, 0.5)
    pts = [(5.5, 0.5, 0.5), (-4.5, 0.5, 0.5), (0.5, 5.5, 0.5), (0.5, -4.5, 0.5), (0.5, 0.5, 3.25),
           (0.5, 0.5, -2.5), (3.5, 3.5, 3.5), (30.5, 0.5, 0.5), (0.75, 0.6, 0.5),
           (0.3, 0.2, 0.1)]
    return kat_params(), [P(pts, ego), ("C",)]


def scene_kat_clear(n_pass):
    """Occupied voxel then `n_pass` rays through it in the next scan (clearing rule, gvom.py:1058)."""
    ego = (0.5, 0.5, 0.5)
    s1 = [(3.5, 0.5, 0.5)] * 3
    s2 = [(6.5, 0.5, 0.5)] * n_pass
    return kat_params(B=1), [P(s1, ego), ("C",), P(s2, ego), ("C",), ("C",)]


def scene_kat_shift():
    """Two slots whose origins differ by one voxel in every axis, then a third overwriting slot 0."""
    rng = np.random.default_rng(11)
    pts1 = rng.uniform(-6, 7, (200, 3)) * [1, 1, 0.5]
    pts2 = rng.uniform(-6, 7, (200, 3)) * [1, 1, 0.5] + 1.0
    pts3 = rng.uniform(-6, 7, (200, 3)) * [1, 1, 0.5] - 1.0
    return kat_params(B=2), [P(pts1, (0.5, 0.5, 0.5)), P(pts2, (1.5, 1.5, 1.5)), ("C",),
                             P(pts3, (-0.5, -0.5, -0.5)), ("C",)]


def scene_kat_planes():
    """A flat and a tilted ground patch plus a wall: slope, roughness, positive obstacles."""
    pts = []
    for x in np.arange(-7.25, 7.5, 0.5):
        for y in np.arange(-7.25, 7.5, 0.5):
            if x < 0:
                z = -1.5 + 0.05  # flat
            else:
                z = -1.5 + 0.05 + 0.15 * x  # tilted
            pts.append((x, y, z))
    for k in range(14):  # a dense wall column at (4.3, -5.7), many hits per voxel
        for rep in range(12):
            pts.append((4.3 + 0.01 * rep, -5.7, -1.4 + 0.25 * k))
    ego = (0.25, 0.25, 0.75)
    return kat_params(robot_radius=1.0), [P(pts, ego), ("C",)]


def scene_kat_guess():
    """Known heights with holes seen only as free space (guess_height, gvom.py:592-714)."""
    pts = []
    rng = np.random.default_rng(5)
    for x in np.arange(-7.5, 7.5, 1.0):
        for y in np.arange(-7.5, 7.5, 1.0):
            if (abs(x - 2.0) < 2.1 and abs(y + 1.0) < 1.6) or (x < -4 and y > 3):
                continue  # hole: rays pass over it, no return
            pts.append((x + rng.uniform(-0.3, 0.3), y + rng.uniform(-0.3, 0.3), -2.5 + rng.uniform(0, 0.4)))
    # rays that pass low over the holes and end far away
    for t in np.linspace(-3.0, 3.0, 25):
        pts.append((40.0, 40.0 * t / 3.0 - 10.0, -12.0))
        pts.append((-40.0, 40.0 * t / 3.0 + 10.0, -12.0))
    ego = (0.5, 0.5, 0.5)
    return kat_params(X=16, Z=8, robot_radius=0.5), [P(pts, ego), ("C",)]


def _cell_point(cx, cy, cz, f=(0.5, 0.5, 0.5)):
    """World point at fraction f inside voxel (cx, cy, cz) of the kat_params() grid (origin -8, -8, -4)."""
    return (cx - 8 + f[0], cy - 8 + f[1], cz - 4 + f[2])


# Point clusters of known covariance, one per voxel (offsets from the voxel centre, 1 m voxels);
# the eigenvalues of each voxel's covariance in closed form (tests/test_oracle_golden.py).
EIGEN_CLUSTERS = {
    "isotropic": ((12, 12, 2), [(0.25, 0, 0), (0, 0.25, 0), (0, 0, 0.25)]),
    "planar": ((4, 12, 2), [(0.25, 0, 0), (0, 0.25, 0)]),
    "linear": ((12, 4, 2), [(0.125, 0, 0), (0.25, 0, 0)]),
    "diagonal_line": ((4, 4, 2), [(0.125, 0.125, 0), (0.25, 0.25, 0)]),
    "tilted_plane": ((8, 13, 5), [(0.125, 0, 0.125), (0, 0.25, 0)]),
    "anisotropic": ((13, 8, 1), [(0.125, 0, 0), (0, 0.1875, 0), (0, 0, 0.25)]),
    "pair_a": ((8, 2, 1), [(0.25, 0, 0)]),
    "pair_b": ((9, 2, 1), [(0, 0.25, 0)]),
}


def scene_kat_eigen():
    """Voxels whose covariance has eigenvalues in closed form (isotropic, planar, linear, rotated,
    distinct), one single-point voxel and two adjacent voxels sharing their neighbourhoods; the
    same scan twice into two slots, then two combines (gvom.py:1249-1371, 888-980, 1423-1487)."""
    pts = []
    for (c, offs) in EIGEN_CLUSTERS.values():
        ctr = np.array(_cell_point(*c))
        for o in offs:
            pts += [tuple(ctr + o), tuple(ctr - np.asarray(o))]
    pts.append(_cell_point(2, 8, 1, (0.6, 0.3, 0.55)))  # single point: zero covariance
    ego = (0.5, 0.5, 0.5)
    return kat_params(B=2), [P(pts, ego), P(pts, ego), ("C",), ("C",)]


def _stack(cx, cy, cz, n, entry):
    """`n` points in voxel (cx, cy, cz).  With `entry` they sit just past the face that a ray from
    (0.5, 0.5, 0.5) enters by, so that its last march step falls short of the voxel (one count per
    point); otherwise near the middle, where the last step counts the voxel again (two)."""
    out = []
    for k in range(n):
        if entry:
            fx = 0.5 if cx == 8 else (0.05 + 0.002 * k if cx > 8 else 0.95 - 0.002 * k)
            fy = 0.5 if cy == 8 else (0.05 + 0.003 * k if cy > 8 else 0.95 - 0.003 * k)
        else:
            fx, fy = 0.3 + 0.4 * k / max(1, n - 1), 0.6
        out.append(_cell_point(cx, cy, cz, (fx, fy, 0.4 + 0.01 * k)))
    return out


# Columns for the positive-obstacle band (gvom.py:515-555): cell -> (ground voxel z, min-height
# fraction, {z: (points, entry)}).  With 1 m voxels, pos_thr 0.5 and robot_h 2 the band is
# [zg + 1, zg + 2] for a fraction below 0.5 and [zg + 2, zg + 2] from 0.5 on.
POSOBS_COLUMNS = {
    "A": ((12, 8), 1, 0.25, {2: (11, False), 3: (10, False)}),  # hit 10 at z=3 is left out
    "B": ((8, 12), 1, 0.5, {2: (20, True), 3: (11, False)}),    # band starts one voxel higher
    "C": ((4, 8), 1, 0.25, {2: (10, False), 3: (10, False)}),   # nothing above 10 hits: 0
    "D": ((8, 4), 6, 0.25, {7: (11, False)}),                   # band top outside the grid: 0
    "E": ((13, 13), 1, 0.25, {2: (29, True)}),                  # 29 / 50: int(57.99999999999999)
    "F": ((4, 12), 1, 0.25, {2: (12, True), 3: (11, False)}),   # both band voxels summed
    "H": ((12, 3), 1, 0.0, {3: (11, True), 4: (15, False)}),    # fraction 0: z=4 is above the band
    "J": ((1, 10), 1, 0.5 - 2.0 ** -22, {2: (20, True), 3: (11, False)}),  # just below 0.5
}


def scene_kat_posobs():
    """Obstacle-band columns at the thresholds (hit > 10, band ends, int() truncation) and a
    steep 3 x 3 patch whose slope alone makes it an obstacle."""
    pts = []
    for (cx, cy), zg, frac, stacks in POSOBS_COLUMNS.values():
        pts.append(_cell_point(cx, cy, zg, (0.5, 0.5, frac)))
        for z, (n, entry) in stacks.items():
            pts += _stack(cx, cy, z, n, entry)
    pts += [(20.5, 20.5, -7.5)] * 21  # rays through column E's band voxel, ending outside the grid
    for i in range(3):
        for j in range(3):
            pts.append(_cell_point(3 + i, 3 + j, 1, (0.5, 0.5, 0.25 + 0.5 * i + 0.25 * j)))
    ego = (0.5, 0.5, 0.5)
    return kat_params(B=1), [P(pts, ego), ("C",)]


def scene_kat_boundaries():
    """Points on and next to voxel faces of a 0.2 m grid (p / res lands on, just under or just over
    an integer in float64), on the min-distance sphere in float32 arithmetic, on the grid's outer
    faces, and with negative zero coordinates (gvom.py:1145-1171, 1254-1264, 1399-1416)."""
    res = 0.2
    pts = []
    for k in range(-14, 15):  # multiples of 0.1 m along each axis, and diagonals
        v = np.float32(0.1 * k)
        pts += [(v, 1.55, 0.15), (1.55, v, 0.15), (1.35, 1.25, v * np.float32(0.5)), (v, v, np.float32(1.1))]
    for v in (0.6, 1.0, 1.2, 1.4, -0.6, -1.0):  # float32 neighbours of face coordinates
        f = np.float32(v)
        for w in (np.nextafter(f, np.float32(-9)), f, np.nextafter(f, np.float32(9))):
            pts += [(w, -1.45, 0.05), (-1.45, w, 0.05), (1.55, 1.45, w * np.float32(0.5))]
    for ang in np.linspace(0.0, 2 * np.pi, 24, endpoint=False):  # on the 1 m min-distance sphere
        pts.append((np.float32(np.cos(ang)), np.float32(np.sin(ang)), np.float32(0.0)))
    pts += [(-0.0, 1.5, -0.0), (1.5, -0.0, 0.0), (0.0, -0.0, 1.25)]
    half = 16 * res  # grid of 32 x 32 x 16 around ego (0.1, 0.1, 0.1): x in [-3.2, 3.2)
    for e in (-half, half):
        f = np.float32(e)
        for w in (np.nextafter(f, np.float32(-9)), f, np.nextafter(f, np.float32(9))):
            pts += [(w, 1.3, 0.05), (1.3, w, 0.05)]
    params = (res, res, 32, 16, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 2.0, 1.0, 1, 1)
    pts = np.asarray(pts, np.float32)
    return params, [("P", pts, (0.1, 0.1, 0.1), None), ("C",),
                    ("P", pts[::-1].copy(), (0.3, -0.1, 0.1), None), ("C",)]


def scene_synthetic(name, X=32, Z=16, res=0.5, B=3, beams=16, columns=256, n_scans=6,
                    combine_after=(1, 2, 4, 5), tdtype=np.float32, pdtype=np.float32,
                    veg=0.0, dropout=0.0, eig=(1, 1), zres=None):
    from gvom_gb300.synthetic import Lidar, Terrain, Vegetation, make_scan, make_trajectory
    terrain = Terrain.make(0, extent=X * res, path_len=n_scans * 0.4)
    vegetation = None
    if veg > 0:
        ext = X * res
        vegetation = Vegetation.make(terrain, (-ext, ext + n_scans), (-ext, ext), density=veg)
    lidar = Lidar(beams=beams, columns=columns)
    poses = make_trajectory(n_scans)
    params = (res, res if zres is None else zres, X, Z, B, 1.0, 0.5, 0.5, 0.3, 2.0, 2.0, 1.0, eig[0], eig[1])
    ops = []
    for i, pose in enumerate(poses):
        s = make_scan(terrain, lidar, pose, i, vegetation=vegetation, footprint=X * res,
                      dropout=dropout, transform_dtype=tdtype)
        ops.append(("P", s.points.astype(pdtype), s.ego, s.transform))
        if i in combine_after:
            ops.append(("C",))
    return params, ops


def scene_small_32x512():
    """One 32x512 scan, 0.2 m voxels, 128x128x32, buffer 2: process then combine."""
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    s = make_workload_scans(w, 1)[0]
    return w.gvom_args(), [("P", s.points, s.ego, s.transform), ("C",)]


SCENES = {
    "kat_rays": scene_kat_rays,
    "kat_clear10": lambda: scene_kat_clear(10),
    "kat_clear11": lambda: scene_kat_clear(11),
    "kat_shift": scene_kat_shift,
    "kat_planes": scene_kat_planes,
    "kat_guess": scene_kat_guess,
    "kat_eigen": scene_kat_eigen,
    "kat_posobs": scene_kat_posobs,
    "kat_boundaries": scene_kat_boundaries,
    "synth_f32": lambda: scene_synthetic("synth_f32"),
    "synth_f64T_veg": lambda: scene_synthetic("synth_f64T_veg", tdtype=np.float64, veg=2.0, n_scans=5,
                                              combine_after=(0, 2, 4)),
    "synth_f64pts_eig20": lambda: scene_synthetic("synth_f64pts_eig20", pdtype=np.float64, eig=(2, 0),
                                                  n_scans=4, combine_after=(1, 3), B=2, dropout=0.3),
    "small_32x512": scene_small_32x512,
    # a long run: 12 scans through a 2-slot ring, a combine after each (counts and pass counts
    # accumulate through the last combined map, gvom.py:242-298)
    "synth_longrun": lambda: scene_synthetic("synth_longrun", B=2, columns=128, n_scans=12,
                                             combine_after=tuple(range(12))),
    # the ROS node's default voxels (scripts/gvom_ros.py:24-25): 0.4 m across, 0.2 m high
    "synth_aniso_z": lambda: scene_synthetic("synth_aniso_z", res=0.4, zres=0.2, n_scans=4, combine_after=(1, 3),
                                             eig=(1, 2)),
    # and the other way round, with float64 transforms
    "synth_aniso_xy": lambda: scene_synthetic("synth_aniso_xy", X=40, Z=12, res=0.25, zres=0.5, n_scans=4,
                                              combine_after=(0, 3), tdtype=np.float64),
    # a 16-slot ring (the largest the library takes): combines with 5, 16 and 17 sources (the ring
    # full plus the previous combined map), then after the ring has wrapped over its oldest slots
    "synth_ring16": lambda: scene_synthetic("synth_ring16", B=16, columns=128, n_scans=20,
                                            combine_after=(3, 15, 16, 19), dropout=0.2),
}


def run_reference(mod, params, ops):
    g = mod.Gvom(*params)
    out = {"params": np.array(params, dtype=np.float64)}
    kinds = []
    pi = ci = 0
    for op in ops:
        if op[0] == "P":
            _, pts, ego, T = op
            kinds.append("P")
            out[f"p{pi}_points"] = pts
            out[f"p{pi}_ego"] = np.array(ego, dtype=np.float64)
            if T is not None:
                out[f"p{pi}_T"] = np.asarray(T)
            g.Process_pointcloud(pts.copy(), tuple(ego), None if T is None else np.asarray(T).copy())
            s = g.last_buffer_index
            can = canonical_map(g.index_buffer[s].copy_to_host(),
                                hit=g.hit_count_buffer[s].copy_to_host(),
                                total=g.total_count_buffer[s].copy_to_host(),
                                min_h=g.min_height_buffer[s].copy_to_host()[: len(g.hit_count_buffer[s])],
                                metrics=g.metrics_buffer[s].copy_to_host())
            for k, v in can.items():
                out[f"p{pi}_slot_{k}"] = v
            out[f"p{pi}_slot_origin"] = g.origin_buffer[s].copy_to_host()
            pi += 1
        else:
            kinds.append("C")
            res = g.combine_maps()
            origin, pos, neg, rough, vis = res
            out[f"c{ci}_origin"] = origin
            out[f"c{ci}_pos"] = pos
            out[f"c{ci}_neg"] = neg
            out[f"c{ci}_rough"] = rough
            out[f"c{ci}_vis"] = vis
            can = canonical_map(g.combined_index_map.copy_to_host(),
                                hit=g.combined_hit_count.copy_to_host(),
                                total=g.combined_total_count.copy_to_host(),
                                min_h=g.combined_min_height.copy_to_host(),
                                metrics=g.combined_metrics.copy_to_host(),
                                eigen=g.voxels_eigenvalues.copy_to_host())
            for k, v in can.items():
                out[f"c{ci}_comb_{k}"] = v
            for k, arr in (("height", g.height_map), ("inferred", g.inferred_height_map),
                           ("slope_x", g.x_slope_map), ("slope_y", g.y_slope_map),
                           ("guess", g.guessed_height_delta)):
                out[f"c{ci}_{k}"] = arr.copy_to_host()
            out[f"c{ci}_debug_voxels"] = g.make_debug_voxel_map()
            out[f"c{ci}_debug_height"] = g.make_debug_height_map()
            out[f"c{ci}_debug_inferred"] = g.make_debug_inferred_height_map()
            ci += 1
    out["ops"] = np.array("".join(kinds))
    return out


# The reference's 2-D image kernels that no caller launches (scripts/gvom.py:807-885), run
# through the stand-in on seeded binary images: sizes, radii / window sizes and fractions that
# reach the image edges, radii with and without a fraction, windows larger than the image.
MORPH_CASES = {
    "expand": [(37, 0.0), (37, 1.0), (37, 1.5), (64, 2.7), (64, 4.0), (23, 30.0), (40, -1.0)],
    "lowpass": [(37, 0, 0.5), (37, 1, 0.5), (64, 2, 0.3), (64, 1, 0.75), (23, 15, 0.2), (40, 3, 1.0)],
}


def make_morph(mod):
    """Outputs of __expand_binary and __lowpass_binary; __convolve cannot run (its radius
    (kernel_size - 1) / 2 is a float, which range() rejects), so it has no fixture."""
    out = {}
    rng = np.random.default_rng(21)
    kexp = mod.Gvom._Gvom__expand_binary
    klow = mod.Gvom._Gvom__lowpass_binary
    tpb = (16, 16)
    for n, (X, r) in enumerate(MORPH_CASES["expand"]):
        img = (rng.uniform(size=(X, X)) < (0.02 if r > 2 else 0.15)).astype(np.int32)
        res = np.full((X, X), -7, np.int32)
        kexp[((X + 15) // 16, (X + 15) // 16), tpb](img, res, X, float(r))
        out[f"expand{n}_img"], out[f"expand{n}_r"], out[f"expand{n}_out"] = img, np.float64(r), res
    for n, (X, fs, frac) in enumerate(MORPH_CASES["lowpass"]):
        img = (rng.uniform(size=(X, X)) < 0.5).astype(np.int32)
        res = np.full((X, X), -7, np.int32)
        klow[((X + 15) // 16, (X + 15) // 16), tpb](img, res, X, int(fs), float(frac))
        out[f"lowpass{n}_img"], out[f"lowpass{n}_fs"] = img, np.int64(fs)
        out[f"lowpass{n}_frac"], out[f"lowpass{n}_out"] = np.float64(frac), res
    return out


def main(argv):
    names = argv or list(SCENES) + ["morph_binary"]
    mod = load_reference()
    if "morph_binary" in names:
        t = time.time()
        path = os.path.join(HERE, "morph_binary.npz")
        np.savez_compressed(path, **make_morph(mod))
        print(f"morph_binary: {time.time() - t:.1f} s, {os.path.getsize(path) / 1024:.0f} KiB", flush=True)
        names = [n for n in names if n != "morph_binary"]
    for name in names:
        t = time.time()
        params, ops = SCENES[name]()
        out = run_reference(mod, params, ops)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{name}: {time.time() - t:.1f} s, {os.path.getsize(path) / 1024:.0f} KiB", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
