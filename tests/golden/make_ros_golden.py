"""Generate tests/golden/ros_epilogue.npz by running the REFERENCE ROS node's
map-publishing callback, unchanged.

`VoxelMapper.cb_timer` of the reference's scripts/gvom_ros.py (:113-166) turns
combine_maps' outputs into five int8 OccupancyGrid payloads with numpy.  This
script loads that file from the reference checkout named by $GVOM_REFERENCE
(required) with stand-in modules for rospy, the ROS message types,
tf and ros_numpy (none is installed, and the callback uses them only to
build and publish messages), feeds it maps, and records the `data` of every
published message.  The maps are the combine outputs stored in the other
golden fixtures plus edge cases: every roughness from -12 to 1 in steps of
1/8 (the clip bounds, and values whose payload leaves int8), NaN,
negative-obstacle values of 0 and 100, densities on both sides of the
threshold, non-default node parameters, and roughness ranges so narrow that
the payload leaves int32.  Run in the build container; the
fixture is committed:

    python tests/golden/make_ros_golden.py
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("GVOM_REFERENCE")
if not REF:
    raise SystemExit("set GVOM_REFERENCE to the reference checkout (the directory holding scripts/gvom.py)")


def _stub_modules():
    ns = types.SimpleNamespace

    class _Time:
        @staticmethod
        def now():
            return 0

    rospy = types.ModuleType("rospy")
    rospy.Time = _Time
    rospy.Duration = lambda *a: None
    rospy.loginfo = lambda *a, **k: None
    rospy.get_param = lambda name, default=None: default

    def occupancy_grid():
        origin = ns(orientation=ns(x=0, y=0, z=0, w=1), position=ns(x=0, y=0, z=0))
        return ns(header=ns(stamp=None, frame_id=None), info=ns(resolution=0, width=0, height=0, origin=origin),
                  data=None)

    nav_msg = types.ModuleType("nav_msgs.msg")
    nav_msg.OccupancyGrid = occupancy_grid
    nav_msg.Odometry = object
    sensor_msg = types.ModuleType("sensor_msgs.msg")
    sensor_msg.PointCloud2 = object
    mods = {
        "rospy": rospy,
        "gvom": types.ModuleType("gvom"),
        "nav_msgs": types.ModuleType("nav_msgs"), "nav_msgs.msg": nav_msg,
        "sensor_msgs": types.ModuleType("sensor_msgs"), "sensor_msgs.msg": sensor_msg,
        "sensor_msgs.point_cloud2": types.ModuleType("sensor_msgs.point_cloud2"),
        "tf2_ros": types.ModuleType("tf2_ros"), "tf": types.ModuleType("tf"),
        "ros_numpy": types.ModuleType("ros_numpy"),
    }
    sys.modules.update(mods)


def load_node():
    _stub_modules()
    path = os.path.join(REF, "scripts", "gvom_ros.py")
    spec = importlib.util.spec_from_file_location("gvom_ros_reference", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Pub:
    def __init__(self, log, name):
        self.log, self.name = log, name

    def publish(self, msg):
        self.log.append((self.name, np.array(msg.data, copy=True)))


class _Mapper:
    def __init__(self, maps):
        self.maps = maps

    def combine_maps(self):
        return self.maps

    def make_debug_voxel_map(self):
        return None

    make_debug_height_map = make_debug_inferred_height_map = make_debug_voxel_map


PUBS = ("h_obstacle_map_pub", "s_obstacle_map_pub", "g_certainty_pub", "a_certainty_pub",
        "n_obstacle_map_pub", "r_map_pub")


def run_callback(mod, maps, density_threshold=50, min_roughness=-10, max_roughness=0):
    node = object.__new__(mod.VoxelMapper)  # the callback's state only, no ROS setup
    X = maps[1].shape[0]
    node.odom_frame, node.xy_resolution, node.width = "odom", 0.4, X
    node.density_threshold, node.min_roughness, node.max_roughness = density_threshold, min_roughness, max_roughness
    node.voxel_mapper = _Mapper(maps)
    log = []
    for p in PUBS:
        setattr(node, p, _Pub(log, p))
    node.cb_timer(None)
    return dict(log)


def edge_maps(X=24):
    rng = np.random.default_rng(3)
    rough = np.arange(X * X, dtype=np.float64).reshape(X, X) / 8.0 - 12.0  # -12 .. 59.875, x fastest in F order
    rough[rough > 1.0] = rng.uniform(-11, 1, np.count_nonzero(rough > 1.0))
    rough[0, 1] = np.nan
    rough[1, 1] = -1.0
    pos = rng.integers(0, 101, (X, X)).astype(np.int32)
    pos[:4, 0] = [0, 49, 50, 51]
    neg = np.where(rng.uniform(size=(X, X)) < 0.3, 100, 0).astype(np.int32)
    vis = (rng.uniform(size=(X, X)) < 0.6).astype(np.int32)
    return (np.zeros(3), pos, neg, rough, vis)


def cases():
    out = []
    for name in ("kat_planes", "kat_guess", "synth_f32", "synth_aniso_z"):
        with np.load(os.path.join(HERE, f"{name}.npz")) as z:
            ci = 0
            maps = (z[f"c{ci}_origin"], z[f"c{ci}_pos"], z[f"c{ci}_neg"], z[f"c{ci}_rough"], z[f"c{ci}_vis"])
        out.append((name, maps, {}))
    e = edge_maps()
    out.append(("edges", e, {}))
    out.append(("edges_params", e, dict(density_threshold=30, min_roughness=-6, max_roughness=-1)))
    # a roughness range so narrow that the payload leaves int32 (about -2e11) or stays just inside it (-2e9)
    out.append(("edges_narrow_out", e, dict(min_roughness=-1.0, max_roughness=-1.0 + 1e-9)))
    out.append(("edges_narrow_in", e, dict(min_roughness=-1.0, max_roughness=-1.0 + 1e-7)))
    return out


def main():
    mod = load_node()
    res = {}
    for name, maps, kw in cases():
        pay = run_callback(mod, maps, **kw)
        res[f"{name}_pos"], res[f"{name}_neg"] = maps[1], maps[2]
        res[f"{name}_rough"], res[f"{name}_vis"] = maps[3], maps[4]
        res[f"{name}_params"] = np.array([kw.get("density_threshold", 50), kw.get("min_roughness", -10),
                                          kw.get("max_roughness", 0)], np.float64)
        for p, v in pay.items():
            res[f"{name}_{p}"] = v
        print(name, {p: (v.dtype.str, v.shape) for p, v in pay.items()})
    res["cases"] = np.array(",".join(n for n, _, _ in cases()))
    np.savez_compressed(os.path.join(HERE, "ros_epilogue.npz"), **res)


if __name__ == "__main__":
    main()
