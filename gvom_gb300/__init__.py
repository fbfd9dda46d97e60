"""GB300-native G-VOM scan->map hot path (drop-in for the reference `Gvom` class).

    from gvom_gb300 import Gvom
    g = Gvom(xy_res, z_res, xy_size, z_size, buffer_size, min_distance, pos_thr, neg_thr,
             slope_thr, robot_height, robot_radius, ground_to_lidar_height, xy_eigen_dist, z_eigen_dist)
    g.process_pointcloud(points, ego_position, transform)
    origin, positive, negative, roughness, visibility = g.combine_maps()

The work runs in libgvom_gb300.so (hand-written sm_103a CUDA behind the C ABI
of include/gvom_gb300.h).  Build it with `python gvom_gb300/build.py`.
"""
from .gvom import Gvom, pose_to_transform  # noqa: F401

__all__ = ["Gvom", "pose_to_transform"]
__version__ = "0.1.0"
