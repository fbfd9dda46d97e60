"""The CPU oracle against the reference's own outputs (tests/golden, made by
running the reference scripts/gvom.py unchanged; see tests/golden/make_golden.py).

The oracle must reproduce every fixture array bit for bit, floats included.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.canonical import canonical_state, sort_debug_voxels
from oracle.oracle import OracleGvom
from replay import assert_exact, load, ops_of, params_of


def _bitwise(a, b, what):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    if a.dtype.kind == "f":
        ok = (a == b) | (np.isnan(a) & np.isnan(b))
        assert ok.all(), f"{what}: {np.count_nonzero(~ok)} differ, max |d| {np.nanmax(np.abs(a - b))}"
    else:
        assert_exact(a, b, what)


@pytest.mark.parametrize("name", golden_files())
def test_oracle_matches_reference_bitwise(name):
    fx = load(os.path.join(GOLDEN, name))
    g = OracleGvom(*params_of(fx))
    for op in ops_of(fx):
        if op[0] == "P":
            _, pi, pts, ego, T = op
            g.Process_pointcloud(pts, ego, T)
            _, last = g.ring_state()
            st = g.slot_state(last)
            can = canonical_state(st)
            for k in ("occ", "free", "hit", "total", "min_h", "metrics"):
                _bitwise(can[k], fx[f"p{pi}_slot_{k}"], f"process {pi} {k}")
            _bitwise(st["origin"], fx[f"p{pi}_slot_origin"], f"process {pi} origin")
        else:
            _, ci = op
            origin, pos, neg, rough, vis = g.combine_maps()
            pre = f"c{ci}_"
            _bitwise(origin, fx[pre + "origin"], "origin")
            _bitwise(pos, fx[pre + "pos"], "positive obstacles")
            _bitwise(neg, fx[pre + "neg"], "negative obstacles")
            _bitwise(rough, fx[pre + "rough"], "roughness")
            _bitwise(vis, fx[pre + "vis"], "visibility")
            can = canonical_state(g.combined_state())
            for k in ("occ", "free", "hit", "total", "min_h", "metrics", "eigen"):
                _bitwise(can[k], fx[pre + "comb_" + k], f"combine {ci} {k}")
            m = g.maps_state()
            for k in ("height", "inferred", "slope_x", "slope_y", "guess"):
                _bitwise(m[k], fx[pre + k], f"combine {ci} {k}")
            dv = sort_debug_voxels(g.make_debug_voxel_map())
            _bitwise(dv, sort_debug_voxels(fx[pre + "debug_voxels"]), "debug voxels (canonical order)")
            _bitwise(g.make_debug_height_map(), fx[pre + "debug_height"], "debug height map")
            _bitwise(g.make_debug_inferred_height_map(), fx[pre + "debug_inferred"], "debug inferred map")


def _slot_counts(g, X):
    _, last = g.ring_state()
    st = g.slot_state(last)
    return st, canonical_state(st)


def test_kat_axis_ray_known_answer():
    """+x ray from (0.5,0.5,0.5) to (5.5,0.5,0.5), 1 m voxels, origin (-8,-8,-4):
    pass-throughs at x = 9..12 (y=8, z=4), hit at x = 13."""
    g = OracleGvom(1.0, 1.0, 16, 8, 2, 0.5, 0.5, 0.5, 0.3, 2.0, 0.5, 1.0, 1, 1)
    g.Process_pointcloud(np.array([[5.5, 0.5, 0.5]], np.float32), (0.5, 0.5, 0.5))
    st, can = _slot_counts(g, 16)
    vid = lambda x, y, z: x + y * 16 + z * 256  # noqa: E731
    assert list(can["occ"]) == [vid(13, 8, 4)]
    assert can["hit"].tolist() == [1] and can["total"].tolist() == [1]
    for x in range(9, 13):
        assert st["index"][vid(x, 8, 4)] == -2
    assert (st["index"] == -1).sum() == 16 * 16 * 8 - 5


def test_kat_diagonal_tie_goes_to_z_and_recounts_hit_voxel():
    """(3,3,3) diagonal: ties pick z; 3 steps; the last step lands in the hit voxel (total 2)."""
    g = OracleGvom(1.0, 1.0, 16, 8, 2, 0.5, 0.5, 0.5, 0.3, 2.0, 0.5, 1.0, 1, 1)
    g.Process_pointcloud(np.array([[3.5, 3.5, 3.5]], np.float32), (0.5, 0.5, 0.5))
    st, can = _slot_counts(g, 16)
    vid = lambda x, y, z: x + y * 16 + z * 256  # noqa: E731
    assert list(can["occ"]) == [vid(11, 11, 7)]
    assert can["total"].tolist() == [2]
    assert st["index"][vid(9, 9, 5)] == -2 and st["index"][vid(10, 10, 6)] == -2


def test_kat_clearing_rule():
    """An occupied voxel crossed by 11 rays is cleared from the combined map, by 10 it stays."""
    for n_pass, stays in ((10, True), (11, False)):
        g = OracleGvom(1.0, 1.0, 16, 8, 1, 0.5, 0.5, 0.5, 0.3, 2.0, 0.5, 1.0, 1, 1)
        g.Process_pointcloud(np.array([[3.5, 0.5, 0.5]] * 3, np.float32), (0.5, 0.5, 0.5))
        g.combine_maps()
        g.Process_pointcloud(np.array([[6.5, 0.5, 0.5]] * n_pass, np.float32), (0.5, 0.5, 0.5))
        g.combine_maps()
        st = g.combined_state()
        v = 11 + 8 * 16 + 4 * 256
        assert (st["index"][v] >= 0) == stays


def test_empty_scan_is_a_valid_slot():
    g = OracleGvom(1.0, 1.0, 16, 8, 2, 0.5, 0.5, 0.5, 0.3, 2.0, 0.5, 1.0, 1, 1)
    assert g.combine_maps() is None
    g.Process_pointcloud(np.zeros((0, 3), np.float32), (0.5, 0.5, 0.5))
    st = g.slot_state(0)
    assert len(st["hit"]) == 0 and (st["index"] == -1).all()
    out = g.combine_maps()
    assert out is not None and (out[4] == 0).all()


def test_nonfinite_points_are_dropped():
    g = OracleGvom(1.0, 1.0, 16, 8, 2, 0.5, 0.5, 0.5, 0.3, 2.0, 0.5, 1.0, 1, 1)
    pts = np.array([[5.5, 0.5, 0.5], [np.nan, 1, 1], [np.inf, 0, 0]], np.float32)
    g.Process_pointcloud(pts, (0.5, 0.5, 0.5))
    assert g.last_process_stats()["valid_points"] == 1


def test_parallel_oracle_integer_results_match_sequential():
    """The OpenMP mode (timed CPU baseline) gives the same integer results."""
    fx = load(os.path.join(GOLDEN, "synth_f32.npz"))
    a = OracleGvom(*params_of(fx))
    b = OracleGvom(*params_of(fx), threads=4)
    for op in ops_of(fx):
        if op[0] == "P":
            a.Process_pointcloud(*op[2:])
            b.Process_pointcloud(*op[2:])
        else:
            ra, rb = a.combine_maps(), b.combine_maps()
            for x, y in zip(ra, rb):
                np.testing.assert_array_equal(x, y) if x.dtype.kind == "i" else np.testing.assert_allclose(x, y, rtol=1e-9)
            ca, cb = canonical_state(a.combined_state()), canonical_state(b.combined_state())
            for k in ("occ", "free", "hit", "total", "min_h"):
                np.testing.assert_array_equal(ca[k], cb[k])


def _comb_row(fx, ci, key, x, y, z, X=16):
    occ = fx[f"c{ci}_comb_occ"]
    r = np.searchsorted(occ, x + y * X + z * X * X)
    assert r < len(occ) and occ[r] == x + y * X + z * X * X, f"voxel {(x, y, z)} not occupied"
    return fx[f"c{ci}_comb_{key}"][r]


# kat_eigen: voxel -> (points per scan, mean in voxel units, eigenvalues in closed form).
# Symmetric clusters about the voxel centre; pair_a / pair_b are adjacent voxels whose
# neighbourhoods take in each other's points (gvom.py:1249-1371).
EIGEN_KAT = {
    (12, 12, 2): (6, (0.5, 0.5, 0.5), (1 / 48, 1 / 48, 1 / 48)),    # isotropic
    (4, 12, 2): (4, (0.5, 0.5, 0.5), (1 / 32, 1 / 32, 0.0)),        # planar
    (12, 4, 2): (4, (0.5, 0.5, 0.5), (5 / 128, 0.0, 0.0)),          # linear along x
    (4, 4, 2): (4, (0.5, 0.5, 0.5), (5 / 64, 0.0, 0.0)),            # linear along x = y
    (8, 13, 5): (4, (0.5, 0.5, 0.5), (1 / 32, 1 / 64, 0.0)),        # plane tilted about y
    (13, 8, 1): (6, (0.5, 0.5, 0.5), (1 / 48, 3 / 256, 1 / 192)),   # distinct axes, sorted
    (2, 8, 1): (1, (0.6, 0.3, 0.55), (0.0, 0.0, 0.0)),              # one point
    (8, 2, 1): (4, (1.0, 0.5, 0.5), (9 / 32, 1 / 32, 0.0)),         # pair_a
    (9, 2, 1): (4, (0.0, 0.5, 0.5), (9 / 32, 1 / 32, 0.0)),         # pair_b
}


def test_kat_eigenvalues_closed_form():
    """The reference's combined statistics and eigenvalues (gvom.py:888-980, 1423-1487) for
    covariances known in closed form; the same scan in two slots, then two combines, so the
    counts double on the second combine through the last combined map."""
    fx = load(os.path.join(GOLDEN, "kat_eigen.npz"))
    for ci, mult in ((0, 2), (1, 4)):
        assert len(fx[f"c{ci}_comb_occ"]) == len(EIGEN_KAT)
        for (x, y, z), (n, mean, lam) in EIGEN_KAT.items():
            m = _comb_row(fx, ci, "metrics", x, y, z)
            assert m[9] == mult * n, ((x, y, z), m[9])
            np.testing.assert_allclose(m[:3], mean, rtol=1e-6, err_msg=str((x, y, z)))
            np.testing.assert_allclose(_comb_row(fx, ci, "eigen", x, y, z), lam, rtol=1e-6, atol=1e-12,
                                       err_msg=str((x, y, z)))


# kat_posobs: cell -> positive-obstacle value, with the band sums behind it
# (1 m voxels, positive threshold 0.5 m, robot height 2 m; gvom.py:515-555).
POSOBS_KAT = {
    (12, 8): 57,   # band z 2..3: z=2 hit 11 / total 19; z=3 hit 10 is not > 10
    (8, 12): 50,   # fraction 0.5: band z 3..3, hit 11 / total 22 (z=2 would add 20 / 20)
    (4, 8): 0,     # hits of 10 only: no density
    (8, 4): 0,     # band top at z = 8, outside the grid: left at 0
    (13, 13): 57,  # 29 / 50 = 0.58, and 0.58 * 100 = 57.99999999999999 truncates to 57
    (4, 12): 67,   # both band voxels: (12 + 11) / (12 + 22)
    (12, 3): 100,  # fraction 0: band z 2..3, hit 11 / total 11; z=4 is above the band
    (1, 10): 81,   # fraction 0.5 - 2^-22: band z 2..3, (20 + 11) / (20 + 18)
}


def test_kat_positive_obstacle_band():
    fx = load(os.path.join(GOLDEN, "kat_posobs.npz"))
    pos = fx["c0_pos"]
    for (x, y), want in POSOBS_KAT.items():
        assert pos[x, y] == want, ((x, y), pos[x, y], want)
    assert int(29 / 50 * 100) == 57  # the float64 quirk the kernel keeps
    hit = _comb_row(fx, 0, "hit", 13, 13, 2)
    total = _comb_row(fx, 0, "total", 13, 13, 2)
    assert (hit, total) == (29, 50)
    # a steep 3 x 3 patch (slope above 0.3 rad) is an obstacle whatever its band holds
    assert (pos[3:6, 3:6] == 100).all()
    assert np.hypot(fx["c0_slope_x"][4, 4], fx["c0_slope_y"][4, 4]) >= 0.3
