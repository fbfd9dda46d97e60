"""Replay a golden scene on a mapper and compare with the fixture / another mapper.

A "mapper" is anything with the reference surface (`Process_pointcloud`,
`combine_maps`, `make_debug_*`) plus the parity accessors `slot_state`,
`combined_state`, `maps_state` and `ring_state` (both `OracleGvom` and
`gvom_gb300.Gvom` provide them).

Tolerances (from the path's parity contract):
  * integer outputs and canonical voxel sets, hit/total/pass counts: exact;
  * heights: 1e-4 m absolute; roughness and slopes: 1e-3 relative;
  * thresholded maps: exact except where the float input lies within
    tolerance of the threshold;
  * per-voxel mean/covariance/eigenvalues (only visible through the debug
    voxel export): see `STAT_ATOL`.
"""
from __future__ import annotations

import numpy as np

from oracle.canonical import canonical_map, canonical_state

HEIGHT_ATOL = 1e-4
REL_TOL = 1e-3
SLOPE_ATOL = 1e-9
# mean/cov are in voxel units (|mean| < 2, cov < 1).
STAT_ATOL = 1e-5
STAT_RTOL = 1e-4
# Eigenvalues: the reference's closed form (scripts/gvom.py:1446-1487) takes
# float32 covariances and forms p1 in float32; near a repeated eigenvalue
# (r -> +-1) its result carries noise of order p*sqrt(eps32) ~ 3e-4 * |l_max|,
# so two correct solvers agree only to that scale.
EIG_RTOL = 1e-3
EIG_ATOL = 1e-6


def load(path):
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def params_of(fx):
    p = fx["params"]
    return (float(p[0]), float(p[1]), int(p[2]), int(p[3]), int(p[4]), float(p[5]), float(p[6]),
            float(p[7]), float(p[8]), float(p[9]), float(p[10]), float(p[11]), int(p[12]), int(p[13]))


def ops_of(fx):
    """Yield ('P', pi, points, ego, T) / ('C', ci) in call order."""
    pi = ci = 0
    for k in str(fx["ops"]):
        if k == "P":
            T = fx.get(f"p{pi}_T")
            yield ("P", pi, fx[f"p{pi}_points"], tuple(fx[f"p{pi}_ego"]), T)
            pi += 1
        else:
            yield ("C", ci)
            ci += 1


def rel_close(a, b, rtol=REL_TOL, atol=1e-9):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)) + atol


def assert_rel(a, b, what, rtol=REL_TOL, atol=1e-9):
    ok = rel_close(a, b, rtol, atol)
    if not ok.all():
        bad = np.flatnonzero(~ok.reshape(-1))
        aa = np.asarray(a).reshape(-1)
        bb = np.asarray(b).reshape(-1)
        raise AssertionError(f"{what}: {bad.size} mismatches, first at {bad[:5]}: "
                             f"{aa[bad[:5]]} vs {bb[bad[:5]]}")


def assert_exact(a, b, what):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        raise AssertionError(f"{what}: shape {a.shape} vs {b.shape}")
    if not np.array_equal(a, b):
        bad = np.flatnonzero((a != b).reshape(-1))
        raise AssertionError(f"{what}: {bad.size} mismatches, first at {bad[:5]}: "
                             f"{a.reshape(-1)[bad[:5]]} vs {b.reshape(-1)[bad[:5]]}")


def assert_stats(a, b, what):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = np.abs(a - b) <= STAT_ATOL + STAT_RTOL * np.abs(b)
    if not ok.all():
        bad = np.flatnonzero(~ok.reshape(-1))
        raise AssertionError(f"{what}: {bad.size} mismatches (max abs err "
                             f"{np.abs(a - b).max():.3g}), first at {bad[:5]}: "
                             f"{a.reshape(-1)[bad[:5]]} vs {b.reshape(-1)[bad[:5]]}")


def assert_eigen(a, b, what, scale=None):
    """Eigenvalue rows (n, 3) (or the debug export's gap columns) within
    EIG_RTOL of the row's largest eigenvalue magnitude."""
    a = np.asarray(a, np.float64).reshape(len(a), -1)
    b = np.asarray(b, np.float64).reshape(len(b), -1)
    if scale is None:
        scale = np.abs(b).max(axis=1, keepdims=True)
    ok = np.abs(a - b) <= EIG_ATOL + EIG_RTOL * scale
    if not ok.all():
        bad = np.flatnonzero(~ok.reshape(-1))
        raise AssertionError(f"{what}: {bad.size} mismatches (max abs err {np.abs(a - b).max():.3g}), "
                             f"first at {bad[:5]}: {a.reshape(-1)[bad[:5]]} vs {b.reshape(-1)[bad[:5]]}")


def compare_slot(got: dict, ref: dict, what: str, stats=True):
    assert_exact(got["occ"], ref["occ"], f"{what} occupied set")
    assert_exact(got["free"], ref["free"], f"{what} free/pass-count map")
    assert_exact(got["hit"], ref["hit"], f"{what} hit")
    assert_exact(got["total"], ref["total"], f"{what} total")
    assert_exact(got["min_h"].astype(np.float32), ref["min_h"].astype(np.float32), f"{what} min_height")
    if stats and "metrics" in ref and "metrics" in got:
        gm = np.asarray(got["metrics"], np.float64)
        rm = np.asarray(ref["metrics"], np.float64)
        assert_exact(gm[:, 9], rm[:, 9], f"{what} point count")
        assert_stats(gm[:, :9], rm[:, :9], f"{what} mean/cov")


def threshold_mask(values, thr, tol):
    """Cells whose float input lies within `tol` of a threshold (allowed to differ)."""
    return np.abs(np.asarray(values, np.float64) - thr) <= tol


def compare_combine(got_out, ref: dict, got_maps: dict, params, what: str):
    """Compare combine_maps outputs and the 2-D intermediate maps."""
    origin, pos, neg, rough, vis = got_out
    assert_exact(np.asarray(origin), ref["origin"], f"{what} origin")
    # heights
    for k in ("height", "inferred"):
        d = np.abs(got_maps[k] - ref[k])
        if not (d <= HEIGHT_ATOL).all():
            raise AssertionError(f"{what} {k}: max err {d.max()}")
    assert_exact(vis, ref["vis"], f"{what} visibility")
    for k in ("slope_x", "slope_y"):
        assert_rel(got_maps[k], ref[k], f"{what} {k}", atol=SLOPE_ATOL)
    assert_rel(got_maps["guess"], ref["guess"], f"{what} guessed height delta", atol=HEIGHT_ATOL)
    assert_rel(rough, ref["rough"], f"{what} roughness", atol=1e-9)
    slope_thr = params[8]
    neg_thr = params[7]
    s = np.sqrt(ref["slope_x"] ** 2 + ref["slope_y"] ** 2)
    near = threshold_mask(s, slope_thr, REL_TOL * max(slope_thr, 1e-12) + 1e-9)
    m = ~near
    assert_exact(pos[m], ref["pos"][m], f"{what} positive obstacles")
    near_n = threshold_mask(ref["guess"], neg_thr, HEIGHT_ATOL + REL_TOL * neg_thr)
    assert_exact(neg[~near_n], ref["neg"][~near_n], f"{what} negative obstacles")


def replay_and_compare(mapper, fx, stats=True, debug=True):
    """Drive `mapper` through the fixture's calls; compare after every call."""
    params = params_of(fx)
    for op in ops_of(fx):
        if op[0] == "P":
            _, pi, pts, ego, T = op
            mapper.Process_pointcloud(pts, ego, T)
            _, last = mapper.ring_state()
            st = mapper.slot_state(last)
            got = canonical_state(st)
            ref = {k[len(f"p{pi}_slot_"):]: v for k, v in fx.items() if k.startswith(f"p{pi}_slot_")}
            assert_exact(st["origin"], ref["origin"], f"process {pi} origin")
            compare_slot(got, ref, f"process {pi} slot", stats=stats)
        else:
            _, ci = op
            out = mapper.combine_maps()
            assert out is not None
            pre = f"c{ci}_"
            ref = {k[len(pre):]: v for k, v in fx.items() if k.startswith(pre)}
            cst = canonical_state(mapper.combined_state())
            rc = {k[len("comb_"):]: v for k, v in ref.items() if k.startswith("comb_")}
            compare_slot(cst, rc, f"combine {ci} combined map", stats=stats)
            if stats:
                assert_eigen(cst["eigen"], rc["eigen"], f"combine {ci} eigenvalues")
            compare_combine(out, ref, mapper.maps_state(), params, f"combine {ci}")
            if debug:
                dv = mapper.make_debug_voxel_map()
                rv = ref["debug_voxels"]
                from oracle.canonical import sort_debug_voxels
                dv = sort_debug_voxels(dv)
                rv = sort_debug_voxels(rv)
                assert_exact(dv[:, :5], rv[:, :5], f"combine {ci} debug voxel rows")
                if stats:
                    lmax = np.abs(rv[:, 5:6] + rv[:, 6:7] + rv[:, 7:8])  # l0 = gaps + l2
                    assert_eigen(dv[:, 5:], rv[:, 5:], f"combine {ci} debug voxel eigen gaps",
                                 scale=np.maximum(lmax, np.abs(rv[:, 5:]).max(axis=1, keepdims=True)))
                dh = mapper.make_debug_height_map()
                rh = ref["debug_height"]
                assert_exact(dh[:, :2], rh[:, :2], f"combine {ci} debug height xy")
                assert np.all(np.abs(dh[:, 2] - rh[:, 2]) <= HEIGHT_ATOL * 10)
                assert_rel(dh[:, 3:], rh[:, 3:], f"combine {ci} debug height rough/slope", rtol=1e-3, atol=1e-6)
                di = mapper.make_debug_inferred_height_map()
                ri = ref["debug_inferred"]
                assert_exact(di[:, :2], ri[:, :2], f"combine {ci} debug inferred xy")
                assert np.all(np.abs(di[:, 2] - ri[:, 2]) <= HEIGHT_ATOL * 10)


def float_errors(got_out, ref: dict, got_maps: dict) -> dict:
    """Largest deviations of the float outputs from the float64 oracle:
    absolute for heights, relative (where the oracle value is non-zero) for
    roughness and slopes."""
    def rel(a, b):
        a = np.asarray(a, np.float64)
        b = np.asarray(b, np.float64)
        m = np.abs(b) > 0
        return float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m]))) if m.any() else 0.0

    rough = got_out[3]
    return {
        "height_abs": float(np.max(np.abs(got_maps["height"] - ref["height"]))),
        "inferred_abs": float(np.max(np.abs(got_maps["inferred"] - ref["inferred"]))),
        "guess_abs": float(np.max(np.abs(got_maps["guess"] - ref["guess"]))),
        "roughness_rel": rel(rough, ref["rough"]),
        "slope_x_rel": rel(got_maps["slope_x"], ref["slope_x"]),
        "slope_y_rel": rel(got_maps["slope_y"], ref["slope_y"]),
    }


def stat_errors(got_state: dict, ref_state: dict) -> dict:
    """Largest deviations of the combined per-voxel statistics from the oracle,
    on canonical states with the same occupied set: absolute for the mean and
    the covariance (voxel units); for the eigenvalues relative to each
    voxel's largest eigenvalue magnitude where that is at least EIG_ATOL,
    and absolute in the voxels below it (a single point, or points on one
    spot, whose eigenvalues are rounding noise around 0)."""
    g = canonical_state(got_state)
    r = canonical_state(ref_state)
    assert_exact(g["occ"], r["occ"], "occupied set")
    gm = np.asarray(g["metrics"], np.float64)
    rm = np.asarray(r["metrics"], np.float64)
    out = {"voxels": int(len(r["occ"])),
           "mean_abs": float(np.max(np.abs(gm[:, :3] - rm[:, :3]))) if len(rm) else 0.0,
           "cov_abs": float(np.max(np.abs(gm[:, 3:9] - rm[:, 3:9]))) if len(rm) else 0.0}
    if "eigen" in g and "eigen" in r and len(rm):
        ge = np.asarray(g["eigen"], np.float64)
        re = np.asarray(r["eigen"], np.float64)
        scale = np.abs(re).max(axis=1)
        err = np.abs(ge - re).max(axis=1)
        big = scale >= EIG_ATOL
        out["eigen_rel_to_max"] = float(np.max(err[big] / scale[big])) if big.any() else 0.0
        out["eigen_abs_below_atol"] = float(np.max(err[~big])) if (~big).any() else 0.0
    return out
