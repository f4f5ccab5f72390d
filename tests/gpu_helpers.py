"""Shared comparison helpers for the GPU parity tests (oracle vs CUDA)."""
import numpy as np

CORNER_TOL_PX = 1e-3  # quad corners: max abs difference allowed, pixels


def _leaf_bytes(a):
    """Per-element bytes of every leaf field (padding excluded), so records
    compare field by field and floats compare by bit pattern."""
    n = len(a)
    if a.dtype.names is None:
        return [np.ascontiguousarray(a).view(np.uint8).reshape(n, -1)] if n else []
    out = []
    for name in a.dtype.names:
        f = a[name]
        if f.dtype.names is not None:  # nested record (possibly a sub-array of records)
            out += _leaf_bytes(f.reshape(n, -1).reshape(-1)) if n else []
            out = [o.reshape(n, -1) for o in out] if n else out
        else:
            out.append(np.ascontiguousarray(f).view(np.uint8).reshape(n, -1) if n else None)
    return [o for o in out if o is not None]


def assert_same(a, b, what=""):
    """Exact (bit-pattern) equality with a short report of where arrays differ."""
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape or a.dtype != b.dtype:
        raise AssertionError(f"{what}: {a.shape}/{a.dtype} != {b.shape}/{b.dtype}")
    if a.size == 0:
        return
    fa, fb = a.reshape(-1), b.reshape(-1)
    la, lb = _leaf_bytes(fa), _leaf_bytes(fb)
    ne = np.zeros(len(fa), bool)
    for x, y in zip(la, lb):
        ne |= (x != y).any(axis=1)
    bad = np.flatnonzero(ne)
    if len(bad):
        i = bad[:5]
        raise AssertionError(f"{what}: {len(bad)} of {fa.size} differ; first at {i.tolist()}: "
                             f"{fa[i].tolist()} vs {fb[i].tolist()}")


def oracle_top10(res):
    """Per filtered cluster: (peak count, first 10 peaks) from the oracle's
    sorted corner list."""
    nclu = len(res["filtered"])
    counts = np.zeros(nclu, np.uint32)
    top = {}
    for pe in res["peak_extents"]:
        seg = res["corners"][pe["start"]: pe["start"] + pe["count"]]
        c = int(seg[0]["cluster_index"])
        counts[c] = pe["count"]
        top[c] = seg[:10]
    return counts, top


def pair_table(views):
    """Occupied slots of the GPU pair table as arrays sorted by key:
    (key, count, x_min, x_max, y_min, y_max, gx_sum, gy_sum, pxgx)."""
    keys = views["pair_keys"]
    occ = np.flatnonzero(keys != np.uint64(0xFFFFFFFFFFFFFFFF))
    occ = occ[np.argsort(keys[occ], kind="stable")]
    bb, gs = views["pair_bbox"][occ], views["pair_gsum"][occ]
    return (keys[occ], views["pair_count"][occ], bb[:, 0], bb[:, 1], bb[:, 2], bb[:, 3], gs[:, 0], gs[:, 1],
            views["pair_pxgx"][occ])


def oracle_pair_table(res):
    b = res["bounds"]
    return (res["bound_keys"], b["count"], b["x_min"], b["x_max"], b["y_min"], b["y_max"], b["gx_sum"],
            b["gy_sum"], b["pxgx_pygy_sum"])


def surviving_point_sets(views, res):
    """(key, packed) of the points of the surviving clusters, sorted, from the
    GPU's point list and from the oracle."""
    pp = views["pair_points"]
    slots = (pp >> np.uint64(32)).astype(np.int64)
    packed = (pp & np.uint64(0xFFFFFFFF)).astype(np.uint64)
    keys = views["pair_keys"][slots]
    keep = np.isin(keys, res["filtered_keys"])
    gk, gp = keys[keep], packed[keep]
    o = np.lexsort((gp, gk))
    p = res["points"]
    op = p["packed_x"].astype(np.uint64) | (p["packed_y"].astype(np.uint64) << np.uint64(16))
    okeep = np.isin(res["keys"], res["filtered_keys"])
    ok, op = res["keys"][okeep], op[okeep]
    o2 = np.lexsort((op, ok))
    return (gk[o], gp[o]), (ok[o2], op[o2])


def assert_quads_match(gpu_q, ora_q, tol=CORNER_TOL_PX):
    assert len(gpu_q) == len(ora_q), (len(gpu_q), len(ora_q))
    if len(gpu_q):
        d = np.abs(gpu_q["corners"].astype(np.float64) - ora_q["corners"].astype(np.float64))
        assert np.all(d <= tol), float(d.max())
        assert np.array_equal(gpu_q["reversed_border"], ora_q["reversed_border"])
        assert np.array_equal(gpu_q["blob_index"], ora_q["blob_index"])


def assert_detect_matches(views, gpu_quads, res, cfg_compat=True):
    st = views["stats"]
    assert st["status"] == 0, hex(int(st["status"]))
    assert (int(st["width"]), int(st["height"])) == (res["width"], res["height"])
    assert_same(views["thresholded"], res["thresholded"], "thresholded")
    assert_same(views["labels"], res["labels"], "labels")
    assert_same(views["sizes"], res["sizes"], "sizes")
    assert int(st["n_points"]) == len(res["points"])
    for name, g, o in zip(("key", "count", "x_min", "x_max", "y_min", "y_max", "gx_sum", "gy_sum", "pxgx"),
                          pair_table(views), oracle_pair_table(res)):
        assert_same(np.asarray(g).astype(np.int64), np.asarray(o).astype(np.int64), f"pair {name}")
    (gk, gp), (ok, op) = surviving_point_sets(views, res)
    assert_same(gk, ok, "surviving point keys")
    assert_same(gp, op, "surviving points")
    assert int(st["n_pairs"]) == len(res["bounds"])
    assert int(st["n_clusters"]) == len(res["filtered"])
    assert_same(views["cluster_keys"], res["filtered_keys"], "cluster_keys")
    assert_same(views["cluster_bounds"], res["filtered"], "cluster_bounds")
    assert_same(views["cluster_extents"], res["extents"], "cluster_extents")
    assert int(st["n_cluster_points"]) == len(res["cluster_points"])
    assert_same(views["cluster_points"], res["cluster_points"], "cluster_points")
    assert_same(views["line_fit"], res["line_fit"], "line_fit")
    counts, top = oracle_top10(res)
    assert_same(views["peak_count"], counts, "peak_count")
    for c, seg in top.items():
        assert_same(views["peaks"][c][: len(seg)], seg, f"peaks of cluster {c}")
    assert int(st["n_corners"]) == len(res["corners"])
    assert int(st["n_peak_clusters"]) == len(res["peak_extents"])
    assert_same(views["peak_extents"], res["peak_extents"], "peak_extents")
    assert_same(views["fitted"], res["fitted"], "fitted")
    assert_quads_match(gpu_quads, res["quads"])
