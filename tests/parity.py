"""Comparison rules for results checked against the reference.

* Buckets: every value bit-identical; ids identical except inside a run of
  exactly tied values, where the reference's heap leaves the tied ids in an
  implementation-defined order (src/Header.h:53-80 compares values only) and
  this library orders them by id. Inside such a run the id multisets must
  agree, unless the run reaches the end of the list, where the reference may
  keep a different member of a tie that straddles the cut.
* Searches: final top-k ids equal in at least 99.9% of queries, any other
  query differing only where the reported scores are near-tied; scores within
  1e-5 relative (the reference's Eigen dot and this library's 8-lane order
  differ in the last bits). For sets of fewer than 1,000 queries the 99.9%
  bar is read as one differing (near-tied) query allowed.
"""
from __future__ import annotations

import hashlib

import numpy as np

SCORE_RTOL = 1e-5
IDS_EQUAL_MIN = 0.999


def sha256(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode() + str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def compare_buckets(ids_a, vals_a, ids_b, vals_b, check_values=True):
    """Returns (ok, n_tie_runs_reordered, message) for [C][2][m] buckets."""
    ids_a = np.asarray(ids_a).reshape(-1, ids_a.shape[-1])
    ids_b = np.asarray(ids_b).reshape(-1, ids_b.shape[-1])
    va = np.asarray(vals_a, np.float32).reshape(ids_a.shape)
    vb = np.asarray(vals_b, np.float32).reshape(ids_b.shape)
    if check_values and not np.array_equal(va.view(np.uint32), vb.view(np.uint32)):
        bad = np.argwhere(va.view(np.uint32) != vb.view(np.uint32))
        return False, 0, f"bucket values differ at {len(bad)} entries, first {bad[0].tolist()}"
    diff_rows = np.nonzero(np.any(ids_a != ids_b, axis=1))[0]
    reordered = 0
    m = ids_a.shape[1]
    for r in diff_rows:
        key = va[r] if check_values else None
        j = 0
        while j < m:
            if ids_a[r, j] == ids_b[r, j]:
                j += 1
                continue
            if key is None:
                return False, reordered, f"bucket ids differ in column end {r} at {j}"
            # the tie run holding position j
            lo = j
            while lo > 0 and key[lo - 1] == key[j]:
                lo -= 1
            hi = j + 1
            while hi < m and key[hi] == key[j]:
                hi += 1
            # a run that reaches the end of the list may continue past the cut
            if hi - lo < 2 and hi < m:
                return False, reordered, (f"bucket ids differ outside a tie in column end {r} at {j}: "
                                          f"{ids_a[r, j]} vs {ids_b[r, j]}")
            if hi < m and sorted(ids_a[r, lo:hi]) != sorted(ids_b[r, lo:hi]):
                return False, reordered, f"tie run [{lo}, {hi}) of column end {r} holds other ids"
            reordered += 1
            j = hi
    return True, reordered, "ok"


def compare_results(ids_a, d_a, ids_b, d_b, rtol=SCORE_RTOL, min_equal=IDS_EQUAL_MIN):
    """Returns (ok, stats) for two (n_queries x k) search results."""
    ids_a, ids_b = np.asarray(ids_a), np.asarray(ids_b)
    d_a, d_b = np.asarray(d_a, np.float64), np.asarray(d_b, np.float64)
    nq = ids_a.shape[0]
    if ids_a.shape != ids_b.shape:
        return False, {"message": f"shapes {ids_a.shape} vs {ids_b.shape}"}
    if nq == 0 or ids_a.shape[1] == 0:
        return True, {"ids_equal_frac": 1.0, "max_rel_score_err": 0.0, "near_tie_rows": 0}
    rows_equal = np.all(ids_a == ids_b, axis=1)
    scale = np.maximum(np.maximum(np.abs(d_a), np.abs(d_b)), 1e-30)
    same = ids_a == ids_b
    rel = np.where(same, np.abs(d_a - d_b) / scale, 0.0)
    max_rel = float(rel.max())
    # a differing row must agree on its score list (the ids differ only among
    # near-tied scores)
    near_tie_rows = 0
    bad_rows = []
    for q in np.nonzero(~rows_equal)[0]:
        if np.all(np.abs(d_a[q] - d_b[q]) <= rtol * scale[q]):
            near_tie_rows += 1
        else:
            bad_rows.append(int(q))
    frac = float(rows_equal.mean())
    stats = {"ids_equal_frac": frac, "max_rel_score_err": max_rel, "near_tie_rows": near_tie_rows,
             "other_rows": bad_rows[:10]}
    allowed = max(1, int(np.floor((1.0 - min_equal) * nq + 1e-9)))
    ok = int((~rows_equal).sum()) <= allowed and max_rel <= rtol and not bad_rows
    return ok, stats
