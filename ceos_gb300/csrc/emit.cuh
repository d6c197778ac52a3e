// Candidate emission of the fused bucket build (PROJ_EMIT), shared by the FP32
// and the tensor-core projection kernels.
//
// A projected value v of column `col` is a candidate of the column's close end
// when fkey(v) >= th[col].x and of its far end when fkey(-v) >= th[col].y
// (src/CEOs.cpp:377-412 keeps the same two ends with two heaps). The kernels
// first test every value against the float bounds thf[col] (emit_bounds), a
// superset test that costs two compares; only values that pass it reach
// emit_exact, which applies the exact key test and appends the packed
// (value, id) key to the column end's candidate list. Which values become
// candidates is therefore decided by the keys alone, as without the prefilter.
// (A NaN projection never passes the float test and is never emitted.)
#pragma once

#include "kernels.h"
#include "common.cuh"

namespace ceos {

CEOS_DEV bool emit_maybe(float v, float2 b) { return v >= b.x || v <= b.y; }

CEOS_DEV void emit_exact(const ProjArgs& a, int col, float v, int id) {
  if (a.col_active && !a.col_active[col]) return;
  const uint2 th = __ldg(reinterpret_cast<const uint2*>(a.th) + col);
  if (fkey(v) >= th.x) {
    const unsigned pos = atomicAdd(&a.cnt[2 * col], 1u);
    if (pos < (unsigned)a.cap) a.cand[((long)2 * col) * a.cap + pos] = pack_key(v, id);
  }
  if (fkey(-v) >= th.y) {
    const unsigned pos = atomicAdd(&a.cnt[2 * col + 1], 1u);
    if (pos < (unsigned)a.cap) a.cand[((long)2 * col + 1) * a.cap + pos] = pack_key(-v, id);
  }
}

// emit_exact for a value that passed the prefilter with the float bounds b
// of its column: for a finite nonzero v the float tests are exact (the bounds
// are the floats of the threshold keys themselves, see key_lower_bound), so
// only zeros (-0 ranks below +0) and infinities read the keys.
CEOS_DEV void emit_exact_b(const ProjArgs& a, int col, float v, int id, float2 b) {
  if (!(v != 0.0f && isfinite(v))) {
    emit_exact(a, col, v, id);
    return;
  }
  if (a.col_active && !a.col_active[col]) return;
  if (v >= b.x) {
    const unsigned pos = atomicAdd(&a.cnt[2 * col], 1u);
    if (pos < (unsigned)a.cap) a.cand[((long)2 * col) * a.cap + pos] = pack_key(v, id);
  }
  if (v <= b.y) {
    const unsigned pos = atomicAdd(&a.cnt[2 * col + 1], 1u);
    if (pos < (unsigned)a.cap) a.cand[((long)2 * col + 1) * a.cap + pos] = pack_key(-v, id);
  }
}

}  // namespace ceos
