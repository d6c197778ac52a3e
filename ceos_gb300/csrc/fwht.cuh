// Bit-exact seeded sign-flip + Walsh-Hadamard projection on the GPU.
//
// The reference computes, for every row x (zero-padded to F = 2^L) and every
// repeat r, three rounds of {v_j *= +-1 ; v = FWHT(v)} and keeps the first D
// outputs (src/CEOs.cpp:58-88, query side :143-161). Its FWHT is FFHT's
// fht_float (src/fht_avx.c:10081), which is bit-identical to the radix-2
// butterfly applied in ASCENDING stage order: stage s maps every pair of
// indices (j, j + 2^s) with bit s of j clear to (a + b, a - b).
//
// GPU form. One warp owns V vectors (V = 1 for F = 1024). The vector lives in
// shared memory between "phases"; a phase applies a contiguous run of stages
// [o, o + b) entirely in registers: a lane loads a "line" of E = 2^b elements
// whose indices differ only in bits [o, o + b), runs the b butterfly stages
// on them in ascending order, and stores them back. The stage order, and
// therefore every rounding, is the reference's. Phase 0 (bits [0, b0)) reads
// contiguous chunks and applies the sign flip of the round while loading, as
// an XOR of the float sign bit (identical to multiplying by +-1.0f, -0.0
// included). The last phase of the last round leaves the outputs in
// registers, where the callers consume them (store, or compare against
// selection thresholds).
//
// Shared memory is padded by 4 floats every 32 so that phase 0 (lane stride of
// E floats) and the last phase (consecutive lanes on consecutive indices) are
// both free of bank conflicts.
#pragma once

#include "common.cuh"

namespace ceos {

template <int L>
struct FwhtCfg {
  static constexpr int F = 1 << L;
  static constexpr int P = (L + 4) / 5;  // phases of at most 5 stages
  __host__ __device__ static constexpr int bits(int p) { return L / P + (p < L % P ? 1 : 0); }
  __host__ __device__ static constexpr int off(int p) { return p == 0 ? 0 : off(p - 1) + bits(p - 1); }
  __host__ __device__ static constexpr int E(int p) { return 1 << bits(p); }
  static constexpr int Emax = 1 << (L / P + (L % P ? 1 : 0));
  static constexpr int V = (32 * Emax / F) > 1 ? (32 * Emax / F) : 1;  // vectors per warp
  __host__ __device__ static constexpr int tasks(int p) { return V * F / (32 * E(p)); }    // lines per lane
  static constexpr int Fpad = F + (F >= 32 ? (F / 32) * 4 : 0);
  // vector stride in smem; an extra 16 floats de-phases the banks of the V
  // vectors that share a warp
  static constexpr int Vstride = Fpad + (V > 1 ? 16 : 0);
  static constexpr int words = F >= 32 ? F / 32 : 1;  // sign words per round
};

CEOS_DEV int padj(int j) { return j + ((j >> 5) << 2); }

// Index of element e of line `line` in a phase covering bits [o, o + b).
CEOS_DEV int line_elem(int line, int e, int o, int b) {
  const int low = line & ((1 << o) - 1);
  const int high = line >> o;
  return low | (e << o) | (high << (o + b));
}

// The line's part and the element's part of an index occupy disjoint bits, so
// padj(line_elem(line, e, o, b)) = padj(line_elem(line, 0, o, b)) + padj(e << o):
// one base per line plus a compile-time offset per element.
__host__ __device__ constexpr int padj_c(int j) { return j + ((j >> 5) << 2); }

// Two butterflies at once: (a0, c0) and (a1, c1) become (a0+c0, a0-c0) and
// (a1+c1, a1-c1), as packed f32x2 adds/subtracts (two IEEE round-to-nearest
// operations each, so the results are those of the scalar form).
CEOS_DEV void bfly2(float& a0, float& a1, float& c0, float& c1) {
  unsigned long long A, C, S, D;
  asm("mov.b64 %0, {%1, %2};" : "=l"(A) : "f"(a0), "f"(a1));
  asm("mov.b64 %0, {%1, %2};" : "=l"(C) : "f"(c0), "f"(c1));
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(S) : "l"(A), "l"(C));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(D) : "l"(A), "l"(C));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a0), "=f"(a1) : "l"(S));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(c0), "=f"(c1) : "l"(D));
}

// Butterfly stages [0, b) of a register line (stage s pairs e and e + 2^s).
// Stages with a stride of 2 or more pair up adjacent butterflies into f32x2
// operations on register pairs (e, e+1) and (e+h, e+h+1).
template <int B>
CEOS_DEV void reg_stages(float (&v)[1 << B]) {
  constexpr int E = 1 << B;
#pragma unroll
  for (int s = 0; s < B; ++s) {
    const int h = 1 << s;
    if (h == 1) {
#pragma unroll
      for (int e = 0; e < E; e += 2) {
        const float a = v[e], c = v[e + 1];
        v[e] = a + c;
        v[e + 1] = a - c;
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; e += 2 * h) {
#pragma unroll
        for (int k = 0; k < h; k += 2) bfly2(v[e + k], v[e + k + 1], v[e + k + h], v[e + k + 1 + h]);
      }
    }
  }
}

// Phase p >= 1 of a round: bits [off(p), off(p) + bits(p)) in registers.
template <int L, int p>
CEOS_DEV void fwht_phase(float* dst, int lane) {
  using Cfg = FwhtCfg<L>;
  constexpr int o = Cfg::off(p);
  constexpr int B = Cfg::bits(p);
  constexpr int E = 1 << B;
  constexpr int lines = Cfg::F / E;
  __syncwarp();
#pragma unroll
  for (int t = 0; t < Cfg::tasks(p); ++t) {
    const int task = lane + 32 * t;
    const int vec = task / lines;
    const int line = task % lines;
    float* d = dst + vec * Cfg::Vstride + padj(line_elem(line, 0, o, B));
    float v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = d[padj_c(e << o)];
    reg_stages<B>(v);
#pragma unroll
    for (int e = 0; e < E; ++e) d[padj_c(e << o)] = v[e];
  }
  if constexpr (p + 1 < Cfg::P) fwht_phase<L, p + 1>(dst, lane);
}

// One full round (sign flip + FWHT) on the warp's V vectors.
//  src: smem base the round reads from (V vectors, stride Vstride)
//  dst: smem base it writes to (may equal src)
//  sw : 32-bit sign words of this round (bit j set => multiply by +1)
// Phase 0 covers the lowest index bits, so its lines are contiguous chunks
// and move as float4 when they are at least 4 elements long.
template <int L>
CEOS_DEV void fwht_round(const float* src, float* dst, const uint32_t* sw, int lane) {
  using Cfg = FwhtCfg<L>;
  constexpr int B = Cfg::bits(0);
  constexpr int E = 1 << B;
  constexpr int lines0 = Cfg::F / E;
#pragma unroll
  for (int t = 0; t < Cfg::tasks(0); ++t) {
    const int task = lane + 32 * t;
    const int vec = task / lines0;
    const int line = task % lines0;
    const int j0 = line * E;
    const float* s = src + vec * Cfg::Vstride + padj(j0);
    float* d = dst + vec * Cfg::Vstride + padj(j0);
    const uint32_t nword = ~(sw[j0 >> 5] >> (j0 & 31));  // bit e set => flip
    float v[E];
    if constexpr (E >= 4) {
#pragma unroll
      for (int k = 0; k < E / 4; ++k) {
        const float4 q = reinterpret_cast<const float4*>(s)[k];
        v[4 * k] = q.x;
        v[4 * k + 1] = q.y;
        v[4 * k + 2] = q.z;
        v[4 * k + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = s[e];
    }
#pragma unroll
    for (int e = 0; e < E; ++e)
      v[e] = __uint_as_float(__float_as_uint(v[e]) ^ ((nword << (31 - e)) & 0x80000000u));
    reg_stages<B>(v);
    if constexpr (E >= 4) {
#pragma unroll
      for (int k = 0; k < E / 4; ++k)
        reinterpret_cast<float4*>(d)[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) d[e] = v[e];
    }
  }
  if constexpr (Cfg::P > 1) fwht_phase<L, 1>(dst, lane);
  __syncwarp();
}

// Phases p.. of a round whose last phase may hand its lines to a consumer
// instead of storing them: when `emit` is set, phase P-1 calls
// out(vec, line, v) with the E = 2^bits(P-1) outputs of each of the lane's
// lines in registers; element e of the line is output
// line_elem(line, e, off(P-1), bits(P-1)) of vector vec. When `emit` is clear
// the round stores its outputs like fwht_round (the branch is warp-uniform).
template <int L, int p, class Out>
CEOS_DEV void fwht_phase_out(float* dst, int lane, bool emit, Out& out) {
  using Cfg = FwhtCfg<L>;
  constexpr int o = Cfg::off(p);
  constexpr int B = Cfg::bits(p);
  constexpr int E = 1 << B;
  constexpr int lines = Cfg::F / E;
  constexpr bool last = (p + 1 == Cfg::P);
  __syncwarp();
#pragma unroll
  for (int t = 0; t < Cfg::tasks(p); ++t) {
    const int task = lane + 32 * t;
    const int vec = task / lines;
    const int line = task % lines;
    float* d = dst + vec * Cfg::Vstride + padj(line_elem(line, 0, o, B));
    float v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = d[padj_c(e << o)];
    reg_stages<B>(v);
    if (last && emit) {
      out(vec, line, v);
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) d[padj_c(e << o)] = v[e];
    }
  }
  if constexpr (!last) fwht_phase_out<L, p + 1>(dst, lane, emit, out);
}

// fwht_round whose last phase feeds `out` (see fwht_phase_out) when `emit`.
template <int L, class Out>
CEOS_DEV void fwht_round_out(const float* src, float* dst, const uint32_t* sw, int lane, bool emit,
                             Out& out) {
  using Cfg = FwhtCfg<L>;
  constexpr int B = Cfg::bits(0);
  constexpr int E = 1 << B;
  constexpr int lines0 = Cfg::F / E;
  constexpr bool last = (Cfg::P == 1);
#pragma unroll
  for (int t = 0; t < Cfg::tasks(0); ++t) {
    const int task = lane + 32 * t;
    const int vec = task / lines0;
    const int line = task % lines0;
    const int j0 = line * E;
    const float* s = src + vec * Cfg::Vstride + padj(j0);
    float* d = dst + vec * Cfg::Vstride + padj(j0);
    const uint32_t nword = ~(sw[j0 >> 5] >> (j0 & 31));  // bit e set => flip
    float v[E];
    if constexpr (E >= 4) {
#pragma unroll
      for (int k = 0; k < E / 4; ++k) {
        const float4 q = reinterpret_cast<const float4*>(s)[k];
        v[4 * k] = q.x;
        v[4 * k + 1] = q.y;
        v[4 * k + 2] = q.z;
        v[4 * k + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = s[e];
    }
#pragma unroll
    for (int e = 0; e < E; ++e)
      v[e] = __uint_as_float(__float_as_uint(v[e]) ^ ((nword << (31 - e)) & 0x80000000u));
    reg_stages<B>(v);
    if (last && emit) {
      out(vec, line, v);
    } else if constexpr (E >= 4) {
#pragma unroll
      for (int k = 0; k < E / 4; ++k)
        reinterpret_cast<float4*>(d)[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) d[e] = v[e];
    }
  }
  if constexpr (Cfg::P > 1) fwht_phase_out<L, 1>(dst, lane, emit, out);
  __syncwarp();
}

// Round 0 with its input in registers (phase-0 line layout: task t of the
// lane holds the E contiguous elements of line lane + 32 t), output to dst.
// Used when the phase-0 lines of a lane fit in 32 registers, so the input row
// needs no shared-memory copy.
template <int L>
struct RegRow {
  static constexpr int E = 1 << FwhtCfg<L>::bits(0);
  static constexpr int T = FwhtCfg<L>::tasks(0);
  static constexpr bool ok = E * T <= 32 && E >= 4;
};

template <int L>
CEOS_DEV void fwht_round_regs(const float (&x)[RegRow<L>::T][RegRow<L>::E], float* dst,
                              const uint32_t* sw, int lane) {
  using Cfg = FwhtCfg<L>;
  constexpr int B = Cfg::bits(0);
  constexpr int E = 1 << B;
  constexpr int lines0 = Cfg::F / E;
#pragma unroll
  for (int t = 0; t < RegRow<L>::T; ++t) {
    const int task = lane + 32 * t;
    const int vec = task / lines0;
    const int line = task % lines0;
    const int j0 = line * E;
    float* d = dst + vec * Cfg::Vstride + padj(j0);
    const uint32_t nword = ~(sw[j0 >> 5] >> (j0 & 31));  // bit e set => flip
    float v[E];
#pragma unroll
    for (int e = 0; e < E; ++e)
      v[e] = __uint_as_float(__float_as_uint(x[t][e]) ^ ((nword << (31 - e)) & 0x80000000u));
    reg_stages<B>(v);
#pragma unroll
    for (int k = 0; k < E / 4; ++k)
      reinterpret_cast<float4*>(d)[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
  }
  if constexpr (Cfg::P > 1) fwht_phase<L, 1>(dst, lane);
  __syncwarp();
}

}  // namespace ceos
