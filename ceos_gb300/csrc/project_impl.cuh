// Kernel body and launcher of the projection kernels; instantiated per
// log2(fhtDim) in project_l*.cu so the instantiations compile in parallel.
#pragma once
// Projection kernels: the reference's per-row projection block
// (src/CEOs.cpp:58-88, :343-372, :746-775; src/streamCEOs.cpp:55-86,
// :229-259) and its query twin (src/CEOs.cpp:143-161, :495-513, :895-913).
//
// One kernel body, three consumers of the projected values:
//   ROWS : row-major [rows][R*D]            (query projections)
//   COLS : column-major [slot][ld]          (dense CEOs-Est index; sample and
//                                            fallback dumps of chosen columns)
//   EMIT : no projection matrix at all. Each value is compared against the
//          per-column selection thresholds of the bucket build and, when it
//          can still be among the column's top-m (close end) or bottom-m
//          (far end), its packed (value, id) key is appended to that column
//          end's candidate list. This fuses the projection with the first
//          pass of the two-ended top-m selection (src/CEOs.cpp:377-432), so
//          the n x (R*D) projection matrix never travels to HBM.
#include "kernels.h"
#include "fwht.cuh"
#include "emit.cuh"

namespace ceos {

// Work split: each warp processes V rows (V vectors) at a time, all R
// repeats, grid-striding over row groups.
// Warps per CTA: 8, or 4 when two 4096-float vectors per warp would not fit.
template <int L>
constexpr int proj_warps() {
  return L >= 12 ? 4 : 8;
}

// When a lane's phase-0 lines fit in registers (RegRow<L>::ok: F = 256, 1024
// and below), the input rows are loaded straight into registers in that
// layout and round 0 starts from them; each warp then needs a single
// shared-memory buffer, which leaves L1 room for the candidate thresholds.
template <int L, int MODE>
__global__ void __launch_bounds__(256, RegRow<L>::ok ? 3 : 1) k_project(ProjArgs a) {
  using Cfg = FwhtCfg<L>;
  constexpr bool kRegRow = RegRow<L>::ok;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int words = Cfg::words;
  uint32_t* s_signs = reinterpret_cast<uint32_t*>(smem_raw);
  const int n_sign_words = a.R * 3 * words;
  float* s_vec = reinterpret_cast<float*>(smem_raw + ((n_sign_words * 4 + 15) & ~15));

  for (int i = threadIdx.x; i < n_sign_words; i += blockDim.x) s_signs[i] = a.signs[i];
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int warps_per_block = blockDim.x >> 5;
  constexpr int kBufs = kRegRow ? 1 : 2;
  float* xbuf = s_vec + (size_t)warp * kBufs * Cfg::V * Cfg::Vstride;
  float* wbuf = xbuf + (kBufs - 1) * Cfg::V * Cfg::Vstride;
  const int C = a.R * a.D;

  const long n_groups = (a.n_rows + Cfg::V - 1) / Cfg::V;
  for (long g = (long)blockIdx.x * warps_per_block + warp; g < n_groups;
       g += (long)gridDim.x * warps_per_block) {
    const long row0 = g * Cfg::V;
    float xr[RegRow<L>::T][RegRow<L>::E];
    if constexpr (kRegRow) {
      // ---- load V rows (zero padded to F) into the phase-0 register layout ----
      constexpr int E = RegRow<L>::E, lines0 = Cfg::F / E;
#pragma unroll
      for (int t = 0; t < RegRow<L>::T; ++t) {
        const int task = lane + 32 * t;
        const int v = task / lines0;
        const int j0 = (task % lines0) * E;
        const long row = row0 + v;
        const float4* src = nullptr;
        if (row < a.n_rows) {
          long r = a.row_map ? a.row_map[row] : row;
          r += a.head;
          if (r >= a.cap_rows) r -= a.cap_rows;
          src = reinterpret_cast<const float4*>(a.X + r * a.ldx + j0);
        }
#pragma unroll
        for (int k = 0; k < E / 4; ++k) {
          // rows are zero padded up to ldx (a multiple of 8)
          const float4 q = (src && j0 + 4 * k < a.ldx) ? __ldg(src + k) : make_float4(0.f, 0.f, 0.f, 0.f);
          xr[t][4 * k] = q.x;
          xr[t][4 * k + 1] = q.y;
          xr[t][4 * k + 2] = q.z;
          xr[t][4 * k + 3] = q.w;
        }
      }
    } else
    // ---- load V rows (zero padded to F) ----
    for (int idx = lane; idx < Cfg::V * Cfg::F; idx += 32) {
      const int v = idx / Cfg::F;
      const int j = idx % Cfg::F;
      const long row = row0 + v;
      float x = 0.0f;
      if (row < a.n_rows && j < a.d) {
        long src = a.row_map ? a.row_map[row] : row;
        src += a.head;
        if (src >= a.cap_rows) src -= a.cap_rows;
        x = a.X[src * a.ldx + j];
      }
      xbuf[v * Cfg::Vstride + padj(j)] = x;
    }
    __syncwarp();
    for (int r = 0; r < a.R; ++r) {
      const uint32_t* sw = s_signs + (size_t)r * 3 * words;
      // Consumer of the last phase of round 2: the lane's output lines in
      // registers, element e of a line at column offset j0 + (e << o).
      auto out = [&](int vec, int line, auto& v) {
        constexpr int o = Cfg::off(Cfg::P - 1);
        constexpr int B = Cfg::bits(Cfg::P - 1);
        constexpr int E = 1 << B;
        const long row = row0 + vec;
        if (row >= a.n_rows) return;
        const int j0 = line_elem(line, 0, o, B);
        const bool all_cols = (a.D == Cfg::F);  // else keep outputs j < D only
        if constexpr (MODE == PROJ_ROWS) {
          float* dst = a.out + row * (long)C + r * a.D + j0;
#pragma unroll
          for (int e = 0; e < E; ++e)
            if (all_cols || j0 + (e << o) < a.D) dst[e << o] = v[e];
        } else if constexpr (MODE == PROJ_COLS) {
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int j = j0 + (e << o);
            if (all_cols || j < a.D) {
              const int col = r * a.D + j;
              const int slot = a.col_slot ? a.col_slot[col] : col;
              if (slot >= 0) a.out[(long)slot * a.ld_out + row] = v[e];
            }
          }
        } else {  // PROJ_EMIT
          // float prefilter of every output into a bit mask, then the exact
          // test of the (few) flagged outputs, read back through this lane's
          // own slots of the vector buffer
          const float2* tb = a.thf + r * a.D + j0;
          uint32_t hit = 0;
#pragma unroll
          for (int e = 0; e < E; ++e)
            if (all_cols || j0 + (e << o) < a.D)
              if (emit_maybe(v[e], __ldg(tb + (e << o)))) hit |= 1u << e;
          if (hit) {
            float* w = wbuf + vec * Cfg::Vstride;
#pragma unroll
            for (int e = 0; e < E; ++e) w[padj(j0) + padj_c(e << o)] = v[e];
            const int id = (int)(a.id_base + (a.row_map ? a.row_map[row] : row));
            do {
              const int e = __ffs((int)hit) - 1;
              hit &= hit - 1;
              const int j = j0 + (e << o);
              emit_exact_b(a, r * a.D + j, w[padj(j)], id, __ldg(tb + (e << o)));
            } while (hit);
          }
        }
      };
      if constexpr (kRegRow) {
        fwht_round_regs<L>(xr, wbuf, sw, lane);
      } else {
        fwht_round<L>(xbuf, wbuf, sw, lane);
      }
#pragma unroll 1
      for (int i = 1; i < 3; ++i) fwht_round_out<L>(wbuf, wbuf, sw + i * words, lane, i == 2, out);
      __syncwarp();
    }
  }
}

template <int L>
static size_t proj_smem(int R) {
  using Cfg = FwhtCfg<L>;
  size_t sw = ((size_t)R * 3 * Cfg::words * 4 + 15) & ~(size_t)15;
  const int bufs = RegRow<L>::ok ? 1 : 2;
  return sw + (size_t)proj_warps<L>() * bufs * Cfg::V * Cfg::Vstride * sizeof(float);
}

template <int L, int MODE>
cudaError_t launch_L(const ProjArgs& a, int num_sms, cudaStream_t st) {
  const size_t smem = proj_smem<L>(a.R);
  cudaError_t e = cudaFuncSetAttribute(k_project<L, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  constexpr int threads = 32 * proj_warps<L>();
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_project<L, MODE>, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  using Cfg = FwhtCfg<L>;
  const long groups = (a.n_rows + Cfg::V - 1) / Cfg::V;
  long blocks = (groups + proj_warps<L>() - 1) / proj_warps<L>();
  const long max_blocks = (long)num_sms * per_sm;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks < 1) blocks = 1;
  k_project<L, MODE><<<(unsigned)blocks, threads, smem, st>>>(a);
  return cudaGetLastError();
}

template <int L>
cudaError_t launch_project_L(const ProjArgs& a, int mode, int num_sms, cudaStream_t st) {
  switch (mode) {
    case PROJ_ROWS: return launch_L<L, PROJ_ROWS>(a, num_sms, st);
    case PROJ_COLS: return launch_L<L, PROJ_COLS>(a, num_sms, st);
    case PROJ_EMIT: return launch_L<L, PROJ_EMIT>(a, num_sms, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ceos
