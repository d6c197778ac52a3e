// Split-precision projection on the tensor cores (no reference counterpart:
// the reference's FFHT is FP32 CUDA-free code, src/fht_avx.c). Same outputs as
// k_project (ROWS / COLS / EMIT, project_impl.cuh) for fhtDim F = FD * FD with
// FD in {16, 32}, i.e. F in {256, 1024}.
//
// With Sylvester ordering H_F = H_FD (x) H_FD, so for a vector x read as the
// FD x FD row-major matrix X, FWHT(x) read the same way is H_FD . X . H_FD.
// Each of the three rounds of a repeat is therefore
//   A = signs (.) X ;  Y = A . H ;  Z = H . Y ;  X <- Z
// computed with warp-level BF16 tensor-core products (mma m16n8k16, FP32
// accumulation). The +-1 entries of H are exact in BF16; every FP32 operand
// v is split into hi = bf16(v) and lo = bf16(v - hi) and both halves are
// multiplied, so the operands carry 16 mantissa bits and the result differs
// from the FP32 butterflies by about 2^-16 relative per round.
//
// Everything stays in registers: the accumulator fragment of Y (rows g, g+8,
// column pairs 2t, 2t+1 of each 16x8 tile) is, packed to BF16 pairs, an 8x8
// matrix fragment; movmatrix.trans turns it into the B-operand fragment of
// H . Y, and the accumulator fragment of Z is already the A-operand fragment
// of the next round's X . H.
//
// Why warp-level mma rather than tcgen05: each vector needs six dependent
// K = 32 products per repeat, with a transpose between the two products of a
// round. tcgen05 takes its B operand (and A unless in TMEM) from shared memory
// and writes its accumulator to tensor memory, so every product would be a
// TMEM -> register -> shared memory round trip plus an mbarrier wait; the
// register-resident chain here has no such traffic.
#include <cstdlib>

#include "kernels.h"
#include "common.cuh"
#include "emit.cuh"

namespace ceos {

namespace {

CEOS_DEV void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// (lo, hi) -> bf16x2 with lo in the low half
CEOS_DEV uint32_t pack_bf16(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// Split two floats into bf16x2 hi and lo parts: v ~= hi + lo.
CEOS_DEV void split2(float v0, float v1, uint32_t& hi, uint32_t& lo) {
  hi = pack_bf16(v0, v1);
  const float h0 = __uint_as_float(hi << 16), h1 = __uint_as_float(hi & 0xffff0000u);
  lo = pack_bf16(v0 - h0, v1 - h1);
}

CEOS_DEV uint32_t trans8x8(uint32_t x) {
  uint32_t r;
  asm volatile("movmatrix.sync.aligned.m8n8.trans.b16 %0, %1;" : "=r"(r) : "r"(x));
  return r;
}

// Sylvester Hadamard entry as bf16 bits: +1 (0x3F80) or -1 (0xBF80).
CEOS_DEV uint32_t hbits(int i, int j) { return (__popc(i & j) & 1) ? 0xBF80u : 0x3F80u; }
CEOS_DEV uint32_t hpair(int i0, int j0, int i1, int j1) { return hbits(i0, j0) | (hbits(i1, j1) << 16); }

// Sign flip of an element whose (inverted) sign bit is bit k of nw.
CEOS_DEV float flipn(float v, uint32_t nw, int k) {
  return __uint_as_float(__float_as_uint(v) ^ ((nw << (31 - k)) & 0x80000000u));
}

}  // namespace

// One warp per vector at a time; grid-strided over rows.
template <int FD, int MODE>
__global__ void __launch_bounds__(128, 4) k_project_tc(ProjArgs a) {
  constexpr int F = FD * FD;
  constexpr int MT = FD / 16;  // 16-row tiles
  constexpr int NT = FD / 8;   // 8-column tiles
  constexpr int KT = FD / 16;  // 16-deep k steps
  constexpr int WORDS = F / 32;
  extern __shared__ __align__(16) uint32_t s_signs[];  // [R][3][WORDS], then the emit scratch
  const int n_sign_words = a.R * 3 * WORDS;
  for (int i = threadIdx.x; i < n_sign_words; i += blockDim.x) s_signs[i] = a.signs[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int C = a.R * a.D;
  // PROJ_EMIT: per warp [32 elements][32 lanes] floats, this lane's column
  float* s_scr = reinterpret_cast<float*>(s_signs + ((n_sign_words + 3) & ~3)) + warp * 32 * 32 + lane;

  // constant H fragments: B operand of X.H (k = rows of H, n = columns) and
  // A operand of H.Y
  uint32_t hb[KT][NT][2], ha[MT][KT][4];
#pragma unroll
  for (int ki = 0; ki < KT; ++ki)
#pragma unroll
    for (int ni = 0; ni < NT; ++ni) {
      const int k0 = 16 * ki + 2 * t, n = 8 * ni + g;
      hb[ki][ni][0] = hpair(k0, n, k0 + 1, n);
      hb[ki][ni][1] = hpair(k0 + 8, n, k0 + 9, n);
    }
#pragma unroll
  for (int mi = 0; mi < MT; ++mi)
#pragma unroll
    for (int ki = 0; ki < KT; ++ki) {
      const int r0 = 16 * mi + g, c0 = 16 * ki + 2 * t;
      ha[mi][ki][0] = hpair(r0, c0, r0, c0 + 1);
      ha[mi][ki][1] = hpair(r0 + 8, c0, r0 + 8, c0 + 1);
      ha[mi][ki][2] = hpair(r0, c0 + 8, r0, c0 + 9);
      ha[mi][ki][3] = hpair(r0 + 8, c0 + 8, r0 + 8, c0 + 9);
    }

  for (long row = (long)blockIdx.x * wpb + warp; row < a.n_rows; row += (long)gridDim.x * wpb) {
    long src = a.row_map ? a.row_map[row] : row;
    src += a.head;
    if (src >= a.cap_rows) src -= a.cap_rows;
    const float* xr = a.X + src * a.ldx;
    long id = 0;
    if constexpr (MODE == PROJ_EMIT) id = a.id_base + (a.row_map ? a.row_map[row] : row);
    for (int r = 0; r < a.R; ++r) {
      // x in accumulator layout: z[mi][ni][e] = X[16mi + g + 8(e>>1)][8ni + 2t + (e&1)]
      // (reloaded per repeat from L1 rather than held in registers)
      float z[MT][NT][4];
#pragma unroll
      for (int mi = 0; mi < MT; ++mi)
#pragma unroll
        for (int ni = 0; ni < NT; ++ni)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            // an even element pair; rows are zero padded up to ldx (a multiple
            // of 8), so a pair starting below ldx lies inside the row
            const int j = (16 * mi + g + 8 * h) * FD + 8 * ni + 2 * t;
            const float2 p = j < a.ldx ? __ldg(reinterpret_cast<const float2*>(xr + j))
                                       : make_float2(0.0f, 0.0f);
            z[mi][ni][2 * h] = p.x;
            z[mi][ni][2 * h + 1] = p.y;
          }
#pragma unroll 1
      for (int round = 0; round < 3; ++round) {
        const uint32_t* sw = s_signs + ((size_t)r * 3 + round) * WORDS;
        // The sign bits of a fragment row i = 16 mi + g + 8 h: element
        // j = 8 ni + 2 t + c of the row has bit (i FD + j) of the round's
        // table, all in word (i FD) >> 5 (j < FD <= 32); nw[mi][h] holds that
        // word inverted (bit set => flip) and shifted so bit 8 ni + c is j's.
        uint32_t nw[MT][2];
#pragma unroll
        for (int mi = 0; mi < MT; ++mi)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int b0 = (16 * mi + g + 8 * h) * FD;
            nw[mi][h] = ~(sw[b0 >> 5] >> ((b0 & 31) + 2 * t));
          }
        // A fragments of signs (.) X, split hi / lo
        uint32_t ah[MT][KT][4], al[MT][KT][4];
#pragma unroll
        for (int mi = 0; mi < MT; ++mi)
#pragma unroll
          for (int ki = 0; ki < KT; ++ki)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              // q: 0 = (row g, cols 2t..), 1 = (row g+8), 2 = (row g, cols +8), 3 = (row g+8, cols +8)
              const int ni = 2 * ki + (q >> 1);
              const int e0 = (q & 1) ? 2 : 0;
              const float v0 = flipn(z[mi][ni][e0], nw[mi][q & 1], 8 * ni);
              const float v1 = flipn(z[mi][ni][e0 + 1], nw[mi][q & 1], 8 * ni + 1);
              split2(v0, v1, ah[mi][ki][q], al[mi][ki][q]);
            }
        // Y = A . H
        float y[MT][NT][4];
#pragma unroll
        for (int mi = 0; mi < MT; ++mi)
#pragma unroll
          for (int ni = 0; ni < NT; ++ni) {
#pragma unroll
            for (int e = 0; e < 4; ++e) y[mi][ni][e] = 0.0f;
#pragma unroll
            for (int ki = 0; ki < KT; ++ki) {
              mma_bf16(y[mi][ni], ah[mi][ki], hb[ki][ni][0], hb[ki][ni][1]);
              mma_bf16(y[mi][ni], al[mi][ki], hb[ki][ni][0], hb[ki][ni][1]);
            }
          }
        // B fragments of Y for H . Y: tile (ki = mi, ni), transposed 8x8 blocks
        uint32_t bh[KT][NT][2], bl[KT][NT][2];
#pragma unroll
        for (int mi = 0; mi < MT; ++mi)
#pragma unroll
          for (int ni = 0; ni < NT; ++ni) {
            uint32_t h0, l0, h1, l1;
            split2(y[mi][ni][0], y[mi][ni][1], h0, l0);
            split2(y[mi][ni][2], y[mi][ni][3], h1, l1);
            bh[mi][ni][0] = trans8x8(h0);
            bl[mi][ni][0] = trans8x8(l0);
            bh[mi][ni][1] = trans8x8(h1);
            bl[mi][ni][1] = trans8x8(l1);
          }
        // Z = H . Y
#pragma unroll
        for (int mi = 0; mi < MT; ++mi)
#pragma unroll
          for (int ni = 0; ni < NT; ++ni) {
#pragma unroll
            for (int e = 0; e < 4; ++e) z[mi][ni][e] = 0.0f;
#pragma unroll
            for (int ki = 0; ki < KT; ++ki) {
              mma_bf16(z[mi][ni], ha[mi][ki], bh[ki][ni][0], bh[ki][ni][1]);
              mma_bf16(z[mi][ni], ha[mi][ki], bl[ki][ni][0], bl[ki][ni][1]);
            }
          }
      }
      // outputs j < D of repeat r; element f = (mi * NT + ni) * 4 + e of the
      // lane is output j = (16 mi + g + 8 (e >> 1)) * FD + 8 ni + 2 t + (e & 1)
      const bool all_cols = (a.D == F);
      if constexpr (MODE == PROJ_EMIT) {
        // float prefilter into a bit mask, then the exact test of the flagged
        // outputs, read back through this lane's column of the warp scratch
        const float2* tb = a.thf + r * a.D;
        uint32_t hit = 0;
#pragma unroll
        for (int mi = 0; mi < MT; ++mi)
#pragma unroll
          for (int ni = 0; ni < NT; ++ni)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const int j = (16 * mi + g + 8 * (e >> 1)) * FD + 8 * ni + 2 * t + (e & 1);
              if (all_cols || j < a.D)
                if (emit_maybe(z[mi][ni][e], __ldg(tb + j))) hit |= 1u << ((mi * NT + ni) * 4 + e);
            }
        if (hit) {
#pragma unroll
          for (int mi = 0; mi < MT; ++mi)
#pragma unroll
            for (int ni = 0; ni < NT; ++ni)
#pragma unroll
              for (int e = 0; e < 4; ++e) s_scr[((mi * NT + ni) * 4 + e) * 32] = z[mi][ni][e];
          do {
            const int f = __ffs((int)hit) - 1;
            hit &= hit - 1;
            const int e = f & 3, ni = (f >> 2) % NT, mi = (f >> 2) / NT;
            const int j = (16 * mi + g + 8 * (e >> 1)) * FD + 8 * ni + 2 * t + (e & 1);
            emit_exact(a, r * a.D + j, s_scr[f * 32], (int)id);
          } while (hit);
        }
      } else {
#pragma unroll
        for (int mi = 0; mi < MT; ++mi)
#pragma unroll
          for (int ni = 0; ni < NT; ++ni)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const int j = (16 * mi + g + 8 * (e >> 1)) * FD + 8 * ni + 2 * t + (e & 1);
              if (!all_cols && j >= a.D) continue;
              const float v = z[mi][ni][e];
              const int col = r * a.D + j;
              if constexpr (MODE == PROJ_ROWS) {
                a.out[row * (long)C + col] = v;
              } else {  // PROJ_COLS
                const int slot = a.col_slot ? a.col_slot[col] : col;
                if (slot >= 0) a.out[(long)slot * a.ld_out + row] = v;
              }
            }
      }
    }
  }
}

template <int FD, int MODE>
static cudaError_t launch_tc(const ProjArgs& a, int num_sms, cudaStream_t st) {
  size_t smem = (((size_t)a.R * 3 * (FD * FD / 32) + 3) & ~(size_t)3) * 4;
  if (MODE == PROJ_EMIT) smem += (size_t)4 * 32 * 32 * 4;  // 4 warps x 32 elements x 32 lanes
  cudaError_t e = cudaFuncSetAttribute(k_project_tc<FD, MODE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_project_tc<FD, MODE>, 128, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  long blocks = (a.n_rows + 3) / 4;
  const long max_blocks = (long)num_sms * per_sm;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks < 1) blocks = 1;
  k_project_tc<FD, MODE><<<(unsigned)blocks, 128, smem, st>>>(a);
  return cudaGetLastError();
}

bool project_tc_supported(int L) { return L == 8 || L == 10; }

cudaError_t launch_project_tc(const ProjArgs& a, int mode, int L, int num_sms, cudaStream_t st) {
  if (a.n_rows <= 0) return cudaSuccess;
  if (L == 10) {
    // fhtDim 1024 runs on tcgen05 (project_t5.cu); CEOS_GB300_T5=0 selects
    // the warp-level form below (1.3x slower at 100k x 960)
    static const bool t5 = [] {
      const char* e = std::getenv("CEOS_GB300_T5");
      return !(e && e[0] == '0');
    }();
    if (t5) return launch_project_t5(a, mode, st, num_sms);
    switch (mode) {
      case PROJ_ROWS: return launch_tc<32, PROJ_ROWS>(a, num_sms, st);
      case PROJ_COLS: return launch_tc<32, PROJ_COLS>(a, num_sms, st);
      case PROJ_EMIT: return launch_tc<32, PROJ_EMIT>(a, num_sms, st);
    }
  } else if (L == 8) {
    switch (mode) {
      case PROJ_ROWS: return launch_tc<16, PROJ_ROWS>(a, num_sms, st);
      case PROJ_COLS: return launch_tc<16, PROJ_COLS>(a, num_sms, st);
      case PROJ_EMIT: return launch_tc<16, PROJ_EMIT>(a, num_sms, st);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace ceos
