// Split-precision projection for fhtDim F = 1024 on the fifth-generation tensor
// cores (tcgen05: operands in shared memory, accumulators in tensor memory).
// Same outputs as k_project (ROWS / COLS / EMIT, project_impl.cuh); no
// reference counterpart (the reference's FFHT is CPU code, src/fht.c).
//
// With Sylvester ordering H_1024 = H_128 (x) H_8: a vector x read as the
// 128 x 8 row-major matrix X transforms as H_128 . X . H_8. Each of the three
// rounds of a repeat, y = H_1024 (s (.) x), is
//   W = (S (.) X) . H_8          CUDA cores: sign flip, three butterfly stages
//   Y = H_128 . W                one tcgen05.mma product, K = 256
// for a tile of 16 vectors at once: the B operand holds W of all 16 vectors
// (N = 16 x 8 = 128 columns n = 8 v + j, MN-major in shared memory), A is
// [H_128 | H_128] (M = 128, K-major, written once), and W enters split into
// bfloat16 hi = bf16(w) (K rows 0..127) and lo = bf16(w - hi) (K rows
// 128..255), so the FP32 accumulator receives H . hi + H . lo. The +-1 entries
// of H are exact in bfloat16.
//
// One CTA per SM: 16 compute warps and one warp that issues the products.
// Two tiles are in flight: compute warps 8 g .. 8 g + 7 serve slot g. Warp w
// owns tensor-memory lane quarter q = w mod 4, i.e. row i = 32 q + l of the
// tile's vectors, for column half c = (w / 4) mod 2 (vectors 8 c .. 8 c + 7):
// lane i of the accumulator is the row that H_128 produced, and its 8 values
// per vector are exactly the row that H_8 mixes next, so no transposes are
// needed between rounds, and each thread writes its hi and lo values of a
// vector as one 16-byte store. While one group prepares its slot's operand,
// the tensor core multiplies the other's.
//
// Tensor memory holds the two 128-column accumulators and, in the other 256
// columns, the two tiles' input rows, staged once per tile and read back at
// the start of every repeat (each thread its own lane and columns). The
// groups and the issuing warp synchronize through mbarriers only: full[g]
// (one arrival per compute warp of group g, after its operand stores are
// fenced for the tensor core) and done[g] (tcgen05.commit of the product).
// Every wait is bounded and also gives up once the other side has recorded a
// fault; the fault (read by project_t5_take_faults) ends the CTA after a
// bounded wait for its products in flight, and the tensor memory is freed.
//
// Candidate emission (PROJ_EMIT): on an output step each warp gathers its
// flagged values in a shared-memory list, one value per lane and pass, and
// appends the list to the global candidate lists after its arrival, one
// entry per lane, while the tensor core multiplies its next operand.
#include "kernels.h"
#include "common.cuh"
#include "emit.cuh"

namespace ceos {

namespace {

constexpr int kT5Threads = 512;  // compute threads; one more warp issues the products
// tiles in flight, one per compute group (four tiles of 8 vectors, N = 64,
// ran slower: twice the products per vector)
constexpr int kSlots = 2;
constexpr int kGroupWarps = kT5Threads / 32 / kSlots;
constexpr int kT5Vec = 32 / kSlots;            // vectors per tile
constexpr int kT5N = kT5Vec * 8;               // accumulator columns per tile
constexpr int kT5K = 256;          // hi and lo rows of the 128-row operand
// A = [H | H]: M = 128 x K = 256 bfloat16, K-major core matrices (8 rows of 16
// bytes along K), 8-K groups 128 bytes apart, 8-row groups 4096 bytes apart
constexpr uint32_t kALbo = 128;
constexpr uint32_t kASbo = 4096;
constexpr uint32_t kABytes = 128 * kT5K * 2;
// B = W: N x K = 256 bfloat16, MN-major core matrices (8 columns of 16 bytes
// along N), 8-column groups 128 bytes apart, 8-K groups N x 16 bytes apart
constexpr uint32_t kBGroupN = 128;
constexpr uint32_t kBGroupK = kT5N * 16;
constexpr uint32_t kBBytes = kT5N * kT5K * 2;
constexpr uint32_t kOffA = 0;
constexpr uint32_t kOffB = kOffA + kABytes;             // one operand buffer per slot
constexpr uint32_t kOffBar = kOffB + kSlots * kBBytes;  // mbarriers, tmem holder, fault flag
// per compute warp, the candidates of an output step: kList (value, id)
// pairs, then their lists (2 column + end)
constexpr int kList = 64;
constexpr uint32_t kListBytes = kList * 12;
constexpr uint32_t kOffList = kOffBar + 128;
constexpr uint32_t kSmem = kOffList + (kT5Threads / 32) * kListBytes;
constexpr int kTmemCols = 2 * kSlots * kT5N;  // accumulators, then staged inputs
// Instruction descriptor (kind::f16): D FP32 (bits 4-5 = 1), A and B
// bfloat16 (bits 7-9, 10-12 = 1), A K-major (bit 15 = 0), B MN-major (bit 16),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 16) | ((uint32_t)(kT5N >> 3) << 17) |
                            ((128u >> 4) << 24);
// a wait gives up after this many polls (each returns within a short,
// system-dependent time; together far beyond any product's latency)
constexpr int kWaitPolls = 1 << 24;
constexpr uint32_t kWaitHintNs = 20000;  // the fault path's waits: suspend hint

__device__ unsigned g_t5_faults = 0;
int g_t5_stall_polls = 0;  // test hook (project_t5_set_stall)

CEOS_DEV uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core-matrix groups along K) and stride-dimension byte
// offset (between groups along M / N), no swizzle, descriptor version 1.
CEOS_DEV uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

CEOS_DEV void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
        "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

CEOS_DEV void tmem_st32(uint32_t taddr, const float (&v)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]),
      "f"(v[9]), "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15]), "f"(v[16]),
      "f"(v[17]), "f"(v[18]), "f"(v[19]), "f"(v[20]), "f"(v[21]), "f"(v[22]), "f"(v[23]), "f"(v[24]),
      "f"(v[25]), "f"(v[26]), "f"(v[27]), "f"(v[28]), "f"(v[29]), "f"(v[30]), "f"(v[31])
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// (lo, hi) -> bfloat16x2 with lo in the low half, rounded to nearest even
CEOS_DEV uint32_t bf16x2(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

}  // namespace

// 17 warps: five of them share one of the SM's four 16,384-register
// partitions, so a thread has at most 96 registers.
// kStall (test hook, a separate instantiation so that the products' path is
// compiled without it): no products are issued, and every wait gives up
// after stall_polls polls.
template <int MODE, bool kStall>
__global__ void __launch_bounds__(kT5Threads + 32, 1) k_project_t5(ProjArgs a, int stall_polls) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int t = threadIdx.x, w = t >> 5, l = t & 31;
  const bool mma_warp = w == kT5Threads / 32;  // the last warp issues the products
  // compute warp w serves slot g = w / kGroupWarps; within its group it owns
  // lane quarter q of the tensor memory and vectors 8 ch .. 8 ch + 7
  const int g = (w / kGroupWarps) % kSlots;
  const int q = w & 3;
  const int ch = (w >> 2) % (kGroupWarps / 4);
  const int row = 32 * q + l;   // the row i of X (and lane of the accumulator)
  unsigned char* sA = sm + kOffA;
  // full[s]: slot s's operand is written (one arrival per compute warp);
  // done[s]: slot s's product has completed (tcgen05.commit)
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + kOffBar);
  uint64_t* done = full + kSlots;
  uint32_t* holder = reinterpret_cast<uint32_t*>(sm + kOffBar + 96);
  volatile int* fault_flag = reinterpret_cast<volatile int*>(sm + kOffBar + 100);
  const int R = a.R, D = a.D, C = a.R * a.D;

  // A = [H | H]: element (m, k) = (-1)^popc(m & (k mod 128))
  for (int e = t; e < 128 * kT5K / 8; e += blockDim.x) {
    const int m = e / (kT5K / 8), kg = e % (kT5K / 8);  // row, 8-K group
    uint32_t wv[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      uint32_t h2 = 0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = (kg * 8 + 2 * p + h) & 127;
        const uint32_t hv = (__popc(m & k) & 1) ? 0xBF80u : 0x3F80u;
        h2 |= hv << (16 * h);
      }
      wv[p] = h2;
    }
    *reinterpret_cast<uint4*>(sA + (m & 7) * 16 + (m >> 3) * kASbo + kg * kALbo) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
  }
  if (t == 0) {
    for (int s = 0; s < kSlots; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(full + s)), "r"(kGroupWarps) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(done + s)) : "memory");
    }
    *fault_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (mma_warp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(holder)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *holder;
  const long n_tiles = (a.n_rows + kT5Vec - 1) / kT5Vec;
  const int steps = 3 * R;

  // a bounded wait that also gives up once the other side has faulted (no
  // suspend hint: a product takes about a microsecond, and a suspended warp
  // wakes later than a polling one)
  const int wait_polls = kStall ? stall_polls : kWaitPolls;
  auto wait = [&](uint64_t* b, uint32_t parity) -> bool {
    for (int it = 0; it < wait_polls; ++it) {
      uint32_t ok;
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}\n"
          : "=r"(ok)
          : "r"(su32(b)), "r"(parity)
          : "memory");
      if (ok) return true;
      if (*fault_flag) return false;
    }
    *fault_flag = 1;
    return false;
  };

  if (mma_warp) {
    // ---- the product issuer: one elected lane ----
    uint32_t fph = 0u;  // bit s: phase of full[s]
    int issued[kSlots];  // commits per slot
#pragma unroll
    for (int s = 0; s < kSlots; ++s) issued[s] = 0;
    bool ok = !kStall;
    for (long t0 = (long)kSlots * blockIdx.x; t0 < n_tiles && ok; t0 += (long)kSlots * gridDim.x) {
      for (int st = 0; st < steps && ok; ++st) {
#pragma unroll
        for (int s = 0; s < kSlots; ++s) {
          if (!ok) break;
          ok = wait(full + s, (fph >> s) & 1u);
          ok = __all_sync(0xffffffffu, ok);
          if (!ok) break;
          fph ^= 1u << s;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          if (l == 0) {
            const uint32_t d = tmem + (uint32_t)(s * kT5N);
            const uint32_t b0 = su32(sm + kOffB + (uint32_t)s * kBBytes);
#pragma unroll
            for (int kk = 0; kk < kT5K / 16; ++kk) {
              const uint64_t da = smem_desc(su32(sA) + kk * 2 * kALbo, kALbo, kASbo);
              const uint64_t db = smem_desc(b0 + kk * 2 * kBGroupK, kBGroupK, kBGroupN);
              asm volatile(
                  "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
                  "l"(da), "l"(db), "r"(kIdesc), "r"(kk)
                  : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             su32(done + s))
                         : "memory");
          }
          __syncwarp();
          ++issued[s];
        }
      }
    }
    if (!ok) {
      // products still in flight finish (bounded) before the tensor memory
      // is released: wait for every commit of each slot
#pragma unroll
      for (int s = 0; s < kSlots; ++s) {
        if (issued[s] == 0) continue;
        const uint32_t last = (uint32_t)((issued[s] - 1) & 1);
        for (int it = 0; it < (1 << 16); ++it) {
          uint32_t r;
          asm volatile(
              "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
              "selp.u32 %0, 1, 0, p;\n\t}\n"
              : "=r"(r)
              : "r"(su32(done + s)), "r"(last), "r"(kWaitHintNs)
              : "memory");
          if (r) break;
        }
      }
    }
  } else {
    // ---- the compute warps: group g prepares slot g's operands ----
    // this thread's lane quarter and its 32 columns of chunk c (vectors
    // 8 ch + 4 c .. + 3) of the accumulator, and of the staged input rows
    auto my_tmem = [&](int c) { return tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(g * kT5N + 64 * ch + 32 * c); };
    auto my_input = [&](int c) { return my_tmem(c) + (uint32_t)(kSlots * kT5N); };
    uint32_t dph = 0u;

    // row pointer of vector v (0..15) of tile `tile`, null past n_rows
    auto vec_src = [&](long tile, int v, long& rid) -> const float* {
      const long r = tile * kT5Vec + v;
      rid = r;
      if (tile < 0 || r >= a.n_rows) return nullptr;
      long src = a.row_map ? a.row_map[r] : r;
      src += a.head;
      if (src >= a.cap_rows) src -= a.cap_rows;
      return a.X + src * a.ldx;
    };

    // The warp's candidate list (PROJ_EMIT): output steps append their
    // flagged values to it in shared memory, and flush() appends the list to
    // the global candidate lists, one entry per lane, so that a step waits for
    // one round of global atomics however its flagged values fall on lanes.
    float2* lval = reinterpret_cast<float2*>(sm + kOffList + (uint32_t)w * kListBytes);  // (v, id bits)
    uint32_t* lend = reinterpret_cast<uint32_t*>(lval + kList);
    int lcount = 0;  // entries in the list (the same in every lane)
    auto flush = [&]() {
      __syncwarp();
      for (int i = l; i < lcount; i += 32) {
        const uint32_t ce = lend[i];
        const float2 e = lval[i];
        const unsigned pos = atomicAdd(&a.cnt[ce], 1u);
        if (pos < (unsigned)a.cap)
          a.cand[(long)ce * a.cap + pos] = pack_key((ce & 1u) ? -e.x : e.x, __float_as_int(e.y));
      }
      __syncwarp();
      lcount = 0;
    };

    // outputs of repeat rr held in x (this thread's row of vectors v0 .. v0 + 3);
    // thb: the float bounds of the 8 output columns (PROJ_EMIT)
    auto output = [&](long tile, int v0, int rr, const float (&x)[32], const float2 (&thb)[8]) {
      const int idx0 = row * 8;  // output index of j = 0
      if constexpr (MODE == PROJ_EMIT) {
        // bit 8 vv + j: value j of vector v0 + vv passes the float prefilter
        uint32_t hit = 0;
#pragma unroll
        for (int e = 0; e < 32; ++e)
          if (emit_maybe(x[e], thb[e & 7])) hit |= 1u << e;
        // only output indices below D, and vectors below n_rows
        const int nj = min(8, max(0, D - idx0));
        const int nv = tile < 0 ? 0 : (int)min(4L, max(0L, a.n_rows - (tile * kT5Vec + v0)));
        const uint32_t jm = (1u << nj) - 1u;
        hit &= (jm | (jm << 8) | (jm << 16) | (jm << 24)) & (nv >= 4 ? 0xffffffffu : (1u << (8 * nv)) - 1u);
        // the few flagged values, one per lane and pass (the loop stays
        // rolled: every warp of the SM shares the instruction cache)
#pragma unroll 1
        while (__any_sync(0xffffffffu, hit != 0)) {
          bool close = false, far = false;
          int col = 0, id = 0;
          float v = 0.0f;
          if (hit != 0) {
            const int e = __ffs(hit) - 1;
            hit &= hit - 1u;
            const int j = e & 7;
            col = rr * D + idx0 + j;
            if (!(a.col_active && !a.col_active[col])) {
              v = x[0];
#pragma unroll
              for (int i = 1; i < 32; ++i)
                if (i == e) v = x[i];
              float2 bj = thb[0];
#pragma unroll
              for (int i = 1; i < 8; ++i)
                if (i == j) bj = thb[i];
              const long rid = tile * kT5Vec + v0 + (e >> 3);
              id = (int)(a.id_base + (a.row_map ? a.row_map[rid] : rid));
              // For a finite nonzero v the float bounds are exact (thb holds
              // the floats of the threshold keys, emit_bounds); zeros (-0 ranks
              // below +0) and infinities take the key test.
              if (v != 0.0f && isfinite(v)) {
                close = v >= bj.x;
                far = v <= bj.y;
              } else {
                const uint2 th = __ldg(reinterpret_cast<const uint2*>(a.th) + col);
                close = fkey(v) >= th.x;
                far = fkey(-v) >= th.y;
              }
            }
          }
          const uint32_t bc = __ballot_sync(0xffffffffu, close);
          const uint32_t bf = __ballot_sync(0xffffffffu, far);
          const int nnew = __popc(bc) + __popc(bf);
          if (lcount + nnew > kList) flush();
          const uint32_t below = (1u << l) - 1u;
          if (close) {
            const int p = lcount + __popc(bc & below);
            lval[p] = make_float2(v, __int_as_float(id));
            lend[p] = 2u * (uint32_t)col;
          }
          if (far) {
            const int p = lcount + __popc(bc) + __popc(bf & below);
            lval[p] = make_float2(v, __int_as_float(id));
            lend[p] = 2u * (uint32_t)col + 1u;
          }
          lcount += nnew;
        }
      } else {
#pragma unroll
        for (int vv = 0; vv < 4; ++vv) {
          long rid;
          if (vec_src(tile, v0 + vv, rid) == nullptr) continue;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int idx = idx0 + j;
            if (idx >= D) continue;
            const int col = rr * D + idx;
            if constexpr (MODE == PROJ_ROWS) {
              a.out[rid * (long)C + col] = x[8 * vv + j];
            } else {  // PROJ_COLS
              const int slot = a.col_slot ? a.col_slot[col] : col;
              if (slot >= 0) a.out[(long)slot * a.ld_out + rid] = x[8 * vv + j];
            }
          }
        }
      }
    };
    // the float bounds of repeat rr's 8 output columns of this thread's row
    auto bounds = [&](int rr, float2 (&thb)[8]) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int idx = row * 8 + j;
        thb[j] = (MODE == PROJ_EMIT && idx < D) ? __ldg(a.thf + rr * D + idx) : make_float2(0.f, 0.f);
      }
    };

    // this thread's input values of the group's tile (2 chunks x 4 vectors x
    // 8, zero past ldx and n_rows), staged in tensor memory for its repeats
    auto stage = [&](long tile) {
#pragma unroll 1
      for (int c = 0; c < 2; ++c) {
        float x[32];
        // (ldx is a multiple of 8, so a row's 8 values are all inside or all past it)
#pragma unroll
        for (int vv = 0; vv < 4; ++vv) {
          long rid;
          const float* src = vec_src(tile, 8 * ch + 4 * c + vv, rid);
          float4 u0 = make_float4(0.f, 0.f, 0.f, 0.f), u1 = u0;
          if (src != nullptr && row * 8 < a.ldx) {
            u0 = __ldg(reinterpret_cast<const float4*>(src + row * 8));
            u1 = __ldg(reinterpret_cast<const float4*>(src + row * 8 + 4));
          }
          x[8 * vv + 0] = u0.x;
          x[8 * vv + 1] = u0.y;
          x[8 * vv + 2] = u0.z;
          x[8 * vv + 3] = u0.w;
          x[8 * vv + 4] = u1.x;
          x[8 * vv + 5] = u1.y;
          x[8 * vv + 6] = u1.z;
          x[8 * vv + 7] = u1.w;
        }
        tmem_st32(my_input(c), x);
      }
    };

    // slot g's last product has completed
    auto ready = [&]() -> bool {
      const bool ok = __all_sync(0xffffffffu, wait(done + g, dph));
      if (!ok) return false;
      dph ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      return true;
    };

    // sign flip of round rnd of repeat rr, H_8, split and operand store of
    // chunk c (4 vectors) from x
    auto prepare = [&](int rr, int rnd, int c, const float (&x)[32]) {
      // signs of elements 8 i .. 8 i + 7 (bit set: +1)
      const uint32_t sw = __ldg(a.signs + (size_t)(rr * 3 + rnd) * 32 + (row >> 2)) >> ((row & 3) * 8);
      const float2 m1 = make_float2(-1.0f, -1.0f);
#pragma unroll
      for (int vv = 0; vv < 4; ++vv) {
        float y[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
          y[j] = __uint_as_float(__float_as_uint(x[8 * vv + j]) ^ ((~sw << (31 - j)) & 0x80000000u));
        // H_8 along the row (natural order). The three butterfly stages
        // commute; strides 4 and 2 run on packed pairs (u - v as fma(v, -1, u),
        // exactly rounded like a subtraction), stride 1 on scalars.
        const float2 a0 = make_float2(y[0], y[1]), a1 = make_float2(y[2], y[3]);
        const float2 b0 = make_float2(y[4], y[5]), b1 = make_float2(y[6], y[7]);
        const float2 s0 = __fadd2_rn(a0, b0), d0 = __ffma2_rn(b0, m1, a0);  // z0 z1 | z4 z5
        const float2 s1 = __fadd2_rn(a1, b1), d1 = __ffma2_rn(b1, m1, a1);  // z2 z3 | z6 z7
        const float2 t0 = __fadd2_rn(s0, s1), t1 = __ffma2_rn(s1, m1, s0);  // w0 w1 | w2 w3
        const float2 t2 = __fadd2_rn(d0, d1), t3 = __ffma2_rn(d1, m1, d0);  // w4 w5 | w6 w7
        const float2 w[4] = {t0, t1, t2, t3};
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          const float2 v2 = make_float2(w[p].x + w[p].y, w[p].x - w[p].y);
          hi[p] = bf16x2(v2.x, v2.y);
          const float2 h2 = make_float2(__uint_as_float(hi[p] << 16), __uint_as_float(hi[p] & 0xffff0000u));
          const float2 r2 = __ffma2_rn(h2, m1, v2);  // the remainders v - hi
          lo[p] = bf16x2(r2.x, r2.y);
        }
        // column n = 8 (8 ch + 4 c + vv) + j of K rows i (hi) and 128 + i (lo)
        unsigned char* pb = sm + kOffB + (uint32_t)g * kBBytes + (uint32_t)(8 * ch + 4 * c + vv) * kBGroupN +
                            (uint32_t)(row & 7) * 16 + (uint32_t)(row >> 3) * kBGroupK;
        *reinterpret_cast<uint4*>(pb) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(pb + 16 * kBGroupK) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
      }
    };

    bool ok = true;
    for (long t0 = (long)kSlots * blockIdx.x; t0 < n_tiles && ok; t0 += (long)kSlots * gridDim.x) {
      const long tile = t0 + g < n_tiles ? t0 + g : -1;
      stage(tile);
      for (int st = 0; st < steps && ok; ++st) {
        const int rr = st / 3, rnd = st % 3;
        float2 thb[8];
        if (st > 0) {
          if (rnd == 0) bounds(rr - 1, thb);  // in flight during the wait
          ok = ready();
          if (!ok) break;
        }
#pragma unroll 1
        for (int c = 0; c < 2; ++c) {
          float x[32];
          if (st > 0) {
            tmem_ld32(my_tmem(c), x);
            if (rnd == 0) output(tile, 8 * ch + 4 * c, rr - 1, x, thb);
          }
          if (rnd == 0) tmem_ld32(my_input(c), x);
          prepare(rr, rnd, c, x);
        }
        // the operand is visible to the tensor core, and this thread's reads
        // of the accumulator are complete, before the warp's arrival
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (l == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(full + g)) : "memory");
        // the step's candidates go out while the tensor core multiplies
        if (MODE == PROJ_EMIT && lcount > 0) flush();
      }
      if (ok) {
        float2 thb[8];
        bounds(R - 1, thb);
        ok = ready();
        if (ok) {
#pragma unroll 1
          for (int c = 0; c < 2; ++c) {
            float x[32];
            tmem_ld32(my_tmem(c), x);
            output(tile, 8 * ch + 4 * c, R - 1, x, thb);
          }
          if (MODE == PROJ_EMIT && lcount > 0) flush();
        }
      }
    }
    if (!ok) *fault_flag = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (mma_warp) {
    if (t == kT5Threads && *fault_flag) atomicAdd(&g_t5_faults, 1u);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

template <int MODE>
static cudaError_t launch_t5(const ProjArgs& a, int num_sms, cudaStream_t st) {
  const bool stall = g_t5_stall_polls > 0;
  auto kern = stall ? k_project_t5<MODE, true> : k_project_t5<MODE, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  if (e != cudaSuccess) return e;
  const long groups = (a.n_rows + kSlots * kT5Vec - 1) / (kSlots * kT5Vec);
  long blocks = num_sms;  // one CTA per SM (shared memory and tensor memory)
  if (blocks > groups) blocks = groups;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, kT5Threads + 32, kSmem, st>>>(a, g_t5_stall_polls);
  return cudaGetLastError();
}

cudaError_t launch_project_t5(const ProjArgs& a, int mode, cudaStream_t st, int num_sms) {
  if (a.n_rows <= 0) return cudaSuccess;
  switch (mode) {
    case PROJ_ROWS: return launch_t5<PROJ_ROWS>(a, num_sms, st);
    case PROJ_COLS: return launch_t5<PROJ_COLS>(a, num_sms, st);
    case PROJ_EMIT: return launch_t5<PROJ_EMIT>(a, num_sms, st);
  }
  return cudaErrorInvalidValue;
}

void project_t5_set_stall(int polls) { g_t5_stall_polls = polls; }

int project_t5_take_faults(cudaStream_t st) {
  unsigned h = 0, zero = 0;
  if (cudaMemcpyFromSymbolAsync(&h, g_t5_faults, sizeof(h), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  if (h) cudaMemcpyToSymbolAsync(g_t5_faults, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, st);
  return (int)h;
}

}  // namespace ceos
