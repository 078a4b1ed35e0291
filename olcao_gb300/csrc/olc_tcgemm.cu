// Blackwell tensor-core GEMM for the complex products of the mixed solver:
// tcgen05.mma issued by one thread, BF16 operands staged by TMA
// (cp.async.bulk.tensor) into 128-byte-swizzled shared memory through a
// four-stage mbarrier pipeline, FP32 accumulators in tensor memory (TMEM)
// drained by eight epilogue warps with tcgen05.ld.
//
// Complex products as one real GEMM.  For C = op(A) B (A: m x k, B: k x n
// complex) the kernel computes the real product D = A' B'^T with
//   A'(r, :)     = [ Re op(A)(r, 0..k) | Im op(A)(r, 0..k) ]            (K' = 2 kp)
//   B'^T(2c, :)   = [ Re B(0..k, c)     | -Im B(0..k, c) ]
//   B'^T(2c+1, :) = [ Im B(0..k, c)     |  Re B(0..k, c) ]
// so that D(r, 2c) = Re C(r, c) and D(r, 2c+1) = Im C(r, c): every epilogue
// thread owns one row and writes interleaved complex results.  Both operands
// are K-major (K contiguous), the layout tcgen05 reads without transposition.
//
// Operands are "planes" of BF16 values: digit planes of a fixed-point split
// or the three BF16 pieces of an FP32 number.  A launch runs a list of
// segments (plane of A, plane of B, K-block range):
//
//  * fixed mode (FP64-accurate products): every row of op(A) and column of B
//    is scaled by a power of two and cut into signed 8-bit digits
//    (|d| <= 255: BF16 holds every integer up to 256 exactly).  One segment is
//    one digit pair (s, t) over at most 256 of K', so that its FP32 sum of at
//    most 256 * 255^2 < 2^24
//    is an exact integer.  Segments alternate between two TMEM accumulators;
//    the epilogue drains each one (tcgen05.ld, exact float -> int) into
//    64-bit fixed point, acc += g << shift(s + t), while the tensor cores fill
//    the other.  Digit pairs whose weight is below the kept precision are not
//    issued.  The result is acc scaled by 2^(e_row + f_col + base): FP64
//    complex, no intermediate in global memory.
//  * f32 mode (FP32-accurate products): x = x0 + x1 + x2 (three BF16 pieces
//    of an FP32 value, 24 bits); the six pairs with weight >= 2^-16
//    accumulate in one FP32 TMEM accumulator; C = alpha D + beta C.
//
// GPU safety: every mbarrier wait is bounded by wall time (%globaltimer);
// on expiry the thread records an error code, the other roles see it and
// stop, the producer waits (bounded) for its copies in flight and the
// allocating warp frees TMEM before the CTA exits.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "olc_common.h"
#include "olc_tcgemm.h"

namespace olc {
namespace tc {

namespace {

constexpr int BM = 128;            // rows per tile (TMEM lanes)
constexpr int BK = 64;             // K per stage: 64 BF16 = one 128-byte swizzle row
constexpr int STAGES = 4;
constexpr int NUM_EPI_WARPS = 8;
constexpr int NUM_THREADS = (NUM_EPI_WARPS + 2) * 32;
constexpr int PRODUCER_WARP = NUM_EPI_WARPS;
constexpr int MMA_WARP = NUM_EPI_WARPS + 1;
// two accumulators of BN columns: 256 (fixed mode) or 512 (f32 mode)
template <int MODE>
constexpr int tmem_cols() { return MODE == 0 ? 256 : 512; }
constexpr long long kWaitNs = 2000000000LL;   // 2 s per wait
// fixed mode: K' per drained segment, the largest multiple of BK with
// kChunkK (2^kBeta - 1)^2 < 2^24 (every FP32 partial sum an exact integer)
constexpr int kChunkK = (int)((16777215LL / (((1LL << kBeta) - 1) * ((1LL << kBeta) - 1))) / BK * BK);
static_assert(kChunkK >= BK, "digit width too large for exact FP32 segments");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of `parity`; false when the wait expired or
// another role of the CTA gave up (error word set).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* cta_err,
                                          int* gerr, int code) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  for (;;) {
    if (mbar_try(bar, parity)) return true;
    if (*cta_err) return false;
    if ((long long)(now_ns() - t0) > kWaitNs) {
      *cta_err = code;
      atomicExch(gerr, code);
      return false;
    }
  }
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of
// 1024 bytes (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// Instruction descriptor of kind::f16: BF16 A and B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void umma(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// 16 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t ta, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(ta));
}
// 32 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t ta, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
        "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(ta));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Tile of a CTA: grouped raster (GM row tiles at a time) so that the CTAs in
// flight share operand panels in L2.
__device__ __forceinline__ void tile_of(int t, int nmt, int nnt, int& mt, int& nt) {
  constexpr int GM = 8;
  const int per_group = GM * nnt;
  const int g = t / per_group, first = g * GM;
  const int gsize = min(GM, nmt - first);
  const int r = t % per_group;
  mt = first + r % gsize;
  nt = r / gsize;
}

struct SmemLayout {
  static constexpr int a_bytes = BM * BK * 2;
  template <int BN>
  static constexpr int b_bytes() { return BN * BK * 2; }
  template <int BN>
  static constexpr int bars_offset() { return STAGES * (a_bytes + b_bytes<BN>()); }
  template <int BN>
  static constexpr int total() { return bars_offset<BN>() + 256 + 1024; }   // barriers + alignment slack
};

}  // namespace

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
// MODE 0 (fixed): BN = 128, two accumulators of 128 columns, int64 drains,
//   FP64 complex output.  Epilogue warp w owns TMEM lanes 32 (w % 4) .. +31
//   and columns 64 (w / 4) .. +63 of the tile (32 complex columns).
// MODE 1 (f32):   BN = 256, one accumulator, FP32 complex output with
//   alpha, beta; warp w owns columns 128 (w / 4) .. +127 (64 complex).
template <int MODE>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const __grid_constant__ TcParams p) {
  constexpr int BN = MODE == 0 ? 128 : 256;
  constexpr uint32_t IDESC = idesc_bf16(BM, BN);
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * SmemLayout::a_bytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + SmemLayout::bars_offset<BN>());
  uint64_t* full = bars;                 // [STAGES] TMA -> MMA
  uint64_t* empty = bars + STAGES;       // [STAGES] MMA -> TMA
  uint64_t* accfull = bars + 2 * STAGES; // [2] MMA -> epilogue
  uint64_t* accempty = accfull + 2;      // [2] epilogue -> MMA
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accempty + 2);
  volatile int* cta_err = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.y;
  int mt, nt;
  tile_of(blockIdx.x, p.nmt, p.nnt, mt, nt);
  const int m0 = mt * BM, n0 = nt * BN;     // n0: first real column of D
  // Hermitian result: a tile whose complex columns all lie left of its first
  // row is wholly below the diagonal (filled afterwards from the upper part)
  if (p.herm_upper && (n0 >> 1) + BN / 2 - 1 < m0) return;
  // lower part wanted: a tile whose complex columns all lie right of its last
  // row is wholly above the diagonal
  if (p.lower_only && (n0 >> 1) > m0 + BM - 1) return;
  // segments: every pair over K chunks of chunk_blocks K-blocks
  const int nchunk = (p.kblocks + p.chunk_blocks - 1) / p.chunk_blocks;
  const int nseg = p.npairs * nchunk;
  // triangular operands (f32 mode): the complex K range [kmin, kmax) this
  // tile needs; a K-block is issued when it meets that range in the real or
  // the imaginary half of K' (every role skips the same blocks and segments)
  int kmin = 0, kmax = p.kp;
  if (p.tri_a_upper) kmin = m0;
  if (p.tri_a_lower) kmax = min(kmax, m0 + BM);
  if (p.tri_b_upper) kmax = min(kmax, (n0 >> 1) + BN / 2);
  const bool tri = kmin > 0 || kmax < p.kp;
  auto kb_needed = [&](int kb) {
    if (!tri) return true;
    const int lo = kb * BK, hi = lo + BK;
    return (lo < kmax && hi > kmin) || (lo < p.kp + kmax && hi > p.kp + kmin);
  };
  auto seg_live = [&](int si) {
    if (!tri) return true;
    const int kb0 = (si % nchunk) * p.chunk_blocks, kb1 = min(p.kblocks, kb0 + p.chunk_blocks);
    for (int kb = kb0; kb < kb1; ++kb)
      if (kb_needed(kb)) return true;
    return false;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&accfull[s], 1);
      mbar_init(&accempty[s], NUM_EPI_WARPS);
    }
    *cta_err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(tmem_cols<MODE>()));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == PRODUCER_WARP) {
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(&tmA) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(&tmB) : "memory");
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0;   // stages filled (bounds the copies still in flight on the error path)
      bool ok = true;
      for (int si = 0; si < nseg && ok; ++si) {
        const TcPair pr = p.pairs[si / nchunk];
        const int kb0 = (si % nchunk) * p.chunk_blocks, kb1 = min(p.kblocks, kb0 + p.chunk_blocks);
        for (int kb = kb0; kb < kb1; ++kb) {
          if (!kb_needed(kb)) continue;
          if (!mbar_wait(&empty[stage], phase ^ 1u, cta_err, p.err, 1)) { ok = false; break; }
          mbar_expect_tx(&full[stage], (uint32_t)(SmemLayout::a_bytes + SmemLayout::b_bytes<BN>()));
          tma_load_3d(sA + stage * SmemLayout::a_bytes, &tmA, &full[stage], kb * BK, m0, b * p.planes_a + pr.pa);
          tma_load_3d(sB + stage * SmemLayout::b_bytes<BN>(), &tmB, &full[stage], kb * BK, n0,
                      b * p.planes_b + pr.pb);
          ++issued;
          if (++stage == STAGES) { stage = 0; phase ^= 1u; }
        }
      }
      if (!ok) {
        // wait (bounded) for the copies still in flight before the CTA exits
        int st = stage;
        uint32_t ph = phase;
        for (int q = 0; q < STAGES && q < issued; ++q) {
          if (--st < 0) { st = STAGES - 1; ph ^= 1u; }
          const unsigned long long t0 = now_ns();
          while (!mbar_try(&full[st], ph) && (long long)(now_ns() - t0) < kWaitNs) {
          }
        }
      }
    }
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      int ls = 0;   // live segments so far (the accumulator ring follows them)
      for (int si = 0; si < nseg && ok; ++si) {
        if (!seg_live(si)) continue;
        const int kb0 = (si % nchunk) * p.chunk_blocks, kb1 = min(p.kblocks, kb0 + p.chunk_blocks);
        const int buf = ls & 1;
        {
          const uint32_t use = (uint32_t)(ls >> 1);
          if (!mbar_wait(&accempty[buf], (use & 1u) ^ 1u, cta_err, p.err, 2)) { ok = false; break; }
          tc_fence_after();
        }
        ++ls;
        const uint32_t dt = tmem + (uint32_t)(buf * BN);
        bool fresh = true;   // the segment's first issued block overwrites the accumulator
        for (int kb = kb0; kb < kb1; ++kb) {
          if (!kb_needed(kb)) continue;
          if (!mbar_wait(&full[stage], phase, cta_err, p.err, 3)) { ok = false; break; }
          tc_fence_after();
          const uint64_t ad = sdesc(smem_u32(sA + stage * SmemLayout::a_bytes));
          const uint64_t bd = sdesc(smem_u32(sB + stage * SmemLayout::b_bytes<BN>()));
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const bool first = fresh && k == 0;
            // +32 bytes of K per instruction: +2 in the descriptor's address field
            umma(dt, ad + 2 * k, bd + 2 * k, IDESC, first ? 0u : 1u);
          }
          umma_commit(&empty[stage]);
          fresh = false;
          if (++stage == STAGES) { stage = 0; phase ^= 1u; }
        }
        if (ok) umma_commit(&accfull[buf]);
      }
    }
  } else {
    // ---------------- epilogue warps ----------------
    const int q = warp & 3, h = warp >> 2;
    const int row = m0 + 32 * q + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
    if (MODE == 0) {
      long long acc[64];
#pragma unroll
      for (int j = 0; j < 64; ++j) acc[j] = 0;
      bool ok = true;
      int ls = 0;
      for (int si = 0; si < nseg; ++si) {
        if (!seg_live(si)) continue;
        const int buf = ls & 1;
        const uint32_t use = (uint32_t)(ls >> 1);
        ++ls;
        ok = __all_sync(0xffffffffu, mbar_wait(&accfull[buf], use & 1u, cta_err, p.err, 4));
        if (!ok) break;
        tc_fence_after();
        const int sh = p.pairs[si / nchunk].shift;
#pragma unroll
        for (int part = 0; part < 4; ++part) {
          uint32_t r[16];
          tmem_ld16(lane_addr + (uint32_t)(buf * BN + 64 * h + 16 * part), r);
          tmem_ld_wait();
          if (part == 3) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&accempty[buf]);
          }
          if (sh >= 0) {
#pragma unroll
            for (int j = 0; j < 16; ++j)
              acc[16 * part + j] += (long long)__float2int_rn(__uint_as_float(r[j])) << sh;
          } else {
            // low-order digit groups: rounded to the accumulator's unit (a
            // plain arithmetic shift would floor, a bias of half a unit per
            // drain that adds up over long K)
            const long long half = 1LL << (-sh - 1);
#pragma unroll
            for (int j = 0; j < 16; ++j)
              acc[16 * part + j] += ((long long)__float2int_rn(__uint_as_float(r[j])) + half) >> (-sh);
          }
        }
      }
      if (ok && row < p.m) {
        const int er = p.ea[(size_t)b * p.m + row] + p.base;
        const int c0 = (n0 >> 1) + 32 * h;     // first complex column of this warp
        double2* out = reinterpret_cast<double2*>(p.c64) + (size_t)b * p.stride_c;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int c = c0 + j;
          if (c < p.ncols) {
            const int e = er + p.fb[(size_t)b * p.ncols + c];
            out[(size_t)c * p.ldc + row] =
                make_double2(scalbn(__ll2double_rn(acc[2 * j]), e), scalbn(__ll2double_rn(acc[2 * j + 1]), e));
          }
        }
      }
    } else {
      // FP32 mode: every segment (one piece pair over at most 512 of K') is
      // drained into register accumulators with round-to-nearest adds, so
      // that long sums of like-signed terms are not left to the tensor
      // core's accumulator alone
      float acc[128];
#pragma unroll
      for (int j = 0; j < 128; ++j) acc[j] = 0.f;
      bool ok = true;
      int ls = 0;
      for (int si = 0; si < nseg; ++si) {
        if (!seg_live(si)) continue;
        const int buf = ls & 1;
        const uint32_t use = (uint32_t)(ls >> 1);
        ++ls;
        ok = __all_sync(0xffffffffu, mbar_wait(&accfull[buf], use & 1u, cta_err, p.err, 4));
        if (!ok) break;
        tc_fence_after();
#pragma unroll
        for (int part = 0; part < 8; ++part) {
          uint32_t r[16];
          tmem_ld16(lane_addr + (uint32_t)(buf * BN + 128 * h + 16 * part), r);
          tmem_ld_wait();
          if (part == 7) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&accempty[buf]);
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) acc[16 * part + j] += __uint_as_float(r[j]);
        }
      }
      if (ok && row < p.m) {
        float2* out = reinterpret_cast<float2*>(p.c32) + (size_t)b * p.stride_c;
        const int cbase = (n0 >> 1) + 64 * h;
#pragma unroll
        for (int j = 0; j < 64; ++j) {
          const int c = cbase + j;
          if (c < p.ncols) {
            float2 v = make_float2(p.alpha * acc[2 * j], p.alpha * acc[2 * j + 1]);
            float2* o = out + (size_t)c * p.ldc + row;
            if (p.beta != 0.f) {
              const float2 old = *o;
              v.x += p.beta * old.x;
              v.y += p.beta * old.y;
            }
            *o = v;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == MMA_WARP) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols<MODE>()));
  }
}

// ---------------------------------------------------------------------------
// operand preparation
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ int expo_field(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }
__device__ __forceinline__ int expo_field(float x) { return (int)((__float_as_uint(x) >> 23) & 0xff); }
// smallest e with |x| < 2^e over a maximum exponent field E (normal numbers)
__device__ __forceinline__ int bound_expo(double, int E) { return E ? E - 1022 : -100000; }
__device__ __forceinline__ int bound_expo(float, int E) { return E ? E - 126 : -100000; }

// trunc(|x| 2^(W - e)) for |x| < 2^e, W <= 62; subnormals count as zero
__device__ __forceinline__ unsigned long long fixed_bits(double x, int e, int W) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
  const int E = (int)(u >> 52);
  if (E == 0) return 0ULL;
  const unsigned long long mant = (u & 0xfffffffffffffULL) | (1ULL << 52);
  const int sh = E - 1075 + W - e;
  if (sh >= 0) return mant << sh;
  if (sh <= -64) return 0ULL;
  return mant >> (-sh);
}
__device__ __forceinline__ unsigned long long fixed_bits(float x, int e, int W) {
  const unsigned u = __float_as_uint(x) & 0x7fffffffu;
  const int E = (int)(u >> 23);
  if (E == 0) return 0ULL;
  const unsigned long long mant = (unsigned long long)((u & 0x7fffffu) | (1u << 23));
  const int sh = E - 150 + W - e;
  if (sh >= 0) return mant << sh;
  if (sh <= -64) return 0ULL;
  return mant >> (-sh);
}

// Exponents of the lines (rows of op(A) or columns of B) that lie contiguous
// in the source: warp per line.
template <class T>
__global__ void line_expo_kernel(const T* __restrict__ src, long long sstride, int ld, int len, int lines, int nb,
                                 int* __restrict__ expo) {
  const size_t gw = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= (size_t)lines * nb) return;
  const int b = (int)(gw / lines), line = (int)(gw % lines);
  const T* s = src + (size_t)b * sstride + 2 * (size_t)line * ld;
  int E = 0;
  for (int i = lane; i < 2 * len; i += 32) E = max(E, expo_field(s[i]));
  for (int o = 16; o; o >>= 1) E = max(E, __shfl_xor_sync(0xffffffffu, E, o));
  if (lane == 0) expo[gw] = bound_expo(T(0), E);
}

// Exponents of the rows of a column-major source (thread per row).
template <class T>
__global__ void row_expo_kernel(const T* __restrict__ src, long long sstride, int ld, int rows, int cols, int nb,
                                int* __restrict__ expo) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)rows * nb) return;
  const int b = (int)(t / rows), r = (int)(t % rows);
  const T* s = src + (size_t)b * sstride;
  int E = 0;
  for (int c = 0; c < cols; ++c) {
    E = max(E, expo_field(s[2 * ((size_t)c * ld + r)]));
    E = max(E, expo_field(s[2 * ((size_t)c * ld + r) + 1]));
  }
  expo[t] = bound_expo(T(0), E);
}

// Value of plane `pl` of x: digit pl of the fixed-point split (beta bits,
// W = nplanes * beta) or BF16 piece pl of an FP32 value.
template <class T>
__device__ __forceinline__ float plane_value(T x, int e, int beta, int W, int pl, bool digits) {
  if (digits) {
    const unsigned long long N = fixed_bits(x, e, W);
    const int d = (int)((N >> (W - beta * (pl + 1))) & ((1ULL << beta) - 1ULL));
    return x < T(0) ? -(float)d : (float)d;
  }
  float r = (float)x;
  float v = 0.f;
  for (int i = 0; i <= pl; ++i) {
    v = __bfloat162float(__float2bfloat16_rn(r));
    r -= v;
  }
  return v;
}

// Left operand planes: out[b][pl][r][Kp] with columns [0, k) = Re op(A)(r, .),
// [kp, kp + k) = Im op(A)(r, .), zero elsewhere (Kp = 2 kp).  op(A) = src or
// src^H; 32 x 32 tiles through shared memory so that reads and writes
// coalesce in both cases.
template <class T>
__global__ void __launch_bounds__(256) slice_a_kernel(const T* __restrict__ src, long long sstride, int ld, bool conj,
                                                      int m, int k, int kp, const int* __restrict__ ea,
                                                      int nplanes, int beta, bool digits,
                                                      __nv_bfloat16* __restrict__ out) {
  __shared__ T tre[32][33], tim[32][33];
  const int b = blockIdx.z;
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;   // rows of op(A), K columns
  const int tx = threadIdx.x, ty = threadIdx.y;
  const T* s = src + (size_t)b * sstride;
  for (int j = ty; j < 32; j += 8) {
    // tre[r][c] = op(A)(r0 + r, c0 + c)
    if (!conj) {
      const int r = r0 + tx, c = c0 + j;
      T vr = T(0), vi = T(0);
      if (r < m && c < k) {
        vr = s[2 * ((size_t)c * ld + r)];
        vi = s[2 * ((size_t)c * ld + r) + 1];
      }
      tre[tx][j] = vr;
      tim[tx][j] = vi;
    } else {
      const int c = c0 + tx, r = r0 + j;
      T vr = T(0), vi = T(0);
      if (r < m && c < k) {
        vr = s[2 * ((size_t)r * ld + c)];
        vi = -s[2 * ((size_t)r * ld + c) + 1];
      }
      tre[j][tx] = vr;
      tim[j][tx] = vi;
    }
  }
  __syncthreads();
  const int W = nplanes * beta;
  const size_t Kp = 2 * (size_t)kp;
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + j, c = c0 + tx;
    if (r >= m || c >= kp) continue;
    const T xr = tre[j][tx], xi = tim[j][tx];
    const int e = digits ? ea[(size_t)b * m + r] : 0;
    for (int pl = 0; pl < nplanes; ++pl) {
      __nv_bfloat16* o = out + (((size_t)b * nplanes + pl) * m + r) * Kp;
      o[c] = __float2bfloat16_rn(c < k ? plane_value(xr, e, beta, W, pl, digits) : 0.f);
      o[kp + c] = __float2bfloat16_rn(c < k ? plane_value(xi, e, beta, W, pl, digits) : 0.f);
    }
  }
}

// Right operand planes: out[b][pl][2c + (0|1)][Kp]: row 2c = [Re B(., c) | -Im B(., c)],
// row 2c+1 = [Im B(., c) | Re B(., c)]; thread per (column, K index).
template <class T>
__global__ void slice_b_kernel(const T* __restrict__ src, long long sstride, int ld, int k, int n, int kp,
                               const int* __restrict__ fb, int nplanes, int beta, bool digits, int nb,
                               __nv_bfloat16* __restrict__ out) {
  const size_t per = (size_t)kp * n, total = per * nb;
  const int W = nplanes * beta;
  const size_t Kp = 2 * (size_t)kp;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(idx / per);
    const size_t q = idx % per;
    const int r = (int)(q % kp), c = (int)(q / kp);
    const T* s = src + (size_t)b * sstride;
    T xr = T(0), xi = T(0);
    if (r < k) {
      xr = s[2 * ((size_t)c * ld + r)];
      xi = s[2 * ((size_t)c * ld + r) + 1];
    }
    const int e = digits ? fb[(size_t)b * n + c] : 0;
    for (int pl = 0; pl < nplanes; ++pl) {
      const float vr = r < k ? plane_value(xr, e, beta, W, pl, digits) : 0.f;
      const float vi = r < k ? plane_value(xi, e, beta, W, pl, digits) : 0.f;
      __nv_bfloat16* o = out + (((size_t)b * nplanes + pl) * 2 * n + 2 * (size_t)c) * Kp;
      o[r] = __float2bfloat16_rn(vr);
      o[kp + r] = __float2bfloat16_rn(-vi);
      o[Kp + r] = __float2bfloat16_rn(vi);
      o[Kp + kp + r] = __float2bfloat16_rn(vr);
    }
  }
}

int grid_of(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

// C(r, c) = conj(C(c, r)) for r > c: the strict lower triangle of a
// Hermitian batch [nb][n][n] (complex FP64, column-major) from its upper one.
__global__ void mirror_lower_kernel(double2* __restrict__ C, int n, int nb) {
  __shared__ double2 tile[32][33];
  const int b = blockIdx.z;
  const int bx = blockIdx.x, by = blockIdx.y;   // tile (rows by, columns bx) of the lower part
  if (bx > by) return;
  double2* Cb = C + (size_t)b * n * n;
  const int tx = threadIdx.x, ty = threadIdx.y;
  // read the upper tile (rows bx, columns by), write its conjugate transpose
  for (int j = ty; j < 32; j += 8) {
    const int r = bx * 32 + tx, c = by * 32 + j;
    if (r < n && c < n) tile[j][tx] = Cb[(size_t)c * n + r];
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int r = by * 32 + tx, c = bx * 32 + j;     // lower element (r, c) = conj(upper (c, r))
    if (r < n && c < n && r > c) {
      const double2 u = tile[tx][j];
      Cb[(size_t)c * n + r] = make_double2(u.x, -u.y);
    }
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  });
  return fn;
}

// 3-D BF16 tensor [planes][rows][Kp] (K contiguous), box 64 x box_rows x 1,
// 128-byte swizzle; rows past `rows` read as zero.
int make_map(CUtensorMap* map, const void* base, size_t Kp, size_t rows, size_t planes, int box_rows) {
  EncodeFn fn = encode_fn();
  if (!fn) return fail(OLC_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (Kp * 2) % 16)
    return fail(OLC_ERR_CUDA, "tensor map operand not 16-byte aligned");
  const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)planes};
  const cuuint64_t strides[2] = {(cuuint64_t)(Kp * 2), (cuuint64_t)(Kp * 2 * rows)};
  const cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(OLC_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return OLC_OK;
}

int* g_err = nullptr;   // device error word shared by the launches of this process
std::mutex g_err_mu;

int launch(olc_context* ctx, int mode, const void* dA, const void* dB, int planes_a, int planes_b, size_t Kp,
           int m, int nreal, int nb, TcParams p, int stage) {
  cudaStream_t st = ctx->stream;
  int s;
  {
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (!g_err) {
      if ((s = cuda_check(cudaMalloc(&g_err, sizeof(int)), "tc error word"))) return s;
      if ((s = cuda_check(cudaMemset(g_err, 0, sizeof(int)), "tc error word"))) return s;
    }
  }
  const int BN = mode == 0 ? 128 : 256;
  CUtensorMap ta, tb;
  if ((s = make_map(&ta, dA, Kp, (size_t)m, (size_t)planes_a * nb, BM))) return s;
  if ((s = make_map(&tb, dB, Kp, (size_t)nreal, (size_t)planes_b * nb, BN))) return s;
  p.planes_a = planes_a;
  p.planes_b = planes_b;
  p.nmt = (m + BM - 1) / BM;
  p.nnt = (nreal + BN - 1) / BN;
  p.kblocks = (int)(Kp / BK);
  p.kp = (int)(Kp / 2);
  p.err = g_err;
  const dim3 grid((unsigned)(p.nmt * p.nnt), (unsigned)nb);
  if (mode == 0) {
    const int smem = SmemLayout::total<128>();
    if ((s = cuda_check(cudaFuncSetAttribute(tc_gemm_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                        "tc smem")))
      return s;
    tc_gemm_kernel<0><<<grid, NUM_THREADS, smem, st>>>(ta, tb, p);
  } else {
    const int smem = SmemLayout::total<256>();
    if ((s = cuda_check(cudaFuncSetAttribute(tc_gemm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                        "tc smem")))
      return s;
    tc_gemm_kernel<1><<<grid, NUM_THREADS, smem, st>>>(ta, tb, p);
  }
  count_launch();
  double frac = 1.0;
  if (p.herm_upper || p.lower_only) {
    long long done = 0;
    for (int mt = 0; mt < p.nmt; ++mt)
      for (int nt = 0; nt < p.nnt; ++nt)
        done += p.herm_upper ? ((nt * BN) / 2 + BN / 2 - 1 >= mt * BM) : ((nt * BN) / 2 <= mt * BM + BM - 1);
    frac = (double)done / ((double)p.nmt * p.nnt);
  }
  add_work(ctx, stage, 2.0 * m * (double)nreal * (double)Kp * p.npairs * nb * frac, 0.0);
  return cuda_check(cudaGetLastError(), "tc_gemm launch");
}

}  // namespace

// Kept-digit plan of a fixed-point product: beta = 7, na / nb digits of A / B,
// pairs (s, t) with s + t <= T kept, T the smallest with the dropped part
// below 2^-(prec + 2) of the scale product.
void fixed_plan(int bits_a, int bits_b, int prec, int* na, int* nbd, int* T) {
  *na = (bits_a + kBeta - 1) / kBeta;
  *nbd = (bits_b + kBeta - 1) / kBeta;
  // dropped pairs with s + t >= T + 1 weigh at most ~4 * 2^(-beta (T + 1))
  int t = 0;
  while (kBeta * (t + 1) - 2 < prec + 2) ++t;
  *T = std::min(t, *na + *nbd - 2);
}

int read_error(int* code) {
  *code = 0;
  if (!g_err) return OLC_OK;
  int s = cuda_check(cudaMemcpy(code, g_err, sizeof(int), cudaMemcpyDeviceToHost), "tc error read");
  if (!s && *code) cudaMemset(g_err, 0, sizeof(int));
  return s;
}

template <class TA, class TB>
int zgemm_fixed(olc_context* ctx, int m, int n, int k, const TA* A, long long sA, int lda, bool conjA, int bits_a,
                const TB* B, long long sB, int ldb, int bits_b, double* C, int nb, int stage, bool hermitian) {
  if (hermitian && m != n) return fail(OLC_ERR_ARG, "hermitian product must be square");
  cudaStream_t st = ctx->stream;
  int na, nbd, T;
  // the product is wanted to the precision of the wider operand (the
  // narrower one is represented exactly or as a consistent basis change)
  fixed_plan(bits_a, bits_b, std::max(bits_a, bits_b), &na, &nbd, &T);
  const int kp = (k + 31) & ~31;
  const size_t Kp = 2 * (size_t)kp;
  // FP32-exact segments: at most kChunkK of K' per drain
  std::vector<TcPair> pairs;
  for (int d = 0; d <= T; ++d)
    for (int s = 0; s < na; ++s) {
      const int t = d - s;
      if (t >= 0 && t < nbd) pairs.push_back(TcPair{(int8_t)s, (int8_t)t, 0});
    }
  if ((int)pairs.size() > kMaxPairs) return fail(OLC_ERR_UNSUPPORTED, "fixed-point product: too many digit pairs");
  // 64-bit fixed point: unit 2^(L - beta (T + 2)) of the scale product
  const double mag = kBeta * T + 2 * kBeta + std::log2(1.03 * (double)Kp);
  const int L = std::max(0, (int)std::ceil(mag - 62.0));
  for (auto& pr : pairs) pr.shift = (int16_t)(kBeta * (T - pr.pa - pr.pb) - L);
  // batch chunk: digit planes below ~8 GB
  const size_t per_b = 2 * Kp * ((size_t)na * m + (size_t)nbd * 2 * n);
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>(nb, (8ULL << 30) / std::max<size_t>(per_b, 1)));
  __nv_bfloat16 *wa = nullptr, *wb = nullptr;
  int *ea = nullptr, *fb = nullptr;
  int s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&wa, 2 * Kp * na * (size_t)m * chunk, st), "malloc digits A")))
    return s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&wb, 2 * Kp * nbd * 2 * (size_t)n * chunk, st), "malloc digits B")))
    return s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&ea, 4ULL * chunk * m, st), "malloc ea"))) return s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&fb, 4ULL * chunk * n, st), "malloc fb"))) return s;
  StageScope scope(ctx, stage, 0);
  for (int b0 = 0; b0 < nb; b0 += chunk) {
    const int cb = std::min(chunk, nb - b0);
    const TA* Ab = A + (size_t)b0 * sA;
    const TB* Bb = B + (size_t)b0 * sB;
    if (conjA)
      line_expo_kernel<TA><<<(int)(((size_t)m * cb * 32 + 255) / 256), 256, 0, st>>>(Ab, sA, lda, k, m, cb, ea);
    else
      row_expo_kernel<TA><<<(int)(((size_t)m * cb + 255) / 256), 256, 0, st>>>(Ab, sA, lda, m, k, cb, ea);
    line_expo_kernel<TB><<<(int)(((size_t)n * cb * 32 + 255) / 256), 256, 0, st>>>(Bb, sB, ldb, k, n, cb, fb);
    slice_a_kernel<TA><<<dim3((m + 31) / 32, (kp + 31) / 32, cb), dim3(32, 8), 0, st>>>(
        Ab, sA, lda, conjA, m, k, kp, ea, na, kBeta, true, wa);
    slice_b_kernel<TB><<<grid_of((size_t)kp * n * cb), 256, 0, st>>>(Bb, sB, ldb, k, n, kp, fb, nbd, kBeta, true,
                                                                     cb, wb);
    scope.add_launches(5);
    TcParams p{};
    p.m = m;
    p.ncols = n;
    p.ldc = m;
    p.stride_c = (long long)m * n;
    p.c64 = C + 2 * (size_t)b0 * m * n;
    p.ea = ea;
    p.fb = fb;
    p.base = L - kBeta * (T + 2);
    p.npairs = (int)pairs.size();
    for (size_t i = 0; i < pairs.size(); ++i) p.pairs[i] = pairs[i];
    p.chunk_blocks = kChunkK / BK;
    p.herm_upper = hermitian ? 1 : 0;
    if ((s = launch(ctx, 0, wa, wb, na, nbd, Kp, m, 2 * n, cb, p, stage))) return s;
    if (hermitian) {
      StageScope ms(ctx, stage, 1);
      mirror_lower_kernel<<<dim3((n + 31) / 32, (n + 31) / 32, cb), dim3(32, 8), 0, st>>>(
          reinterpret_cast<double2*>(C + 2 * (size_t)b0 * m * n), n, cb);
    }
  }
  cudaFreeAsync(wa, st);
  cudaFreeAsync(wb, st);
  cudaFreeAsync(ea, st);
  cudaFreeAsync(fb, st);
  return cuda_check(cudaGetLastError(), "fixed-point tensor-core product");
}

int cgemm_f32(olc_context* ctx, int m, int n, int k, const float* A, long long sA, int lda, bool conjA,
              const float* B, long long sB, int ldb, float alpha, float beta, float* C, long long sC, int ldc,
              int nb, int stage, bool lower, int tri) {
  cudaStream_t st = ctx->stream;
  const int kp = (k + 31) & ~31;
  const size_t Kp = 2 * (size_t)kp;
  // piece pairs by weight: the six down to 2^-16, and with OLC_F32_PAIRS=9 the
  // three of weight 2^-24 and below as well
  static const int8_t pairs[9][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}, {0, 2}, {2, 0}, {1, 2}, {2, 1}, {2, 2}};
  int npairs = 6;
  if (const char* v = std::getenv("OLC_F32_PAIRS")) npairs = std::atoi(v) == 9 ? 9 : 6;
  const size_t per_b = 2 * Kp * 3 * ((size_t)m + 2 * (size_t)n);
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>(nb, (8ULL << 30) / std::max<size_t>(per_b, 1)));
  __nv_bfloat16 *wa = nullptr, *wb = nullptr;
  int s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&wa, 2 * Kp * 3 * (size_t)m * chunk, st), "malloc pieces A")))
    return s;
  if ((s = cuda_check(ctx_malloc(ctx, (void**)&wb, 2 * Kp * 3 * 2 * (size_t)n * chunk, st), "malloc pieces B")))
    return s;
  StageScope scope(ctx, stage, 0);
  for (int b0 = 0; b0 < nb; b0 += chunk) {
    const int cb = std::min(chunk, nb - b0);
    const float* Ab = A + (size_t)b0 * sA;
    const float* Bb = B + (size_t)b0 * sB;
    slice_a_kernel<float><<<dim3((m + 31) / 32, (kp + 31) / 32, cb), dim3(32, 8), 0, st>>>(
        Ab, sA, lda, conjA, m, k, kp, nullptr, 3, 0, false, wa);
    slice_b_kernel<float><<<grid_of((size_t)kp * n * cb), 256, 0, st>>>(Bb, sB, ldb, k, n, kp, nullptr, 3, 0, false,
                                                                        cb, wb);
    scope.add_launches(2);
    TcParams p{};
    p.m = m;
    p.ncols = n;
    p.ldc = ldc;
    p.stride_c = sC / 2;
    p.c32 = C + (size_t)b0 * sC;
    p.alpha = alpha;
    p.beta = beta;
    p.npairs = npairs;
    for (int i = 0; i < npairs; ++i) p.pairs[i] = TcPair{pairs[i][0], pairs[i][1], 0};
    p.chunk_blocks = 512 / BK;
    p.lower_only = lower ? 1 : 0;
    p.tri_a_upper = (tri & kTriAUpper) != 0;
    p.tri_a_lower = (tri & kTriALower) != 0;
    p.tri_b_upper = (tri & kTriBUpper) != 0;
    if ((s = launch(ctx, 1, wa, wb, 3, 3, Kp, m, 2 * n, cb, p, stage))) return s;
  }
  cudaFreeAsync(wa, st);
  cudaFreeAsync(wb, st);
  return cuda_check(cudaGetLastError(), "FP32-accurate tensor-core product");
}

template int zgemm_fixed<double, float>(olc_context*, int, int, int, const double*, long long, int, bool, int,
                                        const float*, long long, int, int, double*, int, int, bool);
template int zgemm_fixed<float, double>(olc_context*, int, int, int, const float*, long long, int, bool, int,
                                        const double*, long long, int, int, double*, int, int, bool);
template int zgemm_fixed<double, double>(olc_context*, int, int, int, const double*, long long, int, bool, int,
                                         const double*, long long, int, int, double*, int, int, bool);

}  // namespace tc
}  // namespace olc
