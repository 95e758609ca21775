// Trailing-update GEMM of the blocked LU on the 5th-generation tensor cores.
//
//   C (FP32, column-major, ldc) -= A * B^T
//   A: M x K, B: N x K, both BF16 or FP16, K-major (row pitch K elements).
//
// One CTA computes a 128 x 256 tile.  K (the LU panel width, a multiple of
// 64) is staged in shared memory by TMA (cp.async.bulk.tensor, 128-byte
// swizzle, one mbarrier with an expected-transaction count); one elected
// thread issues tcgen05.mma (kind::f16, FP32 accumulation in tensor memory,
// M=128, N=256, K=16 per instruction) and commits to an mbarrier; four warps
// then read the accumulator with tcgen05.ld (32 lanes x 32 columns each),
// and apply C -= acc with coalesced column-major read-modify-writes.
//
// The reference factors with cuSOLVER Sgetrf in FP32/TF32 inside lu_ir.so
// (benchmark_mpdok.ipynb:982-993); here the O(N^3) work of the factorization
// runs as BF16/FP16 tensor-core tiles with FP32 accumulation.
//
// Every mbarrier wait is bounded: on time-out the CTA records an error word,
// skips its update, releases its tensor memory and returns.
#include "common.cuh"
#include "tc_gemm.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

namespace mpdok {

namespace tc {

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int BK = 64;           // elements per 128-byte swizzle row
constexpr int THREADS = 128;     // 4 warps: TMEM lane quarters 0..3
constexpr int TMEM_COLS = 256;   // FP32 accumulator columns
constexpr long long WAIT_LIMIT = 1LL << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 64) __nanosleep(32);
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// atoms 1024 bytes apart (stride byte offset), leading byte offset unused (1).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);       // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (ignored for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                        // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                        // swizzle mode: 128B
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, A/B BF16 (1) or FP16 (0),
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_f16(bool bf16, int m, int n) {
  return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared memory: STAGES x ([A 128x64][B 256x64]) ring, then barriers and the
// tensor-memory address slot.
template <int STAGES>
struct Smem {
  static constexpr int A_SUB = BM * BK * 2;   // 16 KB
  static constexpr int B_SUB = BN * BK * 2;   // 32 KB
  static constexpr int STAGE = A_SUB + B_SUB;
  static constexpr int BAR_OFF = STAGES * STAGE;
  static constexpr int TOTAL = BAR_OFF + 8 * (2 * STAGES + 1) + 16;
  static constexpr int ALLOC = TOTAL + 1024;  // slack for 1024-byte alignment
};

// K is consumed in 64-wide blocks through a STAGES-deep ring: lane 0 of warp 0
// is the TMA producer (waits on empty[s], arms full[s] with the stage's bytes),
// lane 0 of warp 1 issues the MMAs (waits on full[s], commits to empty[s]),
// and after the last block commits to done; all four warps then drain the
// accumulator.  The C loads of the epilogue start before the MMAs finish.
template <int STAGES>
__global__ void __launch_bounds__(THREADS, 1)
tc_gemm_update(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, float* C,
               long long ldc, int M, int N, int K, int bf16, int* err) {
  extern __shared__ uint8_t smem_raw[];
  using S = Smem<STAGES>;
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* gbase = smem_raw + (base - raw);
  const uint32_t bar_full = base + S::BAR_OFF;
  const uint32_t bar_empty = bar_full + 8 * STAGES;
  const uint32_t bar_done = bar_empty + 8 * STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + S::BAR_OFF + 8 * (2 * STAGES + 1));
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM;
  const int n0 = blockIdx.y * BN;
  const int KB = K / BK;

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int st = 0; st < STAGES; ++st) {
      mbar_init(bar_full + 8 * st, 1);
      mbar_init(bar_empty + 8 * st, 1);
    }
    mbar_init(bar_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0) {
    // TMA producer
    for (int kb = 0; kb < KB; ++kb) {
      const int st = kb % STAGES, round = kb / STAGES;
      if (round > 0 && !mbar_wait_bounded(bar_empty + 8 * st, (round - 1) & 1)) {
        atomicExch(&s_fail, 1);
        break;
      }
      const uint32_t sa = base + st * S::STAGE;
      mbar_expect_tx(bar_full + 8 * st, (uint32_t)S::STAGE);
      tma_load_2d(sa, &tmA, bar_full + 8 * st, kb * BK, m0);
      tma_load_2d(sa + S::A_SUB, &tmB, bar_full + 8 * st, kb * BK, n0);
    }
  } else if (threadIdx.x == 32) {
    // MMA issuer
    const uint32_t idesc = idesc_f16(bf16 != 0, BM, BN);
    bool ok = true;
    for (int kb = 0; kb < KB && ok; ++kb) {
      const int st = kb % STAGES, round = kb / STAGES;
      if (!mbar_wait_bounded(bar_full + 8 * st, round & 1)) {
        atomicExch(&s_fail, 2);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = base + st * S::STAGE;
#pragma unroll
      for (int k = 0; k < BK / 16; ++k) {
        // advance 16 elements (32 bytes) inside the 128-byte swizzle row
        const uint64_t ad = smem_desc_sw128(sa + k * 32);
        const uint64_t bd = smem_desc_sw128(sa + S::A_SUB + k * 32);
        mma_f16(tmem, ad, bd, idesc, (kb | k) ? 1u : 0u);
      }
      mma_commit(bar_empty + 8 * st);
    }
    if (ok) mma_commit(bar_done);
  }
  // The C tile does not depend on the MMA: load its first 32-column chunk
  // while the tensor cores run.  Loads of a chunk are issued back to back
  // (no interleaved stores), so the chunk costs one memory round trip.
  const int row = m0 + warp * 32 + lane;
  const bool row_ok = row < M;
  float* crow = C + (long long)row;
  float cur[32];
  auto load_chunk = [&](float (&dst)[32], int c0) {
    const int ncol = min(32, N - (n0 + c0));
#pragma unroll
    for (int c = 0; c < 32; ++c)
      dst[c] = (row_ok && c < ncol) ? __ldcg(crow + (long long)(n0 + c0 + c) * ldc) : 0.f;
  };
  // Two chunks are loaded ahead (64 loads in flight per thread): the
  // epilogue is a read-modify-write stream of the FP32 C tile and needs that
  // many bytes in flight per SM to cover the memory latency.
  float nxt[32];
  load_chunk(cur, 0);
  load_chunk(nxt, 32);
  __syncthreads();
  if (s_fail == 0) {
    if (!mbar_wait_bounded(bar_done, 0)) atomicExch(&s_fail, 3);
  }
  __syncthreads();
  if (s_fail == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      float nn[32];
      if (c0 + 64 < BN) load_chunk(nn, c0 + 64);
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (row_ok) {
        const int ncol = min(32, N - (n0 + c0));
#pragma unroll
        for (int c = 0; c < 32; ++c)
          if (c < ncol) __stcg(crow + (long long)(n0 + c0 + c) * ldc, cur[c] - v[c]);
      }
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        cur[c] = nxt[c];
        nxt[c] = nn[c];
      }
    }
  } else if (threadIdx.x == 0 && err) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// ------------------------------------------------------------------------
// Warp-specialised form for the LU's updates (K >= 128): one CTA per SM walks a
// strip of T tiles (128 x 256) that share their A rows, with
//   * a 4-stage TMA ring (48 KB per stage: the A and B blocks of one 64-deep
//     K step), so four loads are in flight while the tensor cores work;
//   * two TMEM accumulators (2 x 256 columns, all 512), so the MMAs of tile
//     t + 1 run while the epilogue drains tile t;
//   * warp 0 the TMA producer, warp 1 the MMA issuer, warps 2..9 the epilogue
//     (warp w reads TMEM lane quarter w % 4, column half (w - 2) / 4, and
//     applies C -= acc as coalesced column-major read-modify-writes with two
//     32-column chunks of C in flight).
// Barriers: full[s] / empty[s] for the ring, acc_full[a] (MMA -> epilogue,
// one commit) and acc_empty[a] (epilogue -> MMA, 8 warp arrivals).  Every
// wait is bounded and also gives up as soon as another role has failed; a
// failed CTA waits (bounded) for its own loads in flight before it releases
// its tensor memory and returns.
namespace ws {

constexpr int STAGES = 4;
constexpr int EPI_WARPS = 8;
constexpr int THREADS = 32 * (2 + EPI_WARPS);
constexpr int TMEM_COLS = 512;
constexpr int A_SUB = BM * BK * 2;   // 16 KB
constexpr int B_SUB = BN * BK * 2;   // 32 KB
constexpr int STAGE = A_SUB + B_SUB;
// epilogue staging: per epilogue warp two 16-column x 32-row FP32 buffers
// ([column][row], 2 KB each), drained into C by TMA reduce-add
constexpr int EPI_COLS = 16;
constexpr int EPI_BUF = 32 * EPI_COLS * 4;
constexpr int STAGING_OFF = STAGES * STAGE;
constexpr int BAR_OFF = STAGING_OFF + EPI_WARPS * 2 * EPI_BUF;
constexpr int NBAR = 2 * STAGES + 5;
constexpr int TOTAL = BAR_OFF + 8 * NBAR + 16;
constexpr int ALLOC = TOTAL + 1024;
static_assert(ALLOC <= 232448, "shared memory of one CTA");

__device__ __forceinline__ bool wait_or_fail(uint32_t bar, uint32_t parity, volatile int* fail) {
  for (long long i = 0; i < WAIT_LIMIT; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 63) {
      if (*fail) return false;
      __nanosleep(32);
    }
  }
  return false;
}

// C += (staged tile) by TMA: the L2 performs the read-modify-write, so the
// epilogue holds no C values and issues no C loads.  Coordinates: x = row
// (a multiple of 32 FP32 elements, 128 bytes), y = column.
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, uint32_t src, int x, int y) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%2, %3}], [%1];"
      ::"l"(reinterpret_cast<uint64_t>(map)), "r"(src), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// at most N bulk groups of this thread still reading shared memory
template <int N>
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait() { asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__global__ void __launch_bounds__(THREADS, 1)
tc_gemm_update_ws(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ CUtensorMap tmC, int M, int N, int K, int T, int bf16, int* err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* gbase = smem_raw + (base - raw);
  const uint32_t bar_full = base + BAR_OFF;
  const uint32_t bar_empty = bar_full + 8 * STAGES;
  const uint32_t bar_accf = bar_empty + 8 * STAGES;
  const uint32_t bar_acce = bar_accf + 16;
  const uint32_t bar_drain = bar_acce + 16;  // the MMA issuer's last commit: all its MMAs are done
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + BAR_OFF + 8 * NBAR);
  __shared__ int s_fail;
  volatile int* fail = &s_fail;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM;
  const int tile0 = blockIdx.y * T;
  const int ntiles_n = (N + BN - 1) / BN;
  const int nt = max(0, min(T, ntiles_n - tile0));
  const int KB = K / BK;

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int st = 0; st < STAGES; ++st) {
      mbar_init(bar_full + 8 * st, 1);
      mbar_init(bar_empty + 8 * st, 1);
    }
    mbar_init(bar_accf, 1);
    mbar_init(bar_accf + 8, 1);
    mbar_init(bar_acce, EPI_WARPS);
    mbar_init(bar_acce + 8, EPI_WARPS);
    mbar_init(bar_drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // TMA producer over every (tile, K block) of the strip
      int g = 0;
      bool ok = true;
      for (int t = 0; t < nt && ok; ++t) {
        const int n0 = (tile0 + t) * BN;
        for (int kb = 0; kb < KB; ++kb, ++g) {
          const int st = g % STAGES, round = g / STAGES;
          if (round > 0 && !wait_or_fail(bar_empty + 8 * st, (round - 1) & 1, fail)) {
            atomicExch(&s_fail, 1);
            ok = false;
            break;
          }
          const uint32_t sa = base + st * STAGE;
          mbar_expect_tx(bar_full + 8 * st, (uint32_t)STAGE);
          tma_load_2d(sa, &tmA, bar_full + 8 * st, kb * BK, m0);
          tma_load_2d(sa + A_SUB, &tmB, bar_full + 8 * st, kb * BK, n0);
        }
      }
      if (!ok || *fail) {
        // loads still in flight land in this CTA's shared memory: wait for
        // each stage's last issued load (bounded) before the CTA may exit
        for (int st = 0; st < STAGES && st < g; ++st) {
          const int last = g - 1 - ((g - 1 - st) % STAGES);
          const int round = last / STAGES;
          for (long long i = 0; i < WAIT_LIMIT && !mbar_try_wait(bar_full + 8 * st, round & 1); ++i) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_f16(bf16 != 0, BM, BN);
      int g = 0;
      bool ok = true;
      for (int t = 0; t < nt && ok; ++t) {
        const int a = t & 1, use = t >> 1;
        if (use > 0 && !wait_or_fail(bar_acce + 8 * a, (use - 1) & 1, fail)) {
          atomicExch(&s_fail, 2);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem + (uint32_t)(a * BN);
        for (int kb = 0; kb < KB; ++kb, ++g) {
          const int st = g % STAGES, round = g / STAGES;
          if (!wait_or_fail(bar_full + 8 * st, round & 1, fail)) {
            atomicExch(&s_fail, 3);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = base + st * STAGE;
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint64_t ad = smem_desc_sw128(sa + k * 32);
            const uint64_t bd = smem_desc_sw128(sa + A_SUB + k * 32);
            mma_f16(dacc, ad, bd, idesc, (kb | k) ? 1u : 0u);
          }
          mma_commit(bar_empty + 8 * st);
        }
        if (ok) mma_commit(bar_accf + 8 * a);
      }
      // before the tensor memory may be released, every MMA issued here must
      // have completed (also after a failure, when no epilogue waited for them)
      mma_commit(bar_drain);
      for (long long i = 0; i < WAIT_LIMIT && !mbar_try_wait(bar_drain, 0); ++i) {
        if (i > 64) __nanosleep(32);
      }
    }
  } else {
    // epilogue: TMEM lane quarter q = warp % 4 (rows m0 + 32 q + lane), column
    // half h.  Per 16-column chunk: tcgen05.ld, -acc into a staging buffer
    // ([column][row], conflict-free), then lane 0 adds it into C with one TMA
    // reduce; two buffers per warp alternate, so the next chunk is staged
    // while the last one drains.
    const int q = warp & 3, h = (warp - 2) >> 2;
    const int ew = warp - 2;
    float* stg = reinterpret_cast<float*>(gbase + STAGING_OFF + ew * 2 * EPI_BUF);
    const uint32_t stg_s = base + STAGING_OFF + ew * 2 * EPI_BUF;
    constexpr int HALF = BN / 2;
    constexpr int NCH = HALF / EPI_COLS;
    int nbuf = 0;
    for (int t = 0; t < nt; ++t) {
      const int a = t & 1, use = t >> 1;
      const int nbase = (tile0 + t) * BN + h * HALF;
      if (!wait_or_fail(bar_accf + 8 * a, use & 1, fail)) {
        atomicExch(&s_fail, 4);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tacc = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * BN + h * HALF);
#pragma unroll 1
      for (int i = 0; i < NCH; ++i) {
        // chunks past N hold nothing to add; skipping them keeps the two
        // staging buffers strictly alternating between issued reduces (a
        // skipped chunk must not overwrite a buffer whose reduce is pending)
        if (nbase + i * EPI_COLS >= N || m0 + q * 32 >= M) break;
        float v[EPI_COLS];
        tmem_ld16(tacc + (uint32_t)(i * EPI_COLS), v);
        const int b = nbuf & 1;
        ++nbuf;
        if (lane == 0) bulk_wait_read<1>();  // the buffer's previous reduce has read it
        __syncwarp();
        float* buf = stg + b * (EPI_BUF / 4);
#pragma unroll
        for (int c = 0; c < EPI_COLS; ++c) buf[c * 32 + lane] = -v[c];
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          tma_reduce_add_2d(&tmC, stg_s + b * EPI_BUF, m0 + q * 32, nbase + i * EPI_COLS);
          bulk_commit();
        }
      }
      // this warp has read its part of accumulator a: hand it back to the MMA
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(bar_acce + 8 * a);
    }
    if (lane == 0) bulk_wait<0>();  // every reduce of this warp has completed
    __syncwarp();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0 && s_fail != 0 && err) atomicExch(err, 1);
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

}  // namespace ws

// CUDA-core comparator with the same operand rounding (test use).
__global__ void simt_gemm_update(const void* A, const void* B, long long ldk, int bf16, float* C, long long ldc,
                                 int M, int N, int K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= M || j >= N) return;
  float acc = 0.f;
  for (int k = 0; k < K; ++k) {
    float a, b;
    if (bf16) {
      a = __bfloat162float(((const __nv_bfloat16*)A)[(long long)i * ldk + k]);
      b = __bfloat162float(((const __nv_bfloat16*)B)[(long long)j * ldk + k]);
    } else {
      a = __half2float(((const __half*)A)[(long long)i * ldk + k]);
      b = __half2float(((const __half*)B)[(long long)j * ldk + k]);
    }
    acc = fmaf(a, b, acc);
  }
  C[i + (long long)j * ldc] -= acc;
}

}  // namespace tc

static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2-D tensor map over a K-major 16-bit operand (rows x K, row pitch ldk elements), box 64 x box_rows.
static int make_map(CUtensorMap* map, const void* ptr, int rows, int K, long long ldk, int box_rows, bool bf16) {
  auto enc = get_encode();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled unavailable from the driver");
    return MPDOK_ERR_UNSUPPORTED;
  }
  cuuint64_t gdim[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)ldk * 2};
  cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                   const_cast<void*>(ptr), gdim, gstride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MPDOK_ERR_CUDA;
  }
  return MPDOK_OK;
}

// 2-D tensor map over the FP32 C (rows x columns, column-major, ldc), box 32
// rows x 16 columns: the target of the epilogue's TMA reduce-adds.
static int make_map_c(CUtensorMap* map, float* C, int M, int N, long long ldc) {
  auto enc = get_encode();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled unavailable from the driver");
    return MPDOK_ERR_UNSUPPORTED;
  }
  cuuint64_t gdim[2] = {(cuuint64_t)M, (cuuint64_t)N};
  cuuint64_t gstride[1] = {(cuuint64_t)ldc * 4};
  cuuint32_t box[2] = {32, (cuuint32_t)tc::ws::EPI_COLS};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, gdim, gstride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled (C) failed (%d)", (int)r);
    return MPDOK_ERR_CUDA;
  }
  return MPDOK_OK;
}

constexpr int TC_STAGES = 2;

// Tiles per CTA of the warp-specialised kernel along N (the strip shares A,
// and the epilogue of one tile overlaps the MMAs of the next).  Two, not
// more: a CTA of the far update then holds its SM for about 25 us at K = 2048,
// so the panel kernels of the other streams find SMs sooner (the 16-bit
// factorization at N=32768: 45.5 ms with four tiles, 45.0 ms with two, 46.0
// ms with one).
constexpr int WS_TILES = 2;
// K from which the warp-specialised kernel is used: every update of the LU
// (K = 128 inside the super-panel) takes it, since its TMA reduce-add epilogue
// keeps C out of registers (the 16-bit factorization at N=32768: 44.1 ms with
// the K = 128 updates on the two-CTA-per-SM kernel, 43.2 ms on this one); the
// other kernel remains for K = 64.
constexpr int WS_MIN_K = 128;

// Streaming multiprocessors of the current device (cached per host thread and
// device).
static int sm_count() {
  constexpr int MAX_DEV = 64;
  thread_local int cnt[MAX_DEV] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) return 1;
  if (cnt[dev] == 0 && cudaDeviceGetAttribute(&cnt[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return cnt[dev];
}

static int launch_tc(const CUtensorMap& ma, const CUtensorMap& mb, float* C, long long ldc, int M, int N, int K,
                     int bf16, int* err, cudaStream_t s) {
  if (K >= WS_MIN_K && aligned16(C) && ldc % 4 == 0) {
    CUtensorMap mc;
    MPDOK_TRY(make_map_c(&mc, C, M, N, ldc));
    MPDOK_TRY(set_smem(tc::ws::tc_gemm_update_ws, tc::ws::ALLOC));
    const int ntm = (M + tc::BM - 1) / tc::BM;
    const int ntn = (N + tc::BN - 1) / tc::BN;
    // fewer tiles per CTA while the strips would not fill the GPU once (the
    // 128-row block updates of the left-looking panels)
    int T = WS_TILES;
    while (T > 1 && (long long)ntm * ((ntn + T - 1) / T) < sm_count()) T >>= 1;
    dim3 grid(ntm, (ntn + T - 1) / T);
    tc::ws::tc_gemm_update_ws<<<grid, tc::ws::THREADS, tc::ws::ALLOC, s>>>(ma, mb, mc, M, N, K, T, bf16, err);
    count_launch();
    MPDOK_LAUNCH_CHECK("tc_gemm_update_ws");
    return MPDOK_OK;
  }
  using S = tc::Smem<TC_STAGES>;
  MPDOK_TRY(set_smem(tc::tc_gemm_update<TC_STAGES>, S::ALLOC));
  dim3 grid((M + tc::BM - 1) / tc::BM, (N + tc::BN - 1) / tc::BN);
  tc::tc_gemm_update<TC_STAGES><<<grid, tc::THREADS, S::ALLOC, s>>>(ma, mb, C, ldc, M, N, K, bf16, err);
  count_launch();
  MPDOK_LAUNCH_CHECK("tc_gemm_update");
  return MPDOK_OK;
}

int gemm_update(float* C, long long ldc, const void* A, const void* B, long long ldk, int M, int N, int K, int fdtype,
                int engine, int* err, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(fdtype == MPDOK_BF16 || fdtype == MPDOK_F16, "factor dtype must be BF16 or FP16");
  MPDOK_ARG_CHECK(ldc >= M, "ldc < M");
  MPDOK_ARG_CHECK(ldk >= K, "operand pitch < K");
  const int bf16 = fdtype == MPDOK_BF16 ? 1 : 0;
  const bool deep = engine != MPDOK_ENGINE_SIMT && K >= WS_MIN_K && aligned16(C) && ldc % 4 == 0;
  const int slot = prof_start(deep ? MPDOK_PROF_LU_GEMM_DEEP : MPDOK_PROF_LU_GEMM, s);
  if (engine == MPDOK_ENGINE_SIMT) {
    dim3 grid((M + 127) / 128, N);
    launch(tc::simt_gemm_update, grid, 128, 0, s, A, B, ldk, bf16, C, ldc, M, N, K);
    MPDOK_LAUNCH_CHECK("simt_gemm_update");
  } else {
    MPDOK_ARG_CHECK(K % tc::BK == 0, "tensor-core update needs K to be a multiple of 64");
    MPDOK_ARG_CHECK(aligned16(A) && aligned16(B) && (ldk * 2) % 16 == 0, "operands must be 16-byte aligned");
    CUtensorMap ma, mb;
    MPDOK_TRY(make_map(&ma, A, M, K, ldk, tc::BM, bf16));
    MPDOK_TRY(make_map(&mb, B, N, K, ldk, tc::BN, bf16));
    MPDOK_TRY(launch_tc(ma, mb, C, ldc, M, N, K, bf16, err, s));
  }
  prof_stop(slot, s, 2.0 * (double)M * (double)N * (double)K);
  // C read and written in FP32, both 16-bit operands read once
  prof_stop_bytes(slot, 8.0 * (double)M * (double)N + 2.0 * (double)K * ((double)M + (double)N));
  return MPDOK_OK;
}

}  // namespace mpdok

using namespace mpdok;

extern "C" int mpdok_gemm_update(float* C, long long ldc, const void* A, const void* B, int M, int N, int K,
                                 int fdtype, int engine, int* err, cudaStream_t stream) {
  MPDOK_ARG_CHECK(M >= 0 && N >= 0 && K >= 0, "negative size");
  if (M == 0 || N == 0 || K == 0) return MPDOK_OK;
  MPDOK_ARG_CHECK(C && A && B, "null pointer");
  return gemm_update(C, ldc, A, B, K, M, N, K, fdtype, engine, err, stream);
}
