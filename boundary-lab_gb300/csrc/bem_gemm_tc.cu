// Tensor-core (tcgen05) trailing update of the complex LU: C -= L21 * U12.
//
// The complex product is run as one real GEMM.  With complex entries stored
// interleaved (re, im), a column of C or U12 is already a real column of twice
// the length, and
//     C' (2M x N) -= A' (2M x 2K) * B' (2K x N)
// where B' is U12's memory read as reals and A' replaces every complex L21
// entry a by the 2 x 2 real block [[re a, -im a], [im a, re a]].
//
// Precision: 3xFP16 with power-of-two scaling (the split-precision tensor-core
// product of Markidis et al., "NVIDIA Tensor Core Programmability, Performance
// & Precision", 2018).  Every operand value x is scaled by a power of two s and
// split as x s = hi + lo, hi = fp16(x s) and lo = fp16(x s - hi); the MMA sums
// hi*hi + hi*lo + lo*hi with FP32 accumulation and the epilogue multiplies by
// 1 / (s_A s_B), exactly.  hi and lo carry 11 significant bits each, like a
// TF32 split, so a product keeps about 2^-22 relative error, while the f16 MMA
// runs at twice the TF32 rate on half the operand bytes.  The scales keep the
// values inside FP16's range: L21 holds the multipliers of partial pivoting,
// |re|, |im| <= 1, scaled by s_A = 2^14; each column j of U12 is scaled by
// s_j = 2^(14 - e_j), e_j the binary exponent of its largest |re| or |im|, so
// its entries lie below 2^14 and an entry loses its lo part to the FP16
// subnormal range only when it is 2^17 below its column's largest (a 2^-28
// normwise error).
//
// Kernel: persistent, one CTA per SM, tiles of 128 x 256 of C'.  A prep kernel
// writes A'hi, A'lo, B'hi, B'lo as K-major (K contiguous) FP16 buffers and the
// column scales; a producer warp brings 32-wide K blocks by TMA into
// 64-byte-swizzled shared memory through a 4-stage mbarrier pipeline; one
// thread issues tcgen05.mma (kind::f16, M=128, N=256, K=16) into one of two
// TMEM accumulators; four epilogue warps read the other accumulator back with
// tcgen05.ld, stage -D / (s_A s_j) in shared memory 32 columns at a time
// (double buffered per warp) and TMA reduce-add it into C
// (cp.reduce.async.bulk.tensor .add.f32), so C is never
// read by the SM: the read-modify-write happens in L2, asynchronously, while
// the next tile's MMAs run.  Every wait is bounded: on timeout the kernel
// records an error, waits (bounded) for its own copies and MMAs, frees its
// TMEM and returns.
//
// General block update (tc_update): C[row0:row0+M, col0:col0+N] -= L U with
// L = A[row0:, kcol0:kcol0+K] and U = A[kcol0:kcol0+K, col0:], K <= 256, so one
// kernel serves the trailing update, the updates inside a wide panel and the
// blocked triangular solve of its U rows.
//
// TMA coordinates into C: the C map spans every whole matrix of the batch
// (x = real row 0..2n, y = column 0..n, z = matrix), so a tile starts at
// x = 2 row0 + m0 + 32 w.  The innermost coordinate times 4 bytes must be a
// multiple of 16: row0 is even (checked; block widths are even, the plan
// refuses odd nb) and m0 + 32 w is a multiple of 32.  All coordinates are >= 0;
// rows x >= 2n and columns y >= n are clipped by the map bounds, and rows or
// columns of a tile beyond M or N receive -0 from zero-padded operands.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "bem_common.cuh"
#include "bem_kernels.h"

namespace bem {
namespace {

constexpr int TM = 128;       // tile rows of C' (real rows)
constexpr int TN = 256;       // tile columns of C'
constexpr int TK = 32;        // K block per stage (32 fp16 = 64 B rows, 64-byte swizzle)
constexpr int KP_MAX = 512;   // K' = 2 K <= 512 (K <= 256 complex), row stride of the split operands
constexpr int A_BYTES = TM * TK * 2;   // 8 KB
constexpr int B_BYTES = TN * TK * 2;   // 16 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // hi + lo of A and B: 48 KB
constexpr float kAScale = 16384.0f;      // s_A = 2^14 (multipliers have |re|, |im| <= 1)
constexpr int kBTarget = 14;             // column j of U12 scaled so its largest |re|, |im| is below 2^14
// mbarrier waits give up after kWaitLimit polls with a 1 us suspend hint each
// (about one second), far above any healthy wait (microseconds).
constexpr long long kWaitLimit = 1LL << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase), "r"(1000)
      : "memory");
  return ok != 0;
}
// Bounded wait; returns false (and records it) when the limit is hit.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, int* err, int code) {
  for (long long i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  atomicCAS(err, 0, code);
  return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 64-byte swizzle, rows of
// 64 B packed in 512-byte groups of 8 (SBO = 512 B).
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);        // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;               // stride byte offset
  d |= (uint64_t)1 << 46;                        // descriptor version
  d |= (uint64_t)4 << 61;                        // 64-byte swizzle
  return d;
}

// Instruction descriptor: kind::f16, D = F32, A = B = F16 (format 0 for both:
// the two operands of one MMA always have the same type), both K-major,
// M = 128, N = 256.
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          dtmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld_32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%"
      "20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// -D tile of one warp (32 real rows x 32 columns, rows contiguous) added into C by TMA.
__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap* map, const void* src, int x, int y, int z) {
  asm volatile("cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                   (uint64_t)map),
               "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// x (already scaled) as hi + lo in FP16, both rounded to nearest.
__device__ __forceinline__ void split_f16(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(x - __half2float(hi));
}

// Both operand splits of one update in one launch.  Blocks [0, nta) split A:
// each takes 32 rows x 16 columns of L21 (complex), loaded along the rows
// (coalesced, through shared memory), scales them by s_A and writes the
// 64 x 32 real-embedded hi / lo tile with the K index fastest (16-byte
// stores).  The remaining blocks split B, one warp per column of U12: the
// warp finds the column's largest |re| or |im|, writes the column scaled by
// s_j = 2^(14 - e) as hi / lo (K fastest on both sides) and 1 / (s_A s_j) to
// inv_scale.  Entries beyond M rows / N columns / K depth are written as zero.
__global__ void __launch_bounds__(256) prep_ab_kernel(const float2* __restrict__ A, long long lda, long long strideA,
                                                      int row0, int col0, int kcol0, int M, int N, int K, int rows_pad,
                                                      int cols_pad, int rows_used, int cols_used, int kp, int nta,
                                                      __half* __restrict__ ahi, __half* __restrict__ alo,
                                                      __half* __restrict__ bhi, __half* __restrict__ blo,
                                                      float* __restrict__ inv_scale) {
  const int b = blockIdx.y;
  const float2* Ab = A + (size_t)b * strideA;
  const int t = threadIdx.x;
  if ((int)blockIdx.x < nta) {
    __shared__ float2 tile[16][33];
    const int tiles_k = kp / 32;
    const int ti = blockIdx.x / tiles_k, tk = blockIdx.x - ti * tiles_k;
    const int i0 = ti * 32, k0 = tk * 16;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = t & 31, k = (t >> 5) + 8 * h;
      float2 a = make_float2(0.f, 0.f);
      if (i0 + i < M && k0 + k < K) a = Ab[(size_t)(kcol0 + k0 + k) * lda + row0 + i0 + i];
      tile[k][i] = make_float2(a.x * kAScale, a.y * kAScale);
    }
    __syncthreads();
    const int rr = t >> 2, q = t & 3;  // embedded row 2 i + e, complex k 4q .. 4q + 3
    const int i = rr >> 1, e = rr & 1;
    __align__(16) __half hi[8], lo[8];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float2 a = tile[4 * q + c][i];
      // row 2i: (re, -im) per k; row 2i + 1: (im, re)
      split_f16(e == 0 ? a.x : a.y, hi[2 * c], lo[2 * c]);
      split_f16(e == 0 ? -a.y : a.x, hi[2 * c + 1], lo[2 * c + 1]);
    }
    const size_t o = ((size_t)b * rows_pad + 2 * i0 + rr) * KP_MAX + 2 * k0 + 8 * q;
    *reinterpret_cast<uint4*>(ahi + o) = *reinterpret_cast<const uint4*>(hi);
    *reinterpret_cast<uint4*>(alo + o) = *reinterpret_cast<const uint4*>(lo);
    return;
  }
  const int lane = t & 31;
  const int j = (int)(blockIdx.x - nta) * 8 + (t >> 5);  // column of U12 (one warp each)
  if (j >= cols_used) return;
  constexpr int KL = KP_MAX / 64;  // complex K entries per lane
  const int kc = kp / 2;           // complex K entries written per column (<= KP_MAX / 2)
  float2 u[KL];
  float amax = 0.0f;
#pragma unroll
  for (int c = 0; c < KL; ++c) {
    const int k = lane + 32 * c;
    u[c] = make_float2(0.f, 0.f);
    if (j < N && k < K) u[c] = Ab[(size_t)(col0 + j) * lda + kcol0 + k];
    amax = fmaxf(amax, fmaxf(fabsf(u[c].x), fabsf(u[c].y)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  int e = 0;
  frexpf(amax, &e);  // amax = m 2^e, 0.5 <= m < 1 (e = 0 for zero)
  const int sh = min(100, max(-114, kBTarget - e));  // s_j = 2^sh, 1 / (s_A s_j) stays a normal float
  const float s = ldexpf(1.0f, sh);
  if (lane == 0) inv_scale[(size_t)b * cols_pad + j] = ldexpf(1.0f, -sh - 14);
#pragma unroll
  for (int c = 0; c < KL; ++c) {
    const int k = lane + 32 * c;
    if (k >= kc) break;
    __align__(4) __half hi[2], lo[2];
    split_f16(u[c].x * s, hi[0], lo[0]);
    split_f16(u[c].y * s, hi[1], lo[1]);
    const size_t o = ((size_t)b * cols_pad + j) * KP_MAX + 2 * k;
    *reinterpret_cast<__half2*>(bhi + o) = *reinterpret_cast<const __half2*>(hi);
    *reinterpret_cast<__half2*>(blo + o) = *reinterpret_cast<const __half2*>(lo);
  }
}

// One CTA per SM walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ... (rows
// of C' fastest, then columns, then matrices).  Warp 0 is the TMA producer,
// warp 1 issues the MMAs, warps 2-9 are the epilogue.  Operands flow through a
// 4-stage pipeline (192 KB) and the accumulator is double-buffered in TMEM
// (2 x 256 columns), so the epilogue of one tile runs while the MMAs of the
// next tile proceed.  A warp reads only its own TMEM lane quarter (warp % 4),
// so epilogue warp w handles rows 32 (w % 4) of a tile, in the even or the odd
// 32-column chunks ((w - 2) / 4): with K = 32 (the updates inside an outer
// block) a tile's MMAs take less time than its epilogue, and two warps per
// quarter halve that.  (The one-tile-per-CTA kernel with two CTAs per SM that
// this replaced was 2-3% slower on the LU.)
constexpr int P_STAGES = 4;
constexpr int P_EPI_WARPS = 8;
constexpr int P_THREADS = 64 + 32 * P_EPI_WARPS;
constexpr int P_TMEM_COLS = 2 * TN;
constexpr size_t P_STAGE_AREA = (size_t)P_STAGES * STAGE_BYTES;  // 192 KB
constexpr size_t P_EPI_BYTES = (size_t)P_EPI_WARPS * 4096;        // one 4 KB buffer per epilogue warp
constexpr size_t P_SMEM = P_STAGE_AREA + P_EPI_BYTES + 1024;

__global__ void __launch_bounds__(P_THREADS, 1)
    trailing_update_f16x3_persistent(const __grid_constant__ CUtensorMap map_ahi,
                                     const __grid_constant__ CUtensorMap map_alo,
                                     const __grid_constant__ CUtensorMap map_bhi,
                                     const __grid_constant__ CUtensorMap map_blo,
                                     const __grid_constant__ CUtensorMap map_c, const float* __restrict__ inv_scale,
                                     int cols_pad, int x0, int y0, int M2, int N, int KB, int tiles_m, int tiles_n,
                                     int n_tiles, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[P_STAGES];
  __shared__ __align__(8) uint64_t empty_bar[P_STAGES];
  __shared__ __align__(8) uint64_t acc_full[2];
  __shared__ __align__(8) uint64_t acc_empty[2];
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int s_fail;
  __shared__ int s_consumed;  // K blocks the MMA warp has taken from the pipeline

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < P_STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], P_EPI_WARPS);
    }
    mbar_init(&done_bar, 1);
    s_fail = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(P_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const int per_matrix = tiles_m * tiles_n;
  int issued = 0;  // producer: K blocks whose loads were started

  if (warp == 0 && lane == 0) {
    // TMA producer
    int it = 0;
    for (int t = blockIdx.x; t < n_tiles && !s_fail; t += gridDim.x) {
      const int bz = t / per_matrix, rem = t - bz * per_matrix;
      const int m0 = (rem % tiles_m) * TM, n0 = (rem / tiles_m) * TN;
      for (int kb = 0; kb < KB; ++kb, ++it) {
        const int s = it % P_STAGES;
        if (it >= P_STAGES && !mbar_wait(&empty_bar[s], ((it / P_STAGES) - 1) & 1, err, 1)) {
          s_fail = 1;
          break;
        }
        unsigned char* st = base + (size_t)s * STAGE_BYTES;
        mbar_expect_tx(&full_bar[s], STAGE_BYTES);
        tma_load_3d(st, &map_ahi, &full_bar[s], kb * TK, m0, bz);
        tma_load_3d(st + A_BYTES, &map_alo, &full_bar[s], kb * TK, m0, bz);
        tma_load_3d(st + 2 * A_BYTES, &map_bhi, &full_bar[s], kb * TK, n0, bz);
        tma_load_3d(st + 2 * A_BYTES + B_BYTES, &map_blo, &full_bar[s], kb * TK, n0, bz);
        issued = it + 1;
      }
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    int it = 0, local = 0;
    for (int t = blockIdx.x; t < n_tiles && !s_fail; t += gridDim.x, ++local) {
      const int buf = local & 1;
      if (local >= 2 && !mbar_wait(&acc_empty[buf], ((local >> 1) - 1) & 1, err, 5)) {
        s_fail = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acc_addr = tmem + (uint32_t)(buf * TN);
      bool ok = true;
      for (int kb = 0; kb < KB; ++kb, ++it) {
        const int s = it % P_STAGES;
        if (!mbar_wait(&full_bar[s], (it / P_STAGES) & 1, err, 2)) {
          ok = false;
          break;
        }
        s_consumed = it + 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        unsigned char* st = base + (size_t)s * STAGE_BYTES;
        const uint32_t a_hi = smem_u32(st), a_lo = smem_u32(st + A_BYTES);
        const uint32_t b_hi = smem_u32(st + 2 * A_BYTES), b_lo = smem_u32(st + 2 * A_BYTES + B_BYTES);
#pragma unroll
        for (int ks = 0; ks < TK / 16; ++ks) {  // K = 16 halves (32 bytes of a 64-byte row) per MMA
          const uint32_t off = ks * 32;
          const uint32_t acc = (kb > 0 || ks > 0) ? 1u : 0u;
          mma_f16(acc_addr, smem_desc_sw64(a_hi + off), smem_desc_sw64(b_hi + off), acc);
          mma_f16(acc_addr, smem_desc_sw64(a_hi + off), smem_desc_sw64(b_lo + off), 1u);
          mma_f16(acc_addr, smem_desc_sw64(a_lo + off), smem_desc_sw64(b_hi + off), 1u);
        }
        mma_commit(&empty_bar[s]);
      }
      if (!ok) {
        s_fail = 1;
        break;
      }
      mma_commit(&acc_full[buf]);  // arrives when this tile's MMAs have completed
    }
    mma_commit(&done_bar);  // arrives once every MMA issued above has completed
  } else if (warp >= 2) {
    // epilogue: TMEM lane quarter q = warp % 4 holds rows m0 + 32 q .. + 31
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;  // this warp's chunks: half, half + 2, ...
    float* sb = (float*)(base + P_STAGE_AREA + (size_t)(warp - 2) * 4096);
    int local = 0;
    for (int t = blockIdx.x; t < n_tiles && !s_fail; t += gridDim.x, ++local) {
      const int buf = local & 1;
      if (!mbar_wait(&acc_full[buf], (local >> 1) & 1, err, 3)) {
        s_fail = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int bz = t / per_matrix, rem = t - bz * per_matrix;
      const int m0 = (rem % tiles_m) * TM, n0 = (rem / tiles_m) * TN;
      const bool rows_live = m0 + q * 32 < M2;
      for (int cc = half; cc < TN / 32; cc += 2) {
        const int col = n0 + cc * 32;
        if (!rows_live || col >= N) continue;  // warp-uniform
        float v[32];
        tmem_ld_32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * TN + cc * 32), v);
        const float* isc = inv_scale + (size_t)bz * cols_pad + col;  // 1 / (s_A s_j) of these 32 columns
        // the reduce that last read this buffer must be done reading it
        if (lane == 0) bulk_wait_read<0>();
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 32; ++j) sb[j * 32 + lane] = -v[j] * __ldg(isc + j);
        fence_async_smem();
        __syncwarp();
        if (lane == 0) {
          tma_reduce_add_3d(&map_c, sb, x0 + m0 + q * 32, y0 + col, bz);
          bulk_commit();
        }
      }
      // this warp has read its quarter of the accumulator: the MMA warp may reuse it
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[buf])) : "memory");
    }
    if (lane == 0) bulk_wait_read<0>();
    __syncwarp();
  }
  __syncwarp();
  __syncthreads();
  if (threadIdx.x == 0) {
    // every MMA this CTA issued has completed before TMEM is released
    mbar_wait(&done_bar, 0, err, 6);
    // loads started but never consumed (only after a failure): wait for them (bounded)
    for (int j = max(s_consumed, issued - P_STAGES); j < issued; ++j)
      mbar_wait(&full_bar[j % P_STAGES], (j / P_STAGES) & 1, err, 4);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(P_TMEM_COLS));
}


typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Driver entry point of cuTensorMapEncodeTiled, resolved once (thread-safe
// static initialisation); null when the driver does not provide it.
EncodeTiledFn encode_fn() {
  static const EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (EncodeTiledFn)p;
    cudaGetLastError();
    return nullptr;
  }();
  return fn;
}

// Split operand map: x = K' (FP16, KP_MAX per row), y = row, z = matrix; box TK x box_rows.
bool make_map(CUtensorMap* map, __half* buf, int rows_pad, int batch, int box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return false;
  cuuint64_t dims[3] = {(cuuint64_t)KP_MAX, (cuuint64_t)rows_pad, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)KP_MAX * 2, (cuuint64_t)rows_pad * KP_MAX * 2};
  cuuint32_t box[3] = {(cuuint32_t)TK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, buf, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// C map: every whole matrix of the batch as reals, x = real row (2n), y = column (n),
// z = matrix; box 32 x 32, no swizzle.
bool make_c_map(CUtensorMap* map, float* base, int n, long long lda, long long strideA, int batch) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return false;
  cuuint64_t dims[3] = {(cuuint64_t)2 * n, (cuuint64_t)n, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)lda * 8, (cuuint64_t)strideA * 8};
  cuuint32_t box[3] = {32, 32, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// Number of SMs of the current device (the persistent grid), cached per device.
int sm_count() {
  static int cached[16] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 16) dev = 0;
  if (cached[dev] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = n > 0 ? n : 1;
  }
  return cached[dev];
}

}  // namespace bem

namespace bem {
// Workspace for one batched factorisation: split operand buffers sized for the
// first (largest) trailing update, the column scales of U12, tensor maps built
// once, and an error word.
struct TcGemmPlan {
  __half *ahi = nullptr, *alo = nullptr, *bhi = nullptr, *blo = nullptr;
  float* inv_scale = nullptr;
  int* err = nullptr;
  int rows_pad = 0, cols_pad = 0, batch = 0;
  CUtensorMap mahi, malo, mbhi, mblo, mc;
};

size_t tc_gemm_workspace_bytes(int n, int batch) {
  const size_t rows_pad = ((size_t)2 * n + TM - 1) / TM * TM;
  const size_t cols_pad = ((size_t)n + TN - 1) / TN * TN;
  return (2 * rows_pad + 2 * cols_pad) * KP_MAX * sizeof(__half) * batch + cols_pad * sizeof(float) * batch + 256 * 6;
}

bool tc_gemm_available() { return encode_fn() != nullptr; }

// Build the plan inside caller-provided workspace (tc_gemm_workspace_bytes(n, batch) bytes)
// for the batch of matrices at A (column-major, leading dimension lda, lda * n apart).
// Refuses (returns false) when a TMA coordinate or stride into A could break the
// 16-byte rule: odd nb, odd lda, or A not 16-byte aligned.
bool tc_gemm_plan(TcGemmPlan* p, void* workspace, int n, int batch, float2* A, long long lda, int nb) {
  if ((nb & 1) || (lda & 1) || ((uintptr_t)A & 15)) return false;
  const size_t rows_pad = ((size_t)2 * n + TM - 1) / TM * TM;
  const size_t cols_pad = ((size_t)n + TN - 1) / TN * TN;
  char* w = (char*)workspace;
  auto take = [&](size_t bytes) {
    char* r = w;
    w += (bytes + 255) / 256 * 256;
    return r;
  };
  p->rows_pad = (int)rows_pad;
  p->cols_pad = (int)cols_pad;
  p->batch = batch;
  p->ahi = (__half*)take(rows_pad * KP_MAX * sizeof(__half) * batch);
  p->alo = (__half*)take(rows_pad * KP_MAX * sizeof(__half) * batch);
  p->bhi = (__half*)take(cols_pad * KP_MAX * sizeof(__half) * batch);
  p->blo = (__half*)take(cols_pad * KP_MAX * sizeof(__half) * batch);
  p->inv_scale = (float*)take(cols_pad * sizeof(float) * batch);
  p->err = (int*)take(sizeof(int));
  return make_map(&p->mahi, p->ahi, (int)rows_pad, batch, TM) && make_map(&p->malo, p->alo, (int)rows_pad, batch, TM) &&
         make_map(&p->mbhi, p->bhi, (int)cols_pad, batch, TN) && make_map(&p->mblo, p->blo, (int)cols_pad, batch, TN) &&
         make_c_map(&p->mc, (float*)A, n, lda, lda * (long long)n, batch);
}

// C[row0:row0+M, col0:col0+N] -= A[row0:row0+M, kcol0:kcol0+K] * A[kcol0:kcol0+K, col0:col0+N]
// for every matrix of the batch (K <= 256).  Rows beyond M and columns beyond N
// inside the last tiles receive -0 (their split operands are zero).
cudaError_t tc_update(TcGemmPlan* p, float2* A, long long lda, long long strideA, int row0, int M, int col0, int N,
                      int kcol0, int K, cudaStream_t stream) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  if (2 * K > KP_MAX) return cudaErrorInvalidValue;
  if (row0 & 1) return cudaErrorInvalidValue;  // x coordinate 2 row0 must be a multiple of 4
  const int M2 = 2 * M;
  const int rows_used = (M2 + TM - 1) / TM * TM;
  const int cols_used = (N + TN - 1) / TN * TN;
  if (rows_used > p->rows_pad || cols_used > p->cols_pad) return cudaErrorInvalidValue;
  const int kp = (2 * K + TK - 1) / TK * TK;
  {
    const int nta = (rows_used / 64) * (kp / 32);  // A tiles: 64 embedded rows x 32
    const int nb_b = cols_used / 8;                 // B: one warp per column, eight per block
    dim3 g((unsigned)(nta + nb_b), p->batch);
    prep_ab_kernel<<<g, 256, 0, stream>>>(A, lda, strideA, row0, col0, kcol0, M, N, K, p->rows_pad, p->cols_pad,
                                          rows_used, cols_used, kp, nta, p->ahi, p->alo, p->bhi, p->blo,
                                          p->inv_scale);
  }
  const int tiles_m = rows_used / TM, tiles_n = cols_used / TN;
  const long long n_tiles = (long long)tiles_m * tiles_n * p->batch;
  if (!ensure_smem_limit((const void*)trailing_update_f16x3_persistent, P_SMEM)) return cudaErrorInvalidValue;
  const int grid = (int)std::min<long long>(n_tiles, sm_count());
  trailing_update_f16x3_persistent<<<grid, P_THREADS, P_SMEM, stream>>>(
      p->mahi, p->malo, p->mbhi, p->mblo, p->mc, p->inv_scale, p->cols_pad, 2 * row0, col0, M2, N, kp / TK, tiles_m,
      tiles_n, (int)n_tiles, p->err);
  return cudaGetLastError();
}

// C -= L21 * U12 for the block column at k (width kb) of every matrix in the batch.
cudaError_t tc_trailing_update(TcGemmPlan* p, float2* A, long long lda, long long strideA, int n, int k, int kb,
                               cudaStream_t stream) {
  return tc_update(p, A, lda, strideA, k + kb, n - k - kb, k + kb, n - k - kb, k, kb, stream);
}

int* tc_gemm_error_word(TcGemmPlan* p) { return p->err; }

size_t tc_gemm_plan_size() { return sizeof(TcGemmPlan); }

}  // namespace bem
