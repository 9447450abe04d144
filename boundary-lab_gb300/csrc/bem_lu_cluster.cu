// Cluster-resident LU panel factorisation and cluster triangular solves (sm_103a).
//
// Panel: the m x nb panel of one matrix is spread over the shared memory of a
// thread-block cluster (CL CTAs, each holding a contiguous block of panel rows,
// column-major).  Each column step does a local pivot search, publishes the
// CTA's candidate row, one cluster barrier, a pivot decision from the CL
// candidates read through distributed shared memory (DSMEM), then the swap,
// scaling and rank-1 update entirely in shared memory.
// Nothing touches global memory between the initial load and the final store,
// where the previous single-CTA kernel streamed the whole panel through L2 at
// every column.  Pivot choice is LAPACK's (first maximum of |re| + |im|).
//
// Solves: pivots are turned into a row permutation once per factorisation
// (lu_perm_kernel, in shared memory); each right-hand side is then solved by
// one cluster whose CTAs own blocks of rows: the owner of a 32-row diagonal
// block solves it with one warp, publishes the 32 values in a double-buffered
// shared slot, and after one cluster barrier every CTA applies the block's
// columns to its own rows.
//
// Cluster barriers are hardware barriers (barrier.cluster); every CTA of a
// cluster executes the same sequence of them, and the kernels end with a
// barrier so no CTA leaves while another may still read its shared memory.
#include <cooperative_groups.h>
#include <limits.h>

#include <type_traits>

#include "bem_common.cuh"
#include "bem_kernels.h"

namespace cg = cooperative_groups;

namespace bem {
namespace {

template <typename R> struct CT2;
template <> struct CT2<float> { typedef float2 C2; };
template <> struct CT2<double> { typedef double2 C2; };

template <typename C2> __device__ __forceinline__ auto abs1(C2 v) -> decltype(v.x) { return fabs(v.x) + fabs(v.y); }

template <typename C2> __device__ __forceinline__ C2 inverse(C2 d) {
  auto m = d.x * d.x + d.y * d.y;
  C2 r;
  r.x = d.x / m;
  r.y = -d.y / m;
  return r;
}

constexpr int kPanelThreads = 512;

// First maximum of (value, index): larger value wins, ties go to the smaller index
// (LAPACK's first maximum of |re| + |im| when indices are row numbers).
template <typename R> __device__ __forceinline__ void argmax_merge(R& b, int& x, R ov, int oi) {
  if (ov > b || (ov == b && oi < x)) {
    b = ov;
    x = oi;
  }
}
template <typename R> __device__ __forceinline__ void warp_argmax(R& b, int& x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) argmax_merge(b, x, __shfl_xor_sync(0xffffffffu, b, o), __shfl_xor_sync(0xffffffffu, x, o));
}

// Net row permutation of the interchanges (j, pivs[j]), j = 0..kb-1, applied in
// order (LAPACK laswp): row r of every column ends up holding the data of row
// src(r).  Computed by one warp: the rows of the diagonal block in top[], other
// pivot rows in a list searched with a ballot.  Writes [count, (k + r, k + src(r))
// for every moved row] (at most 2 kb pairs).
template <int NB> __device__ void net_row_map(const int* pivs, int kb, int k, int* out) {
  __shared__ int top[NB], erow[NB], econt[NB];
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < kb; i += 32) top[i] = i;
  __syncwarp();
  int n_ext = 0;
  for (int j = 0; j < kb; ++j) {
    const int p = pivs[j];
    if (p == j) continue;
    if (p < kb) {
      if (lane == 0) {
        const int t = top[j];
        top[j] = top[p];
        top[p] = t;
      }
      __syncwarp();
      continue;
    }
    int found = -1;
    for (int base = 0; base < n_ext && found < 0; base += 32) {
      const int idx = base + lane;
      const unsigned hit = __ballot_sync(0xffffffffu, idx < n_ext && erow[idx] == p);
      if (hit) found = base + __ffs(hit) - 1;
    }
    if (found < 0) {
      found = n_ext++;
      if (lane == 0) {
        erow[found] = p;
        econt[found] = p;
      }
    }
    __syncwarp();
    if (lane == 0) {
      const int t = top[j];
      top[j] = econt[found];
      econt[found] = t;
    }
    __syncwarp();
  }
  if (lane == 0) {
    int cnt = 0;
    for (int r = 0; r < kb; ++r)
      if (top[r] != r) {
        out[1 + 2 * cnt] = k + r;
        out[2 + 2 * cnt] = k + top[r];
        ++cnt;
      }
    for (int e = 0; e < n_ext; ++e)
      if (econt[e] != erow[e]) {
        out[1 + 2 * cnt] = k + erow[e];
        out[2 + 2 * cnt] = k + econt[e];
        ++cnt;
      }
    out[0] = cnt;
  }
}

// Apply a net row permutation to the columns outside the panel: one warp per
// column loads every source row (at most 4 per lane, all in flight), then
// stores every destination row.
template <typename C2>
__global__ void __launch_bounds__(256) lu_swap_rows_kernel(C2* A, long long lda, long long strideA, int n, int k,
                                                          int kb, const int* rowmap) {
  __shared__ int sdst[128], ssrc[128];
  __shared__ int s_cnt;
  const int* rm = rowmap + (size_t)blockIdx.y * kRowmapStride;
  if (threadIdx.x == 0) s_cnt = min(max(rm[0], 0), 128);
  __syncthreads();
  const int cnt = s_cnt;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    sdst[e] = rm[1 + 2 * e];
    ssrc[e] = rm[2 + 2 * e];
  }
  __syncthreads();
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * (blockDim.x >> 5) + wid;
  if (cnt == 0 || t >= n - kb) return;
  const int c = t < k ? t : t + kb;
  C2* a = A + (size_t)blockIdx.y * strideA + (size_t)c * lda;
  C2 v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int e = lane + 32 * q;
    if (e < cnt && (unsigned)ssrc[e] < (unsigned)n) v[q] = a[ssrc[e]];
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int e = lane + 32 * q;
    if (e < cnt && (unsigned)ssrc[e] < (unsigned)n && (unsigned)sdst[e] < (unsigned)n) a[sdst[e]] = v[q];
  }
}

// One column step has a single cluster barrier.  Before it, every CTA
// publishes its local pivot candidate (value, row) and the candidate's whole
// panel row, and the owner of row j publishes row j, into slot j & 1.  After
// it, every CTA reads the CL candidates (one lane each), takes the first
// maximum, copies the winning row and row j from their owners' slots, and
// finishes the column locally.  A slot is rewritten two columns later, after
// the next barrier, by which time every CTA has finished reading it.
template <typename R, int NB>
__global__ void __launch_bounds__(kPanelThreads) lu_panel_cluster_kernel(typename CT2<R>::C2* A, long long lda,
                                                                         long long strideA, int n, int k, int kb,
                                                                         int chunk, int* ipiv, int* info,
                                                                         int* rowmap) {
  typedef typename CT2<R>::C2 C2;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int CL = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int NW = blockDim.x >> 5;
  __shared__ int s_pivs[NB];  // pivot row of each column, panel-local (rank 0)
  C2* M = A + (size_t)blockIdx.y * strideA;
  int* piv = ipiv + (size_t)blockIdx.y * n;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2* P = reinterpret_cast<C2*>(smem_raw);  // [NB][chunk], this CTA's panel rows
  C2* pub = P + (size_t)NB * chunk;         // [2][NB] published candidate row
  C2* dg = pub + 2 * NB;                    // [2][NB] published row j (owner of row j)
  C2* urow = dg + 2 * NB;                   // pivot row after the interchange
  C2* drow = urow + NB;                     // row j before the interchange
  R* cval = reinterpret_cast<R*>(drow + NB);         // [2] published candidate value
  int* cidx = reinterpret_cast<int*>(cval + 2);      // [2] published candidate row
  __shared__ R wval[32];
  __shared__ int widx[32];
  __shared__ int s_bi, s_p, s_fallback;

  const int m = n - k;
  const int r0 = rank * chunk;
  const int rows = max(0, min(chunk, m - r0));
  // panel load: each thread owns rows, 16 independent column loads in flight
  for (int i = tid; i < rows; i += blockDim.x) {
    const C2* src = M + (size_t)k * lda + k + r0 + i;
#pragma unroll 16
    for (int c = 0; c < NB; ++c)
      if (c < kb) P[(size_t)c * chunk + i] = src[(size_t)c * lda];
  }
  __syncthreads();

  for (int j = 0; j < kb; ++j) {
    const int s = j & 1;
    const int owner_j = j / chunk;
    // local pivot candidate among this CTA's panel rows >= j
    R best = R(-1);
    int bi = INT_MAX;
    const C2* Pj = P + (size_t)j * chunk;
    for (int i = max(0, j - r0) + tid; i < rows; i += blockDim.x) argmax_merge(best, bi, abs1(Pj[i]), r0 + i);
    warp_argmax(best, bi);
    if (lane == 0) {
      wval[wid] = best;
      widx[wid] = bi;
    }
    __syncthreads();
    if (wid == 0) {
      R b = lane < NW ? wval[lane] : R(-1);
      int x = lane < NW ? widx[lane] : INT_MAX;
      warp_argmax(b, x);
      if (lane == 0) {
        cval[s] = b;
        cidx[s] = x;
        s_bi = x;
      }
    }
    __syncthreads();
    const int bi_loc = s_bi;
    if (bi_loc != INT_MAX)
      for (int c = tid; c < kb; c += blockDim.x) pub[s * NB + c] = P[(size_t)c * chunk + (bi_loc - r0)];
    if (rank == owner_j)
      for (int c = tid; c < kb; c += blockDim.x) dg[s * NB + c] = P[(size_t)c * chunk + (j - r0)];
    cluster.sync();  // candidates, candidate rows and row j of this column are published
    if (wid == 0) {
      R b = R(-1);
      int x = INT_MAX;
      if (lane < CL) {
        b = *cluster.map_shared_rank(cval + s, lane);
        x = *cluster.map_shared_rank(cidx + s, lane);
      }
      warp_argmax(b, x);
      if (lane == 0) {
        s_fallback = x == INT_MAX;  // no comparable candidate (all NaN): keep row j
        s_p = x == INT_MAX ? j : x;
      }
    }
    __syncthreads();
    const int p = s_p;
    const int owner_p = p / chunk;
    {
      const C2* src_u = s_fallback ? cluster.map_shared_rank(dg + s * NB, owner_j)
                                   : cluster.map_shared_rank(pub + s * NB, owner_p);
      const C2* src_d = cluster.map_shared_rank(dg + s * NB, owner_j);
      for (int c = tid; c < kb; c += blockDim.x) {
        urow[c] = src_u[c];
        drow[c] = src_d[c];
      }
    }
    __syncthreads();
    if (p != j) {
      if (rank == owner_j)
        for (int c = tid; c < kb; c += blockDim.x) P[(size_t)c * chunk + (j - r0)] = urow[c];
      if (rank == owner_p)
        for (int c = tid; c < kb; c += blockDim.x) P[(size_t)c * chunk + (p - r0)] = drow[c];
    }
    if (rank == 0 && tid == 0) {
      piv[k + j] = k + p;
      s_pivs[j] = p;
    }
    __syncthreads();
    const C2 d = urow[j];
    C2 inv;
    if (d.x == R(0) && d.y == R(0)) {
      inv.x = R(0);
      inv.y = R(0);
      if (rank == 0 && tid == 0 && info[blockIdx.y] == 0) info[blockIdx.y] = k + j + 1;
    } else {
      inv = inverse(d);
    }
    const int i0 = min(rows, max(0, j + 1 - r0));  // first local row below the diagonal
    C2* Pcol = P + (size_t)j * chunk;
    for (int i = i0 + tid; i < rows; i += blockDim.x) Pcol[i] = cmul(Pcol[i], inv);
    __syncthreads();
    // rank-1 update of columns j+1.. : warps take columns, lanes take rows
    for (int c = j + 1 + wid; c < kb; c += NW) {
      const C2 u = urow[c];
      C2* Pc = P + (size_t)c * chunk;
      for (int i = i0 + lane; i < rows; i += 32) {
        const C2 l = Pcol[i];
        C2 v = Pc[i];
        v.x -= l.x * u.x - l.y * u.y;
        v.y -= l.x * u.y + l.y * u.x;
        Pc[i] = v;
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < rows; i += blockDim.x) {
    C2* dst = M + (size_t)k * lda + k + r0 + i;
#pragma unroll 16
    for (int c = 0; c < NB; ++c)
      if (c < kb) dst[(size_t)c * lda] = P[(size_t)c * chunk + i];
  }
  if (rank == 0 && wid == 0 && rowmap != nullptr) net_row_map<NB>(s_pivs, kb, k, rowmap + (size_t)blockIdx.y * kRowmapStride);
  cluster.sync();  // no CTA leaves while others may still read its shared memory
}

// Register-resident panel (mixed form, 32 columns): one thread per panel row.
// The thread keeps the part of its row right of the current column in
// registers, shifted so that the current column is always a[0] (every register
// index is a constant, and the step loop stays rolled); the multipliers it
// produces go to shared memory (Lb[column][thread]).  Interchanges are virtual:
// each thread carries the logical row index lg of its physical row, the pivot
// search compares logical indices (LAPACK's first maximum of |re| + |im|), and
// every row is written once, at the end, to its logical position.  A step:
//  1. this CTA's candidate row (the smallest lg among the largest) and the
//     candidate (value, lg) are pushed into slot j & 1 of every CTA (DSMEM
//     stores), and the row with lg = j is copied into the local row-j slot;
//     the writers fence (acq_rel, cluster scope);
//  2. cluster barrier (relaxed arrive, acquiring wait);
//  3. every warp takes the pivot and reads the pivot row from its own shared
//     memory (the pivot's U row j: columns j.. as u[0..]); rank 0 stores it;
//     only if every candidate is NaN is row j fetched from its CTA instead;
//  4. the pivot row leaves (lg = j), the row with lg = j takes the pivot's old
//     lg; every other active row stores l = a[0] / pivot, subtracts l u and
//     shifts; the next candidate is reduced per warp; CTA barrier.
// Requires a full panel (kb = 32) and chunk <= kRegPanelThreads.
constexpr int kRegPanelThreads = 640;
constexpr int kRegPanelWarps = kRegPanelThreads / 32;

// Pivot candidates as one 64-bit key: the bits of |re| + |im| (non-negative,
// so their unsigned order is the value order) above the complement of the
// logical row, so the largest key is the first maximum (larger value, then
// smaller row).  NaN values and rows without a candidate get key 0, which no
// candidate key equals (the low word ~row is at least 2^31).
__device__ __forceinline__ unsigned long long pivot_key(float v, int row) {
  return v == v ? ((unsigned long long)__float_as_uint(v) << 32) | (unsigned)~row : 0ull;
}
__device__ __forceinline__ int key_row(unsigned long long key) { return (int)~(unsigned)key; }
__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long k) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(0xffffffffu, k, o);
    k = ok > k ? ok : k;
  }
  return k;
}

__global__ void __launch_bounds__(kRegPanelThreads, 1) lu_panel_reg_kernel(float2* A, long long lda, long long strideA,
                                                                           int n, int k, int kb, int chunk, int* ipiv,
                                                                           int* info, int* rowmap) {
  constexpr int NB = 32;
  constexpr int NW = kRegPanelWarps;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int CL = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* Lb = reinterpret_cast<float2*>(smem_raw);  // [NB][kRegPanelThreads] multipliers by column, thread
  __shared__ float2 rowsC[2][16][NB];  // pushed candidate rows, by source CTA
  __shared__ float2 pub[NB], dg[2][NB];
  __shared__ float2 urow[NB];
  __shared__ unsigned long long ckey[2][16], wkey[NW];
  __shared__ int chasj[2][16];
  __shared__ int s_pivs[NB];
  float2* M = A + (size_t)blockIdx.y * strideA;
  int* piv = ipiv + (size_t)blockIdx.y * n;
  const int m = n - k;
  const int r0 = rank * chunk;
  const int rows = max(0, min(chunk, m - r0));
  const bool mine = tid < rows;
  int lg = r0 + tid;         // logical row of this thread's physical row
  int done_at = -1;          // step at which this row became the pivot row
  float2 a[NB];
  {
    const float2* src = M + (size_t)k * lda + k + r0 + tid;
#pragma unroll
    for (int c = 0; c < NB; ++c) a[c] = mine ? src[(size_t)c * lda] : make_float2(0.f, 0.f);
  }
  auto candidate = [&]() {  // the warp's candidate key for the current column
    return warp_max_key(mine && done_at < 0 ? pivot_key(abs1(a[0]), lg) : 0ull);
  };
  {
    const unsigned long long key = candidate();
    if (lane == 0) wkey[wid] = key;
  }
  __syncthreads();
#pragma unroll 1
  for (int j = 0; j < NB; ++j) {
    const int s = j & 1;
    {  // 1. publish and push
      const unsigned long long key = warp_max_key(lane < NW ? wkey[lane] : 0ull);
      const bool active = mine && done_at < 0;
      if (key != 0ull && active && lg == key_row(key)) {  // this CTA's candidate row (logical rows are distinct)
#pragma unroll
        for (int c = 0; c < NB; ++c) pub[c] = a[c];
      }
      const bool hasj = active && lg == j;
      if (hasj) {
#pragma unroll
        for (int c = 0; c < NB; ++c) dg[s][c] = a[c];
      }
      const int cnt = __syncthreads_or(hasj);
      bool wrote = hasj;
      if (key != 0ull && tid < CL * NB) {  // the candidate row into every CTA
        *cluster.map_shared_rank(&rowsC[s][rank][tid & (NB - 1)], tid / NB) = pub[tid & (NB - 1)];
        wrote = true;
      }
      if (tid < CL) {
        *cluster.map_shared_rank(&ckey[s][rank], tid) = key;
        *cluster.map_shared_rank(&chasj[s][rank], tid) = cnt;
        wrote = true;
      }
      if (wrote) asm volatile("fence.acq_rel.cluster;" ::: "memory");
    }
    // 2. the writes above were fenced by their writers; the wait acquires them
    asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.aligned;" ::: "memory");
    // 3. pivot (logical row p, held by CTA pr), in every warp
    const unsigned long long ck = lane < CL ? ckey[s][lane] : 0ull;
    const unsigned long long km = warp_max_key(ck);
    const bool fallback = km == 0ull;  // no comparable candidate (all NaN): keep row j
    const int pr = __ffs(__ballot_sync(0xffffffffu, lane < CL && ck == km)) - 1;  // keys are distinct
    const int p = fallback ? j : key_row(km);
    const float2* U = &rowsC[s][fallback ? 0 : pr][0];  // the pivot row, u[c] = U(j, j + c) (zero beyond the panel)
    if (fallback) {  // every CTA takes this branch together
      if (wid == 0) {
        int jr = 0;  // CTA holding logical row j
        const unsigned hb = __ballot_sync(0xffffffffu, lane < CL && chasj[s][lane] != 0);
        if (hb) jr = __ffs(hb) - 1;
        urow[lane] = *cluster.map_shared_rank(&dg[s][lane], jr);
      }
      __syncthreads();
      U = urow;
    }
    if (rank == 0 && wid == 0 && lane < NB - j)  // U row j
      M[(size_t)(k + j + lane) * lda + k + j] = U[lane];
    if (rank == 0 && tid == 0) {
      piv[k + j] = k + p;
      s_pivs[j] = p;
    }
    const float2 d = U[0];
    float2 inv;
    if (d.x == 0.f && d.y == 0.f) {
      inv = make_float2(0.f, 0.f);
      if (rank == 0 && tid == 0 && info[blockIdx.y] == 0) info[blockIdx.y] = k + j + 1;
    } else {
      inv = inverse(d);
    }
    // 4. this thread's row
    if (mine && done_at < 0) {
      if (lg == p) {  // the pivot row: it is logical row j now, finished
        lg = j;
        done_at = j;
      } else {
        if (lg == j) lg = p;  // the old row j moves to the pivot's place
        const float2 l = cmul(a[0], inv);
        Lb[(size_t)j * kRegPanelThreads + tid] = l;
        // a[c - 1] = a[c] - l u[c] for columns j + 1.. .  From step j the window holds 32 - j
        // live columns, so the update runs over the smallest multiple of 8 covering them (the
        // columns beyond are zero).  (Packed FP32x2 FMAs on a duplicated copy of the pivot
        // row took 4 more registers than the 96 a 640-thread CTA allows and spilled.)
        auto update = [&](auto width) {
          constexpr int W = decltype(width)::value;
#pragma unroll
          for (int c = 1; c < W; ++c) {
            const float2 u = U[c];
            a[c - 1].x = fmaf(-l.x, u.x, fmaf(l.y, u.y, a[c].x));
            a[c - 1].y = fmaf(-l.x, u.y, fmaf(-l.y, u.x, a[c].y));
          }
          a[W - 1] = make_float2(0.f, 0.f);
        };
        if (j < 8)
          update(std::integral_constant<int, 32>{});
        else if (j < 16)
          update(std::integral_constant<int, 24>{});
        else if (j < 24)
          update(std::integral_constant<int, 16>{});
        else
          update(std::integral_constant<int, 8>{});
      }
    }
    {
      const unsigned long long key = candidate();
      if (lane == 0) wkey[wid] = key;  // every thread read wkey in this step's push, before the cluster barrier
    }
    __syncthreads();
  }
  // every row to its logical position: the multipliers left of its pivot column
  // (all 32 for rows that never became the pivot)
  if (mine) {
    const int ncol = done_at < 0 ? NB : done_at;
    float2* dst = M + (size_t)k * lda + k + lg;
    for (int c = 0; c < ncol; ++c) dst[(size_t)c * lda] = Lb[(size_t)c * kRegPanelThreads + tid];
  }
  if (rank == 0 && wid == 0 && rowmap != nullptr) net_row_map<NB>(s_pivs, NB, k, rowmap + (size_t)blockIdx.y * kRowmapStride);
  cluster.sync();  // no CTA leaves while others may still read its shared memory
}

// perm[i] such that (P b)[i] = b[perm[i]], from LAPACK-style interchanges.
__global__ void lu_perm_kernel(const int* __restrict__ ipiv, int n, int* __restrict__ perm) {
  extern __shared__ int sp[];
  const int* piv = ipiv + (size_t)blockIdx.x * n;
  int* out = perm + (size_t)blockIdx.x * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) sp[i] = i;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < n; ++i) {
      const int p = piv[i];
      if (p != i && p >= 0 && p < n) {
        const int t = sp[i];
        sp[i] = sp[p];
        sp[p] = t;
      }
    }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = sp[i];
}

constexpr int kSolveThreads = 512;

// One cluster per (matrix, right-hand side): x = U^{-1} L^{-1} (P b), in place in B.
// Pull rows [lo, hi) of columns [c0, c0 + 32) of M (column-major, clipped to
// the n x n matrix) into L2 ahead of their use: one prefetch per 128-byte line,
// spread over the CTA's threads.
template <typename C2>
__device__ __forceinline__ void prefetch_strip_l2(const C2* M, long long lda, int n, int c0, int lo, int hi) {
  constexpr int kPerLine = 128 / (int)sizeof(C2);
  lo = max(lo, 0);
  hi = min(hi, n);
  if (hi <= lo || c0 >= n) return;
  const int first = lo / kPerLine, last = (hi - 1) / kPerLine;
  const int lines = last - first + 1;
  const int cols = min(32, n - c0);
  for (int i = threadIdx.x; i < lines * cols; i += blockDim.x) {
    const int c = i / lines, l = i - c * lines;
    const C2* ptr = M + (size_t)(c0 + c) * lda + (size_t)(first + l) * kPerLine;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr));
  }
}

template <typename R>
__global__ void __launch_bounds__(kSolveThreads) lu_solve_cluster_kernel(const typename CT2<R>::C2* A, long long lda,
                                                                         long long strideA, int n,
                                                                         const int* __restrict__ perm,
                                                                         typename CT2<R>::C2* B, long long ldb,
                                                                         int nrhs, int chunk) {
  typedef typename CT2<R>::C2 C2;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31;
  const int sys = blockIdx.y;
  const int mat = sys / nrhs;
  const C2* M = A + (size_t)mat * strideA;
  C2* b = B + (size_t)sys * ldb;
  const int* pm = perm + (size_t)mat * n;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2* x = reinterpret_cast<C2*>(smem_raw);  // my rows [r0, r0 + chunk)
  C2* pub = x + chunk;                      // [2][32] published block solutions
  const int r0 = rank * chunk;
  const int rows = max(0, min(chunk, n - r0));
  for (int i = tid; i < rows; i += blockDim.x) x[i] = b[pm[r0 + i]];
  cluster.sync();  // every CTA has read b before anyone writes it back
  const int nblk = (n + 31) / 32;
  // forward substitution with unit lower L
  if (rows > 0) prefetch_strip_l2(M, lda, n, 0, r0, r0 + rows);
  for (int t = 0; t < nblk; ++t) {
    const int k0 = t * 32, kb = min(32, n - k0);
    const int owner = k0 / chunk;
    C2* slot = pub + 32 * (t & 1);
    // the next step's columns of my rows (its diagonal block included) stream into L2 meanwhile
    if (rows > 0 && t + 1 < nblk) prefetch_strip_l2(M, lda, n, k0 + 32, max(r0, k0 + 32), r0 + rows);
    if (rank == owner && tid < 32) {
      // this lane's row of the diagonal block, loaded up front (independent loads)
      C2 Lr[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        if (j < kb && lane < kb) {
          Lr[j] = M[(size_t)(k0 + j) * lda + k0 + lane];
        } else {
          Lr[j].x = 0;
          Lr[j].y = 0;
        }
      }
      C2 v;
      v.x = 0;
      v.y = 0;
      if (lane < kb) v = x[k0 - r0 + lane];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        C2 xj;
        xj.x = __shfl_sync(0xffffffffu, v.x, j);
        xj.y = __shfl_sync(0xffffffffu, v.y, j);
        if (lane > j) {
          v.x -= Lr[j].x * xj.x - Lr[j].y * xj.y;
          v.y -= Lr[j].x * xj.y + Lr[j].y * xj.x;
        }
      }
      if (lane < kb) {
        x[k0 - r0 + lane] = v;
        slot[lane] = v;
      }
    }
    cluster.sync();
    __shared__ C2 xs[32];
    if (tid < kb) xs[tid] = cluster.map_shared_rank(slot, owner)[tid];
    __syncthreads();
    for (int i = tid; i < rows; i += blockDim.x) {
      const int r = r0 + i;
      if (r < k0 + kb) continue;
      C2 v = x[i];
      if (sizeof(C2) == sizeof(float2) && kb == 32) {  // FP32: all 32 loads in flight at once
        C2 l[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) l[j] = M[(size_t)(k0 + j) * lda + r];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const C2 s = xs[j];
          v.x -= l[j].x * s.x - l[j].y * s.y;
          v.y -= l[j].x * s.y + l[j].y * s.x;
        }
      } else {
#pragma unroll 8
        for (int j = 0; j < kb; ++j) {
          const C2 l = M[(size_t)(k0 + j) * lda + r];
          const C2 s = xs[j];
          v.x -= l.x * s.x - l.y * s.y;
          v.y -= l.x * s.y + l.y * s.x;
        }
      }
      x[i] = v;
    }
    __syncthreads();
  }
  // backward substitution with U
  if (rows > 0) prefetch_strip_l2(M, lda, n, (nblk - 1) * 32, r0, min(r0 + rows, n));
  for (int t = nblk - 1; t >= 0; --t) {
    const int k0 = t * 32, kb = min(32, n - k0);
    const int owner = k0 / chunk;
    // the next (lower) block's columns of my rows above its diagonal block's end
    if (rows > 0 && t > 0) prefetch_strip_l2(M, lda, n, k0 - 32, r0, min(r0 + rows, k0));
    // the slot alternates over the whole sequence of blocks (forward then backward)
    C2* slot = pub + 32 * ((nblk + (nblk - 1 - t)) & 1);
    if (rank == owner && tid < 32) {
      C2 Ur[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        if (j < kb && lane < kb) {
          Ur[j] = M[(size_t)(k0 + j) * lda + k0 + lane];
        } else {
          Ur[j].x = 0;
          Ur[j].y = 0;
        }
      }
      C2 dinv;
      dinv.x = 0;
      dinv.y = 0;
      if (lane < kb) dinv = inverse(M[(size_t)(k0 + lane) * lda + k0 + lane]);
      C2 v;
      v.x = 0;
      v.y = 0;
      if (lane < kb) v = x[k0 - r0 + lane];
#pragma unroll
      for (int j = 31; j >= 0; --j) {
        if (lane == j) v = cmul(v, dinv);
        C2 xj;
        xj.x = __shfl_sync(0xffffffffu, v.x, j);
        xj.y = __shfl_sync(0xffffffffu, v.y, j);
        if (lane < j) {
          v.x -= Ur[j].x * xj.x - Ur[j].y * xj.y;
          v.y -= Ur[j].x * xj.y + Ur[j].y * xj.x;
        }
      }
      if (lane < kb) {
        x[k0 - r0 + lane] = v;
        slot[lane] = v;
      }
    }
    cluster.sync();
    __shared__ C2 ys[32];
    if (tid < kb) ys[tid] = cluster.map_shared_rank(slot, owner)[tid];
    __syncthreads();
    for (int i = tid; i < rows; i += blockDim.x) {
      const int r = r0 + i;
      if (r >= k0) continue;
      C2 v = x[i];
      if (sizeof(C2) == sizeof(float2) && kb == 32) {  // FP32: all 32 loads in flight at once
        C2 u[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) u[j] = M[(size_t)(k0 + j) * lda + r];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const C2 s = ys[j];
          v.x -= u[j].x * s.x - u[j].y * s.y;
          v.y -= u[j].x * s.y + u[j].y * s.x;
        }
      } else {
#pragma unroll 8
        for (int j = 0; j < kb; ++j) {
          const C2 u = M[(size_t)(k0 + j) * lda + r];
          const C2 s = ys[j];
          v.x -= u.x * s.x - u.y * s.y;
          v.y -= u.x * s.y + u.y * s.x;
        }
      }
      x[i] = v;
    }
    __syncthreads();
  }
  for (int i = tid; i < rows; i += blockDim.x) b[r0 + i] = x[i];
  cluster.sync();
}

template <typename K>
cudaError_t launch_cluster(K kern, dim3 grid, int threads, size_t smem, int cl, cudaStream_t stream,
                           void** args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, (const void*)kern, args);
}

// Largest cluster size the kernel can be launched with at this shared-memory size.
template <typename K> int max_cluster(K kern, int threads, size_t smem) {
  if (!ensure_smem_limit((const void*)kern, smem)) return 0;
  cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(16, 1);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  int cl = 0;
  if (cudaOccupancyMaxPotentialClusterSize(&cl, (const void*)kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return cl;
}

constexpr size_t kPanelSmemBudget = 200 * 1024;

template <typename R, int NB> size_t panel_smem(int chunk) {
  typedef typename CT2<R>::C2 C2;
  return (size_t)NB * chunk * sizeof(C2) + 6 * NB * sizeof(C2) + 64;
}

// Clusters of size cl that can be resident at once for this kernel and shared memory.
template <typename K> int active_clusters(K kern, int threads, size_t smem, int cl) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cl, 1);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int num = 0;
  if (cudaOccupancyMaxActiveClusters(&num, (const void*)kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return num;
}

// Panel width and cluster size for an n x n batch.  The panel is latency-bound
// (a cluster barrier per column), so the batch's panels should run in as few
// waves of clusters as possible: among the (width, cluster size) pairs whose
// panel fits in shared memory, take the fewest waves (batch / resident
// clusters), then the wider panel, then the smaller cluster.  want_nb > 0 fixes
// the width.
template <typename R> bool choose_panel(int n, int want_nb, int batch, int& nb, int& cl) {
  bool found = false;
  int best_waves = 0;
  if (sizeof(R) == 4 && (want_nb == 0 || want_nb == 32)) {
    // the register-resident panel (32 wide) where a cluster of at most 16 CTAs
    // holds the rows at one per thread: the fewest waves, then the smallest cluster
    for (int c : {1, 2, 4, 8, 16}) {
      if ((n + c - 1) / c > kRegPanelThreads) continue;
      const size_t sm = (size_t)32 * kRegPanelThreads * sizeof(float2);
      if (c > 1 && max_cluster(lu_panel_reg_kernel, kRegPanelThreads, sm) < c) continue;
      if (c == 1 && !ensure_smem_limit((const void*)lu_panel_reg_kernel, sm)) continue;
      const int act = active_clusters(lu_panel_reg_kernel, kRegPanelThreads, sm, c);
      if (act < 1) continue;
      const int waves = (std::max(batch, 1) + act - 1) / act;
      if (!found || waves < best_waves) {
        found = true;
        best_waves = waves;
        nb = 32;
        cl = c;
      }
    }
    if (found) return true;
  }
  for (int w : {64, 32}) {
    if (want_nb > 0 && w != want_nb) continue;
    for (int c : {4, 8, 16}) {
      const int chunk = (n + c - 1) / c;
      const size_t sm = w == 64 ? panel_smem<R, 64>(chunk) : panel_smem<R, 32>(chunk);
      if (sm > kPanelSmemBudget) continue;
      const int maxcl = w == 64 ? max_cluster(lu_panel_cluster_kernel<R, 64>, kPanelThreads, sm)
                                : max_cluster(lu_panel_cluster_kernel<R, 32>, kPanelThreads, sm);
      if (maxcl < c) continue;
      const int act = w == 64 ? active_clusters(lu_panel_cluster_kernel<R, 64>, kPanelThreads, sm, c)
                              : active_clusters(lu_panel_cluster_kernel<R, 32>, kPanelThreads, sm, c);
      if (act < 1) continue;
      const int waves = (std::max(batch, 1) + act - 1) / act;
      if (!found || waves < best_waves) {  // candidates come wider first, then smaller clusters
        found = true;
        best_waves = waves;
        nb = w;
        cl = c;
      }
    }
  }
  return found;
}

}  // namespace

bool lu_cluster_plan(Precision prec, int n, int want_nb, int batch, int* nb, int* cl) {
  struct Key {
    int n = -1, want = 0, batch = 0;
  };
  static thread_local Key last[2];
  static thread_local int last_nb[2] = {0, 0}, last_cl[2] = {0, 0};
  static thread_local bool last_ok[2] = {false, false};
  const int pi = prec == Precision::Mixed ? 1 : 0;
  if (last[pi].n != n || last[pi].want != want_nb || last[pi].batch != batch) {
    int b = 0, c = 0;
    last_ok[pi] = prec == Precision::Mixed ? choose_panel<float>(n, want_nb, batch, b, c)
                                           : choose_panel<double>(n, want_nb, batch, b, c);
    last[pi].n = n;
    last[pi].want = want_nb;
    last[pi].batch = batch;
    last_nb[pi] = b;
    last_cl[pi] = c;
  }
  *nb = last_nb[pi];
  *cl = last_cl[pi];
  return last_ok[pi];
}

// Matrices whose cluster panels are resident at once (one wave) for an n x n
// factorisation with the panel plan of a large batch: a batch beyond this
// runs every panel in two waves.
int lu_resident_batch(Precision prec, int n) {
  int nb = 0, cl = 0;
  if (!lu_cluster_plan(prec, n, 0, 64, &nb, &cl)) return 64;
  const int chunk = (n + cl - 1) / cl;
  int act = 0;
  if (prec == Precision::Mixed && nb == 32 && chunk <= kRegPanelThreads)
    act = active_clusters(lu_panel_reg_kernel, kRegPanelThreads, (size_t)32 * kRegPanelThreads * sizeof(float2), cl);
  else if (prec == Precision::Mixed)
    act = nb == 64 ? active_clusters(lu_panel_cluster_kernel<float, 64>, kPanelThreads, panel_smem<float, 64>(chunk), cl)
                   : active_clusters(lu_panel_cluster_kernel<float, 32>, kPanelThreads, panel_smem<float, 32>(chunk), cl);
  else
    act = nb == 64 ? active_clusters(lu_panel_cluster_kernel<double, 64>, kPanelThreads, panel_smem<double, 64>(chunk), cl)
                   : active_clusters(lu_panel_cluster_kernel<double, 32>, kPanelThreads, panel_smem<double, 32>(chunk), cl);
  return std::max(1, act);
}

cudaError_t lu_panel_cluster(Precision prec, void* A, long long lda, long long strideA, int n, int k, int kb, int nb,
                             int cl, int batch, int* ipiv, int* info, cudaStream_t stream, int* rowmap) {
  const int m = n - k;
  const int chunk = (m + cl - 1) / cl;
  void* args[] = {&A, &lda, &strideA, &n, &k, &kb, (void*)&chunk, &ipiv, &info, &rowmap};
  dim3 grid(cl, batch);
  if (prec == Precision::Mixed && nb == 32 && chunk <= kRegPanelThreads && kb == 32) {
    const size_t sm = (size_t)32 * kRegPanelThreads * sizeof(float2);
    ensure_smem_limit((const void*)lu_panel_reg_kernel, sm);
    cudaFuncSetAttribute(lu_panel_reg_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return launch_cluster(lu_panel_reg_kernel, grid, kRegPanelThreads, sm, cl, stream, args);
  }
  if (prec == Precision::Mixed) {
    if (nb == 64) {
      const size_t sm = panel_smem<float, 64>(chunk);
      ensure_smem_limit((const void*)lu_panel_cluster_kernel<float, 64>, sm);
      cudaFuncSetAttribute(lu_panel_cluster_kernel<float, 64>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      return launch_cluster(lu_panel_cluster_kernel<float, 64>, grid, kPanelThreads, sm, cl, stream, args);
    }
    const size_t sm = panel_smem<float, 32>(chunk);
    ensure_smem_limit((const void*)lu_panel_cluster_kernel<float, 32>, sm);
    cudaFuncSetAttribute(lu_panel_cluster_kernel<float, 32>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return launch_cluster(lu_panel_cluster_kernel<float, 32>, grid, kPanelThreads, sm, cl, stream, args);
  }
  if (nb == 64) {
    const size_t sm = panel_smem<double, 64>(chunk);
    ensure_smem_limit((const void*)lu_panel_cluster_kernel<double, 64>, sm);
    cudaFuncSetAttribute(lu_panel_cluster_kernel<double, 64>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return launch_cluster(lu_panel_cluster_kernel<double, 64>, grid, kPanelThreads, sm, cl, stream, args);
  }
  const size_t sm = panel_smem<double, 32>(chunk);
  ensure_smem_limit((const void*)lu_panel_cluster_kernel<double, 32>, sm);
  cudaFuncSetAttribute(lu_panel_cluster_kernel<double, 32>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return launch_cluster(lu_panel_cluster_kernel<double, 32>, grid, kPanelThreads, sm, cl, stream, args);
}

cudaError_t lu_swap_rows_batched(Precision prec, void* A, long long lda, long long strideA, int n, int k, int kb,
                                 int batch, const int* rowmap, cudaStream_t stream) {
  if (n - kb <= 0) return cudaSuccess;
  dim3 g((unsigned)((n - kb + 7) / 8), batch);
  if (prec == Precision::Mixed)
    lu_swap_rows_kernel<float2><<<g, 256, 0, stream>>>((float2*)A, lda, strideA, n, k, kb, rowmap);
  else
    lu_swap_rows_kernel<double2><<<g, 256, 0, stream>>>((double2*)A, lda, strideA, n, k, kb, rowmap);
  return cudaGetLastError();
}

cudaError_t lu_perm_batched(const int* ipiv, int n, int batch, int* perm, cudaStream_t stream) {
  const size_t sm = (size_t)n * sizeof(int);
  if (sm > 48 * 1024) ensure_smem_limit((const void*)lu_perm_kernel, sm);
  lu_perm_kernel<<<batch, 256, sm, stream>>>(ipiv, n, perm);
  return cudaGetLastError();
}

cudaError_t lu_solve_cluster_batched(Precision prec, const void* LU, long long lda, int n, int batch, const int* perm,
                                     void* B, long long ldb, int nrhs, cudaStream_t stream) {
  const long long strideA = lda * (long long)n;
  const size_t esz = prec == Precision::Mixed ? sizeof(float2) : sizeof(double2);
  // rows per CTA: a multiple of 32 so that each 32-row block has one owner
  int cl = 8;
  int chunk = ((n + cl - 1) / cl + 31) / 32 * 32;
  const size_t sm = (size_t)(chunk + 64) * esz;
  dim3 grid(cl, batch * nrhs);
  if (prec == Precision::Mixed) {
    ensure_smem_limit((const void*)lu_solve_cluster_kernel<float>, sm);
    void* args[] = {&LU, &lda, (void*)&strideA, &n, &perm, &B, &ldb, &nrhs, &chunk};
    return launch_cluster(lu_solve_cluster_kernel<float>, grid, kSolveThreads, sm, cl, stream, args);
  }
  ensure_smem_limit((const void*)lu_solve_cluster_kernel<double>, sm);
  void* args[] = {&LU, &lda, (void*)&strideA, &n, &perm, &B, &ldb, &nrhs, &chunk};
  return launch_cluster(lu_solve_cluster_kernel<double>, grid, kSolveThreads, sm, cl, stream, args);
}

}  // namespace bem
