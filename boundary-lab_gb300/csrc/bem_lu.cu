// Dense complex LU with partial pivoting, triangular solves and the FP64
// residual for iterative refinement (sm_103a).
//
// The reference solves each Burton-Miller system with CUDA.jl's `\`
// (cuSOLVER getrf + getrs, src/blab/solvers/julia_local/src/
// BeatEngineCore.jl:1206) and refactors for every channel.  Here the matrix of
// one frequency is factored once and every excitation is solved against the
// factors; many frequencies are factored together as a batch so that
// panel-factorisation latency of one matrix overlaps the work of others.
//
// Blocked right-looking LU, per block column k of width nb:
//   lu_panel_kernel   pivot search (|re|+|im| as LAPACK's icamax), row swap,
//                     scaling and rank-1 updates inside the panel; one CTA per
//                     matrix of the batch
//   lu_swap_kernel    the panel's row interchanges applied to the other columns
//   lu_trsm_kernel    U12 = L11^{-1} A12 (unit lower), L11 staged in shared memory
//   trailing update   A22 -= L21 U12 : a batched complex GEMM
#include <cublas_v2.h>

#include <vector>

#include "bem_common.cuh"
#include "bem_kernels.h"

namespace bem {
namespace {

template <typename R> struct CT;
template <> struct CT<float> { typedef float2 C2; };
template <> struct CT<double> { typedef double2 C2; };

template <typename C2> __device__ __forceinline__ auto cabs1(C2 v) -> decltype(v.x) { return fabs(v.x) + fabs(v.y); }

template <typename C2> __device__ __forceinline__ C2 cinv(C2 d) {
  auto m = d.x * d.x + d.y * d.y;
  C2 r;
  r.x = d.x / m;
  r.y = -d.y / m;
  return r;
}

template <typename R>
__global__ void __launch_bounds__(1024) lu_panel_kernel(typename CT<R>::C2* A, long long lda, long long strideA, int n,
                                                        int k, int kb, int* ipiv, int* info) {
  typedef typename CT<R>::C2 C2;
  C2* M = A + (size_t)blockIdx.x * strideA;
  int* piv = ipiv + (size_t)blockIdx.x * n;
  __shared__ R s_val[32];
  __shared__ int s_idx[32];
  __shared__ C2 s_row[64];
  __shared__ int s_p;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  for (int j = 0; j < kb; ++j) {
    const int col = k + j;
    const C2* Mc = M + (size_t)col * lda;
    R best = R(-1);
    int bi = n;
    for (int r = col + tid; r < n; r += blockDim.x) {
      R v = cabs1(Mc[r]);
      if (v > best) {  // first maximum in row order within this thread's stride
        best = v;
        bi = r;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      R ov = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      s_val[wid] = best;
      s_idx[wid] = bi;
    }
    __syncthreads();
    if (wid == 0) {
      best = lane < nw ? s_val[lane] : R(-1);
      bi = lane < nw ? s_idx[lane] : n;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        R ov = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) {
        s_p = bi < n ? bi : col;
        piv[col] = s_p;
      }
    }
    __syncthreads();
    const int p = s_p;
    if (p != col) {
      for (int c = tid; c < kb; c += blockDim.x) {
        C2* a = M + (size_t)(k + c) * lda;
        C2 t = a[col];
        a[col] = a[p];
        a[p] = t;
      }
    }
    __syncthreads();
    for (int c = tid; c < kb; c += blockDim.x) s_row[c] = M[(size_t)(k + c) * lda + col];
    __syncthreads();
    const C2 d = s_row[j];
    C2 inv;
    if (d.x == R(0) && d.y == R(0)) {
      inv.x = R(0);
      inv.y = R(0);
      if (tid == 0 && info[blockIdx.x] == 0) info[blockIdx.x] = col + 1;
    } else {
      inv = cinv(d);
    }
    for (int r = col + 1 + tid; r < n; r += blockDim.x) {
      C2 l = cmul(M[(size_t)col * lda + r], inv);
      M[(size_t)col * lda + r] = l;
      for (int c = j + 1; c < kb; ++c) {
        C2* a = M + (size_t)(k + c) * lda + r;
        C2 u = s_row[c];
        C2 v = *a;
        v.x -= l.x * u.x - l.y * u.y;
        v.y -= l.x * u.y + l.y * u.x;
        *a = v;
      }
    }
    __syncthreads();
  }
}

template <typename C2>
__global__ void lu_swap_kernel(C2* A, long long lda, long long strideA, int n, int k, int kb, const int* ipiv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ncols = n - kb;
  if (t >= ncols) return;
  const int c = t < k ? t : t + kb;
  C2* a = A + (size_t)blockIdx.y * strideA + (size_t)c * lda;
  const int* piv = ipiv + (size_t)blockIdx.y * n;
  for (int j = 0; j < kb; ++j) {
    const int r1 = k + j, r2 = piv[k + j];
    if (r2 != r1) {
      C2 tmp = a[r1];
      a[r1] = a[r2];
      a[r2] = tmp;
    }
  }
}

// U12 = L11^{-1} A12 for rows [k, k+kb) and columns [c_begin, c_end), with L11 the
// unit lower triangle of A[k:k+kb, k:k+kb]; blockDim columns per CTA.  The
// column block is staged through shared memory with coalesced loads and stores
// (a warp per column, lanes along its rows); the substitution runs one thread
// per column.  X has a padded row stride so both access patterns are
// conflict-free.
template <typename C2>
__global__ void lu_trsm_kernel(C2* A, long long lda, long long strideA, int n, int k, int kb, int c_begin, int c_end) {
  extern __shared__ unsigned char smem_raw[];
  C2* L = reinterpret_cast<C2*>(smem_raw);  // kb x kb, column-major
  C2* X = L + kb * kb;                      // kb x (blockDim + 1)
  const int ldx = blockDim.x + 1;
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C2* M = A + (size_t)blockIdx.y * strideA;
  for (int i = threadIdx.x; i < kb * kb; i += blockDim.x) {
    const int r = i % kb, c = i / kb;
    L[i] = M[(size_t)(k + c) * lda + k + r];
  }
  const int c0 = c_begin + blockIdx.x * blockDim.x;
  const int ncol = min((int)blockDim.x, c_end - c0);
  // 8 columns x 2 row halves per warp and batch: 16 independent loads in flight
  for (int cb = wid; cb < ncol; cb += 8 * nw) {
    C2 v[8][2];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int cl = cb + u * nw, r = lane + 32 * h;
        if (cl < ncol && r < kb) v[u][h] = M[(size_t)(c0 + cl) * lda + k + r];
      }
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int cl = cb + u * nw, r = lane + 32 * h;
        if (cl < ncol && r < kb) X[r * ldx + cl] = v[u][h];
      }
  }
  __syncthreads();
  if ((int)threadIdx.x < ncol) {
    const int t = threadIdx.x;
    for (int j = 0; j < kb; ++j) {
      const C2 xj = X[j * ldx + t];
      for (int i = j + 1; i < kb; ++i) {
        const C2 l = L[j * kb + i];
        C2 v = X[i * ldx + t];
        v.x -= l.x * xj.x - l.y * xj.y;
        v.y -= l.x * xj.y + l.y * xj.x;
        X[i * ldx + t] = v;
      }
    }
  }
  __syncthreads();
  for (int cl = wid; cl < ncol; cl += nw) {
    C2* dst = M + (size_t)(c0 + cl) * lda + k;
    for (int r = lane; r < kb; r += 32) dst[r] = X[r * ldx + cl];
  }
}

// U12 = L11^{-1} A12 for a 32-row block (mixed form): one thread per column,
// the column's 32 complex entries in registers (the 32 x 32 substitution is
// fully unrolled, so every index is a constant); L11 (unit lower) in shared
// memory, read as broadcasts.  Replaces lu_trsm_kernel's shared-memory column
// for kb = 32: 496 multiply-adds per column with no shared-memory traffic for X.
__global__ void __launch_bounds__(128) lu_trsm32_kernel(float2* A, long long lda, long long strideA, int k,
                                                        int c_begin, int c_end) {
  __shared__ float2 L[32 * 32];  // column-major
  float2* M = A + (size_t)blockIdx.y * strideA;
  for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
    const int r = i & 31, c = i >> 5;
    L[i] = M[(size_t)(k + c) * lda + k + r];
  }
  __syncthreads();
  const int col = c_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= c_end) return;
  float4* src = reinterpret_cast<float4*>(M + (size_t)col * lda + k);  // 16-byte aligned: lda and k are even
  float2 x[32];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const float4 v = src[q];
    x[2 * q] = make_float2(v.x, v.y);
    x[2 * q + 1] = make_float2(v.z, v.w);
  }
#pragma unroll
  for (int j = 0; j < 31; ++j) {
    const float2 xj = x[j];
#pragma unroll
    for (int i = j + 1; i < 32; ++i) {
      const float2 l = L[j * 32 + i];
      x[i].x = fmaf(-l.x, xj.x, fmaf(l.y, xj.y, x[i].x));
      x[i].y = fmaf(-l.x, xj.y, fmaf(-l.y, xj.x, x[i].y));
    }
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) src[q] = make_float4(x[2 * q].x, x[2 * q].y, x[2 * q + 1].x, x[2 * q + 1].y);
}

// One CTA per (matrix, right-hand side): P, then L (unit lower), then U.
template <typename R>
__global__ void __launch_bounds__(1024) lu_solve_kernel(const typename CT<R>::C2* A, long long lda, long long strideA,
                                                        int n, const int* ipiv, typename CT<R>::C2* B, long long ldb,
                                                        int nrhs) {
  typedef typename CT<R>::C2 C2;
  const int mat = blockIdx.x / nrhs, rhs = blockIdx.x % nrhs;
  const C2* M = A + (size_t)mat * strideA;
  const int* piv = ipiv + (size_t)mat * n;
  C2* b = B + ((size_t)mat * nrhs + rhs) * ldb;
  __shared__ C2 xs[32];
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid == 0)
    for (int i = 0; i < n; ++i) {
      const int p = piv[i];
      if (p != i) {
        C2 t = b[i];
        b[i] = b[p];
        b[p] = t;
      }
    }
  __syncthreads();
  // forward substitution, blocks of 32 rows
  for (int k0 = 0; k0 < n; k0 += 32) {
    const int kb = min(32, n - k0);
    if (tid < 32) {
      C2 v;
      v.x = 0;
      v.y = 0;
      if (lane < kb) v = b[k0 + lane];
      for (int j = 0; j < kb; ++j) {
        C2 xj;
        xj.x = __shfl_sync(0xffffffffu, v.x, j);
        xj.y = __shfl_sync(0xffffffffu, v.y, j);
        if (lane > j && lane < kb) {
          const C2 l = M[(size_t)(k0 + j) * lda + k0 + lane];
          v.x -= l.x * xj.x - l.y * xj.y;
          v.y -= l.x * xj.y + l.y * xj.x;
        }
      }
      if (lane < kb) {
        b[k0 + lane] = v;
        xs[lane] = v;
      }
    }
    __syncthreads();
    for (int r = k0 + kb + tid; r < n; r += blockDim.x) {
      C2 v = b[r];
      for (int j = 0; j < kb; ++j) {
        const C2 l = M[(size_t)(k0 + j) * lda + r];
        const C2 x = xs[j];
        v.x -= l.x * x.x - l.y * x.y;
        v.y -= l.x * x.y + l.y * x.x;
      }
      b[r] = v;
    }
    __syncthreads();
  }
  // backward substitution
  const int nblk = (n + 31) / 32;
  for (int bi = nblk - 1; bi >= 0; --bi) {
    const int k0 = bi * 32;
    const int kb = min(32, n - k0);
    if (tid < 32) {
      C2 v;
      v.x = 0;
      v.y = 0;
      if (lane < kb) v = b[k0 + lane];
      for (int j = kb - 1; j >= 0; --j) {
        C2 xj;
        if (lane == j) {
          const C2 d = M[(size_t)(k0 + j) * lda + k0 + j];
          v = cmul(v, cinv(d));
        }
        xj.x = __shfl_sync(0xffffffffu, v.x, j);
        xj.y = __shfl_sync(0xffffffffu, v.y, j);
        if (lane < j) {
          const C2 u = M[(size_t)(k0 + j) * lda + k0 + lane];
          v.x -= u.x * xj.x - u.y * xj.y;
          v.y -= u.x * xj.y + u.y * xj.x;
        }
      }
      if (lane < kb) {
        b[k0 + lane] = v;
        xs[lane] = v;
      }
    }
    __syncthreads();
    for (int r = tid; r < k0; r += blockDim.x) {
      C2 v = b[r];
      for (int j = 0; j < kb; ++j) {
        const C2 u = M[(size_t)(k0 + j) * lda + r];
        const C2 x = xs[j];
        v.x -= u.x * x.x - u.y * x.y;
        v.y -= u.x * x.y + u.y * x.x;
      }
      b[r] = v;
    }
    __syncthreads();
  }
}

template <typename C2>
__global__ void residual_kernel(const C2* __restrict__ A, long long lda, long long strideA, int n,
                                const double2* __restrict__ x, const double2* __restrict__ b, long long ldb, int nrhs,
                                double2* __restrict__ r) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  const int mat = blockIdx.y / nrhs, rhs = blockIdx.y % nrhs;
  if (row >= n) return;
  const C2* M = A + (size_t)mat * strideA;
  const size_t off = ((size_t)mat * nrhs + rhs) * ldb;
  const double2* xv = x + off;
  double sr = 0.0, si = 0.0;
  for (int j = 0; j < n; ++j) {
    const C2 a = M[(size_t)j * lda + row];
    const double2 xj = xv[j];
    const double ar = (double)a.x, ai = (double)a.y;
    sr = fma(ar, xj.x, sr);
    sr = fma(-ai, xj.y, sr);
    si = fma(ar, xj.y, si);
    si = fma(ai, xj.x, si);
  }
  const double2 bb = b[off + row];
  r[off + row] = make_double2(bb.x - sr, bb.y - si);
}

// r = b - A x for an FP32 matrix A and FP64 x (the mixed form's refinement
// residual) with no FP64 arithmetic in the inner loop: this part's FP64 rate is
// a small fraction of its FP32 rate.  Per tile of 256 columns, x is split into
// float pairs x = xh + xl in shared memory; every product a * xh is formed
// exactly as p + fma(a, xh, -p), the p are summed in double-float (two_sum),
// and the small terms (product errors and a * xl) in FP32.  The tile sums are
// added in FP64, so the result carries about 2^-40 relative error per tile:
// far below the 1e-10 refinement target.
__device__ __forceinline__ void acc_exact_prod(float& sh, float& sl, float& e, float a, float xh, float xl) {
  const float p = a * xh;
  const float pe = fmaf(a, xh, -p);
  const float t = sh + p;
  const float bb = t - sh;
  sl += (sh - (t - bb)) + (p - bb);
  sh = t;
  e = fmaf(a, xl, e + pe);
}

// x (FP64) as float hi / lo pairs (re hi, im hi, re lo, im lo), once per residual,
// so the residual kernel below runs no FP64 instruction in its inner loop.
__global__ void split_x_kernel(const double2* __restrict__ x, float4* __restrict__ xs, long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const double2 v = x[i];
  const float hr = (float)v.x, hi = (float)v.y;
  xs[i] = make_float4(hr, hi, (float)(v.x - (double)hr), (float)(v.y - (double)hi));
}

// r = b - A x with A in FP32 and x in FP64: every product a * (x_hi + x_lo) is
// formed exactly (two FMAs) and summed in double-float, so r carries the
// accuracy of an FP64 product with the FP32 matrix.  A CTA covers 64 rows; its
// four groups of 64 threads take interleaved 64-column slices of each
// 256-column block of x staged in shared memory, each thread keeping two
// independent double-float sums (even / odd columns).  The four partial sums of
// a row are added in a fixed order at the end (deterministic).
__global__ void __launch_bounds__(256) residual_f32a_kernel(const float2* __restrict__ A, long long lda,
                                                            long long strideA, int n, const float4* __restrict__ xs,
                                                            const double2* __restrict__ b, long long ldb, int nrhs,
                                                            double2* __restrict__ r) {
  __shared__ float4 xsh[256];
  __shared__ double part[2][4][64];
  const int rl = threadIdx.x & 63, cg = threadIdx.x >> 6;
  const int row = blockIdx.x * 64 + rl;
  const int mat = blockIdx.y / nrhs, rhs = blockIdx.y % nrhs;
  const float2* M = A + (size_t)mat * strideA;
  const size_t off = ((size_t)mat * nrhs + rhs) * ldb;
  const float4* xv = xs + off;
  float srh = 0.f, srl = 0.f, er = 0.f, sih = 0.f, sil = 0.f, ei = 0.f;      // even columns
  float trh = 0.f, trl = 0.f, fr = 0.f, tih = 0.f, til = 0.f, fi = 0.f;      // odd columns
  for (int j0 = 0; j0 < n; j0 += 256) {
    __syncthreads();
    {
      const int j = j0 + threadIdx.x;
      xsh[threadIdx.x] = j < n ? xv[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const int cb = j0 + cg * 64;
    const int jn = min(64, n - cb);
    if (row < n && jn > 0) {
      const float2* col = M + (size_t)cb * lda + row;
      const float4* xg = xsh + cg * 64;
      int t = 0;
#pragma unroll 4
      for (; t + 1 < jn; t += 2) {
        const float2 a0 = col[(size_t)t * lda], a1 = col[(size_t)(t + 1) * lda];
        const float4 x0 = xg[t], x1 = xg[t + 1];
        // re += a.x xr - a.y xi ; im += a.x xi + a.y xr
        acc_exact_prod(srh, srl, er, a0.x, x0.x, x0.z);
        acc_exact_prod(srh, srl, er, -a0.y, x0.y, x0.w);
        acc_exact_prod(sih, sil, ei, a0.x, x0.y, x0.w);
        acc_exact_prod(sih, sil, ei, a0.y, x0.x, x0.z);
        acc_exact_prod(trh, trl, fr, a1.x, x1.x, x1.z);
        acc_exact_prod(trh, trl, fr, -a1.y, x1.y, x1.w);
        acc_exact_prod(tih, til, fi, a1.x, x1.y, x1.w);
        acc_exact_prod(tih, til, fi, a1.y, x1.x, x1.z);
      }
      if (t < jn) {
        const float2 a0 = col[(size_t)t * lda];
        const float4 x0 = xg[t];
        acc_exact_prod(srh, srl, er, a0.x, x0.x, x0.z);
        acc_exact_prod(srh, srl, er, -a0.y, x0.y, x0.w);
        acc_exact_prod(sih, sil, ei, a0.x, x0.y, x0.w);
        acc_exact_prod(sih, sil, ei, a0.y, x0.x, x0.z);
      }
    }
  }
  part[0][cg][rl] = ((double)srh + ((double)srl + (double)er)) + ((double)trh + ((double)trl + (double)fr));
  part[1][cg][rl] = ((double)sih + ((double)sil + (double)ei)) + ((double)tih + ((double)til + (double)fi));
  __syncthreads();
  if (cg == 0 && row < n) {
    const double accr = ((part[0][0][rl] + part[0][1][rl]) + part[0][2][rl]) + part[0][3][rl];
    const double acci = ((part[1][0][rl] + part[1][1][rl]) + part[1][2][rl]) + part[1][3][rl];
    const double2 bb = b[off + row];
    r[off + row] = make_double2(bb.x - accr, bb.y - acci);
  }
}

__global__ void norms_kernel(const double2* __restrict__ r, const double2* __restrict__ b, long long ldb, int n,
                             double* out) {
  const double2* rv = r + (size_t)blockIdx.x * ldb;
  const double2* bv = b + (size_t)blockIdx.x * ldb;
  double sr = 0.0, sb = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    sr += rv[i].x * rv[i].x + rv[i].y * rv[i].y;
    sb += bv[i].x * bv[i].x + bv[i].y * bv[i].y;
  }
  __shared__ double s1[32], s2[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s1[threadIdx.x >> 5] = sr;
    s2[threadIdx.x >> 5] = sb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, c = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += s1[w];
      c += s2[w];
    }
    out[2 * blockIdx.x] = a;
    out[2 * blockIdx.x + 1] = c;
  }
}

__global__ void axpy_kernel(const float2* d, double2* x, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    x[i].x += (double)d[i].x;
    x[i].y += (double)d[i].y;
  }
}
__global__ void f64_to_f32_kernel(const double2* s, float2* d, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = make_float2((float)s[i].x, (float)s[i].y);
}
__global__ void f32_to_f64_kernel(const float2* s, double2* d, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = make_double2((double)s[i].x, (double)s[i].y);
}

}  // namespace

bool tc_gemm_plan(TcGemmPlan* p, void* workspace, int n, int batch, float2* A, long long lda, int nb);
cudaError_t tc_trailing_update(TcGemmPlan* p, float2* A, long long lda, long long strideA, int n, int k, int kb,
                               cudaStream_t stream);
cudaError_t tc_update(TcGemmPlan* p, float2* A, long long lda, long long strideA, int row0, int M, int col0, int N,
                      int kcol0, int K, cudaStream_t stream);
size_t tc_gemm_plan_size();

namespace {

// State of one batched factorisation for the two-level driver.
struct LuJob {
  Precision prec;
  void* A;
  long long lda, strideA;
  int n, batch, nb, cl;
  int* ipiv;
  int* info;
  int* rowmap;
  TcGemmPlan* plan;  // tcgen05 updates (mixed form); null: cuBLAS
  cublasHandle_t h;
  cudaStream_t stream;
};

// U rows [k, k+kb) of columns [c0, c1): U = L^{-1} A with L the unit lower triangle of A[k:k+kb, k:k+kb].
cudaError_t trsm_cols(const LuJob& j, int k, int kb, int c0, int c1) {
  if (c1 <= c0 || kb <= 0) return cudaSuccess;
  if (j.prec == Precision::Mixed && kb == 32 && (j.lda & 1) == 0 && (k & 1) == 0) {
    dim3 g((unsigned)((c1 - c0 + 127) / 128), j.batch);
    lu_trsm32_kernel<<<g, 128, 0, j.stream>>>((float2*)j.A, j.lda, j.strideA, k, c0, c1);
    return cudaGetLastError();
  }
  const int tpb = 128;
  dim3 g((unsigned)((c1 - c0 + tpb - 1) / tpb), j.batch);
  if (j.prec == Precision::Mixed) {
    const size_t sm = (size_t)kb * kb * sizeof(float2) + (size_t)kb * (tpb + 1) * sizeof(float2);
    if (sm > 48 * 1024) ensure_smem_limit((const void*)lu_trsm_kernel<float2>, sm);
    lu_trsm_kernel<float2><<<g, tpb, sm, j.stream>>>((float2*)j.A, j.lda, j.strideA, j.n, k, kb, c0, c1);
  } else {
    const size_t sm = (size_t)kb * kb * sizeof(double2) + (size_t)kb * (tpb + 1) * sizeof(double2);
    if (sm > 48 * 1024) ensure_smem_limit((const void*)lu_trsm_kernel<double2>, sm);
    lu_trsm_kernel<double2><<<g, tpb, sm, j.stream>>>((double2*)j.A, j.lda, j.strideA, j.n, k, kb, c0, c1);
  }
  return cudaGetLastError();
}

// A[r0:r0+M, c0:c0+N] -= A[r0:r0+M, kc:kc+K] * A[kc:kc+K, c0:c0+N] for every matrix.
cudaError_t block_update(const LuJob& j, int r0, int M, int c0, int N, int kc, int K) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  if (j.plan) return tc_update(j.plan, (float2*)j.A, j.lda, j.strideA, r0, M, c0, N, kc, K, j.stream);
  const int ld = (int)j.lda;
  if (j.prec == Precision::Mixed) {
    const cuComplex alpha = make_cuComplex(-1.f, 0.f), beta = make_cuComplex(1.f, 0.f);
    const cuComplex* base = (const cuComplex*)j.A;
    const cublasStatus_t st = cublasCgemmStridedBatched(
        j.h, CUBLAS_OP_N, CUBLAS_OP_N, M, N, K, &alpha, base + r0 + (size_t)kc * j.lda, ld, j.strideA,
        base + kc + (size_t)c0 * j.lda, ld, j.strideA, &beta, (cuComplex*)j.A + r0 + (size_t)c0 * j.lda, ld, j.strideA,
        j.batch);
    return st == CUBLAS_STATUS_SUCCESS ? cudaSuccess : cudaErrorUnknown;
  }
  const cuDoubleComplex alpha = make_cuDoubleComplex(-1.0, 0.0), beta = make_cuDoubleComplex(1.0, 0.0);
  const cuDoubleComplex* base = (const cuDoubleComplex*)j.A;
  const cublasStatus_t st = cublasZgemmStridedBatched(
      j.h, CUBLAS_OP_N, CUBLAS_OP_N, M, N, K, &alpha, base + r0 + (size_t)kc * j.lda, ld, j.strideA,
      base + kc + (size_t)c0 * j.lda, ld, j.strideA, &beta, (cuDoubleComplex*)j.A + r0 + (size_t)c0 * j.lda, ld,
      j.strideA, j.batch);
  return st == CUBLAS_STATUS_SUCCESS ? cudaSuccess : cudaErrorUnknown;
}

#define BEM_TRY(x)                          \
  do {                                      \
    const cudaError_t e_ = (x);             \
    if (e_ != cudaSuccess) return e_;       \
  } while (0)

// Two-level right-looking LU.  The matrix is factored in outer block columns of
// width NB (kOuterBlock, 256): each is factored as sub-panels of width nb (the cluster panel
// width, 32 or 64) with their row interchanges applied to every other column
// and the rest of the outer block updated after each sub-panel; then the outer
// block's U rows are solved block by block and the trailing matrix takes one
// update of depth NB.  The trailing matrix is read and written once per NB
// columns instead of once per nb, which at block depth 64 bounds the LU by HBM.
cudaError_t lu_two_level(const LuJob& j, int NB) {
  const int n = j.n, nb = j.nb;
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int KB = std::min(NB, n - k0);
    for (int j0 = 0; j0 < KB; j0 += nb) {
      const int kb = std::min(nb, KB - j0), kk = k0 + j0;
      BEM_TRY(lu_panel_cluster(j.prec, j.A, j.lda, j.strideA, n, kk, kb, nb, j.cl, j.batch, j.ipiv, j.info, j.stream,
                               j.rowmap));
      BEM_TRY(lu_swap_rows_batched(j.prec, j.A, j.lda, j.strideA, n, kk, kb, j.batch, j.rowmap, j.stream));
      if (j0 + kb < KB) {  // the rest of the outer block
        BEM_TRY(trsm_cols(j, kk, kb, kk + kb, k0 + KB));
        BEM_TRY(block_update(j, kk + kb, n - kk - kb, kk + kb, k0 + KB - kk - kb, kk, kb));
      }
    }
    if (k0 + KB < n) {
      // U rows of the outer block for the trailing columns: blocked forward substitution
      for (int i0 = 0; i0 < KB; i0 += nb) {
        const int kb = std::min(nb, KB - i0), kk = k0 + i0;
        BEM_TRY(trsm_cols(j, kk, kb, k0 + KB, n));
        if (i0 + kb < KB) BEM_TRY(block_update(j, kk + kb, k0 + KB - kk - kb, k0 + KB, n - k0 - KB, kk, kb));
      }
      BEM_TRY(block_update(j, k0 + KB, n - k0 - KB, k0 + KB, n - k0 - KB, k0, KB));
    }
  }
  return cudaGetLastError();
}

}  // namespace

int lu_launch_count(int n, int nb, int NB, bool tensor) {
  const int per_update = tensor ? 2 : 0;  // operand split + tcgen05 kernel (cuBLAS kernels are not counted)
  int count = 0;
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int KB = std::min(NB, n - k0);
    for (int j0 = 0; j0 < KB; j0 += nb) {
      const int kb = std::min(nb, KB - j0);
      count += 2;                                        // panel, row swaps
      if (j0 + kb < KB) count += 1 + (n - k0 - j0 - kb > 0 ? per_update : 0);
    }
    if (k0 + KB < n) {
      for (int i0 = 0; i0 < KB; i0 += nb) count += 1 + (i0 + std::min(nb, KB - i0) < KB ? per_update : 0);
      count += per_update;
    }
  }
  return count;
}

cudaError_t lu_factor_batched(Precision prec, void* A, long long lda, int n, int batch, int* ipiv, int* info, int nb,
                              void* cublas_handle, cudaStream_t stream, LuGemm gemm, void* tc_workspace,
                              bool* used_tensor, int** tc_err, int* rowmap, int* n_launches) {
  cublasHandle_t h = (cublasHandle_t)cublas_handle;
  cublasSetStream(h, stream);
  const long long strideA = lda * (long long)n;
  const bool mixed = prec == Precision::Mixed;
  const int want_nb = (nb == 32 || nb == 64) ? nb : 0;  // 0: automatic
  nb = nb > 0 ? std::min(nb, 64) : (mixed ? 64 : 32);
  const size_t esz = mixed ? sizeof(float2) : sizeof(double2);
  int cnb = 0, ccl = 0;
  const bool cluster_panel = lu_cluster_plan(prec, n, want_nb, batch, &cnb, &ccl);
  if (cluster_panel) nb = cnb;
  // tensor-core trailing update (mixed precision only; K = 2 nb <= 128)
  std::vector<unsigned char> plan_storage;
  TcGemmPlan* plan = nullptr;
  if (mixed && gemm != LuGemm::Cublas && tc_workspace && nb <= 64 && tc_gemm_available()) {
    plan_storage.resize(tc_gemm_plan_size());
    plan = reinterpret_cast<TcGemmPlan*>(plan_storage.data());
    if (!tc_gemm_plan(plan, tc_workspace, n, batch, (float2*)A, lda, nb)) plan = nullptr;
  }
  if (gemm == LuGemm::Tensor && mixed && !plan) return cudaErrorNotSupported;
  if (used_tensor) *used_tensor = plan != nullptr;
  if (plan) {
    if (tc_err) *tc_err = tc_gemm_error_word(plan);
    cudaMemsetAsync(tc_gemm_error_word(plan), 0, sizeof(int), stream);
  }
  // The two-level schedule serves the HBM-bound tcgen05 update; cuBLAS (the FP64
  // form, or lu_gemm = 1) keeps one level: its kernels for the skinny panel
  // shapes of the two-level schedule are slow.
  if (cluster_panel && rowmap && plan) {
    LuJob job{prec, A, lda, strideA, n, batch, nb, ccl, ipiv, info, rowmap, plan, h, stream};
    if (n_launches) *n_launches = lu_launch_count(n, nb, kOuterBlock, plan != nullptr);
    return lu_two_level(job, kOuterBlock);
  }
  if (n_launches) *n_launches = 0;
  for (int k = 0; k < n; k += nb) {
    const int kb = std::min(nb, n - k);
    if (n_launches) *n_launches += 2 + (n - k - kb > 0 ? 1 + (plan ? 2 : 0) : 0);
    if (cluster_panel) {
      cudaError_t e = lu_panel_cluster(prec, A, lda, strideA, n, k, kb, nb, ccl, batch, ipiv, info, stream, rowmap);
      if (e != cudaSuccess) return e;
    } else if (mixed)
      lu_panel_kernel<float><<<batch, 1024, 0, stream>>>((float2*)A, lda, strideA, n, k, kb, ipiv, info);
    else
      lu_panel_kernel<double><<<batch, 1024, 0, stream>>>((double2*)A, lda, strideA, n, k, kb, ipiv, info);
    if (n - kb > 0 && cluster_panel && rowmap) {
      cudaError_t e = lu_swap_rows_batched(prec, A, lda, strideA, n, k, kb, batch, rowmap, stream);
      if (e != cudaSuccess) return e;
    } else if (n - kb > 0) {
      dim3 g((n - kb + 127) / 128, batch);
      if (mixed)
        lu_swap_kernel<float2><<<g, 128, 0, stream>>>((float2*)A, lda, strideA, n, k, kb, ipiv);
      else
        lu_swap_kernel<double2><<<g, 128, 0, stream>>>((double2*)A, lda, strideA, n, k, kb, ipiv);
    }
    const int rest = n - k - kb;
    if (rest > 0) {
      const int tpb = 128;
      dim3 g((rest + tpb - 1) / tpb, batch);
      const size_t sm = (size_t)kb * kb * esz + (size_t)kb * (tpb + 1) * esz;
      if (mixed) {
        if (sm > 48 * 1024) ensure_smem_limit((const void*)lu_trsm_kernel<float2>, sm);
        lu_trsm_kernel<float2><<<g, tpb, sm, stream>>>((float2*)A, lda, strideA, n, k, kb, k + kb, n);
        if (plan) {
          cudaError_t e = tc_trailing_update(plan, (float2*)A, lda, strideA, n, k, kb, stream);
          if (e != cudaSuccess) return e;
          continue;
        }
        const cuComplex alpha = make_cuComplex(-1.f, 0.f), beta = make_cuComplex(1.f, 0.f);
        float2* base = (float2*)A;
        cublasStatus_t st = cublasCgemmStridedBatched(
            h, CUBLAS_OP_N, CUBLAS_OP_N, rest, rest, kb, &alpha, (const cuComplex*)(base + (k + kb) + (size_t)k * lda),
            (int)lda, strideA, (const cuComplex*)(base + k + (size_t)(k + kb) * lda), (int)lda, strideA, &beta,
            (cuComplex*)(base + (k + kb) + (size_t)(k + kb) * lda), (int)lda, strideA, batch);
        if (st != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
      } else {
        if (sm > 48 * 1024) ensure_smem_limit((const void*)lu_trsm_kernel<double2>, sm);
        lu_trsm_kernel<double2><<<g, tpb, sm, stream>>>((double2*)A, lda, strideA, n, k, kb, k + kb, n);
        const cuDoubleComplex alpha = make_cuDoubleComplex(-1.0, 0.0), beta = make_cuDoubleComplex(1.0, 0.0);
        double2* base = (double2*)A;
        cublasStatus_t st = cublasZgemmStridedBatched(
            h, CUBLAS_OP_N, CUBLAS_OP_N, rest, rest, kb, &alpha,
            (const cuDoubleComplex*)(base + (k + kb) + (size_t)k * lda), (int)lda, strideA,
            (const cuDoubleComplex*)(base + k + (size_t)(k + kb) * lda), (int)lda, strideA, &beta,
            (cuDoubleComplex*)(base + (k + kb) + (size_t)(k + kb) * lda), (int)lda, strideA, batch);
        if (st != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
      }
    }
  }
  return cudaGetLastError();
}

cudaError_t lu_solve_batched(Precision prec, const void* LU, long long lda, int n, int batch, const int* ipiv, void* B,
                             long long ldb, int nrhs, int /*nb*/, cudaStream_t stream) {
  const long long strideA = lda * (long long)n;
  if (prec == Precision::Mixed)
    lu_solve_kernel<float><<<batch * nrhs, 1024, 0, stream>>>((const float2*)LU, lda, strideA, n, ipiv, (float2*)B,
                                                             ldb, nrhs);
  else
    lu_solve_kernel<double><<<batch * nrhs, 1024, 0, stream>>>((const double2*)LU, lda, strideA, n, ipiv,
                                                              (double2*)B, ldb, nrhs);
  return cudaGetLastError();
}

cudaError_t residual_batched(Precision prec, const void* A, long long lda, int n, int batch, const double2* x,
                             const double2* b, long long ldb, int nrhs, double2* r, void* xsplit, cudaStream_t stream) {
  const long long strideA = lda * (long long)n;
  if (prec == Precision::Mixed) {
    const long long count = (long long)batch * nrhs * ldb;
    split_x_kernel<<<(unsigned)((count + 255) / 256), 256, 0, stream>>>(x, (float4*)xsplit, count);
    dim3 g((n + 63) / 64, batch * nrhs);
    residual_f32a_kernel<<<g, 256, 0, stream>>>((const float2*)A, lda, strideA, n, (const float4*)xsplit, b, ldb,
                                                 nrhs, r);
  } else {
    dim3 g((n + 255) / 256, batch * nrhs);
    residual_kernel<double2><<<g, 256, 0, stream>>>((const double2*)A, lda, strideA, n, x, b, ldb, nrhs, r);
  }
  return cudaGetLastError();
}

cudaError_t norms_batched(const double2* r, const double2* b, long long ldb, int n, int count, double* out,
                          cudaStream_t stream) {
  norms_kernel<<<count, 256, 0, stream>>>(r, b, ldb, n, out);
  return cudaGetLastError();
}

cudaError_t axpy_f32_into_f64(const float2* d, double2* x, long long n, cudaStream_t stream) {
  axpy_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(d, x, n);
  return cudaGetLastError();
}
cudaError_t convert_f64_to_f32(const double2* src, float2* dst, long long n, cudaStream_t stream) {
  f64_to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError();
}
cudaError_t convert_f32_to_f64(const float2* src, double2* dst, long long n, cudaStream_t stream) {
  f32_to_f64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError();
}

}  // namespace bem
