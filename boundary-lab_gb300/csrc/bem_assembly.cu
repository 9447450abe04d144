// Operator assembly kernels for the exterior Burton-Miller Galerkin P1/DP0
// Helmholtz BEM (sm_103a).
//
// The reference assembles four dense operators S, D, K', H with one CUDA
// thread per element pair and float atomics
// (src/blab/solvers/julia_local/src/BeatEngineCudaRegularKernels.jl:1-406,
// BeatEngineCudaSingular.jl:301-530), then forms the Burton-Miller matrix
// 1/2 M - D + eta H with a broadcast (BeatEngineCore.jl:1197).  Here one fused
// pass writes the requested linear combination  cD*D + cH*H + cM*M11  of the
// P1 x P1 operators straight into a column-major matrix, and the right-hand
// side  (cS*S + cK*K' + cM10*M10) q  is formed matrix-free from the driven
// faces only.  The integrands are those of the reference CPU pair integrals
// (BeatEngineCpuAssembly.jl:151-218 and 278-373).
//
// Data flow for one frequency:
//   regular_*_kernel      face pairs that share no vertex, 6x6 quadrature
//                         -> Rext[(g*3+b)][e]  (extended rows e, trial face g)
//   singular_dyn_kernel   vertex-sharing pairs (Duffy rules): k-dependent part,
//                         combined with the k-independent FP64 moments
//                         precomputed once per mesh -> per-pair 3x3 blocks
//   singular_scatter      adds the singular blocks into Rext (one thread per
//                         target entry, contributions in pair order:
//                         deterministic, no atomics)
//   gather_columns        A[:, j] = sum over (g, b) in star(j) of Rext[g*3+b],
//                         then halo extended rows folded into their rows
#include <complex>
#include <map>
#include <mutex>

#include "bem_common.cuh"
#include "bem_internal.h"
#include "bem_kernels.h"

namespace bem {

bool ensure_smem_limit(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> limit;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = limit[{dev, func}];
  if (bytes <= std::max<size_t>(cur, 48 * 1024)) return true;
  if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) return false;
  cur = bytes;
  return true;
}

namespace {

__device__ __forceinline__ double tr_sign_x(int tr) { return (tr & 1) ? -1.0 : 1.0; }
__device__ __forceinline__ double tr_sign_y(int tr) { return (tr & 2) ? -1.0 : 1.0; }

__device__ __forceinline__ bool share_vertex(const int* a, int b0, int b1, int b2) {
  return a[0] == b0 || a[0] == b1 || a[0] == b2 || a[1] == b0 || a[1] == b1 || a[1] == b2 || a[2] == b0 ||
         a[2] == b1 || a[2] == b2;
}

// ------------------------------------------------------------------------
// Regular pairs, compensated FP32.
//
// Phase: k*r is split as k*|C| + k*(r - |C|), C = anchor_g - anchor_f.  The
// first term is formed in double-float once per pair and reduced mod 2pi; the
// second is small (|r - |C|| <= element size) and is computed in FP32 from
// r - |C| = (2 C.d + d.d) / (r + |C|), d = off_g - off_f, which has no
// cancellation.  Plain FP32 k*r loses ~kr * 6e-8 rad; this keeps the phase
// error near 1e-7 rad for any kr.
// ------------------------------------------------------------------------
struct PairF32 {
  float Cf[3];   // C rounded to float
  float R0;      // |C| rounded to float
  float theta0;  // k|C| mod 2pi
};

__device__ __forceinline__ PairF32 pair_setup_f32(const float* ahi_g, const float* alo_g, const float* ahi_f,
                                                  const float* alo_f, df kdf) {
  PairF32 P;
  df C[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    df s = two_sum(ahi_g[d], -ahi_f[d]);
    s.lo += alo_g[d] - alo_f[d];
    C[d] = quick_two_sum(s.hi, s.lo);
    P.Cf[d] = C[d].hi + C[d].lo;
  }
  df r2 = df_add(df_add(df_mul(C[0], C[0]), df_mul(C[1], C[1])), df_mul(C[2], C[2]));
  df R = df_sqrt(r2);
  P.R0 = R.hi + R.lo;
  P.theta0 = df_reduce_two_pi(df_mul(kdf, R));
  return P;
}

// Green's function and the radial factor of its gradient at one q-pair
// (points never coincide for the pairs this is used on).
__device__ __forceinline__ void green_f32(const PairF32& P, const float* d, float k, float& rinv, float rv[3],
                                          float2& G) {
  rv[0] = P.Cf[0] + d[0];
  rv[1] = P.Cf[1] + d[1];
  rv[2] = P.Cf[2] + d[2];
  float r2 = fmaf(rv[0], rv[0], fmaf(rv[1], rv[1], rv[2] * rv[2]));
  rinv = r2 > 1e-30f ? rsqrt_ftz(r2) : 0.0f;
  float r = r2 * rinv;
  float cd = fmaf(P.Cf[0], d[0], fmaf(P.Cf[1], d[1], P.Cf[2] * d[2]));
  float dd = fmaf(d[0], d[0], fmaf(d[1], d[1], d[2] * d[2]));
  float den = fmaxf(r + P.R0, 1e-30f);
  float delta = fmaf(2.0f, cd, dd) * rcp_ftz(den);
  float theta = reduce_two_pi(fmaf(k, delta, P.theta0));
  float s, c;
  sincos_ftz(theta, &s, &c);
  float sc = rinv * BEM_INV_FOUR_PI;
  G = make_float2(c * sc, s * sc);
}

// Frequency-independent part of the pair set-up: C = anchor_g - anchor_f in
// double-float, Cf = C rounded to float, and |C| as double-float.
struct PairGeomF32 {
  float Cf[3];
  df R;
};

__device__ __forceinline__ PairGeomF32 pair_geom_f32(const float* ahi_g, const float* alo_g, const float* ahi_f,
                                                     const float* alo_f) {
  PairGeomF32 P;
  df C[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    df s = two_sum(ahi_g[d], -ahi_f[d]);
    s.lo += alo_g[d] - alo_f[d];
    C[d] = quick_two_sum(s.hi, s.lo);
    P.Cf[d] = C[d].hi + C[d].lo;
  }
  P.R = df_sqrt(df_add(df_add(df_mul(C[0], C[0]), df_mul(C[1], C[1])), df_mul(C[2], C[2])));
  return P;
}

// Parameters of one regular-assembly launch over NFQ frequencies (kernel
// parameters, so meshes with different rules run concurrently on different
// streams).  cw[a*Q + q] = phi_a(xi_q) * w_q of the regular rule; w_q = sum_a cw.
template <int NFQ, bool DT> struct RegParamsF32 {
  float2 cw2[3 * kMaxQ];  // (cw, cw) at [a*Q + q]: operand pairs of the packed FP32x2 FMAs
  float2 w2[kMaxQ];       // (w, w)
  float2 cwp[3][kMaxQ];   // (cw, cw) at [b][n], zero for the padding point of an odd rule
  float2 wp[kMaxQ];       // (w, w) at [n], zero for the padding point
  df kdf[NFQ];     // wavenumbers as double-float
  float k[NFQ], k2[NFQ];
  float2 cHn[NFQ];  // cH / cD (cH when the launch has no double-layer term)
  float2 cDn[NFQ];  // cD (1 when the launch has no double-layer term)
  float2 cH[NFQ];
};

// Regular face pairs for NFQ frequencies at once.  Per q-pair (test point m,
// trial point n) the frequency-independent part (r, 1/r, the compensated
// r - |C|, t = (r . n_g) / r, t / r, t / r^2) is formed once, then per
// frequency the phase kr and
//   H = e^{ikr} E'',  E'' = (1/r) (t (ik - 1/r) + cnn'),  cnn' = -k^2 (n_f . n_g) cH / cD,
// so that cD H = G (cD t (ik - 1/r) - k^2 nn cH), G = e^{ikr} / r: the
// double-layer kernel times cD plus the -k^2 nn cH part of the hypersingular
// kernel in one complex weight.  Per test point the trial-basis sums
// Hs[b] = sum_n cw[b][n] H and Gs = sum_n w_n G are folded into
// W[a][b] += cw[a][m] Hs[b] and S0 += w_m Gs, and each pair adds
//   jac * (cD W[a][b] + (curl_a . curl_b) cH S0)
// (BeatEngineCpuAssembly.jl:278-373: the D and H regular integrals, with
// S0 = sum_{a,b} of the single-layer integrals of the basis products, because
// the P1 basis functions sum to one).  DT = false (cD = 0) drops the
// double-layer term: E'' = cnn / r, with cH in place of cH / cD.
//
// The phase kr = k|C| + k(r - |C|) is taken in radians without a per-q-pair
// reduction: k|C| is reduced mod 2pi per pair in double-float and
// |k(r - |C|)| <= k h (h the element size), so |kr| stays a few pi at most
// for any mesh that resolves the wavelength.
// Resident CTAs per SM the regular kernel is compiled for: three with up to two
// frequencies per launch (<= 168 registers), two with three or four (<= 255
// registers; the per-warp accumulators of four frequencies take 112 KB per CTA
// on 291-row tiles, so two CTAs still fit in shared memory).
template <int NFQ> struct RegularOccupancy {
  static constexpr int kCtasPerSm = NFQ <= 2 ? 3 : 2;
};

template <int Q, int WARPS, int NFQ, bool DT>
__global__ void __launch_bounds__(WARPS * 32, RegularOccupancy<NFQ>::kCtasPerSm)
    regular_f32_kernel(const FaceF32* __restrict__ faces, int nf, const int* __restrict__ tile_group_ptr,
                       const LaneSlot* __restrict__ slots, const float* __restrict__ group_faces,
                       const int* __restrict__ tile_row_base, int max_rows,
                       float2* __restrict__ Rext, long long ldR, long long strideR, RegParamsF32<NFQ, DT> p, int ntr,
                       int4 trs, const unsigned char* __restrict__ fix_mask) {
  extern __shared__ float2 smem_acc32[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.y;
  const int g = blockIdx.x * WARPS + warp;
  const int base = tile_row_base[tile];
  const int rows = tile_row_base[tile + 1] - base;
  float2* acc = smem_acc32 + (size_t)warp * NFQ * 3 * max_rows;  // [NFQ][3][max_rows]
  // rule coefficients of the (not unrolled) test-point loop, indexed at run time
  __shared__ float2 s_cw2[3 * kMaxQ], s_w2[kMaxQ];
  if (threadIdx.x < 3 * kMaxQ) s_cw2[threadIdx.x] = p.cw2[threadIdx.x];
  if (threadIdx.x < kMaxQ) s_w2[threadIdx.x] = p.w2[threadIdx.x];
  for (int i = lane; i < NFQ * 3 * max_rows; i += 32) acc[i] = make_float2(0.0f, 0.0f);
  __syncthreads();
  if (g >= nf) return;

  // trial face (warp-uniform): quadrature offsets og[n] with og.og and og.n_g
  const FaceF32& T = faces[g];
  // Trial points are taken two at a time (n = 2j, 2j + 1) in the lanes of
  // packed FP32x2 registers; an odd rule is padded with the centroid at zero
  // weight.
  constexpr int NP = (Q + 1) / 2;
  float ahi_g[3], alo_g[3], ng[3], cg[9];
  float2 ogp[NP][3], ggp[NP], ngnp[NP];  // offsets, og.og, -og.n_g
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ahi_g[d] = T.anchor_hi[d];
    alo_g[d] = T.anchor_lo[d];
    ng[d] = T.normal[d];
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) cg[i] = T.curls[i];
#pragma unroll
  for (int j = 0; j < NP; ++j) {
    float o[2][3], gg[2], gn[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int n = 2 * j + e;
#pragma unroll
      for (int d = 0; d < 3; ++d) o[e][d] = n < Q ? T.off[3 * n + d] : 0.0f;
      gg[e] = fmaf(o[e][0], o[e][0], fmaf(o[e][1], o[e][1], o[e][2] * o[e][2]));
      gn[e] = fmaf(o[e][0], ng[0], fmaf(o[e][1], ng[1], o[e][2] * ng[2]));
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) ogp[j][d] = make_float2(o[0][d], o[1][d]);
    ggp[j] = make_float2(gg[0], gg[1]);
    ngnp[j] = make_float2(-gn[0], -gn[1]);
  }
  const float a2g = T.area2;
  const int gv0 = T.verts[0], gv1 = T.verts[1], gv2 = T.verts[2];

  // Symmetry images of the trial face (BeatEngineCpuAssembly.jl:411-445): the
  // same test faces against the reflected trial face, added to the same trial
  // columns.  The trial data are reflected in place from one transform to the
  // next; pairs whose faces touch on the reflecting planes are left to the
  // singular (Duffy) pass, like vertex-sharing pairs of the identity.
  int prev_tr = 0;
  for (int ti = 0; ti < ntr; ++ti) {
    const int tr = ti == 0 ? trs.x : ti == 1 ? trs.y : ti == 2 ? trs.z : trs.w;
    {
      const int dlt = tr ^ prev_tr;
      const float fx = (dlt & 1) ? -1.f : 1.f, fy = (dlt & 2) ? -1.f : 1.f, dr = fx * fy;
      ahi_g[0] *= fx;
      ahi_g[1] *= fy;
      alo_g[0] *= fx;
      alo_g[1] *= fy;
      ng[0] *= fx;
      ng[1] *= fy;
#pragma unroll
      for (int j = 0; j < NP; ++j) {  // og.og and og.n_g are unchanged by a reflection
        ogp[j][0] = __fmul2_rn(ogp[j][0], make_float2(fx, fx));
        ogp[j][1] = __fmul2_rn(ogp[j][1], make_float2(fy, fy));
      }
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        cg[3 * b] *= fx * dr;
        cg[3 * b + 1] *= fy * dr;
        cg[3 * b + 2] *= dr;
      }
      prev_tr = tr;
    }
    const int sv0 = (tr == 0 || (fix_mask[gv0] & tr) == tr) ? gv0 : -2;
    const int sv1 = (tr == 0 || (fix_mask[gv1] & tr) == tr) ? gv1 : -2;
    const int sv2 = (tr == 0 || (fix_mask[gv2] & tr) == tr) ? gv2 : -2;

  // Software pipeline over the lane groups: the slot of group grp + 2 and the
  // face header (vertices, anchor) of group grp + 1 are loaded while group grp
  // is integrated, so the pair set-up never waits on a global load.  The test
  // faces of a group are stored field-major (group_faces[grp][word][lane], the
  // words of FaceF32), so every field load of the warp is one 128-byte line.
  const int g0 = tile_group_ptr[tile], g1 = tile_group_ptr[tile + 1];
  LaneSlot s_next{-1, {0, 0, 0}}, s_cur{-1, {0, 0, 0}};
  int hv[3] = {-1, -1, -1};
  float hhi[3] = {0.f, 0.f, 0.f}, hlo[3] = {0.f, 0.f, 0.f};
  auto load_head = [&](int grp) {
    const float* H = group_faces + (size_t)grp * kFaceWords * 32 + lane;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      hv[d] = __float_as_int(H[(kFwVerts + d) * 32]);
      hhi[d] = H[(kFwAnchorHi + d) * 32];
      hlo[d] = H[(kFwAnchorLo + d) * 32];
    }
  };
  if (g0 < g1) {
    s_cur = slots[(size_t)g0 * 32 + lane];
    load_head(g0);
  }
  if (g0 + 1 < g1) s_next = slots[(size_t)(g0 + 1) * 32 + lane];
  for (int grp = g0; grp < g1; ++grp) {
    const LaneSlot s = s_cur;
    const int fv[3] = {hv[0], hv[1], hv[2]};
    const float ahi_f[3] = {hhi[0], hhi[1], hhi[2]}, alo_f[3] = {hlo[0], hlo[1], hlo[2]};
    if (grp + 1 < g1) {
      s_cur = s_next;
      load_head(grp + 1);
    }
    if (grp + 2 < g1) s_next = slots[(size_t)(grp + 2) * 32 + lane];
    if (s.face >= 0) {
      const float* F = group_faces + (size_t)grp * kFaceWords * 32 + lane;  // this lane's test face: word w at F[32 w]
      if (!share_vertex(fv, sv0, sv1, sv2)) {
        // With C = anchor_g - anchor_f, x_n = anchor_g + og[n], y_m = anchor_f + of[m]
        // and d = og[n] - of[m]:  r = |C + d|, and
        //   r - |C| = (2 C.d + d.d) / (r + |C|),
        //   2 C.d + d.d = Pg[n] + Pf[m] - 2 og[n].of[m],
        //   Pg[n] = 2 C.og[n] + og[n].og[n],  Pf[m] = of[m].of[m] - 2 C.of[m],
        // every term of size |C| h or h^2 (no cancellation against |C|^2).
        const PairGeomF32 P = pair_geom_f32(ahi_g, alo_g, ahi_f, alo_f);
        const float R0 = fmaxf(P.R.hi + P.R.lo, 1e-30f);
        float2 Pgp[NP];  // 2 C.og + og.og
        {
          const float2 c0 = make_float2(2.0f * P.Cf[0], 2.0f * P.Cf[0]);
          const float2 c1 = make_float2(2.0f * P.Cf[1], 2.0f * P.Cf[1]);
          const float2 c2 = make_float2(2.0f * P.Cf[2], 2.0f * P.Cf[2]);
#pragma unroll
          for (int j = 0; j < NP; ++j)
            Pgp[j] = __ffma2_rn(c0, ogp[j][0], __ffma2_rn(c1, ogp[j][1], __ffma2_rn(c2, ogp[j][2], ggp[j])));
        }
        const float2 R0p = make_float2(R0, R0);
        // test-face data
        const float nn =
            fmaf(F[32 * kFwNormal], ng[0], fmaf(F[32 * (kFwNormal + 1)], ng[1], F[32 * (kFwNormal + 2)] * ng[2]));
        const float jac = F[32 * kFwArea2] * a2g * BEM_INV_FOUR_PI;
        float2 th0[NFQ];            // k|C| mod 2pi in [-pi, pi], both lanes
        float2 cnnx[NFQ], cnny[NFQ];  // cnn' = -k^2 nn cHn, each part in both lanes
        float2 W[NFQ][3][3], S0[NFQ];
#pragma unroll
        for (int f = 0; f < NFQ; ++f) {
          const float th = df_reduce_two_pi(df_mul(p.kdf[f], P.R));
          th0[f] = make_float2(th, th);
          const float s = -p.k2[f] * nn;
          cnnx[f] = make_float2(s * p.cHn[f].x, s * p.cHn[f].x);
          cnny[f] = make_float2(s * p.cHn[f].y, s * p.cHn[f].y);
          S0[f] = make_float2(0.f, 0.f);
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) W[f][a][b] = make_float2(0.f, 0.f);
        }
        // The test-point loop is kept rolled: fully unrolling 6 x 6 Green
        // evaluations overflowed the instruction cache (no_instruction stalls).
        const float* Foff = F + 32 * kFwOff;
        float nf0 = Foff[0], nf1 = Foff[32], nf2 = Foff[64];
#pragma unroll 1
        for (int m = 0; m < Q; ++m) {
          const float f0 = nf0, f1 = nf1, f2 = nf2;
          {  // offsets of test point m + 1, consumed in the next iteration
            const int mn = m + 1 < Q ? m + 1 : m;
            nf0 = Foff[96 * mn];
            nf1 = Foff[96 * mn + 32];
            nf2 = Foff[96 * mn + 64];
          }
          const float cm0 = P.Cf[0] - f0, cm1 = P.Cf[1] - f1, cm2 = P.Cf[2] - f2;
          const float Pf = fmaf(-2.0f, fmaf(P.Cf[0], f0, fmaf(P.Cf[1], f1, P.Cf[2] * f2)),
                                fmaf(f0, f0, fmaf(f1, f1, f2 * f2)));
          const float ncmn = -fmaf(cm0, ng[0], fmaf(cm1, ng[1], cm2 * ng[2]));
          const float2 cm0p = make_float2(cm0, cm0), cm1p = make_float2(cm1, cm1), cm2p = make_float2(cm2, cm2);
          const float2 m2f0 = make_float2(-2.0f * f0, -2.0f * f0), m2f1 = make_float2(-2.0f * f1, -2.0f * f1),
                       m2f2 = make_float2(-2.0f * f2, -2.0f * f2);
          const float2 Pfp = make_float2(Pf, Pf), ncmnp = make_float2(ncmn, ncmn);
          float2 Hs[NFQ][3], Gs[NFQ];
#pragma unroll
          for (int f = 0; f < NFQ; ++f) {
            Gs[f] = make_float2(0.f, 0.f);
#pragma unroll
            for (int b = 0; b < 3; ++b) Hs[f][b] = make_float2(0.f, 0.f);
          }
#pragma unroll
          for (int j = 0; j < NP; ++j) {
            // frequency-independent, two trial points per instruction: r vector
            // y_m -> x_n, 1/r, r - |C|, -t = -(r . n_g) / r, -t / r, -t / r^2, w / r
            const float2 r0 = __fadd2_rn(cm0p, ogp[j][0]), r1 = __fadd2_rn(cm1p, ogp[j][1]),
                         r2v = __fadd2_rn(cm2p, ogp[j][2]);
            float2 r2 = __ffma2_rn(r0, r0, __ffma2_rn(r1, r1, __fmul2_rn(r2v, r2v)));
            r2 = make_float2(fmaxf(r2.x, 1e-30f), fmaxf(r2.y, 1e-30f));
            const float2 rinv = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
            const float2 num =
                __ffma2_rn(ogp[j][0], m2f0, __ffma2_rn(ogp[j][1], m2f1, __ffma2_rn(ogp[j][2], m2f2, __fadd2_rn(Pgp[j], Pfp))));
            const float2 den = __ffma2_rn(r2, rinv, R0p);
            const float2 delta = __fmul2_rn(num, make_float2(rcp_ftz(den.x), rcp_ftz(den.y)));
            const float2 nt = __fmul2_rn(__fadd2_rn(ncmnp, ngnp[j]), rinv);
            const float2 ntr = __fmul2_rn(nt, rinv);
            const float2 ntrr = __fmul2_rn(ntr, rinv);
            const float2 wr = __fmul2_rn(make_float2(p.wp[2 * j].x, p.wp[2 * j + 1].x), rinv);
#pragma unroll
            for (int f = 0; f < NFQ; ++f) {
              const float2 th = __ffma2_rn(make_float2(p.k[f], p.k[f]), delta, th0[f]);  // kr - 2 pi n
              // E'' = (-t/r^2 + cnn'.x / r, k t / r + cnn'.y / r)
              float2 Ex, Ey;
              if (DT) {
                Ex = __ffma2_rn(rinv, cnnx[f], ntrr);
                Ey = __ffma2_rn(rinv, cnny[f], __fmul2_rn(make_float2(-p.k[f], -p.k[f]), ntr));
              } else {
                Ex = __fmul2_rn(rinv, cnnx[f]);
                Ey = __fmul2_rn(rinv, cnny[f]);
              }
#pragma unroll
              for (int e = 0; e < 2; ++e) {
                const int n = 2 * j + e;
                const float ex = e ? Ex.y : Ex.x, ey = e ? Ey.y : Ey.x, w = e ? wr.y : wr.x;
                float sn, cs;
                sincos_ftz(e ? th.y : th.x, &sn, &cs);
                const float2 H = make_float2(fmaf(cs, ex, -sn * ey), fmaf(cs, ey, sn * ex));  // e^{ikr} E''
#pragma unroll
                for (int b = 0; b < 3; ++b) Hs[f][b] = __ffma2_rn(p.cwp[b][n], H, Hs[f][b]);
                Gs[f] = __ffma2_rn(make_float2(w, w), make_float2(cs, sn), Gs[f]);  // w e^{ikr} / r
              }
            }
          }
#pragma unroll
          for (int f = 0; f < NFQ; ++f) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              const float2 c = s_cw2[a * Q + m];
#pragma unroll
              for (int b = 0; b < 3; ++b) W[f][a][b] = __ffma2_rn(c, Hs[f][b], W[f][a][b]);
            }
            S0[f] = __ffma2_rn(s_w2[m], Gs[f], S0[f]);
          }
        }
        // L[a][b] = jac (cD W[a][b] + (curl_a . curl_b) cH S0)
        float2 Bc[NFQ];
#pragma unroll
        for (int f = 0; f < NFQ; ++f) {
          Bc[f] = cmul(p.cH[f], S0[f]);
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) W[f][a][b] = cmul(p.cDn[f], W[f][a][b]);
        }
        const float2 jj = make_float2(jac, jac);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float cf0 = F[32 * (kFwCurls + 3 * a)], cf1 = F[32 * (kFwCurls + 3 * a + 1)],
                      cf2 = F[32 * (kFwCurls + 3 * a + 2)];
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            const float cc = jac * fmaf(cf0, cg[3 * b], fmaf(cf1, cg[3 * b + 1], cf2 * cg[3 * b + 2]));
#pragma unroll
            for (int f = 0; f < NFQ; ++f) {
              float2* dst = &acc[(f * 3 + b) * max_rows + s.loc[a]];
              *dst = __fadd2_rn(*dst, __ffma2_rn(jj, W[f][a][b], __fmul2_rn(make_float2(cc, cc), Bc[f])));
            }
          }
        }
      }
    }
    __syncwarp();
  }
  }  // symmetry transforms
  // write this warp's extended-row segments: three per frequency
  for (int i = lane; i < NFQ * 3 * rows; i += 32) {
    const int fb = i / rows, loc = i - fb * rows;
    const int f = fb / 3, b = fb - 3 * f;
    Rext[(size_t)f * strideR + (size_t)(3 * g + b) * ldR + base + loc] = acc[fb * max_rows + loc];
  }
}

// ------------------------------------------------------------------------
// Regular pairs, FP64 (the plain FP64 form).
// ------------------------------------------------------------------------
struct RegParamsF64 {
  double k, k2;
  double2 cD, cH;
  double cw[3 * kMaxQ];
};

template <int Q, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) regular_f64_kernel(const FaceF64* __restrict__ faces, int nf,
                                                                 const int* __restrict__ tile_group_ptr,
                                                                 const LaneSlot* __restrict__ slots,
                                                                 const int* __restrict__ tile_row_base,
                                                                 int max_rows, double2* __restrict__ Rext,
                                                                 long long ldR, RegParamsF64 p, int ntr, int4 trs,
                                                                 const unsigned char* __restrict__ fix_mask) {
  extern __shared__ double2 smem_acc64[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.y;
  const int g = blockIdx.x * WARPS + warp;
  const int base = tile_row_base[tile];
  const int rows = tile_row_base[tile + 1] - base;
  double2* acc = smem_acc64 + (size_t)warp * 3 * max_rows;
  for (int i = lane; i < 3 * max_rows; i += 32) acc[i] = make_double2(0.0, 0.0);
  __syncwarp();
  if (g >= nf) return;
  const FaceF64& T = faces[g];
  double ag[3], ng[3], og[Q][3], cg[9];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ag[d] = T.anchor[d];
    ng[d] = T.normal[d];
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) cg[i] = T.curls[i];
#pragma unroll
  for (int n = 0; n < Q; ++n)
#pragma unroll
    for (int d = 0; d < 3; ++d) og[n][d] = T.off[3 * n + d];
  const double a2g = T.area2;
  const int gv0 = T.verts[0], gv1 = T.verts[1], gv2 = T.verts[2];
  const int g0 = tile_group_ptr[tile], g1 = tile_group_ptr[tile + 1];
  int prev_tr = 0;
  for (int ti = 0; ti < ntr; ++ti) {  // symmetry images, as in regular_f32_kernel
    const int tr = ti == 0 ? trs.x : ti == 1 ? trs.y : ti == 2 ? trs.z : trs.w;
    {
      const int dlt = tr ^ prev_tr;
      const double fx = (dlt & 1) ? -1.0 : 1.0, fy = (dlt & 2) ? -1.0 : 1.0, dr = fx * fy;
      ag[0] *= fx;
      ag[1] *= fy;
      ng[0] *= fx;
      ng[1] *= fy;
#pragma unroll
      for (int n = 0; n < Q; ++n) {
        og[n][0] *= fx;
        og[n][1] *= fy;
      }
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        cg[3 * b] *= fx * dr;
        cg[3 * b + 1] *= fy * dr;
        cg[3 * b + 2] *= dr;
      }
      prev_tr = tr;
    }
    const int sv0 = (tr == 0 || (fix_mask[gv0] & tr) == tr) ? gv0 : -2;
    const int sv1 = (tr == 0 || (fix_mask[gv1] & tr) == tr) ? gv1 : -2;
    const int sv2 = (tr == 0 || (fix_mask[gv2] & tr) == tr) ? gv2 : -2;
  for (int grp = g0; grp < g1; ++grp) {
    const LaneSlot s = slots[(size_t)grp * 32 + lane];
    if (s.face >= 0) {
      const FaceF64& F = faces[s.face];
      int fv[3] = {F.verts[0], F.verts[1], F.verts[2]};
      if (!share_vertex(fv, sv0, sv1, sv2)) {
        double C[3] = {ag[0] - F.anchor[0], ag[1] - F.anchor[1], ag[2] - F.anchor[2]};
        double2 IG[3][3], ID[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            IG[a][b] = make_double2(0., 0.);
            ID[a][b] = make_double2(0., 0.);
          }
#pragma unroll 1
        for (int m = 0; m < Q; ++m) {
          const double of[3] = {F.off[3 * m], F.off[3 * m + 1], F.off[3 * m + 2]};
          double2 u[3], v[3];
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            u[b] = make_double2(0., 0.);
            v[b] = make_double2(0., 0.);
          }
#pragma unroll
          for (int n = 0; n < Q; ++n) {
            const double rv[3] = {C[0] + (og[n][0] - of[0]), C[1] + (og[n][1] - of[1]), C[2] + (og[n][2] - of[2])};
            const double r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
            if (r2 == 0.0) continue;
            const double r = sqrt(r2);
            const double rinv = 1.0 / r;
            double s, c;
            sincos(p.k * r, &s, &c);
            const double sc = rinv * (0.25 / CUDART_PI);
            const double2 G = make_double2(c * sc, s * sc);
            const double t = (rv[0] * ng[0] + rv[1] * ng[1] + rv[2] * ng[2]) * rinv;
            const double2 Dk = make_double2(t * (-G.x * rinv - G.y * p.k), t * (G.x * p.k - G.y * rinv));
#pragma unroll
            for (int b = 0; b < 3; ++b) {
              const double cw = p.cw[b * Q + n];
              u[b].x += cw * G.x;
              u[b].y += cw * G.y;
              v[b].x += cw * Dk.x;
              v[b].y += cw * Dk.y;
            }
          }
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const double cw = p.cw[a * Q + m];
#pragma unroll
            for (int b = 0; b < 3; ++b) {
              IG[a][b].x += cw * u[b].x;
              IG[a][b].y += cw * u[b].y;
              ID[a][b].x += cw * v[b].x;
              ID[a][b].y += cw * v[b].y;
            }
          }
        }
        double2 S0 = make_double2(0., 0.);
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) S0 = cadd(S0, IG[a][b]);
        const double nn = F.normal[0] * ng[0] + F.normal[1] * ng[1] + F.normal[2] * ng[2];
        const double jac = F.area2 * a2g;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            const double cc = F.curls[3 * a] * cg[3 * b] + F.curls[3 * a + 1] * cg[3 * b + 1] +
                              F.curls[3 * a + 2] * cg[3 * b + 2];
            double2 H = make_double2(cc * S0.x - p.k2 * nn * IG[a][b].x, cc * S0.y - p.k2 * nn * IG[a][b].y);
            double2 L = cadd(cmul(p.cD, ID[a][b]), cmul(p.cH, H));
            double2* dst = &acc[b * max_rows + s.loc[a]];
            double2 o = *dst;
            o.x += jac * L.x;
            o.y += jac * L.y;
            *dst = o;
          }
        }
      }
    }
    __syncwarp();
  }
  }  // symmetry transforms
  for (int i = lane; i < 3 * rows; i += 32) {
    const int b = i / rows, loc = i - b * rows;
    Rext[(size_t)(3 * g + b) * ldR + base + loc] = acc[b * max_rows + loc];
  }
}

// ------------------------------------------------------------------------
// Singular (vertex-sharing) pairs.
//
// The Green's function is split into a k-independent singular part and a
// smooth k-dependent remainder, both integrated with the same Duffy points:
//   G            = s + R,                 s = 1/(4 pi r),  R = s (e^{ikr} - 1)
//   dG/dn_y      = -(r.n_y) s / r^2 + h(kr) (r.n_y) s / r^2
//   adjoint      = +(r.n_x) s / r^2 - h(kr) (r.n_x) s / r^2
//   h(z)         = e^{iz}(iz - 1) + 1 = (1 - cos z - z sin z) + i (z cos z - sin z)
// The k-independent moments are integrated once per mesh in FP64; the
// remainder is integrated per frequency (FP32 in the mixed form, FP64 in the
// plain form).  The sum is the reference's Duffy quadrature of the full kernel
// (BeatEngineCpuAssembly.jl:151-218) up to rounding.
//
// Static moments per pair (24 doubles, all times jac):
//   [0..2]  SG0[a] = sum w phi_a(x) s
//   [3..11] IG0[a][b] = sum w phi_a(x) phi_b(y) s
//   [12..20] ID0[a][b] = sum w phi_a phi_b (-(r.n_y) s / r^2)
//   [21..23] IK0[a] = sum w phi_a(x) (+(r.n_x) s / r^2)
// ------------------------------------------------------------------------
constexpr int kStatic = 24;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct SingularGeom {
  const double* verts;  // nv x 3
  const int* faces;     // nf x 3
  const double* normal;
};

// Per-pair record of the mixed form (kPairRec floats), written once per mesh by
// the moments kernel below so that the per-frequency FP32 singular kernel runs
// no FP64 instruction (on this part the FP64 pipe, not FP32, limited it):
//   [0..20]  e1t, e2t, d0, e1r, e2r, n_test, n_trial (3 each; the trial side
//            reflected for image pairs), each rounded from its FP64 value
//   [21] jac   [22] n_test . (S n_trial)   [23] 2 A_test
//   [24..32] curl_a(test) . curl_b(trial image), a-major, summed in FP64
//   [33] SG0[0] + SG0[1] + SG0[2] (FP64 sum)   [34..57] the 24 static moments
constexpr int kRecGeom = 0, kRecJac = 21, kRecNprod = 22, kRecA2 = 23, kRecCurl = 24, kRecS0 = 33, kRecMom = 34;
static_assert(kRecMom + kStatic <= kPairRec, "pair record layout");

// Double-float helpers of the moments kernel.
__device__ __forceinline__ df to_df(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }
// 1 / sqrt(a) for a > 0: one Newton step in double-float on the FP32 approximate
// reciprocal root (relative error about 2^-44).
__device__ __forceinline__ df df_rsqrt(df a) {
  const float y = rsqrt_ftz(a.hi);
  const df y2 = two_prod(y, y);
  const df ay2 = df_mul(a, y2);
  const df res = df_sub(df{1.0f, 0.0f}, ay2);  // about 2^-22
  return quick_two_sum(y, 0.5f * y * res.hi);
}

// Pair setup (one thread per pair, FP64): the pair's geometry as double-float
// for the moments kernel, and the FP32 record fields that do not depend on the
// moments (geometry, jac, n_t . S n_r, 2 A_test, curl products).
//   pairgeo_df[p]: e1t e2t d0 e1r e2r n_test n_trial (21 double-floats = 42
//   floats), jac (2 floats), padding.
__global__ void pair_setup_kernel(SingularGeom geo, const SingularPair* __restrict__ pairs, int npairs,
                                  const double* __restrict__ curls, const double* __restrict__ area,
                                  float* __restrict__ geo_df, float* __restrict__ rec) {
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid >= npairs) return;
  const SingularPair P = pairs[pid];
  const int* ft = geo.faces + 3 * P.test;
  const int* fr = geo.faces + 3 * P.trial;
  double g[21];
  for (int d = 0; d < 3; ++d) {
    // image pairs: the trial face reflected by P.tr (points and normal S p)
    const double sd = d == 0 ? tr_sign_x(P.tr) : d == 1 ? tr_sign_y(P.tr) : 1.0;
    const double t0 = geo.verts[3 * ft[0] + d];
    const double r0 = sd * geo.verts[3 * fr[0] + d];
    g[d] = geo.verts[3 * ft[1] + d] - t0;            // e1t
    g[3 + d] = geo.verts[3 * ft[2] + d] - t0;        // e2t
    g[6 + d] = r0 - t0;                               // d0
    g[9 + d] = sd * geo.verts[3 * fr[1] + d] - r0;    // e1r
    g[12 + d] = sd * geo.verts[3 * fr[2] + d] - r0;   // e2r
    g[15 + d] = geo.normal[3 * P.test + d];           // n_test
    g[18 + d] = sd * geo.normal[3 * P.trial + d];     // n_trial (reflected)
  }
  float* G = geo_df + (size_t)kPairGeoDf * pid;
  float* o = rec + (size_t)kPairRec * pid;
  for (int i = 0; i < 21; ++i) {
    const df v = to_df(g[i]);
    G[2 * i] = v.hi;
    G[2 * i + 1] = v.lo;
    o[kRecGeom + i] = v.hi;
  }
  const df jd = to_df(P.jac);
  G[42] = jd.hi;
  G[43] = jd.lo;
  for (int i = 44; i < kPairGeoDf; ++i) G[i] = 0.0f;
  o[kRecJac] = (float)P.jac;
  o[kRecNprod] = (float)P.nprod;
  o[kRecA2] = (float)(2.0 * area[P.test]);
  const double* ct = curls + 9 * (size_t)P.test;
  const double* cr0 = curls + 9 * (size_t)P.trial;
  const double sx = tr_sign_x(P.tr), sy = tr_sign_y(P.tr), det = sx * sy;
  double cr[9];  // reflected trial curls det(S) S c
  for (int b = 0; b < 3; ++b) {
    cr[3 * b] = det * sx * cr0[3 * b];
    cr[3 * b + 1] = det * sy * cr0[3 * b + 1];
    cr[3 * b + 2] = det * cr0[3 * b + 2];
  }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      o[kRecCurl + 3 * a + b] =
          (float)(ct[3 * a] * cr[3 * b] + ct[3 * a + 1] * cr[3 * b + 1] + ct[3 * a + 2] * cr[3 * b + 2]);
  for (int i = kRecMom + kStatic; i < kPairRec; ++i) o[i] = 0.0f;
}

// Compensated accumulation in the style of Dot2 (Ogita, Rump and Oishi, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 26, 2005): a double-float
// accumulator whose high part takes each term through two-sum and whose low part
// sums the rounding errors and the terms' low parts in plain FP32.  A term is a
// double-float value or the exact product of two (two-product of the high parts
// plus the cross terms), so a term costs 8 or 12 FP32 instructions instead of the
// 20 of a df_add (27 with the df_mul before it); the low part is folded back by
// two-sum every few terms.  The result carries about 44 bits, as df arithmetic does.
__device__ __forceinline__ void dacc_add(df& a, float th, float tl) {
  const df s = two_sum(a.hi, th);
  a.hi = s.hi;
  a.lo += s.lo + tl;
}
__device__ __forceinline__ void dacc_mul(df& a, df x, df y) {
  const float p = x.hi * y.hi;
  dacc_add(a, p, fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, fmaf(x.hi, y.hi, -p))));
}
__device__ __forceinline__ df dacc_norm(df a) { return two_sum(a.hi, a.lo); }

// warp_reduce_halving for double-float values, every addition a full df_add:
// afterwards v[0..3) of lane l hold the warp sums of entries 3 (l >> s) ..
// 3 (l >> s) + 2, s = 5 - log2(N / 3).
template <int N, int O>
__device__ __forceinline__ void warp_reduce_halving_df(df* v, int lane) {
  if constexpr (O > 0) {
    if constexpr (N > 3) {
      constexpr int H = N / 2;
      const bool upper = (lane & O) != 0;
#pragma unroll
      for (int i = 0; i < H; ++i) {
        const df send = upper ? v[i] : v[H + i];
        const df keep = upper ? v[H + i] : v[i];
        v[i] = df_add(keep, df{__shfl_xor_sync(0xffffffffu, send.hi, O), __shfl_xor_sync(0xffffffffu, send.lo, O)});
      }
      warp_reduce_halving_df<H, O / 2>(v, lane);
    } else {
#pragma unroll
      for (int i = 0; i < 3; ++i)
        v[i] = df_add(v[i], df{__shfl_xor_sync(0xffffffffu, v[i].hi, O), __shfl_xor_sync(0xffffffffu, v[i].lo, O)});
      warp_reduce_halving_df<N, O / 2>(v, lane);
    }
  }
}

// The 24 k-independent moments of a pair (one warp per pair, lanes over the
// Duffy points), in double-float arithmetic on the FP32 pipe: every product,
// sum, the reciprocal root and the accumulation carry about 44 bits, which is
// FP64 accuracy for these sums at the FP32 rate (this part's FP64 rate is
// 1/64 of it).  The 24 moments are summed by the compensated accumulation
// above (renormalised every eight points).  The lanes' partial
// sums are combined by a reduce-scatter in full df_add; lane 4 j then holds
// sums 3 j .. 3 j + 2 and writes moments = jac * sum in FP64 and their float
// copies into the pair record; lane 0 also writes the record's S0 term.
__global__ void __launch_bounds__(256)
    singular_moments_df_kernel(const SingularPair* __restrict__ pairs, int npairs, const int* __restrict__ rule_ptr,
                               const float* __restrict__ duffy_df, const float* __restrict__ geo_df,
                               double* __restrict__ moments, float* __restrict__ rec) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= npairs) return;
  const SingularPair P = pairs[warp];
  const float* G = geo_df + (size_t)kPairGeoDf * warp;
  df g[21];
#pragma unroll
  for (int i = 0; i < 21; ++i) g[i] = df{__ldg(G + 2 * i), __ldg(G + 2 * i + 1)};
  const df* e1t = g;
  const df* e2t = g + 3;
  const df* d0 = g + 6;
  const df* e1r = g + 9;
  const df* e2r = g + 12;
  const df* nt = g + 15;
  const df* nr = g + 18;
  const df inv4pi = {7.95774683356285095215e-02f, 3.21031911247035257e-09f};  // 1/(4 pi) as hi + lo
  df acc[kStatic];
#pragma unroll
  for (int i = 0; i < kStatic; ++i) acc[i] = df{0.0f, 0.0f};
  const int q0 = rule_ptr[P.rule], q1 = rule_ptr[P.rule + 1];
  int it = 0;
  for (int q = q0 + lane; q < q1; q += 32) {
    const float* pt = duffy_df + 10 * (size_t)q;
    const df tu = {pt[0], pt[1]}, tv = {pt[2], pt[3]}, ru = {pt[4], pt[5]}, rvv = {pt[6], pt[7]}, w = {pt[8], pt[9]};
    const df one = {1.0f, 0.0f};
    const df px[3] = {df_sub(df_sub(one, tu), tv), tu, tv};
    const df py[3] = {df_sub(df_sub(one, ru), rvv), ru, rvv};
    // the point and the normal components in full df arithmetic: on a coincident
    // pair (r . n = 0 in exact arithmetic) this keeps the double-layer moments at
    // their rounding level; a compensated sum of the five terms of r left them
    // about 50 times larger
    df rv[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const df yr = df_add(df_add(d0[d], df_mul(ru, e1r[d])), df_mul(rvv, e2r[d]));
      const df xt = df_add(df_mul(tu, e1t[d]), df_mul(tv, e2t[d]));
      rv[d] = df_sub(yr, xt);
    }
    const df r2 = df_add(df_add(df_mul(rv[0], rv[0]), df_mul(rv[1], rv[1])), df_mul(rv[2], rv[2]));
    if (r2.hi == 0.0f) continue;
    const df rinv = df_rsqrt(r2);
    const df s = df_mul(rinv, inv4pi);
    const df srr = df_mul(s, df_mul(rinv, rinv));
    const df dotn_r = df_add(df_add(df_mul(rv[0], nr[0]), df_mul(rv[1], nr[1])), df_mul(rv[2], nr[2]));
    const df dotn_t = df_add(df_add(df_mul(rv[0], nt[0]), df_mul(rv[1], nt[1])), df_mul(rv[2], nt[2]));
    const df ws = df_mul(w, s);
    const df wd = df_neg(df_mul(w, df_mul(dotn_r, srr)));  // w dG0/dn_y
    const df wn = df_mul(w, df_mul(dotn_t, srr));           // w dG0/dn_x
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const df was = df_mul(ws, px[a]);
      const df wad = df_mul(wd, px[a]);
      dacc_add(acc[a], was.hi, was.lo);
      dacc_mul(acc[21 + a], wn, px[a]);
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        dacc_mul(acc[3 + 3 * a + b], was, py[b]);
        dacc_mul(acc[12 + 3 * a + b], wad, py[b]);
      }
    }
    if ((++it & 7) == 0) {
#pragma unroll
      for (int i = 0; i < kStatic; ++i) acc[i] = dacc_norm(acc[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < kStatic; ++i) acc[i] = dacc_norm(acc[i]);
  warp_reduce_halving_df<kStatic, 16>(acc, lane);
  float* o = rec + (size_t)kPairRec * warp;
  if ((lane & 3) == 0) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double mine = df_to_double(acc[j]) * P.jac;
      moments[(size_t)kStatic * warp + 3 * (lane >> 2) + j] = mine;
      o[kRecMom + 3 * (lane >> 2) + j] = (float)mine;
    }
  }
  if (lane == 0) {
    const double m0 = df_to_double(acc[0]) * P.jac, m1 = df_to_double(acc[1]) * P.jac,
                 m2 = df_to_double(acc[2]) * P.jac;
    o[kRecS0] = (float)(m0 + m1 + m2);
  }
}

template <typename R> struct SingParams;
template <> struct SingParams<float> {
  float k, k2;
  float2 cD, cH, cM, cS, cK, cM10;
};
template <> struct SingParams<double> {
  double k, k2;
  double2 cD, cH, cM, cS, cK, cM10;
};

// Per pair output: 9 LHS block entries then 3 RHS-operator entries (complex).
constexpr int kSingOut = 12;

// The plain FP64 form's singular kernel (the mixed form uses singular_dyn_f32_kernel below).
template <typename R>
__global__ void __launch_bounds__(256, 1)
    singular_dyn_kernel(SingularGeom geo, const SingularPair* __restrict__ pairs, int npairs,
                                    const int* __restrict__ rule_ptr, const R* __restrict__ duffy,
                                    const double* __restrict__ moments, const double* __restrict__ curls,
                                    const double* __restrict__ area, const double* __restrict__ m11m10,
                                    SingParams<R> p, typename cplx<R>::type* __restrict__ out) {
  typedef typename cplx<R>::type C2;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= npairs) return;
  const SingularPair P = pairs[warp];
  const int* ft = geo.faces + 3 * P.test;
  const int* fr = geo.faces + 3 * P.trial;
  R e1t[3], e2t[3], d0[3], e1r[3], e2r[3], nt[3], nr[3];
  for (int d = 0; d < 3; ++d) {
    const double sd = d == 0 ? tr_sign_x(P.tr) : d == 1 ? tr_sign_y(P.tr) : 1.0;  // image pairs: S p
    const double t0 = geo.verts[3 * ft[0] + d];
    const double r0 = sd * geo.verts[3 * fr[0] + d];
    e1t[d] = (R)(geo.verts[3 * ft[1] + d] - t0);
    e2t[d] = (R)(geo.verts[3 * ft[2] + d] - t0);
    d0[d] = (R)(r0 - t0);
    e1r[d] = (R)(sd * geo.verts[3 * fr[1] + d] - r0);
    e2r[d] = (R)(sd * geo.verts[3 * fr[2] + d] - r0);
    nt[d] = (R)geo.normal[3 * P.test + d];
    nr[d] = (R)(sd * geo.normal[3 * P.trial + d]);
  }
  // accumulators: SR[3], IR[9], IDh[9], IKh[3] (complex) = 48 reals
  R acc[48];
#pragma unroll
  for (int i = 0; i < 48; ++i) acc[i] = R(0);
  const R inv4pi = R(0.25 / CUDART_PI);
  const int q0 = rule_ptr[P.rule], q1 = rule_ptr[P.rule + 1];
  for (int q = q0 + lane; q < q1; q += 32) {
    const R* pt = duffy + 5 * (size_t)q;
    const R tu = pt[0], tv = pt[1], ru = pt[2], rvv = pt[3], w = pt[4];
    const R px[3] = {R(1) - tu - tv, tu, tv};
    const R py[3] = {R(1) - ru - rvv, ru, rvv};
    R rv[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) rv[d] = (d0[d] + ru * e1r[d] + rvv * e2r[d]) - (tu * e1t[d] + tv * e2t[d]);
    const R r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
    if (r2 == R(0)) continue;
    R sh, ch;
    const R rinv = rsqrt(r2);
    const R r = r2 * rinv;
    sincos(R(0.5) * p.k * r, &sh, &ch);
    const R z = p.k * r;
    const R s = rinv * inv4pi;
    const R sinz = R(2) * sh * ch;
    const R omc = R(2) * sh * sh;  // 1 - cos z
    const R cosz = R(1) - omc;
    // R = s (cos z - 1 + i sin z)
    const R Rr = -s * omc, Ri = s * sinz;
    // h(z) = (1 - cos z - z sin z) + i (z cos z - sin z)
    const R hr = omc - z * sinz, hi = z * cosz - sinz;
    const R fy = (rv[0] * nr[0] + rv[1] * nr[1] + rv[2] * nr[2]) * s * rinv * rinv;
    const R fx = -(rv[0] * nt[0] + rv[1] * nt[1] + rv[2] * nt[2]) * s * rinv * rinv;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const R wa = w * px[a];
      acc[2 * a] += wa * Rr;
      acc[2 * a + 1] += wa * Ri;
      acc[42 + 2 * a] += wa * hr * fx;
      acc[42 + 2 * a + 1] += wa * hi * fx;
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const R wab = wa * py[b];
        acc[6 + 2 * (3 * a + b)] += wab * Rr;
        acc[6 + 2 * (3 * a + b) + 1] += wab * Ri;
        acc[24 + 2 * (3 * a + b)] += wab * hr * fy;
        acc[24 + 2 * (3 * a + b) + 1] += wab * hi * fy;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 48; ++i) acc[i] = warp_sum(acc[i]);
  if (lane != 0) return;
  const double* M = moments + (size_t)kStatic * warp;
  const R jac = (R)P.jac;
  C2 SR[3], IR[9], IDh[9], IKh[3];
  for (int a = 0; a < 3; ++a) {
    SR[a] = cplx<R>::make(acc[2 * a] * jac, acc[2 * a + 1] * jac);
    IKh[a] = cplx<R>::make(acc[42 + 2 * a] * jac, acc[42 + 2 * a + 1] * jac);
  }
  for (int i = 0; i < 9; ++i) {
    IR[i] = cplx<R>::make(acc[6 + 2 * i] * jac, acc[6 + 2 * i + 1] * jac);
    IDh[i] = cplx<R>::make(acc[24 + 2 * i] * jac, acc[24 + 2 * i + 1] * jac);
  }
  // S0 = sum w G (static + dynamic)
  C2 S0 = cplx<R>::make((R)(M[0] + M[1] + M[2]), R(0));
  for (int a = 0; a < 3; ++a) S0 = cadd(S0, SR[a]);
  const double* ct = curls + 9 * (size_t)P.test;
  const double* cr0 = curls + 9 * (size_t)P.trial;
  double cr[9];  // image pairs: reflected curls det(S) S c
  {
    const double sx = tr_sign_x(P.tr), sy = tr_sign_y(P.tr), det = sx * sy;
    for (int b = 0; b < 3; ++b) {
      cr[3 * b] = det * sx * cr0[3 * b];
      cr[3 * b + 1] = det * sy * cr0[3 * b + 1];
      cr[3 * b + 2] = det * cr0[3 * b + 2];
    }
  }
  const R kk_nn = p.k2 * (R)P.nprod;
  const bool coincident = P.kind == 1 && P.tr == 0;  // mass terms: the face with itself, never with an image
  const R a2 = (R)(2.0 * area[P.test]);
  C2* o = out + (size_t)kSingOut * warp;
  for (int a = 0; a < 3; ++a) {
    for (int b = 0; b < 3; ++b) {
      const R cc = (R)(ct[3 * a] * cr[3 * b] + ct[3 * a + 1] * cr[3 * b + 1] + ct[3 * a + 2] * cr[3 * b + 2]);
      const int i = 3 * a + b;
      C2 D = cplx<R>::make((R)M[12 + i] + IDh[i].x, IDh[i].y);
      C2 IGt = cplx<R>::make((R)M[3 + i] + IR[i].x, IR[i].y);
      C2 H = cplx<R>::make(cc * S0.x - kk_nn * IGt.x, cc * S0.y - kk_nn * IGt.y);
      C2 L = cadd(cmul(p.cD, D), cmul(p.cH, H));
      if (coincident) L = cadd(L, cscale(p.cM, a2 * (R)m11m10[i]));
      o[i] = L;
    }
    C2 S = cplx<R>::make((R)M[a] + SR[a].x, SR[a].y);
    C2 K = cplx<R>::make((R)M[21 + a] + IKh[a].x, IKh[a].y);
    C2 rhs = cadd(cmul(p.cS, S), cmul(p.cK, K));
    if (coincident) rhs = cadd(rhs, cscale(p.cM10, a2 * (R)m11m10[9 + a]));
    o[9 + a] = rhs;
  }
}

// Warp reduce-scatter by recursive halving of N = 3 x 2^j values per lane (N <= 96).  At
// exchange offset O a lane keeps one half of its values (the upper half when bit O of its
// lane index is set) and adds its partner's copy of that half, so each level moves half as
// many values as the one before; once three values remain, the remaining offsets are plain
// butterflies.  Afterwards v[0..3) of lane l hold the warp sums of entries 3 (l >> s) ..
// 3 (l >> s) + 2, s = 5 - log2(N / 3).  For 96 values the five levels move 48 + 24 + 12 +
// 6 + 3 values per lane, against 5 x 96 for a butterfly of every value.
template <int N, int O>
__device__ __forceinline__ void warp_reduce_halving(float* v, int lane) {
  if constexpr (O > 0) {
    if constexpr (N > 3) {
      constexpr int H = N / 2;
      const bool upper = (lane & O) != 0;
#pragma unroll
      for (int i = 0; i < H; ++i) {
        const float send = upper ? v[i] : v[H + i];
        const float keep = upper ? v[H + i] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, O);
      }
      warp_reduce_halving<H, O / 2>(v, lane);
    } else {
#pragma unroll
      for (int i = 0; i < 3; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], O);
      warp_reduce_halving<N, O / 2>(v, lane);
    }
  }
}

// The mixed form's singular kernel: the same Duffy remainder as
// singular_dyn_kernel<float>, with every per-pair FP64 quantity (geometry,
// curl products, static moments) read from the pair record instead of being
// formed from FP64 data per frequency.  One warp per pair, lanes over the
// Duffy points; after the warp reduction (every lane holds every sum) lanes
// 0-8 form the nine LHS entries and lanes 9-11 the three RHS-operator entries.
struct SingParamsF32 {
  float k, k2;
  float2 cD, cH, cM, cS, cK, cM10;
  float m11m10[12];
};

// NFQ frequencies per launch share each Duffy point's frequency-independent part
// (the point, r, 1/r, the normal-derivative factors, the basis weights); per
// frequency remain the phase, the remainder kernels and the 24 accumulators.
template <int NFQ> struct SingParamsF32N {
  SingParamsF32 f[NFQ];
};

template <int NFQ>
__global__ void __launch_bounds__(NFQ == 1 ? 256 : 128, NFQ == 1 ? 2 : 3)
    singular_dyn_f32_kernel(const SingularPair* __restrict__ pairs, int npairs, const int* __restrict__ rule_ptr,
                            const float* __restrict__ duffy, const float* __restrict__ rec, SingParamsF32N<NFQ> pn,
                            float2* __restrict__ out, long long out_stride) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= npairs) return;
  const SingularPair P = pairs[warp];
  const float* G = rec + (size_t)kPairRec * warp;
  float g[24];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(G) + i);
    g[4 * i] = v.x;
    g[4 * i + 1] = v.y;
    g[4 * i + 2] = v.z;
    g[4 * i + 3] = v.w;
  }
  const float* e1t = g + kRecGeom;
  const float* e2t = g + kRecGeom + 3;
  const float* d0 = g + kRecGeom + 6;
  const float* e1r = g + kRecGeom + 9;
  const float* e2r = g + kRecGeom + 12;
  const float* nt = g + kRecGeom + 15;
  const float* nr = g + kRecGeom + 18;
  float2 acc2[NFQ][24];  // per frequency: SR[3], IR[9], IDh[9], IKh[3] as (re, im)
#pragma unroll
  for (int f = 0; f < NFQ; ++f)
#pragma unroll
    for (int i = 0; i < 24; ++i) acc2[f][i] = make_float2(0.f, 0.f);
  const float inv4pi = (float)(0.25 / CUDART_PI);
  const int q0 = rule_ptr[P.rule], q1 = rule_ptr[P.rule + 1];
  // the next point's five values are loaded one iteration ahead
  float nx[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  if (q0 + lane < q1) {
#pragma unroll
    for (int i = 0; i < 5; ++i) nx[i] = __ldg(duffy + 5 * (size_t)(q0 + lane) + i);
  }
  for (int q = q0 + lane; q < q1; q += 32) {
    const float tu = nx[0], tv = nx[1], ru = nx[2], rvv = nx[3], w = nx[4];
    if (q + 32 < q1) {
#pragma unroll
      for (int i = 0; i < 5; ++i) nx[i] = __ldg(duffy + 5 * (size_t)(q + 32) + i);
    }
    const float px[3] = {1.f - tu - tv, tu, tv};
    const float py[3] = {1.f - ru - rvv, ru, rvv};
    float rv[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) rv[d] = (d0[d] + ru * e1r[d] + rvv * e2r[d]) - (tu * e1t[d] + tv * e2t[d]);
    const float r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
    if (r2 == 0.f) continue;
    const float rinv = rsqrt_ftz(r2);
    const float r = r2 * rinv;
    const float s = rinv * inv4pi;
    const float fy = (rv[0] * nr[0] + rv[1] * nr[1] + rv[2] * nr[2]) * s * rinv * rinv;
    const float fx = -(rv[0] * nt[0] + rv[1] * nt[1] + rv[2] * nt[2]) * s * rinv * rinv;
#pragma unroll
    for (int f = 0; f < NFQ; ++f) {
      const SingParamsF32& p = pn.f[f];
      float sh, ch;
      sincos_taylor(0.5f * p.k * r, &sh, &ch);
      const float z = p.k * r;
      const float sinz = 2.f * sh * ch;
      const float omc = 2.f * sh * sh;  // 1 - cos z
      const float cosz = 1.f - omc;
      const float Rr = -s * omc, Ri = s * sinz;
      const float hr = omc - z * sinz, hi = z * cosz - sinz;
      const float2 G2 = make_float2(Rr, Ri), Hy = make_float2(hr * fy, hi * fy), Hx = make_float2(hr * fx, hi * fx);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float wa = w * px[a];
        const float2 wa2 = make_float2(wa, wa);
        acc2[f][a] = __ffma2_rn(wa2, G2, acc2[f][a]);
        acc2[f][21 + a] = __ffma2_rn(wa2, Hx, acc2[f][21 + a]);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          const float2 wab = __fmul2_rn(wa2, make_float2(py[b], py[b]));
          acc2[f][3 + 3 * a + b] = __ffma2_rn(wab, G2, acc2[f][3 + 3 * a + b]);
          acc2[f][12 + 3 * a + b] = __ffma2_rn(wab, Hy, acc2[f][12 + 3 * a + b]);
        }
      }
    }
  }
  const float jac = g[kRecJac];
  const bool coincident = P.kind == 1 && P.tr == 0;  // mass terms: the face with itself, never with an image
  const float a2 = g[kRecA2];
  // Warp reduction of the NFQ x 48 sums by recursive halving (warp_reduce_halving): with
  // two frequencies lane L ends with sums 3L .. 3L + 2 of the flattened array (acc2[f][i].x
  // at 48 f + 2 i, .y next to it); with one, lanes 2m and 2m + 1 both hold sums 3m .. 3m + 2.
  // The sums go through shared memory to the lanes that form the outputs.
  constexpr int T = NFQ * 48;
  constexpr int WPB = (NFQ == 1 ? 256 : 128) / 32;
  __shared__ float red[WPB][T];
  {
    float v[T];
#pragma unroll
    for (int f = 0; f < NFQ; ++f)
#pragma unroll
      for (int i = 0; i < 24; ++i) {
        v[48 * f + 2 * i] = acc2[f][i].x;
        v[48 * f + 2 * i + 1] = acc2[f][i].y;
      }
    warp_reduce_halving<T, 16>(v, lane);
    float* r = red[threadIdx.x >> 5];
    constexpr int sh = NFQ == 2 ? 0 : 1;
    if ((lane & ((1 << sh) - 1)) == 0) {
#pragma unroll
      for (int j = 0; j < 3; ++j) r[3 * (lane >> sh) + j] = v[j];
    }
    __syncwarp();
  }
  const float* red_w = red[threadIdx.x >> 5];
  auto sum2 = [&](int f, int i) { return make_float2(red_w[48 * f + 2 * i], red_w[48 * f + 2 * i + 1]); };
#pragma unroll
  for (int f = 0; f < NFQ; ++f) {
    const SingParamsF32& p = pn.f[f];
    if (lane >= 12) continue;
    float2* o = out + (size_t)f * out_stride + (size_t)kSingOut * warp;
    if (lane < 9) {
      const int i = lane;
      // S0 = sum w G (static + dynamic)
      float2 S0 = make_float2(G[kRecS0], 0.f);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float2 sa = sum2(f, a);
        S0 = cadd(S0, make_float2(sa.x * jac, sa.y * jac));
      }
      const float2 ir = sum2(f, 3 + i), idh = sum2(f, 12 + i);
      const float2 IR = make_float2(ir.x * jac, ir.y * jac), IDh = make_float2(idh.x * jac, idh.y * jac);
      const float kk_nn = p.k2 * g[kRecNprod];
      const float cc = G[kRecCurl + i];
      const float2 D = make_float2(G[kRecMom + 12 + i] + IDh.x, IDh.y);
      const float2 IGt = make_float2(G[kRecMom + 3 + i] + IR.x, IR.y);
      const float2 H = make_float2(cc * S0.x - kk_nn * IGt.x, cc * S0.y - kk_nn * IGt.y);
      float2 L = cadd(cmul(p.cD, D), cmul(p.cH, H));
      if (coincident) L = cadd(L, cscale(p.cM, a2 * p.m11m10[i]));
      o[i] = L;
    } else {
      const int a = lane - 9;
      const float2 sr = sum2(f, a), ikh = sum2(f, 21 + a);
      const float2 SR = make_float2(sr.x * jac, sr.y * jac), IKh = make_float2(ikh.x * jac, ikh.y * jac);
      const float2 S = make_float2(G[kRecMom + a] + SR.x, SR.y);
      const float2 K = make_float2(G[kRecMom + 21 + a] + IKh.x, IKh.y);
      float2 rhs = cadd(cmul(p.cS, S), cmul(p.cK, K));
      if (coincident) rhs = cadd(rhs, cscale(p.cM10, a2 * p.m11m10[9 + a]));
      o[9 + a] = rhs;
    }
  }
}

// ------------------------------------------------------------------------
// The mixed form's singular remainder through a Chebyshev expansion in r.
//
// singular_dyn_f32_kernel sums, over a pair's Duffy points, basis weights times
//   G2 = (e^{ikr} - 1) / (4 pi r)             (SR, IR: 12 sums)
//   Hy = g2(r) (r . n_r) / (4 pi r),  Hx = -g2(r) (r . n_t) / (4 pi r)   (IDh, IKh: 12 sums)
// with g2(r) = (1 - (1 - ikr) e^{ikr}) / r^2: the point's G2 = f1(r) / (4 pi) with
// f1(r) = (e^{ikr} - 1) / r, and its hr + i hi = 1 - (1 - ikr) e^{ikr}.  f1 and g2 are
// smooth (entire) functions of r, so on [0, R], R bounding every pair's point distances,
// f1(r) = sum_n c1_n T_n(2 r / R - 1) and g2 likewise with c2_n, to a truncation error
// that the host checks per frequency.  The k-independent sums
//   M[n][i] = sum over the pair's Duffy points of (the point's weight for sum i) T_n(x)
// are formed once per mesh, and each frequency's 24 sums become sum_n c_n M[n][i]: the same
// quadrature (the reference's Duffy rules), evaluated with 24 terms per sum instead of one
// kernel evaluation per point and frequency.
// ------------------------------------------------------------------------

// Chebyshev moments (once per mesh, for the first nterms terms, a multiple of four): one
// warp per pair, lanes over the Duffy points (point geometry as in singular_dyn_f32_kernel,
// from the pair record), the terms in chunks of four (96 sums per lane), reduced by
// recursive halving; lane L then holds entries 3L .. 3L + 2 of the chunk, which are
// contiguous in cheb[((pair kChebN) + n) 24 + i].  The single-layer sums SR[a] (entries
// 0-2) are not formed: the P1 trial basis sums to one, so SR[a] = IR[a][0] + IR[a][1] +
// IR[a][2], and the per-frequency kernel adds them up there.
__global__ void __launch_bounds__(256)
    singular_cheb_moments_kernel(const SingularPair* __restrict__ pairs, int npairs, const int* __restrict__ rule_ptr,
                                 const float* __restrict__ duffy, const float* __restrict__ rec, float two_over_R,
                                 int nterms, float* __restrict__ cheb) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= npairs) return;
  const SingularPair P = pairs[warp];
  const float* G = rec + (size_t)kPairRec * warp;
  float g[21];
#pragma unroll
  for (int i = 0; i < 21; ++i) g[i] = __ldg(G + kRecGeom + i);
  const float* e1t = g;
  const float* e2t = g + 3;
  const float* d0 = g + 6;
  const float* e1r = g + 9;
  const float* e2r = g + 12;
  const float* nt = g + 15;
  const float* nr = g + 18;
  const float inv4pi = (float)(0.25 / CUDART_PI);
  const int q0 = rule_ptr[P.rule], q1 = rule_ptr[P.rule + 1];
  constexpr int NCH = 4;
  static_assert(kChebN % NCH == 0, "whole chunks");
  // one chunk of NCH terms starting at N0 (a compile-time constant, so that every register
  // index below is one)
  auto chunk = [&](auto n0_c) {
    constexpr int n0 = decltype(n0_c)::value;
    float v[NCH * 24];
#pragma unroll
    for (int i = 0; i < NCH * 24; ++i) v[i] = 0.f;
    for (int q = q0 + lane; q < q1; q += 32) {
      const float tu = __ldg(duffy + 5 * (size_t)q), tv = __ldg(duffy + 5 * (size_t)q + 1);
      const float ru = __ldg(duffy + 5 * (size_t)q + 2), rvv = __ldg(duffy + 5 * (size_t)q + 3);
      const float w = __ldg(duffy + 5 * (size_t)q + 4);
      const float px[3] = {1.f - tu - tv, tu, tv};
      const float py[3] = {1.f - ru - rvv, ru, rvv};
      float rv[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) rv[d] = (d0[d] + ru * e1r[d] + rvv * e2r[d]) - (tu * e1t[d] + tv * e2t[d]);
      const float r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
      if (r2 == 0.f) continue;
      const float rinv = rsqrt_ftz(r2);
      const float r = r2 * rinv;
      const float s = rinv * inv4pi;
      const float fy = (rv[0] * nr[0] + rv[1] * nr[1] + rv[2] * nr[2]) * s;     // (r . n_r) / (4 pi r)
      const float fx = -(rv[0] * nt[0] + rv[1] * nt[1] + rv[2] * nt[2]) * s;    // -(r . n_t) / (4 pi r)
      const float x = fminf(1.f, fmaf(r, two_over_R, -1.f));
      // T_n(x) for the chunk's n by the three-term recurrence
      float T[NCH];
      {
        float tm1 = 1.f, t0 = x;
#pragma unroll
        for (int n = 0; n < n0 + NCH; ++n) {
          float tn;
          if (n == 0) {
            tn = 1.f;
          } else if (n == 1) {
            tn = x;
          } else {
            tn = fmaf(2.f * x, t0, -tm1);
            tm1 = t0;
            t0 = tn;
          }
          if (n >= n0) T[n - n0] = tn;
        }
      }
      float wa[3], wab[9];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        wa[a] = w * px[a];
#pragma unroll
        for (int b = 0; b < 3; ++b) wab[3 * a + b] = wa[a] * py[b];
      }
#pragma unroll
      for (int j = 0; j < NCH; ++j) {
        float* vj = v + 24 * j;
        const float tg = T[j] * inv4pi;
#pragma unroll
        for (int a = 0; a < 3; ++a) vj[21 + a] = fmaf(wa[a] * fx, T[j], vj[21 + a]);
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          vj[3 + i] = fmaf(wab[i], tg, vj[3 + i]);
          vj[12 + i] = fmaf(wab[i] * fy, T[j], vj[12 + i]);
        }
      }
    }
    warp_reduce_halving<NCH * 24, 16>(v, lane);
    float* o = cheb + ((size_t)warp * kChebN + n0) * 24 + 3 * lane;
#pragma unroll
    for (int j = 0; j < 3; ++j) o[j] = v[j];
  };
  chunk(std::integral_constant<int, 0>{});
  chunk(std::integral_constant<int, 4>{});
  if (nterms > 8) chunk(std::integral_constant<int, 8>{});
  if (nterms > 12) chunk(std::integral_constant<int, 12>{});
  if (nterms > 16) chunk(std::integral_constant<int, 16>{});
  if (nterms > 20) chunk(std::integral_constant<int, 20>{});
  static_assert(kChebN == 24, "one chunk call per four terms");
}

// Per frequency: the 24 sums from the moments and the expansion coefficients (c1 for sums
// 0-11, c2 for 12-23), then the nine LHS and three RHS-operator entries exactly as in
// singular_dyn_f32_kernel.  One warp per pair; lane i < 24 forms sum i of every frequency
// (the pair's moments are read once for the NFQ frequencies).
template <int NFQ> struct ChebParamsF32 {
  float2 c1[NFQ][kChebN], c2[NFQ][kChebN];
  SingParamsF32 f[NFQ];
  long long off[NFQ];  // element offset of each frequency's blocks in out
};

template <int NFQ>
__global__ void __launch_bounds__(128)
    singular_cheb_f32_kernel(const SingularPair* __restrict__ pairs, int npairs, const float* __restrict__ rec,
                             const float* __restrict__ cheb, int nterms, ChebParamsF32<NFQ> cp,
                             float2* __restrict__ out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= npairs) return;
  const SingularPair P = pairs[warp];
  const float* G = rec + (size_t)kPairRec * warp;
  float2 acc[NFQ];
#pragma unroll
  for (int f = 0; f < NFQ; ++f) acc[f] = make_float2(0.f, 0.f);
  if (lane >= 3 && lane < 24) {
    const float* M = cheb + (size_t)warp * kChebN * 24 + lane;
    const bool second = lane >= 12;
#pragma unroll 4
    for (int n = 0; n < nterms; ++n) {
      const float m = __ldg(M + 24 * n);
#pragma unroll
      for (int f = 0; f < NFQ; ++f) {
        const float2 c = second ? cp.c2[f][n] : cp.c1[f][n];
        acc[f].x = fmaf(c.x, m, acc[f].x);
        acc[f].y = fmaf(c.y, m, acc[f].y);
      }
    }
  }
  const float jac = G[kRecJac];
  const bool coincident = P.kind == 1 && P.tr == 0;  // mass terms: the face with itself, never with an image
  const float a2 = G[kRecA2];
  const int srcA = 3 + lane;   // IR (lanes 0-8)
  const int srcB = 12 + lane;  // IDh (lanes 0-8) or IKh (lanes 9-11)
#pragma unroll
  for (int f = 0; f < NFQ; ++f) {
    float2 s3[3];  // SR[a] = IR[a][0] + IR[a][1] + IR[a][2]
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      s3[a] = make_float2(0.f, 0.f);
#pragma unroll
      for (int b = 0; b < 3; ++b)
        s3[a] = cadd(s3[a], make_float2(__shfl_sync(0xffffffffu, acc[f].x, 3 + 3 * a + b),
                                        __shfl_sync(0xffffffffu, acc[f].y, 3 + 3 * a + b)));
    }
    const float2 ir = make_float2(__shfl_sync(0xffffffffu, acc[f].x, srcA & 31),
                                  __shfl_sync(0xffffffffu, acc[f].y, srcA & 31));
    const float2 sb = make_float2(__shfl_sync(0xffffffffu, acc[f].x, srcB & 31),
                                  __shfl_sync(0xffffffffu, acc[f].y, srcB & 31));
    if (lane >= 12) continue;
    const SingParamsF32& p = cp.f[f];
    float2* o = out + cp.off[f] + (size_t)kSingOut * warp;
    if (lane < 9) {
      const int i = lane;
      float2 S0 = make_float2(G[kRecS0], 0.f);
#pragma unroll
      for (int a = 0; a < 3; ++a) S0 = cadd(S0, make_float2(s3[a].x * jac, s3[a].y * jac));
      const float2 IR = make_float2(ir.x * jac, ir.y * jac), IDh = make_float2(sb.x * jac, sb.y * jac);
      const float kk_nn = p.k2 * G[kRecNprod];
      const float cc = G[kRecCurl + i];
      const float2 D = make_float2(G[kRecMom + 12 + i] + IDh.x, IDh.y);
      const float2 IGt = make_float2(G[kRecMom + 3 + i] + IR.x, IR.y);
      const float2 H = make_float2(cc * S0.x - kk_nn * IGt.x, cc * S0.y - kk_nn * IGt.y);
      float2 L = cadd(cmul(p.cD, D), cmul(p.cH, H));
      if (coincident) L = cadd(L, cscale(p.cM, a2 * p.m11m10[i]));
      o[i] = L;
    } else {
      const int a = lane - 9;
      const float2 sr = a == 0 ? s3[0] : a == 1 ? s3[1] : s3[2];
      const float2 SR = make_float2(sr.x * jac, sr.y * jac), IKh = make_float2(sb.x * jac, sb.y * jac);
      const float2 S = make_float2(G[kRecMom + a] + SR.x, SR.y);
      const float2 K = make_float2(G[kRecMom + 21 + a] + IKh.x, IKh.y);
      float2 rhs = cadd(cmul(p.cS, S), cmul(p.cK, K));
      if (coincident) rhs = cadd(rhs, cscale(p.cM10, a2 * p.m11m10[9 + a]));
      o[9 + a] = rhs;
    }
  }
}

// The singular blocks into the extended rows: one thread per distinct target
// entry (planned once per mesh), adding that entry's contributions in pair order,
// so the sums are those of one thread walking each trial face's pairs, without
// that walk's chain of dependent read-modify-writes.
template <typename C2>
__global__ void singular_scatter_kernel(const int* __restrict__ scat_col, const int* __restrict__ scat_row,
                                        const int* __restrict__ scat_ptr, const int* __restrict__ scat_src,
                                        int n_entries, const C2* __restrict__ blocks, C2* __restrict__ Rext,
                                        long long ldR) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_entries) return;
  C2* dst = &Rext[(size_t)scat_col[i] * ldR + scat_row[i]];
  C2 v = *dst;
  for (int s = scat_ptr[i]; s < scat_ptr[i + 1]; ++s) v = cadd(v, blocks[scat_src[s]]);
  *dst = v;
}

// One CTA per column: A[:, j] in permuted row order.
template <typename C2>
__global__ void gather_columns_kernel(const C2* __restrict__ Rext, long long ldR, const int* __restrict__ col_ptr,
                                      const int* __restrict__ col_fb, const int* __restrict__ ext_row,
                                      const int* __restrict__ halo_slot_of_ext, const int* __restrict__ halo_row_ptr,
                                      const int* __restrict__ halo_row, int n_ext, int n_halo_rows,
                                      C2* __restrict__ A, long long lda, C2* __restrict__ A2, int col0,
                                      const double* __restrict__ row_weight) {
  extern __shared__ unsigned char smem_raw[];
  C2* hb = reinterpret_cast<C2*>(smem_raw);
  const int j = col0 + blockIdx.x;
  const int k0 = col_ptr[j], k1 = col_ptr[j + 1];
  C2* Aj = A + (size_t)j * lda;
  C2* A2j = A2 ? A2 + (size_t)j * lda : nullptr;
  for (int e = threadIdx.x; e < n_ext; e += blockDim.x) {
    C2 v;
    v.x = 0;
    v.y = 0;
    for (int k = k0; k < k1; ++k) v = cadd(v, Rext[(size_t)col_fb[k] * ldR + e]);
    const int hs = halo_slot_of_ext[e];
    if (hs < 0) {
      if (row_weight) v = cscale(v, (decltype(v.x))row_weight[ext_row[e]]);  // symmetry orbit weight of the row
      Aj[ext_row[e]] = v;
      if (A2j) A2j[ext_row[e]] = v;
    } else {
      hb[hs] = v;
    }
  }
  __syncthreads();
  for (int h = threadIdx.x; h < n_halo_rows; h += blockDim.x) {
    C2 s;
    s.x = 0;
    s.y = 0;
    for (int i = halo_row_ptr[h]; i < halo_row_ptr[h + 1]; ++i) s = cadd(s, hb[i]);
    const int r = halo_row[h];
    if (row_weight) s = cscale(s, (decltype(s.x))row_weight[r]);
    Aj[r] = cadd(Aj[r], s);
    if (A2j) A2j[r] = cadd(A2j[r], s);
  }
}

// ------------------------------------------------------------------------
// Right-hand side, regular part: warp per test face, lanes over driven faces.
//   rb[f][a][c] = sum_{g driven, not adjacent} q_c[g] (cS S_fg[a] + cK K'_fg[a])
//                 + sum over singular pairs (f, g) of q_c[g] * block_rhs[a]
// q_c[g] = qscale * drive[c][g]  (qscale = i rho omega).
// ------------------------------------------------------------------------
template <typename R> struct RhsParams;
template <> struct RhsParams<float> {
  df kdf;
  float k;
  float2 cS, cK, qscale;
  float cw[3 * kMaxQ];
};
template <> struct RhsParams<double> {
  double k;
  double2 cS, cK, qscale;
  double cw[3 * kMaxQ];
};

template <typename R> struct FaceRec;
template <> struct FaceRec<float> { typedef FaceF32 type; };
template <> struct FaceRec<double> { typedef FaceF64 type; };

template <int Q>
// sx, sy: reflection of the trial face (symmetry images; 1, 1 for the face itself).
__device__ __forceinline__ void rhs_pair_f32(const FaceF32& F, const FaceF32& Gf, const RhsParams<float>& p,
                                             float2 S[3], float2 K[3], float sx = 1.f, float sy = 1.f) {
  const float ghi[3] = {sx * Gf.anchor_hi[0], sy * Gf.anchor_hi[1], Gf.anchor_hi[2]};
  const float glo[3] = {sx * Gf.anchor_lo[0], sy * Gf.anchor_lo[1], Gf.anchor_lo[2]};
  PairF32 P = pair_setup_f32(ghi, glo, F.anchor_hi, F.anchor_lo, p.kdf);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    S[a] = make_float2(0.f, 0.f);
    K[a] = make_float2(0.f, 0.f);
  }
#pragma unroll 1
  for (int m = 0; m < Q; ++m) {
    float of[3] = {F.off[3 * m], F.off[3 * m + 1], F.off[3 * m + 2]};
    float2 us = make_float2(0.f, 0.f), uk = make_float2(0.f, 0.f);
#pragma unroll
    for (int n = 0; n < Q; ++n) {
      float d[3] = {sx * Gf.off[3 * n] - of[0], sy * Gf.off[3 * n + 1] - of[1], Gf.off[3 * n + 2] - of[2]};
      float rinv, rv[3];
      float2 G;
      green_f32(P, d, p.k, rinv, rv, G);
      // adjoint double layer: G (-1/r + ik) * (-(r . n_x)/r)
      float t = -fmaf(rv[0], F.normal[0], fmaf(rv[1], F.normal[1], rv[2] * F.normal[2])) * rinv;
      float2 Kk = make_float2(t * (-G.x * rinv - G.y * p.k), t * (G.x * p.k - G.y * rinv));
      // DP0 trial basis: weight is w_n only (sum_b phi_b w_n)
      float wn = p.cw[n] + p.cw[Q + n] + p.cw[2 * Q + n];
      us.x = fmaf(wn, G.x, us.x);
      us.y = fmaf(wn, G.y, us.y);
      uk.x = fmaf(wn, Kk.x, uk.x);
      uk.y = fmaf(wn, Kk.y, uk.y);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float c = p.cw[a * Q + m];
      S[a].x = fmaf(c, us.x, S[a].x);
      S[a].y = fmaf(c, us.y, S[a].y);
      K[a].x = fmaf(c, uk.x, K[a].x);
      K[a].y = fmaf(c, uk.y, K[a].y);
    }
  }
  const float jac = F.area2 * Gf.area2;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    S[a] = cscale(S[a], jac);
    K[a] = cscale(K[a], jac);
  }
}

template <int Q>
__device__ __forceinline__ void rhs_pair_f64(const FaceF64& F, const FaceF64& Gf, const RhsParams<double>& p,
                                             double2 S[3], double2 K[3], double sx = 1.0, double sy = 1.0) {
  const double sg[3] = {sx, sy, 1.0};
  const double C[3] = {sx * Gf.anchor[0] - F.anchor[0], sy * Gf.anchor[1] - F.anchor[1], Gf.anchor[2] - F.anchor[2]};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    S[a] = make_double2(0., 0.);
    K[a] = make_double2(0., 0.);
  }
#pragma unroll 1
  for (int m = 0; m < Q; ++m) {
    double2 us = make_double2(0., 0.), uk = make_double2(0., 0.);
#pragma unroll
    for (int n = 0; n < Q; ++n) {
      double rv[3];
      for (int d = 0; d < 3; ++d) rv[d] = C[d] + (sg[d] * Gf.off[3 * n + d] - F.off[3 * m + d]);
      const double r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
      if (r2 == 0.0) continue;
      const double r = sqrt(r2), rinv = 1.0 / r;
      double s, c;
      sincos(p.k * r, &s, &c);
      const double sc = rinv * (0.25 / CUDART_PI);
      const double2 G = make_double2(c * sc, s * sc);
      const double t = -(rv[0] * F.normal[0] + rv[1] * F.normal[1] + rv[2] * F.normal[2]) * rinv;
      const double2 Kk = make_double2(t * (-G.x * rinv - G.y * p.k), t * (G.x * p.k - G.y * rinv));
      const double wn = p.cw[n] + p.cw[Q + n] + p.cw[2 * Q + n];
      us.x += wn * G.x;
      us.y += wn * G.y;
      uk.x += wn * Kk.x;
      uk.y += wn * Kk.y;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double c = p.cw[a * Q + m];
      S[a].x += c * us.x;
      S[a].y += c * us.y;
      K[a].x += c * uk.x;
      K[a].y += c * uk.y;
    }
  }
  const double jac = F.area2 * Gf.area2;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    S[a] = cscale(S[a], jac);
    K[a] = cscale(K[a], jac);
  }
}

template <typename R, int Q, int NC>
__global__ void rhs_faces_kernel(const typename FaceRec<R>::type* __restrict__ faces, int nf,
                                 const int* __restrict__ driven, int ndriven,
                                 const typename cplx<R>::type* __restrict__ drive,  // NC x nf
                                 const SingularPair* __restrict__ pairs, const int* __restrict__ by_test_ptr,
                                 const int* __restrict__ by_test, const typename cplx<R>::type* __restrict__ sblocks,
                                 RhsParams<R> p, typename cplx<R>::type* __restrict__ rb, int ntr, int4 trs,
                                 const unsigned char* __restrict__ fix_mask) {
  typedef typename cplx<R>::type C2;
  const int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (f >= nf) return;
  const auto& F = faces[f];
  C2 acc[3][NC];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[a][c] = cplx<R>::make(0, 0);
  // driven faces and their symmetry images (touching pairs are in the singular blocks)
  for (int ti = 0; ti < ntr; ++ti)
  for (int i = lane; i < ndriven; i += 32) {
    const int tr = ti == 0 ? trs.x : ti == 1 ? trs.y : ti == 2 ? trs.z : trs.w;
    const int g = driven[i];
    const auto& Gf = faces[g];
    int sv[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) sv[b] = (tr == 0 || (fix_mask[Gf.verts[b]] & tr) == tr) ? Gf.verts[b] : -2;
    if (share_vertex(F.verts, sv[0], sv[1], sv[2])) continue;
    C2 S[3], K[3];
    if constexpr (sizeof(R) == 4)
      rhs_pair_f32<Q>(F, Gf, p, S, K, (float)tr_sign_x(tr), (float)tr_sign_y(tr));
    else
      rhs_pair_f64<Q>(F, Gf, p, S, K, tr_sign_x(tr), tr_sign_y(tr));
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const C2 q = cmul(p.qscale, drive[(size_t)c * nf + g]);
#pragma unroll
      for (int a = 0; a < 3; ++a) acc[a][c] = cadd(acc[a][c], cmul(q, cadd(cmul(p.cS, S[a]), cmul(p.cK, K[a]))));
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      acc[a][c].x = warp_sum(acc[a][c].x);
      acc[a][c].y = warp_sum(acc[a][c].y);
    }
  if (lane != 0) return;
  for (int k = by_test_ptr[f]; k < by_test_ptr[f + 1]; ++k) {
    const int pid = by_test[k];
    const int g = pairs[pid].trial;
    const C2* blk = sblocks + (size_t)kSingOut * pid;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const C2 q = cmul(p.qscale, drive[(size_t)c * nf + g]);
      if (q.x == 0 && q.y == 0) continue;
#pragma unroll
      for (int a = 0; a < 3; ++a) acc[a][c] = cadd(acc[a][c], cmul(q, blk[9 + a]));
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < NC; ++c) rb[((size_t)c * nf + f) * 3 + a] = acc[a][c];
}

// Right-hand side of NFQ frequencies at once (mixed form).  The frequency-independent part of
// every q-pair (the pair's C and |C|, r, 1/r, the compensated r - |C| and the
// adjoint-double-layer factor t) is formed once and shared; per frequency follow the phase,
// e^{ikr} and the sums, in the operations and order of rhs_faces_kernel<float> and
// rhs_pair_f32.  rb holds frequency fq's columns at rb[((fq NC + c) nf + f) 3 + a]; its
// singular blocks start at sblocks + fq sblocks_stride.
template <int NFQ> struct RhsParamsF32N {
  df kdf[NFQ];
  float k[NFQ];
  float2 cS[NFQ], cK[NFQ], qscale[NFQ];
  float cw[3 * kMaxQ];
};

template <int Q, int NFQ>
__device__ __forceinline__ void rhs_pair_f32_freqs(const FaceF32& F, const FaceF32& Gf, const RhsParamsF32N<NFQ>& p,
                                                   float2 S[NFQ][3], float2 K[NFQ][3], float sx, float sy) {
  const float ghi[3] = {sx * Gf.anchor_hi[0], sy * Gf.anchor_hi[1], Gf.anchor_hi[2]};
  const float glo[3] = {sx * Gf.anchor_lo[0], sy * Gf.anchor_lo[1], Gf.anchor_lo[2]};
  const PairGeomF32 P = pair_geom_f32(ghi, glo, F.anchor_hi, F.anchor_lo);
  const float R0 = P.R.hi + P.R.lo;
  float th0[NFQ];
#pragma unroll
  for (int fq = 0; fq < NFQ; ++fq) {
    th0[fq] = df_reduce_two_pi(df_mul(p.kdf[fq], P.R));
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      S[fq][a] = make_float2(0.f, 0.f);
      K[fq][a] = make_float2(0.f, 0.f);
    }
  }
#pragma unroll 1
  for (int m = 0; m < Q; ++m) {
    const float of[3] = {F.off[3 * m], F.off[3 * m + 1], F.off[3 * m + 2]};
    float2 us[NFQ], uk[NFQ];
#pragma unroll
    for (int fq = 0; fq < NFQ; ++fq) {
      us[fq] = make_float2(0.f, 0.f);
      uk[fq] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int n = 0; n < Q; ++n) {
      const float d[3] = {sx * Gf.off[3 * n] - of[0], sy * Gf.off[3 * n + 1] - of[1], Gf.off[3 * n + 2] - of[2]};
      float rv[3];
      rv[0] = P.Cf[0] + d[0];
      rv[1] = P.Cf[1] + d[1];
      rv[2] = P.Cf[2] + d[2];
      const float r2 = fmaf(rv[0], rv[0], fmaf(rv[1], rv[1], rv[2] * rv[2]));
      const float rinv = r2 > 1e-30f ? rsqrt_ftz(r2) : 0.0f;
      const float r = r2 * rinv;
      const float cd = fmaf(P.Cf[0], d[0], fmaf(P.Cf[1], d[1], P.Cf[2] * d[2]));
      const float dd = fmaf(d[0], d[0], fmaf(d[1], d[1], d[2] * d[2]));
      const float den = fmaxf(r + R0, 1e-30f);
      const float delta = fmaf(2.0f, cd, dd) * rcp_ftz(den);
      const float sc = rinv * BEM_INV_FOUR_PI;
      // adjoint double layer: G (-1/r + ik) * (-(r . n_x)/r)
      const float t = -fmaf(rv[0], F.normal[0], fmaf(rv[1], F.normal[1], rv[2] * F.normal[2])) * rinv;
      const float wn = p.cw[n] + p.cw[Q + n] + p.cw[2 * Q + n];  // DP0 trial basis
#pragma unroll
      for (int fq = 0; fq < NFQ; ++fq) {
        const float theta = reduce_two_pi(fmaf(p.k[fq], delta, th0[fq]));
        float s, c;
        sincos_ftz(theta, &s, &c);
        const float2 G = make_float2(c * sc, s * sc);
        const float2 Kk = make_float2(t * (-G.x * rinv - G.y * p.k[fq]), t * (G.x * p.k[fq] - G.y * rinv));
        us[fq].x = fmaf(wn, G.x, us[fq].x);
        us[fq].y = fmaf(wn, G.y, us[fq].y);
        uk[fq].x = fmaf(wn, Kk.x, uk[fq].x);
        uk[fq].y = fmaf(wn, Kk.y, uk[fq].y);
      }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float c = p.cw[a * Q + m];
#pragma unroll
      for (int fq = 0; fq < NFQ; ++fq) {
        S[fq][a].x = fmaf(c, us[fq].x, S[fq][a].x);
        S[fq][a].y = fmaf(c, us[fq].y, S[fq][a].y);
        K[fq][a].x = fmaf(c, uk[fq].x, K[fq][a].x);
        K[fq][a].y = fmaf(c, uk[fq].y, K[fq][a].y);
      }
    }
  }
  const float jac = F.area2 * Gf.area2;
#pragma unroll
  for (int fq = 0; fq < NFQ; ++fq)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      S[fq][a] = cscale(S[fq][a], jac);
      K[fq][a] = cscale(K[fq][a], jac);
    }
}

template <int Q, int NC, int NFQ>
__global__ void __launch_bounds__(128) rhs_faces_f32_freqs_kernel(
    const FaceF32* __restrict__ faces, int nf, const int* __restrict__ driven, int ndriven,
    const float2* __restrict__ drive, const SingularPair* __restrict__ pairs, const int* __restrict__ by_test_ptr,
    const int* __restrict__ by_test, const float2* __restrict__ sblocks, long long sblocks_stride,
    RhsParamsF32N<NFQ> p, float2* __restrict__ rb, int ntr, int4 trs, const unsigned char* __restrict__ fix_mask) {
  const int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (f >= nf) return;
  const FaceF32& F = faces[f];
  float2 acc[NFQ][3][NC];
#pragma unroll
  for (int fq = 0; fq < NFQ; ++fq)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[fq][a][c] = make_float2(0.f, 0.f);
  // driven faces and their symmetry images (touching pairs are in the singular blocks)
  for (int ti = 0; ti < ntr; ++ti)
    for (int i = lane; i < ndriven; i += 32) {
      const int tr = ti == 0 ? trs.x : ti == 1 ? trs.y : ti == 2 ? trs.z : trs.w;
      const int g = driven[i];
      const FaceF32& Gf = faces[g];
      int sv[3];
#pragma unroll
      for (int b = 0; b < 3; ++b) sv[b] = (tr == 0 || (fix_mask[Gf.verts[b]] & tr) == tr) ? Gf.verts[b] : -2;
      if (share_vertex(F.verts, sv[0], sv[1], sv[2])) continue;
      float2 S[NFQ][3], K[NFQ][3];
      rhs_pair_f32_freqs<Q, NFQ>(F, Gf, p, S, K, (float)tr_sign_x(tr), (float)tr_sign_y(tr));
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const float2 dg = drive[(size_t)c * nf + g];
#pragma unroll
        for (int fq = 0; fq < NFQ; ++fq) {
          const float2 q = cmul(p.qscale[fq], dg);
#pragma unroll
          for (int a = 0; a < 3; ++a)
            acc[fq][a][c] = cadd(acc[fq][a][c], cmul(q, cadd(cmul(p.cS[fq], S[fq][a]), cmul(p.cK[fq], K[fq][a]))));
        }
      }
    }
#pragma unroll
  for (int fq = 0; fq < NFQ; ++fq)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        acc[fq][a][c].x = warp_sum(acc[fq][a][c].x);
        acc[fq][a][c].y = warp_sum(acc[fq][a][c].y);
      }
  if (lane != 0) return;
  for (int kk = by_test_ptr[f]; kk < by_test_ptr[f + 1]; ++kk) {
    const int pid = by_test[kk];
    const int g = pairs[pid].trial;
#pragma unroll
    for (int fq = 0; fq < NFQ; ++fq) {
      const float2* blk = sblocks + (size_t)fq * sblocks_stride + (size_t)kSingOut * pid;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const float2 q = cmul(p.qscale[fq], drive[(size_t)c * nf + g]);
        if (q.x == 0 && q.y == 0) continue;
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[fq][a][c] = cadd(acc[fq][a][c], cmul(q, blk[9 + a]));
      }
    }
  }
#pragma unroll
  for (int fq = 0; fq < NFQ; ++fq)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < NC; ++c) rb[(((size_t)fq * NC + c) * nf + f) * 3 + a] = acc[fq][a][c];
}

// b[row(j)][c] = sum over (f, a) in star(j) of rb[c][f][a]
template <typename C2>
__global__ void rhs_gather_kernel(const C2* __restrict__ rb, int nf, int nc, const int* __restrict__ col_ptr,
                                  const int* __restrict__ col_fb, const int* __restrict__ vertex_row, int nv,
                                  C2* __restrict__ b, long long ldb, const double* __restrict__ row_weight) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  for (int c = 0; c < nc; ++c) {
    C2 s;
    s.x = 0;
    s.y = 0;
    for (int k = col_ptr[j]; k < col_ptr[j + 1]; ++k) s = cadd(s, rb[(size_t)c * nf * 3 + col_fb[k]]);
    if (row_weight) s = cscale(s, (decltype(s.x))row_weight[vertex_row[j]]);
    b[(size_t)c * ldb + vertex_row[j]] = s;
  }
}

// Rows/columns of vertices that no face references: identity (pressure 0).
template <typename C2>
__global__ void isolated_identity_kernel(const int* __restrict__ iso, int n, const int* __restrict__ vertex_row,
                                         C2* A, long long lda, C2* A2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int v = iso[i];
  C2 one;
  one.x = 1;
  one.y = 0;
  A[(size_t)v * lda + vertex_row[v]] = one;
  if (A2) A2[(size_t)v * lda + vertex_row[v]] = one;
}

}  // namespace

// --------------------------------------------------------------- launchers --

static inline float2 f2(double2 v) { return make_float2((float)v.x, (float)v.y); }

static df make_df(double x) {
  df r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}

namespace {
template <int NFQ, bool DT>
cudaError_t launch_regular_f32(const DeviceMesh& m, const double* k, const double2* cD, const double2* cH,
                               float2* Rext, long long ldR, long long strideR, cudaStream_t stream) {
  constexpr int W = 4;
  dim3 grid((m.nf + W - 1) / W, m.n_tiles);
  RegParamsF32<NFQ, DT> p;
  for (int i = 0; i < 3 * kMaxQ; ++i) p.cw2[i] = make_float2((float)m.rule_cw[i], (float)m.rule_cw[i]);
  for (int q = 0; q < kMaxQ; ++q) {  // w_q = sum_a phi_a(xi_q) w_q (the basis sums to one)
    const float w = q < m.Q ? (float)(m.rule_cw[q] + m.rule_cw[m.Q + q] + m.rule_cw[2 * m.Q + q]) : 0.0f;
    p.w2[q] = make_float2(w, w);
    p.wp[q] = make_float2(w, w);
    for (int b = 0; b < 3; ++b) {
      const float c = q < m.Q ? (float)m.rule_cw[b * m.Q + q] : 0.0f;
      p.cwp[b][q] = make_float2(c, c);
    }
  }
  for (int f = 0; f < NFQ; ++f) {
    p.kdf[f] = make_df(k[f]);
    p.k[f] = (float)k[f];
    p.k2[f] = (float)(k[f] * k[f]);
    p.cH[f] = f2(cH[f]);
    if (DT) {
      const double d = cD[f].x * cD[f].x + cD[f].y * cD[f].y;  // cH / cD
      p.cHn[f] = make_float2((float)((cH[f].x * cD[f].x + cH[f].y * cD[f].y) / d),
                             (float)((cH[f].y * cD[f].x - cH[f].x * cD[f].y) / d));
      p.cDn[f] = f2(cD[f]);
    } else {
      p.cHn[f] = f2(cH[f]);
      p.cDn[f] = make_float2(1.0f, 0.0f);
    }
  }
  const size_t sm = (size_t)W * NFQ * 3 * m.max_tile_rows * sizeof(float2);
  auto launch = [&](auto kern) {
    ensure_smem_limit((const void*)kern, sm);
    kern<<<grid, W * 32, sm, stream>>>(m.faces32, m.nf, m.tile_group_ptr, m.lane_slots, m.group_faces32,
                                       m.tile_row_base, m.max_tile_rows, Rext, ldR, strideR, p, m.ntr,
                                       make_int4(m.tr[0], m.tr[1], m.tr[2], m.tr[3]), m.fix_mask);
  };
  if (m.Q == 6)
    launch(regular_f32_kernel<6, W, NFQ, DT>);
  else if (m.Q == 3)
    launch(regular_f32_kernel<3, W, NFQ, DT>);
  else
    launch(regular_f32_kernel<1, W, NFQ, DT>);
  return cudaGetLastError();
}
}  // namespace

// Frequencies per regular-kernel launch for a group of n that all carry the
// double-layer term: the widest NFQ (4, else 3, else 2) whose per-warp
// accumulators still let two CTAs share an SM's shared memory; a remainder that
// would leave a single frequency alone (which shares nothing) is split into
// 3 + 2 (NFQ 4) or 2 + 2 (NFQ 3).
int regular_width(const DeviceMesh& m) {
  for (int w = 4; w >= 3; --w)
    if ((size_t)4 * w * 3 * m.max_tile_rows * sizeof(float2) <= (size_t)112 * 1024) return w;
  return 2;
}

int regular_split(int n, int width, int* sizes) {
  int cnt = 0;
  if (width <= 2) {
    for (; n >= 2; n -= 2) sizes[cnt++] = 2;
    if (n) sizes[cnt++] = 1;
    return cnt;
  }
  int q = n / width, r = n % width;
  if (r == 1 && q >= 1) {  // width + 1 = (width - 1) + 2
    --q;
    for (int i = 0; i < q; ++i) sizes[cnt++] = width;
    sizes[cnt++] = width - 1;
    sizes[cnt++] = 2;
    return cnt;
  }
  for (int i = 0; i < q; ++i) sizes[cnt++] = width;
  if (r) sizes[cnt++] = r;
  return cnt;
}

cudaError_t launch_regular(const DeviceMesh& m, Precision prec, int nfreq, const double* k, const double2* cD,
                           const double2* cH, void* Rext, long long ldR, long long strideR, cudaStream_t stream) {
  if (prec == Precision::Mixed) {
    // up to four frequencies per launch share the frequency-independent geometry;
    // an operator without the double-layer term (cD = 0) runs one per launch
    const int width = regular_width(m);
    int f = 0;
    while (f < nfreq) {
      float2* R = (float2*)Rext + (size_t)f * strideR;
      auto dt_at = [&](int i) { return cD[i].x != 0.0 || cD[i].y != 0.0; };
      if (!dt_at(f)) {
        cudaError_t e = launch_regular_f32<1, false>(m, k + f, cD + f, cH + f, R, ldR, strideR, stream);
        if (e != cudaSuccess) return e;
        ++f;
        continue;
      }
      int run = 1;  // consecutive frequencies with the double-layer term
      while (f + run < nfreq && dt_at(f + run)) ++run;
      int sizes[64];
      const int cnt = regular_split(run, width, sizes);
      for (int i = 0; i < cnt; ++i) {
        R = (float2*)Rext + (size_t)f * strideR;
        cudaError_t e = sizes[i] == 4   ? launch_regular_f32<4, true>(m, k + f, cD + f, cH + f, R, ldR, strideR, stream)
                        : sizes[i] == 3 ? launch_regular_f32<3, true>(m, k + f, cD + f, cH + f, R, ldR, strideR, stream)
                        : sizes[i] == 2 ? launch_regular_f32<2, true>(m, k + f, cD + f, cH + f, R, ldR, strideR, stream)
                                        : launch_regular_f32<1, true>(m, k + f, cD + f, cH + f, R, ldR, strideR, stream);
        if (e != cudaSuccess) return e;
        f += sizes[i];
      }
    }
    return cudaSuccess;
  }
  for (int f = 0; f < nfreq; ++f) {
    cudaError_t e = launch_regular_f64(m, k[f], cD[f], cH[f], (double2*)Rext + (size_t)f * strideR, ldR, stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

int regular_groups(const DeviceMesh& m, Precision prec, int nfreq, int* sizes) {
  if (prec != Precision::Mixed) {
    for (int i = 0; i < nfreq; ++i) sizes[i] = 1;
    return nfreq;
  }
  return regular_split(nfreq, regular_width(m), sizes);
}

double regular_flop_per_qpair(int w) {
  // per quadrature pair and frequency, counted from regular_f32_kernel: the
  // frequency-independent geometry of the pair (23) and of its test point (23 / Q
  // with Q = 6 trial points) shared by the w frequencies of a launch; per
  // frequency the phase and weight (7), e^{ikr} E'' and the basis sums (22), and
  // the test point's W and S0 updates (40 / 6)
  return 7.0 + 22.0 + 40.0 / 6.0 + (23.0 + 23.0 / 6.0) / (double)w;
}

int regular_launches(const DeviceMesh& m, Precision prec, int nfreq) {
  int sizes[64];
  return regular_groups(m, prec, nfreq, sizes);
}

cudaError_t launch_regular_f64(const DeviceMesh& m, double k, double2 cD, double2 cH, double2* Rext, long long ldR,
                               cudaStream_t stream) {
  const int W = 4;
  dim3 grid((m.nf + W - 1) / W, m.n_tiles);
  {
    RegParamsF64 p;
    p.k = k;
    p.k2 = k * k;
    p.cD = cD;
    p.cH = cH;
    for (int i = 0; i < 3 * kMaxQ; ++i) p.cw[i] = m.rule_cw[i];
    size_t sm = (size_t)W * 3 * m.max_tile_rows * sizeof(double2);
    auto launch = [&](auto kern) {
      ensure_smem_limit((const void*)kern, sm);
      kern<<<grid, W * 32, sm, stream>>>(m.faces64, m.nf, m.tile_group_ptr, m.lane_slots, m.tile_row_base,
                                         m.max_tile_rows, (double2*)Rext, ldR, p, m.ntr,
                                         make_int4(m.tr[0], m.tr[1], m.tr[2], m.tr[3]), m.fix_mask);
    };
    if (m.Q == 6)
      launch(regular_f64_kernel<6, W>);
    else if (m.Q == 3)
      launch(regular_f64_kernel<3, W>);
    else
      launch(regular_f64_kernel<1, W>);
  }
  return cudaGetLastError();
}

cudaError_t launch_singular_static(const DeviceMesh& m, double* moments, float* pairrec, cudaStream_t stream) {
  if (m.npairs == 0) return cudaSuccess;
  SingularGeom geo{m.verts, m.faces, m.normal};
  pair_setup_kernel<<<(m.npairs + 127) / 128, 128, 0, stream>>>(geo, m.pairs, m.npairs, m.curls, m.area, m.pairgeo_df,
                                                                pairrec);
  const int threads = 256;
  const int blocks = (int)(((long long)m.npairs * 32 + threads - 1) / threads);
  singular_moments_df_kernel<<<blocks, threads, 0, stream>>>(m.pairs, m.npairs, m.rule_ptr, m.duffy_df, m.pairgeo_df,
                                                             moments, pairrec);
  return cudaGetLastError();
}

namespace {
// Chebyshev coefficients on r in [0, R] of f1(r) = (e^{ikr} - 1) / r and
// g2(r) = (1 - (1 - ikr) e^{ikr}) / r^2 (FP64), by interpolation at the N <= kChebN
// Chebyshev points: f(r) ~ sum_n c_n T_n(2 r / R - 1).  Below z = kr = 1/2 both come from their
// Taylor series (f1 = k sum_{n>=1} i^n z^(n-1) / n!, g2 = k^2 sum_{n>=2} (n - 1) i^n
// z^(n-2) / n!), which has no cancellation.  Returns false when the last two coefficients
// of either are above 1e-9 of its largest: the expansion has not converged (kR too large
// for N terms) and the caller integrates point by point instead.
bool cheb_coefficients(double k, double R, int N, double2* c1, double2* c2) {
  typedef std::complex<double> cd;
  cd f1[kChebN], g2[kChebN];
  const double pi = 3.14159265358979323846;
  for (int j = 0; j < N; ++j) {
    const double x = std::cos(pi * (j + 0.5) / N), r = 0.5 * R * (1.0 + x), z = k * r;
    if (z < 0.5) {
      cd s1(0.0, 0.0), s2(0.0, 0.0), ipow(0.0, 1.0);  // ipow = i^n, from n = 1
      double zp1 = 1.0, zp2 = 0.0, fact = 1.0;        // z^(n-1), z^(n-2), n!
      for (int n = 1; n <= 30; ++n) {
        fact *= n;
        s1 += ipow * (zp1 / fact);                           // i^n z^(n-1) / n!
        if (n >= 2) s2 += ipow * ((n - 1) * zp2 / fact);     // i^n (n-1) z^(n-2) / n!
        zp2 = zp1;
        zp1 *= z;
        ipow *= cd(0.0, 1.0);
      }
      f1[j] = k * s1;
      g2[j] = k * k * s2;
    } else {
      const double sh = std::sin(0.5 * z), sz = std::sin(z), cz = std::cos(z);
      const cd e(cz, sz);
      f1[j] = cd(-2.0 * sh * sh, sz) / r;
      g2[j] = (cd(1.0, 0.0) - cd(1.0, -z) * e) / (r * r);
    }
  }
  double m1 = 0.0, m2 = 0.0;
  cd a1[kChebN], a2[kChebN];
  for (int n = 0; n < N; ++n) {
    cd s1(0.0, 0.0), s2(0.0, 0.0);
    for (int j = 0; j < N; ++j) {
      const double t = std::cos(pi * n * (j + 0.5) / N);
      s1 += f1[j] * t;
      s2 += g2[j] * t;
    }
    const double sc = (n == 0 ? 1.0 : 2.0) / N;
    a1[n] = s1 * sc;
    a2[n] = s2 * sc;
    m1 = std::max(m1, std::abs(a1[n]));
    m2 = std::max(m2, std::abs(a2[n]));
    c1[n] = make_double2(a1[n].real(), a1[n].imag());
    c2[n] = make_double2(a2[n].real(), a2[n].imag());
  }
  const double t1 = std::abs(a1[N - 1]) + std::abs(a1[N - 2]), t2 = std::abs(a2[N - 1]) + std::abs(a2[N - 2]);
  return t1 <= 1e-9 * m1 && t2 <= 1e-9 * m2;
}
}  // namespace

int cheb_terms(double k, double R) {
  if (!(R > 0.0)) return 0;
  double2 c1[kChebN], c2[kChebN];
  for (int n = 8; n <= kChebN; n += 4)
    if (cheb_coefficients(k, R, n, c1, c2)) return n;
  return 0;
}

cudaError_t launch_cheb_moments(const DeviceMesh& m, int nterms, cudaStream_t stream) {
  if (m.npairs == 0 || !m.cheb || nterms < 4 || nterms > kChebN || nterms % 4 || !(m.cheb_R > 0.0))
    return cudaErrorInvalidValue;
  const int threads = 256;
  const int blocks = (int)(((long long)m.npairs * 32 + threads - 1) / threads);
  singular_cheb_moments_kernel<<<blocks, threads, 0, stream>>>(m.pairs, m.npairs, m.rule_ptr, m.duffy32, m.pairrec,
                                                               (float)(2.0 / m.cheb_R), nterms, m.cheb);
  return cudaGetLastError();
}

cudaError_t launch_singular_dyn(const DeviceMesh& m, Precision prec, int nfreq, const double* k,
                                const OperatorCoeffs* c, void* blocks, long long blocks_stride, cudaStream_t stream,
                                long long* launched, long long* cheb_freqs, bool use_cheb) {
  if (m.npairs == 0) return cudaSuccess;
  SingularGeom geo{m.verts, m.faces, m.normal};
  long long nl = 0;
  if (prec == Precision::Mixed) {
    auto params = [&](int f) {
      SingParamsF32 p;
      p.k = (float)k[f];
      p.k2 = (float)(k[f] * k[f]);
      p.cD = f2(c[f].cD);
      p.cH = f2(c[f].cH);
      p.cM = f2(c[f].cM);
      p.cS = f2(c[f].cS);
      p.cK = f2(c[f].cK);
      p.cM10 = f2(c[f].cM10);
      for (int i = 0; i < 12; ++i) p.m11m10[i] = m.m11m10f[i];
      return p;
    };
    // point by point: two frequencies per launch share each point's geometry; a lone last one runs alone
    auto direct = [&](int f0, int count) {
      for (int f = f0; f < f0 + count;) {
        float2* o = (float2*)blocks + (size_t)f * blocks_stride;
        if (f + 1 < f0 + count) {
          SingParamsF32N<2> pn;
          pn.f[0] = params(f);
          pn.f[1] = params(f + 1);
          const int threads = 128;
          const int nblk = (int)(((long long)m.npairs * 32 + threads - 1) / threads);
          singular_dyn_f32_kernel<2><<<nblk, threads, 0, stream>>>(m.pairs, m.npairs, m.rule_ptr, m.duffy32,
                                                                   m.pairrec, pn, o, blocks_stride);
          f += 2;
        } else {
          SingParamsF32N<1> pn;
          pn.f[0] = params(f);
          const int threads = 256;
          const int nblk = (int)(((long long)m.npairs * 32 + threads - 1) / threads);
          singular_dyn_f32_kernel<1><<<nblk, threads, 0, stream>>>(m.pairs, m.npairs, m.rule_ptr, m.duffy32,
                                                                   m.pairrec, pn, o, blocks_stride);
          f += 1;
        }
        ++nl;
      }
    };
    // through the Chebyshev moments: up to four frequencies per launch read each pair's
    // moments once.  Frequency f uses exactly the N(k_f) terms its expansion needs
    // (cheb_terms; the coefficients beyond are zero), so its blocks do not depend on how
    // many terms the moments hold or on which frequencies share the launch.  Frequencies
    // whose expansion needs more terms than the moments hold, or none converges, run point
    // by point, consecutive ones paired.
    std::vector<double2> c1((size_t)nfreq * kChebN, make_double2(0.0, 0.0)), c2((size_t)nfreq * kChebN,
                                                                              make_double2(0.0, 0.0));
    std::vector<int> good, bad, terms(nfreq, 0);
    for (int f = 0; f < nfreq; ++f) {
      if (use_cheb && m.cheb != nullptr && m.cheb_n > 0 && m.cheb_R > 0.0) {
        const int nt = cheb_terms(k[f], m.cheb_R);
        if (nt > 0 && nt <= m.cheb_n &&
            cheb_coefficients(k[f], m.cheb_R, nt, &c1[(size_t)f * kChebN], &c2[(size_t)f * kChebN]))
          terms[f] = nt;
      }
      (terms[f] > 0 ? good : bad).push_back(f);
    }
    for (size_t g0 = 0; g0 < good.size(); g0 += 4) {
      const int w = (int)std::min<size_t>(4, good.size() - g0);
      const int threads = 128;
      const int nblk = (int)(((long long)m.npairs * 32 + threads - 1) / threads);
      auto run = [&](auto nfq_c) {
        constexpr int NFQ = decltype(nfq_c)::value;
        ChebParamsF32<NFQ> cp;
        int nmax = 0;
        for (int i = 0; i < NFQ; ++i) {
          const int f = good[g0 + i];
          cp.f[i] = params(f);
          cp.off[i] = (long long)f * blocks_stride;
          nmax = std::max(nmax, terms[f]);
          for (int n = 0; n < kChebN; ++n) {
            const double2 a = c1[(size_t)f * kChebN + n], b = c2[(size_t)f * kChebN + n];
            cp.c1[i][n] = n < terms[f] ? make_float2((float)a.x, (float)a.y) : make_float2(0.f, 0.f);
            cp.c2[i][n] = n < terms[f] ? make_float2((float)b.x, (float)b.y) : make_float2(0.f, 0.f);
          }
        }
        singular_cheb_f32_kernel<NFQ><<<nblk, threads, 0, stream>>>(m.pairs, m.npairs, m.pairrec, m.cheb, nmax, cp,
                                                                    (float2*)blocks);
      };
      if (w == 4)
        run(std::integral_constant<int, 4>{});
      else if (w == 3)
        run(std::integral_constant<int, 3>{});
      else if (w == 2)
        run(std::integral_constant<int, 2>{});
      else
        run(std::integral_constant<int, 1>{});
      ++nl;
      if (cheb_freqs) *cheb_freqs += w;
    }
    for (size_t i = 0; i < bad.size();) {
      size_t j = i + 1;
      while (j < bad.size() && bad[j] == bad[j - 1] + 1) ++j;
      direct(bad[i], (int)(j - i));
      i = j;
    }
    if (launched) *launched += nl;
    return cudaGetLastError();
  }
  const int threads = 256;
  const int nblk = (int)(((long long)m.npairs * 32 + threads - 1) / threads);
  for (int f = 0; f < nfreq; ++f) {
    SingParams<double> p;
    p.k = k[f];
    p.k2 = k[f] * k[f];
    p.cD = c[f].cD;
    p.cH = c[f].cH;
    p.cM = c[f].cM;
    p.cS = c[f].cS;
    p.cK = c[f].cK;
    p.cM10 = c[f].cM10;
    singular_dyn_kernel<double><<<nblk, threads, 0, stream>>>(geo, m.pairs, m.npairs, m.rule_ptr, m.duffy,
                                                              m.moments, m.curls, m.area, m.m11m10, p,
                                                              (double2*)blocks + (size_t)f * blocks_stride);
  }
  if (launched) *launched += nfreq;
  return cudaGetLastError();
}

cudaError_t launch_singular_scatter(const DeviceMesh& m, Precision prec, const void* blocks, void* Rext,
                                    long long ldR, cudaStream_t stream) {
  if (m.n_scat == 0) return cudaSuccess;
  const int threads = 256;
  const int nblk = (m.n_scat + threads - 1) / threads;
  if (prec == Precision::Mixed)
    singular_scatter_kernel<float2><<<nblk, threads, 0, stream>>>(m.scat_col, m.scat_row, m.scat_ptr, m.scat_src,
                                                                  m.n_scat, (const float2*)blocks, (float2*)Rext, ldR);
  else
    singular_scatter_kernel<double2><<<nblk, threads, 0, stream>>>(m.scat_col, m.scat_row, m.scat_ptr, m.scat_src,
                                                                   m.n_scat, (const double2*)blocks, (double2*)Rext,
                                                                   ldR);
  return cudaGetLastError();
}

cudaError_t launch_gather(const DeviceMesh& m, Precision prec, const void* Rext, long long ldR, void* A, long long lda,
                          void* A2, cudaStream_t stream) {
  const int threads = 256;
  const int n_halo = m.n_halo;
  if (prec == Precision::Mixed) {
    size_t sm = (size_t)std::max(1, n_halo) * sizeof(float2);
    if (sm > 48 * 1024) ensure_smem_limit((const void*)gather_columns_kernel<float2>, sm);
    gather_columns_kernel<float2><<<m.nv, threads, sm, stream>>>(
        (const float2*)Rext, ldR, m.col_ptr, m.col_fb, m.ext_row, m.halo_slot_of_ext, m.halo_row_ptr, m.halo_row,
        m.n_ext, m.n_halo_rows, (float2*)A, lda, (float2*)A2, 0, m.row_weight);
    if (m.n_isolated)
      isolated_identity_kernel<float2><<<(m.n_isolated + 127) / 128, 128, 0, stream>>>(
          m.isolated, m.n_isolated, m.vertex_row, (float2*)A, lda, (float2*)A2);
  } else {
    size_t sm = (size_t)std::max(1, n_halo) * sizeof(double2);
    if (sm > 48 * 1024) ensure_smem_limit((const void*)gather_columns_kernel<double2>, sm);
    gather_columns_kernel<double2><<<m.nv, threads, sm, stream>>>(
        (const double2*)Rext, ldR, m.col_ptr, m.col_fb, m.ext_row, m.halo_slot_of_ext, m.halo_row_ptr,
        m.halo_row, m.n_ext, m.n_halo_rows, (double2*)A, lda, (double2*)A2, 0, m.row_weight);
    if (m.n_isolated)
      isolated_identity_kernel<double2><<<(m.n_isolated + 127) / 128, 128, 0, stream>>>(
          m.isolated, m.n_isolated, m.vertex_row, (double2*)A, lda, (double2*)A2);
  }
  return cudaGetLastError();
}

cudaError_t launch_rhs(const DeviceMesh& m, Precision prec, double k, const OperatorCoeffs& c, double2 qscale,
                       const void* drive, int nc, const void* sblocks, void* rb, void* b, long long ldb,
                       cudaStream_t stream) {
  const int threads = 128;
  const int nblk = (int)(((long long)m.nf * 32 + threads - 1) / threads);
  if (prec == Precision::Mixed) {
    RhsParams<float> p;
    p.kdf = make_df(k);
    p.k = (float)k;
    p.cS = f2(c.cS);
    p.cK = f2(c.cK);
    p.qscale = f2(qscale);
    for (int i = 0; i < 3 * kMaxQ; ++i) p.cw[i] = (float)m.rule_cw[i];
#define BEM_RHS32(QQ, NCC)                                                                                   \
  rhs_faces_kernel<float, QQ, NCC><<<nblk, threads, 0, stream>>>(m.faces32, m.nf, m.driven, m.ndriven,        \
                                                                 (const float2*)drive, m.pairs,              \
                                                                 m.pairs_by_test_ptr, m.pairs_by_test,       \
                                                                 (const float2*)sblocks, p, (float2*)rb,     \
                                                                 m.ntr, make_int4(m.tr[0], m.tr[1], m.tr[2], \
                                                                 m.tr[3]), m.fix_mask)
#define BEM_RHS32_Q(NCC)        \
  if (m.Q == 6)                 \
    BEM_RHS32(6, NCC);          \
  else if (m.Q == 3)            \
    BEM_RHS32(3, NCC);          \
  else                          \
    BEM_RHS32(1, NCC);
    switch (nc) {
      case 1: BEM_RHS32_Q(1) break;
      case 2: BEM_RHS32_Q(2) break;
      case 3: BEM_RHS32_Q(3) break;
      case 4: BEM_RHS32_Q(4) break;
      default: return cudaErrorInvalidValue;
    }
    rhs_gather_kernel<float2><<<(m.nv + 127) / 128, 128, 0, stream>>>((const float2*)rb, m.nf, nc, m.col_ptr,
                                                                       m.col_fb, m.vertex_row, m.nv, (float2*)b,
                                                                       ldb, m.row_weight);
  } else {
    RhsParams<double> p;
    p.k = k;
    p.cS = c.cS;
    p.cK = c.cK;
    p.qscale = qscale;
    for (int i = 0; i < 3 * kMaxQ; ++i) p.cw[i] = m.rule_cw[i];
#define BEM_RHS64(QQ, NCC)                                                                                   \
  rhs_faces_kernel<double, QQ, NCC><<<nblk, threads, 0, stream>>>(m.faces64, m.nf, m.driven, m.ndriven,       \
                                                                  (const double2*)drive, m.pairs,            \
                                                                  m.pairs_by_test_ptr, m.pairs_by_test,      \
                                                                  (const double2*)sblocks, p, (double2*)rb,  \
                                                                  m.ntr, make_int4(m.tr[0], m.tr[1], m.tr[2], \
                                                                  m.tr[3]), m.fix_mask)
#define BEM_RHS64_Q(NCC)        \
  if (m.Q == 6)                 \
    BEM_RHS64(6, NCC);          \
  else if (m.Q == 3)            \
    BEM_RHS64(3, NCC);          \
  else                          \
    BEM_RHS64(1, NCC);
    switch (nc) {
      case 1: BEM_RHS64_Q(1) break;
      case 2: BEM_RHS64_Q(2) break;
      case 3: BEM_RHS64_Q(3) break;
      case 4: BEM_RHS64_Q(4) break;
      default: return cudaErrorInvalidValue;
    }
    rhs_gather_kernel<double2><<<(m.nv + 127) / 128, 128, 0, stream>>>((const double2*)rb, m.nf, nc, m.col_ptr,
                                                                        m.col_fb, m.vertex_row, m.nv,
                                                                        (double2*)b, ldb, m.row_weight);
  }
  return cudaGetLastError();
}

// Frequencies that share one right-hand-side launch: four with one excitation, two with
// two (the accumulators of NFQ x 3 x NC complex values stay in registers), else one.
int rhs_width(Precision prec, int nc) { return prec == Precision::Mixed ? (nc == 1 ? 4 : nc == 2 ? 2 : 1) : 1; }

cudaError_t launch_rhs_freqs(const DeviceMesh& m, Precision prec, int nfreq, const double* k, const OperatorCoeffs* c,
                             const double2* qscale, const void* drive, int nc, const void* sblocks,
                             long long sblocks_stride, void* rb, void* const* b, long long ldb, cudaStream_t stream) {
  const int width = rhs_width(prec, nc);
  const size_t esz = prec == Precision::Mixed ? sizeof(float2) : sizeof(double2);
  for (int f0 = 0; f0 < nfreq;) {
    const int w = std::min(width, nfreq - f0);
    if (w == 1) {
      const cudaError_t e = launch_rhs(m, prec, k[f0], c[f0], qscale[f0], drive, nc,
                                       (const char*)sblocks + (size_t)f0 * sblocks_stride * esz, rb, b[f0], ldb, stream);
      if (e != cudaSuccess) return e;
      ++f0;
      continue;
    }
    const int threads = 128;
    const int nblk = (int)(((long long)m.nf * 32 + threads - 1) / threads);
    const float2* sb = (const float2*)sblocks + (size_t)f0 * sblocks_stride;
    const int4 trs = make_int4(m.tr[0], m.tr[1], m.tr[2], m.tr[3]);
    auto run = [&](auto nfq_c, auto nc_c) {
      constexpr int NFQ = decltype(nfq_c)::value, NC = decltype(nc_c)::value;
      RhsParamsF32N<NFQ> p;
      for (int i = 0; i < NFQ; ++i) {
        p.kdf[i] = make_df(k[f0 + i]);
        p.k[i] = (float)k[f0 + i];
        p.cS[i] = f2(c[f0 + i].cS);
        p.cK[i] = f2(c[f0 + i].cK);
        p.qscale[i] = f2(qscale[f0 + i]);
      }
      for (int i = 0; i < 3 * kMaxQ; ++i) p.cw[i] = (float)m.rule_cw[i];
      auto go = [&](auto kern) {
        kern<<<nblk, threads, 0, stream>>>(m.faces32, m.nf, m.driven, m.ndriven, (const float2*)drive, m.pairs,
                                           m.pairs_by_test_ptr, m.pairs_by_test, sb, sblocks_stride, p, (float2*)rb,
                                           m.ntr, trs, m.fix_mask);
      };
      if (m.Q == 6)
        go(rhs_faces_f32_freqs_kernel<6, NC, NFQ>);
      else if (m.Q == 3)
        go(rhs_faces_f32_freqs_kernel<3, NC, NFQ>);
      else
        go(rhs_faces_f32_freqs_kernel<1, NC, NFQ>);
    };
    if (nc == 2)
      run(std::integral_constant<int, 2>{}, std::integral_constant<int, 2>{});
    else if (w == 4)
      run(std::integral_constant<int, 4>{}, std::integral_constant<int, 1>{});
    else if (w == 3)
      run(std::integral_constant<int, 3>{}, std::integral_constant<int, 1>{});
    else
      run(std::integral_constant<int, 2>{}, std::integral_constant<int, 1>{});
    for (int i = 0; i < w; ++i)
      rhs_gather_kernel<float2><<<(m.nv + 127) / 128, 128, 0, stream>>>(
          (const float2*)rb + (size_t)i * nc * m.nf * 3, m.nf, nc, m.col_ptr, m.col_fb, m.vertex_row, m.nv,
          (float2*)b[f0 + i], ldb, m.row_weight);
    f0 += w;
  }
  return cudaGetLastError();
}

// Kernel launches of launch_rhs_freqs for nfreq frequencies.
int rhs_launches(Precision prec, int nc, int nfreq) {
  const int width = rhs_width(prec, nc);
  return nfreq + (nfreq + width - 1) / width;  // one gather per frequency, one face kernel per group
}

}  // namespace bem
