// Exterior field evaluation (sm_103a).
//
// u(x) = sum over source points y_s of [dG/dn_y(x, y_s) p(y_s) - G(x, y_s) q_s] w_s
// with the sources at the regular quadrature points of every face, p
// interpolated with the P1 basis and q the DP0 Neumann data: the reference's
// evaluate_galerkin_field_cpu (src/blab/solvers/julia_local/src/
// BeatEngineCpuField.jl:1-45) over build_field_evaluation_cache
// (BeatEngineCore.jl:1240-1280, symmetry off).  The reference's CUDA version
// uses one block per observation point with an FP32 shared-memory reduction
// (BeatEngineCudaField.jl:102-189).
//
// Here: a prologue kernel forms the weighted sources p_s w_s (all frequencies
// and excitations of a batch), then the FP32 kernel runs one CTA per (32
// observation points, frequency) and the FP64 kernel one CTA per (observation
// point, frequency), each sweeping the faces.  The mixed form uses the same compensated
// phase as the assembly (double-float k|c_g - x| per face, FP32 correction per
// point), Kahan-compensated FP32 partial sums per thread and an FP64 block
// reduction; the far field sits at kr ~ 500 rad at 16 kHz, where plain FP32
// phase would lose ~3e-5 rad.
#include "bem_common.cuh"
#include "bem_kernels.h"

namespace bem {
namespace {

// Rule weights w_q and basis values phi_a(xi_q) (a-major), passed by value.
template <typename R> struct FieldRule {
  R w[kMaxQ];
  R phi[3 * kMaxQ];
};

// sources[((bt*nc + c)*nf + g)*Q + q] = 2A_g w_q sum_a phi_a(xi_q) p[bt][c][v(g,a)]
template <typename R>
__global__ void field_sources_kernel(const int* __restrict__ faces, const double* __restrict__ area, int nf, int Q,
                                     int nc, const typename cplx<R>::type* __restrict__ p, long long ldp,
                                     typename cplx<R>::type* __restrict__ src, int total, FieldRule<R> fr) {
  typedef typename cplx<R>::type C2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int q = i % Q;
  const int g = (i / Q) % nf;
  const int bc = i / (Q * nf);  // bt*nc + c
  const C2* pv = p + (size_t)bc * ldp;
  const R w = fr.w[q], phi0 = fr.phi[q], phi1 = fr.phi[Q + q], phi2 = fr.phi[2 * Q + q];
  const C2 a = pv[faces[3 * g]], b = pv[faces[3 * g + 1]], c = pv[faces[3 * g + 2]];
  const R s = (R)(2.0 * area[g]) * w;
  C2 v;
  v.x = (phi0 * a.x + phi1 * b.x + phi2 * c.x) * s;
  v.y = (phi0 * a.y + phi1 * b.y + phi2 * c.y) * s;
  src[i] = v;
}

struct FieldParamsF32 {
  df kdf[64];
  float k[64];
  float2 qscale[64];
};

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  float y = x - c;
  float t = s + y;
  c = (t - s) - y;
  s = t;
}

// One CTA per (32 observation points, frequency): lane = observation point,
// warp w sweeps faces w, w + 8, ...  Every lane of a warp works on the same
// face, so face records, sources and drives are broadcast loads, and the
// compensated phase set-up (double-float k|c_g - x|) is done once per
// (point, face).  The Q point terms of a face are summed in FP32 and added to
// a Kahan-compensated per-lane sum; the 8 warps' sums are added in FP64.
constexpr int kFieldWarps = 8;

template <int Q, int NC>
__global__ void __launch_bounds__(256) field_f32_kernel(const FaceF32* __restrict__ faces, int nf,
                                                        const float2* __restrict__ src,
                                                        const float2* __restrict__ drive,  // NC x nf
                                                        const double* __restrict__ obs, int nobs,
                                                        const FieldParamsF32* __restrict__ prm,
                                                        double2* __restrict__ out, FieldRule<float> fr, int ntr,
                                                        int4 trs) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int o = blockIdx.x * 32 + lane, bt = blockIdx.y;
  const bool live = o < nobs;
  const int oc = live ? o : nobs - 1;  // idle lanes repeat a live point; their result is dropped
  const double xo[3] = {obs[3 * oc], obs[3 * oc + 1], obs[3 * oc + 2]};
  float xhi[3], xlo[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    xhi[d] = (float)xo[d];
    xlo[d] = (float)(xo[d] - (double)xhi[d]);
  }
  const df kdf = prm->kdf[bt];
  const float k = prm->k[bt];
  const float2 qs = prm->qscale[bt];
  float ar[NC], ac[NC], br[NC], bcmp[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    ar[c] = 0.f;
    ac[c] = 0.f;
    br[c] = 0.f;
    bcmp[c] = 0.f;
  }
  // sources: every face and, under symmetry, its images (BeatEngineCore.jl:1240-1280)
  for (int ti = 0; ti < ntr; ++ti)
  for (int g = wid; g < nf; g += kFieldWarps) {
    const FaceF32& F = faces[g];
    const int tr = ti == 0 ? trs.x : ti == 1 ? trs.y : ti == 2 ? trs.z : trs.w;
    const float sg[3] = {(tr & 1) ? -1.f : 1.f, (tr & 2) ? -1.f : 1.f, 1.f};
    const float nrm[3] = {sg[0] * F.normal[0], sg[1] * F.normal[1], F.normal[2]};
    // base phase k|c_g - x| in double-float
    df C[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      df s = two_sum(sg[d] * F.anchor_hi[d], -xhi[d]);
      s.lo += sg[d] * F.anchor_lo[d] - xlo[d];
      C[d] = quick_two_sum(s.hi, s.lo);
    }
    df r2 = df_add(df_add(df_mul(C[0], C[0]), df_mul(C[1], C[1])), df_mul(C[2], C[2]));
    df R = df_sqrt(r2);
    const float R0 = R.hi + R.lo;
    const float theta0 = df_reduce_two_pi(df_mul(kdf, R));
    const float Cf[3] = {C[0].hi + C[0].lo, C[1].hi + C[1].lo, C[2].hi + C[2].lo};
    const float Cn = fmaf(Cf[0], nrm[0], fmaf(Cf[1], nrm[1], Cf[2] * nrm[2]));
    float2 qg[NC], fs[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      qg[c] = cscale(cmul(qs, drive[(size_t)c * nf + g]), F.area2);
      fs[c] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int n = 0; n < Q; ++n) {
      const float d[3] = {sg[0] * F.off[3 * n], sg[1] * F.off[3 * n + 1], F.off[3 * n + 2]};
      const float rv[3] = {Cf[0] + d[0], Cf[1] + d[1], Cf[2] + d[2]};
      const float rr = fmaf(rv[0], rv[0], fmaf(rv[1], rv[1], rv[2] * rv[2]));
      const float rinv = rr > 1e-30f ? rsqrt_ftz(rr) : 0.f;
      const float r = rr * rinv;
      const float cd = fmaf(Cf[0], d[0], fmaf(Cf[1], d[1], Cf[2] * d[2]));
      const float dd = fmaf(d[0], d[0], fmaf(d[1], d[1], d[2] * d[2]));
      const float delta = fmaf(2.f, cd, dd) * rcp_ftz(fmaxf(r + R0, 1e-30f));
      const float th = reduce_two_pi(fmaf(k, delta, theta0));
      float sn, cs;
      sincos_ftz(th, &sn, &cs);
      const float sc = rinv * BEM_INV_FOUR_PI;
      const float2 G = make_float2(cs * sc, sn * sc);
      // (r . n_y) / r with r . n_y = C . n + d . n (d . n = 0 for points on the face plane, kept for generality)
      const float t = (Cn + fmaf(d[0], nrm[0], fmaf(d[1], nrm[1], d[2] * nrm[2]))) * rinv;
      const float2 Dk = make_float2(t * (-G.x * rinv - G.y * k), t * (G.x * k - G.y * rinv));
      const float wn = fr.w[n];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const float2 ps = src[(((size_t)bt * NC + c) * nf + g) * Q + n];
        const float2 qq = cscale(qg[c], wn);
        fs[c] = cadd(fs[c], csub(cmul(Dk, ps), cmul(G, qq)));
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      kahan_add(ar[c], ac[c], fs[c].x);
      kahan_add(br[c], bcmp[c], fs[c].y);
    }
  }
  __shared__ double2 red[kFieldWarps][NC][32];
#pragma unroll
  for (int c = 0; c < NC; ++c)
    red[wid][c][lane] = make_double2((double)ar[c] - (double)ac[c], (double)br[c] - (double)bcmp[c]);
  __syncthreads();
  if (wid == 0 && live) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double vr = 0.0, vi = 0.0;
      for (int w = 0; w < kFieldWarps; ++w) {
        vr += red[w][c][lane].x;
        vi += red[w][c][lane].y;
      }
      out[((size_t)bt * NC + c) * nobs + o] = make_double2(vr, vi);
    }
  }
}

// The same sums for NFQ frequencies of a batch per CTA (blockIdx.y = group of
// NFQ frequencies starting at NFQ * blockIdx.y).  Everything that does not
// depend on the frequency is formed once per (point, face) and once per
// (point, source) and shared by the NFQ frequencies: the double-float
// distance |c_g - x| to the face anchor, the FP32 offset geometry, 1/r, the
// compensated r - |c_g - x| and the normal derivative factor t.  Per frequency
// remain the reduction of k|c_g - x|, the phase of each source, e^{ikr} and the
// accumulation, with the arithmetic and the order of every sum of
// field_f32_kernel.  Frequencies of
// the last group beyond the batch are computed on the batch's last frequency and
// not stored.
template <int Q, int NC, int NFQ>
__global__ void __launch_bounds__(256) field_f32_freqs_kernel(const FaceF32* __restrict__ faces, int nf,
                                                              const float2* __restrict__ src,
                                                              const float2* __restrict__ drive,  // NC x nf
                                                              const double* __restrict__ obs, int nobs,
                                                              const FieldParamsF32* __restrict__ prm, int batch,
                                                              double2* __restrict__ out, FieldRule<float> fr, int ntr,
                                                              int4 trs) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int o = blockIdx.x * 32 + lane;
  const int f0 = blockIdx.y * NFQ;
  const bool live = o < nobs;
  const int oc = live ? o : nobs - 1;  // idle lanes repeat a live point; their result is dropped
  const double xo[3] = {obs[3 * oc], obs[3 * oc + 1], obs[3 * oc + 2]};
  float xhi[3], xlo[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    xhi[d] = (float)xo[d];
    xlo[d] = (float)(xo[d] - (double)xhi[d]);
  }
  int bt[NFQ];
  df kdf[NFQ];
  float k[NFQ];
  float2 qs[NFQ];
#pragma unroll
  for (int f = 0; f < NFQ; ++f) {
    bt[f] = min(f0 + f, batch - 1);
    kdf[f] = prm->kdf[bt[f]];
    k[f] = prm->k[bt[f]];
    qs[f] = prm->qscale[bt[f]];
  }
  float ar[NFQ][NC], ac[NFQ][NC], br[NFQ][NC], bcmp[NFQ][NC];
#pragma unroll
  for (int f = 0; f < NFQ; ++f)
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      ar[f][c] = 0.f;
      ac[f][c] = 0.f;
      br[f][c] = 0.f;
      bcmp[f][c] = 0.f;
    }
  for (int ti = 0; ti < ntr; ++ti)
  for (int g = wid; g < nf; g += kFieldWarps) {
    const FaceF32& F = faces[g];
    const int tr = ti == 0 ? trs.x : ti == 1 ? trs.y : ti == 2 ? trs.z : trs.w;
    const float sg[3] = {(tr & 1) ? -1.f : 1.f, (tr & 2) ? -1.f : 1.f, 1.f};
    const float nrm[3] = {sg[0] * F.normal[0], sg[1] * F.normal[1], F.normal[2]};
    df C[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      df s = two_sum(sg[d] * F.anchor_hi[d], -xhi[d]);
      s.lo += sg[d] * F.anchor_lo[d] - xlo[d];
      C[d] = quick_two_sum(s.hi, s.lo);
    }
    df r2 = df_add(df_add(df_mul(C[0], C[0]), df_mul(C[1], C[1])), df_mul(C[2], C[2]));
    df R = df_sqrt(r2);
    const float R0 = R.hi + R.lo;
    float theta0[NFQ];
#pragma unroll
    for (int f = 0; f < NFQ; ++f) theta0[f] = df_reduce_two_pi(df_mul(kdf[f], R));
    const float Cf[3] = {C[0].hi + C[0].lo, C[1].hi + C[1].lo, C[2].hi + C[2].lo};
    const float Cn = fmaf(Cf[0], nrm[0], fmaf(Cf[1], nrm[1], Cf[2] * nrm[2]));
    float2 qg[NFQ][NC], fs[NFQ][NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const float2 dr = drive[(size_t)c * nf + g];
#pragma unroll
      for (int f = 0; f < NFQ; ++f) {
        qg[f][c] = cscale(cmul(qs[f], dr), F.area2);
        fs[f][c] = make_float2(0.f, 0.f);
      }
    }
#pragma unroll
    for (int n = 0; n < Q; ++n) {
      const float d[3] = {sg[0] * F.off[3 * n], sg[1] * F.off[3 * n + 1], F.off[3 * n + 2]};
      const float rv[3] = {Cf[0] + d[0], Cf[1] + d[1], Cf[2] + d[2]};
      const float rr = fmaf(rv[0], rv[0], fmaf(rv[1], rv[1], rv[2] * rv[2]));
      const float rinv = rr > 1e-30f ? rsqrt_ftz(rr) : 0.f;
      const float r = rr * rinv;
      const float cd = fmaf(Cf[0], d[0], fmaf(Cf[1], d[1], Cf[2] * d[2]));
      const float dd = fmaf(d[0], d[0], fmaf(d[1], d[1], d[2] * d[2]));
      const float delta = fmaf(2.f, cd, dd) * rcp_ftz(fmaxf(r + R0, 1e-30f));
      const float sc = rinv * BEM_INV_FOUR_PI;
      const float t = (Cn + fmaf(d[0], nrm[0], fmaf(d[1], nrm[1], d[2] * nrm[2]))) * rinv;
      const float wn = fr.w[n];
#pragma unroll
      for (int f = 0; f < NFQ; ++f) {
        const float th = reduce_two_pi(fmaf(k[f], delta, theta0[f]));
        float sn, cs;
        sincos_ftz(th, &sn, &cs);
        const float2 G = make_float2(cs * sc, sn * sc);
        const float2 Dk = make_float2(t * (-G.x * rinv - G.y * k[f]), t * (G.x * k[f] - G.y * rinv));
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const float2 ps = src[(((size_t)bt[f] * NC + c) * nf + g) * Q + n];
          const float2 qq = cscale(qg[f][c], wn);
          fs[f][c] = cadd(fs[f][c], csub(cmul(Dk, ps), cmul(G, qq)));
        }
      }
    }
#pragma unroll
    for (int f = 0; f < NFQ; ++f)
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        kahan_add(ar[f][c], ac[f][c], fs[f][c].x);
        kahan_add(br[f][c], bcmp[f][c], fs[f][c].y);
      }
  }
  __shared__ double2 red[kFieldWarps][NC][32];
#pragma unroll
  for (int f = 0; f < NFQ; ++f) {
#pragma unroll
    for (int c = 0; c < NC; ++c)
      red[wid][c][lane] =
          make_double2((double)ar[f][c] - (double)ac[f][c], (double)br[f][c] - (double)bcmp[f][c]);
    __syncthreads();
    if (wid == 0 && live && f0 + f < batch) {
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        double vr = 0.0, vi = 0.0;
        for (int w = 0; w < kFieldWarps; ++w) {
          vr += red[w][c][lane].x;
          vi += red[w][c][lane].y;
        }
        out[((size_t)(f0 + f) * NC + c) * nobs + o] = make_double2(vr, vi);
      }
    }
    __syncthreads();
  }
}

struct FieldParamsF64 {
  double k[64];
  double2 qscale[64];
};

template <int Q, int NC>
__global__ void __launch_bounds__(256) field_f64_kernel(const FaceF64* __restrict__ faces, int nf,
                                                        const double2* __restrict__ src,
                                                        const double2* __restrict__ drive,
                                                        const double* __restrict__ obs, int nobs,
                                                        const FieldParamsF64* __restrict__ prm,
                                                        double2* __restrict__ out, FieldRule<double> fr, int ntr,
                                                        int4 trs) {
  const int o = blockIdx.x, bt = blockIdx.y;
  const double xo[3] = {obs[3 * o], obs[3 * o + 1], obs[3 * o + 2]};
  const double k = prm->k[bt];
  const double2 qs = prm->qscale[bt];
  double2 acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = make_double2(0., 0.);
  for (int ti = 0; ti < ntr; ++ti)  // every face and its symmetry images
  for (int g = threadIdx.x; g < nf; g += blockDim.x) {
    const FaceF64& F = faces[g];
    const int tr = ti == 0 ? trs.x : ti == 1 ? trs.y : ti == 2 ? trs.z : trs.w;
    const double sg[3] = {(tr & 1) ? -1.0 : 1.0, (tr & 2) ? -1.0 : 1.0, 1.0};
    double2 qg[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) qg[c] = cscale(cmul(qs, drive[(size_t)c * nf + g]), F.area2);
#pragma unroll
    for (int n = 0; n < Q; ++n) {
      double rv[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) rv[d] = (sg[d] * F.anchor[d] - xo[d]) + sg[d] * F.off[3 * n + d];
      const double rr = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
      if (rr == 0.0) continue;
      const double r = sqrt(rr), rinv = 1.0 / r;
      double sn, cs;
      sincos(k * r, &sn, &cs);
      const double sc = rinv * (0.25 / CUDART_PI);
      const double2 G = make_double2(cs * sc, sn * sc);
      const double t = (rv[0] * sg[0] * F.normal[0] + rv[1] * sg[1] * F.normal[1] + rv[2] * F.normal[2]) * rinv;
      const double2 Dk = make_double2(t * (-G.x * rinv - G.y * k), t * (G.x * k - G.y * rinv));
      const double wn = fr.w[n];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const double2 ps = src[(((size_t)bt * NC + c) * nf + g) * Q + n];
        const double2 qq = cscale(qg[c], wn);
        acc[c] = cadd(acc[c], csub(cmul(Dk, ps), cmul(G, qq)));
      }
    }
  }
  __shared__ double red[2 * NC][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    double vr = acc[c].x, vi = acc[c].y;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      vr += __shfl_xor_sync(0xffffffffu, vr, s);
      vi += __shfl_xor_sync(0xffffffffu, vi, s);
    }
    if (lane == 0) {
      red[2 * c][wid] = vr;
      red[2 * c + 1][wid] = vi;
    }
  }
  __syncthreads();
  if (threadIdx.x < NC) {
    const int c = threadIdx.x;
    double vr = 0, vi = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      vr += red[2 * c][w];
      vi += red[2 * c + 1][w];
    }
    out[((size_t)bt * NC + c) * nobs + o] = make_double2(vr, vi);
  }
}

}  // namespace

static df host_df(double x) {
  df r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}

cudaError_t launch_field(const DeviceMesh& m, Precision prec, int batch, const double* k, const double2* qscale,
                         const void* pressure, long long ldp, int nc, const void* drive, const double* obs, int nobs,
                         void* sources, double2* out, cudaStream_t stream) {
  if (batch > 64 || nc < 1 || nc > 4 || nobs <= 0) return cudaErrorInvalidValue;
  FieldRule<float> fr32;
  FieldRule<double> fr64;
  for (int i = 0; i < kMaxQ; ++i) {
    fr32.w[i] = (float)m.rule_w[i];
    fr64.w[i] = m.rule_w[i];
  }
  for (int i = 0; i < 3 * kMaxQ; ++i) {
    fr32.phi[i] = (float)m.rule_phi[i];
    fr64.phi[i] = m.rule_phi[i];
  }
  const int total = batch * nc * m.nf * m.Q;
  dim3 grid(nobs, batch);
  if (prec == Precision::Mixed) {
    field_sources_kernel<float><<<(total + 255) / 256, 256, 0, stream>>>(m.faces, m.area, m.nf, m.Q, nc,
                                                                         (const float2*)pressure, ldp,
                                                                         (float2*)sources, total, fr32);
    FieldParamsF32 hp;
    for (int b = 0; b < batch; ++b) {
      hp.kdf[b] = host_df(k[b]);
      hp.k[b] = (float)k[b];
      hp.qscale[b] = make_float2((float)qscale[b].x, (float)qscale[b].y);
    }
    FieldParamsF32* dp = (FieldParamsF32*)((char*)sources + (((size_t)total * sizeof(float2) + 255) / 256) * 256);
    cudaMemcpyAsync(dp, &hp, sizeof(hp), cudaMemcpyHostToDevice, stream);
    // NFQ frequencies per CTA share the frequency-independent geometry; the
    // largest NFQ (4 or 2, NFQ x nc <= 4) whose grid still gives every SM a CTA
    // (at 10k with 2,146 points and 15 frequencies: four per CTA, 272 CTAs, field
    // 0.36 -> 0.30 ms per frequency against the twice-filled grid of two per CTA)
    const long long pt_blocks = (nobs + 31) / 32;
    int nfq = 1;
    for (int cand = 4; cand >= 2; cand /= 2)
      if (cand * nc <= 4 && cand <= batch && pt_blocks * ((batch + cand - 1) / cand) >= (long long)sm_count()) {
        nfq = cand;
        break;
      }
    const int4 trs = make_int4(m.tr[0], m.tr[1], m.tr[2], m.tr[3]);
    auto run = [&](auto kern, int nf_per_cta) {
      dim3 g((unsigned)pt_blocks, (unsigned)((batch + nf_per_cta - 1) / nf_per_cta));
      kern<<<g, 256, 0, stream>>>(m.faces32, m.nf, (const float2*)sources, (const float2*)drive, obs, nobs, dp,
                                  batch, out, fr32, m.ntr, trs);
    };
#define BEM_F32(QQ, NCC, NFQQ) run(field_f32_freqs_kernel<QQ, NCC, NFQQ>, NFQQ)
#define BEM_F32_Q(NCC, NFQQ) \
  if (m.Q == 6)              \
    BEM_F32(6, NCC, NFQQ);   \
  else if (m.Q == 3)         \
    BEM_F32(3, NCC, NFQQ);   \
  else                       \
    BEM_F32(1, NCC, NFQQ);
    if (nc == 1 && nfq == 4) {
      BEM_F32_Q(1, 4)
    } else if (nc == 1 && nfq == 2) {
      BEM_F32_Q(1, 2)
    } else if (nc == 2 && nfq == 2) {
      BEM_F32_Q(2, 2)
    } else {
      switch (nc) {
        case 1: BEM_F32_Q(1, 1) break;
        case 2: BEM_F32_Q(2, 1) break;
        case 3: BEM_F32_Q(3, 1) break;
        default: BEM_F32_Q(4, 1) break;
      }
    }
#undef BEM_F32_Q
#undef BEM_F32
  } else {
    field_sources_kernel<double><<<(total + 255) / 256, 256, 0, stream>>>(m.faces, m.area, m.nf, m.Q, nc,
                                                                          (const double2*)pressure, ldp,
                                                                          (double2*)sources, total, fr64);
    FieldParamsF64 hp;
    for (int b = 0; b < batch; ++b) {
      hp.k[b] = k[b];
      hp.qscale[b] = qscale[b];
    }
    FieldParamsF64* dp = (FieldParamsF64*)((char*)sources + (((size_t)total * sizeof(double2) + 255) / 256) * 256);
    cudaMemcpyAsync(dp, &hp, sizeof(hp), cudaMemcpyHostToDevice, stream);
#define BEM_F64(QQ, NCC)                                                                                   \
  field_f64_kernel<QQ, NCC><<<grid, 256, 0, stream>>>(m.faces64, m.nf, (const double2*)sources,            \
                                                      (const double2*)drive, obs, nobs, dp, out, fr64, m.ntr, \
                                                      make_int4(m.tr[0], m.tr[1], m.tr[2], m.tr[3]))
#define BEM_F64_Q(NCC)    \
  if (m.Q == 6)           \
    BEM_F64(6, NCC);      \
  else if (m.Q == 3)      \
    BEM_F64(3, NCC);      \
  else                    \
    BEM_F64(1, NCC);
    switch (nc) {
      case 1: BEM_F64_Q(1) break;
      case 2: BEM_F64_Q(2) break;
      case 3: BEM_F64_Q(3) break;
      default: BEM_F64_Q(4) break;
    }
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Single-excitation, single-frequency field evaluation from caller-placed
// buffers (face records, weighted sources, drive, parameter block).  Used by
// the allocation-free entry point in bem_noalloc.cu; the parameter block is
// written on the device by write_field_params so no host staging is needed.
namespace {
__global__ void write_field_params_f32(FieldParamsF32* prm, double k) {
  df v;
  v.hi = (float)k;
  v.lo = (float)(k - (double)v.hi);
  prm->kdf[0] = v;
  prm->k[0] = (float)k;
  prm->qscale[0] = make_float2(1.0f, 0.0f);
}
__global__ void write_field_params_f64(FieldParamsF64* prm, double k) {
  prm->k[0] = k;
  prm->qscale[0] = make_double2(1.0, 0.0);
}
}  // namespace

size_t field_params_bytes() { return sizeof(FieldParamsF32) > sizeof(FieldParamsF64) ? sizeof(FieldParamsF32) : sizeof(FieldParamsF64); }

cudaError_t launch_field_single(Precision prec, const void* faces, int nf, int Q, const double* rule_w,
                                const double* rule_phi, const void* sources, const void* drive, const double* obs,
                                int nobs, double k, void* params, double2* out, cudaStream_t stream) {
  FieldRule<float> fr32;
  FieldRule<double> fr64;
  for (int i = 0; i < kMaxQ; ++i) {
    fr32.w[i] = (float)rule_w[i];
    fr64.w[i] = rule_w[i];
  }
  for (int i = 0; i < 3 * kMaxQ; ++i) {
    fr32.phi[i] = (float)rule_phi[i];
    fr64.phi[i] = rule_phi[i];
  }
  dim3 grid(nobs, 1);
  dim3 grid32((nobs + 31) / 32, 1);
  if (prec == Precision::Mixed) {
    FieldParamsF32* dp = (FieldParamsF32*)params;
    write_field_params_f32<<<1, 1, 0, stream>>>(dp, k);
    const FaceF32* f = (const FaceF32*)faces;
    const float2* s = (const float2*)sources;
    const float2* d = (const float2*)drive;
    if (Q == 6)
      field_f32_kernel<6, 1><<<grid32, 256, 0, stream>>>(f, nf, s, d, obs, nobs, dp, out, fr32, 1, make_int4(0, 0, 0, 0));
    else if (Q == 3)
      field_f32_kernel<3, 1><<<grid32, 256, 0, stream>>>(f, nf, s, d, obs, nobs, dp, out, fr32, 1, make_int4(0, 0, 0, 0));
    else
      field_f32_kernel<1, 1><<<grid32, 256, 0, stream>>>(f, nf, s, d, obs, nobs, dp, out, fr32, 1, make_int4(0, 0, 0, 0));
  } else {
    FieldParamsF64* dp = (FieldParamsF64*)params;
    write_field_params_f64<<<1, 1, 0, stream>>>(dp, k);
    const FaceF64* f = (const FaceF64*)faces;
    const double2* s = (const double2*)sources;
    const double2* d = (const double2*)drive;
    if (Q == 6)
      field_f64_kernel<6, 1><<<grid, 256, 0, stream>>>(f, nf, s, d, obs, nobs, dp, out, fr64, 1, make_int4(0, 0, 0, 0));
    else if (Q == 3)
      field_f64_kernel<3, 1><<<grid, 256, 0, stream>>>(f, nf, s, d, obs, nobs, dp, out, fr64, 1, make_int4(0, 0, 0, 0));
    else
      field_f64_kernel<1, 1><<<grid, 256, 0, stream>>>(f, nf, s, d, obs, nobs, dp, out, fr64, 1, make_int4(0, 0, 0, 0));
  }
  return cudaGetLastError();
}

}  // namespace bem
