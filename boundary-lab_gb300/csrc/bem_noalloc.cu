// Exterior field evaluation for callers that cannot allocate device memory.
//
// Some hosts of this library are not allowed to call cudaMalloc at the point
// where they need a field: an audio plug-in's real-time processing callback
// (an allocation can block for an unbounded time and must not happen there),
// or a framework that owns all device memory through its own pool and forbids
// raw allocations.  bem_evaluate_field_noalloc serves them: the caller passes
// every input and output as a device buffer it already owns, and the only
// other memory the call touches is one fixed scratch array compiled into the
// library (g_field_scratch below).
//
// Consequences a caller must know:
//  * The scratch array exists once per GPU for the life of the process
//    (kNoAllocScratchBytes, ~6.5 MB), whether or not the entry point is used.
//  * Every call shares it.  Two calls whose work overlaps on the GPU (different
//    streams, or different host threads on the same device) race on it and can
//    return wrong fields; serialise them.  A call leaves the scratch holding its
//    own face records and sources; nothing in it has to start at zero, because
//    each call writes every scratch entry it later reads.
//  * The first call on a device looks up the device address of the scratch
//    array (cudaGetSymbolAddress) with that device current.  The address is kept
//    for the life of the process: do not use the entry point across a
//    cudaDeviceReset of that device.  The stream must belong to the current
//    device (checked).
//  * Each call waits for its stream (cudaStreamSynchronize) before it returns,
//    to read the mesh check the kernels wrote.
//  * On an error return the contents of d_field_out are undefined (a bad mesh
//    is reported after the field kernels ran).
//  * Limits: n_faces <= kNoAllocMaxFaces; larger meshes are rejected with
//    BEM_ERR_INVALID_ARGUMENT and a message.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/gb300_bem.h"
#include "bem_common.cuh"
#include "bem_internal.h"
#include "bem_kernels.h"

namespace bem {
namespace {

constexpr int kNoAllocMaxFaces = 16384;
constexpr int kMaxDevices = 64;
constexpr size_t kRecordBytes = (size_t)kNoAllocMaxFaces * sizeof(FaceF64);         // face records
constexpr size_t kSourceBytes = (size_t)kNoAllocMaxFaces * kMaxQ * sizeof(double2);  // weighted sources
constexpr size_t kDriveBytes = (size_t)kNoAllocMaxFaces * sizeof(double2);           // Neumann data
constexpr size_t kParamBytes = 4096;                                                 // field parameter block
constexpr size_t kNoAllocScratchBytes = kRecordBytes + kSourceBytes + kDriveBytes + kParamBytes;

// Host code only ever sees this name as a stand-in: the kernels receive the
// device address obtained with cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_field_scratch[kNoAllocScratchBytes];

std::mutex g_lookup_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Regular rule as in the reference's triangle_rule (BeatEngineCore.jl:517-549).
void rule_for(int order, double* pts, double* w, int& Q) {
  static const double p4[12] = {0.4459484909159651, 0.4459484909159651, 0.0915762135097710, 0.0915762135097700,
                                0.1081030181680700, 0.4459484909159651, 0.4459484909159651, 0.1081030181680700,
                                0.8168475729804590, 0.0915762135097700, 0.0915762135097710, 0.8168475729804580};
  static const double w4[6] = {0.2233815896780110, 0.1099517436553220, 0.2233815896780110,
                               0.2233815896780110, 0.1099517436553220, 0.1099517436553220};
  if (order <= 1) {
    Q = 1;
    pts[0] = pts[1] = 1.0 / 3.0;
    w[0] = 0.5;
  } else if (order == 4) {
    Q = 6;
    for (int i = 0; i < 12; ++i) pts[i] = p4[i];
    for (int i = 0; i < 6; ++i) w[i] = 0.5 * w4[i];
  } else {
    Q = 3;
    const double p3[6] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
    for (int i = 0; i < 6; ++i) pts[i] = p3[i];
    for (int i = 0; i < 3; ++i) w[i] = 1.0 / 6.0;
  }
}

struct RulePts {
  double p[2 * kMaxQ];
};

// Face records from raw vertices/faces (the same geometry as the host planner,
// evaluated on the device in FP64).
template <bool F32>
__global__ void noalloc_face_records(const double* __restrict__ verts, int nv, const int* __restrict__ faces, int nf,
                                     int Q, RulePts rp, void* records, int* bad) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  int i0 = faces[3 * f], i1 = faces[3 * f + 1], i2 = faces[3 * f + 2];
  if (i0 < 0 || i0 >= nv || i1 < 0 || i1 >= nv || i2 < 0 || i2 >= nv) {
    atomicExch(bad, 2);  // index out of range: record a harmless face, report, skip the reads
    i0 = i1 = i2 = 0;
  }
  double v[3][3];
  for (int d = 0; d < 3; ++d) {
    v[0][d] = verts[3 * i0 + d];
    v[1][d] = verts[3 * i1 + d];
    v[2][d] = verts[3 * i2 + d];
  }
  const double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
  const double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
  const double cp[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
  const double nn = sqrt(cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2]);
  if (!(nn > 0.0)) atomicMax(bad, 1);
  const double c[3] = {(v[0][0] + v[1][0] + v[2][0]) / 3.0, (v[0][1] + v[1][1] + v[2][1]) / 3.0,
                       (v[0][2] + v[1][2] + v[2][2]) / 3.0};
  if (F32) {
    FaceF32& R = ((FaceF32*)records)[f];
    for (int d = 0; d < 3; ++d) {
      R.anchor_hi[d] = (float)c[d];
      R.anchor_lo[d] = (float)(c[d] - (double)R.anchor_hi[d]);
      R.normal[d] = (float)(cp[d] / nn);
    }
    R.area2 = (float)nn;
    for (int i = 0; i < 9; ++i) R.curls[i] = 0.0f;
    for (int q = 0; q < kMaxQ; ++q)
      for (int d = 0; d < 3; ++d) {
        const double u = rp.p[2 * q], w = rp.p[2 * q + 1];
        R.off[3 * q + d] = q < Q ? (float)(((1.0 - u - w) * v[0][d] + u * v[1][d] + w * v[2][d]) - c[d]) : 0.0f;
      }
    R.verts[0] = i0;
    R.verts[1] = i1;
    R.verts[2] = i2;
  } else {
    FaceF64& R = ((FaceF64*)records)[f];
    for (int d = 0; d < 3; ++d) {
      R.anchor[d] = c[d];
      R.normal[d] = cp[d] / nn;
    }
    R.area2 = nn;
    for (int i = 0; i < 9; ++i) R.curls[i] = 0.0;
    for (int q = 0; q < kMaxQ; ++q)
      for (int d = 0; d < 3; ++d) {
        const double u = rp.p[2 * q], w = rp.p[2 * q + 1];
        R.off[3 * q + d] = q < Q ? ((1.0 - u - w) * v[0][d] + u * v[1][d] + w * v[2][d]) - c[d] : 0.0;
      }
    R.verts[0] = i0;
    R.verts[1] = i1;
    R.verts[2] = i2;
    R.pad = 0;
  }
}

struct RuleWP {
  double w[kMaxQ];
  double phi[3 * kMaxQ];
};

// Weighted sources 2A_g w_q sum_a phi_a(xi_q) p[v(g,a)] and the drive (Neumann
// data) in the working precision.
template <typename C2>
__global__ void noalloc_sources(const int* __restrict__ faces, int nv, const void* __restrict__ records, int nf,
                                int Q, const double2* __restrict__ p, const double2* __restrict__ q, RuleWP r,
                                bool f32, C2* __restrict__ src, C2* __restrict__ drive) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf * Q) return;
  const int g = i / Q, qq = i - g * Q;
  const double area2 = f32 ? (double)((const FaceF32*)records)[g].area2 : ((const FaceF64*)records)[g].area2;
  int i0 = faces[3 * g], i1 = faces[3 * g + 1], i2 = faces[3 * g + 2];
  if (i0 < 0 || i0 >= nv || i1 < 0 || i1 >= nv || i2 < 0 || i2 >= nv) i0 = i1 = i2 = 0;  // reported by the records kernel
  const double2 a = p[i0], b = p[i1], c = p[i2];
  const double s = area2 * r.w[qq];
  const double p0 = r.phi[qq], p1 = r.phi[Q + qq], p2 = r.phi[2 * Q + qq];
  C2 v;
  v.x = (p0 * a.x + p1 * b.x + p2 * c.x) * s;
  v.y = (p0 * a.y + p1 * b.y + p2 * c.y) * s;
  src[i] = v;
  if (qq == 0) {
    C2 d;
    d.x = q[g].x;
    d.y = q[g].y;
    drive[g] = d;
  }
}

}  // namespace
}  // namespace bem

extern "C" int bem_evaluate_field_noalloc(const double* d_vertices, int n_vertices, const int* d_faces, int n_faces,
                                          int regular_order, double k, const double* d_pressure,
                                          const double* d_neumann, const double* d_points, int n_points, int precision,
                                          double* d_field_out, void* stream, char* err, int err_cap) {
  using namespace bem;
  auto fail = [&](int code, const char* msg) {
    if (err && err_cap > 0) {
      std::snprintf(err, (size_t)err_cap, "%s", msg);
    }
    return code;
  };
  if (err && err_cap > 0) err[0] = '\0';
  if (!d_vertices || !d_faces || !d_pressure || !d_neumann || !d_points || !d_field_out)
    return fail(BEM_ERR_INVALID_ARGUMENT, "null device pointer argument");
  if (n_vertices < 3 || n_faces < 1 || n_points < 1) return fail(BEM_ERR_INVALID_ARGUMENT, "empty mesh or no points");
  if (n_faces > kNoAllocMaxFaces) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "n_faces = %d exceeds the allocation-free limit of %d faces", n_faces,
                  kNoAllocMaxFaces);
    return fail(BEM_ERR_INVALID_ARGUMENT, msg);
  }
  if (!(k > 0.0) || !std::isfinite(k)) return fail(BEM_ERR_INVALID_ARGUMENT, "wavenumber must be finite and > 0");
  if (precision != BEM_PRECISION_FP64 && precision != BEM_PRECISION_MIXED)
    return fail(BEM_ERR_INVALID_ARGUMENT, "unknown precision");
  if (regular_order < 1 || regular_order > 4) return fail(BEM_ERR_INVALID_ARGUMENT, "regular order must be 1..4");
  if (field_params_bytes() > kParamBytes) return fail(BEM_ERR_CUDA, "internal: parameter block too small");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(BEM_ERR_CUDA, "no current CUDA device");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_lookup_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_field_scratch);
      if (e != cudaSuccess || !p) return fail(BEM_ERR_CUDA, cudaGetErrorString(e));
      g_scratch_addr[dev] = p;
    }
    base = g_scratch_addr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (s) {
    int sdev = -1;
    if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) return fail(BEM_ERR_INVALID_ARGUMENT, "invalid stream");
    if (sdev != dev) return fail(BEM_ERR_INVALID_ARGUMENT, "stream belongs to another device than the current one");
  }
  char* records = (char*)base;
  char* sources = records + kRecordBytes;
  char* drive = sources + kSourceBytes;
  char* params = drive + kDriveBytes;

  double pts[2 * kMaxQ] = {0}, w[kMaxQ] = {0};
  int Q = 0;
  rule_for(regular_order, pts, w, Q);
  RulePts rp;
  RuleWP rwp;
  std::memset(&rwp, 0, sizeof(rwp));
  for (int i = 0; i < 2 * kMaxQ; ++i) rp.p[i] = pts[i];
  for (int q = 0; q < Q; ++q) {
    rwp.w[q] = w[q];
    rwp.phi[q] = 1.0 - pts[2 * q] - pts[2 * q + 1];
    rwp.phi[Q + q] = pts[2 * q];
    rwp.phi[2 * Q + q] = pts[2 * q + 1];
  }
  const bool f32 = precision == BEM_PRECISION_MIXED;
  // The degenerate-face flag lives in the parameter block's last word.
  int* bad = (int*)(params + kParamBytes - sizeof(int));
  if (cudaMemsetAsync(bad, 0, sizeof(int), s) != cudaSuccess) return fail(BEM_ERR_CUDA, "cudaMemsetAsync failed");
  const int tpb = 128;
  if (f32)
    noalloc_face_records<true><<<(n_faces + tpb - 1) / tpb, tpb, 0, s>>>(d_vertices, n_vertices, d_faces, n_faces, Q, rp,
                                                                         records, bad);
  else
    noalloc_face_records<false><<<(n_faces + tpb - 1) / tpb, tpb, 0, s>>>(d_vertices, n_vertices, d_faces, n_faces, Q,
                                                                          rp, records, bad);
  const int total = n_faces * Q;
  if (f32)
    noalloc_sources<float2><<<(total + 255) / 256, 256, 0, s>>>(d_faces, n_vertices, records, n_faces, Q, (const double2*)d_pressure,
                                                                (const double2*)d_neumann, rwp, true, (float2*)sources,
                                                                (float2*)drive);
  else
    noalloc_sources<double2><<<(total + 255) / 256, 256, 0, s>>>(d_faces, n_vertices, records, n_faces, Q,
                                                                 (const double2*)d_pressure, (const double2*)d_neumann,
                                                                 rwp, false, (double2*)sources, (double2*)drive);
  cudaError_t e = launch_field_single(f32 ? Precision::Mixed : Precision::FP64, records, n_faces, Q, rwp.w, rwp.phi,
                                      sources, drive, d_points, n_points, k, params, (double2*)d_field_out, s);
  if (e != cudaSuccess) return fail(BEM_ERR_CUDA, cudaGetErrorString(e));
  int hbad = 0;
  if (cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return fail(BEM_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  if (hbad == 2) return fail(BEM_ERR_INVALID_ARGUMENT, "face references a vertex index out of range");
  if (hbad) return fail(BEM_ERR_INVALID_ARGUMENT, "mesh contains a degenerate (zero-area) triangle");
  return BEM_OK;
}
