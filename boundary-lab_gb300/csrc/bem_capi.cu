// C ABI of the GB300 BEM library: contexts, meshes, the batched frequency
// solve and the parity entry points.  See include/gb300_bem.h for the contract.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <functional>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gb300_bem.h"
#include "bem_internal.h"
#include "bem_kernels.h"

namespace {

// Library memory pool of one device.  Every device allocation of the library
// is stream-ordered (cudaMallocFromPoolAsync / cudaFreeAsync on the owning
// context's stream): unlike cudaMalloc / cudaFree it implies no device-wide
// synchronisation, so contexts on different streams keep running concurrently
// while one of them grows or frees its scratch.  Freed memory stays cached in
// the pool (no release threshold) until bem_trim_context trims it.
cudaMemPool_t device_pool(int device) {
  static std::mutex mu;
  static std::vector<cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)pools.size() <= device) pools.resize(device + 1, nullptr);
  if (!pools[device]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return nullptr;
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[device] = pool;
  }
  return pools[device];
}

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;  // owning stream (set by the owner before first use)
  cudaMemPool_t pool = nullptr;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (!pool) return cudaErrorInitializationError;
    if (p) cudaFreeAsync(p, stream);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocFromPoolAsync(&p, n, pool, stream);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFreeAsync(p, stream);
    p = nullptr;
    bytes = 0;
  }
};

struct BemError {
  int code;
  std::string msg;
};

inline void ck(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  int code = (e == cudaErrorMemoryAllocation) ? BEM_ERR_OUT_OF_MEMORY : BEM_ERR_CUDA;
  throw BemError{code, std::string(what) + ": " + cudaGetErrorString(e)};
}

}  // namespace

struct bem_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // once-per-mesh FP64 singular moments, overlapped with the first assembly
  cublasHandle_t cublas = nullptr;
  std::string err;
  cudaMemPool_t pool = nullptr;
  DevBuf rext, mats, mats2, ipiv, perm, info, sblocks, rb, b32, b64, x64, r64, d32, fsrc, fout, norms, pout, tcws, rowmap;
  DevBuf ftrace_p, ftrace_q, fpoints;  // bem_evaluate_field: boundary traces and points
  DevBuf xsplit;                       // the refinement's x as float hi / lo pairs
  std::vector<DevBuf*> scratch() {
    return {&rext, &mats, &mats2, &ipiv, &perm, &info, &sblocks, &rb, &b32, &b64, &x64, &r64, &d32, &fsrc, &fout, &norms,
            &pout, &tcws, &rowmap, &ftrace_p, &ftrace_q, &fpoints, &xsplit};
  }
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  void* stage = nullptr;  // pinned host staging of mesh uploads (grown on demand)
  size_t stage_bytes = 0;
  std::vector<bem_mesh*> meshes;
  // the extra lanes of a multi-lane sweep (options.lanes > 1): contexts of their own on the
  // same device whose streams and scratch take their share of the batches; created on first use
  std::vector<bem_context*> lanes;
  // optional per-kernel-family timing (options.profile)
  bool prof = false;
  std::vector<cudaEvent_t> pev;
  std::vector<int> pslot;
  size_t pev_used = 0;
};

struct bem_mesh {
  bem_context* ctx = nullptr;
  bem::MeshPlan plan;
  bem::DeviceMesh dm;
  std::vector<void*> allocs;
  int nc = 0;
  DevBuf drive32, drive64, obs;
  int nobs = 0;
  DevBuf driven;
  cudaEvent_t moments_ready = nullptr;  // recorded on ctx->side after the singular moments kernel
  cudaEvent_t cheb_ready = nullptr;     // recorded on ctx->side after the Chebyshev moments kernel
  long long singular_points = 0;
};

namespace {

void* mesh_alloc(bem_mesh* m, size_t bytes, const char* what) {
  void* p = nullptr;
  ck(cudaMallocFromPoolAsync(&p, bytes, m->ctx->pool, m->ctx->stream), what);
  m->allocs.push_back(p);
  return p;
}

// The arrays of one mesh upload, packed at 256-byte offsets into one device
// allocation and sent in one copy from the context's pinned staging buffer
// (instead of one pageable copy and one allocation per array).
struct UploadPack {
  struct Part {
    size_t off, bytes;
    const void* src;
    std::function<void(char*)> bind;
  };
  std::vector<Part> parts;
  size_t total = 0;
  template <typename T, typename A> void add(T*& dst, const std::vector<T, A>& v) {
    dst = nullptr;
    if (v.empty()) return;
    const size_t off = (total + 255) & ~(size_t)255;
    const size_t bytes = v.size() * sizeof(T);
    T** d = &dst;
    parts.push_back({off, bytes, v.data(), [d, off](char* base) { *d = (T*)(base + off); }});
    total = off + bytes;
  }
  void commit(bem_mesh* m) {
    if (total == 0) return;
    bem_context* ctx = m->ctx;
    if (ctx->stage_bytes < total) {
      if (ctx->stage) {
        ck(cudaStreamSynchronize(ctx->stream), "upload staging");
        cudaFreeHost(ctx->stage);
        ctx->stage = nullptr;
        ctx->stage_bytes = 0;
      }
      const size_t want = total + total / 4;
      ck(cudaHostAlloc(&ctx->stage, want, cudaHostAllocDefault), "allocate upload staging");
      ctx->stage_bytes = want;
    }
    char* base = (char*)mesh_alloc(m, total, "allocate mesh data");
    // the host copies into the staging buffer, in pieces of at most 1 MB spread
    // over a few threads (one thread below 4 MB)
    struct Piece {
      size_t off, bytes;
      const char* src;
    };
    std::vector<Piece> pieces;
    constexpr size_t kPiece = (size_t)1 << 20;
    for (const Part& p : parts) {
      p.bind(base);
      for (size_t o = 0; o < p.bytes; o += kPiece)
        pieces.push_back({p.off + o, std::min(kPiece, p.bytes - o), (const char*)p.src + o});
    }
    const int nt = total < ((size_t)4 << 20)
                       ? 1
                       : (int)std::min<size_t>({8, pieces.size(), std::max(1u, std::thread::hardware_concurrency())});
    auto copy = [&](int t) {
      for (size_t i = t; i < pieces.size(); i += nt)
        std::memcpy((char*)ctx->stage + pieces[i].off, pieces[i].src, pieces[i].bytes);
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) {
      try {
        th.emplace_back(copy, t);
      } catch (...) {  // no thread: this one copies that share
        copy(t);
      }
    }
    copy(0);
    for (auto& t : th) t.join();
    ck(cudaMemcpyAsync(base, ctx->stage, total, cudaMemcpyHostToDevice, ctx->stream), "upload");
  }
};

// Profiling marks: the time between two consecutive marks is charged to the
// slot of the later mark.
void prof_mark(bem_context* c, int slot) {
  if (!c->prof) return;
  if (c->pev_used == c->pev.size()) {
    cudaEvent_t e;
    ck(cudaEventCreate(&e), "cudaEventCreate");
    c->pev.push_back(e);
  }
  ck(cudaEventRecord(c->pev[c->pev_used], c->stream), "cudaEventRecord");
  c->pslot.push_back(slot);
  c->pev_used++;
}
void prof_begin(bem_context* c) {
  c->pev_used = 0;
  c->pslot.clear();
  prof_mark(c, -1);
}
void prof_collect(bem_context* c, double* acc) {
  if (!c->prof) return;
  for (size_t i = 1; i < c->pev_used; ++i) {
    float ms = 0;
    cudaEventElapsedTime(&ms, c->pev[i - 1], c->pev[i]);
    if (c->pslot[i] >= 0 && c->pslot[i] < BEM_K_SLOTS) acc[c->pslot[i]] += ms * 1e-3;
  }
  c->pev_used = 0;
  c->pslot.clear();
}

int fail(bem_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

template <typename F> int guarded(bem_context* ctx, F&& f) {
  try {
    if (ctx) {
      ctx->err.clear();
      cudaSetDevice(ctx->device);
    }
    return f();
  } catch (const BemError& e) {
    return fail(ctx, e.code, e.msg);
  } catch (const std::bad_alloc&) {
    return fail(ctx, BEM_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(ctx, BEM_ERR_INVALID_ARGUMENT, e.what());
  }
}

inline long long round_up(long long x, long long a) { return (x + a - 1) / a * a; }

bem::OperatorCoeffs bm_coeffs(double k) {
  bem::OperatorCoeffs c;
  const double eta = 1.0 / k;  // eta = i/k
  c.cD = make_double2(-1.0, 0.0);
  c.cH = make_double2(0.0, eta);
  c.cM = make_double2(0.5, 0.0);
  c.cS = make_double2(-1.0, 0.0);
  c.cK = make_double2(0.0, -eta);
  c.cM10 = make_double2(0.0, -0.5 * eta);
  return c;
}

// Shapes of the scratch layout for one mesh / batch.
struct Layout {
  long long ldR, lda, ldb;
  size_t esz;
};
Layout layout_for(const bem::DeviceMesh& dm, bem::Precision prec) {
  Layout L;
  L.esz = prec == bem::Precision::Mixed ? sizeof(float2) : sizeof(double2);
  L.ldR = round_up(std::max(dm.n_ext, 1), 32);
  L.lda = round_up(dm.nv, 32);
  L.ldb = round_up(dm.nv, 32);
  return L;
}

// Frequencies a mixed-form call needs before its singular remainders go through the mesh's
// Chebyshev moments: forming them costs about as much as six frequencies of the point-by-
// point singular kernel at 16 terms (more at more terms, at most 24), and each frequency
// through them costs a fifteenth of one.  A shorter call runs point by point even when the
// moments exist, so a call's results depend on its own inputs only.
constexpr int kChebMinFreqs = 12;

// Forms (or extends) the mesh's Chebyshev moments on the side stream for the call's
// wavenumbers k[0..n): with the fewest terms (a multiple of four) that cover every
// frequency whose expansion converges within kChebN terms, or twice the terms the moments
// had, up to kChebN.  Nothing when no frequency converges (those run point by point).
void ensure_cheb(bem_context* ctx, bem_mesh* m, const double* k, int n) {
  bem::DeviceMesh& d = m->dm;
  if (d.npairs == 0 || !(d.cheb_R > 0.0)) return;
  int need = 0;
  for (int i = 0; i < n; ++i) need = std::max(need, bem::cheb_terms(k[i], d.cheb_R));
  if (need == 0 || d.cheb_n >= need) return;
  const int nterms = std::min(bem::kChebN, std::max(need, 2 * d.cheb_n));
  if (!d.cheb)
    d.cheb = (float*)mesh_alloc(m, (size_t)d.npairs * bem::kChebN * 24 * sizeof(float), "allocate Chebyshev moments");
  // the side stream must see the allocation (made on the context's stream), the pair
  // records (written on the side stream) are in order there, and no singular kernel of an
  // earlier sweep may still read the moments being rewritten
  // (nor one still running on a lane's stream)
  std::vector<cudaStream_t> before{ctx->stream};
  for (bem_context* cl : ctx->lanes) before.push_back(cl->stream);
  for (cudaStream_t st : before) {
    cudaEvent_t ev = nullptr;
    ck(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "create event");
    ck(cudaEventRecord(ev, st), "record event");
    ck(cudaStreamWaitEvent(ctx->side, ev, 0), "wait for an earlier stream");
    cudaEventDestroy(ev);
  }
  ck(bem::launch_cheb_moments(d, nterms, ctx->side), "Chebyshev moments kernel");
  if (!m->cheb_ready) ck(cudaEventCreateWithFlags(&m->cheb_ready, cudaEventDisableTiming), "create event");
  ck(cudaEventRecord(m->cheb_ready, ctx->side), "record event");
  d.cheb_n = nterms;
}

// Assemble the LHS (c[i].cD, cH, cM) of cnt frequencies into A[i] (and A2[i] if
// given; column-major, leading dimension lda) and, if nc > 0, the RHS into b[i]
// (nc columns, leading dimension ldb, permuted rows).  lda / ldb <= 0: the mesh's
// own layout.  Returns the number of kernels launched.
long long assemble_frequencies(bem_context* ctx, bem_mesh* m, bem::Precision prec, int cnt, const double* k,
                               const bem::OperatorCoeffs* c, void* const* A, void* const* A2, const double2* qscale,
                               int nc, const void* drive, void* const* b, long long lda = 0, long long ldb = 0,
                               double* regular_flop = nullptr, long long* cheb_freqs = nullptr,
                               bool use_cheb = false) {
  const bem::DeviceMesh& dm = m->dm;
  Layout L = layout_for(dm, prec);
  if (lda > 0) L.lda = lda;
  if (ldb > 0) L.ldb = ldb;
  int sizes[64];
  const int ngroups = bem::regular_groups(dm, prec, cnt, sizes);
  int G = 1;
  for (int i = 0; i < ngroups; ++i) G = std::max(G, sizes[i]);
  const size_t rext_n = (size_t)L.ldR * 3 * dm.nf;         // elements per extended-row buffer
  const size_t sblk_n = (size_t)std::max(dm.npairs, 1) * 12;  // elements per singular-block buffer
  ck(ctx->rext.ensure(rext_n * L.esz * G), "alloc extended rows");
  ck(ctx->sblocks.ensure(sblk_n * L.esz * G), "alloc singular blocks");
  if (nc > 0) ck(ctx->rb.ensure((size_t)std::max(4, nc) * dm.nf * 3 * L.esz), "alloc rhs faces");
  auto rext = [&](int i) { return (void*)((char*)ctx->rext.p + rext_n * L.esz * i); };
  auto sblk = [&](int i) { return (void*)((char*)ctx->sblocks.p + sblk_n * L.esz * i); };
  long long launches = 0;
  int f0 = 0;
  for (int gi = 0; gi < ngroups; f0 += sizes[gi], ++gi) {
    const int g = sizes[gi];
    double2 cD[4], cH[4];
    for (int i = 0; i < g; ++i) {
      cD[i] = c[f0 + i].cD;
      cH[i] = c[f0 + i].cH;
    }
    // regular pairs first: on a freshly uploaded mesh they run while the side stream
    // still integrates the FP64 singular moments that the singular kernel reads
    ck(bem::launch_regular(dm, prec, g, k + f0, cD, cH, rext(0), L.ldR, (long long)rext_n, ctx->stream),
       "regular kernel");
    prof_mark(ctx, BEM_K_REGULAR);
    if (m->moments_ready) ck(cudaStreamWaitEvent(ctx->stream, m->moments_ready, 0), "wait for singular moments");
    if (m->cheb_ready) ck(cudaStreamWaitEvent(ctx->stream, m->cheb_ready, 0), "wait for Chebyshev moments");
    long long sing_launches = 0;
    ck(bem::launch_singular_dyn(dm, prec, g, k + f0, c + f0, sblk(0), (long long)sblk_n, ctx->stream,
                                &sing_launches, cheb_freqs, use_cheb),
       "singular kernel");
    prof_mark(ctx, BEM_K_SINGULAR);
    for (int i = 0; i < g; ++i) {
      void* Ai = A[f0 + i];
      void* A2i = A2 ? A2[f0 + i] : nullptr;
      ck(bem::launch_singular_scatter(dm, prec, sblk(i), rext(i), L.ldR, ctx->stream), "singular scatter");
      if (dm.n_isolated) {
        ck(cudaMemsetAsync(Ai, 0, (size_t)L.lda * dm.nv * L.esz, ctx->stream), "memset");
        if (A2i) ck(cudaMemsetAsync(A2i, 0, (size_t)L.lda * dm.nv * L.esz, ctx->stream), "memset");
      }
      ck(bem::launch_gather(dm, prec, rext(i), L.ldR, Ai, L.lda, A2i, ctx->stream), "gather kernel");
    }
    prof_mark(ctx, BEM_K_GATHER);
    if (nc > 0) {
      ck(bem::launch_rhs_freqs(dm, prec, g, k + f0, c + f0, qscale + f0, drive, nc, sblk(0), (long long)sblk_n,
                               ctx->rb.p, b + f0, L.ldb, ctx->stream),
         "rhs kernel");
      prof_mark(ctx, BEM_K_RHS);
    }
    // per frequency: scatter, gather (+ isolated rows); per group the regular, singular and
    // right-hand-side launches
    launches += (long long)g * (2 + (dm.n_isolated ? 1 : 0)) + (nc > 0 ? bem::rhs_launches(prec, nc, g) : 0) +
                bem::regular_launches(dm, prec, g) + sing_launches;
    if (regular_flop && prec == bem::Precision::Mixed) {
      const double qpairs = ((double)dm.ntr * dm.nf * dm.nf - dm.npairs) * dm.Q * dm.Q;
      *regular_flop += g * qpairs * bem::regular_flop_per_qpair(g);
    }
  }
  return launches;
}

// One frequency's operators as a long sweep assembles them (the mixed form's singular
// remainder through the mesh's Chebyshev moments wherever their expansion converges).
void assemble_one(bem_mesh* m, bem::Precision prec, double k, const bem::OperatorCoeffs& c, void* A, void* A2,
                  double2 qscale, int nc, const void* drive, void* b) {
  const bool cheb = prec == bem::Precision::Mixed;
  if (cheb) ensure_cheb(m->ctx, m, &k, 1);
  assemble_frequencies(m->ctx, m, prec, 1, &k, &c, &A, A2 ? &A2 : nullptr, &qscale, nc, drive, &b, 0, 0, nullptr,
                       nullptr, cheb);
}

void free_mesh_device(bem_mesh* m) {
  if (m->cheb_ready) {  // the side stream may still read the mesh data
    cudaStreamWaitEvent(m->ctx->stream, m->cheb_ready, 0);
    cudaEventDestroy(m->cheb_ready);
    m->cheb_ready = nullptr;
  }
  if (m->moments_ready) {
    cudaStreamWaitEvent(m->ctx->stream, m->moments_ready, 0);
    cudaEventDestroy(m->moments_ready);
    m->moments_ready = nullptr;
  }
  for (void* p : m->allocs) cudaFreeAsync(p, m->ctx->stream);
  m->allocs.clear();
  m->drive32.release();
  m->drive64.release();
  m->obs.release();
  m->driven.release();
}

}  // namespace

extern "C" {

int bem_abi_version(void) { return GB300_BEM_ABI_VERSION; }

const char* bem_last_error(const bem_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* bem_context_stream(const bem_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int bem_create_context(int device, bem_context** out) {
  if (!out) return BEM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return BEM_ERR_CUDA;
  if (device < 0 || device >= count) return BEM_ERR_INVALID_ARGUMENT;
  bem_context* ctx = new bem_context();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return BEM_ERR_CUDA;
  }
  if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return BEM_ERR_CUDA;
  }
  if (cublasCreate(&ctx->cublas) != CUBLAS_STATUS_SUCCESS) {
    cudaStreamDestroy(ctx->side);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return BEM_ERR_CUDA;
  }
  cublasSetStream(ctx->cublas, ctx->stream);
  ctx->pool = device_pool(device);
  if (!ctx->pool) {
    cublasDestroy(ctx->cublas);
    cudaStreamDestroy(ctx->side);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return BEM_ERR_CUDA;
  }
  for (DevBuf* b : ctx->scratch()) {
    b->stream = ctx->stream;
    b->pool = ctx->pool;
  }
  for (auto& e : ctx->ev) cudaEventCreate(&e);
  *out = ctx;
  return BEM_OK;
}

void bem_destroy_context(bem_context* ctx) {
  if (!ctx) return;
  for (bem_context* l : ctx->lanes) bem_destroy_context(l);
  ctx->lanes.clear();
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (bem_mesh* m : ctx->meshes) {
    free_mesh_device(m);
    delete m;
  }
  ctx->meshes.clear();
  for (DevBuf* b : ctx->scratch()) b->release();
  cudaStreamSynchronize(ctx->stream);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : ctx->pev) cudaEventDestroy(e);
  if (ctx->stage) cudaFreeHost(ctx->stage);
  if (ctx->cublas) cublasDestroy(ctx->cublas);
  if (ctx->side) {
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
  }
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int bem_trim_context(bem_context* ctx) {
  if (!ctx) return BEM_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&]() -> int {
    for (DevBuf* b : ctx->scratch()) b->release();
    for (bem_context* l : ctx->lanes) {
      for (DevBuf* b : l->scratch()) b->release();
      ck(cudaStreamSynchronize(l->stream), "trim scratch");
    }
    ck(cudaStreamSynchronize(ctx->stream), "trim scratch");
    ck(cudaMemPoolTrimTo(ctx->pool, 0), "trim memory pool");
    return BEM_OK;
  });
}

long long bem_context_scratch_bytes(const bem_context* ctx) {
  if (!ctx) return -1;
  long long total = 0;
  for (DevBuf* b : const_cast<bem_context*>(ctx)->scratch()) total += (long long)b->bytes;
  for (const bem_context* l : ctx->lanes) total += bem_context_scratch_bytes(l);
  return total;
}

int bem_upload_mesh(bem_context* ctx, const double* vertices, int n_vertices, const int* faces, int n_faces,
                    int regular_order, int singular_order, bem_mesh** out) {
  return bem_upload_mesh_symmetric(ctx, vertices, n_vertices, faces, n_faces, regular_order, singular_order,
                                   BEM_SYMMETRY_OFF, out);
}

int bem_upload_mesh_symmetric(bem_context* ctx, const double* vertices, int n_vertices, const int* faces,
                              int n_faces, int regular_order, int singular_order, int symmetry, bem_mesh** out) {
  if (!ctx) return BEM_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&]() -> int {
    if (!out || !vertices || !faces) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "null pointer argument");
    *out = nullptr;
    bem_mesh* m = new bem_mesh();
    m->ctx = ctx;
    for (DevBuf* b : {&m->drive32, &m->drive64, &m->obs, &m->driven}) {
      b->stream = ctx->stream;
      b->pool = ctx->pool;
    }
    std::string e = bem::build_mesh_plan(vertices, n_vertices, faces, n_faces, regular_order, singular_order, 512, m->plan,
                                         symmetry);
    if (!e.empty()) {
      delete m;
      return fail(ctx, BEM_ERR_INVALID_ARGUMENT, e);
    }
    try {
      const bem::MeshPlan& P = m->plan;
      bem::DeviceMesh& d = m->dm;
      d.nv = P.nv;
      d.nf = P.nf;
      d.Q = P.Q;
      d.n_tiles = P.n_tiles;
      d.max_tile_rows = P.max_tile_rows;
      d.n_ext = P.n_ext;
      d.n_halo = (int)P.halo_ext.size();
      d.n_halo_rows = (int)P.halo_row.size();
      d.npairs = (int)P.pairs.size();
      d.n_scat = (int)P.scat_col.size();
      d.ntr = (int)P.transforms.size();
      for (int i = 0; i < d.ntr && i < 4; ++i) d.tr[i] = P.transforms[i];
      std::vector<int> iso;
      for (int v = 0; v < P.nv; ++v)
        if (P.col_ptr[v] == P.col_ptr[v + 1]) iso.push_back(v);
      d.n_isolated = (int)iso.size();
      const std::vector<float> duffy32(P.duffy.begin(), P.duffy.end());
      std::vector<float> duffy_df(2 * P.duffy.size());
      for (size_t i = 0; i < P.duffy.size(); ++i) {
        const float hi = (float)P.duffy[i];
        duffy_df[2 * i] = hi;
        duffy_df[2 * i + 1] = (float)(P.duffy[i] - (double)hi);
      }
      std::vector<double> mm(12);
      for (int i = 0; i < 9; ++i) mm[i] = P.m11[i];
      for (int i = 0; i < 3; ++i) mm[9 + i] = P.m10[i];
      UploadPack pack;
      if (P.symmetry != 0) {
        pack.add(d.fix_mask, P.fix_mask);
        pack.add(d.row_weight, P.row_weight);
      }
      pack.add(d.faces32, P.faces32);
      pack.add(d.faces64, P.faces64);
      pack.add(d.tile_group_ptr, P.tile_group_ptr);
      pack.add(d.lane_slots, P.lane_slots);
      pack.add(d.group_faces32, P.group_faces32);
      pack.add(d.tile_row_base, P.tile_row_base);
      pack.add(d.ext_row, P.ext_row);
      pack.add(d.halo_slot_of_ext, P.halo_slot_of_ext);
      pack.add(d.halo_row_ptr, P.halo_row_ptr);
      pack.add(d.halo_row, P.halo_row);
      pack.add(d.col_ptr, P.col_ptr);
      pack.add(d.col_fb, P.col_fb);
      pack.add(d.face_ext, P.face_ext);
      pack.add(d.vertex_row, P.vertex_row);
      pack.add(d.isolated, iso);
      pack.add(d.pairs, P.pairs);
      pack.add(d.pairs_by_trial_ptr, P.pairs_by_trial_ptr);
      pack.add(d.pairs_by_test_ptr, P.pairs_by_test_ptr);
      pack.add(d.pairs_by_test, P.pairs_by_test);
      pack.add(d.scat_col, P.scat_col);
      pack.add(d.scat_row, P.scat_row);
      pack.add(d.scat_ptr, P.scat_ptr);
      pack.add(d.scat_src, P.scat_src);
      pack.add(d.rule_ptr, P.rule_ptr);
      pack.add(d.duffy, P.duffy);
      pack.add(d.duffy32, duffy32);
      pack.add(d.duffy_df, duffy_df);
      pack.add(d.verts, P.verts);
      pack.add(d.faces, P.faces);
      pack.add(d.normal, P.normal);
      pack.add(d.curls, P.curls);
      pack.add(d.area, P.area);
      pack.add(d.m11m10, mm);
      pack.commit(m);
      for (int q = 0; q < P.Q; ++q) {
        const double u = P.rule_pts[2 * q], v = P.rule_pts[2 * q + 1];
        const double phi[3] = {1.0 - u - v, u, v};
        d.rule_w[q] = P.rule_w[q];
        for (int a = 0; a < 3; ++a) {
          d.rule_phi[a * P.Q + q] = phi[a];
          d.rule_cw[a * P.Q + q] = phi[a] * P.rule_w[q];
        }
      }
      m->singular_points = P.singular_points;
      for (int i = 0; i < 12; ++i) d.m11m10f[i] = (float)mm[i];
      if (d.npairs > 0) {
        d.moments = (double*)mesh_alloc(m, (size_t)d.npairs * 24 * sizeof(double), "allocate singular moments");
        d.pairrec = (float*)mesh_alloc(m, (size_t)d.npairs * bem::kPairRec * sizeof(float), "allocate pair records");
        d.pairgeo_df = (float*)mesh_alloc(m, (size_t)d.npairs * bem::kPairGeoDf * sizeof(float), "allocate pair geometry");
        // the Chebyshev expansion interval of the singular remainder: every point distance
        // of a pair lies below the largest distance between its vertices (a little margin
        // for rounding); the moments themselves are formed by the first sweep that uses them
        d.cheb_R = 1.000001 * P.pair_radius;
      }
      ck(cudaStreamSynchronize(ctx->stream), "mesh upload");
      if (d.npairs > 0) {
        // the k-independent moments (FP64) on the side stream; the first singular kernel
        // of a solve waits for them, the regular assembly before it does not
        ck(bem::launch_singular_static(d, d.moments, d.pairrec, ctx->side), "singular moments kernel");
        ck(cudaEventCreateWithFlags(&m->moments_ready, cudaEventDisableTiming), "create event");
        ck(cudaEventRecord(m->moments_ready, ctx->side), "record event");
      }
    } catch (...) {
      free_mesh_device(m);
      delete m;
      throw;
    }
    ctx->meshes.push_back(m);
    *out = m;
    return BEM_OK;
  });
}

void bem_release_mesh(bem_mesh* mesh) {
  if (!mesh) return;
  bem_context* ctx = mesh->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_mesh_device(mesh);
  ctx->meshes.erase(std::remove(ctx->meshes.begin(), ctx->meshes.end(), mesh), ctx->meshes.end());
  delete mesh;
}

int bem_mesh_info(const bem_mesh* mesh, int* n_vertices, int* n_faces, int* n_singular_pairs) {
  if (!mesh) return BEM_ERR_INVALID_ARGUMENT;
  if (n_vertices) *n_vertices = mesh->dm.nv;
  if (n_faces) *n_faces = mesh->dm.nf;
  if (n_singular_pairs) *n_singular_pairs = mesh->dm.npairs;
  return BEM_OK;
}

int bem_set_excitation(bem_mesh* m, const double* unit_drive, int n_rhs) {
  if (!m) return BEM_ERR_INVALID_ARGUMENT;
  bem_context* ctx = m->ctx;
  return guarded(ctx, [&]() -> int {
    if (!unit_drive || n_rhs < 1 || n_rhs > 4) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "need 1..4 excitations");
    const int nf = m->dm.nf;
    std::vector<float2> d32((size_t)n_rhs * nf);
    std::vector<double2> d64((size_t)n_rhs * nf);
    std::vector<int> driven;
    for (int f = 0; f < nf; ++f) {
      bool any = false;
      for (int c = 0; c < n_rhs; ++c) {
        const double re = unit_drive[2 * ((size_t)c * nf + f)], im = unit_drive[2 * ((size_t)c * nf + f) + 1];
        if (!std::isfinite(re) || !std::isfinite(im)) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "drive must be finite");
        d32[(size_t)c * nf + f] = make_float2((float)re, (float)im);
        d64[(size_t)c * nf + f] = make_double2(re, im);
        any = any || re != 0.0 || im != 0.0;
      }
      if (any) driven.push_back(f);
    }
    ck(cudaStreamSynchronize(ctx->stream), "sync");
    ck(m->drive32.ensure(d32.size() * sizeof(float2)), "alloc drive");
    ck(m->drive64.ensure(d64.size() * sizeof(double2)), "alloc drive");
    ck(m->driven.ensure(std::max<size_t>(1, driven.size()) * sizeof(int)), "alloc driven");
    ck(cudaMemcpyAsync(m->drive32.p, d32.data(), d32.size() * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream),
       "copy drive");
    ck(cudaMemcpyAsync(m->drive64.p, d64.data(), d64.size() * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream),
       "copy drive");
    if (!driven.empty())
      ck(cudaMemcpyAsync(m->driven.p, driven.data(), driven.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream),
         "copy driven");
    ck(cudaStreamSynchronize(ctx->stream), "copy drive");
    m->dm.driven = (int*)m->driven.p;
    m->dm.ndriven = (int)driven.size();
    m->nc = n_rhs;
    return BEM_OK;
  });
}

int bem_set_observation_points(bem_mesh* m, const double* points, int n_points) {
  if (!m) return BEM_ERR_INVALID_ARGUMENT;
  bem_context* ctx = m->ctx;
  return guarded(ctx, [&]() -> int {
    if (!points || n_points < 1) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "need at least one observation point");
    for (long long i = 0; i < 3LL * n_points; ++i)
      if (!std::isfinite(points[i])) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "observation points must be finite");
    ck(cudaStreamSynchronize(ctx->stream), "sync");
    ck(m->obs.ensure((size_t)n_points * 3 * sizeof(double)), "alloc observation points");
    ck(cudaMemcpyAsync(m->obs.p, points, (size_t)n_points * 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
       "copy points");
    ck(cudaStreamSynchronize(ctx->stream), "copy points");
    m->nobs = n_points;
    return BEM_OK;
  });
}

int bem_evaluate_field(bem_mesh* m, double k, int precision, const double* pressure, const double* neumann,
                       const double* points, int n_points, double* field_out) {
  if (!m) return BEM_ERR_INVALID_ARGUMENT;
  bem_context* ctx = m->ctx;
  return guarded(ctx, [&]() -> int {
    if (!pressure || !neumann || !points || !field_out || n_points < 1)
      return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "bad arguments");
    if (!(k > 0) || !std::isfinite(k)) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "wavenumber must be finite and > 0");
    if (precision != BEM_PRECISION_FP64 && precision != BEM_PRECISION_MIXED)
      return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "unknown precision");
    const bem::DeviceMesh& dm = m->dm;
    const int nv = dm.nv, nf = dm.nf;
    for (long long i = 0; i < 3LL * n_points; ++i)
      if (!std::isfinite(points[i])) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "points must be finite");
    for (long long i = 0; i < 2LL * nv; ++i)
      if (!std::isfinite(pressure[i])) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "boundary pressure must be finite");
    for (long long i = 0; i < 2LL * nf; ++i)
      if (!std::isfinite(neumann[i])) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "boundary normal derivative must be finite");
    const bem::Precision prec = precision == BEM_PRECISION_MIXED ? bem::Precision::Mixed : bem::Precision::FP64;
    const bool mixed = prec == bem::Precision::Mixed;
    const size_t esz = mixed ? sizeof(float2) : sizeof(double2);
    const long long ldp = round_up(nv, 32);
    // traces in the working precision: pressure [ldp] (vertex order), normal derivative [nf]
    std::vector<char> hp((size_t)ldp * esz, 0), hq((size_t)nf * esz);
    for (int i = 0; i < nv; ++i) {
      if (mixed)
        ((float2*)hp.data())[i] = make_float2((float)pressure[2 * i], (float)pressure[2 * i + 1]);
      else
        ((double2*)hp.data())[i] = make_double2(pressure[2 * i], pressure[2 * i + 1]);
    }
    for (int i = 0; i < nf; ++i) {
      if (mixed)
        ((float2*)hq.data())[i] = make_float2((float)neumann[2 * i], (float)neumann[2 * i + 1]);
      else
        ((double2*)hq.data())[i] = make_double2(neumann[2 * i], neumann[2 * i + 1]);
    }
    ck(ctx->ftrace_p.ensure(hp.size()), "alloc boundary pressure");
    ck(ctx->ftrace_q.ensure(hq.size()), "alloc boundary normal derivative");
    ck(ctx->fpoints.ensure((size_t)n_points * 3 * sizeof(double)), "alloc points");
    const size_t srcb = (size_t)nf * dm.Q * esz;
    ck(ctx->fsrc.ensure(round_up(srcb, 256) + 4096), "alloc field sources");
    ck(ctx->fout.ensure((size_t)n_points * sizeof(double2)), "alloc field out");
    ck(cudaMemcpyAsync(ctx->ftrace_p.p, hp.data(), hp.size(), cudaMemcpyHostToDevice, ctx->stream), "copy pressure");
    ck(cudaMemcpyAsync(ctx->ftrace_q.p, hq.data(), hq.size(), cudaMemcpyHostToDevice, ctx->stream), "copy normal derivative");
    ck(cudaMemcpyAsync(ctx->fpoints.p, points, (size_t)n_points * 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
       "copy points");
    const double2 one = make_double2(1.0, 0.0);
    ck(bem::launch_field(dm, prec, 1, &k, &one, ctx->ftrace_p.p, ldp, 1, ctx->ftrace_q.p, (const double*)ctx->fpoints.p,
                         n_points, ctx->fsrc.p, (double2*)ctx->fout.p, ctx->stream),
       "field kernel");
    ck(cudaMemcpyAsync(field_out, ctx->fout.p, (size_t)n_points * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream),
       "copy field");
    ck(cudaStreamSynchronize(ctx->stream), "field sync");
    return BEM_OK;
  });
}

void bem_default_options(bem_solve_options* opt) {
  if (!opt) return;
  opt->precision = BEM_PRECISION_MIXED;
  opt->sound_speed = 343.0;
  opt->rho = 1.21;
  opt->refine_tol = 1e-10;
  opt->max_refine = 8;
  opt->batch = 0;
  opt->lu_block = 0;
  opt->outputs_on_device = 0;
  opt->profile = 0;
  opt->lu_gemm = 0;
  opt->lanes = 1;
}

}  // extern "C"

namespace {
// Automatic batch: the matrices of a batch within ~16 GiB, at most 32, and at
// most as many as the LU's cluster panels keep resident at once (a larger batch
// runs every panel in two waves); the sweep is then split into equal batches.
int auto_batch_order(int nv, bem::Precision prec, int n_freq) {
  const double esz = prec == bem::Precision::Mixed ? sizeof(float2) : sizeof(double2);
  const double per = (double)round_up(nv, 32) * nv * esz * (prec == bem::Precision::Mixed ? 2 : 1);
  int cap = (int)std::max(1.0, std::min(32.0, std::floor(16.0 * (1ull << 30) / per)));
  cap = std::max(1, std::min(cap, bem::lu_resident_batch(prec, nv)));
  if (n_freq <= 0) return cap;  // the largest batch
  const int nbatch = (n_freq + cap - 1) / cap;
  return (n_freq + nbatch - 1) / nbatch;
}
int auto_batch(const bem_mesh* m, bem::Precision prec, int n_freq) { return auto_batch_order(m->dm.nv, prec, n_freq); }

// Rows and columns nv .. n-1 of cnt matrices of order n (leading dimension lda,
// stride) hold the identity: zero below row nv in columns < nv, and a unit
// column in each column >= nv.  Grid (n, cnt).
template <typename C2>
__global__ void pad_identity_kernel(C2* A, C2* A2, long long lda, long long stride, int nv, int n) {
  const int j = blockIdx.x;
  const size_t off = (size_t)blockIdx.y * stride + (size_t)j * lda;
  for (int r = (j < nv ? nv : 0) + threadIdx.x; r < n; r += blockDim.x) {
    C2 v;
    v.x = r == j ? 1 : 0;
    v.y = 0;
    A[off + r] = v;
    if (A2) A2[off + r] = v;
  }
}

// cnt consecutive frequencies of one mesh inside a combined batch, with the
// places their results go (already offset; either may be null).
// Streams a sweep's batches may be spread over: a third lane measured no faster than two at
// 10k (106.2 against 106.6 frequency solves/s), as the two already keep the GPU busy.
constexpr int kMaxLanes = 2;

struct Slice {
  bem_mesh* m;
  const double* freqs;
  int cnt;
  double* pressure_out;  // [cnt][nc][nv] complex
  double* field_out;     // [cnt][nc][nobs] complex
  bool cheb = false;     // mixed form: singular remainders through the mesh's Chebyshev moments
};

// Totals over the batches of one call.
struct SolveTotals {
  double kacc[BEM_K_SLOTS] = {0};
  double regular_flop = 0;
  long long cheb_freqs = 0;
  double t_asm = 0, t_sol = 0, t_fld = 0, max_res = 0;
  int max_steps = 0, batches = 0, gemm_used = 0;
  long long launches = 0;
};

// One batch: every slice's frequencies are assembled on the slice's own mesh into
// matrices of order n (n >= each slice mesh's nv; the rows and columns beyond a
// mesh's nv hold the identity and its right-hand sides are zero there), all the
// matrices are factored, solved and refined together (one launch sequence), and
// each slice's field is evaluated on its own mesh.  The identity block cannot
// change a pivot (its rows are zero in the mesh's columns), so each mesh's
// factors are those of its own matrix.  Every slice has the same number of
// excitations nc.
void solve_combined(bem_context* ctx, const std::vector<Slice>& sl, int n, const bem_solve_options& o, int nc,
                    SolveTotals& T) {
  const bem::Precision prec = o.precision == BEM_PRECISION_MIXED ? bem::Precision::Mixed : bem::Precision::FP64;
  const bool mixed = prec == bem::Precision::Mixed;
  const size_t esz = mixed ? sizeof(float2) : sizeof(double2);
  const long long lda = round_up(n, 32), ldb = round_up(n, 32);
  int B = 0;
  for (const Slice& x : sl) B += x.cnt;
  const int nb = o.lu_block > 0 ? std::min(o.lu_block, 64) : 0;  // 0: the LU chooses
  const size_t matsz = (size_t)lda * n * esz;
  ck(ctx->mats.ensure(matsz * B), "alloc matrices");
  if (mixed) ck(ctx->mats2.ensure(matsz * B), "alloc matrix copies");
  ck(ctx->ipiv.ensure((size_t)B * n * sizeof(int)), "alloc pivots");
  ck(ctx->perm.ensure((size_t)B * n * sizeof(int)), "alloc permutation");
  ck(ctx->info.ensure((size_t)B * sizeof(int)), "alloc info");
  ck(ctx->rowmap.ensure((size_t)B * bem::kRowmapStride * sizeof(int)), "alloc row map");
  const size_t vecn = (size_t)B * nc * ldb;
  ck(ctx->b32.ensure(vecn * esz), "alloc rhs");
  if (mixed) {
    ck(ctx->b64.ensure(vecn * sizeof(double2)), "alloc rhs64");
    ck(ctx->x64.ensure(vecn * sizeof(double2)), "alloc x");
    ck(ctx->r64.ensure(vecn * sizeof(double2)), "alloc r");
    ck(ctx->d32.ensure(vecn * sizeof(float2)), "alloc d");
    ck(ctx->xsplit.ensure(vecn * sizeof(float4)), "alloc x split");
    ck(ctx->norms.ensure((size_t)B * nc * 2 * sizeof(double)), "alloc norms");
  }
  bool any_field = false;
  for (const Slice& x : sl) {
    if (!x.field_out) continue;
    any_field = true;
    const bem::DeviceMesh& dm = x.m->dm;
    const size_t srcb = (size_t)x.cnt * nc * dm.nf * dm.Q * esz;
    ck(ctx->fsrc.ensure(round_up(srcb, 256) + 4096), "alloc field sources");
    ck(ctx->fout.ensure((size_t)x.cnt * nc * x.m->nobs * sizeof(double2)), "alloc field out");
  }
  if (any_field && mixed) ck(ctx->pout.ensure(vecn * sizeof(float2)), "alloc pressure f32");
  std::vector<double> norms((size_t)B * nc * 2);
  std::vector<int> info(B);
  std::vector<double> ks(B), fz(B);
  std::vector<double2> qs(B);
  std::vector<bem::OperatorCoeffs> cs(B);
  std::vector<void*> As(B), A2s(B), bs(B);
  ++T.batches;
  cudaEventRecord(ctx->ev[0], ctx->stream);
  prof_begin(ctx);
  int i0 = 0;
  for (const Slice& x : sl) {
    for (int i = 0; i < x.cnt; ++i) {
      const int g = i0 + i;
      const double omega = 2.0 * M_PI * x.freqs[i];
      const double k = omega / o.sound_speed;
      fz[g] = x.freqs[i];
      ks[g] = k;
      qs[g] = make_double2(0.0, o.rho * omega);
      cs[g] = bm_coeffs(k);
      As[g] = (char*)ctx->mats.p + matsz * g;
      A2s[g] = mixed ? (char*)ctx->mats2.p + matsz * g : nullptr;
      bs[g] = (char*)ctx->b32.p + (size_t)g * nc * ldb * esz;
    }
    const int nvm = x.m->dm.nv;
    if (nvm < n)
      ck(cudaMemsetAsync(bs[i0], 0, (size_t)x.cnt * nc * ldb * esz, ctx->stream), "memset padded rhs");
    const void* drive = mixed ? x.m->drive32.p : x.m->drive64.p;
    T.launches += assemble_frequencies(ctx, x.m, prec, x.cnt, ks.data() + i0, cs.data() + i0, As.data() + i0,
                                       mixed ? A2s.data() + i0 : nullptr, qs.data() + i0, nc, drive, bs.data() + i0,
                                       lda, ldb, &T.regular_flop, &T.cheb_freqs, x.cheb);
    if (nvm < n) {
      dim3 g((unsigned)n, (unsigned)x.cnt);
      if (mixed)
        pad_identity_kernel<float2><<<g, 128, 0, ctx->stream>>>((float2*)As[i0], (float2*)A2s[i0], lda,
                                                                (long long)lda * n, nvm, n);
      else
        pad_identity_kernel<double2><<<g, 128, 0, ctx->stream>>>((double2*)As[i0], nullptr, lda, (long long)lda * n,
                                                                 nvm, n);
      ck(cudaGetLastError(), "pad kernel");
      T.launches += 1;
    }
    i0 += x.cnt;
  }
  cudaEventRecord(ctx->ev[1], ctx->stream);
  ck(cudaMemsetAsync(ctx->info.p, 0, (size_t)B * sizeof(int), ctx->stream), "memset info");
  bool used_tensor = false;
  int* tc_err = nullptr;
  void* tcws = nullptr;
  if (mixed && o.lu_gemm != (int)bem::LuGemm::Cublas && bem::tc_gemm_available()) {
    ck(ctx->tcws.ensure(bem::tc_gemm_workspace_bytes(n, B)), "alloc tensor-core workspace");
    tcws = ctx->tcws.p;
  }
  int lu_launches = 0;
  ck(bem::lu_factor_batched(prec, ctx->mats.p, lda, n, B, (int*)ctx->ipiv.p, (int*)ctx->info.p, nb, ctx->cublas,
                            ctx->stream, (bem::LuGemm)o.lu_gemm, tcws, &used_tensor, &tc_err, (int*)ctx->rowmap.p,
                            &lu_launches),
     "LU factorisation");
  // kernels of this batch besides the assembly: the LU, the permutation, the solves
  // (mixed: 6 + 6 per refinement step), the field (2, +1 mixed, per slice)
  T.launches += lu_launches + 1;
  T.gemm_used = mixed ? (used_tensor ? 2 : 1) : 0;
  ck(bem::lu_perm_batched((const int*)ctx->ipiv.p, n, B, (int*)ctx->perm.p, ctx->stream), "pivot permutation");
  prof_mark(ctx, BEM_K_LU);
  ck(cudaMemcpyAsync(info.data(), ctx->info.p, (size_t)B * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream),
     "copy info");
  const long long nvec = (long long)B * nc * ldb;
  if (!mixed) {
    ck(bem::lu_solve_cluster_batched(prec, ctx->mats.p, lda, n, B, (const int*)ctx->perm.p, ctx->b32.p, ldb, nc,
                                     ctx->stream),
       "LU solve");
    T.launches += 1;
  } else {
    double2* x = (double2*)ctx->x64.p;
    double2* r = (double2*)ctx->r64.p;
    double2* b64 = (double2*)ctx->b64.p;
    float2* d = (float2*)ctx->d32.p;
    ck(bem::convert_f32_to_f64((const float2*)ctx->b32.p, b64, nvec, ctx->stream), "convert rhs");
    ck(cudaMemcpyAsync(d, ctx->b32.p, nvec * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream), "copy rhs");
    ck(bem::lu_solve_cluster_batched(prec, ctx->mats.p, lda, n, B, (const int*)ctx->perm.p, d, ldb, nc, ctx->stream),
       "LU solve");
    ck(cudaMemsetAsync(x, 0, nvec * sizeof(double2), ctx->stream), "memset x");
    ck(bem::axpy_f32_into_f64(d, x, nvec, ctx->stream), "axpy");
    int steps = 0;
    double worst = 0;
    for (;;) {
      ck(bem::residual_batched(prec, ctx->mats2.p, lda, n, B, x, b64, ldb, nc, r, ctx->xsplit.p, ctx->stream),
         "residual");
      ck(bem::norms_batched(r, b64, ldb, n, B * nc, (double*)ctx->norms.p, ctx->stream), "norms");
      ck(cudaMemcpyAsync(norms.data(), ctx->norms.p, (size_t)B * nc * 2 * sizeof(double), cudaMemcpyDeviceToHost,
                         ctx->stream),
         "copy norms");
      ck(cudaStreamSynchronize(ctx->stream), "refinement sync");
      worst = 0;
      for (int i = 0; i < B * nc; ++i) {
        const double rel = norms[2 * i + 1] > 0 ? std::sqrt(norms[2 * i] / norms[2 * i + 1]) : std::sqrt(norms[2 * i]);
        if (!std::isfinite(rel)) worst = INFINITY;
        else worst = std::max(worst, rel);
      }
      if (worst <= o.refine_tol || steps >= o.max_refine || !std::isfinite(worst)) break;
      ck(bem::convert_f64_to_f32(r, d, nvec, ctx->stream), "convert residual");
      ck(bem::lu_solve_cluster_batched(prec, ctx->mats.p, lda, n, B, (const int*)ctx->perm.p, d, ldb, nc,
                                       ctx->stream),
         "LU solve");
      ck(bem::axpy_f32_into_f64(d, x, nvec, ctx->stream), "axpy");
      ++steps;
    }
    T.max_steps = std::max(T.max_steps, steps);
    T.max_res = std::max(T.max_res, worst);
    T.launches += 6 + 6LL * steps;  // 3 + (x split, residual, norms) per check + (convert, solve, axpy) per step
  }
  prof_mark(ctx, BEM_K_SOLVE);
  cudaEventRecord(ctx->ev[2], ctx->stream);
  ck(cudaStreamSynchronize(ctx->stream), "solve sync");
  if (used_tensor && tc_err) {
    int h = 0;
    ck(cudaMemcpyAsync(&h, tc_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "read tensor-core status");
    ck(cudaStreamSynchronize(ctx->stream), "read tensor-core status");
    if (h != 0)
      throw BemError{BEM_ERR_CUDA, "tensor-core LU update gave up waiting (status " + std::to_string(h) + ")"};
  }
  for (int i = 0; i < B; ++i)
    if (info[i] != 0)
      throw BemError{BEM_ERR_SINGULAR, "zero pivot in LU factorisation (frequency " + std::to_string(fz[i]) + " Hz)"};
  // solutions (vertex order) as [B][nc][ldb]
  const char* sol = mixed ? (const char*)ctx->x64.p : (const char*)ctx->b32.p;
  const cudaMemcpyKind kind = o.outputs_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (any_field && mixed)
    ck(bem::convert_f64_to_f32((const double2*)ctx->x64.p, (float2*)ctx->pout.p, nvec, ctx->stream), "convert");
  i0 = 0;
  for (const Slice& x : sl) {
    if (x.field_out) {
      const bem::DeviceMesh& dm = x.m->dm;
      const void* p_for_field = mixed ? (const void*)((const float2*)ctx->pout.p + (size_t)i0 * nc * ldb)
                                      : (const void*)((const double2*)ctx->b32.p + (size_t)i0 * nc * ldb);
      const void* drive = mixed ? x.m->drive32.p : x.m->drive64.p;
      ck(bem::launch_field(dm, prec, x.cnt, ks.data() + i0, qs.data() + i0, p_for_field, ldb, nc, drive,
                           (const double*)x.m->obs.p, x.m->nobs, ctx->fsrc.p, (double2*)ctx->fout.p, ctx->stream),
         "field kernel");
      T.launches += 2;
      ck(cudaMemcpyAsync(x.field_out, ctx->fout.p, (size_t)x.cnt * nc * x.m->nobs * sizeof(double2), kind,
                         ctx->stream),
         "copy field");
    }
    i0 += x.cnt;
  }
  if (any_field) {
    if (mixed) T.launches += 1;
    prof_mark(ctx, BEM_K_FIELD);
  }
  cudaEventRecord(ctx->ev[3], ctx->stream);
  i0 = 0;
  for (const Slice& x : sl) {
    if (x.pressure_out) {  // [cnt][nc][nv] complex128 from [cnt][nc][ldb]
      const int nvm = x.m->dm.nv;
      ck(cudaMemcpy2DAsync(x.pressure_out, (size_t)nvm * sizeof(double2), sol + (size_t)i0 * nc * ldb * sizeof(double2),
                           (size_t)ldb * sizeof(double2), (size_t)nvm * sizeof(double2), (size_t)x.cnt * nc, kind,
                           ctx->stream),
         "copy pressure");
    }
    i0 += x.cnt;
  }
  ck(cudaStreamSynchronize(ctx->stream), "batch sync");
  prof_collect(ctx, T.kacc);
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  T.t_asm += ms * 1e-3;
  cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
  T.t_sol += ms * 1e-3;
  cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
  T.t_fld += ms * 1e-3;
}

void fill_stats(bem_solve_stats* stats, const SolveTotals& T) {
  if (!stats) return;
  stats->assembly_s = T.t_asm;
  stats->solve_s = T.t_sol;
  stats->field_s = T.t_fld;
  stats->max_refine_steps = T.max_steps;
  stats->max_rel_residual = T.max_res;
  stats->batches = T.batches;
  for (int i = 0; i < 8; ++i) stats->kernel_s[i] = T.kacc[i];
  stats->lu_gemm_used = T.gemm_used;
  stats->kernel_launches = T.launches;
  stats->regular_flop = T.regular_flop;
  stats->singular_cheb_freqs = T.cheb_freqs;
}

bool valid_options(bem_context* ctx, const bem_solve_options& o) {
  if (!(o.sound_speed > 0) || !(o.rho > 0)) {
    fail(ctx, BEM_ERR_INVALID_ARGUMENT, "sound_speed and rho must be > 0");
    return false;
  }
  if (o.precision != BEM_PRECISION_FP64 && o.precision != BEM_PRECISION_MIXED) {
    fail(ctx, BEM_ERR_INVALID_ARGUMENT, "unknown precision");
    return false;
  }
  return true;
}

bool valid_freqs(bem_context* ctx, const double* freqs_hz, int n_freq) {
  if (!freqs_hz || n_freq < 1) {
    fail(ctx, BEM_ERR_INVALID_ARGUMENT, "need at least one frequency");
    return false;
  }
  for (int i = 0; i < n_freq; ++i)
    if (!(freqs_hz[i] > 0) || !std::isfinite(freqs_hz[i])) {
      fail(ctx, BEM_ERR_INVALID_ARGUMENT, "frequencies must be finite and positive");
      return false;
    }
  return true;
}
}  // namespace

extern "C" {

int bem_auto_batch(bem_mesh* m, int precision, int n_freq) {
  if (!m) return 0;
  return guarded(m->ctx, [&]() -> int {
    return auto_batch(m, precision == BEM_PRECISION_FP64 ? bem::Precision::FP64 : bem::Precision::Mixed, n_freq);
  });
}

long long bem_estimate_device_bytes(int nv, int nf, int npairs, int nrhs, int npts, int batch, int precision) {
  const long long esz = precision == BEM_PRECISION_MIXED ? 8 : 16;
  const long long lda = round_up(nv, 32);
  const long long n_ext = (long long)(nv * 1.3) + 64;
  long long bytes = 0;
  const long long group = precision == BEM_PRECISION_MIXED ? 4 : 1;        // frequencies assembled together
  bytes += round_up(n_ext, 32) * 3LL * nf * esz * group;                    // extended rows
  bytes += (long long)batch * lda * nv * esz * (precision == BEM_PRECISION_MIXED ? 2 : 1);  // matrices (+copy)
  bytes += (long long)npairs * (12 * esz * group + 24 * 8 + 48 + (bem::kPairRec + bem::kPairGeoDf) * 4 + 96 +
                                bem::kChebN * 24 * 4);  // singular blocks, moments, pairs, records, scatter plan, Chebyshev moments
  bytes += (long long)batch * nrhs * lda * (esz + 3 * 16 + 16);             // rhs, x, r, b64, d
  bytes += (long long)batch * nrhs * ((long long)nf * 6 * esz + (long long)npts * 16);  // field sources + out
  bytes += (long long)nf * (2 * 160 + 288 + 64);                            // face records (+ lane-group copy), maps
  if (precision == BEM_PRECISION_MIXED)                                      // tensor-core update operands
    bytes += (long long)bem::tc_gemm_workspace_bytes(nv, batch);
  bytes += 64LL << 20;                                                      // cuBLAS workspace and slack
  return bytes;
}

int bem_solve_frequencies(bem_mesh* m, const double* freqs_hz, int n_freq, const bem_solve_options* opt,
                          double* pressure_out, double* field_out, bem_solve_stats* stats) {
  if (!m) return BEM_ERR_INVALID_ARGUMENT;
  bem_context* ctx = m->ctx;
  return guarded(ctx, [&]() -> int {
    bem_solve_options o;
    bem_default_options(&o);
    if (opt) o = *opt;
    if (!valid_freqs(ctx, freqs_hz, n_freq)) return BEM_ERR_INVALID_ARGUMENT;
    if (m->nc < 1) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "no excitation set (bem_set_excitation)");
    if (field_out && m->nobs < 1) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "no observation points set");
    if (!valid_options(ctx, o)) return BEM_ERR_INVALID_ARGUMENT;
    const bem::Precision prec = o.precision == BEM_PRECISION_MIXED ? bem::Precision::Mixed : bem::Precision::FP64;
    const bool cheb = prec == bem::Precision::Mixed && n_freq >= kChebMinFreqs;
    if (cheb) {
      std::vector<double> kw(n_freq);
      for (int i = 0; i < n_freq; ++i) kw[i] = 2.0 * M_PI * freqs_hz[i] / o.sound_speed;
      ensure_cheb(ctx, m, kw.data(), n_freq);
    }
    const bem::DeviceMesh& dm = m->dm;
    const int nv = dm.nv, nc = m->nc;
    int B = o.batch > 0 ? std::min(o.batch, 64) : auto_batch(m, prec, n_freq);
    B = std::min(B, n_freq);
    ctx->prof = o.profile != 0;
    const int nbatch = (n_freq + B - 1) / B;
    auto slice_of = [&](int bi) {
      const int f0 = bi * B, bt = std::min(B, n_freq - f0);
      return Slice{m, freqs_hz + f0, bt, pressure_out ? pressure_out + 2 * (size_t)f0 * nc * nv : nullptr,
                   field_out ? field_out + 2 * (size_t)f0 * nc * m->nobs : nullptr, cheb};
    };
    SolveTotals T;
    const int nl = std::max(1, std::min({o.lanes, kMaxLanes, nbatch}));
    if (nl >= 2) {
      // batch bi goes to lane bi % nl: lane 0 is this context, the others are helper contexts
      // driven from their own host threads; the mesh is shared read-only
      while ((int)ctx->lanes.size() < nl - 1) {
        bem_context* c2 = nullptr;
        const int rc = bem_create_context(ctx->device, &c2);
        if (rc != BEM_OK) return fail(ctx, rc, "cannot create a lane's context");
        ctx->lanes.push_back(c2);
      }
      std::vector<SolveTotals> TL(nl - 1);
      std::vector<int> failed(nl - 1, 0);
      std::vector<BemError> errs(nl - 1, BemError{BEM_OK, std::string()});
      std::vector<std::thread> threads;
      for (int l = 1; l < nl; ++l) {
        bem_context* cl = ctx->lanes[l - 1];
        cl->prof = ctx->prof;
        threads.emplace_back([&, l, cl] {
          cudaSetDevice(ctx->device);
          try {
            for (int bi = l; bi < nbatch; bi += nl) solve_combined(cl, {slice_of(bi)}, nv, o, nc, TL[l - 1]);
          } catch (const BemError& e) {
            errs[l - 1] = e;
            failed[l - 1] = 1;
          } catch (const std::exception& e) {
            errs[l - 1] = BemError{BEM_ERR_CUDA, std::string("lane: ") + e.what()};
            failed[l - 1] = 1;
          }
        });
      }
      try {
        for (int bi = 0; bi < nbatch; bi += nl) solve_combined(ctx, {slice_of(bi)}, nv, o, nc, T);
      } catch (...) {
        for (auto& t : threads) t.join();
        throw;
      }
      for (auto& t : threads) t.join();
      for (int l = 0; l < nl - 1; ++l)
        if (failed[l]) throw errs[l];
      for (const SolveTotals& T2 : TL) {
        for (int i = 0; i < BEM_K_SLOTS; ++i) T.kacc[i] += T2.kacc[i];
        T.regular_flop += T2.regular_flop;
        T.cheb_freqs += T2.cheb_freqs;
        T.t_asm += T2.t_asm;
        T.t_sol += T2.t_sol;
        T.t_fld += T2.t_fld;
        T.max_res = std::max(T.max_res, T2.max_res);
        T.max_steps = std::max(T.max_steps, T2.max_steps);
        T.batches += T2.batches;
        T.gemm_used = std::max(T.gemm_used, T2.gemm_used);
        T.launches += T2.launches;
      }
    } else {
      for (int bi = 0; bi < nbatch; ++bi) solve_combined(ctx, {slice_of(bi)}, nv, o, nc, T);
    }
    fill_stats(stats, T);
    if (stats) {
      stats->regular_pairs = (long long)dm.ntr * dm.nf * dm.nf - dm.npairs;  // identity and image pairs
      stats->singular_pairs = dm.npairs;
      stats->singular_points = m->singular_points;
    }
    if (prec == bem::Precision::Mixed && !(T.max_res <= o.refine_tol)) {
      ctx->err = "iterative refinement stopped at relative residual " + std::to_string(T.max_res);
      return BEM_ERR_NOT_CONVERGED;
    }
    return BEM_OK;
  });
}

int bem_solve_jobs(bem_context* ctx, const bem_job* jobs, int n_jobs, const bem_solve_options* opt,
                   bem_solve_stats* stats) {
  if (!ctx) return BEM_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&]() -> int {
    bem_solve_options o;
    bem_default_options(&o);
    if (opt) o = *opt;
    if (!jobs || n_jobs < 1) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "need at least one job");
    if (!valid_options(ctx, o)) return BEM_ERR_INVALID_ARGUMENT;
    int n = 0, nc = -1, total = 0;
    for (int j = 0; j < n_jobs; ++j) {
      const bem_job& J = jobs[j];
      if (!J.mesh || J.mesh->ctx != ctx) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "job mesh missing or of another context");
      if (!valid_freqs(ctx, J.freqs_hz, J.n_freq)) return BEM_ERR_INVALID_ARGUMENT;
      if (J.mesh->nc < 1) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "no excitation set (bem_set_excitation)");
      if (nc >= 0 && J.mesh->nc != nc)
        return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "every job of a call needs the same number of excitations");
      nc = J.mesh->nc;
      if (J.field_out && J.mesh->nobs < 1) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "no observation points set");
      n = std::max(n, J.mesh->dm.nv);
      total += J.n_freq;
    }
    const bem::Precision prec = o.precision == BEM_PRECISION_MIXED ? bem::Precision::Mixed : bem::Precision::FP64;
    int B = o.batch > 0 ? std::min(o.batch, 64) : auto_batch_order(n, prec, total);
    B = std::max(1, std::min(B, total));
    ctx->prof = o.profile != 0;
    SolveTotals T;
    // walk the jobs' frequencies in order, cutting them into batches of B
    int j = 0, f = 0;
    while (j < n_jobs) {
      std::vector<Slice> batch;
      int left = B;
      while (left > 0 && j < n_jobs) {
        const bem_job& J = jobs[j];
        const int take = std::min(left, J.n_freq - f);
        const int nvj = J.mesh->dm.nv;
        batch.push_back(Slice{J.mesh, J.freqs_hz + f, take,
                              J.pressure_out ? J.pressure_out + 2 * (size_t)f * nc * nvj : nullptr,
                              J.field_out ? J.field_out + 2 * (size_t)f * nc * J.mesh->nobs : nullptr});
        left -= take;
        f += take;
        if (f == J.n_freq) {
          ++j;
          f = 0;
        }
      }
      solve_combined(ctx, batch, n, o, nc, T);
    }
    fill_stats(stats, T);
    if (stats) {  // summed over the jobs' meshes
      stats->regular_pairs = stats->singular_pairs = stats->singular_points = 0;
      for (int q = 0; q < n_jobs; ++q) {
        const bem::DeviceMesh& dm = jobs[q].mesh->dm;
        stats->regular_pairs += (long long)dm.ntr * dm.nf * dm.nf - dm.npairs;
        stats->singular_pairs += dm.npairs;
        stats->singular_points += jobs[q].mesh->singular_points;
      }
    }
    if (prec == bem::Precision::Mixed && !(T.max_res <= o.refine_tol)) {
      ctx->err = "iterative refinement stopped at relative residual " + std::to_string(T.max_res);
      return BEM_ERR_NOT_CONVERGED;
    }
    return BEM_OK;
  });
}

int bem_lu_factor_dense(bem_context* ctx, int n, double* a, int* ipiv, int precision, int lu_gemm) {
  if (!ctx) return BEM_ERR_INVALID_ARGUMENT;
  return guarded(ctx, [&]() -> int {
    if (!a || !ipiv || n < 1) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "bad arguments");
    const bool mixed = precision == BEM_PRECISION_MIXED;
    const bem::Precision prec = mixed ? bem::Precision::Mixed : bem::Precision::FP64;
    const long long lda = round_up(n, 32);
    const size_t esz = mixed ? sizeof(float2) : sizeof(double2);
    ck(ctx->mats.ensure((size_t)lda * n * esz), "alloc matrix");
    ck(ctx->ipiv.ensure((size_t)n * sizeof(int)), "alloc pivots");
    ck(ctx->info.ensure(sizeof(int)), "alloc info");
    ck(ctx->rowmap.ensure(bem::kRowmapStride * sizeof(int)), "alloc row map");
    std::vector<char> host((size_t)lda * n * esz, 0);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double re = a[2 * ((size_t)j * n + i)], im = a[2 * ((size_t)j * n + i) + 1];
        if (mixed)
          ((float2*)host.data())[(size_t)j * lda + i] = make_float2((float)re, (float)im);
        else
          ((double2*)host.data())[(size_t)j * lda + i] = make_double2(re, im);
      }
    ck(cudaMemcpyAsync(ctx->mats.p, host.data(), host.size(), cudaMemcpyHostToDevice, ctx->stream), "copy matrix");
    ck(cudaMemsetAsync(ctx->info.p, 0, sizeof(int), ctx->stream), "memset info");
    void* tcws = nullptr;
    if (mixed && lu_gemm != (int)bem::LuGemm::Cublas && bem::tc_gemm_available()) {
      ck(ctx->tcws.ensure(bem::tc_gemm_workspace_bytes(n, 1)), "alloc tensor-core workspace");
      tcws = ctx->tcws.p;
    }
    bool used_tensor = false;
    int* tc_err = nullptr;
    ck(bem::lu_factor_batched(prec, ctx->mats.p, lda, n, 1, (int*)ctx->ipiv.p, (int*)ctx->info.p, 0, ctx->cublas,
                              ctx->stream, (bem::LuGemm)lu_gemm, tcws, &used_tensor, &tc_err, (int*)ctx->rowmap.p),
       "LU factorisation");
    int info = 0;
    ck(cudaMemcpyAsync(host.data(), ctx->mats.p, host.size(), cudaMemcpyDeviceToHost, ctx->stream), "copy factors");
    ck(cudaMemcpyAsync(ipiv, ctx->ipiv.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "copy pivots");
    ck(cudaMemcpyAsync(&info, ctx->info.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "copy info");
    ck(cudaStreamSynchronize(ctx->stream), "sync");
    if (used_tensor && tc_err) {
      int h = 0;
      ck(cudaMemcpyAsync(&h, tc_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "read tensor-core status");
      ck(cudaStreamSynchronize(ctx->stream), "read tensor-core status");
      if (h != 0) return fail(ctx, BEM_ERR_CUDA, "tensor-core LU update gave up waiting");
    }
    if (lu_gemm == (int)bem::LuGemm::Tensor && mixed && !used_tensor)
      return fail(ctx, BEM_ERR_CUDA, "tensor-core trailing update unavailable");
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double re, im;
        if (mixed) {
          const float2 x = ((const float2*)host.data())[(size_t)j * lda + i];
          re = x.x;
          im = x.y;
        } else {
          const double2 x = ((const double2*)host.data())[(size_t)j * lda + i];
          re = x.x;
          im = x.y;
        }
        a[2 * ((size_t)j * n + i)] = re;
        a[2 * ((size_t)j * n + i) + 1] = im;
      }
    if (info != 0) return fail(ctx, BEM_ERR_SINGULAR, "zero pivot at column " + std::to_string(info - 1));
    return BEM_OK;
  });
}

int bem_assemble_lhs(bem_mesh* m, double k, int precision, const double* coeffs, double* out) {
  if (!m) return BEM_ERR_INVALID_ARGUMENT;
  bem_context* ctx = m->ctx;
  return guarded(ctx, [&]() -> int {
    if (!coeffs || !out || !(k > 0)) return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "bad arguments");
    const bem::Precision prec = precision == BEM_PRECISION_MIXED ? bem::Precision::Mixed : bem::Precision::FP64;
    const bem::DeviceMesh& dm = m->dm;
    Layout L = layout_for(dm, prec);
    bem::OperatorCoeffs c{};
    c.cD = make_double2(coeffs[0], coeffs[1]);
    c.cH = make_double2(coeffs[2], coeffs[3]);
    c.cM = make_double2(coeffs[4], coeffs[5]);
    const size_t matsz = (size_t)L.lda * dm.nv * L.esz;
    ck(ctx->mats.ensure(matsz), "alloc matrix");
    assemble_one(m, prec, k, c, ctx->mats.p, nullptr, make_double2(0, 0), 0, nullptr, nullptr);
    std::vector<char> host(matsz);
    ck(cudaMemcpyAsync(host.data(), ctx->mats.p, matsz, cudaMemcpyDeviceToHost, ctx->stream), "copy matrix");
    ck(cudaStreamSynchronize(ctx->stream), "sync");
    const int nv = dm.nv;
    for (int j = 0; j < nv; ++j)
      for (int r = 0; r < nv; ++r) {
        const int v = m->plan.row_vertex[r];
        double re, im;
        if (prec == bem::Precision::Mixed) {
          const float2 x = ((const float2*)host.data())[(size_t)j * L.lda + r];
          re = x.x;
          im = x.y;
        } else {
          const double2 x = ((const double2*)host.data())[(size_t)j * L.lda + r];
          re = x.x;
          im = x.y;
        }
        out[2 * ((size_t)j * nv + v)] = re;
        out[2 * ((size_t)j * nv + v) + 1] = im;
      }
    return BEM_OK;
  });
}

int bem_apply_rhs_operator(bem_mesh* m, double k, int precision, const double* coeffs, const double* q, int n_rhs,
                           double* out) {
  if (!m) return BEM_ERR_INVALID_ARGUMENT;
  bem_context* ctx = m->ctx;
  return guarded(ctx, [&]() -> int {
    if (!coeffs || !q || !out || n_rhs < 1 || n_rhs > 4 || !(k > 0))
      return fail(ctx, BEM_ERR_INVALID_ARGUMENT, "bad arguments");
    const bem::Precision prec = precision == BEM_PRECISION_MIXED ? bem::Precision::Mixed : bem::Precision::FP64;
    // route q through the excitation slots with qscale = 1
    const int saved_nc = m->nc;
    int rc = bem_set_excitation(m, q, n_rhs);
    if (rc != BEM_OK) return rc;
    const bem::DeviceMesh& dm = m->dm;
    Layout L = layout_for(dm, prec);
    bem::OperatorCoeffs c{};
    c.cS = make_double2(coeffs[0], coeffs[1]);
    c.cK = make_double2(coeffs[2], coeffs[3]);
    c.cM10 = make_double2(coeffs[4], coeffs[5]);
    const size_t matsz = (size_t)L.lda * dm.nv * L.esz;
    ck(ctx->mats.ensure(matsz), "alloc matrix");
    ck(ctx->b32.ensure((size_t)n_rhs * L.ldb * L.esz), "alloc rhs");
    const void* drive = prec == bem::Precision::Mixed ? m->drive32.p : m->drive64.p;
    assemble_one(m, prec, k, c, ctx->mats.p, nullptr, make_double2(1.0, 0.0), n_rhs, drive, ctx->b32.p);
    std::vector<char> host((size_t)n_rhs * L.ldb * L.esz);
    ck(cudaMemcpyAsync(host.data(), ctx->b32.p, host.size(), cudaMemcpyDeviceToHost, ctx->stream), "copy rhs");
    ck(cudaStreamSynchronize(ctx->stream), "sync");
    (void)saved_nc;
    const int nv = dm.nv;
    for (int c2 = 0; c2 < n_rhs; ++c2)
      for (int r = 0; r < nv; ++r) {
        const int v = m->plan.row_vertex[r];
        double re, im;
        if (prec == bem::Precision::Mixed) {
          const float2 x = ((const float2*)host.data())[(size_t)c2 * L.ldb + r];
          re = x.x;
          im = x.y;
        } else {
          const double2 x = ((const double2*)host.data())[(size_t)c2 * L.ldb + r];
          re = x.x;
          im = x.y;
        }
        out[2 * ((size_t)c2 * nv + v)] = re;
        out[2 * ((size_t)c2 * nv + v) + 1] = im;
      }
    return BEM_OK;
  });
}

}  // extern "C"
