// Internal launcher interface between the context layer (bem_capi.cu) and the
// kernel files.  Not part of the public C ABI (see include/gb300_bem.h).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "bem_internal.h"

namespace bem {

// Raise a kernel's dynamic shared-memory limit (cudaFuncAttributeMaxDynamic-
// SharedMemorySize) to at least `bytes` on the current device.  The attribute
// belongs to the function, process-wide: contexts on other threads launch the
// same kernels with other sizes, so the limit only ever grows (under a lock) and
// a concurrent caller can never lower it between another's set and launch.
bool ensure_smem_limit(const void* func, size_t bytes);


enum class Precision : int { FP64 = 0, Mixed = 1 };

// Linear-combination coefficients.  LHS = cD*D + cH*H + cM*M11;
// RHS operator = cS*S + cK*K' + cM10*M10.  The Burton-Miller system of the
// reference (BeatEngineCpuSolve.jl:45-53) is cD=-1, cH=i/k, cM=1/2,
// cS=-1, cK=-i/k, cM10=-i/(2k).
struct OperatorCoeffs {
  double2 cD, cH, cM, cS, cK, cM10;
};

struct DeviceMesh {
  int nv = 0, nf = 0, Q = 0;
  int n_tiles = 0, max_tile_rows = 0, n_ext = 0, n_halo = 0, n_halo_rows = 0;
  int npairs = 0, n_isolated = 0, ndriven = 0;
  FaceF32* faces32 = nullptr;
  FaceF64* faces64 = nullptr;
  int* tile_group_ptr = nullptr;
  LaneSlot* lane_slots = nullptr;
  float* group_faces32 = nullptr;  // lane groups' test faces, field-major
  int* tile_row_base = nullptr;
  int* ext_row = nullptr;
  int* halo_slot_of_ext = nullptr;
  int* halo_row_ptr = nullptr;
  int* halo_row = nullptr;
  int* col_ptr = nullptr;
  int* col_fb = nullptr;
  int* face_ext = nullptr;
  int* vertex_row = nullptr;
  int* isolated = nullptr;
  SingularPair* pairs = nullptr;
  int* pairs_by_trial_ptr = nullptr;
  int* pairs_by_test_ptr = nullptr;
  int* pairs_by_test = nullptr;
  int n_scat = 0;  // singular scatter entries (see MeshPlan::scat_*)
  int* scat_col = nullptr;
  int* scat_row = nullptr;
  int* scat_ptr = nullptr;
  int* scat_src = nullptr;
  int* rule_ptr = nullptr;
  double* duffy = nullptr;
  float* duffy32 = nullptr;  // the same table rounded to float (mixed form)
  float* duffy_df = nullptr;  // the same table as double-float (hi, lo) pairs: 10 floats per point
  float* pairgeo_df = nullptr;  // npairs x kPairGeoDf: per-pair geometry as double-float (moments kernel)
  double* moments = nullptr;
  float* pairrec = nullptr;  // npairs x kPairRec: FP32 record of each pair for the mixed-form singular kernel
  // Chebyshev moments of the singular remainder (mixed form; npairs x kChebN x 24 floats, see
  // singular_cheb_moments_kernel) on r in [0, cheb_R], cheb_R bounding every vertex-sharing
  // pair's point distances; allocated by the first sweep that uses them
  float* cheb = nullptr;
  double cheb_R = 0.0;
  int cheb_n = 0;  // terms the moments hold (0: none yet)
  double* verts = nullptr;
  int* faces = nullptr;
  double* normal = nullptr;
  double* curls = nullptr;
  double* area = nullptr;
  double* m11m10 = nullptr;  // 9 + 3 doubles
  float m11m10f[12] = {0};   // the same, rounded to float (host copy, passed as a kernel parameter)
  int* driven = nullptr;
  // symmetry: transforms applied to trial faces (0 identity, 1 x, 2 y, 3 xy),
  // per-vertex plane masks, per-matrix-row orbit weights (null when off)
  int ntr = 1;
  int tr[4] = {0, 0, 0, 0};
  unsigned char* fix_mask = nullptr;
  double* row_weight = nullptr;
  // regular rule: weights w_q, basis values phi_a(xi_q) (a-major, 3 x Q) and
  // their products cw[a*Q + q] = phi_a(xi_q) w_q
  double rule_w[kMaxQ] = {0};
  double rule_phi[3 * kMaxQ] = {0};
  double rule_cw[3 * kMaxQ] = {0};
};

// assembly (bem_assembly.cu)
// Regular pairs of nfreq frequencies into nfreq extended-row buffers (Rext +
// f * strideR elements); the mixed form evaluates two frequencies per launch.
cudaError_t launch_regular(const DeviceMesh& m, Precision prec, int nfreq, const double* k, const double2* cD,
                           const double2* cH, void* Rext, long long ldR, long long strideR, cudaStream_t stream);
// Frequencies assembled per regular-kernel launch for a batch of nfreq (mixed:
// fours, or twos when four frequencies' accumulators do not fit two CTAs per SM;
// FP64: ones); writes the group sizes (nfreq <= 64) and returns their count.
int regular_groups(const DeviceMesh& m, Precision prec, int nfreq, int* sizes);
int regular_launches(const DeviceMesh& m, Precision prec, int nfreq);
// FP32 flop per quadrature pair and frequency of the mixed-form regular kernel
// when w frequencies share a launch (FMA = 2, counted from its source).
double regular_flop_per_qpair(int w);
cudaError_t launch_regular_f64(const DeviceMesh& m, double k, double2 cD, double2 cH, double2* Rext, long long ldR,
                               cudaStream_t stream);
// Per-pair FP32 record written at upload by the pair setup and moments kernels (see bem_assembly.cu).
constexpr int kPairRec = 64;
// Chebyshev terms of the mixed form's singular remainder expansion (bem_assembly.cu).
constexpr int kChebN = 24;
constexpr int kPairGeoDf = 48;
cudaError_t launch_singular_static(const DeviceMesh& m, double* moments, float* pairrec, cudaStream_t stream);
// Singular blocks of nfreq frequencies; frequency f's blocks start at element
// f * blocks_stride of blocks (the mixed form takes two frequencies per launch).
// use_cheb (mixed form): take the mesh's Chebyshev moments for the frequencies whose
// expansion they cover.  Adds the kernels it launched to *launched and the frequencies it
// formed from the moments to *cheb_freqs (when not null).
cudaError_t launch_singular_dyn(const DeviceMesh& m, Precision prec, int nfreq, const double* k,
                                const OperatorCoeffs* c, void* blocks, long long blocks_stride, cudaStream_t stream,
                                long long* launched = nullptr, long long* cheb_freqs = nullptr,
                                bool use_cheb = false);
// Chebyshev terms (a multiple of four, 8..kChebN) that expand the singular remainder of
// wavenumber k on [0, R] to 1e-9; 0 when kChebN terms are not enough.
int cheb_terms(double k, double R);
// The mesh's Chebyshev moments for the first nterms terms into m.cheb (after the pair setup).
cudaError_t launch_cheb_moments(const DeviceMesh& m, int nterms, cudaStream_t stream);
cudaError_t launch_singular_scatter(const DeviceMesh& m, Precision prec, const void* blocks, void* Rext,
                                    long long ldR, cudaStream_t stream);
cudaError_t launch_gather(const DeviceMesh& m, Precision prec, const void* Rext, long long ldR, void* A, long long lda,
                          void* A2, cudaStream_t stream);
cudaError_t launch_rhs(const DeviceMesh& m, Precision prec, double k, const OperatorCoeffs& c, double2 qscale,
                       const void* drive, int nc, const void* sblocks, void* rb, void* b, long long ldb,
                       cudaStream_t stream);
// Right-hand sides of nfreq frequencies, up to rhs_width(prec, nc) per face-kernel launch;
// frequency f's singular blocks start at element f * sblocks_stride of sblocks, and rb needs
// room for max(4, nc) * nf * 3 complex values.
int rhs_width(Precision prec, int nc);
cudaError_t launch_rhs_freqs(const DeviceMesh& m, Precision prec, int nfreq, const double* k, const OperatorCoeffs* c,
                             const double2* qscale, const void* drive, int nc, const void* sblocks,
                             long long sblocks_stride, void* rb, void* const* b, long long ldb, cudaStream_t stream);
int rhs_launches(Precision prec, int nc, int nfreq);

// dense LU and solves (bem_lu.cu).  Matrices are column-major, batched with a
// stride of lda*n elements; pivots are 0-based, ipiv stride n.
// Trailing-update GEMM of the mixed-precision LU: 0 = automatic (tensor cores
// when available), 1 = cuBLAS cgemm (FP32), 2 = tcgen05 3xFP16, scaled (bem_gemm_tc.cu).
enum class LuGemm : int { Auto = 0, Cublas = 1, Tensor = 2 };
struct TcGemmPlan;
size_t tc_gemm_workspace_bytes(int n, int batch);
bool tc_gemm_available();
// Number of SMs of the current device, cached per device (bem_gemm_tc.cu).
int sm_count();
int* tc_gemm_error_word(TcGemmPlan* p);
// Factor `batch` matrices in place.  tc_workspace (tc_gemm_workspace_bytes(n,
// batch) bytes, may be null) enables the tensor-core update; *used_tensor tells
// which update ran; *tc_err receives the device address of the kernel's error word.
// rowmap (batch * kRowmapStride ints, may be null) lets the cluster panel hand
// the net row permutation of its interchanges to the row-swap kernel.
constexpr int kRowmapStride = 512;
// Outer block width of the two-level LU (trailing-update depth); a multiple of
// every cluster panel width (32, 64) and at most the tcgen05 update's K (256).
// At 256 the trailing matrix is read and written once per 256 columns: with the
// 3xFP16 update that halves the HBM traffic that bounds it (LU 2.91 -> 2.79 ms
// per frequency at n = 4,976 against 128).
constexpr int kOuterBlock = 256;
// Kernels the two-level LU launches for one batch (cuBLAS kernels not counted).
int lu_launch_count(int n, int nb, int NB, bool tensor);
cudaError_t lu_factor_batched(Precision prec, void* A, long long lda, int n, int batch, int* ipiv, int* info,
                              int nb, void* cublas_handle, cudaStream_t stream, LuGemm gemm = LuGemm::Cublas,
                              void* tc_workspace = nullptr, bool* used_tensor = nullptr, int** tc_err = nullptr,
                              int* rowmap = nullptr, int* n_launches = nullptr);
// Solve (LU) X = B in place for nrhs columns per matrix (B stride ldb*nrhs per matrix), working precision.
cudaError_t lu_solve_batched(Precision prec, const void* LU, long long lda, int n, int batch, const int* ipiv,
                             void* B, long long ldb, int nrhs, int nb, cudaStream_t stream);
// r = b - A x in FP64 arithmetic: A (complex64 or complex128), x, b, r complex128.
cudaError_t residual_batched(Precision prec, const void* A, long long lda, int n, int batch, const double2* x,
                             const double2* b, long long ldb, int nrhs, double2* r, void* xsplit, cudaStream_t stream);
// Per (matrix, rhs): out[2*i] = ||r_i||^2 and out[2*i+1] = ||b_i||^2.
cudaError_t norms_batched(const double2* r, const double2* b, long long ldb, int n, int count, double* out,
                          cudaStream_t stream);
// Cluster-resident panel (bem_lu_cluster.cu).  lu_cluster_plan picks the panel
// width (64 or 32) and cluster size for an n x n matrix; false when no cluster
// configuration fits (then the single-CTA panel is used).
bool lu_cluster_plan(Precision prec, int n, int want_nb, int batch, int* nb, int* cl);
int lu_resident_batch(Precision prec, int n);
// rowmap: if not null, receives per matrix [count, (dst row, src row) x count]:
// the net effect of the panel's kb interchanges on any column (at most 2 kb rows).
cudaError_t lu_panel_cluster(Precision prec, void* A, long long lda, long long strideA, int n, int k, int kb, int nb,
                             int cl, int batch, int* ipiv, int* info, cudaStream_t stream, int* rowmap = nullptr);
// Apply a panel's net row permutation (rowmap) to every column outside the panel.
cudaError_t lu_swap_rows_batched(Precision prec, void* A, long long lda, long long strideA, int n, int k, int kb,
                                 int batch, const int* rowmap, cudaStream_t stream);
// perm[i]: (P b)[i] = b[perm[i]]; then one cluster per right-hand side solves in place.
cudaError_t lu_perm_batched(const int* ipiv, int n, int batch, int* perm, cudaStream_t stream);
cudaError_t lu_solve_cluster_batched(Precision prec, const void* LU, long long lda, int n, int batch, const int* perm,
                                     void* B, long long ldb, int nrhs, cudaStream_t stream);
// x += d (d complex64) ; copy / convert helpers
cudaError_t axpy_f32_into_f64(const float2* d, double2* x, long long n, cudaStream_t stream);
cudaError_t convert_f64_to_f32(const double2* src, float2* dst, long long n, cudaStream_t stream);
cudaError_t convert_f32_to_f64(const float2* src, double2* dst, long long n, cudaStream_t stream);

// far field (bem_field.cu)
cudaError_t launch_field(const DeviceMesh& m, Precision prec, int batch, const double* k, const double2* qscale,
                         const void* pressure, long long ldp, int nc, const void* drive, const double* obs, int nobs,
                         void* sources, double2* out, cudaStream_t stream);
// One frequency, one excitation, everything in caller-placed device buffers
// (face records FaceF32/FaceF64, weighted sources, drive with qscale = 1, a
// parameter block of field_params_bytes()).  Used by bem_noalloc.cu.
size_t field_params_bytes();
cudaError_t launch_field_single(Precision prec, const void* faces, int nf, int Q, const double* rule_w,
                                const double* rule_phi, const void* sources, const void* drive, const double* obs,
                                int nobs, double k, void* params, double2* out, cudaStream_t stream);

}  // namespace bem
