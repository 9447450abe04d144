/*
 * gb300_bem.h - C ABI of the GB300 exterior Helmholtz BEM backend.
 *
 * The reference (JWSound/boundary-lab) runs its exterior solve in a Julia
 * worker process; the Python adapter talks to it over a JSON request file and
 * NDJSON events (src/blab/solvers/beat_engine_backend.py:140-221, 286-462).
 * This library replaces the numerical part of that worker: the per-frequency
 * body of solve_request_impl (src/blab/solvers/julia_local/solver.jl:805-997),
 * i.e. operator assembly, the Burton-Miller LU solve and the field evaluation.
 * Each entry point below names the reference function it stands in for.
 *
 * Conventions
 *  - Every function returns an int status (BEM_OK == 0); on failure the
 *    context's last error message says why (bem_last_error).
 *  - Plain pointers and sizes only.  Host buffers are owned by the caller;
 *    device memory is owned by the context and freed by bem_destroy_context.
 *  - Complex arrays are interleaved (re, im) doubles.
 *  - Vertex and face indices are 0-based; faces are int32 triples.
 *  - A context owns one CUDA stream on one device and is thread-compatible:
 *    use one context per host thread (or serialise calls).
 *  - Frequencies of one call are solved as batches; results are identical to
 *    solving them one by one up to rounding order within FP32/FP64.
 */
#ifndef GB300_BEM_H
#define GB300_BEM_H

#ifdef __cplusplus
extern "C" {
#endif

#define GB300_BEM_ABI_VERSION 3

typedef struct bem_context bem_context;
typedef struct bem_mesh bem_mesh;

enum bem_status {
  BEM_OK = 0,
  BEM_ERR_INVALID_ARGUMENT = 1,
  BEM_ERR_CUDA = 2,
  BEM_ERR_OUT_OF_MEMORY = 3,
  BEM_ERR_SINGULAR = 4,     /* zero pivot in the LU factorisation */
  BEM_ERR_NOT_CONVERGED = 5 /* iterative refinement missed its tolerance */
};

enum bem_precision {
  BEM_PRECISION_FP64 = 0,  /* FP64 assembly, FP64 LU, FP64 field ("plain FP64 GPU form") */
  BEM_PRECISION_MIXED = 1  /* compensated FP32 assembly, FP32 LU, FP64 iterative refinement,
                              FP64-accurate singular moments, compensated FP32 field */
};

/* Library ABI version (GB300_BEM_ABI_VERSION). */
int bem_abi_version(void);

/* Create a context on CUDA device `device`.  Replaces the reference's
 * accelerator set-up in solver.jl:752-767 (device caches built per job). */
int bem_create_context(int device, bem_context** out);
void bem_destroy_context(bem_context* ctx);
/* Message of the last failed call on this context ("" if none). */
const char* bem_last_error(const bem_context* ctx);
/* The context's CUDA stream (a cudaStream_t), so a caller can order its own
 * work or record timing events against the library's launches. */
void* bem_context_stream(const bem_context* ctx);

/* Scratch memory control for schedulers that run several contexts on one GPU
 * (no direct counterpart in the reference, whose worker frees per-frequency
 * operator storage with release_operator_storage!, solver.jl:956).  A context
 * keeps its per-solve scratch (matrices, factors, right-hand sides) between
 * calls; all library device memory comes from one stream-ordered pool per
 * device.  bem_trim_context frees the context's scratch, waits for its stream
 * and returns unused pool memory to the device; uploaded meshes stay valid.
 * bem_context_scratch_bytes reports the scratch bytes the context holds now. */
int bem_trim_context(bem_context* ctx);
long long bem_context_scratch_bytes(const bem_context* ctx);

/* Upload a triangle mesh and build every frequency-independent cache: face
 * geometry and surface curls, the regular rule, singular (vertex-sharing) pair
 * list with remapped Duffy rules, and the k-independent singular moments (FP64
 * accuracy, computed in double-float on a second stream; the first solve waits for them).
 * Replaces load_combined_mesh + build_p1/dp0_space + triangle_rule +
 * build_singular_correction_cache + build_cuda_regular_assembly_cache +
 * build_cuda_singular_correction_cache (solver.jl:717-767,
 * BeatEngineCore.jl:236-256, 517-549, 875-915).
 * regular_order: 1..4 (4 = the six-point rule); singular_order: 1..4. */
int bem_upload_mesh(bem_context* ctx, const double* vertices, int n_vertices, const int* faces, int n_faces,
                    int regular_order, int singular_order, bem_mesh** out);
/* Symmetric models (no separate reference entry point: symmetry_mode of
 * solve_request_impl, solver.jl:685-736, with BeatEngineCore.jl:323-439): the
 * mesh is the fundamental domain (x >= 0 for BEM_SYMMETRY_X; x, y >= 0 for
 * BEM_SYMMETRY_XY), vertices within max(1e-9, 1e-6 x bounding-box diagonal) of a
 * plane are snapped onto it (a vertex on the negative side is an error), and
 * every operator, the right-hand side and the field include the reflected
 * images of every face (BeatEngineCpuAssembly.jl:411-445, 571-634), with rows
 * weighted by the vertex orbit weights.  Solutions are those of the full model
 * restricted to the fundamental domain. */
enum bem_symmetry { BEM_SYMMETRY_OFF = 0, BEM_SYMMETRY_X = 1, BEM_SYMMETRY_XY = 2 };
int bem_upload_mesh_symmetric(bem_context* ctx, const double* vertices, int n_vertices, const int* faces,
                              int n_faces, int regular_order, int singular_order, int symmetry, bem_mesh** out);
void bem_release_mesh(bem_mesh* mesh);
/* Sizes of an uploaded mesh (any output pointer may be NULL). */
int bem_mesh_info(const bem_mesh* mesh, int* n_vertices, int* n_faces, int* n_singular_pairs);

/* Excitations: n_rhs unit drive patterns, complex, row-major [n_rhs][n_faces].
 * The Neumann data of excitation c at angular frequency w is
 * q_c = i * rho * w * drive[c], as in pressure_for_drives (solver.jl:434-459).
 * 1 <= n_rhs <= 4. */
int bem_set_excitation(bem_mesh* mesh, const double* unit_drive, int n_rhs);
/* Observation points, row-major [n_points][3] in metres (solver.jl:320-388). */
int bem_set_observation_points(bem_mesh* mesh, const double* points, int n_points);

typedef struct bem_solve_options {
  int precision;         /* enum bem_precision */
  double sound_speed;    /* m/s */
  double rho;            /* kg/m^3 */
  double refine_tol;     /* mixed form: stop when ||b - A x|| / ||b|| <= refine_tol (FP64 residual) */
  int max_refine;        /* mixed form: maximum refinement steps */
  int batch;             /* frequencies factored together (<= 64); 0 = automatic (bem_auto_batch) */
  int lu_block;          /* LU panel width, 32 or 64 (trailing updates are 128 deep);
                            0 = automatic (the width whose panels run in the fewest waves) */
  int outputs_on_device; /* 1: pressure_out / field_out are device pointers of the context's device */
  int profile;           /* 1: also time each kernel family with CUDA events (stats.kernel_s) */
  int lu_gemm;           /* LU trailing update of the mixed form: 0 automatic (tensor cores when
                            available), 1 cuBLAS cgemm (FP32), 2 tcgen05 3xFP16 tensor cores  */
  int lanes;             /* 1 (default): batches one after another on the context's stream;
                            2: a sweep of several batches deals them round-robin to the context and a
                            helper context of its own (own stream and scratch, created on first
                            use, freed with the context), so one batch's latency-bound LU panels overlap
                            the other's assembly and tensor-core updates; larger values act as 2.
                            Per-kernel times in stats are then summed over the lanes. */
} bem_solve_options;

/* stats.kernel_s slots (filled when options.profile == 1), seconds summed over the call */
enum bem_kernel_slot {
  BEM_K_SINGULAR = 0, /* singular (Duffy) pair blocks */
  BEM_K_REGULAR = 1,  /* regular pair assembly */
  BEM_K_GATHER = 2,   /* singular scatter + column gather */
  BEM_K_RHS = 3,      /* matrix-free right-hand side */
  BEM_K_LU = 4,       /* LU factorisation */
  BEM_K_SOLVE = 5,    /* triangular solves and FP64 refinement */
  BEM_K_FIELD = 6,    /* field sources + field evaluation */
  BEM_K_SLOTS = 8
};

typedef struct bem_solve_stats {
  double assembly_s;      /* summed over the call, seconds (CUDA events) */
  double solve_s;
  double field_s;
  int max_refine_steps;   /* over all frequencies and excitations */
  double max_rel_residual;
  int batches;
  double kernel_s[8];     /* per kernel family, see enum bem_kernel_slot */
  long long regular_pairs;  /* face pairs integrated with the regular rule, per frequency */
  long long singular_pairs; /* vertex-sharing pairs integrated with Duffy rules, per frequency */
  long long singular_points; /* Duffy points summed over the singular pairs, per frequency */
  int lu_gemm_used;       /* trailing update that ran: 1 cuBLAS, 2 tensor cores (0 FP64 form) */
  long long kernel_launches; /* kernels of this library launched by the call (cuBLAS kernels not counted) */
  double regular_flop;    /* mixed form: FP32 flop (FMA = 2) the regular-pair kernel executed in the call,
                             counted from its source per quadrature pair and frequency: 35.67 + 26.83 / w,
                             w = frequencies sharing one launch's frequency-independent geometry */
  long long singular_cheb_freqs; /* mixed form: frequencies whose singular remainder was formed from the
                                    mesh's Chebyshev moments (calls of at least 12 frequencies, where the
                                    expansion converges); the rest point by point on the Duffy rules */
} bem_solve_stats;

void bem_default_options(bem_solve_options* opt);

/* The hot path: for every frequency, assemble the Burton-Miller system
 * 1/2 M - D + (i/k) H, factor it once, solve every excitation, and evaluate
 * the exterior field at the observation points.  Replaces the per-frequency
 * body of solve_request_impl (solver.jl:805-920): assemble_regular_galerkin_
 * operators, pressure_for_drives / solve_burton_miller_neumann and
 * field_for_points.
 * pressure_out: [n_freq][n_rhs][n_vertices] complex (may be NULL)
 * field_out:    [n_freq][n_rhs][n_points] complex (may be NULL)
 * stats may be NULL. */
int bem_solve_frequencies(bem_mesh* mesh, const double* freqs_hz, int n_freq, const bem_solve_options* opt,
                          double* pressure_out, double* field_out, bem_solve_stats* stats);

/* Several jobs solved together (no single counterpart in the reference, which
 * runs one job per GPU at a time: beat_engine_backend.py:314-334; each job is
 * one solve_request_impl sweep, solver.jl:805-920).  The jobs' meshes belong to
 * this context and carry their excitations (the same n_rhs for every job) and,
 * for a field, their observation points.  Their frequencies are taken in job
 * order and cut into batches (options.batch, or automatic for the largest
 * mesh); inside a batch every (job, frequency) is assembled on its own mesh into
 * a matrix of the order of the largest mesh in the call, padded with an identity
 * block, and all the matrices of the batch are factored, solved and refined in
 * one launch sequence, so many small jobs share the LU's launches instead of
 * running one after the other.  The padding changes no pivot, so each job's
 * results are those of bem_solve_frequencies on its own mesh up to the rounding
 * of its sums; the padding costs (n_max / n_job)^3 of the LU work, so callers
 * group jobs of similar size.  Outputs per job as in bem_solve_frequencies;
 * stats cover the whole call (pair counts summed over the jobs' meshes). */
typedef struct bem_job {
  bem_mesh* mesh;
  const double* freqs_hz;
  int n_freq;
  double* pressure_out; /* [n_freq][n_rhs][n_vertices] complex, or NULL */
  double* field_out;    /* [n_freq][n_rhs][n_points] complex, or NULL */
} bem_job;
int bem_solve_jobs(bem_context* ctx, const bem_job* jobs, int n_jobs, const bem_solve_options* opt,
                   bem_solve_stats* stats);

/* The batch bem_solve_frequencies uses for options.batch = 0 on a sweep of
 * n_freq frequencies (returned; 0 on a bad argument): at most B_max, the sweep
 * split into equal batches.  B_max (returned for n_freq <= 0): matrices within
 * ~16 GiB, at most 32, and at most as many as the LU's cluster panels keep
 * resident on this GPU at once (a larger batch runs every panel in two waves). */
int bem_auto_batch(bem_mesh* mesh, int precision, int n_freq);

/* Parity entry point: the dense P1 x P1 operator cD*D + cH*H + cM*M11 at
 * wavenumber k, written column-major [n_vertices][n_vertices] complex (row i
 * of column j at out[2*(j*n + i)]).  coeffs = {cD.re, cD.im, cH.re, cH.im,
 * cM.re, cM.im}.  The Burton-Miller left-hand side of
 * burton_miller_neumann_matrices (BeatEngineCpuSolve.jl:45-53) is
 * cD = -1, cH = i/k, cM = 1/2.  The mixed form assembles as a call of
 * bem_solve_frequencies with at least 12 frequencies does (the singular
 * remainder from the mesh's Chebyshev moments where their expansion converges;
 * the first such use forms them). */
int bem_assemble_lhs(bem_mesh* mesh, double k, int precision, const double* coeffs, double* out);

/* Parity entry point: out = (cS*S + cK*K' + cM10*M10) q for n_rhs face-data
 * columns q (column-major [n_rhs][n_faces] complex); out is column-major
 * [n_rhs][n_vertices] complex.  coeffs = {cS, cK, cM10} as (re, im) pairs.
 * The Burton-Miller right-hand side operator of BeatEngineCpuSolve.jl:50 is
 * cS = -1, cK = -i/k, cM10 = -i/(2k); this is the matrix-free right-hand side
 * of _cuda_burton_miller_rhs (BeatEngineCore.jl:1178-1184).  The mixed form
 * assembles as bem_assemble_lhs does. */
int bem_apply_rhs_operator(bem_mesh* mesh, double k, int precision, const double* coeffs, const double* q, int n_rhs,
                           double* out);

/* Exterior field of retained boundary traces on an uploaded mesh: the
 * reference's bem_field operation (evaluate_bem_field_request,
 * coupled_solver.jl:2438-2497, evaluate_galerkin_field_*), used after a
 * physical-system solve.  u(x) = sum over the mesh's quadrature sources of
 * [dG/dn_y p(y) - G q] w, with the mesh's regular rule and symmetry images.
 * pressure: [n_vertices] complex (P1); neumann: [n_faces] complex (DP0 normal
 * derivative); points: [n_points][3]; field_out: [n_points] complex.  Host
 * buffers; the mesh's excitation and observation points are not touched. */
int bem_evaluate_field(bem_mesh* mesh, double k, int precision, const double* pressure, const double* neumann,
                       const double* points, int n_points, double* field_out);

/* Exterior field for callers that cannot allocate device memory (no
 * counterpart in the reference).  Some callers cannot call cudaMalloc where they
 * need a field: a real-time audio callback, where an allocation may block for an
 * unbounded time, or a host framework that owns all device memory through its
 * own pool and forbids raw allocations.  This entry point allocates nothing:
 * every input and output is a device buffer the caller owns, and its scratch is
 * one fixed array inside the library (about 6.5 MB per GPU, held until the
 * process exits).  Inputs (device pointers): vertices [n_vertices][3] doubles,
 * faces [n_faces][3] int32, pressure [n_vertices] complex, neumann [n_faces]
 * complex (q = i rho omega v_n), points [n_points][3]; output field [n_points]
 * complex.  Same quadrature and precision forms as bem_solve_frequencies
 * (regular_order 1..4; BEM_PRECISION_FP64 or BEM_PRECISION_MIXED).  Limits:
 * n_faces <= 16384, else BEM_ERR_INVALID_ARGUMENT.  All calls share the scratch
 * array: calls whose work overlaps on the GPU race and must be serialised by the
 * caller.  The first call on a device resolves the scratch address with that
 * device current (kept for the process's life: not valid across a
 * cudaDeviceReset).  `stream` is
 * a cudaStream_t of the current device (NULL = legacy default stream); the call
 * synchronises that stream before it returns.  On an error return the contents
 * of field_out are undefined (an out-of-range vertex index or a zero-area
 * triangle is reported after the kernels ran).  err/err_cap: optional buffer for
 * a message on failure. */
int bem_evaluate_field_noalloc(const double* d_vertices, int n_vertices, const int* d_faces, int n_faces,
                               int regular_order, double k, const double* d_pressure, const double* d_neumann,
                               const double* d_points, int n_points, int precision, double* d_field_out,
                               void* stream, char* err, int err_cap);

/* Parity entry point: LU factorisation with partial pivoting of one dense
 * n x n matrix, as LAPACK getrf (the reference's `\` / lu!, BeatEngineCore.jl:1206,
 * BeatEngineCpuSolve.jl:63).  a: column-major complex [n][n] (host), overwritten
 * with L (unit lower, below the diagonal) and U; ipiv: 0-based row interchanges
 * (row i was swapped with ipiv[i]).  precision selects FP64 or the mixed form's
 * FP32 factorisation; lu_gemm as in bem_solve_options.  Returns BEM_ERR_SINGULAR
 * on a zero pivot. */
int bem_lu_factor_dense(bem_context* ctx, int n, double* a, int* ipiv, int precision, int lu_gemm);

/* Device bytes needed to solve `batch` frequencies of a mesh of this size
 * (scratch + matrices + factors), for admission control by a scheduler. */
long long bem_estimate_device_bytes(int n_vertices, int n_faces, int n_singular_pairs, int n_rhs, int n_points,
                                    int batch, int precision);

#ifdef __cplusplus
}
#endif

#endif /* GB300_BEM_H */
