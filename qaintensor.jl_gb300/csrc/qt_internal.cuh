// Internal definitions shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/qaintensor_gb300.h"

// ---------------------------------------------------------------------------
// handle and MPS objects
// ---------------------------------------------------------------------------

struct qt_rank_model;  // learned-rank MLP state (k_mlp.cu)

// Per-launch device timing (CUDA events on the handle's stream), grouped by
// kernel name; enabled with qt_profile_enable.
struct qt_profile_rec {
  const char* name;
  cudaEvent_t start, stop;
};

// Internal return code (never crosses the ABI): a chosen-mode rank decision
// that the FP32-level split cannot certify; the caller takes the exact FP64
// split instead.
constexpr int QT_UNCERTIFIED = 1;
// How a chosen-mode rank decision was certified (qt_cert_counters slots).
enum { QT_CERT_NONE = 0, QT_CERT_RESOLVED = 1, QT_CERT_CAP = 2, QT_CERT_STRUCT = 3, QT_CERT_SLOTS = 4 };

struct qt_handle {
  qt_config cfg;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;   // stream-ordered pool owned by the handle
  std::string err;
  int64_t launches = 0;           // kernel launches issued through this handle
  int* d_flags = nullptr;         // device status words (see QT_FLAG_*)
  int* h_flags = nullptr;         // pinned host mirror
  int* d_status = nullptr;        // sticky device status of the tensor-core GEMM's bounded waits
  qt_rank_model* rank_model = nullptr;
  uint64_t sketch_counter = 0;    // advances the sketch RNG stream per update
  // algorithmic work issued (cumulative): Jacobi rounds and the bytes of X and
  // V they must move (every pair's columns read once per round, rotated pairs
  // written back and their V rows read and written); tensor-core GEMM TF32
  // flops (24 M N K per complex product) and launches
  double work_jacobi_bytes = 0, work_jacobi_rounds = 0, work_tc_flops = 0, work_tc_launches = 0;
  double work_jacobi_pairs = 0, work_jacobi_inner = 0;  // rotated pairs, pair-solver inner sweeps
  double work_jacobi_gram_bytes = 0, work_jacobi_rot_bytes = 0;  // X read by the Gram products; X, V rewritten
  int64_t cert_count[QT_CERT_SLOTS] = {};  // chosen-mode rank decisions by QT_CERT_* (NONE: fell back)
  bool prof = false;
  std::vector<qt_profile_rec> prof_recs;
  std::vector<cudaEvent_t> event_pool;
  size_t event_next = 0;
  cudaEvent_t timers[8] = {};
};

// profiling hooks used by QT_LAUNCH
void qt_prof_before(qt_handle* h, const char* name);
void qt_prof_after(qt_handle* h);

enum {
  QT_FLAG_ROTATED = 0,   // Jacobi: pairs rotated in the current sweep
  QT_FLAG_NONFINITE = 1, // a kernel met a non-finite value
  QT_FLAG_CHOL = 2,      // a Cholesky factorisation lost positive definiteness
  QT_FLAG_OFFMAX = 3,    // Jacobi: largest relative off-diagonal above tol this sweep (float bits)
  QT_FLAG_INNER = 4,     // Jacobi: inner sweeps of the pair solvers this sweep
  QT_FLAG_OFFBIG = 5,    // Jacobi: OFFMAX over pairs of columns above 1e-3 ||X||_F (float bits)
  QT_FLAG_ABORT = 6,     // Jacobi sweep kernel: a bounded round wait gave up
  QT_FLAG_OFFKEPT = 7,   // Jacobi sweep kernel: OFFMAX over pairs with a column above the keep threshold
  QT_FLAG_STALL = 8,     // never set: the bounded-wait test hook of the sweep kernel waits on it
  QT_FLAG_COUNT = 9
};

struct qt_mps {
  int nsites = 0;
  int dtype = QT_C128;
  std::vector<int64_t> chil, chir;
  std::vector<void*> site;        // device buffers (chiL*2*chiR elements)
  std::vector<size_t> cap;        // bytes allocated per site
  std::vector<std::vector<double>> spectrum;  // last kept spectrum per bond (nsites-1)
  std::vector<int> bond_updates;  // updates applied per bond
  int circuit_layer = 0;          // caller-set circuit position (rank-model feature)
  int circuit_depth = 0;
};

// ---------------------------------------------------------------------------
// error handling
// ---------------------------------------------------------------------------

int qt_fail(qt_handle* h, int code, const std::string& msg);
// Reads and clears the sticky device status (after the work queued so far):
// QT_ETIMEOUT when a tensor-core GEMM's pipeline wait (status 1) or a grid
// barrier of the one-launch orthonormalisation (status 2) gave up.
int qt_check_status(qt_handle* h);

#define QT_CHECK_CUDA(h, call)                                                    \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return qt_fail((h), (e_ == cudaErrorMemoryAllocation) ? QT_ENOMEM : QT_ECUDA, \
                     std::string(#call) + ": " + cudaGetErrorString(e_));         \
  } while (0)

#define QT_TRY(expr)              \
  do {                            \
    int rc_ = (expr);             \
    if (rc_ != QT_OK) return rc_; \
  } while (0)

// Launch a kernel on the handle's stream, count it and check the launch.
#define QT_LAUNCH(h, kernel, grid, block, smem, ...)                                    \
  do {                                                                                  \
    if ((h)->prof) qt_prof_before((h), #kernel);                                         \
    kernel<<<(grid), (block), (smem), (h)->stream>>>(__VA_ARGS__);                      \
    if ((h)->prof) qt_prof_after((h));                                                   \
    (h)->launches++;                                                                    \
    cudaError_t e_ = cudaGetLastError();                                                \
    if (e_ != cudaSuccess)                                                              \
      return qt_fail((h), QT_ECUDA, std::string("launch " #kernel ": ") + cudaGetErrorString(e_)); \
  } while (0)

// ---------------------------------------------------------------------------
// device memory from the handle's pool
// ---------------------------------------------------------------------------

int qt_dmalloc(qt_handle* h, void** p, size_t bytes);
void qt_dfree(qt_handle* h, void* p);

// RAII list of pool allocations released (stream-ordered) at scope exit.
struct qt_scratch {
  qt_handle* h;
  std::vector<void*> ptrs;
  explicit qt_scratch(qt_handle* hh) : h(hh) {}
  ~qt_scratch() {
    for (void* p : ptrs) qt_dfree(h, p);
  }
  template <typename T>
  int get(T** p, size_t count) {
    void* v = nullptr;
    int rc = qt_dmalloc(h, &v, count * sizeof(T) + 16);
    if (rc != QT_OK) return rc;
    ptrs.push_back(v);
    *p = static_cast<T*>(v);
    return QT_OK;
  }
};

// ---------------------------------------------------------------------------
// complex helpers (interleaved {re, im})
// ---------------------------------------------------------------------------

template <typename T> struct cplx_of;
template <> struct cplx_of<float> { typedef float2 type; };
template <> struct cplx_of<double> { typedef double2 type; };
template <typename C> struct real_of;
template <> struct real_of<float2> { typedef float type; };
template <> struct real_of<double2> { typedef double type; };

__host__ __device__ inline double2 mk(double r, double i) { return make_double2(r, i); }
__host__ __device__ inline float2 mk(float r, float i) { return make_float2(r, i); }

template <typename C> __host__ __device__ inline C czero() { C z; z.x = 0; z.y = 0; return z; }
template <typename C, typename D> __host__ __device__ inline C ccast(D a) { C z; z.x = a.x; z.y = a.y; return z; }
template <typename C> __host__ __device__ inline C cconj(C a) { a.y = -a.y; return a; }
template <typename C> __host__ __device__ inline C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __host__ __device__ inline C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __host__ __device__ inline C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C, typename R> __host__ __device__ inline C cscale(C a, R s) { a.x *= s; a.y *= s; return a; }
// acc += a * b
template <typename C> __host__ __device__ inline void cfma(C& acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename C> __host__ __device__ inline void cfma_conj(C& acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}
template <typename C> __host__ __device__ inline typename real_of<C>::type cabs2(C a) { return a.x * a.x + a.y * a.y; }

// ---------------------------------------------------------------------------
// launchers implemented in the kernel translation units
// ---------------------------------------------------------------------------

enum qt_op { QT_OP_N = 0, QT_OP_T = 1, QT_OP_C = 2 };

// k_gemm.cu ------------------------------------------------------------------
// theta'(2chiL x 2chiR) = G (x) (A_mat . B_mat), gate folded in the epilogue.
// A (chiL,2,chiM), B (chiM,2,chiR) of element type TI; output of type TO.
// prec: 0 = FP64 accumulation, 1 = FP32 accumulation.
int qt_theta_gate(qt_handle* h, int dtype_in, const void* A, const void* B, int64_t chil,
                  int64_t chim, int64_t chir, const double* G, int prec, void* theta_out);
// C(M x N) = alpha op(A) op(B) + beta C, column-major; T = float2 or double2.
template <typename C>
int qt_cgemm(qt_handle* h, int opA, int opB, int64_t M, int64_t N, int64_t K, C alpha,
             const C* A, int64_t lda, const C* B, int64_t ldb, C beta, C* Cm, int64_t ldc);
// k_tcgemm.cu: complex64 GEMM on the tcgen05 tensor cores (split-TF32x3), op in {N, C}
int qt_cgemm_tc(qt_handle* h, int opA, int opB, int64_t M, int64_t N, int64_t K, float2 alpha, const float2* A,
                int64_t lda, const float2* B, int64_t ldb, float2 beta, float2* C, int64_t ldc);
// C (M x N, ld M) = A_view B_view on the tensor cores with the operands read
// through device offset tables: A_view(m, k) = A[a_row[m] + a_col[k]],
// B_view(k, n) = B[b_row[k] + b_col[n]] (the ncon permutes folded into the
// operand gathers); *_rows_fast: the source's unit-stride leg is a row leg.
int qt_cgemm_tc_mapped(qt_handle* h, int64_t M, int64_t N, int64_t K, const float2* A, const int64_t* a_row,
                       const int64_t* a_col, int a_rows_fast, const float2* B, const int64_t* b_row,
                       const int64_t* b_col, int b_rows_fast, float2* C);
// complex64 GEMM dispatch: tensor cores when cfg.tc_gemm is set and the
// problem fills a tile, the SIMT kernel otherwise.
int qt_cgemm_c64(qt_handle* h, int opA, int opB, int64_t M, int64_t N, int64_t K, float2 alpha, const float2* A,
                 int64_t lda, const float2* B, int64_t ldb, float2 beta, float2* C, int64_t ldc);
inline int qt_gemm_any(qt_handle* h, int opA, int opB, int64_t M, int64_t N, int64_t K, float2 alpha,
                       const float2* A, int64_t lda, const float2* B, int64_t ldb, float2 beta, float2* C,
                       int64_t ldc) {
  return qt_cgemm_c64(h, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}
inline int qt_gemm_any(qt_handle* h, int opA, int opB, int64_t M, int64_t N, int64_t K, double2 alpha,
                       const double2* A, int64_t lda, const double2* B, int64_t ldb, double2 beta, double2* C,
                       int64_t ldc) {
  return qt_cgemm<double2>(h, opA, opB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}
// theta (2chiL x 2chiR, complex64) <- G applied on the physical legs, in place
int qt_apply_gate_inplace(qt_handle* h, float2* theta, int64_t chil, int64_t chir, const double* G);
// element conversions / copies
int qt_convert(qt_handle* h, const void* src, int src_dtype, void* dst, int dst_dtype, int64_t n);
template <typename C>
int qt_adjoint_copy(qt_handle* h, const C* src, int64_t m, int64_t n, int64_t lds, C* dst, int64_t ldd);
template <typename C>
int qt_set_identity(qt_handle* h, C* V, int64_t n, int64_t ld);
// sum |x|^2 over n complex values into *out (device double), FP64 accumulation
template <typename C>
int qt_norm2(qt_handle* h, const C* x, int64_t n, double* d_out);

// k_jacobi.cu ----------------------------------------------------------------
// One-sided block Jacobi SVD of X (mm x nn, mm >= nn) in place: X <- X V with
// orthogonal columns, V (nn x nn) accumulated (V = nullptr: not accumulated).
// TS = storage type.
template <typename TS>
int qt_jacobi_svd(qt_handle* h, TS* X, int64_t mm, int64_t nn, int64_t ldx, TS* V, int64_t ldv,
                  double tol, int max_sweeps, int* sweeps_out, double nu_rel = -1.0, int keep_count = 0);
// The same with a caller-supplied partial-Gram workspace of qt_jacobi_layout() double2 entries.
// nu_rel > 0: columns with norm <= nu_rel ||X||_F are frozen (not rotated,
// not tested); <= 0: the default for the storage precision.
// keep_count > 0: the caller keeps only the keep_count largest columns (a
// chi_max cap); the FP32 sweep kernel then ends the iteration once the weight
// outside the keep_count largest columns (an upper bound of the truncation
// error) has settled -- it moved by at most 1e-3 of itself over a sweep and
// 1e-2 over the one before -- or once a sweep rotated no pair holding a
// column within a factor 4 of the cut or above it.  Only columns far below
// the cut, which the caller discards, are left unconverged.
template <typename TS>
int qt_jacobi_svd_ws(qt_handle* h, TS* X, int64_t mm, int64_t nn, int64_t ldx, TS* V, int64_t ldv, double tol,
                     int max_sweeps, int* sweeps_out, double2* parts, double nu_rel = -1.0, int keep_count = 0);
int qt_jacobi_layout(int64_t mm, int64_t nn, int* nb_out, int* chunks_out);

// k_trunc.cu -----------------------------------------------------------------
// Column norms of X (mm x nn) in FP64; sort descending -> d_sigma (sorted), d_perm.
template <typename TS>
int qt_sorted_column_norms(qt_handle* h, const TS* X, int64_t mm, int64_t nn, int64_t ldx,
                           double* d_sigma, int* d_perm);
// tail rule on the device-sorted spectrum: returns k (clamped >= 1) and stats
int qt_tail_rule_host(const std::vector<double>& s, double cutoff, int* k_cutoff);
// A' columns j < k: Ucols[:, perm[j]] * uscale_j ; B' rows: see k_trunc.cu
template <typename TS, typename TO>
int qt_absorb(qt_handle* h, int transposed, const TS* X, int64_t ldx, const TS* Vx, int64_t ldv,
              const double* d_sigma, const int* d_perm, int64_t m, int64_t n, int k, double sscale,
              TO* Aout, TO* Bout);

// k_rsvd.cu ------------------------------------------------------------------
template <typename C>
int qt_gaussian(qt_handle* h, C* out, int64_t rows, int64_t cols, int64_t ld, uint64_t seed);
// Block classical Gram-Schmidt with re-orthogonalisation, intra-block shifted
// CholeskyQR2 (FP64 Gram / Cholesky): Y (m x l, ld m) -> orthonormal columns.
// What an orthonormalised FP32 basis is for (the one-launch kernel's passes
// per 32-column block): an orthonormal basis kept as such (project, shifted
// CholeskyQR, project, two CholeskyQR passes), the final basis of a sketch
// (one CholeskyQR pass fewer) and a range carried to the next product of a
// power iteration (one projection, two CholeskyQR passes).
enum { QT_ORTH_USE_BASIS = 0, QT_ORTH_USE_SKETCH = 1, QT_ORTH_USE_RANGE = 2 };
template <typename C>
int qt_orthonormalize(qt_handle* h, C* Y, int64_t m, int64_t l, int use = QT_ORTH_USE_BASIS);

// k_ncon.cu ------------------------------------------------------------------
// device buffer of a qt_tensor (column-major, its dtype's element)
void* qt_tensor_data(const qt_tensor* t);
// the truncated split of a device matrix (qt_engine.cu): M ~ A (m x k) B (k x n)
int qt_split_device(qt_handle* h, int dtype, const void* M, int64_t m, int64_t n, double cutoff, int chi_max, int mode,
                    void** A, void** B, int* k, double* discarded, int64_t struct_rank);

// k_obs.cu -------------------------------------------------------------------
int qt_mps_expect(qt_handle* h, const qt_mps* mps, int site, int nops, double* out);
