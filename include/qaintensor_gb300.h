/*
 * qaintensor_gb300.h -- C ABI of the GB300 (sm_103a) engine for the
 * Qaintensor.jl contraction + truncated-SVD hot path.
 *
 * Conventions (all entry points):
 *   - Tensors are column-major (Julia order) with interleaved complex
 *     elements: QT_C64 = {float re, im}, QT_C128 = {double re, im}.
 *   - An MPS site is (chiL, 2, chiR); the first site of an open chain may have
 *     chiL = 1 and the last chiR = 1 (the memory of the reference's 2-leg end
 *     tensors (2, chi) / (chi, 2)).
 *   - Site numbers at this ABI are 0-based; the Julia/Python layers add 1.
 *   - A 4x4 gate G is complex128, column-major, interleaved; its matrix index
 *     is b_i + 2 b_{i+1} for wires (i, i+1): wire i is the fastest bit
 *     (src/decompose.jl:16-31, src/mpo.jl:41-57 -- the gate acts on the input legs).
 *   - Every call returns 0 (QT_OK) or a negative qt_status; no exception
 *     crosses the ABI.  qt_last_error() gives the message of the last failure
 *     on that handle.  The reference's own messages are returned verbatim
 *     where the reference has one.
 *   - A handle owns one CUDA stream on one device and is not thread-safe;
 *     calls are synchronous from the caller's view.
 */
#ifndef QAINTENSOR_GB300_H
#define QAINTENSOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QT_ABI_VERSION 1

typedef enum {
  QT_OK = 0,
  QT_EINVAL_ERR_NEG = -1,      /* "Error must be positive"            src/svd.jl:9, src/mps.jl:192 */
  QT_EDIM_MISMATCH = -2,       /* "Dimensions of contraction legs do not match"  src/svd.jl:16 */
  QT_ENOMEM = -3,              /* device allocation failed */
  QT_ECUDA = -4,               /* a CUDA runtime call failed */
  QT_ETIMEOUT = -5,            /* a bounded device-side wait gave up */
  QT_ENUMERIC = -6,            /* non-finite input or a factorisation broke down */
  QT_EFALLBACK_FAILED = -7,    /* the exact fallback itself failed */
  QT_EINVAL = -8,              /* bad argument (null pointer, bad dtype, bad mode) */
  QT_EPERIODIC = -9,           /* "Function doesn't support periodic boundary conditions for now" src/mps.jl:195 */
  QT_EBOUNDS = -10,            /* site index out of range (BoundsError in src/switch.jl) */
  QT_ENOTSUP = -11             /* size or mode not supported by this build */
} qt_status;

typedef enum { QT_C64 = 0, QT_C128 = 1 } qt_dtype;

typedef enum {
  QT_MODE_PLAIN = 0,     /* FP64 everywhere: FP64 GEMM + exact FP64 one-sided Jacobi SVD */
  QT_MODE_CHOSEN = 1,    /* complex64: FP32-level products (tcgen05 split-TF32x3),
                            randomized range finder sized by the rank predictor,
                            FP32-storage Jacobi split with FP64 norms and tail sums;
                            the exact FP64 split as fallback (cuSOLVER zgesvd from
                            min(m, n) = 512, the FP64 Jacobi below), also whenever
                            the rank decision at the caller's cutoff lies below the
                            FP32 resolution and no certificate holds
                            (qt_cert_counters) */
  QT_MODE_CUSOLVER = 2   /* cross-check: FP64 GEMM + cuSOLVER zgesvd (library) */
} qt_mode;

typedef struct {
  int device;              /* CUDA device ordinal */
  int mode;                /* qt_mode used when a call passes mode < 0 */
  double cutoff;           /* tail-norm cutoff (src/svd.jl:29-33), used when a call passes cutoff < 0 */
  int chi_max;             /* kept-rank cap (<= 0: none), used when a call passes chi_max < 0 */
  int oversample;          /* randomized SVD: extra probes beyond the predicted rank */
  int power_iters;         /* randomized SVD: subspace iterations */
  int renormalize;         /* rescale kept values to the full spectrum's norm */
  int use_rank_model;      /* size the sketch with the learned-rank MLP when trained */
  int max_sweeps;          /* Jacobi sweep limit */
  double jacobi_tol;       /* Jacobi orthogonality tolerance (relative) */
  double noise_floor;      /* chosen mode: resolution of the FP32-level split relative to
                              ||theta||_F (0: 4 sqrt(max(m, n)) 2^-24); a cutoff below it is
                              honoured through a certificate or the exact FP64 split */
  uint64_t seed;           /* sketch RNG seed */
  int tc_gemm;             /* chosen mode: 1 = tcgen05 split-TF32x3 products, 0 = FP32 SIMT */
  int jacobi_kernel;       /* Jacobi round: 0 = automatic (FP32 storage: one cooperative launch per
                              sweep, each round rebuilding its columns from the previous round's
                              unitaries, where one CTA per pair fits on the device, else 3; FP64:
                              one launch with cluster-resident pair rows where they fit shared
                              memory), 1 = three kernels (Gram partials, pair solver, rotation),
                              2 = the one-launch cluster round, 3 = FP32 two launches per round
                              (Gram + pair solver, then rotation) */
  double cap_sketch;       /* chosen mode: sketch width of a rank pinned at the chi_max cap, as a
                              multiple of chi_max (0: 1.125; the autotuner chooses it per chi_max) */
} qt_config;

typedef struct {
  int rank;                /* kept rank k */
  int rank_cutoff;         /* rank from the tail rule before chi_max */
  int predicted_rank;      /* learned-rank prediction (-1 when unused) */
  int sketch_size;         /* probes used (0: exact path) */
  int fallback;            /* 1 when the chosen mode fell back to the exact SVD */
  int sweeps;              /* Jacobi sweeps run */
  double discarded_weight; /* sum of discarded s_i^2 over the computed spectrum */
  double norm2;            /* sum of s_i^2 over the computed spectrum */
  double residual;         /* chosen mode: ||theta - Q Q^H theta||_F estimate */
} qt_update_stats;

typedef struct qt_handle qt_handle;
typedef struct qt_mps qt_mps;
typedef struct qt_batch qt_batch;

/* ---- handle ------------------------------------------------------------ */
int qt_config_default(qt_config* cfg);
int qt_create(qt_handle** out, const qt_config* cfg);
int qt_destroy(qt_handle* h);
const char* qt_last_error(const qt_handle* h);
int qt_abi_version(void);
/* Kernel launches issued by this handle since creation (a monotone counter). */
int64_t qt_launch_count(const qt_handle* h);
/* Algorithmic work issued by this handle since creation (no counterpart in
 * the reference; measurement hook): out[0] bytes of X and V the Jacobi rounds
 * must move (every pair's columns read once per round; rotated pairs written
 * back, their V rows read and written), out[1] Jacobi rounds, out[2] TF32
 * flops of the tensor-core GEMMs (24 M N K per complex product), out[3] their
 * launches, out[4] Jacobi pair rotations, out[5] inner sweeps of the 16x16
 * pair solvers, out[6] the part of out[0] read by the rounds' Gram products
 * (every column of X once per round), out[7] bytes of X and V columns
 * written by rotations (out holds 8 doubles). */
int qt_work_counters(const qt_handle* h, double* out);

/* Chosen-mode rank decisions issued by this handle since creation (no
 * counterpart in the reference), out[4]: [0] decided by the exact FP64
 * fallback (no certificate), [1] cutoff at or above the FP32 resolution,
 * [2] certified by the chi_max cap (the computed tail beyond chi_max exceeds
 * cutoff + resolution), [3] certified by the exact rank bound (exactly as
 * many values above the resolution as the gate's operator-Schmidt rank times
 * the inner bond or the Hilbert-space dimensions allow). */
int qt_cert_counters(const qt_handle* h, int64_t* out);

/* ---- measurement helpers ------------------------------------------------ */
/* CUDA events on the handle's stream: record into slot 0..7, elapsed a -> b. */
int qt_timer_record(qt_handle* h, int slot);
int qt_timer_elapsed(qt_handle* h, int slot_a, int slot_b, double* ms);
int qt_sync(qt_handle* h);
/* Write a 256 MiB device buffer on the handle's stream (evicts the 129 MB L2). */
int qt_l2_flush(qt_handle* h);
/* Per-launch device time of every kernel launch while enabled (events around
 * each launch on the handle's stream); collect aggregates by kernel name. */
int qt_profile_enable(qt_handle* h, int on);
int qt_profile_collect(qt_handle* h);
int qt_profile_get(int idx, char* name, int namelen, int64_t* launches, double* total_ms);
/* Pinned host memory for host-buffer (end-to-end) callers. */
void* qt_host_alloc(size_t bytes);
int qt_host_free(void* p);

/* ---- dense primitives on host buffers ----------------------------------- */

/* Pairwise contraction with ncon semantics: contract legs axesA[i] of A with
 * axesB[i] of B (0-based); the result's legs are A's free legs in order, then
 * B's.  Replaces the TensorOperations.ncon pairwise step called at
 * src/contract.jl:257,263 (and the products of src/svd.jl:35).  The operands
 * are uploaded and contracted by qt_tensor_contract (permutes folded into the
 * GEMM operand gathers on the device). */
int qt_contract_pair(qt_handle* h, int dtype,
                     int ndA, const int64_t* dimsA, const void* A,
                     int ndB, const int64_t* dimsB, const void* B,
                     int ncontract, const int* axesA, const int* axesB, void* C);

/* C = alpha op(A) op(B) + beta C, column-major host buffers, op in
 * {QT_OP_N = 0, QT_OP_C = 2 (conjugate transpose)}; alpha and beta are
 * {re, im}.  complex64: the tcgen05 split-TF32x3 kernel when cfg.tc_gemm is
 * set and the product fills a tile, FP32 SIMT otherwise; complex128: FP64
 * SIMT.  The GEMM of the pairwise contraction (TensorOperations' BLAS gemm
 * under src/contract.jl:257,263) exposed with explicit operands. */
int qt_gemm(qt_handle* h, int dtype, int opA, int opB, int64_t M, int64_t N, int64_t K,
            const double* alpha, const void* A, int64_t lda, const void* B, int64_t ldb,
            const double* beta, void* C, int64_t ldc);

/* Thin SVD of the m x n matrix M truncated by the tail rule of src/svd.jl:29-33
 * (cutoff = er) and chi_max: U (m x k), S (k), Vh (k x n).  Outputs are sized
 * for kcap = min(m, n) columns/rows; *k receives the kept rank.  Replaces the
 * svd() calls at src/svd.jl:26-27, src/switch.jl (svd of the swapped pair),
 * src/mps.jl:63,73, src/mpo.jl:53,62, src/decompose.jl:26,38.
 * mode PLAIN: FP64 one-sided Jacobi; CUSOLVER: zgesvd; CHOSEN with a
 * complex64 M: FP32-storage Jacobi when the cutoff is at or above its
 * resolution 4 sqrt(max(m,n)) 5.96e-8 ||M||_F or the chi_max cap decides the
 * rank, the exact FP64 split otherwise. */
int qt_truncated_svd(qt_handle* h, int dtype, int64_t m, int64_t n, const void* M,
                     double cutoff, int chi_max, int mode,
                     void* U, double* S, void* Vh, int* k, double* discarded);

/* Truncated SVD of a device matrix for callers that cannot allocate device
 * memory (no counterpart in the reference).  Embedding frameworks that own
 * every device byte through their own arena or budget, and code that must
 * not trigger a cudaMalloc, pass only their input and output buffers; the
 * scratch lives in a fixed file-scope device array (about 2.6 MB, resident
 * on every device that loads the library until exit), so this call makes no
 * cudaMalloc, cudaFree or allocating library call.
 *   dM: m x n complex128, column-major (ld m), not modified;
 *   dU: m x min(m,n), dS: min(m,n) doubles, dVh: min(m,n) x n (ld k on return),
 *   *k: kept rank (tail rule of src/svd.jl:29-33 with `cutoff`, then chi_max).
 * m, n <= 256, otherwise QT_ENOTSUP.  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress) -- make it before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU race
 * and must be serialised by the caller.  Runs on `stream` and synchronises it. */
int qt_truncated_svd_noalloc(int64_t m, int64_t n, const void* dM, double cutoff, int chi_max, void* dU, double* dS,
                             void* dVh, int* k, void* stream);

/* contract_svd(T1, T2, (i1, i2); er) of src/svd.jl:7-38 (i1, i2 are 1-based,
 * as in Julia).  out holds the free legs of T1 then of T2, column-major. */
int qt_contract_svd(qt_handle* h, int dtype,
                    int nd1, const int64_t* dims1, const void* T1,
                    int nd2, const int64_t* dims2, const void* T2,
                    int i1, int i2, double er, void* out);

/* ---- device-resident tensors (the operands of ncon's pairwise steps) ----
 * A qt_tensor is a column-major complex64/complex128 tensor in HBM.  A
 * network is contracted by uploading its tensors once and chaining
 * qt_tensor_contract / qt_tensor_trace steps in ncon's order (the schedule
 * of TensorOperations.ncon under src/contract.jl:257,263), downloading only
 * the result: no intermediate leaves the device and no permute runs on the
 * host. */
typedef struct qt_tensor qt_tensor;
/* host may be NULL (a zero tensor); the library copies the data. */
int qt_tensor_create(qt_handle* h, int dtype, int nd, const int64_t* dims, const void* host, qt_tensor** out);
int qt_tensor_free(qt_handle* h, qt_tensor* t);
int qt_tensor_ndims(const qt_tensor* t);
int qt_tensor_dims(const qt_tensor* t, int64_t* dims);
int qt_tensor_download(qt_handle* h, const qt_tensor* t, void* host);
/* *out = A contracted with B over legs axesA[i] <-> axesB[i] (0-based); its
 * legs are A's free legs then B's, reordered by out_perm when not NULL
 * (out leg i = natural leg out_perm[i]).  ncontract = 0 is the outer product.
 * complex64 with cfg.tc_gemm runs the tcgen05 split-TF32x3 GEMM, its operand
 * planes gathered straight from A and B through offset tables; otherwise a
 * tiled gather writes the operand matrices for the SIMT GEMM. */
int qt_tensor_contract(qt_handle* h, const qt_tensor* A, const qt_tensor* B, int ncontract, const int* axesA,
                       const int* axesB, const int* out_perm, qt_tensor** out);
/* *out = the legs of A in the order perm (out leg i = leg perm[i] of A):
 * permutedims of src/contract.jl:243-245 and ncon's final leg order. */
int qt_tensor_permute(qt_handle* h, const qt_tensor* A, const int* perm, qt_tensor** out);
/* *out = A traced over legs ax1 and ax2 (a label repeated on one tensor). */
int qt_tensor_trace(qt_handle* h, const qt_tensor* A, int ax1, int ax2, qt_tensor** out);

/* ---- device-resident MPS ------------------------------------------------ */

/* dims: 3 per site (chiL, 2, chiR).  host_sites may be NULL for |0...0>
 * (then every dim must be (1,2,1)).  The library copies the data. */
int qt_mps_create(qt_handle* h, int nsites, const int64_t* dims,
                  const void* const* host_sites, int dtype, qt_mps** out);
int qt_mps_free(qt_handle* h, qt_mps* mps);
/* Device-to-device copy of an MPS (stream-ordered; no host round trip). */
int qt_mps_clone(qt_handle* h, const qt_mps* src, qt_mps** out);
int qt_mps_nsites(const qt_mps* mps);
int qt_mps_site_dims(const qt_mps* mps, int site, int64_t* dims3);
int qt_mps_download(qt_handle* h, const qt_mps* mps, int site, void* host);
int qt_mps_upload_site(qt_handle* h, qt_mps* mps, int site, const int64_t* dims3, const void* host);

/* The two-qubit gate + truncated-SVD update on sites (site, site+1):
 * theta = A.B, theta' = G on the input legs, SVD, tail rule + chi_max,
 * A' = U[:, :k], B' = diag(S_k) V'[:k, :]  (src/switch.jl split convention).
 * cutoff < 0 / chi_max < 0 / mode < 0 take the handle's configuration. */
int qt_apply_2q(qt_handle* h, qt_mps* mps, int site, const double* G,
                double cutoff, int chi_max, int mode, qt_update_stats* stats);

/* switch!(mps, i) of src/switch.jl:18-56: swap the
 * physical legs of sites (site, site+1) with an untruncated SVD split. */
int qt_switch(qt_handle* h, qt_mps* mps, int site);

/* <psi|Z_site|psi>/<psi|psi>, <psi|Z_site Z_site+1|psi>/<psi|psi> and <psi|psi>
 * (no reference counterpart: its observables are closure networks contracted
 * with ncon, examples/expectation_value_optimization_example.ipynb). */
int qt_expect_z(qt_handle* h, const qt_mps* mps, int site, double* out);
int qt_expect_zz(qt_handle* h, const qt_mps* mps, int site, double* out);
int qt_mps_norm2(qt_handle* h, const qt_mps* mps, double* out);

/* MPO on the device MPS.  W[i] is MPO site i, (bl, 2, 2, br) complex128
 * column-major (out leg 2, in leg 3, as src/mpo.jl:66), dims 4 per site; end
 * sites have bl = 1 / br = 1.  qt_mps_apply_mpo contracts the MPO into the
 * MPS (bond chi*b), replacing the lazy wiring of apply_MPO (src/mpo.jl:184-216)
 * followed by contract.  qt_mps_compress left-canonicalises with QRs,
 * optionally normalises, then truncates right to left by the tail rule of
 * src/svd.jl:29-33 and chi_max (ranks/discarded: nsites-1 entries, may be
 * NULL); mode picks the split as in qt_truncated_svd (complex128 sites:
 * QT_MODE_CUSOLVER uses cuSOLVER, any other mode the FP64 Jacobi).
 * qt_mps_expect_mpo returns <psi|H|psi>/<psi|psi>. */
int qt_mps_apply_mpo(qt_handle* h, qt_mps* mps, const double* const* W, const int64_t* dims);
int qt_mps_compress(qt_handle* h, qt_mps* mps, double cutoff, int chi_max, int mode, int normalize, int* ranks,
                    double* discarded);
int qt_mps_expect_mpo(qt_handle* h, const qt_mps* mps, const double* const* W, const int64_t* dims, double* out);

/* Context for the rank model: the spectrum last kept at a bond (the engine
 * records it after every update; callers that built the MPS elsewhere may
 * supply it) and the circuit position (layer of depth) of the next update. */
int qt_mps_set_bond_spectrum(qt_mps* mps, int bond, const double* s, int n);
int qt_mps_set_circuit_position(qt_mps* mps, int layer, int depth);

/* ---- learned-rank model (16-64-64-1 ReLU MLP; no reference counterpart:
 * the reference's only rank rule is src/svd.jl:29-33) -------------------- */
int qt_rank_model_nparams(void);
int qt_rank_model_set_logging(qt_handle* h, int on);   /* log (features, k/k_max) of plain updates */
int64_t qt_rank_model_log_size(const qt_handle* h);
int qt_rank_model_get_log(const qt_handle* h, float* X /* n x 16 row-major */, float* Y /* n */);
int qt_rank_model_clear_log(qt_handle* h);
int qt_rank_model_set_params(qt_handle* h, const float* params, int nparams, int enable);
int qt_rank_model_get_params(const qt_handle* h, float* params, int nparams);
int qt_rank_model_enable(qt_handle* h, int on);
int qt_rank_model_set_margin(qt_handle* h, double margin);
/* Adam on minibatches with the GPU forward/backward kernels; init may be NULL. */
int qt_rank_model_train(qt_handle* h, int64_t n, const float* X, const float* Y, const float* init, int epochs,
                        int batch, double lr, uint64_t seed, double* final_loss);
int qt_mlp_forward(qt_handle* h, int64_t n, const float* X, float* out);
int qt_mlp_loss_grad(qt_handle* h, int64_t n, const float* X, const float* Y, const float* params, float* grad,
                     double* loss);
/* The 16 features of the update of bond (site, site+1) with gate G. */
int qt_rank_features_of(const qt_mps* mps, int site, const double* G, double cutoff, int chi_max, float* f);

/* ---- batched circuits (no reference counterpart: the reference runs one
 * network at a time) --------------------------------------------------------
 * Many independent MPS (complex64, |0...0> at creation) with per-circuit qubit
 * counts and bond caps chi_max <= 128.  A program is a list of layers of
 * (circuit, site, gate) tasks; tasks of one layer must touch disjoint sites.
 * Each layer runs as one persistent kernel whose CTAs take tasks from a
 * device counter (mixed precision: FP32 products and Jacobi, FP64 norms and
 * tail rule at the caller's cutoff; a rank decision below the FP32 resolution
 * that neither the cap nor the exact rank bound certifies is redone as an
 * FP64 split by the same CTA); the whole program is captured in one CUDA
 * graph when use_graph is set. */
int qt_batch_create(qt_handle* h, int ncirc, const int* nqubits, const int* chi_max, qt_batch** out);
int qt_batch_free(qt_handle* h, qt_batch* b);
int qt_batch_run(qt_handle* h, qt_batch* b, int nlayers, const int* layer_start, const int* circ, const int* site,
                 const double* gates /* 32 doubles per task */, double cutoff, int use_graph);
int qt_batch_replay(qt_handle* h, qt_batch* b);
int qt_batch_reset(qt_handle* h, qt_batch* b);
int qt_batch_task_stats(qt_handle* h, const qt_batch* b, int* rank, int* sweeps, float* discarded);
/* Launch shape of the persistent layer kernel for circuits whose bond cap
 * lies in the bucket bucket_cap (16: caps <= 16, 32, 64, 128): threads per CTA
 * (128, 256, 512 or 1024) and CTAs per SM (1 to 4).  A program runs one launch per
 * layer and bucket; set the shapes before qt_batch_run (the graph captures
 * them).  Defaults 256 threads, 1 CTA per SM; the autotuner chooses them. */
int qt_batch_set_launch(qt_handle* h, qt_batch* b, int bucket_cap, int threads, int ctas_per_sm);
int qt_batch_get_launch(const qt_batch* b, int bucket_cap, int* threads, int* ctas_per_sm);
/* Rank decisions of the last program's tasks by certificate, as qt_cert_counters. */
int qt_batch_cert_counts(qt_handle* h, const qt_batch* b, int64_t* out /* 4 */);
int qt_batch_bond_dims(qt_handle* h, const qt_batch* b, int circ, int* dims /* nqubits + 1 */);
int qt_batch_download_site(qt_handle* h, const qt_batch* b, int circ, int site, void* host);
int qt_batch_expect_z(qt_handle* h, qt_batch* b, int site, double* out /* one per circuit */);

#ifdef __cplusplus
}
#endif
#endif /* QAINTENSOR_GB300_H */
