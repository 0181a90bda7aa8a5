// One-sided block Jacobi SVD (Hestenes).
//
// Replaces the dense LAPACK ?gesdd called by LinearAlgebra.svd at
// src/svd.jl:26-27 and in switch! (src/switch.jl, file line 77): X (mm x nn,
// mm >= nn) is driven to orthogonal columns, X <- X V, so X = U diag(s) and
// the input equals U diag(s) V^H.
//
// Columns are split into blocks of JW = 8.  One sweep is a round-robin
// tournament over the blocks; a round processes every block pair (16
// columns) at once in two kernels:
//   gram   -- grid (pair, row chunk): the 16x16 Gram of the pair over one row
//             chunk, written as a partial (no atomics: the reduction below
//             runs in a fixed order, so results are reproducible);
//   rotate -- grid (pair, row chunk): sums the partials, tests the pair
//             against `tol` (relative), diagonalises the Gram with a cyclic
//             two-sided Jacobi in FP64 whose 2x2 rotations use the
//             relative-accuracy formula (tan from zeta = (beta-alpha)/(2|gamma|),
//             the smaller root), and applies the 16x16 unitary to its row
//             chunk of X and of V.  Every chunk solves the same 16x16 problem
//             with the same arithmetic, so all chunks apply the same unitary.
// A sweep in which no pair rotates ends the iteration.
//
// Storage / Gram accumulation: double2 / FP64 for the exact path; float2 /
// FP32 for the FP32-storage path (whose achievable orthogonality is FP32
// anyway); the 16x16 eigen-solve and the rotation angles are FP64 in both.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "qt_internal.cuh"

namespace {

constexpr int JW = 8;        // columns per block
constexpr int JC = 2 * JW;   // columns per block pair
constexpr int JR = 64;       // rows per shared-memory slab
constexpr int NT = 256;      // threads per CTA
constexpr int MAX_INNER = 12;
constexpr int NGRAM = JC * JC;

__device__ inline void tournament(int r, int q, int n, int& a, int& b) {
  // circle method over n (even) players, round r, table q
  if (q == 0) { a = r % (n - 1); b = n - 1; }
  else { a = (r + q) % (n - 1); b = (r - q + (n - 1)) % (n - 1); }
  if (a > b) { const int t = a; a = b; b = t; }
}

__device__ inline void pair_columns(int round, int pair, int nb, int nn, int* col) {
  int bi, bj;
  tournament(round, pair, nb, bi, bj);
  if (threadIdx.x < JC) {
    const int c = threadIdx.x;
    const int gc = (c < JW) ? bi * JW + c : bj * JW + (c - JW);
    col[c] = (gc < nn) ? gc : -1;
  }
}

template <typename T> struct acc_of;
template <> struct acc_of<double> { typedef double2 type; };
template <> struct acc_of<float> { typedef float2 type; };

// Partial Gram of one pair over rows [r_begin, r_end) -> part (16x16 double2).
template <typename TS, typename TG>
__global__ void __launch_bounds__(NT)
gram_kernel(const TS* __restrict__ X, int64_t ldx, int mm, int nn, int nb, int round, int rows_per_chunk,
            double2* __restrict__ parts) {
  typedef typename acc_of<TG>::type CG;
  __shared__ TS Xs[JR][JC + 1];
  __shared__ int col[JC];
  const int pair = blockIdx.x, chunk = blockIdx.y;
  pair_columns(round, pair, nb, nn, col);
  __syncthreads();
  const int t = threadIdx.x;
  int gi = -1, gj = -1;
  if (t < JC * (JC + 1) / 2) {
    int r = 0, rem = t;
    while (rem >= JC - r) { rem -= JC - r; r++; }
    gi = r; gj = r + rem;
  }
  CG acc = czero<CG>();
  const int r_begin = chunk * rows_per_chunk, r_end = min(mm, r_begin + rows_per_chunk);
  for (int r0 = r_begin; r0 < r_end; r0 += JR) {
    for (int idx = t; idx < JR * JC; idx += NT) {
      const int rr = idx % JR, c = idx / JR, gr = r0 + rr;
      TS v = czero<TS>();
      if (gr < r_end && col[c] >= 0) v = X[gr + ldx * col[c]];
      Xs[rr][c] = v;
    }
    __syncthreads();
    if (gi >= 0) {
      const int lim = min(JR, r_end - r0);
      for (int rr = 0; rr < lim; rr++) cfma_conj(acc, ccast<CG>(Xs[rr][gi]), ccast<CG>(Xs[rr][gj]));
    }
    __syncthreads();
  }
  double2* out = parts + ((size_t)pair * gridDim.y + chunk) * NGRAM;
  if (gi >= 0) {
    out[gi * JC + gj] = ccast<double2>(acc);
    out[gj * JC + gi] = cconj(ccast<double2>(acc));
  }
}

template <typename TS>
__device__ void apply_rows(TS* __restrict__ M, int64_t ld, int r_begin, int r_end, const int* col,
                           const typename cplx_of<typename real_of<TS>::type>::type (*Wt)[JC + 1],
                           TS (*Xs)[JC + 1]) {
  typedef typename real_of<TS>::type RS;
  typedef typename cplx_of<RS>::type CS;
  const int t = threadIdx.x;
  for (int r0 = r_begin; r0 < r_end; r0 += JR) {
    for (int idx = t; idx < JR * JC; idx += NT) {
      const int rr = idx % JR, c = idx / JR, gr = r0 + rr;
      TS v = czero<TS>();
      if (gr < r_end && col[c] >= 0) v = M[gr + ld * col[c]];
      Xs[rr][c] = v;
    }
    __syncthreads();
    for (int idx = t; idx < JR * JC; idx += NT) {
      const int c = idx % JC, rr = idx / JC, gr = r0 + rr;
      if (gr >= r_end || col[c] < 0) continue;
      CS acc = czero<CS>();
#pragma unroll
      for (int k = 0; k < JC; k++) cfma(acc, ccast<CS>(Xs[rr][k]), Wt[k][c]);
      M[gr + ld * col[c]] = ccast<TS>(acc);
    }
    __syncthreads();
  }
}

template <typename TS>
__global__ void __launch_bounds__(NT)
rotate_kernel(TS* __restrict__ X, int64_t ldx, int mm, TS* __restrict__ V, int64_t ldv, int nn, int nb, int round,
              int nparts, int x_rows_per_chunk, int v_rows_per_chunk, const double2* __restrict__ parts, double tol,
              double nu_rel2, const double* __restrict__ xnorm2, int* __restrict__ flags) {
  typedef typename real_of<TS>::type RS;
  typedef typename cplx_of<RS>::type CS;
  __shared__ double2 G[JC][JC + 1];
  __shared__ double2 W[JC][JC + 1];
  __shared__ CS Wt[JC][JC + 1];
  __shared__ TS Xs[JR][JC + 1];
  __shared__ int col[JC];
  __shared__ int rp[JC / 2], rq[JC / 2], ron[JC / 2];
  __shared__ double rc[JC / 2], rs[JC / 2], rt[JC / 2], ra[JC / 2], rb[JC / 2];
  __shared__ double2 re[JC / 2];
  __shared__ int any_rot, inner_rot, bad;

  const int t = threadIdx.x;
  const int pair = blockIdx.x, chunk = blockIdx.y;
  // columns with |x|^2 <= nu2 are at the rounding level of X: their values
  // are known only to ~nu absolutely, so they are neither rotated nor tested
  const double nu2 = nu_rel2 * (*xnorm2);
  pair_columns(round, pair, nb, nn, col);
  if (t == 0) { any_rot = 0; bad = 0; }
  __syncthreads();
  // sum the partial Grams of this pair in a fixed order
  for (int e = t; e < NGRAM; e += NT) {
    double2 s = make_double2(0, 0);
    for (int c = 0; c < nparts; c++) s = cadd(s, parts[((size_t)pair * nparts + c) * NGRAM + e]);
    G[e / JC][e % JC] = s;
    W[e / JC][e % JC] = make_double2((e / JC) == (e % JC) ? 1.0 : 0.0, 0.0);
    if (!isfinite(s.x) || !isfinite(s.y)) bad = 1;
  }
  __syncthreads();
  if (bad) {
    if (t == 0 && chunk == 0) atomicOr(&flags[QT_FLAG_NONFINITE], 1);
    return;
  }
  // is this pair already orthogonal to tol?  (the largest relative
  // off-diagonal above tol is recorded as float bits)
  for (int e = t; e < NGRAM; e += NT) {
    const int i = e / JC, j = e % JC;
    if (i < j && col[i] >= 0 && col[j] >= 0) {
      const double a = G[i][i].x, b = G[j][j].x;
      const double g = sqrt(cabs2(G[i][j]));
      if (a > nu2 && b > nu2 && g > tol * sqrt(a * b)) {
        any_rot = 1;
        if (chunk == 0) {
          const float rel = (a > 0 && b > 0) ? (float)fmin(g / sqrt(a * b), 1.0) : 1.0f;
          atomicMax(&flags[QT_FLAG_OFFMAX], __float_as_int(rel));
        }
      }
    }
  }
  __syncthreads();
  if (!any_rot) return;
  if (t == 0 && chunk == 0) atomicAdd(&flags[QT_FLAG_ROTATED], 1);

  // cyclic two-sided Jacobi on the 16x16 Gram, diagonalised well below the
  // outer threshold so that the rounding of the applied rotation (in the
  // storage precision) cannot leave the pair just above `tol`
  const double tol_inner = fmin(tol, 1e-14);
  for (int sweep = 0; sweep < MAX_INNER; sweep++) {
    __syncthreads();  // every thread has read inner_rot of the previous sweep
    if (t == 0) inner_rot = 0;
    __syncthreads();
    for (int ir = 0; ir < JC - 1; ir++) {
      if (t < JC / 2) {
        int p, q;
        tournament(ir, t, JC, p, q);
        rp[t] = p; rq[t] = q; ron[t] = 0;
        if (col[p] >= 0 && col[q] >= 0) {
          // the running diagonal is clamped at zero (see the update below)
          const double a = fmax(G[p][p].x, 0.0), b = fmax(G[q][q].x, 0.0);
          const double2 g = G[p][q];
          const double ag = sqrt(cabs2(g));
          if (a > nu2 && b > nu2 && ag > tol_inner * sqrt(a * b)) {
            const double zeta = (b - a) / (2.0 * ag);
            const double tt = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            const double c = 1.0 / sqrt(1.0 + tt * tt);
            ron[t] = 1; rc[t] = c; rs[t] = c * tt; rt[t] = tt * ag; ra[t] = a; rb[t] = b;
            re[t] = make_double2(g.x / ag, g.y / ag);  // e^{i phi}
            inner_rot = 1;
          }
        }
      }
      __syncthreads();
      // columns p, q of G and W:  [x_p, x_q] <- [c x_p - s e^{-i phi} x_q,  s e^{i phi} x_p + c x_q]
      {
        const int task = t & 127, k = task >> 4, r = task & 15;
        if (ron[k]) {
          double2 (*M)[JC + 1] = (t < 128) ? G : W;
          const int p = rp[k], q = rq[k];
          const double c = rc[k], s = rs[k];
          const double2 e = re[k];
          const double2 xp = M[r][p], xq = M[r][q];
          const double2 sem = make_double2(s * e.x, -s * e.y), sep = make_double2(s * e.x, s * e.y);
          M[r][p] = csub(cscale(xp, c), cmul(sem, xq));
          M[r][q] = cadd(cmul(sep, xp), cscale(xq, c));
        }
      }
      __syncthreads();
      // rows p, q of G:  [g_p; g_q] <- [c g_p - s e^{i phi} g_q;  s e^{-i phi} g_p + c g_q]
      if (t < 128) {
        const int k = t >> 4, r = t & 15;
        if (ron[k]) {
          const int p = rp[k], q = rq[k];
          const double c = rc[k], s = rs[k];
          const double2 e = re[k];
          const double2 gp = G[p][r], gq = G[q][r];
          const double2 sep = make_double2(s * e.x, s * e.y), sem = make_double2(s * e.x, -s * e.y);
          G[p][r] = csub(cscale(gp, c), cmul(sep, gq));
          G[q][r] = cadd(cmul(sem, gp), cscale(gq, c));
        }
      }
      __syncthreads();
      if (t < JC / 2 && ron[t]) {
        // The rotated 2x2 block is diag(alpha - t|gamma|, beta + t|gamma|).
        // For nearly parallel columns of very different norms alpha - t|gamma|
        // cancels and can round below zero; it is clamped at zero so no NaN
        // reaches a later comparison (the next outer sweep recomputes the
        // Gram from the rotated vectors themselves).
        const int p = rp[t], q = rq[t];
        G[p][q] = make_double2(0, 0);
        G[q][p] = make_double2(0, 0);
        G[p][p] = make_double2(fmax(ra[t] - rt[t], 0.0), 0);
        G[q][q] = make_double2(rb[t] + rt[t], 0);
      }
      __syncthreads();
    }
    const int again = inner_rot;  // read after the round's closing barrier
    if (!again) break;
  }
  for (int e = t; e < NGRAM; e += NT) Wt[e / JC][e % JC] = ccast<CS>(W[e / JC][e % JC]);
  __syncthreads();

  // apply the 16x16 unitary to this chunk's rows of X and of V
  const int xb = chunk * x_rows_per_chunk, vb = chunk * v_rows_per_chunk;
  apply_rows<TS>(X, ldx, xb, min(mm, xb + x_rows_per_chunk), col, Wt, Xs);
  apply_rows<TS>(V, ldv, vb, min(nn, vb + v_rows_per_chunk), col, Wt, Xs);
}

// ||X||_F^2 in FP64, one CTA per column, added into *out.
template <typename TS>
__global__ void frob_kernel(const TS* __restrict__ X, int64_t ldx, int mm, double* out) {
  double s = 0;
  for (int i = threadIdx.x; i < mm; i += blockDim.x) {
    const double re = X[i + ldx * blockIdx.x].x, im = X[i + ldx * blockIdx.x].y;
    s = fma(re, re, s);
    s = fma(im, im, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

template <typename TS> struct gram_of;
template <> struct gram_of<double2> { typedef double type; };
template <> struct gram_of<float2> { typedef float type; };

}  // namespace

int qt_jacobi_layout(int64_t mm, int64_t nn, int* nb_out, int* chunks_out) {
  int nb = (int)((nn + JW - 1) / JW);
  if (nb % 2) nb++;
  if (nb < 2) nb = 2;
  const int pairs = nb / 2;
  // enough CTAs to cover the 152 SMs about twice, each chunk at least 128 rows
  int chunks = (int)((2 * 152 + pairs - 1) / pairs);
  chunks = std::max(1, std::min<int>(chunks, (int)((mm + 127) / 128)));
  *nb_out = nb;
  *chunks_out = chunks;
  return pairs * chunks * NGRAM + 1;  // double2 entries: partial Grams + ||X||_F^2
}

template <typename TS>
int qt_jacobi_svd_ws(qt_handle* h, TS* X, int64_t mm, int64_t nn, int64_t ldx, TS* V, int64_t ldv, double tol,
                     int max_sweeps, int* sweeps_out, double2* parts) {
  typedef typename gram_of<TS>::type TG;
  if (mm < nn) return qt_fail(h, QT_EINVAL, "jacobi: needs rows >= columns");
  QT_TRY(qt_set_identity<TS>(h, V, nn, ldv));
  *sweeps_out = 0;
  if (nn <= 1) return QT_OK;
  int nb = 0, chunks = 1;
  qt_jacobi_layout(mm, nn, &nb, &chunks);
  const int pairs = nb / 2, rounds = nb - 1;
  const int xrows = (int)(((mm + chunks - 1) / chunks + JR - 1) / JR * JR);
  const int vrows = (int)(((nn + chunks - 1) / chunks + JR - 1) / JR * JR);
  const dim3 grid(pairs, chunks);
  // the last workspace entry holds ||X||_F^2 (rotation-invariant); the noise
  // floor is nu = 4 sqrt(rows) u ||X||_F with u the storage unit roundoff
  double* xnorm2 = reinterpret_cast<double*>(parts + (size_t)pairs * chunks * NGRAM);
  {
    // ||X||_F^2 over the nn columns (ldx may exceed mm)
    QT_CHECK_CUDA(h, cudaMemsetAsync(xnorm2, 0, sizeof(double), h->stream));
    QT_LAUNCH(h, frob_kernel<TS>, (unsigned)nn, 256, 0, X, ldx, (int)mm, xnorm2);
  }
  const double u = (sizeof(typename real_of<TS>::type) == 8) ? 1.11e-16 : 5.96e-8;
  const double nu_rel = 4.0 * std::sqrt((double)std::max<int64_t>(mm, 16)) * u;
  const double nu_rel2 = nu_rel * nu_rel;
  int sweep = 0;
  for (; sweep < max_sweeps; sweep++) {
    QT_CHECK_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(int) * QT_FLAG_COUNT, h->stream));
    for (int r = 0; r < rounds; r++) {
      QT_LAUNCH(h, (gram_kernel<TS, TG>), grid, NT, 0, X, ldx, (int)mm, (int)nn, nb, r, xrows, parts);
      QT_LAUNCH(h, rotate_kernel<TS>, grid, NT, 0, X, ldx, (int)mm, V, ldv, (int)nn, nb, r, chunks, xrows, vrows,
                (const double2*)parts, tol, nu_rel2, (const double*)xnorm2, h->d_flags);
    }
    QT_CHECK_CUDA(h, cudaMemcpyAsync(h->h_flags, h->d_flags, sizeof(int) * QT_FLAG_COUNT, cudaMemcpyDeviceToHost,
                                     h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->h_flags[QT_FLAG_NONFINITE]) return qt_fail(h, QT_ENUMERIC, "jacobi: non-finite value in the matrix");
    if (h->h_flags[QT_FLAG_ROTATED] == 0) break;
  }
  *sweeps_out = sweep + (sweep < max_sweeps ? 1 : 0);
  if (sweep >= max_sweeps) {
    // Out of sweeps: accept when the worst remaining pair is orthogonal to
    // 1e-6 relative (its effect on the singular values is below 1e-12).
    float off;
    std::memcpy(&off, &h->h_flags[QT_FLAG_OFFMAX], sizeof(float));
    if (off < 1e-6f) return QT_OK;
    return qt_fail(h, QT_ENUMERIC, "jacobi: no convergence within the sweep limit (off " + std::to_string(off) + ")");
  }
  return QT_OK;
}
template int qt_jacobi_svd_ws<double2>(qt_handle*, double2*, int64_t, int64_t, int64_t, double2*, int64_t, double,
                                       int, int*, double2*);
template int qt_jacobi_svd_ws<float2>(qt_handle*, float2*, int64_t, int64_t, int64_t, float2*, int64_t, double, int,
                                      int*, double2*);

template <typename TS>
int qt_jacobi_svd(qt_handle* h, TS* X, int64_t mm, int64_t nn, int64_t ldx, TS* V, int64_t ldv, double tol,
                  int max_sweeps, int* sweeps_out) {
  int nb = 0, chunks = 0;
  const int nparts = qt_jacobi_layout(mm, nn, &nb, &chunks);
  qt_scratch s(h);
  double2* parts;
  QT_TRY(s.get(&parts, (size_t)nparts));
  return qt_jacobi_svd_ws<TS>(h, X, mm, nn, ldx, V, ldv, tol, max_sweeps, sweeps_out, parts);
}
template int qt_jacobi_svd<double2>(qt_handle*, double2*, int64_t, int64_t, int64_t, double2*, int64_t, double, int,
                                    int*);
template int qt_jacobi_svd<float2>(qt_handle*, float2*, int64_t, int64_t, int64_t, float2*, int64_t, double, int,
                                   int*);
