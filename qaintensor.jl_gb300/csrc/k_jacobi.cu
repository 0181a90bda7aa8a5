// One-sided block Jacobi SVD (Hestenes), FP64 Gram and rotation angles.
//
// Replaces the dense LAPACK ?gesdd called by LinearAlgebra.svd at
// src/svd.jl:26-27 and in switch! (src/switch.jl, file line 77): X (mm x nn,
// mm >= nn) is driven to orthogonal columns, X <- X V, so X = U diag(s) and
// the input equals U diag(s) V^H.
//
// Columns are split into blocks of JW = 8.  One sweep is a round-robin
// tournament over the blocks: in every round each CTA takes one block pair
// (16 columns), forms their 16x16 Gram matrix in FP64, diagonalises it with a
// cyclic two-sided Jacobi whose 2x2 rotations use the relative-accuracy
// formula (tan from zeta = (beta-alpha)/(2|gamma|), the smaller root), and
// applies the accumulated 16x16 unitary to the 16 columns of X and of V.
// Pairs whose Gram is already diagonal to `tol` (relative) are skipped; a
// sweep in which no pair rotates ends the iteration.  Storage TS is double2
// (exact path) or float2 (FP32 storage, FP64 Gram and angles).
#include <cuda_runtime.h>

#include "qt_internal.cuh"

namespace {

constexpr int JW = 8;        // columns per block
constexpr int JC = 2 * JW;   // columns per block pair
constexpr int JR = 64;       // rows per shared-memory chunk
constexpr int NT = 256;      // threads per CTA
constexpr int MAX_INNER = 12;

__device__ inline void tournament(int r, int q, int n, int& a, int& b) {
  // circle method over n (even) players, round r, table q
  if (q == 0) { a = r % (n - 1); b = n - 1; }
  else { a = (r + q) % (n - 1); b = (r - q + (n - 1)) % (n - 1); }
  if (a > b) { const int t = a; a = b; b = t; }
}

template <typename TS>
__device__ void apply_rows(TS* __restrict__ M, int64_t ld, int rows, const int* col,
                           const typename cplx_of<typename real_of<TS>::type>::type (*Wt)[JC + 1],
                           TS (*Xs)[JC + 1]) {
  typedef typename real_of<TS>::type RS;
  typedef typename cplx_of<RS>::type CS;
  const int t = threadIdx.x;
  for (int r0 = 0; r0 < rows; r0 += JR) {
    for (int idx = t; idx < JR * JC; idx += NT) {
      const int rr = idx % JR, c = idx / JR, gr = r0 + rr;
      TS v = czero<TS>();
      if (gr < rows && col[c] >= 0) v = M[gr + ld * col[c]];
      Xs[rr][c] = v;
    }
    __syncthreads();
    for (int idx = t; idx < JR * JC; idx += NT) {
      const int c = idx % JC, rr = idx / JC, gr = r0 + rr;
      if (gr >= rows || col[c] < 0) continue;
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
jacobi_pair_kernel(TS* __restrict__ X, int64_t ldx, int mm, TS* __restrict__ V, int64_t ldv, int nn, int nb, int round,
                   double tol, int* __restrict__ flags) {
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
  int bi, bj;
  tournament(round, blockIdx.x, nb, bi, bj);
  if (t < JC) {
    const int gc = (t < JW) ? bi * JW + t : bj * JW + (t - JW);
    col[t] = (gc < nn) ? gc : -1;
  }
  if (t == 0) { any_rot = 0; bad = 0; }
  __syncthreads();

  // ---- phase 1: Gram matrix of the 16 columns, FP64 accumulation ----
  int gi = -1, gj = -1;
  if (t < JC * (JC + 1) / 2) {
    int r = 0, rem = t;
    while (rem >= JC - r) { rem -= JC - r; r++; }
    gi = r; gj = r + rem;
  }
  double2 acc = make_double2(0, 0);
  for (int r0 = 0; r0 < mm; r0 += JR) {
    for (int idx = t; idx < JR * JC; idx += NT) {
      const int rr = idx % JR, c = idx / JR, gr = r0 + rr;
      TS v = czero<TS>();
      if (gr < mm && col[c] >= 0) v = X[gr + ldx * col[c]];
      Xs[rr][c] = v;
    }
    __syncthreads();
    if (gi >= 0) {
      const int lim = min(JR, mm - r0);
      for (int rr = 0; rr < lim; rr++) cfma_conj(acc, ccast<double2>(Xs[rr][gi]), ccast<double2>(Xs[rr][gj]));
    }
    __syncthreads();
  }
  if (gi >= 0) {
    if (!isfinite(acc.x) || !isfinite(acc.y)) bad = 1;
    G[gi][gj] = acc;
    G[gj][gi] = cconj(acc);
  }
  for (int e = t; e < JC * JC; e += NT) W[e / JC][e % JC] = make_double2((e / JC) == (e % JC) ? 1.0 : 0.0, 0.0);
  __syncthreads();
  if (bad) {
    if (t == 0) atomicOr(&flags[QT_FLAG_NONFINITE], 1);
    return;
  }

  // ---- is this pair already orthogonal to tol? ----
  for (int e = t; e < JC * JC; e += NT) {
    const int i = e / JC, j = e % JC;
    if (i < j && col[i] >= 0 && col[j] >= 0) {
      const double a = G[i][i].x, b = G[j][j].x;
      const double g = sqrt(cabs2(G[i][j]));
      if (g > tol * sqrt(a * b)) any_rot = 1;
    }
  }
  __syncthreads();
  if (!any_rot) return;
  if (t == 0) atomicAdd(&flags[QT_FLAG_ROTATED], 1);

  // ---- phase 2: cyclic two-sided Jacobi on the 16x16 Gram ----
  for (int sweep = 0; sweep < MAX_INNER; sweep++) {
    if (t == 0) inner_rot = 0;
    __syncthreads();
    for (int ir = 0; ir < JC - 1; ir++) {
      if (t < JC / 2) {
        int p, q;
        tournament(ir, t, JC, p, q);
        rp[t] = p; rq[t] = q; ron[t] = 0;
        if (col[p] >= 0 && col[q] >= 0) {
          const double a = G[p][p].x, b = G[q][q].x;
          const double2 g = G[p][q];
          const double ag = sqrt(cabs2(g));
          if (ag > 0.0 && ag > tol * sqrt(a * b)) {
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
        // the rotated 2x2 block is diag(alpha - t|gamma|, beta + t|gamma|) exactly
        const int p = rp[t], q = rq[t];
        G[p][q] = make_double2(0, 0);
        G[q][p] = make_double2(0, 0);
        G[p][p] = make_double2(ra[t] - rt[t], 0);
        G[q][q] = make_double2(rb[t] + rt[t], 0);
      }
      __syncthreads();
    }
    if (!inner_rot) break;
  }
  for (int e = t; e < JC * JC; e += NT) Wt[e / JC][e % JC] = ccast<CS>(W[e / JC][e % JC]);
  __syncthreads();

  // ---- phase 3: apply the 16x16 unitary to X and V ----
  apply_rows<TS>(X, ldx, mm, col, Wt, Xs);
  apply_rows<TS>(V, ldv, nn, col, Wt, Xs);
}

}  // namespace

template <typename TS>
int qt_jacobi_svd(qt_handle* h, TS* X, int64_t mm, int64_t nn, int64_t ldx, TS* V, int64_t ldv, double tol,
                  int max_sweeps, int* sweeps_out) {
  if (mm < nn) return qt_fail(h, QT_EINVAL, "jacobi: needs rows >= columns");
  QT_TRY(qt_set_identity<TS>(h, V, nn, ldv));
  *sweeps_out = 0;
  if (nn <= 1) return QT_OK;
  int nb = (int)((nn + JW - 1) / JW);
  if (nb % 2) nb++;
  if (nb < 2) nb = 2;
  const int pairs = nb / 2, rounds = nb - 1;
  int sweep = 0;
  for (; sweep < max_sweeps; sweep++) {
    QT_CHECK_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(int) * QT_FLAG_COUNT, h->stream));
    for (int r = 0; r < rounds; r++)
      QT_LAUNCH(h, jacobi_pair_kernel<TS>, pairs, NT, 0, X, ldx, (int)mm, V, ldv, (int)nn, nb, r, tol, h->d_flags);
    QT_CHECK_CUDA(h, cudaMemcpyAsync(h->h_flags, h->d_flags, sizeof(int) * QT_FLAG_COUNT, cudaMemcpyDeviceToHost,
                                     h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->h_flags[QT_FLAG_NONFINITE]) return qt_fail(h, QT_ENUMERIC, "jacobi: non-finite value in the matrix");
    if (h->h_flags[QT_FLAG_ROTATED] == 0) break;
  }
  *sweeps_out = sweep + (sweep < max_sweeps ? 1 : 0);
  if (sweep >= max_sweeps) return qt_fail(h, QT_ENUMERIC, "jacobi: no convergence within the sweep limit");
  return QT_OK;
}
template int qt_jacobi_svd<double2>(qt_handle*, double2*, int64_t, int64_t, int64_t, double2*, int64_t, double, int,
                                    int*);
template int qt_jacobi_svd<float2>(qt_handle*, float2*, int64_t, int64_t, int64_t, float2*, int64_t, double, int,
                                   int*);
