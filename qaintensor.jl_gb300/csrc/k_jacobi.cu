// One-sided block Jacobi SVD (Hestenes).
//
// Replaces the dense LAPACK ?gesdd called by LinearAlgebra.svd at
// src/svd.jl:26-27 and in switch! (src/switch.jl:39): X (mm x nn,
// mm >= nn) is driven to orthogonal columns, X <- X V, so X = U diag(s) and
// the input equals U diag(s) V^H.
//
// Columns are split into blocks of JW = 8.  One sweep is a round-robin
// tournament over the blocks (circle method); a round processes every block
// pair (16 columns) at once: the pair's 16x16 Gram is formed, tested against
// `tol` (relative off-diagonals), diagonalised by a cyclic two-sided Jacobi
// (the pair solver) and the resulting unitary applied to the pair's columns
// of X (and rows of V).  A sweep in which no pair rotates ends the iteration.
// Round implementations:
//   FP32 storage, default: jacobi_sweep32_kernel -- one cooperative launch
//     per sweep, each round rebuilding its columns from the previous round's
//     unitaries (see the comment above that kernel);
//   FP32 storage, two launches per round: pair_eig32_kernel (Gram + test +
//     pair solver) and pair_apply32_kernel (rotation);
//   FP64 storage, default: pair_round_kernel -- one launch per round, a
//     thread-block cluster holding the pair's rows in shared memory;
//   any storage: gram_kernel + eig_kernel + apply_kernel (partial Grams
//     over row chunks, FP64 pair solver, rotation).
// The FP64-storage solvers work on the FP64 Gram; the FP32-storage solvers
// on the scaled FP32 Gram (cosines), see pair_eig_scaled below.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <functional>
#include <vector>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include <cooperative_groups.h>

#include <type_traits>

#include "qt_internal.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int JW = 8;        // columns per block
constexpr int JC = 2 * JW;   // columns per block pair
constexpr int JR = 64;       // rows per shared-memory slab
constexpr int NT = 256;      // threads per CTA
constexpr int MAX_INNER = 12;
constexpr int NGRAM = JC * JC;
static_assert(NT == NGRAM, "the round kernel maps one Gram entry to each thread");

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

// Shared state of the 16x16 pair diagonalisation: the Gram and the rotation
// angles in FP64 (the relative accuracy of the small columns lives in the
// Gram's small entries, which an FP32 update would swamp with the rounding
// of the large ones); the accumulated unitary W in RW (the storage
// precision, in which it is applied).
template <typename RW>
struct pair_eig_shared {
  typedef typename cplx_of<RW>::type CW;
  double2 G[JC][JC + 1];  // the pair's Gram, driven to diagonal
  CW W[JC][JC + 1];       // accumulated unitary
  int rp[JC / 2], rq[JC / 2], ron[JC / 2];
  double rc[JC / 2], rt[JC / 2], ra[JC / 2], rb[JC / 2];
  double2 rse[JC / 2];    // s e^{i phi}
  int inner_rot;
};

// Cyclic two-sided Jacobi on sh.G (Hermitian 16x16, every thread of the CTA
// calls it), W accumulating the rotations.  Each 2x2 rotation uses the
// relative-accuracy formula: tan from zeta = (beta-alpha)/(2|gamma|), the
// smaller root.  Columns with |x|^2 <= nu2 are at the rounding level of X and
// are neither rotated nor tested.
template <typename RW>
__device__ int diagonalise_pair(pair_eig_shared<RW>& sh, const int* col, double tol_inner, double nu2) {
  typedef typename cplx_of<RW>::type CW;
  const int t = threadIdx.x;
  int sweep = 0;
  for (; sweep < MAX_INNER; sweep++) {
    __syncthreads();  // every thread has read inner_rot of the previous sweep
    if (t == 0) sh.inner_rot = 0;
    __syncthreads();
    for (int ir = 0; ir < JC - 1; ir++) {
      if (t < JC / 2) {
        int p, q;
        tournament(ir, t, JC, p, q);
        sh.rp[t] = p; sh.rq[t] = q; sh.ron[t] = 0;
        if (col[p] >= 0 && col[q] >= 0) {
          // the running diagonal is clamped at zero (see the update below)
          const double a = fmax(sh.G[p][p].x, 0.0), b = fmax(sh.G[q][q].x, 0.0);
          const double2 g = sh.G[p][q];
          const double ag = sqrt(cabs2(g));
          if (a > nu2 && b > nu2 && ag > tol_inner * sqrt(a * b)) {
            const double zeta = (b - a) / (2.0 * ag);
            const double tt = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            const double c = 1.0 / sqrt(1.0 + tt * tt);
            const double sa = c * tt / ag;  // s / |gamma|: s e^{i phi} = sa * gamma
            sh.ron[t] = 1; sh.rc[t] = c; sh.rt[t] = tt * ag; sh.ra[t] = a; sh.rb[t] = b;
            sh.rse[t] = make_double2(sa * g.x, sa * g.y);
            sh.inner_rot = 1;
          }
        }
      }
      __syncthreads();
      // columns p, q of G and W:  [x_p, x_q] <- [c x_p - conj(se) x_q,  se x_p + c x_q]
      {
        const int task = t & 127, k = task >> 4, r = task & 15;
        if (sh.ron[k]) {
          const int p = sh.rp[k], q = sh.rq[k];
          const double c = sh.rc[k];
          const double2 se = sh.rse[k];
          if (t < 128) {
            const double2 xp = sh.G[r][p], xq = sh.G[r][q];
            sh.G[r][p] = csub(cscale(xp, c), cmul(cconj(se), xq));
            sh.G[r][q] = cadd(cmul(se, xp), cscale(xq, c));
          } else {
            const CW cw = ccast<CW>(make_double2(c, 0.0));
            const CW sew = ccast<CW>(se);
            const CW xp = sh.W[r][p], xq = sh.W[r][q];
            sh.W[r][p] = csub(cmul(cw, xp), cmul(cconj(sew), xq));
            sh.W[r][q] = cadd(cmul(sew, xp), cmul(cw, xq));
          }
        }
      }
      __syncthreads();
      // rows p, q of G:  [g_p; g_q] <- [c g_p - se g_q;  conj(se) g_p + c g_q]
      if (t < 128) {
        const int k = t >> 4, r = t & 15;
        if (sh.ron[k]) {
          const int p = sh.rp[k], q = sh.rq[k];
          const double c = sh.rc[k];
          const double2 se = sh.rse[k];
          const double2 gp = sh.G[p][r], gq = sh.G[q][r];
          sh.G[p][r] = csub(cscale(gp, c), cmul(se, gq));
          sh.G[q][r] = cadd(cmul(cconj(se), gp), cscale(gq, c));
        }
      }
      __syncthreads();
      if (t < JC / 2 && sh.ron[t]) {
        // The rotated 2x2 block is diag(alpha - t|gamma|, beta + t|gamma|).
        // For nearly parallel columns of very different norms alpha - t|gamma|
        // cancels and can round below zero; it is clamped at zero so no NaN
        // reaches a later comparison (the next outer sweep recomputes the
        // Gram from the rotated vectors themselves).
        const int p = sh.rp[t], q = sh.rq[t];
        sh.G[p][q] = make_double2(0, 0);
        sh.G[q][p] = make_double2(0, 0);
        sh.G[p][p] = make_double2(fmax(sh.ra[t] - sh.rt[t], 0.0), 0);
        sh.G[q][q] = make_double2(sh.rb[t] + sh.rt[t], 0);
      }
      __syncthreads();
    }
    const int again = sh.inner_rot;  // read after the round's closing barrier
    if (!again) break;
  }
  __syncthreads();
  return sweep + (sweep < MAX_INNER ? 1 : 0);
}

// FP32 variant for FP32 storage: the two-sided Jacobi runs on the scaled
// Gram Ghat = D^{-1/2} G D^{-1/2} (unit diagonal, off-diagonals are the
// cosines between columns) with the diagonal D tracked separately.  The
// cosines are O(1) numbers, so FP32 keeps each one accurate to ~u of its
// own pair whatever the spread of the column norms -- the property the
// unscaled FP32 Gram loses.  A rotation J of pair (p, q) acts on Ghat
// through Jt = D^{1/2} J D'^{-1/2}: Jt_pp = c sqrt(a/a'),
// Jt_qp = -s e^{-i phi} sqrt(b/a'), Jt_pq = s e^{i phi} sqrt(a/b'),
// Jt_qq = c sqrt(b/b'), with a' = a - t|gamma|, b' = b + t|gamma|.
// The unitary is accumulated in the same scaled form, Wt = D0^{1/2} W D^{-1/2}
// (D0 the initial diagonal): its entries are O(1), so their FP32 rounding is
// relative to each output column's own norm once W = D0^{-1/2} Wt D^{1/2} is
// formed -- small columns are not contaminated by the rounding of large ones.
struct pair_eig_scaled {
  float d[JC];            // current diagonal of G
  float d0[JC];           // initial diagonal
  float2 G[JC][JC + 1];   // scaled Gram (diagonal implicit 1)
  float2 W[JC][JC + 1];   // scaled unitary Wt, then W
  int rp[JC / 2], rq[JC / 2], ron[JC / 2];
  float na[JC / 2], nb[JC / 2], kpp[JC / 2], kqq[JC / 2];
  float2 kqp[JC / 2], kpq[JC / 2];
  int inner_rot;
};

// The scaled iteration with one update phase per round: the 16 indices form
// 8 disjoint pairs, so every entry of Jt^H Ghat Jt is a 2x2 combination of
// old entries -- G'[x][y] = sum_{a in {x,x'}} sum_{b in {y,y'}} conj(Jt[a][x])
// Ghat[a][b] Jt[b][y] (x' the partner of x, Jt = I on a pair that does not
// rotate) -- and every entry of Wt Jt a combination of two.  Thread t < 256
// owns entry (t / 16, t % 16) of both; the new values go to the other
// buffer, so a round costs two barriers (parameters, update).  Every thread
// of the block calls it (the barriers are block-wide).
struct pair_eig_scaled2 {
  float d[2][JC];
  float d0[JC];
  float2 G[2][JC][JC + 1];
  float2 W[2][JC][JC + 1];
  int partner[JC];          // partner index of each index in this round
  float2 jt[JC][2];         // Jt[x][x] (real in .x) and Jt[x'][x] for column x
  int inner_rot;
};

__device__ int diagonalise_scaled2(pair_eig_scaled2& sh, const int* col, float tol_inner, float nu2, int max_inner,
                                   int* buf_out) {
  const int t = threadIdx.x, x = (t >> 4) & 15, y = t & 15;
  const bool owner = t < NGRAM;
  int cur = 0, sweep = 0;
  // inner_rot holds the number (1-based) of the last sweep that rotated; the
  // caller zeroes it before the first call
  for (; sweep < max_inner; sweep++) {
    for (int ir = 0; ir < JC - 1; ir++) {
      if (t < JC / 2) {
        int p, q;
        tournament(ir, t, JC, p, q);
        sh.partner[p] = q; sh.partner[q] = p;
        const float a = sh.d[cur][p], b = sh.d[cur][q];
        const float2 gs = sh.G[cur][p][q];
        const float ags = sqrtf(gs.x * gs.x + gs.y * gs.y);
        float2 jpp = make_float2(1.f, 0.f), jqp = make_float2(0.f, 0.f), jpq = jqp, jqq = jpp;
        float a2 = a, b2 = b;
        if (col[p] >= 0 && col[q] >= 0 && a > nu2 && b > nu2 && ags > tol_inner) {
          const float ag = ags * sqrtf(a * b);  // |gamma|
          const float zeta = __fdividef(b - a, 2.f * ag);
          const float r1 = sqrtf(fmaf(zeta, zeta, 1.f));
          const float tt = copysignf(__frcp_rn(fabsf(zeta) + r1), zeta);
          const float c = rsqrtf(fmaf(tt, tt, 1.f)), sn = c * tt;
          const float inv = __frcp_rn(ags);
          const float2 e = make_float2(gs.x * inv, gs.y * inv);
          a2 = fmaxf(a - tt * ag, nu2);  // a column driven to the noise level is frozen
          b2 = b + tt * ag;
          const float ia2 = rsqrtf(a2), ib2 = rsqrtf(b2), sqa = sqrtf(a), sqb = sqrtf(b);
          jpp = make_float2(c * sqa * ia2, 0.f);
          jqp = make_float2(-sn * e.x * sqb * ia2, sn * e.y * sqb * ia2);  // -s conj(e) sqrt(b/a')
          jpq = make_float2(sn * e.x * sqa * ib2, sn * e.y * sqa * ib2);   //  s e sqrt(a/b')
          jqq = make_float2(c * sqb * ib2, 0.f);
          sh.inner_rot = sweep + 1;
        }
        // column p of Jt: rows p (jpp) and q (jqp); column q: rows q (jqq) and p (jpq)
        sh.jt[p][0] = jpp; sh.jt[p][1] = jqp;
        sh.jt[q][0] = jqq; sh.jt[q][1] = jpq;
        sh.d[cur ^ 1][p] = a2; sh.d[cur ^ 1][q] = b2;
      }
      __syncthreads();
      if (owner) {
        const int xp = sh.partner[x], yp = sh.partner[y];
        const float2 jxx = sh.jt[x][0], jpx = sh.jt[x][1];  // Jt[x][x], Jt[x'][x]
        const float2 jyy = sh.jt[y][0], jpy = sh.jt[y][1];  // Jt[y][y], Jt[y'][y]
        // Ghat: diagonal implicit 1; the off-diagonal of a rotated pair is
        // zero, that of a pair left alone keeps its (sub-tolerance) value
        float2 gnew = make_float2(0.f, 0.f);
        if (xp == y && x != y) {
          const bool rotated = jxx.x != 1.f || jxx.y != 0.f || jpx.x != 0.f || jpx.y != 0.f;
          if (!rotated) gnew = sh.G[cur][x][y];
        } else if (x != y) {
          const float2 g_xy = sh.G[cur][x][y], g_xq = sh.G[cur][x][yp];
          const float2 g_py = sh.G[cur][xp][y], g_pq = sh.G[cur][xp][yp];
          // column step: h_a = G[a][y] Jt[y][y] + G[a][y'] Jt[y'][y] for a in {x, x'}
          const float2 hx = cadd(cmul(g_xy, jyy), cmul(g_xq, jpy));
          const float2 hp = cadd(cmul(g_py, jyy), cmul(g_pq, jpy));
          // row step: conj(Jt[x][x]) h_x + conj(Jt[x'][x]) h_x'
          gnew = cadd(cmul(cconj(jxx), hx), cmul(cconj(jpx), hp));
        }
        sh.G[cur ^ 1][x][y] = gnew;
        // Wt Jt: column y
        const float2 w_xy = sh.W[cur][x][y], w_xq = sh.W[cur][x][yp];
        sh.W[cur ^ 1][x][y] = cadd(cmul(w_xy, jyy), cmul(w_xq, jpy));
      }
      cur ^= 1;
      __syncthreads();
    }
    const int again = sh.inner_rot == sweep + 1;  // written before the round's closing barrier
    __syncthreads();  // every thread has read it before the next sweep may write it again
    if (!again) break;
  }
  // W = D0^{-1/2} Wt D^{1/2}
  if (owner) {
    const float d0 = sh.d0[x];
    sh.W[cur][x][y] = d0 > 0.f ? cscale(sh.W[cur][x][y], sqrtf(sh.d[cur][y] / d0))
                               : make_float2(x == y ? 1.f : 0.f, 0.f);
  }
  __syncthreads();
  *buf_out = cur;
  return sweep + (sweep < max_inner ? 1 : 0);
}

// The same iteration run by one warp (lanes 0-31 of the calling CTA; the
// other warps skip it and wait at the caller's barrier): the per-round
// barriers become __syncwarp, and the idle warps leave the SM's issue slots
// to the other CTAs resident on it.  Rotation parameters are computed by
// lanes 0-7 (one pair each) and kept in shared memory; the column updates
// (256 row tasks over G and Wt) and row updates (128) are spread over the
// 32 lanes.
__device__ int diagonalise_scaled_warp(pair_eig_scaled& sh, const int* col, float tol_inner, float nu2,
                                       int max_inner) {
  const int lane = threadIdx.x & 31;
  int sweep = 0;
  for (; sweep < max_inner; sweep++) {
    int rotated = 0;
    for (int ir = 0; ir < JC - 1; ir++) {
      int on = 0;
      if (lane < JC / 2) {
        int p, q;
        tournament(ir, lane, JC, p, q);
        sh.rp[lane] = p; sh.rq[lane] = q;
        const float a = sh.d[p], b = sh.d[q];
        const float2 gs = sh.G[p][q];
        const float ags = sqrtf(gs.x * gs.x + gs.y * gs.y);
        if (col[p] >= 0 && col[q] >= 0 && a > nu2 && b > nu2 && ags > tol_inner) {
          const float ag = ags * sqrtf(a * b);  // |gamma|
          const float zeta = __fdividef(b - a, 2.f * ag);
          const float r1 = sqrtf(fmaf(zeta, zeta, 1.f));
          const float tt = copysignf(__frcp_rn(fabsf(zeta) + r1), zeta);
          const float c = rsqrtf(fmaf(tt, tt, 1.f)), sn = c * tt;
          const float inv = __frcp_rn(ags);
          const float2 e = make_float2(gs.x * inv, gs.y * inv);
          const float a2 = fmaxf(a - tt * ag, nu2), b2 = b + tt * ag;
          const float ia2 = rsqrtf(a2), ib2 = rsqrtf(b2), sqa = sqrtf(a), sqb = sqrtf(b);
          sh.na[lane] = a2; sh.nb[lane] = b2;
          sh.kpp[lane] = c * sqa * ia2;
          sh.kqp[lane] = make_float2(-sn * e.x * sqb * ia2, sn * e.y * sqb * ia2);
          sh.kpq[lane] = make_float2(sn * e.x * sqa * ib2, sn * e.y * sqa * ib2);
          sh.kqq[lane] = c * sqb * ib2;
          on = 1;
        }
        sh.ron[lane] = on;
      }
      rotated |= __any_sync(0xffffffffu, on);
      __syncwarp();
      // columns p, q: tasks (matrix, pair k, row r) = lane + 32 i
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const int task = lane + 32 * i, mat = task >> 7, k = (task >> 4) & 7, r = task & 15;
        if (!sh.ron[k]) continue;
        const int p = sh.rp[k], q = sh.rq[k];
        if (mat == 0 && (r == p || r == q)) continue;
        float2 (*M)[JC + 1] = mat == 0 ? sh.G : sh.W;
        const float2 xp = M[r][p], xq = M[r][q];
        M[r][p] = cadd(cscale(xp, sh.kpp[k]), cmul(sh.kqp[k], xq));
        M[r][q] = cadd(cmul(sh.kpq[k], xp), cscale(xq, sh.kqq[k]));
      }
      __syncwarp();
      // rows p, q of Ghat; the pair's own 2x2 block and diagonal
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int task = lane + 32 * i, k = task >> 4, r = task & 15;
        if (!sh.ron[k]) continue;
        const int p = sh.rp[k], q = sh.rq[k];
        if (r != p && r != q) {
          const float2 gp = sh.G[p][r], gq = sh.G[q][r];
          sh.G[p][r] = cadd(cscale(gp, sh.kpp[k]), cmul(cconj(sh.kqp[k]), gq));
          sh.G[q][r] = cadd(cmul(cconj(sh.kpq[k]), gp), cscale(gq, sh.kqq[k]));
        } else if (r == p) {
          sh.G[p][q] = make_float2(0.f, 0.f);
          sh.G[q][p] = make_float2(0.f, 0.f);
          sh.d[p] = sh.na[k];
          sh.d[q] = sh.nb[k];
        }
      }
      __syncwarp();
    }
    if (!rotated) break;
  }
  // W = D0^{-1/2} Wt D^{1/2}
  for (int e = lane; e < NGRAM; e += 32) {
    const int i = e >> 4, j = e & 15;
    const float d0 = sh.d0[i];
    sh.W[i][j] = d0 > 0.f ? cscale(sh.W[i][j], sqrtf(sh.d[j] / d0)) : make_float2(i == j ? 1.f : 0.f, 0.f);
  }
  __syncwarp();
  return sweep + (sweep < max_inner ? 1 : 0);
}

// One CTA per block pair: sum the partial Grams, test the pair, and when it
// needs rotating diagonalise its 16x16 Gram; the unitary goes to wout[pair]
// and the decision to rot[pair] (the apply kernel reads both).
__global__ void __launch_bounds__(NT)
eig_kernel(int nn, int nb, int round, int nparts, const double2* __restrict__ parts, double tol, double nu_rel2,
           const double* __restrict__ xnorm2, double2* __restrict__ wout, int* __restrict__ rot,
           int* __restrict__ flags) {
  __shared__ pair_eig_shared<double> sh;
  __shared__ int col[JC];
  __shared__ int any_rot, bad, offmax_blk, offbig_blk;

  const int t = threadIdx.x;
  const int pair = blockIdx.x;
  const double nu2 = nu_rel2 * (*xnorm2);
  pair_columns(round, pair, nb, nn, col);
  if (t == 0) { any_rot = 0; bad = 0; offmax_blk = 0; offbig_blk = 0; }
  __syncthreads();
  // sum the partial Grams of this pair in a fixed order
  for (int e = t; e < NGRAM; e += NT) {
    double2 s = make_double2(0, 0);
    for (int c = 0; c < nparts; c++) s = cadd(s, parts[((size_t)pair * nparts + c) * NGRAM + e]);
    sh.G[e / JC][e % JC] = s;
    sh.W[e / JC][e % JC] = make_double2((e / JC) == (e % JC) ? 1.0 : 0.0, 0.0);
    if (!isfinite(s.x) || !isfinite(s.y)) bad = 1;
  }
  __syncthreads();
  if (bad) {
    if (t == 0) {
      atomicOr(&flags[QT_FLAG_NONFINITE], 1);
      rot[pair] = 0;
    }
    return;
  }
  // is this pair already orthogonal to tol?  (the largest relative
  // off-diagonal above tol is recorded as float bits, one atomic per pair)
  float relmax = 0.f, relbig = 0.f;
  const double big2 = 1e-6 * (*xnorm2);
  for (int e = t; e < NGRAM; e += NT) {
    const int i = e / JC, j = e % JC;
    if (i < j && col[i] >= 0 && col[j] >= 0) {
      const double a = sh.G[i][i].x, b = sh.G[j][j].x;
      const double g = sqrt(cabs2(sh.G[i][j]));
      if (a > nu2 && b > nu2 && g > tol * sqrt(a * b)) {
        any_rot = 1;
        const float rel = (a > 0 && b > 0) ? (float)fmin(g / sqrt(a * b), 1.0) : 1.0f;
        relmax = fmaxf(relmax, rel);
        if (a > big2 && b > big2) relbig = fmaxf(relbig, rel);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    relmax = fmaxf(relmax, __shfl_xor_sync(0xffffffffu, relmax, o));
    relbig = fmaxf(relbig, __shfl_xor_sync(0xffffffffu, relbig, o));
  }
  if ((t & 31) == 0 && relmax > 0.f) atomicMax(&offmax_blk, __float_as_int(relmax));
  if ((t & 31) == 0 && relbig > 0.f) atomicMax(&offbig_blk, __float_as_int(relbig));
  __syncthreads();
  if (t == 0 && offmax_blk > 0) atomicMax(&flags[QT_FLAG_OFFMAX], offmax_blk);
  if (t == 0 && offbig_blk > 0) atomicMax(&flags[QT_FLAG_OFFBIG], offbig_blk);
  __syncthreads();
  if (t == 0) rot[pair] = any_rot;
  if (!any_rot) return;
  if (t == 0) atomicAdd(&flags[QT_FLAG_ROTATED], 1);
  // diagonalised well below the outer threshold so that the rounding of the
  // applied rotation (in the storage precision) cannot leave the pair just
  // above `tol`
  const int inner = diagonalise_pair<double>(sh, col, fmin(tol, 1e-14), nu2);
  if (t == 0) atomicAdd(&flags[QT_FLAG_INNER], inner);
  for (int e = t; e < NGRAM; e += NT) wout[(size_t)pair * NGRAM + e] = sh.W[e / JC][e % JC];
}

// out[r, col[c]] = sum_k Xs[k*lds + r] W[k][c] for r < nrows: each thread a
// 4-row x 4-column tile (rows lane + 32 i, columns 4 cq + j), so one shared
// load of X feeds four complex FMAs and the global stores run along rows.
template <typename TS>
__device__ void rotate_rows(const TS* __restrict__ Xs, int lds, int nrows, TS* __restrict__ out, int64_t ld,
                            const int* col, const TS (*W)[JC + 1]) {
  const int t = threadIdx.x, lane = t & 31, cq = (t >> 5) & 3, rg = t >> 7;
  for (int r0 = rg * 128; r0 < nrows; r0 += 256) {
    TS acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = czero<TS>();
#pragma unroll 4
    for (int k = 0; k < JC; k++) {
      TS w[4], x[4];
#pragma unroll
      for (int j = 0; j < 4; j++) w[j] = W[k][cq * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int r = r0 + lane + 32 * i;
        x[i] = (r < nrows) ? Xs[k * lds + r] : czero<TS>();
      }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) cfma(acc[i][j], x[i], w[j]);
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int r = r0 + lane + 32 * i;
      if (r >= nrows) continue;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int c = col[cq * 4 + j];
        if (c >= 0) out[r + ld * c] = acc[i][j];
      }
    }
  }
}

// rows [0, nrows) of the pair's columns of M -> Xs (column c at Xs + c*lds).
// Thread t copies rows t, t + NT, ...: for each row it issues the 16 column
// loads back to back (independent, coalesced across the warp) before storing.
template <typename TS>
__device__ void stage_rows(const TS* __restrict__ M, int64_t ld, int nrows, int rows_alloc, const int* col,
                           TS* __restrict__ Xs, int lds) {
  for (int rr = threadIdx.x; rr < rows_alloc; rr += NT) {
    TS v[JC];
#pragma unroll
    for (int c = 0; c < JC; c++) v[c] = (rr < nrows && col[c] >= 0) ? M[rr + ld * col[c]] : czero<TS>();
#pragma unroll
    for (int c = 0; c < JC; c++) Xs[c * lds + rr] = v[c];
  }
}

// One round of the sweep in one launch.  A thread-block cluster of `csize`
// CTAs owns one block pair; CTA q of the cluster holds rows
// [q*xrows_c, (q+1)*xrows_c) of the pair's 16 columns of X in shared memory.
// Each CTA forms its partial Gram (accumulated in the storage precision: each
// entry is then accurate relative to its own column norms), the partials are
// summed in FP64 over the cluster through distributed shared memory in rank
// order, CTA 0 of the cluster tests the pair and diagonalises the Gram, the
// other CTAs copy its unitary through distributed shared memory, and every
// CTA rotates its own rows of X and its share of the rows of V.
template <typename TS>
__global__ void __launch_bounds__(NT)
pair_round_kernel(TS* __restrict__ X, int64_t ldx, int mm, TS* __restrict__ V, int64_t ldv, int nn, int nb, int round,
                  int csize, int xrows_c, int vrows_c, int lds, double tol, double tol_inner, double nu_rel2,
                  const double* __restrict__ xnorm2, int* __restrict__ flags, int max_inner,
                  unsigned long long* __restrict__ phase_ns) {
  typedef typename real_of<TS>::type RE;
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  TS* Xs = reinterpret_cast<TS*>(dyn_smem);
  constexpr bool F32 = sizeof(RE) == 4;
  __shared__ typename std::conditional<F32, pair_eig_scaled, pair_eig_shared<double>>::type sh;
  __shared__ TS gpart[NGRAM];
  __shared__ int col[JC];
  __shared__ int any_rot, bad, offmax_blk, offbig_blk;
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = (int)cluster.block_rank();
  const int pair = blockIdx.x / csize;
  const int t = threadIdx.x;
  // optional phase timing (diagnostics): thread 0 of each CTA adds the time
  // spent in each phase to phase_ns[8 * (crank != 0) + phase]
  unsigned long long tp = 0;
  auto phase = [&](int ph) {
    if (phase_ns && t == 0) {
      unsigned long long tn;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(tn));
      if (ph > 0) atomicAdd(&phase_ns[8 * (crank != 0) + ph - 1], tn - tp);
      tp = tn;
    }
  };
  phase(0);
  pair_columns(round, pair, nb, nn, col);
  if (t == 0) { any_rot = 0; bad = 0; offmax_blk = 0; offbig_blk = 0; }
  __syncthreads();
  const int xb = crank * xrows_c;
  const int xr = max(0, min(mm, xb + xrows_c) - xb);
  stage_rows<TS>(X + xb, ldx, xr, xrows_c, col, Xs, lds);
  __syncthreads();
  phase(1);  // 0: stage
  // partial Gram over this CTA's rows: the 36 upper 2x2 tiles of the 16x16
  // Gram, four threads per tile on interleaved rows (four independent
  // complex accumulators each), reduced with shuffles in a fixed order
  if (t < 160) {
    const int tile = t >> 2, g = t & 3;
    const bool act = tile < 36;
    int bi = 0, rem = act ? tile : 0;
    while (rem >= 8 - bi) { rem -= 8 - bi; bi++; }
    const int bj = bi + rem;
    const TS* x0 = Xs + (2 * bi) * lds;
    const TS* x1 = x0 + lds;
    const TS* y0 = Xs + (2 * bj) * lds;
    const TS* y1 = y0 + lds;
    TS a00 = czero<TS>(), a01 = czero<TS>(), a10 = czero<TS>(), a11 = czero<TS>();
    if (act) {
      for (int rr = g; rr < xr; rr += 4) {
        const TS p0 = x0[rr], p1 = x1[rr], q0 = y0[rr], q1 = y1[rr];
        cfma_conj(a00, p0, q0);
        cfma_conj(a01, p0, q1);
        cfma_conj(a10, p1, q0);
        cfma_conj(a11, p1, q1);
      }
    }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
      a00.x += __shfl_xor_sync(0xffffffffu, a00.x, o); a00.y += __shfl_xor_sync(0xffffffffu, a00.y, o);
      a01.x += __shfl_xor_sync(0xffffffffu, a01.x, o); a01.y += __shfl_xor_sync(0xffffffffu, a01.y, o);
      a10.x += __shfl_xor_sync(0xffffffffu, a10.x, o); a10.y += __shfl_xor_sync(0xffffffffu, a10.y, o);
      a11.x += __shfl_xor_sync(0xffffffffu, a11.x, o); a11.y += __shfl_xor_sync(0xffffffffu, a11.y, o);
    }
    if (act && g == 0) {
      const int i0 = 2 * bi, j0 = 2 * bj;
      gpart[i0 * JC + j0] = a00;             gpart[j0 * JC + i0] = cconj(a00);
      gpart[(i0 + 1) * JC + j0 + 1] = a11;   gpart[(j0 + 1) * JC + i0 + 1] = cconj(a11);
      gpart[i0 * JC + j0 + 1] = a01;         gpart[(j0 + 1) * JC + i0] = cconj(a01);
      if (bi != bj) { gpart[(i0 + 1) * JC + j0] = a10; gpart[j0 * JC + i0 + 1] = cconj(a10); }
    }
  }
  __syncthreads();
  phase(2);  // 1: Gram
  cluster.sync();
  phase(3);  // 2: first cluster barrier
  const double nu2 = nu_rel2 * (*xnorm2);
  if (crank == 0) {
    // FP64 sums of the partials in rank order; the remote loads are issued
    // together (independent) before the sum
    double2 sum_e;
    {
      const int e = t;  // NT == NGRAM: one Gram entry per thread
      TS v[8];
#pragma unroll
      for (int q = 0; q < 8; q++) v[q] = q < csize ? cluster.map_shared_rank(gpart, q)[e] : czero<TS>();
      sum_e = make_double2(0, 0);
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (q < csize) sum_e = cadd(sum_e, ccast<double2>(v[q]));
      if (!isfinite(sum_e.x) || !isfinite(sum_e.y)) bad = 1;
    }
    if constexpr (F32) {
      __shared__ double dd[JC];
      const int i = t / JC, j = t % JC;
      if (i == j) {
        dd[i] = sum_e.x;
        sh.d[i] = (float)sum_e.x;
        sh.d0[i] = (float)sum_e.x;
      }
      __syncthreads();
      float2 v = make_float2(0.f, 0.f);
      if (i != j && dd[i] > nu2 && dd[j] > nu2) {
        const double sc = 1.0 / sqrt(dd[i] * dd[j]);
        v = make_float2((float)(sum_e.x * sc), (float)(sum_e.y * sc));
      }
      sh.G[i][j] = v;
      sh.W[i][j] = make_float2(i == j ? 1.f : 0.f, 0.f);
    } else {
      sh.G[t / JC][t % JC] = sum_e;
      sh.W[t / JC][t % JC] = mk((RE)((t / JC) == (t % JC) ? 1 : 0), (RE)0);
    }
  }
  cluster.sync();  // the partials have been read: CTAs 1.. may leave or move on
  phase(4);  // 3: partial sums + second barrier
  if (crank == 0) {
    // is this pair already orthogonal to tol?  (the largest relative
    // off-diagonal above tol is recorded as float bits)
    if (!bad) {
      // the largest relative off-diagonal above tol: a block maximum first,
      // then one global atomic per pair (thousands of same-address atomics
      // per round would serialise in L2)
      float relmax = 0.f, relbig = 0.f;
      const double big2 = 1e-6 * (*xnorm2);
      for (int e = t; e < NGRAM; e += NT) {
        const int i = e / JC, j = e % JC;
        if (i < j && col[i] >= 0 && col[j] >= 0) {
          double rel = 0, a, b;
          bool live;
          if constexpr (F32) {
            a = sh.d[i]; b = sh.d[j];
            rel = sqrt((double)cabs2(sh.G[i][j]));
          } else {
            a = sh.G[i][i].x; b = sh.G[j][j].x;
            if (a > nu2 && b > nu2) rel = sqrt(cabs2(sh.G[i][j])) / sqrt(a * b);
          }
          live = a > nu2 && b > nu2;
          if (live && rel > tol) {
            any_rot = 1;
            relmax = fmaxf(relmax, (float)fmin(rel, 1.0));
            if (a > big2 && b > big2) relbig = fmaxf(relbig, (float)fmin(rel, 1.0));
          }
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        relmax = fmaxf(relmax, __shfl_xor_sync(0xffffffffu, relmax, o));
        relbig = fmaxf(relbig, __shfl_xor_sync(0xffffffffu, relbig, o));
      }
      if ((t & 31) == 0 && relmax > 0.f) atomicMax(&offmax_blk, __float_as_int(relmax));
      if ((t & 31) == 0 && relbig > 0.f) atomicMax(&offbig_blk, __float_as_int(relbig));
      __syncthreads();
      if (t == 0 && offmax_blk > 0) atomicMax(&flags[QT_FLAG_OFFMAX], offmax_blk);
      if (t == 0 && offbig_blk > 0) atomicMax(&flags[QT_FLAG_OFFBIG], offbig_blk);
    } else if (t == 0) {
      atomicOr(&flags[QT_FLAG_NONFINITE], 1);
    }
    __syncthreads();
    if (any_rot) {
      if (t == 0) atomicAdd(&flags[QT_FLAG_ROTATED], 1);
      int inner;
      if constexpr (F32) {
        inner = 0;
        if (t < 32) inner = diagonalise_scaled_warp(sh, col, (float)tol_inner, (float)nu2, max_inner);
        __syncthreads();
      } else {
        inner = diagonalise_pair<RE>(sh, col, tol_inner, nu2);
      }
      if (t == 0) atomicAdd(&flags[QT_FLAG_INNER], inner);
    }
  }
  __syncthreads();
  phase(5);  // 4: test + pair solver (CTA 0)
  cluster.sync();  // CTA 0's decision and unitary are ready
  if (crank != 0) {
    if (t == 0) any_rot = *cluster.map_shared_rank(&any_rot, 0);
    for (int e = t; e < NGRAM; e += NT) sh.W[e / JC][e % JC] = cluster.map_shared_rank(&sh.W[0][0], 0)[(e / JC) * (JC + 1) + e % JC];
  }
  cluster.sync();  // CTA 0 stays resident until every copy is done
  phase(6);  // 5: third/fourth barrier + unitary copy
  if (!any_rot) return;  // the same decision in every CTA of the cluster
  rotate_rows<TS>(Xs, lds, xr, X + xb, ldx, col, sh.W);
  __syncthreads();
  phase(7);  // 6: rotate X
  __syncthreads();  // Xs is reused for V
  if (V == nullptr) return;  // no accumulated rotations wanted
  const int vb = crank * vrows_c;
  const int vr = max(0, min(nn, vb + vrows_c) - vb);
  stage_rows<TS>(V + vb, ldv, vr, vrows_c, col, Xs, lds);
  __syncthreads();
  rotate_rows<TS>(Xs, lds, vr, V + vb, ldv, col, sh.W);
}

// grid (pair, row chunk): apply the pair's unitary to this chunk's rows of X and V.
template <typename TS>
__global__ void __launch_bounds__(NT)
apply_kernel(TS* __restrict__ X, int64_t ldx, int mm, TS* __restrict__ V, int64_t ldv, int nn, int nb, int round,
             int x_rows_per_chunk, int v_rows_per_chunk, const double2* __restrict__ win, const int* __restrict__ rot) {
  typedef typename real_of<TS>::type RS;
  typedef typename cplx_of<RS>::type CS;
  __shared__ CS Wt[JC][JC + 1];
  __shared__ TS Xs[JR][JC + 1];
  __shared__ int col[JC];
  const int pair = blockIdx.x, chunk = blockIdx.y;
  if (!rot[pair]) return;
  pair_columns(round, pair, nb, nn, col);
  for (int e = threadIdx.x; e < NGRAM; e += NT) Wt[e / JC][e % JC] = ccast<CS>(win[(size_t)pair * NGRAM + e]);
  __syncthreads();
  const int xb = chunk * x_rows_per_chunk, vb = chunk * v_rows_per_chunk;
  apply_rows<TS>(X, ldx, xb, min(mm, xb + x_rows_per_chunk), col, Wt, Xs);
  if (V) apply_rows<TS>(V, ldv, vb, min(nn, vb + v_rows_per_chunk), col, Wt, Xs);
}

// ---------------------------------------------------------------------------
// FP32 storage, two launches per round
// ---------------------------------------------------------------------------

constexpr int SLAB = 256;  // rows per shared-memory slab of the Gram kernel
constexpr int NTG = 512;   // threads of the Gram kernel

// grid = pairs: one CTA of 512 threads forms the whole 16x16 Gram of its pair
// (rows streamed through a 256-row shared-memory slab -- each thread loads
// half a row, the next slab prefetched into registers during the current
// one's products; the 36 upper 2x2 tiles, 14 threads each on interleaved
// rows, FP32 accumulation, reduction in a fixed order), tests the pair, and
// runs the scaled pair solver.  The unitary goes to wout[pair], the decision
// to rot[pair].
__global__ void __launch_bounds__(NTG, 1)
pair_eig32_kernel(const float2* __restrict__ X, int64_t ldx, int mm, int nn, int nb, int round, double tol,
                  float tol_inner, double nu_rel2, const double* __restrict__ xnorm2, float2* __restrict__ wout,
                  int* __restrict__ rot, int* __restrict__ flags, int max_inner, unsigned long long* phase_ns) {
  __shared__ float2 slab[SLAB][JC + 1];
  __shared__ float2 gram[NGRAM];
  __shared__ pair_eig_scaled2 sh;
  __shared__ int col[JC];
  __shared__ int any_rot, bad, offmax_blk, offbig_blk;
  const int t = threadIdx.x, pair = blockIdx.x;
  unsigned long long tp = 0;
  auto phase = [&](int ph) {  // optional diagnostics: time per phase into phase_ns[ph - 1]
    if (phase_ns && t == 0) {
      unsigned long long tn;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(tn));
      if (ph > 0) atomicAdd(&phase_ns[ph - 1], tn - tp);
      tp = tn;
    }
  };
  phase(0);
  pair_columns(round, pair, nb, nn, col);
  if (t == 0) { any_rot = 0; bad = 0; offmax_blk = 0; offbig_blk = 0; sh.inner_rot = 0; }
  __syncthreads();
  // slab loads: thread t covers row (t & 255) of columns 8 (t >> 8) .. + 7
  const int lr = t & (SLAB - 1), ch = 8 * (t >> 8);
  const float2* cp[8];
#pragma unroll
  for (int c = 0; c < 8; c++) cp[c] = col[ch + c] >= 0 ? X + ldx * col[ch + c] : nullptr;
  float2 pf[8];
#pragma unroll
  for (int c = 0; c < 8; c++) pf[c] = (cp[c] && lr < mm) ? cp[c][lr] : make_float2(0.f, 0.f);
  // 36 upper 2x2 tiles x 14 row groups = 504 threads; group g takes rows
  // g, g + 14, ... of each slab
  constexpr int NGRP = 14;
  const int tile = t / NGRP, g = t - NGRP * (t / NGRP);
  const bool act = t < 36 * NGRP;
  int bi = 0, rem = act ? tile : 0;
  while (rem >= 8 - bi) { rem -= 8 - bi; bi++; }
  const int bj = bi + rem;
  float2 a00 = make_float2(0.f, 0.f), a01 = a00, a10 = a00, a11 = a00;
  for (int r0 = 0; r0 < mm; r0 += SLAB) {
#pragma unroll
    for (int c = 0; c < 8; c++) slab[lr][ch + c] = pf[c];
    __syncthreads();
    const int rn = r0 + SLAB + lr;
#pragma unroll
    for (int c = 0; c < 8; c++) pf[c] = (cp[c] && rn < mm) ? cp[c][rn] : make_float2(0.f, 0.f);
    if (act) {
#pragma unroll 4
      for (int rr = g; rr < SLAB; rr += NGRP) {
        const float2 p0 = slab[rr][2 * bi], p1 = slab[rr][2 * bi + 1], q0 = slab[rr][2 * bj], q1 = slab[rr][2 * bj + 1];
        cfma_conj(a00, p0, q0);
        cfma_conj(a01, p0, q1);
        cfma_conj(a10, p1, q0);
        cfma_conj(a11, p1, q1);
      }
    }
    __syncthreads();
  }
  phase(1);  // 0: Gram products
  // reduce the row groups in a fixed order (partials in the slab buffer)
  float2* red = &slab[0][0];
  if (act) {
    red[(g * 36 + tile) * 4 + 0] = a00;
    red[(g * 36 + tile) * 4 + 1] = a01;
    red[(g * 36 + tile) * 4 + 2] = a10;
    red[(g * 36 + tile) * 4 + 3] = a11;
  }
  __syncthreads();
  if (t < 144) {
    const int tl = t >> 2, q = t & 3;
    float2 v = red[tl * 4 + q];
    for (int gg = 1; gg < NGRP; gg++) v = cadd(v, red[(gg * 36 + tl) * 4 + q]);
    int ti = 0, tr = tl;
    while (tr >= 8 - ti) { tr -= 8 - ti; ti++; }
    const int tj = ti + tr;
    const int r = 2 * ti + (q >> 1), c = 2 * tj + (q & 1);
    if (ti != tj || r <= c) {
      gram[r * JC + c] = v;
      gram[c * JC + r] = cconj(v);
    }
  }
  __syncthreads();
  // scaled Gram, diagonal, test
  const double nu2 = nu_rel2 * (*xnorm2);
  const bool owner = t < NGRAM;
  const int i = (t / JC) & 15, j = t % JC;
  if (owner) {
    const float2 v = gram[t];
    if (!isfinite(v.x) || !isfinite(v.y)) bad = 1;
    if (i == j) { sh.d[0][i] = v.x; sh.d0[i] = v.x; }
  }
  __syncthreads();
  if (owner) {
    const float di = sh.d[0][i], dj = sh.d[0][j];
    float2 v = make_float2(0.f, 0.f);
    if (i != j && di > nu2 && dj > nu2) v = cscale(gram[t], (float)(1.0 / sqrt((double)di * (double)dj)));
    sh.G[0][i][j] = v;
    sh.W[0][i][j] = make_float2(i == j ? 1.f : 0.f, 0.f);
  }
  __syncthreads();
  if (bad) {
    if (t == 0) { atomicOr(&flags[QT_FLAG_NONFINITE], 1); rot[pair] = 0; }
    return;
  }
  {
    float relmax = 0.f, relbig = 0.f;
    const double big2 = 1e-6 * (*xnorm2);
    if (owner && i < j && col[i] >= 0 && col[j] >= 0 && sh.d[0][i] > nu2 && sh.d[0][j] > nu2) {
      const float rel = fminf(sqrtf(cabs2(sh.G[0][i][j])), 1.f);
      if (rel > tol) {
        any_rot = 1;
        relmax = rel;
        if (sh.d[0][i] > big2 && sh.d[0][j] > big2) relbig = rel;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      relmax = fmaxf(relmax, __shfl_xor_sync(0xffffffffu, relmax, o));
      relbig = fmaxf(relbig, __shfl_xor_sync(0xffffffffu, relbig, o));
    }
    if ((t & 31) == 0 && relmax > 0.f) atomicMax(&offmax_blk, __float_as_int(relmax));
    if ((t & 31) == 0 && relbig > 0.f) atomicMax(&offbig_blk, __float_as_int(relbig));
  }
  __syncthreads();
  if (t == 0) {
    rot[pair] = any_rot;
    if (offmax_blk > 0) atomicMax(&flags[QT_FLAG_OFFMAX], offmax_blk);
    if (offbig_blk > 0) atomicMax(&flags[QT_FLAG_OFFBIG], offbig_blk);
    if (any_rot) atomicAdd(&flags[QT_FLAG_ROTATED], 1);
  }
  phase(2);  // 1: reduction, scaled Gram, test
  if (!any_rot) return;
  int buf = 0;
  const int inner = diagonalise_scaled2(sh, col, tol_inner, (float)nu2, max_inner, &buf);
  if (t == 0) atomicAdd(&flags[QT_FLAG_INNER], inner);
  if (owner) wout[(size_t)pair * NGRAM + t] = sh.W[buf][i][j];
  phase(3);  // 2: pair solver
}

// grid (pair, row chunk): rotate this chunk's rows of X (and of V) by the
// pair's unitary.  One row per thread: its 16 values are loaded together
// (independent, coalesced across the warp), multiplied by W from shared
// memory (two entries per 16-byte broadcast load) and stored; no staging,
// no barriers after W is loaded.
__global__ void __launch_bounds__(NT, 3)
pair_apply32_kernel(float2* __restrict__ X, int64_t ldx, int mm, float2* __restrict__ V, int64_t ldv, int nn, int nb,
                    int round, int x_rows_per_chunk, int v_rows_per_chunk, const float2* __restrict__ win,
                    const int* __restrict__ rot) {
  __shared__ __align__(16) float2 Wt[JC][JC];
  __shared__ int col[JC];
  const int pair = blockIdx.x, chunk = blockIdx.y;
  if (!rot[pair]) return;
  pair_columns(round, pair, nb, nn, col);
  Wt[threadIdx.x / JC][threadIdx.x % JC] = win[(size_t)pair * NGRAM + threadIdx.x];
  __syncthreads();
  int cidx[JC];
#pragma unroll
  for (int c = 0; c < JC; c++) cidx[c] = col[c];
  for (int pass = 0; pass < 2; pass++) {
    float2* M = pass == 0 ? X : V;
    if (M == nullptr) break;
    const int64_t ld = pass == 0 ? ldx : ldv;
    const int per = pass == 0 ? x_rows_per_chunk : v_rows_per_chunk;
    const int lim = pass == 0 ? mm : nn;
    const int e = min(lim, chunk * per + per);
    for (int r = chunk * per + threadIdx.x; r < e; r += NT) {
      float2 x[JC];
#pragma unroll
      for (int k = 0; k < JC; k++) x[k] = cidx[k] >= 0 ? M[r + ld * cidx[k]] : make_float2(0.f, 0.f);
      float2 acc[JC];
#pragma unroll
      for (int c = 0; c < JC; c++) acc[c] = make_float2(0.f, 0.f);
      // keep the 256 W entries in shared memory (re-read per row) rather than
      // letting them be hoisted into registers across the row loop
      asm volatile("" ::: "memory");
#pragma unroll
      for (int k = 0; k < JC; k++) {
#pragma unroll
        for (int c = 0; c < JC; c += 2) {
          const float4 w = *reinterpret_cast<const float4*>(&Wt[k][c]);
          cfma(acc[c], x[k], make_float2(w.x, w.y));
          cfma(acc[c + 1], x[k], make_float2(w.z, w.w));
        }
      }
#pragma unroll
      for (int c = 0; c < JC; c++)
        if (cidx[c] >= 0) M[r + ld * cidx[c]] = acc[c];
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 storage: one cooperative launch per sweep
// ---------------------------------------------------------------------------
//
// CTA q owns table q of every round.  Round g (counted over the whole
// iteration) rebuilds its two blocks from the previous round's data and
// unitaries: a block whose round g-1 pair rotated becomes that pair's 16
// columns times the matching 16x8 block of its unitary, otherwise it is
// copied.  The rebuilt columns go to the other buffer of a ping-pong pair
// (round g reads buffer (g-1)&1 and writes buffer g&1), and on their way
// through shared memory they feed the Gram products, so a round reads and
// writes every column once and needs no separate rotation pass.  Rounds are
// chained per CTA through done[q] (the last round CTA q finished): round g
// waits for the round g-1 CTAs whose output it reads (read after write) and
// for those that read what it overwrites -- the previous contents of its
// destination columns and of its unitary slot (write after read).  Every
// wait is bounded; a wait that gives up sets QT_FLAG_ABORT, which ends the
// other CTAs' waits too.  The pending unitaries of the last round are applied
// in place by pair_apply32_kernel after the last sweep.
//
// With halves = 2 each pair is served by two CTAs, CTA 2q + h holding rows
// [row_lo(h), row_hi(h)) of the pair's columns (and the matching rows of V;
// both splits at a multiple of 32 rows, clamped to the matrix, so a V of
// fewer than 32 rows belongs to half 0 alone).
// A row half reads and writes only its own rows, so each half runs the round
// protocol above on its own copies of the round flags, unitaries and rotate
// decisions (done, wbuf, rotbuf offset by h); the two halves of a pair meet
// once per round: each publishes its partial Gram (the 160 upper-tile entries
// of its rows) in gx and its round in xflag, waits (bounded) for the other's,
// and both add the two partials in the same order.  Both then run the same
// pair solver on the same Gram and reach the same unitary, bit for bit.

constexpr int PS_SLAB = 256;                 // rows per slab
constexpr int PS_LDS = JC + 2;               // slab row stride in float2 (16-byte aligned rows)
constexpr int PS_TILES = 10;                 // upper 4x4 tiles of the 16x16 Gram
constexpr int PS_TE = 16;                    // entries per tile
constexpr int PS_NGRP = NTG / PS_TILES;      // 51 row groups per tile
constexpr size_t PS_SMEM = 2 * PS_SLAB * PS_LDS * sizeof(float2);  // double-buffered slab, 73,728 bytes
constexpr int PS_SPIN = 1 << 23;             // polls of a round wait before it gives up
static_assert(PS_TILES * PS_NGRP * PS_TE <= 2 * PS_SLAB * PS_LDS, "Gram partials reuse the slab buffer");

// tile -> (row quad ti, column quad tj), ti <= tj, ordered by ti
__device__ inline void ps_tile(int tile, int& ti, int& tj) {
  ti = 0;
  int rem = tile;
  while (rem >= 4 - ti) { rem -= 4 - ti; ti++; }
  tj = ti + rem;
}

// table q and side (0: first block of the pair, 1: second) of block `blk` in
// round `round` of the circle tournament over n players
__device__ inline void pair_of(int round, int blk, int n, int& q, int& side) {
  if (blk == n - 1) { q = 0; side = 1; return; }
  const int rr = round % (n - 1);
  if (blk == rr) { q = 0; side = 0; return; }
  const int d = (blk - rr + (n - 1)) % (n - 1);
  int partner;
  if (d <= n / 2 - 1) { q = d; partner = (rr - q + (n - 1)) % (n - 1); }
  else { q = n - 1 - d; partner = (rr + q) % (n - 1); }
  side = blk > partner ? 1 : 0;
}

__device__ inline int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

struct sweep_solver {
  float d[2][JC];
  float d0[JC];
  float2 G[2][JC][JC + 1];
  float2 W[2][JC][JC + 1];
};

// partner of index y in inner round ir of the circle tournament over the 16
// columns of a pair (the pairing of tournament(ir, ., 16)): 15 meets ir, the
// others meet 2 ir - y (mod 15).  (Pairing the two blocks' columns first and
// each block's own after converged in more outer sweeps.)
__device__ inline int inner_partner(int ir, int y) {
  if (y == JC - 1) return ir;
  if (y == ir) return JC - 1;
  return (2 * ir - y + (JC - 1)) % (JC - 1);
}

// named barrier of the 256 solver threads (warps 0-7)
__device__ inline void solver_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// The scaled pair solver, run by warps 0-7 alone (the caller's other warps
// skip it and wait at its next block barrier): thread (x, y) computes the
// rotation of y's pair itself (the two half-warps compute the same 16,
// bit-identically) and takes x's from lane x by shuffle, then updates
// Ghat[x][y] and Wt[x][y] into the other buffer -- one named barrier per
// inner round.  An inner round in which no pair needs a rotation is skipped
// by every warp alike (a warp vote over the same 16 decisions).  Same
// iteration as diagonalise_scaled2; the rotation is evaluated with the
// special-function unit's square roots and reciprocals (a few ulps: the
// rotation stays unitary to FP32 rounding, and the one-sided iteration
// re-measures every pair from the data in the next round anyway).
__device__ int diagonalise_lanes(sweep_solver& sh, const int* col, float tol_inner, float nu2, int max_inner,
                                 int* buf_out) {
  const int t = threadIdx.x, x = (t >> 4) & 15, y = t & 15;
  if (t >= NGRAM) return 0;  // warps 8-15
  const float tol2 = tol_inner * tol_inner;
  int cur = 0, sweep = 0;
  for (; sweep < max_inner; sweep++) {
    bool rotated_any = false;
    for (int ir = 0; ir < JC - 1; ir++) {
      const int yp = inner_partner(ir, y), xp = inner_partner(ir, x);
      const int p = min(y, yp), q = max(y, yp);
      const float a = sh.d[cur][p], b = sh.d[cur][q];
      const float2 gs = sh.G[cur][p][q];
      const float ags2 = gs.x * gs.x + gs.y * gs.y;
      const bool rotp = col[p] >= 0 && col[q] >= 0 && a > nu2 && b > nu2 && ags2 > tol2;
      if (!__any_sync(0xffffffffu, rotp)) continue;  // the same vote in every solver warp
      rotated_any = true;
      float2 jpp = make_float2(1.f, 0.f), jqp = make_float2(0.f, 0.f), jpq = jqp, jqq = jpp;
      float a2 = a, b2 = b;
      if (rotp) {
        const float ria = rsqrtf(a), rib = rsqrtf(b), rags = rsqrtf(ags2);
        const float sqa = a * ria, sqb = b * rib;
        const float ag = ags2 * rags * sqa * sqb;  // |gamma|
        const float zeta = __fdividef(b - a, 2.f * ag);
        const float z2 = fmaf(zeta, zeta, 1.f);
        const float r1 = z2 * rsqrtf(z2);
        const float tt = copysignf(__fdividef(1.f, fabsf(zeta) + r1), zeta);
        const float c = rsqrtf(fmaf(tt, tt, 1.f)), sn = c * tt;
        const float2 e = make_float2(gs.x * rags, gs.y * rags);
        a2 = fmaxf(fmaf(-tt, ag, a), nu2);  // a column driven to the noise level is frozen
        b2 = fmaf(tt, ag, b);
        const float ia2 = rsqrtf(a2), ib2 = rsqrtf(b2);
        const float fa = sqa * ia2, fb = sqb * ib2, fab = sqb * ia2, fba = sqa * ib2;
        jpp = make_float2(c * fa, 0.f);
        jqp = make_float2(-sn * e.x * fab, sn * e.y * fab);  // -s conj(e) sqrt(b/a')
        jpq = make_float2(sn * e.x * fba, sn * e.y * fba);   //  s e sqrt(a/b')
        jqq = make_float2(c * fb, 0.f);
      }
      // column y of Jt: rows y and y'
      const bool low = y == p;
      const float2 jyy = low ? jpp : jqq, jpy = low ? jqp : jpq;
      // column x of Jt from lane x (which holds y == x)
      float2 jxx, jpx;
      jxx.x = __shfl_sync(0xffffffffu, jyy.x, x);
      jxx.y = __shfl_sync(0xffffffffu, jyy.y, x);
      jpx.x = __shfl_sync(0xffffffffu, jpy.x, x);
      jpx.y = __shfl_sync(0xffffffffu, jpy.y, x);
      if (x == y) sh.d[cur ^ 1][y] = low ? a2 : b2;
      float2 gnew = make_float2(0.f, 0.f);
      if (xp == y && x != y) {
        const bool rotated = jxx.x != 1.f || jxx.y != 0.f || jpx.x != 0.f || jpx.y != 0.f;
        if (!rotated) gnew = sh.G[cur][x][y];
      } else if (x != y) {
        const float2 g_xy = sh.G[cur][x][y], g_xq = sh.G[cur][x][yp];
        const float2 g_py = sh.G[cur][xp][y], g_pq = sh.G[cur][xp][yp];
        const float2 hx = cadd(cmul(g_xy, jyy), cmul(g_xq, jpy));
        const float2 hp = cadd(cmul(g_py, jyy), cmul(g_pq, jpy));
        gnew = cadd(cmul(cconj(jxx), hx), cmul(cconj(jpx), hp));
      }
      sh.G[cur ^ 1][x][y] = gnew;
      const float2 w_xy = sh.W[cur][x][y], w_xq = sh.W[cur][x][yp];
      sh.W[cur ^ 1][x][y] = cadd(cmul(w_xy, jyy), cmul(w_xq, jpy));
      cur ^= 1;
      solver_sync();
    }
    if (!rotated_any) break;  // every solver warp took the same votes
  }
  {
    const float d0 = sh.d0[x];
    sh.W[cur][x][y] = d0 > 0.f ? cscale(sh.W[cur][x][y], sqrtf(sh.d[cur][y]) * rsqrtf(d0))
                               : make_float2(x == y ? 1.f : 0.f, 0.f);
  }
  *buf_out = cur;
  return sweep + (sweep < max_inner ? 1 : 0);
}

// One sweep (rounds g0 .. g0 + nb - 2).  xb[0] is X itself, xb[1] a scratch
// copy of its shape (likewise vb for V); wbuf holds 2 x pairs unitaries,
// rotbuf 2 x pairs decisions, done[pairs] the completed round of each CTA.
__global__ void __launch_bounds__(NTG, 1)
jacobi_sweep32_kernel(float2* __restrict__ xb0, float2* __restrict__ xb1, int64_t ldx, int mm,
                      float2* __restrict__ vb0, float2* __restrict__ vb1, int64_t ldv, int nn, int nb, int g0,
                      int has_prev, double tol, float tol_inner, double nu_rel2, const double* __restrict__ xnorm2,
                      float2* __restrict__ wbuf, int* __restrict__ rotbuf, int* __restrict__ done,
                      int* __restrict__ flags, int max_inner, float keep2, float* __restrict__ dnorm,
                      unsigned long long* phase_ns, int spin, int stall, int halves, int row_mid, int vrow_mid,
                      float2* __restrict__ gx, int* __restrict__ xflag) {
  extern __shared__ __align__(16) float2 ps_slab[];  // [2][PS_SLAB][PS_LDS]
  __shared__ __align__(16) float2 wsub[2][JC][JW];    // 16x8 unitary blocks that rebuild the two blocks
  __shared__ float2 psum[3][PS_TILES * PS_TE];
  __shared__ float2 gram[NGRAM];
  __shared__ sweep_solver sh;
  __shared__ int col[JC], scol[2][JC], srcq[2], sside[2], srot[2];
  __shared__ int any_rot, bad, offmax_blk, offbig_blk, offkept_blk;
  const int H = halves, t = threadIdx.x, q = blockIdx.x / H, hf = blockIdx.x % H, pairs = gridDim.x / H,
            R = nb - 1;
  // this CTA's rows of X and V, and its half's copies of the round state
  const int row_lo = hf ? row_mid : 0, row_hi = (hf || H == 1) ? mm : row_mid;
  const int vrow_lo = hf ? vrow_mid : 0, vrow_hi = (hf || H == 1) ? nn : vrow_mid;
  done += (size_t)hf * pairs;
  wbuf += (size_t)hf * 2 * pairs * NGRAM;
  rotbuf += (size_t)hf * 2 * pairs;
  if (hf) { phase_ns = nullptr; dnorm = nullptr; }  // half 0 reports for the pair
  __shared__ unsigned long long tp;
  auto phase = [&](int ph) {  // optional diagnostics: time per phase into phase_ns[ph - 1]
    if (phase_ns && t == 0) {
      unsigned long long tn;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(tn));
      if (ph > 0) atomicAdd(&phase_ns[ph - 1], tn - tp);
      tp = tn;
    }
  };
  const float nu2 = (float)(nu_rel2 * (*xnorm2));
  const float big2 = (float)(1e-6 * (*xnorm2));
  const float tolf = (float)tol;
  // slab rows: thread t rebuilds row (t & 255) of block (t >> 8)
  const int lr = t & (PS_SLAB - 1), h = t >> 8;
  // Gram products: rows 4 ti .. 4 ti + 3 against columns 4 tj .. 4 tj + 3, row group grp
  const int tile = t / PS_NGRP, grp = t - PS_NGRP * (t / PS_NGRP);
  const bool act = tile < PS_TILES;
  int ti = 0, tj = 0;
  if (act) ps_tile(tile, ti, tj);
  const int nslab = (row_hi - row_lo + PS_SLAB - 1) / PS_SLAB;
  for (int r = 0; r < R; r++) {
    const int g = g0 + r;
    const bool prev = r > 0 || has_prev;
    const int rp = r > 0 ? r - 1 : R - 1;  // round (within its sweep) of g - 1
    const int rpp = (r + 2 * R - 2) % R;   // ... of g - 2
    phase(0);
    int bi, bj;
    tournament(r, q, nb, bi, bj);
    // ---- wait for the round g - 1 CTAs this round depends on
    int gave_up = 0;
    if (stall && q == 0 && t == 0 && r == 0) {
      // test hook (QT_JACOBI_STALL_TEST): a bounded wait on a status word that
      // nothing sets, which must end in QT_ETIMEOUT with the context usable
      int it = 0;
      for (; it < spin; it++) {
        if (ld_acquire_gpu(flags + QT_FLAG_STALL) != 0) break;
        if (*(volatile int*)(flags + QT_FLAG_ABORT)) { it = spin; break; }
        __nanosleep(64);
      }
      if (it >= spin) { gave_up = 1; atomicExch(flags + QT_FLAG_ABORT, 1); }
    }
    if (prev && t < 6) {
      int target = -1, qq, s;
      if (t < 2) {  // read after write: the pairs that held our blocks in round g - 1
        pair_of(rp, t == 0 ? bi : bj, nb, qq, s);
        target = qq;
      } else if (g >= 2 && t < 4) {  // write after read: readers of our blocks' round g - 2 columns
        const int blk = t == 2 ? bi : bj;
        int a2, b2;
        pair_of(rpp, blk, nb, qq, s);
        tournament(rpp, qq, nb, a2, b2);
        pair_of(rp, a2 == blk ? b2 : a2, nb, qq, s);
        target = qq;
      } else if (g >= 2) {  // write after read: readers of unitary slot q of round g - 2
        int a2, b2;
        tournament(rpp, q, nb, a2, b2);
        pair_of(rp, t == 4 ? a2 : b2, nb, qq, s);
        target = qq;
      }
      if (target >= 0) {
        int it = 0;
        for (; it < spin; it++) {
          if (ld_acquire_gpu(done + target) >= g - 1) break;
          if ((it & 7) == 7 && *(volatile int*)(flags + QT_FLAG_ABORT)) { it = spin; break; }
          __nanosleep(64);
        }
        if (it >= spin) { gave_up = 1; atomicExch(flags + QT_FLAG_ABORT, 1); }
      }
    }
    if (__syncthreads_or(gave_up)) return;
    phase(1);  // 0: waits
    pair_columns(r, q, nb, nn, col);
    if (t == 0) { any_rot = 0; bad = 0; offmax_blk = 0; offbig_blk = 0; offkept_blk = 0; }
    if (prev && t < 2) {
      int qq, s;
      pair_of(rp, t == 0 ? bi : bj, nb, qq, s);
      srcq[t] = qq;
      sside[t] = s;
      srot[t] = __ldcg(rotbuf + (size_t)((g - 1) & 1) * pairs + qq);
    }
    if (!prev && t < 2) srot[t] = 0;
    __syncthreads();
    if (t < 2 * JC) {  // source columns of each half: the round g - 1 pair, or the block itself
      const int hh = t / JC, c = t % JC;
      int gc;
      if (srot[hh]) {
        int a2, b2;
        tournament(rp, srcq[hh], nb, a2, b2);
        gc = c < JW ? a2 * JW + c : b2 * JW + (c - JW);
      } else {
        gc = c < JW ? (hh == 0 ? bi : bj) * JW + c : -1;
      }
      scol[hh][c] = gc < nn ? gc : -1;
    }
    if (t < 2 * JC * JW) {
      const int hh = t / (JC * JW), k = (t / JW) % JC, c = t % JW;
      if (srot[hh])
        wsub[hh][k][c] = __ldcg(wbuf + (size_t)((g - 1) & 1) * pairs * NGRAM + (size_t)srcq[hh] * NGRAM + k * JC +
                                sside[hh] * JW + c);
    }
    __syncthreads();
    const float2* __restrict__ src = prev ? (((g - 1) & 1) ? xb1 : xb0) : ((g & 1) ? xb1 : xb0);
    float2* __restrict__ dst = (g & 1) ? xb1 : xb0;
    const bool hrot = srot[h] != 0;
    // column indices stay in shared memory (warp-uniform broadcast reads)
    const int* sc = scol[h];
    const int* oc = col + h * JW;
    // ---- rebuild the rows slab by slab; Gram products on the previous slab meanwhile
    float2 xr[JC];
    auto load_row = [&](const float2* __restrict__ M, int64_t ld, int lim, int rr) {
      if (hrot) {
#pragma unroll
        for (int k = 0; k < JC; k++)
          xr[k] = (sc[k] >= 0 && rr < lim) ? __ldcg(M + rr + ld * sc[k]) : make_float2(0.f, 0.f);
      } else {
#pragma unroll
        for (int k = 0; k < JW; k++)
          xr[k] = (sc[k] >= 0 && rr < lim) ? __ldcg(M + rr + ld * sc[k]) : make_float2(0.f, 0.f);
      }
    };
    auto rebuild = [&](float2* out) {
      if (hrot) {
        // two partial sums per output (the real and the imaginary part of
        // x_k each feed their own): four independent FMAs per complex
        // product instead of two dependent pairs
        float2 ob[JW];
#pragma unroll
        for (int c = 0; c < JW; c++) { out[c] = make_float2(0.f, 0.f); ob[c] = out[c]; }
        asm volatile("" ::: "memory");  // keep wsub in shared memory
#pragma unroll
        for (int k = 0; k < JC; k++) {
#pragma unroll
          for (int c = 0; c < JW; c += 2) {
            const float4 w = *reinterpret_cast<const float4*>(&wsub[h][k][c]);
            out[c].x = fmaf(xr[k].x, w.x, out[c].x);
            out[c].y = fmaf(xr[k].x, w.y, out[c].y);
            ob[c].x = fmaf(-xr[k].y, w.y, ob[c].x);
            ob[c].y = fmaf(xr[k].y, w.x, ob[c].y);
            out[c + 1].x = fmaf(xr[k].x, w.z, out[c + 1].x);
            out[c + 1].y = fmaf(xr[k].x, w.w, out[c + 1].y);
            ob[c + 1].x = fmaf(-xr[k].y, w.w, ob[c + 1].x);
            ob[c + 1].y = fmaf(xr[k].y, w.z, ob[c + 1].y);
          }
        }
#pragma unroll
        for (int c = 0; c < JW; c++) out[c] = cadd(out[c], ob[c]);
      } else {
#pragma unroll
        for (int c = 0; c < JW; c++) out[c] = xr[c];
      }
    };
    auto build_slab = [&](int s) {
      const int rr = row_lo + s * PS_SLAB + lr;
      float2 o[JW];
      rebuild(o);
      if (prev && rr < row_hi) {
#pragma unroll
        for (int c = 0; c < JW; c++)
          if (oc[c] >= 0) __stcg(dst + rr + ldx * oc[c], o[c]);
      }
      float4* sp = reinterpret_cast<float4*>(ps_slab + ((size_t)(s & 1) * PS_SLAB + lr) * PS_LDS + h * JW);
#pragma unroll
      for (int c = 0; c < JW; c += 2) sp[c / 2] = make_float4(o[c].x, o[c].y, o[c + 1].x, o[c + 1].y);
    };
    float2 acc[PS_TE];
#pragma unroll
    for (int e = 0; e < PS_TE; e++) acc[e] = make_float2(0.f, 0.f);
    load_row(src, ldx, row_hi, row_lo + lr);
    build_slab(0);
    __syncthreads();
    for (int s = 0; s < nslab; s++) {
      if (s + 1 < nslab) load_row(src, ldx, row_hi, row_lo + (s + 1) * PS_SLAB + lr);
      if (act) {
        const float2* base = ps_slab + (size_t)(s & 1) * PS_SLAB * PS_LDS;
        const int rows = min(PS_SLAB, row_hi - row_lo - s * PS_SLAB);
#pragma unroll 1
        for (int rr = grp; rr < rows; rr += PS_NGRP) {
          const float4* rowp = reinterpret_cast<const float4*>(base + (size_t)rr * PS_LDS);
          const float4 p01 = rowp[2 * ti], p23 = rowp[2 * ti + 1], q01 = rowp[2 * tj], q23 = rowp[2 * tj + 1];
          const float2 pv[4] = {make_float2(p01.x, p01.y), make_float2(p01.z, p01.w), make_float2(p23.x, p23.y),
                                make_float2(p23.z, p23.w)};
          const float2 qv[4] = {make_float2(q01.x, q01.y), make_float2(q01.z, q01.w), make_float2(q23.x, q23.y),
                                make_float2(q23.z, q23.w)};
#pragma unroll
          for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) cfma_conj(acc[a * 4 + b], pv[a], qv[b]);
        }
      }
      if (s + 1 < nslab) build_slab(s + 1);
      __syncthreads();
    }
    // ---- V rows (rotation only)
    if (prev && vb0) {
      const float2* __restrict__ vsrc = ((g - 1) & 1) ? vb1 : vb0;
      float2* __restrict__ vdst = (g & 1) ? vb1 : vb0;
      for (int rr = vrow_lo + lr; rr < vrow_hi; rr += PS_SLAB) {
        load_row(vsrc, ldv, vrow_hi, rr);
        float2 o[JW];
        rebuild(o);
#pragma unroll
        for (int c = 0; c < JW; c++)
          if (oc[c] >= 0) __stcg(vdst + rr + ldv * oc[c], o[c]);
      }
    }
    phase(2);  // 1: rebuild + Gram products
    // ---- reduce the row groups in a fixed order: three partial sums of 17
    // groups each, then their sum; the diagonal goes to the solver's D
    float2* red = ps_slab;
    if (act) {
#pragma unroll
      for (int e = 0; e < PS_TE; e++) red[(grp * PS_TILES + tile) * PS_TE + e] = acc[e];
    }
    __syncthreads();
    static_assert(PS_NGRP == 3 * 17, "three partial sums of 17 row groups");
    if (t < 3 * PS_TILES * PS_TE) {
      const int ent = t / 3, part = t % 3;
      const float2* rp0 = red + (size_t)(part * 17) * PS_TILES * PS_TE + ent;
      float2 v = rp0[0];
#pragma unroll
      for (int gg = 1; gg < 17; gg++) v = cadd(v, rp0[(size_t)gg * PS_TILES * PS_TE]);
      psum[part][ent] = v;
    }
    __syncthreads();
    float2 xv = make_float2(0.f, 0.f);
    if (t < PS_TILES * PS_TE) {
      xv = cadd(cadd(psum[0][t], psum[1][t]), psum[2][t]);
      if (H > 1) __stcg(gx + (((size_t)(g & 1) * pairs + q) * H + hf) * (PS_TILES * PS_TE) + t, xv);
    }
    if (H > 1) {
      // the two row halves of the pair exchange their partial Grams (bounded wait)
      __threadfence();
      __syncthreads();
      int gave = 0;
      if (t == 0) {
        st_release_gpu(xflag + (size_t)hf * pairs + q, g);
        int it = 0;
        for (; it < spin; it++) {
          if (ld_acquire_gpu(xflag + (size_t)(1 - hf) * pairs + q) >= g) break;
          if ((it & 7) == 7 && *(volatile int*)(flags + QT_FLAG_ABORT)) { it = spin; break; }
          __nanosleep(32);
        }
        if (it >= spin) { gave = 1; atomicExch(flags + QT_FLAG_ABORT, 1); }
      }
      if (__syncthreads_or(gave)) return;
      if (t < PS_TILES * PS_TE) {
        const float2 o = __ldcg(gx + (((size_t)(g & 1) * pairs + q) * H + (1 - hf)) * (PS_TILES * PS_TE) + t);
        xv = hf == 0 ? cadd(xv, o) : cadd(o, xv);  // (half 0) + (half 1) in both CTAs
      }
    }
    if (t < PS_TILES * PS_TE) {
      const float2 v = xv;
      int ai, aj;
      ps_tile(t / PS_TE, ai, aj);
      const int e = t % PS_TE;
      const int rw = 4 * ai + e / 4, cl = 4 * aj + e % 4;
      if (ai != aj || rw <= cl) {
        if (!isfinite(v.x) || !isfinite(v.y)) bad = 1;
        gram[rw * JC + cl] = v;
        gram[cl * JC + rw] = cconj(v);
        if (rw == cl) {
          sh.d[0][rw] = v.x;
          sh.d0[rw] = v.x;
          // the last round of the sweep reports every column's squared norm
          if (dnorm && r == R - 1 && col[rw] >= 0) dnorm[col[rw]] = v.x;
        }
      }
    }
    __syncthreads();
    // ---- scaled Gram, test
    const bool owner = t < NGRAM;
    const int i = (t / JC) & 15, j = t % JC;
    {
      float relmax = 0.f, relbig = 0.f, relkept = 0.f;
      if (owner) {
        const float di = sh.d[0][i], dj = sh.d[0][j];
        const bool live = i != j && di > nu2 && dj > nu2;
        const float2 v = live ? cscale(gram[t], rsqrtf(di) * rsqrtf(dj)) : make_float2(0.f, 0.f);
        sh.G[0][i][j] = v;
        sh.W[0][i][j] = make_float2(i == j ? 1.f : 0.f, 0.f);
        if (!bad && live && i < j && col[i] >= 0 && col[j] >= 0) {
          const float rel = fminf(sqrtf(cabs2(v)), 1.f);
          if (rel > tolf) {
            any_rot = 1;
            relmax = rel;
            if (di > big2 && dj > big2) relbig = rel;
            if (fmaxf(di, dj) > keep2) relkept = rel;
          }
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        relmax = fmaxf(relmax, __shfl_xor_sync(0xffffffffu, relmax, o));
        relbig = fmaxf(relbig, __shfl_xor_sync(0xffffffffu, relbig, o));
        relkept = fmaxf(relkept, __shfl_xor_sync(0xffffffffu, relkept, o));
      }
      if ((t & 31) == 0 && relmax > 0.f) atomicMax(&offmax_blk, __float_as_int(relmax));
      if ((t & 31) == 0 && relbig > 0.f) atomicMax(&offbig_blk, __float_as_int(relbig));
      if ((t & 31) == 0 && relkept > 0.f) atomicMax(&offkept_blk, __float_as_int(relkept));
    }
    __syncthreads();
    if (t == 0) {
      if (bad) atomicOr(&flags[QT_FLAG_NONFINITE], 1);
      __stcg(rotbuf + (size_t)(g & 1) * pairs + q, any_rot);
      if (hf == 0) {  // the pair's statistics, once
        if (offmax_blk > 0) atomicMax(&flags[QT_FLAG_OFFMAX], offmax_blk);
        if (offbig_blk > 0) atomicMax(&flags[QT_FLAG_OFFBIG], offbig_blk);
        if (offkept_blk > 0) atomicMax(&flags[QT_FLAG_OFFKEPT], offkept_blk);
        if (any_rot) atomicAdd(&flags[QT_FLAG_ROTATED], 1);
      }
    }
    phase(3);  // 2: reduction, scaled Gram, test
    if (any_rot) {
      int buf = 0;
      const int inner = diagonalise_lanes(sh, col, tol_inner, nu2, max_inner, &buf);
      if (t == 0 && hf == 0) atomicAdd(&flags[QT_FLAG_INNER], inner);
      // each solver thread stores the entry it finished itself
      if (owner) __stcg(wbuf + (size_t)(g & 1) * pairs * NGRAM + (size_t)q * NGRAM + t, sh.W[buf][i][j]);
    }
    phase(4);  // 3: pair solver
    // ---- publish round g
    __threadfence();
    __syncthreads();
    if (t == 0) st_release_gpu(done + q, g);
  }
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
  // double2 entries: partial Grams, ||X||_F^2, two round slots of one 16x16
  // unitary per pair, two round slots of the pairs' rotate flags
  return pairs * chunks * NGRAM + 1 + pairs * NGRAM + pairs;
}

// Cluster shape of the one-launch round: the smallest cluster (<= 8 CTAs)
// whose row slice of the 16 pair columns fits in FUSED_SMEM bytes of shared
// memory, widened while the grid would leave SMs idle.  0 = does not fit.
constexpr size_t FUSED_SMEM = 100 * 1024;
static int fused_shape(int64_t mm, int pairs, size_t elem, int* rows_c, int* lds, size_t* smem) {
  int csize = 0;
  for (int c = 1; c <= 8; c *= 2) {
    const int64_t rc = (mm + c - 1) / c;
    if ((size_t)(((rc + 15) / 16) * 16 + 1) * JC * elem <= FUSED_SMEM) { csize = c; break; }
  }
  if (csize == 0) return 0;
  while (csize < 8 && (int64_t)pairs * csize < 152 && (mm + 2 * csize - 1) / (2 * csize) >= 64) csize *= 2;
  // QT_JACOBI_CLUSTER=c (1, 2, 4 or 8) overrides the cluster size when the slice still fits
  if (const char* env = std::getenv("QT_JACOBI_CLUSTER")) {
    const int c = std::atoi(env);
    const int64_t rc = (mm + c - 1) / c;
    if ((c == 1 || c == 2 || c == 4 || c == 8) && (size_t)(((rc + 15) / 16) * 16 + 1) * JC * elem <= 200 * 1024)
      csize = c;
  }
  const int64_t rc = (mm + csize - 1) / csize;
  *rows_c = (int)rc;
  *lds = (int)(((rc + 15) / 16) * 16 + 1);  // odd multiple-of-16-plus-one stride: conflict-free Gram reads
  *smem = (size_t)(*lds) * JC * elem;
  return csize;
}

template <typename TS>
static int launch_pair_round(qt_handle* h, int csize, int pairs, size_t smem, TS* X, int64_t ldx, int mm, TS* V,
                             int64_t ldv, int nn, int nb, int round, int xrows_c, int vrows_c, int lds, double tol,
                             double tol_inner, double nu_rel2, const double* xnorm2, int max_inner,
                             unsigned long long* phase_ns) {
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)(pairs * csize));
  lc.blockDim = dim3(NT);
  lc.dynamicSmemBytes = smem;
  lc.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  if (h->prof) qt_prof_before(h, "pair_round_kernel<TS>");
  const cudaError_t e = cudaLaunchKernelEx(&lc, pair_round_kernel<TS>, X, ldx, mm, V, ldv, nn, nb, round, csize,
                                           xrows_c, vrows_c, lds, tol, tol_inner, nu_rel2, xnorm2, h->d_flags, max_inner,
                                           phase_ns);
  if (h->prof) qt_prof_after(h);
  h->launches++;
  if (e != cudaSuccess) return qt_fail(h, QT_ECUDA, std::string("launch pair_round_kernel: ") + cudaGetErrorString(e));
  return QT_OK;
}

// Whether one CTA per pair of jacobi_sweep32_kernel can be resident at once
// (the cooperative launch needs it).
static bool sweep32_fits(qt_handle* h, int pairs) {
  static int max_ctas = -1;
  if (max_ctas < 0) {
    int dev = 0, coop = 0, sms = 0, per_sm = 0;
    max_ctas = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        cudaFuncSetAttribute(jacobi_sweep32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PS_SMEM) ==
            cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_sweep32_kernel, NTG, PS_SMEM) == cudaSuccess)
      max_ctas = per_sm * sms;
    cudaGetLastError();
  }
  (void)h;
  return pairs <= max_ctas;
}

static int launch_sweep32(qt_handle* h, int pairs, float2* x0, float2* x1, int64_t ldx, int mm, float2* v0,
                          float2* v1, int64_t ldv, int nn, int nb, int g0, int has_prev, double tol, float tol_inner,
                          double nu_rel2, const double* xnorm2, float2* wbuf, int* rotbuf, int* done, int max_inner,
                          float keep2, float* dnorm, unsigned long long* phase_ns, int halves, float2* gx,
                          int* xflag) {
  // row split of the two halves of a pair: at a multiple of 32 rows, never
  // past the last row (a V of fewer than 32 rows belongs to half 0 alone)
  const int row_mid = std::min(((mm / 2 + 31) / 32) * 32, mm);
  const int vrow_mid = std::min(((nn / 2 + 31) / 32) * 32, nn);
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)(pairs * halves));
  lc.blockDim = dim3(NTG);
  lc.dynamicSmemBytes = PS_SMEM;
  lc.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  // QT_JACOBI_STALL_TEST=N (tests only): CTA 0 waits at most N polls on a
  // status word nothing sets, and every round wait is limited to N polls
  const char* stall_env = std::getenv("QT_JACOBI_STALL_TEST");
  const int stall_polls = stall_env ? std::atoi(stall_env) : 0;
  const int spin = stall_polls > 0 ? stall_polls : PS_SPIN;
  const int stall = stall_polls > 0 ? 1 : 0;
  if (h->prof) qt_prof_before(h, "jacobi_sweep32_kernel");
  const cudaError_t e = cudaLaunchKernelEx(&lc, jacobi_sweep32_kernel, x0, x1, ldx, mm, v0, v1, ldv, nn, nb, g0,
                                           has_prev, tol, tol_inner, nu_rel2, xnorm2, wbuf, rotbuf, done, h->d_flags,
                                           max_inner, keep2, dnorm, phase_ns, spin, stall, halves, row_mid, vrow_mid,
                                           gx, xflag);
  if (h->prof) qt_prof_after(h);
  h->launches++;
  if (e != cudaSuccess)
    return qt_fail(h, QT_ECUDA, std::string("launch jacobi_sweep32_kernel: ") + cudaGetErrorString(e));
  return QT_OK;
}

template <typename TS>
int qt_jacobi_svd_ws(qt_handle* h, TS* X, int64_t mm, int64_t nn, int64_t ldx, TS* V, int64_t ldv, double tol,
                     int max_sweeps, int* sweeps_out, double2* parts, double nu_rel_in, int keep_count) {
  typedef typename gram_of<TS>::type TG;
  if (mm < nn) return qt_fail(h, QT_EINVAL, "jacobi: needs rows >= columns");
  if (V) QT_TRY(qt_set_identity<TS>(h, V, nn, ldv));
  *sweeps_out = 0;
  if (nn <= 1) return QT_OK;
  int nb = 0, chunks = 1;
  qt_jacobi_layout(mm, nn, &nb, &chunks);
  const int pairs = nb / 2, rounds = nb - 1;
  const int xrows = (int)(((mm + chunks - 1) / chunks + JR - 1) / JR * JR);
  const int vrows = (int)(((nn + chunks - 1) / chunks + JR - 1) / JR * JR);
  const dim3 grid(pairs, chunks);
  // the last workspace entry holds ||X||_F^2 (rotation-invariant); the noise
  // floor nu (below) is relative to ||X||_F
  double* xnorm2 = reinterpret_cast<double*>(parts + (size_t)pairs * chunks * NGRAM);
  double2* wbuf = parts + (size_t)pairs * chunks * NGRAM + 1;
  int* rotf = reinterpret_cast<int*>(wbuf + (size_t)pairs * NGRAM);
  {
    // ||X||_F^2 over the nn columns (ldx may exceed mm)
    QT_CHECK_CUDA(h, cudaMemsetAsync(xnorm2, 0, sizeof(double), h->stream));
    QT_LAUNCH(h, frob_kernel<TS>, (unsigned)nn, 256, 0, X, ldx, (int)mm, xnorm2);
  }
  const bool fp32 = sizeof(typename real_of<TS>::type) == 4;
  const double u = fp32 ? 5.96e-8 : 1.11e-16;
  // Frozen-column threshold nu (relative to ||X||_F).  FP64: 4 sqrt(rows) u.
  // FP32 default: 4 u, so that the weight of the frozen columns stays below
  // the chosen mode's noise floor and the tail rule can resolve values near
  // it.  Columns between 4 u and sqrt(rows) u are rounding noise of FP32
  // products that keep rotating with O(1) cosines for tens of sweeps; callers
  // whose rank is decided far above them (a chi_max cap, a cutoff well above
  // the floor) pass nu_rel = sqrt(rows) u and save those sweeps.
  const double nu_rel = nu_rel_in > 0 ? nu_rel_in
                        : (fp32 ? 4.0 * u : 4.0 * std::sqrt((double)std::max<int64_t>(mm, 16)) * u);
  const double nu_rel2 = nu_rel * nu_rel;
  // Round implementation (cfg.jacobi_kernel): FP32 storage by default runs
  // two launches per round (Gram + pair solver, then the rotation); 2 asks
  // for the one-launch cluster round, 1 for the three-kernel round.  FP64
  // storage uses the one-launch round where a pair's rows fit a cluster's
  // shared memory.
  const int jk = h->cfg.jacobi_kernel;
  const bool sweep_kernel = fp32 && jk == 0 && sweep32_fits(h, pairs);
  const bool two_launch = fp32 && (jk == 3 || (jk == 0 && !sweep_kernel));
  int xrows_c = 0, lds = 0;
  size_t smem = 0;
  const int csize = (jk == 1 || two_launch || sweep_kernel) ? 0 : fused_shape(mm, pairs, sizeof(TS), &xrows_c, &lds, &smem);
  // two-launch shape: one row per rotation thread, about eight CTAs per SM
  int achunks = std::max(1, std::min<int>((8 * 152 + pairs - 1) / pairs, (int)((mm + NT - 1) / NT)));
  const int axrows = (int)(((mm + achunks - 1) / achunks + 31) / 32 * 32);
  const int avrows = (int)(((nn + achunks - 1) / achunks + 31) / 32 * 32);
  const int vrows_c = csize ? (int)((nn + csize - 1) / csize) : 0;
  // the inner eigen-solve is driven well below the outer threshold so that the
  // rounding of the applied rotation cannot leave the pair just above `tol`
  const double tol_inner = fp32 ? tol / 16.0 : std::min(tol, 1e-14);
  if (csize)
    QT_CHECK_CUDA(h, cudaFuncSetAttribute(pair_round_kernel<TS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
  // QT_JACOBI_TRACE=1 in the environment prints one line per sweep to stderr;
  // QT_JACOBI_PHASES=1 adds the average time per phase of the one-launch
  // rounds at the end (CTA 0 of each cluster / the others); a handle without
  // a pool (the allocation-free entry point's) allocates nothing and skips them
  static const bool trace = std::getenv("QT_JACOBI_TRACE") != nullptr;
  static const bool phases = std::getenv("QT_JACOBI_PHASES") != nullptr;
  unsigned long long* phase_ns = nullptr;
  qt_scratch pscratch(h);
  if (phases && h->pool && (csize || two_launch || sweep_kernel)) {
    QT_TRY(pscratch.get(&phase_ns, 16));
    QT_CHECK_CUDA(h, cudaMemsetAsync(phase_ns, 0, 16 * sizeof(unsigned long long), h->stream));
  }
  // sweep kernel: ping-pong copies of X and V, the round counter, and
  // whether the last round's unitaries are still to be applied
  TS* X1 = nullptr;
  TS* V1 = nullptr;
  int* done = reinterpret_cast<int*>(parts);
  int gcount = 0;
  bool pending = false;
  // kept-set convergence (keep_count > 0, sweep kernel): the last round of
  // each sweep reports the squared column norms; a column within a factor
  // keep_margin of the keep_count-th largest norm counts as kept
  static const double keep_margin =
      std::getenv("QT_JACOBI_KEEP_MARGIN") ? std::atof(std::getenv("QT_JACOBI_KEEP_MARGIN")) : 0.25;
  static const bool keep_stop = !std::getenv("QT_JACOBI_KEEP_STOP") || std::atoi(std::getenv("QT_JACOBI_KEEP_STOP"));
  const bool keep_track = sweep_kernel && keep_count > 0 && keep_count < nn;
  float* dnorm = nullptr;
  std::vector<float> hnorm;
  float keep2 = 0.f;
  double prev_tail2 = -1.0, prev_change = -1.0;
  static const double keep_tol =
      std::getenv("QT_JACOBI_KEEP_TOL") ? std::atof(std::getenv("QT_JACOBI_KEEP_TOL")) : 1e-3;
  // Two CTAs per pair (each holding half of the rows) when the doubled grid
  // is still resident and each half has rows to work on; QT_JACOBI_HALVES=1
  // keeps one CTA per pair.  The halves run on their own copies of the round
  // flags, unitaries and rotate decisions, and exchange partial Grams.
  const int halves_env = std::getenv("QT_JACOBI_HALVES") ? std::atoi(std::getenv("QT_JACOBI_HALVES")) : 2;
  const int halves = (sweep_kernel && halves_env == 2 && mm >= 512 && sweep32_fits(h, 2 * pairs)) ? 2 : 1;
  float2* gx = nullptr;
  int* xflag = nullptr;
  if (sweep_kernel && halves == 2) {
    double2* wb2;
    int *rf2, *dn2;
    QT_TRY(pscratch.get(&wb2, (size_t)2 * pairs * NGRAM));  // 2 halves x 2 round slots x pairs x NGRAM float2
    QT_TRY(pscratch.get(&rf2, (size_t)4 * pairs));
    QT_TRY(pscratch.get(&dn2, (size_t)2 * pairs));
    QT_TRY(pscratch.get(&xflag, (size_t)2 * pairs));
    QT_TRY(pscratch.get(&gx, (size_t)2 * pairs * 2 * 160));
    wbuf = wb2;
    rotf = rf2;
    done = dn2;
    QT_CHECK_CUDA(h, cudaMemsetAsync(xflag, 0xff, sizeof(int) * 2 * pairs, h->stream));
  }
  if (sweep_kernel) {
    QT_TRY(pscratch.get(&X1, (size_t)ldx * nn));
    if (V) QT_TRY(pscratch.get(&V1, (size_t)ldv * nn));
    QT_CHECK_CUDA(h, cudaMemsetAsync(done, 0xff, sizeof(int) * pairs * halves, h->stream));
    if (keep_track) {
      QT_TRY(pscratch.get(&dnorm, (size_t)nn));
      hnorm.resize(nn);
    }
  }
  int sweep = 0;
  for (; sweep < max_sweeps; sweep++) {
    // the pair solver runs up to 12 inner sweeps in the first two outer
    // sweeps (FP32 storage: 2, which measured fastest overall); once the
    // pairs are close to orthogonal one inner sweep of rotations reduces
    // them quadratically and the outer test decides convergence
    // (QT_JACOBI_INNER0 / QT_JACOBI_INNER override the two caps)
    static const int inner_cap = std::getenv("QT_JACOBI_INNER") ? std::atoi(std::getenv("QT_JACOBI_INNER")) : 1;
    static const int inner_cap0 =
        std::getenv("QT_JACOBI_INNER0") ? std::atoi(std::getenv("QT_JACOBI_INNER0")) : (fp32 ? 2 : MAX_INNER);
    const int max_inner = std::max(1, std::min(sweep < 2 ? inner_cap0 : inner_cap, MAX_INNER));
    QT_CHECK_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(int) * QT_FLAG_COUNT, h->stream));
    if (sweep_kernel) {
      if constexpr (sizeof(typename real_of<TS>::type) == 4) {
        QT_TRY(launch_sweep32(h, pairs, (float2*)X, (float2*)X1, ldx, (int)mm, (float2*)V, (float2*)V1, ldv, (int)nn,
                              nb, gcount, pending ? 1 : 0, tol, (float)tol_inner, nu_rel2, (const double*)xnorm2,
                              (float2*)wbuf, rotf, done, max_inner, keep2, dnorm, phase_ns, halves, gx, xflag));
      }
      gcount += rounds;
      pending = true;
    }
    for (int r = 0; r < rounds && !sweep_kernel; r++) {
      if (two_launch) {
        if constexpr (sizeof(typename real_of<TS>::type) == 4) {
          QT_LAUNCH(h, pair_eig32_kernel, pairs, NTG, 0, (const float2*)X, ldx, (int)mm, (int)nn, nb, r, tol,
                    (float)tol_inner, nu_rel2, (const double*)xnorm2, (float2*)wbuf, rotf, h->d_flags, max_inner,
                    phase_ns);
          QT_LAUNCH(h, pair_apply32_kernel, dim3(pairs, achunks), NT, 0, (float2*)X, ldx, (int)mm, (float2*)V, ldv,
                    (int)nn, nb, r, axrows, avrows, (const float2*)wbuf, (const int*)rotf);
        }
        continue;
      }
      if (csize) {
        QT_TRY(launch_pair_round<TS>(h, csize, pairs, smem, X, ldx, (int)mm, V, ldv, (int)nn, nb, r, xrows_c, vrows_c,
                                     lds, tol, tol_inner, nu_rel2, xnorm2, max_inner, phase_ns));
        continue;
      }
      QT_LAUNCH(h, (gram_kernel<TS, TG>), grid, NT, 0, X, ldx, (int)mm, (int)nn, nb, r, xrows, parts);
      QT_LAUNCH(h, eig_kernel, pairs, NT, 0, (int)nn, nb, r, chunks, (const double2*)parts, tol, nu_rel2,
                (const double*)xnorm2, wbuf, rotf, h->d_flags);
      QT_LAUNCH(h, apply_kernel<TS>, grid, NT, 0, X, ldx, (int)mm, V, ldv, (int)nn, nb, r, xrows, vrows,
                (const double2*)wbuf, (const int*)rotf);
    }
    QT_CHECK_CUDA(h, cudaMemcpyAsync(h->h_flags, h->d_flags, sizeof(int) * QT_FLAG_COUNT, cudaMemcpyDeviceToHost,
                                     h->stream));
    if (keep_track)
      QT_CHECK_CUDA(h, cudaMemcpyAsync(hnorm.data(), dnorm, sizeof(float) * nn, cudaMemcpyDeviceToHost, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    {
      const double es = (double)sizeof(TS);
      h->work_jacobi_rounds += rounds;
      h->work_jacobi_pairs += h->h_flags[QT_FLAG_ROTATED];
      h->work_jacobi_inner += h->h_flags[QT_FLAG_INNER];
      h->work_jacobi_bytes += (double)rounds * (double)mm * (double)nn * es +
                              (double)h->h_flags[QT_FLAG_ROTATED] * JC * es * ((double)mm + (V ? 2.0 * (double)nn : 0.0));
      h->work_jacobi_gram_bytes += (double)rounds * (double)mm * (double)nn * es;
      h->work_jacobi_rot_bytes += (double)h->h_flags[QT_FLAG_ROTATED] * JC * es * ((double)mm + (V ? (double)nn : 0.0));
    }
    float offkept = 0.f;
    std::memcpy(&offkept, &h->h_flags[QT_FLAG_OFFKEPT], sizeof(float));
    const float keep2_used = keep2;
    double tail2 = -1.0, tail2_change = -1.0;
    if (keep_track) {
      // the weight left outside the keep_count largest columns bounds the
      // truncation error of the final split from above (those columns span
      // at least their own weight); its change over the sweep measures how
      // much the kept set still moves
      std::vector<float> srt(hnorm);
      std::nth_element(srt.begin(), srt.begin() + (keep_count - 1), srt.end(), std::greater<float>());
      keep2 = (float)(keep_margin * keep_margin) * srt[keep_count - 1];
      tail2 = 0.0;
      for (int64_t c = keep_count; c < nn; c++) tail2 += (double)srt[c];
      if (prev_tail2 >= 0.0) tail2_change = prev_tail2 - tail2;
      prev_tail2 = tail2;
    }
    if (trace) {
      float off;
      std::memcpy(&off, &h->h_flags[QT_FLAG_OFFMAX], sizeof(float));
      float offbig;
      std::memcpy(&offbig, &h->h_flags[QT_FLAG_OFFBIG], sizeof(float));
      std::fprintf(stderr,
                   "jacobi %lldx%lld sweep %d: rotated pairs %d, inner sweeps %d, max rel off-diagonal %.3e "
                   "(columns above 1e-3 ||X||: %.3e; above the keep threshold %.3e: %.3e); tail weight %.6e, "
                   "change %.3e\n",
                   (long long)mm, (long long)nn, sweep, h->h_flags[QT_FLAG_ROTATED], h->h_flags[QT_FLAG_INNER], off,
                   offbig, std::sqrt((double)keep2_used), offkept, tail2, tail2_change);
    }
    if (h->h_flags[QT_FLAG_ABORT]) return qt_fail(h, QT_ETIMEOUT, "jacobi: a round of the sweep kernel gave up waiting");
    if (h->h_flags[QT_FLAG_NONFINITE]) return qt_fail(h, QT_ENUMERIC, "jacobi: non-finite value in the matrix");
    if (h->h_flags[QT_FLAG_ROTATED] == 0) break;
    // kept set converged: no pair with a column above the threshold rotated,
    // or the tail weight moved by at most keep_tol of itself over this sweep
    // after at most 10 keep_tol over the previous one (the iteration is in
    // its fast-converging phase, where the remaining sweeps would change the
    // tail by about as much again: the truncation error is then final to
    // ~keep_tol / 2 relative)
    if (keep_track && keep_stop && keep2_used > 0.f && offkept == 0.f) break;
    if (keep_track && keep_stop && tail2_change >= 0.0 && prev_change >= 0.0 && tail2_change <= keep_tol * tail2 &&
        prev_change <= 10.0 * keep_tol * tail2)
      break;
    prev_change = tail2_change;
  }
  *sweeps_out = sweep + (sweep < max_sweeps ? 1 : 0);
  if (sweep_kernel && pending) {
    // the last round's unitaries, in place, then the data back into X and V
    if constexpr (sizeof(typename real_of<TS>::type) == 4) {
      const int b = (gcount - 1) & 1;
      float2* xf = (float2*)(b ? X1 : X);
      float2* vf = V ? (float2*)(b ? V1 : V) : nullptr;
      QT_LAUNCH(h, pair_apply32_kernel, dim3(pairs, achunks), NT, 0, xf, ldx, (int)mm, vf, ldv, (int)nn, nb,
                rounds - 1, axrows, avrows, (const float2*)wbuf + (size_t)b * pairs * NGRAM, (const int*)rotf + b * pairs);
      if (b) {
        QT_CHECK_CUDA(h, cudaMemcpy2DAsync(X, ldx * sizeof(TS), X1, ldx * sizeof(TS), mm * sizeof(TS), nn,
                                           cudaMemcpyDeviceToDevice, h->stream));
        if (V)
          QT_CHECK_CUDA(h, cudaMemcpy2DAsync(V, ldv * sizeof(TS), V1, ldv * sizeof(TS), nn * sizeof(TS), nn,
                                             cudaMemcpyDeviceToDevice, h->stream));
      }
    }
  }
  if (phase_ns) QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));  // the counters are written on h->stream
  if (phase_ns && sweep_kernel) {
    unsigned long long hp[4];
    QT_CHECK_CUDA(h, cudaMemcpy(hp, phase_ns, sizeof(hp), cudaMemcpyDeviceToHost));
    const double ctas = (double)gcount * pairs;
    std::fprintf(stderr, "jacobi sweep kernel, us per CTA per round: waits %.2f, rebuild+products %.2f, "
                 "reduction+test %.2f, solver %.2f\n", hp[0] / ctas * 1e-3, hp[1] / ctas * 1e-3, hp[2] / ctas * 1e-3,
                 hp[3] / ctas * 1e-3);
  } else if (phase_ns && two_launch) {
    unsigned long long hp[3];
    QT_CHECK_CUDA(h, cudaMemcpy(hp, phase_ns, sizeof(hp), cudaMemcpyDeviceToHost));
    const double launches = (double)(*sweeps_out) * rounds * pairs;
    std::fprintf(stderr, "jacobi Gram kernel, us per CTA: products %.2f, reduction+test %.2f, solver (rotating pairs "
                 "only, averaged over all) %.2f\n", hp[0] / launches * 1e-3, hp[1] / launches * 1e-3,
                 hp[2] / launches * 1e-3);
  } else if (phase_ns) {
    unsigned long long hp[16];
    QT_CHECK_CUDA(h, cudaMemcpy(hp, phase_ns, sizeof(hp), cudaMemcpyDeviceToHost));
    const double launches = (double)(*sweeps_out) * rounds;
    const char* nm[7] = {"stage", "gram", "barrier1", "sums+barrier2", "test+solver", "barriers+copy", "rotate"};
    for (int g = 0; g < 2; g++) {
      const double ctas = launches * pairs * (g == 0 ? 1 : csize - 1);
      std::fprintf(stderr, "jacobi phases (%s), us per CTA per round:", g == 0 ? "CTA 0" : "other CTAs");
      for (int i = 0; i < 7; i++) std::fprintf(stderr, " %s %.2f", nm[i], ctas > 0 ? hp[8 * g + i] / ctas * 1e-3 : 0.0);
      std::fprintf(stderr, "\n");
    }
  }
  if (sweep >= max_sweeps) {
    // Out of sweeps: accept when the worst remaining pair is orthogonal to
    // 1e-6 relative (its effect on the singular values is below 1e-12), or --
    // FP32 storage -- when every column above 1e-3 ||X||_F has converged and
    // only columns near the rounding level still rotate (their total weight,
    // all the tail rule needs of them, is rotation-invariant).
    float off, offbig;
    std::memcpy(&off, &h->h_flags[QT_FLAG_OFFMAX], sizeof(float));
    std::memcpy(&offbig, &h->h_flags[QT_FLAG_OFFBIG], sizeof(float));
    if (off < 1e-6f) return QT_OK;
    if (fp32 && offbig <= tol) return QT_OK;
    return qt_fail(h, QT_ENUMERIC, "jacobi: no convergence within the sweep limit (off " + std::to_string(off) + ")");
  }
  return QT_OK;
}
template int qt_jacobi_svd_ws<double2>(qt_handle*, double2*, int64_t, int64_t, int64_t, double2*, int64_t, double,
                                       int, int*, double2*, double, int);
template int qt_jacobi_svd_ws<float2>(qt_handle*, float2*, int64_t, int64_t, int64_t, float2*, int64_t, double, int,
                                      int*, double2*, double, int);

template <typename TS>
int qt_jacobi_svd(qt_handle* h, TS* X, int64_t mm, int64_t nn, int64_t ldx, TS* V, int64_t ldv, double tol,
                  int max_sweeps, int* sweeps_out, double nu_rel, int keep_count) {
  int nb = 0, chunks = 0;
  const int nparts = qt_jacobi_layout(mm, nn, &nb, &chunks);
  qt_scratch s(h);
  double2* parts;
  QT_TRY(s.get(&parts, (size_t)nparts));
  return qt_jacobi_svd_ws<TS>(h, X, mm, nn, ldx, V, ldv, tol, max_sweeps, sweeps_out, parts, nu_rel, keep_count);
}
template int qt_jacobi_svd<double2>(qt_handle*, double2*, int64_t, int64_t, int64_t, double2*, int64_t, double, int,
                                    int*, double, int);
template int qt_jacobi_svd<float2>(qt_handle*, float2*, int64_t, int64_t, int64_t, float2*, int64_t, double, int,
                                   int*, double, int);
