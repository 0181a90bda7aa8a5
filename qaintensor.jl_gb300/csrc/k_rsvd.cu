// Randomized-SVD helpers: Gaussian probes and the sketch orthogonalisation.
//
// The range finder (Halko, Martinsson and Tropp 2011, Alg. 4.1/4.4) needs an
// orthonormal basis of Y = theta' Omega.  It is built by block classical
// Gram-Schmidt with one re-orthogonalisation pass (BCGS2), each 32-column
// block orthonormalised internally by CholeskyQR2 -- the first pass shifted
// (Fukaya, Kannan, Nakatsukasa, Zhang, Yamamoto 2020) so that numerically
// rank-deficient blocks still factor.  Block Gram matrices are accumulated in
// FP64 from the stored values and factored in FP64; the basis itself is
// stored in the element type of Y.
#include <cuda_runtime.h>

#include <cmath>

#include "qt_internal.cuh"

namespace {

constexpr int BW = 32;  // block width of the orthogonalisation

__device__ inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Standard complex Gaussian entries (E|z|^2 = 1) by Box-Muller on a
// counter-based hash of (seed, row, col): reproducible for any launch shape.
template <typename C>
__global__ void gaussian_kernel(C* __restrict__ out, int64_t rows, int64_t cols, int64_t ld, uint64_t seed) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < rows * cols;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    const uint64_t h = splitmix64(seed ^ splitmix64((uint64_t)i * 0x100000001B3ull + (uint64_t)j));
    const double u1 = ((h >> 11) + 1.0) * (1.0 / 9007199254740993.0);  // (0, 1]
    const double u2 = (double)(splitmix64(h) >> 11) * (1.0 / 9007199254740992.0);
    const double r = sqrt(-log(u1));  // |z|^2 = r^2 ~ Exp(1)
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    C z;
    z.x = r * c;
    z.y = r * s;
    out[i + ld * j] = z;
  }
}

// Gram of the b (<= 32) columns of Yb, added into G (32 x 32, upper
// triangle, FP64) with atomics.  Each CTA sums GR rows at a time over a grid-strided
// set of row tiles; the per-tile partial sums run in the element precision of
// Y (each entry then carries a relative error of a few u of its own column
// norms) and are accumulated across tiles and CTAs in FP64.
constexpr int GR = 16;
template <typename C>
__global__ void __launch_bounds__(256) block_gram_kernel(const C* __restrict__ Y, int64_t m, int b, double2* __restrict__ G) {
  __shared__ C Ys[GR][BW + 1];
  // thread t owns entries e = t + 256 h (h = 0..3) of the 32 x 32 Gram: i = e % 32, j = e / 32
  double2 acc[4];
#pragma unroll
  for (int h = 0; h < 4; h++) acc[h] = make_double2(0, 0);
  for (int64_t r0 = (int64_t)blockIdx.x * GR; r0 < m; r0 += (int64_t)gridDim.x * GR) {
    for (int idx = threadIdx.x; idx < GR * BW; idx += 256) {
      const int rr = idx % GR, c = idx / GR;
      C v = czero<C>();
      if (r0 + rr < m && c < b) v = Y[(r0 + rr) + m * (int64_t)c];
      Ys[rr][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 4; h++) {
      const int e = threadIdx.x + 256 * h;
      const int i = e % BW, j = e / BW;
      if (i <= j && j < b) {
        C s = czero<C>();
#pragma unroll
        for (int rr = 0; rr < GR; rr++) cfma_conj(s, Ys[rr][i], Ys[rr][j]);
        acc[h] = cadd(acc[h], ccast<double2>(s));
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int h = 0; h < 4; h++) {
    const int e = threadIdx.x + 256 * h;
    const int i = e % BW, j = e / BW;
    if (i <= j && j < b) {
      atomicAdd(&G[i + BW * j].x, acc[h].x);
      atomicAdd(&G[i + BW * j].y, acc[h].y);
    }
  }
}

// Cholesky G = R^H R (R upper); R replaces the upper triangle of G (the
// Gram is accumulated in FP64 either way).  RT is the arithmetic: FP64 for
// an FP64 basis; FP32 for an FP32 basis, whose shifted first pass adds
// 11 (m b + b (b+1)) u_fp32 (about 4 % of the trace at m = 2048) and whose
// later passes see a block orthonormal to a few percent, so FP32 pivots
// lose nothing the stored basis could keep (GB300 runs FP32 at 64x the FP64
// rate).  `shift` adds shift * trace(G) to the diagonal first.  A
// non-positive pivot sets QT_FLAG_CHOL and is replaced by a tiny positive
// value.  One thread per entry (32 x 32 threads), right-looking: at step k
// one thread forms the pivot, the pivot row is scaled and the trailing upper
// triangle updated, in barrier-separated phases.
template <typename RT>
__global__ void __launch_bounds__(BW * BW) chol_kernel(double2* __restrict__ G, int b, double shift,
                                                       int* __restrict__ flags) {
  typedef typename cplx_of<RT>::type CT;
  __shared__ CT R[BW][BW + 1];
  __shared__ CT X[BW][BW + 1];
  __shared__ RT piv[2], rdiag[BW];
  __shared__ double tr;
  const int t = threadIdx.x, i = t / BW, j = t % BW;  // thread t owns entry (i, j)
  const double2 g = (i < b && j < b && i <= j) ? G[i + BW * j] : make_double2(0, 0);
  if (t < 32) {
    double s = (t < b) ? G[t + BW * t].x : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (t == 0) tr = s;
  }
  __syncthreads();
  R[i][j] = ccast<CT>(i == j && i < b ? make_double2(g.x + shift * tr, 0.0) : g);
  __syncthreads();
  for (int k = 0; k < b; k++) {
    // row k: R[k][k] = sqrt(d), R[k][j] /= R[k][k] for j > k.  One thread
    // forms the pivot.  FP64: 1/sqrt(d) from the single-precision estimate
    // refined by two Newton steps y <- y (3 - d y^2) / 2 (quadratic
    // convergence: ~2^-22 -> 2^-44 -> below 2^-52); sqrt(d) = d / sqrt(d).
    if (t == 0) {
      RT d = R[k][k].x;
      if (!(d > (RT)0)) {
        atomicOr(&flags[QT_FLAG_CHOL], 1);
        d = (RT)(fabs(tr) * 1e-30 + (sizeof(RT) == 8 ? 1e-300 : 1e-37));
      }
      RT y = (RT)rsqrtf((float)d);
      if (sizeof(RT) == 8) {
        if (!(y > (RT)0) || isinf(y)) y = (RT)(1.0 / sqrt((double)d));  // d outside the FP32 range
        y = y * ((RT)1.5 - (RT)0.5 * d * y * y);
        y = y * ((RT)1.5 - (RT)0.5 * d * y * y);
      }
      piv[0] = d * y;
      piv[1] = y;
      rdiag[k] = y;
    }
    __syncthreads();
    if (i == k && j == k) R[k][k] = mk(piv[0], (RT)0);
    if (i == k && j > k && j < b) R[k][j] = cscale(R[k][j], piv[1]);
    __syncthreads();
    // trailing update: R[i][j] -= conj(R[k][i]) R[k][j], k < i <= j
    if (i > k && j >= i && j < b) R[i][j] = csub(R[i][j], cmul(cconj(R[k][i]), R[k][j]));
    __syncthreads();
  }
  // X = R^{-1} (upper) by column sweeps of R X = I, one entry per thread:
  // for k = b-1 .. 0, row k of X is final once scaled by 1 / R[k][k], and
  // its multiples R[r][k] X[k][:] are removed from the rows r < k.
  X[i][j] = mk((RT)(i == j && i < b ? 1 : 0), (RT)0);
  __syncthreads();
  for (int k = b - 1; k >= 0; k--) {
    if (i == k) X[k][j] = cscale(X[k][j], rdiag[k]);
    __syncthreads();
    if (i < k) X[i][j] = csub(X[i][j], cmul(R[i][k], X[k][j]));
    __syncthreads();
  }
  G[i + BW * j] = (i <= j) ? ccast<double2>(R[i][j]) : make_double2(0, 0);
  G[BW * BW + i + BW * j] = ccast<double2>(X[i][j]);
}

// Yb <- Yb R^{-1} with the explicit inverse X = R^{-1} (upper triangular,
// formed by chol_kernel): 16 rows per CTA, thread (row t >> 4, columns
// 2 (t & 15) and + 1), out_j = sum_{k <= j} y_k X[k][j] in the element
// precision of Y.  The block's rows are read into shared memory before any
// is written.
template <typename C>
__global__ void __launch_bounds__(256) apply_rinv_kernel(C* __restrict__ Y, int64_t m, int b,
                                                         const double2* __restrict__ Xinv) {
  __shared__ C Xs[BW][BW + 1];
  __shared__ C Ys[16][BW + 1];
  const int t = threadIdx.x, rl = t >> 4, jp = t & 15;
  const int64_t r0 = (int64_t)blockIdx.x * 16;
  for (int e = t; e < BW * BW; e += 256) Xs[e % BW][e / BW] = ccast<C>(Xinv[e]);
  for (int e = t; e < 16 * BW; e += 256) {
    const int rr = e % 16, c = e / 16;
    Ys[rr][c] = (r0 + rr < m && c < b) ? Y[r0 + rr + m * (int64_t)c] : czero<C>();
  }
  __syncthreads();
  const int j0 = 2 * jp, j1 = 2 * jp + 1;
  C a0 = czero<C>(), a1 = czero<C>();
#pragma unroll 8
  for (int k = 0; k < BW; k++) {
    const C y = Ys[rl][k];
    if (k <= j0) cfma(a0, y, Xs[k][j0]);
    if (k <= j1) cfma(a1, y, Xs[k][j1]);
  }
  const int64_t r = r0 + rl;
  if (r < m) {
    if (j0 < b) Y[r + m * (int64_t)j0] = a0;
    if (j1 < b) Y[r + m * (int64_t)j1] = a1;
  }
}

// Block Gram-Schmidt projection of the block Yb (m x b, b <= 32) against the
// j0 columns before it: coef = Y[:, :j0]^H Yb, then Yb -= Y[:, :j0] coef.
// The coefficients are summed over row chunks of PJ_ROWS rows: each CTA of
// proj_coef_kernel owns one chunk and 128 of the j0 columns (4 x 4 entries
// per thread, rows staged 32 (FP64: 16) at a time, the next stage loaded
// into registers meanwhile) and writes its partial; the chunks are added in
// chunk order by coef_reduce_kernel (reproducible, no atomics).
constexpr int PJ_ROWS = 64;   // rows per coefficient chunk
constexpr int PJ_K = 128;     // previous columns per coefficient CTA
constexpr int PJ_R = 16;      // rows per CTA of the update
template <typename C>
__global__ void __launch_bounds__(256) proj_coef_kernel(const C* __restrict__ Y, int64_t m, int j0,
                                                        const C* __restrict__ Yb, int b, C* __restrict__ part) {
  constexpr int SR = sizeof(C) == 8 ? 32 : 16;  // rows staged at a time (static shared memory <= 48 KB)
  constexpr int NY = SR * PJ_K / 256, NB = SR * BW / 256;
  __shared__ C Ys[SR][PJ_K + 1];
  __shared__ C Bs[SR][BW + 1];
  const int t = threadIdx.x, kq = t & 31, jq = t >> 5;  // entries k = 4 kq + a, j = 4 jq + c
  const int64_t r_begin = (int64_t)blockIdx.x * PJ_ROWS, r_end = min(m, r_begin + (int64_t)PJ_ROWS);
  const int k0 = blockIdx.y * PJ_K;
  C acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[a][c] = czero<C>();
  // the next stage's values wait in registers while the current one is used
  C py[NY], pb[NB];
  auto fetch = [&](int64_t r0) {
#pragma unroll
    for (int u = 0; u < NY; u++) {
      const int e = t + 256 * u, rr = e % SR, kk = e / SR;
      const int64_t r = r0 + rr;
      py[u] = (r < r_end && k0 + kk < j0) ? Y[r + m * (int64_t)(k0 + kk)] : czero<C>();
    }
#pragma unroll
    for (int u = 0; u < NB; u++) {
      const int e = t + 256 * u, rr = e % SR, jj = e / SR;
      const int64_t r = r0 + rr;
      pb[u] = (r < r_end && jj < b) ? Yb[r + m * (int64_t)jj] : czero<C>();
    }
  };
  fetch(r_begin);
  for (int64_t r0 = r_begin; r0 < r_end; r0 += SR) {
#pragma unroll
    for (int u = 0; u < NY; u++) { const int e = t + 256 * u; Ys[e % SR][e / SR] = py[u]; }
#pragma unroll
    for (int u = 0; u < NB; u++) { const int e = t + 256 * u; Bs[e % SR][e / SR] = pb[u]; }
    __syncthreads();
    if (r0 + SR < r_end) fetch(r0 + SR);
#pragma unroll 4
    for (int rr = 0; rr < SR; rr++) {
      C y[4], z[4];
#pragma unroll
      for (int a = 0; a < 4; a++) y[a] = Ys[rr][4 * kq + a];
#pragma unroll
      for (int c = 0; c < 4; c++) z[c] = Bs[rr][4 * jq + c];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int c = 0; c < 4; c++) cfma_conj(acc[a][c], y[a], z[c]);
    }
    __syncthreads();
  }
  // part[chunk][k][j], k over the padded j0
  const int jp = gridDim.y * PJ_K;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++)
      part[((size_t)blockIdx.x * jp + k0 + 4 * kq + a) * BW + 4 * jq + c] = acc[a][c];
}

template <typename C>
__global__ void coef_reduce_kernel(const C* __restrict__ part, int nchunk, int jp, int j0, C* __restrict__ coef) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // e = k * BW + j
  if (e >= j0 * BW) return;
  C v = part[e];
  for (int c = 1; c < nchunk; c++) v = cadd(v, part[(size_t)c * jp * BW + e]);
  coef[e] = v;
}

// Yb[r][j] -= sum_k Y[r][k] coef[k][j]: PJ_R rows per CTA, thread (row t >> 4,
// columns 2 (t & 15), + 1), previous columns staged KT at a time.
template <typename C>
__global__ void __launch_bounds__(256) proj_apply_kernel(const C* __restrict__ Y, int64_t m, int j0,
                                                         const C* __restrict__ coef, C* __restrict__ Yb, int b) {
  constexpr int KT = sizeof(C) == 8 ? 64 : 32;  // static shared memory <= 48 KB
  constexpr int NC = KT * BW / 256, NY = PJ_R * KT / 256;
  __shared__ __align__(16) C Cs[KT][BW];
  __shared__ C Ys[PJ_R][KT + 1];
  const int t = threadIdx.x, rl = t >> 4, jp = t & 15;
  const int64_t r = (int64_t)blockIdx.x * PJ_R + rl;
  C a0 = czero<C>(), a1 = czero<C>();
  // the next tile waits in registers while the current one is used
  C pc[NC], py[NY];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int u = 0; u < NC; u++) {
      const int e = t + 256 * u, kk = e / BW, jj = e % BW;
      pc[u] = (k0 + kk < j0) ? coef[(size_t)(k0 + kk) * BW + jj] : czero<C>();
    }
#pragma unroll
    for (int u = 0; u < NY; u++) {
      const int e = t + 256 * u, rr = e % PJ_R, kk = e / PJ_R;
      const int64_t gr = (int64_t)blockIdx.x * PJ_R + rr;
      py[u] = (gr < m && k0 + kk < j0) ? Y[gr + m * (int64_t)(k0 + kk)] : czero<C>();
    }
  };
  fetch(0);
  for (int k0 = 0; k0 < j0; k0 += KT) {
#pragma unroll
    for (int u = 0; u < NC; u++) { const int e = t + 256 * u; Cs[e / BW][e % BW] = pc[u]; }
#pragma unroll
    for (int u = 0; u < NY; u++) { const int e = t + 256 * u; Ys[e % PJ_R][e / PJ_R] = py[u]; }
    __syncthreads();
    if (k0 + KT < j0) fetch(k0 + KT);
#pragma unroll 8
    for (int kk = 0; kk < KT; kk++) {
      const C y = Ys[rl][kk];
      cfma(a0, y, Cs[kk][2 * jp]);
      cfma(a1, y, Cs[kk][2 * jp + 1]);
    }
    __syncthreads();
  }
  if (r < m) {
    if (2 * jp < b) Yb[r + m * (int64_t)(2 * jp)] = csub(Yb[r + m * (int64_t)(2 * jp)], a0);
    if (2 * jp + 1 < b) Yb[r + m * (int64_t)(2 * jp + 1)] = csub(Yb[r + m * (int64_t)(2 * jp + 1)], a1);
  }
}

template <typename C>
int block_project(qt_handle* h, const C* Y, int64_t m, int j0, C* Yb, int b, C* part, C* coef) {
  const int nchunk = (int)((m + PJ_ROWS - 1) / PJ_ROWS), nk = (j0 + PJ_K - 1) / PJ_K;
  QT_LAUNCH(h, proj_coef_kernel<C>, dim3(nchunk, nk), 256, 0, Y, m, j0, Yb, b, part);
  QT_LAUNCH(h, coef_reduce_kernel<C>, (unsigned)((j0 * BW + 255) / 256), 256, 0, (const C*)part, nchunk, nk * PJ_K,
            j0, coef);
  QT_LAUNCH(h, proj_apply_kernel<C>, (unsigned)((m + PJ_R - 1) / PJ_R), 256, 0, Y, m, j0, (const C*)coef, Yb, b);
  return QT_OK;
}

template <typename C>
int block_cholqr(qt_handle* h, C* Yb, int64_t m, int b, bool shifted, double2* dG) {
  QT_CHECK_CUDA(h, cudaMemsetAsync(dG, 0, sizeof(double2) * BW * BW, h->stream));  // the Gram; chol writes R, R^{-1}
  const unsigned gg = (unsigned)std::min<int64_t>((m + GR - 1) / GR, 2 * 152);
  QT_LAUNCH(h, block_gram_kernel<C>, gg, 256, 0, Yb, m, b, dG);
  // shift of shifted CholeskyQR3, sized by the unit roundoff of the stored
  // basis (the Gram and the Cholesky run in FP64, but Y R^{-1} is formed and
  // stored in the element type of Y)
  const double u = (sizeof(typename real_of<C>::type) == 8) ? 1.11e-16 : 5.96e-8;
  const double shift = shifted ? 11.0 * ((double)m * b + (double)b * (b + 1)) * u : 0.0;
  QT_LAUNCH(h, chol_kernel<typename real_of<C>::type>, 1, BW * BW, 0, dG, b, shift, h->d_flags);
  QT_LAUNCH(h, apply_rinv_kernel<C>, (unsigned)((m + 15) / 16), 256, 0, Yb, m, b, (const double2*)dG + BW * BW);
  return QT_OK;
}

}  // namespace

template <typename C>
int qt_gaussian(qt_handle* h, C* out, int64_t rows, int64_t cols, int64_t ld, uint64_t seed) {
  int64_t g = (rows * cols + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  QT_LAUNCH(h, gaussian_kernel<C>, (unsigned)g, 256, 0, out, rows, cols, ld, seed);
  return QT_OK;
}
template int qt_gaussian<float2>(qt_handle*, float2*, int64_t, int64_t, int64_t, uint64_t);
template int qt_gaussian<double2>(qt_handle*, double2*, int64_t, int64_t, int64_t, uint64_t);

template <typename C>
int qt_orthonormalize(qt_handle* h, C* Y, int64_t m, int64_t l) {
  if (l > m) return qt_fail(h, QT_EINVAL, "orthonormalize: more columns than rows");
  qt_scratch s(h);
  double2* dG;
  C *coef, *part;
  const int64_t nchunk = (m + PJ_ROWS - 1) / PJ_ROWS, lpad = (l + PJ_K - 1) / PJ_K * PJ_K;
  QT_TRY(s.get(&dG, 2 * BW * BW));
  QT_TRY(s.get(&coef, (size_t)l * BW));
  QT_TRY(s.get(&part, (size_t)nchunk * lpad * BW));
  for (int64_t j0 = 0; j0 < l; j0 += BW) {
    const int b = (int)std::min<int64_t>(BW, l - j0);
    C* Yb = Y + m * j0;
    for (int pass = 0; pass < 2; pass++) {
      if (j0 > 0) QT_TRY(block_project<C>(h, Y, m, (int)j0, Yb, b, part, coef));
      QT_TRY(block_cholqr<C>(h, Yb, m, b, pass == 0, dG));
    }
    // one more CholeskyQR (shifted CholeskyQR3): after a shifted pass with
    // the FP32 shift the block is only well conditioned, not orthonormal
    if (sizeof(typename real_of<C>::type) == 4) QT_TRY(block_cholqr<C>(h, Yb, m, b, false, dG));
  }
  return QT_OK;
}
template int qt_orthonormalize<float2>(qt_handle*, float2*, int64_t, int64_t);
template int qt_orthonormalize<double2>(qt_handle*, double2*, int64_t, int64_t);
