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

// Cholesky G = R^H R (R upper) in FP64 on one warp; R replaces the upper
// triangle of G.  `shift` adds shift * trace(G) to the diagonal first.  A
// non-positive pivot sets QT_FLAG_CHOL and is replaced by a tiny positive
// value.  Thread t owns column t.
__global__ void chol_kernel(double2* __restrict__ G, int b, double shift, int* __restrict__ flags) {
  __shared__ double2 R[BW][BW + 1];
  __shared__ double rdiag[BW];  // 1 / R[k][k]: one division per pivot
  __shared__ double tr;
  const int t = threadIdx.x;  // 32 threads
  if (t == 0) {
    double s = 0;
    for (int i = 0; i < b; i++) s += G[i + BW * i].x;
    tr = s;
  }
  __syncwarp();
  for (int i = 0; i < BW; i++) R[i][t] = (t < b && i <= t) ? G[i + BW * t] : make_double2(0, 0);
  __syncwarp();
  if (t < b) R[t][t] = make_double2(R[t][t].x + shift * tr, 0.0);
  __syncwarp();
  for (int k = 0; k < b; k++) {
    if (t == 0) {
      double d = R[k][k].x;
      if (!(d > 0.0)) {
        atomicOr(&flags[QT_FLAG_CHOL], 1);
        d = fabs(tr) * 1e-30 + 1e-300;
      }
      const double r = sqrt(d);
      R[k][k] = make_double2(r, 0.0);
      rdiag[k] = 1.0 / r;
    }
    __syncwarp();
    if (t > k && t < b) R[k][t] = cscale(R[k][t], rdiag[k]);
    __syncwarp();
    // trailing update of the upper triangle: A[i][t] -= conj(R[k][i]) R[k][t], k < i <= t
    if (t > k && t < b)
      for (int i = k + 1; i <= t; i++) R[i][t] = csub(R[i][t], cmul(cconj(R[k][i]), R[k][t]));
    __syncwarp();
  }
  for (int i = 0; i < BW; i++) G[i + BW * t] = (i <= t) ? R[i][t] : make_double2(0, 0);
}

// Yb <- Yb R^{-1} (R upper triangular b x b): each thread forward-substitutes
// one row (y R = x, y_j = (x_j - sum_{k<j} y_k R_kj) / R_jj) in the element
// precision of Y, with R rounded to it.
template <typename C>
__global__ void __launch_bounds__(128) apply_rinv_kernel(C* __restrict__ Y, int64_t m, int b, const double2* __restrict__ R) {
  typedef typename real_of<C>::type RS;
  __shared__ C Rs[BW][BW + 1];
  __shared__ RS rinv[BW];
  for (int e = threadIdx.x; e < BW * BW; e += blockDim.x) {
    const int i = e % BW, j = e / BW;
    Rs[i][j] = (i < b && j < b) ? ccast<C>(R[e]) : czero<C>();
  }
  for (int j = threadIdx.x; j < BW; j += blockDim.x) rinv[j] = (j < b) ? (RS)(1.0 / R[j + BW * j].x) : (RS)0;
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    C y[BW];
#pragma unroll
    for (int j = 0; j < BW; j++) {
      if (j >= b) break;
      C s = Y[i + m * (int64_t)j];
#pragma unroll
      for (int k = 0; k < j; k++) {
        const C r = Rs[k][j];
        s.x -= y[k].x * r.x - y[k].y * r.y;
        s.y -= y[k].x * r.y + y[k].y * r.x;
      }
      y[j] = cscale(s, rinv[j]);
      Y[i + m * (int64_t)j] = y[j];
    }
  }
}

template <typename C>
int block_cholqr(qt_handle* h, C* Yb, int64_t m, int b, bool shifted, double2* dG) {
  QT_CHECK_CUDA(h, cudaMemsetAsync(dG, 0, sizeof(double2) * BW * BW, h->stream));
  const unsigned gg = (unsigned)std::min<int64_t>((m + GR - 1) / GR, 2 * 152);
  QT_LAUNCH(h, block_gram_kernel<C>, gg, 256, 0, Yb, m, b, dG);
  // shift of shifted CholeskyQR3, sized by the unit roundoff of the stored
  // basis (the Gram and the Cholesky run in FP64, but Y R^{-1} is formed and
  // stored in the element type of Y)
  const double u = (sizeof(typename real_of<C>::type) == 8) ? 1.11e-16 : 5.96e-8;
  const double shift = shifted ? 11.0 * ((double)m * b + (double)b * (b + 1)) * u : 0.0;
  QT_LAUNCH(h, chol_kernel, 1, 32, 0, dG, b, shift, h->d_flags);
  QT_LAUNCH(h, apply_rinv_kernel<C>, (unsigned)std::min<int64_t>((m + 127) / 128, 4 * 152), 128, 0, Yb, m, b,
            (const double2*)dG);
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
  C* coef;
  QT_TRY(s.get(&dG, BW * BW));
  QT_TRY(s.get(&coef, (size_t)l * BW));
  C one, zero, mone;
  one.x = 1; one.y = 0; zero.x = 0; zero.y = 0; mone.x = -1; mone.y = 0;
  for (int64_t j0 = 0; j0 < l; j0 += BW) {
    const int b = (int)std::min<int64_t>(BW, l - j0);
    C* Yb = Y + m * j0;
    for (int pass = 0; pass < 2; pass++) {
      if (j0 > 0) {
        QT_TRY(qt_gemm_any(h, QT_OP_C, QT_OP_N, j0, b, m, one, Y, m, Yb, m, zero, coef, j0));
        QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, m, b, j0, mone, Y, m, coef, j0, one, Yb, m));
      }
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
