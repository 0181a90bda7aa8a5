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

// Partial Gram of the b (<= 32) columns of Yb over a 64-row slice, added into
// G (b x b, FP64, full matrix) with atomics.
template <typename C>
__global__ void __launch_bounds__(256) block_gram_kernel(const C* __restrict__ Y, int64_t m, int b, double2* __restrict__ G) {
  __shared__ double2 Ys[64][BW + 1];
  const int64_t r0 = blockIdx.x * 64;
  for (int idx = threadIdx.x; idx < 64 * BW; idx += 256) {
    const int rr = idx % 64, c = idx / 64;
    double2 v = make_double2(0, 0);
    if (r0 + rr < m && c < b) v = ccast<double2>(Y[(r0 + rr) + m * (int64_t)c]);
    Ys[rr][c] = v;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < b * b; e += 256) {
    const int i = e % b, j = e / b;
    if (i > j) continue;
    double2 acc = make_double2(0, 0);
    for (int rr = 0; rr < 64; rr++) cfma_conj(acc, Ys[rr][i], Ys[rr][j]);
    atomicAdd(&G[i + BW * j].x, acc.x);
    atomicAdd(&G[i + BW * j].y, acc.y);
  }
}

// Cholesky G = R^H R (R upper) in FP64 on one warp, then Rinv = R^{-1}.
// `shift` adds shift * trace(G) to the diagonal first.  A non-positive pivot
// sets QT_FLAG_CHOL and is replaced by a tiny positive value.  Thread t owns
// column t of R and of Rinv.
__global__ void chol_inv_kernel(double2* __restrict__ G, int b, double shift, int* __restrict__ flags) {
  __shared__ double2 R[BW][BW + 1];
  __shared__ double2 Ri[BW][BW + 1];
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
      R[k][k] = make_double2(sqrt(d), 0.0);
    }
    __syncwarp();
    if (t > k && t < b) R[k][t] = cscale(R[k][t], 1.0 / R[k][k].x);
    __syncwarp();
    // trailing update of the upper triangle: A[i][t] -= conj(R[k][i]) R[k][t], k < i <= t
    if (t > k && t < b)
      for (int i = k + 1; i <= t; i++) R[i][t] = csub(R[i][t], cmul(cconj(R[k][i]), R[k][t]));
    __syncwarp();
  }
  // upper-triangular inverse by back substitution, column t
  for (int i = 0; i < BW; i++) Ri[i][t] = make_double2(0, 0);
  if (t < b) {
    for (int i = t; i >= 0; i--) {
      double2 s = make_double2(i == t ? 1.0 : 0.0, 0.0);
      for (int j = i + 1; j <= t; j++) s = csub(s, cmul(R[i][j], Ri[j][t]));
      Ri[i][t] = cscale(s, 1.0 / R[i][i].x);
    }
  }
  __syncwarp();
  for (int i = 0; i < BW; i++) G[i + BW * t] = Ri[i][t];
}

// Yb <- Yb Rinv (Rinv upper triangular b x b, FP64 entries).
template <typename C>
__global__ void __launch_bounds__(256) apply_rinv_kernel(C* __restrict__ Y, int64_t m, int b, const double2* __restrict__ Ri) {
  __shared__ double2 Rs[BW][BW + 1];
  for (int e = threadIdx.x; e < BW * BW; e += 256) Rs[e % BW][e / BW] = (e % BW < b && e / BW < b) ? Ri[e] : make_double2(0, 0);
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    double2 y[BW];
#pragma unroll
    for (int k = 0; k < BW; k++) y[k] = (k < b) ? ccast<double2>(Y[i + m * (int64_t)k]) : make_double2(0, 0);
#pragma unroll
    for (int j = BW - 1; j >= 0; j--) {
      if (j >= b) continue;
      double2 s = make_double2(0, 0);
#pragma unroll
      for (int k = 0; k <= j; k++) cfma(s, y[k], Rs[k][j]);
      Y[i + m * (int64_t)j] = ccast<C>(s);
    }
  }
}

template <typename C>
int block_cholqr(qt_handle* h, C* Yb, int64_t m, int b, bool shifted, double2* dG) {
  QT_CHECK_CUDA(h, cudaMemsetAsync(dG, 0, sizeof(double2) * BW * BW, h->stream));
  QT_LAUNCH(h, block_gram_kernel<C>, (unsigned)((m + 63) / 64), 256, 0, Yb, m, b, dG);
  // shift of shifted CholeskyQR3, sized by the unit roundoff of the stored
  // basis (the Gram and the Cholesky run in FP64, but Y R^{-1} is formed and
  // stored in the element type of Y)
  const double u = (sizeof(typename real_of<C>::type) == 8) ? 1.11e-16 : 5.96e-8;
  const double shift = shifted ? 11.0 * ((double)m * b + (double)b * (b + 1)) * u : 0.0;
  QT_LAUNCH(h, chol_inv_kernel, 1, 32, 0, dG, b, shift, h->d_flags);
  QT_LAUNCH(h, apply_rinv_kernel<C>, (unsigned)std::min<int64_t>((m + 255) / 256, 1024), 256, 0, Yb, m, b,
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
