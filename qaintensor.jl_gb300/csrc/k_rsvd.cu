// Randomized-SVD helpers: Gaussian probes and the sketch orthogonalisation.
//
// The range finder (Halko, Martinsson and Tropp 2011, Alg. 4.1/4.4) needs an
// orthonormal basis of the sketch Y.  It is built by block classical
// Gram-Schmidt with one re-orthogonalisation pass (BCGS2), each 32-column
// block orthonormalised by CholeskyQR passes -- the first one shifted
// (Fukaya, Kannan, Nakatsukasa, Zhang, Yamamoto 2020) so that numerically
// rank-deficient blocks still factor, and a third one for an FP32 basis.  The
// basis is stored in the element type of Y.  Three implementations:
//   - FP32 bases of up to 2368 rows (whose rows fit the shared memory of one
//     CTA per 16 rows): the whole orthonormalisation in one cooperative
//     launch (orth_one_launch_kernel), grid barriers between its phases.
//   - Other FP32 bases, blocks of up to 4096 rows: per block the projection
//     kernels and one thread-block cluster launch per run of CholeskyQR
//     passes (cholqr_cluster_kernel).  The block's rows stay in shared
//     memory; the Gram is summed in FP32 tiles and float-float across row
//     groups and CTAs, and R and R^{-1} are formed in FP32.
//   - FP64 blocks and taller FP32 blocks: four launches per pass (the Gram in
//     FP64 over many CTAs, a one-CTA Cholesky and inverse, the block update).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "qt_internal.cuh"

namespace cg = cooperative_groups;

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

constexpr int CQ_LDY = BW + 2;       // row stride of the staged rows: 272 B, an odd number of 16-byte granules
constexpr int CQ_TILES = 36;         // upper 4 x 4 tiles of the 32 x 32 Gram, tile (ti <= tj) at tj (tj+1)/2 + ti
constexpr int CQ_E = CQ_TILES * 16;  // Gram entries held, e = 36 (4 (i & 3) + (j & 3)) + tile
constexpr int CQ_GROUPS = 7;         // row groups of the Gram threads (7 x 36 = 252 of 256 threads)
constexpr int CQ_RS = BW + 1;        // row stride of R

__device__ inline void cq_tile(int T, int& ti, int& tj) {
  ti = T;
  tj = 0;
  while (ti > tj) {
    ti -= tj + 1;
    tj++;
  }
}

// float-float (hi, lo) + (h2, l2), normalised (TwoSum; Ogita-Rump-Oishi
// cascaded summation: FP64-like accuracy at FP32 cost)
__device__ inline void ff_add1(float& h, float& l, float h2, float l2) {
  const float s = h + h2, bb = s - h;
  const float e = ((h - (s - bb)) + (h2 - bb)) + (l + l2);
  h = s + e;
  l = e - (h - s);
}
// float-float complex (re hi, re lo, im hi, im lo)
__device__ inline float4 ff4_add(float4 a, const float4 b) {
  ff_add1(a.x, a.y, b.x, b.y);
  ff_add1(a.z, a.w, b.z, b.w);
  return a;
}

// rows staged per CTA: 32 NRB, padded to whole row groups of the Gram
__host__ __device__ constexpr int cq_alloc_rows(int nrb) { return (32 * nrb + CQ_GROUPS - 1) / CQ_GROUPS * CQ_GROUPS; }
__host__ __device__ constexpr size_t cq_smem_bytes(int nrb) {
  return (size_t)cq_alloc_rows(nrb) * CQ_LDY * sizeof(float2) + (size_t)(CQ_GROUPS + 3) * CQ_E * sizeof(float4) +
         (size_t)BW * CQ_RS * sizeof(float2) + (size_t)BW * BW * sizeof(float2) +
         BW * sizeof(double) + BW * sizeof(float) + 16;
}

// Step (E) of a CholeskyQR pass, called by all 256 threads of the CTA.
// From the FP32 Gram in the upper triangle of Gl (row stride CQ_RS) and its
// FP64 diagonal Gd: R = chol(G + shift trace(G) I) in place of the Gram's
// upper triangle, then X = R^{-1}, both blocked by 8 columns.  Cholesky: for
// each diagonal block, warp 0 runs its 8 pivot steps on the block's rows
// of every column to the right (lane l: column k0 + l, an 8-row register
// window moving down one row per step, rows travelling by shuffles), then
// all threads subtract the block's rank-8 product from the trailing upper
// triangle.  Inverse: the four 8 x 8 diagonal blocks by column sweeps (one
// warp each), then the blocks at distance d = 1, 2, 3 from the diagonal,
// X_ij = -X_ii (sum_{i < l <= j} R_il X_lj).  Pivots past b are skipped
// (1 / R[k][k] = 0 there), so X is zero outside the leading b x b block.
// Ry receives 1 / R[k][k] (and the tiny pivot at Ry[BW]), Xs = R^{-1}
// (BW x BW, row-major), Tb is 256 entries of scratch.  `report` marks the
// one CTA that raises QT_FLAG_CHOL for a non-positive pivot.
__device__ void cq_factor(float2* __restrict__ Gl, const double* __restrict__ Gd, float* __restrict__ Ry,
                          float2* __restrict__ Xs, float2* __restrict__ Tb, int b, double shift,
                          int* __restrict__ flags, bool report) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  float* trs = (float*)(Ry + BW);
  if (w == 0) {
    double tr = lane < b ? Gd[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
    if (lane < b) Gl[lane * CQ_RS + lane] = make_float2((float)(Gd[lane] + shift * tr), 0.f);
    Ry[lane] = 0.f;
    if (lane == 0) trs[0] = (float)(fabs(tr) * 1e-30 + 1e-37);
  }
  __syncthreads();
  for (int k0 = 0; k0 < b; k0 += 8) {
    if (w == 0) {
      const int col = k0 + lane;
      float2 c[8];
#pragma unroll
      for (int r = 0; r < 8; r++)
        c[r] = (col < BW && k0 + r <= col) ? Gl[(k0 + r) * CQ_RS + col] : make_float2(0.f, 0.f);
      // dn: the next pivot as seen by its own lane (lane kk + 1 holds
      // R[k][k + 1] itself), so the pivot chain needs no row shuffle
      float dn = c[0].x;
#pragma unroll
      for (int kk = 0; kk < 8; kk++) {
        const int k = k0 + kk;
        if (k < b) {
          float d = __shfl_sync(0xffffffffu, dn, kk);
          if (!(d > 0.f)) {
            if (lane == 0 && report) atomicOr(&flags[QT_FLAG_CHOL], 1);
            d = trs[0];
          }
          const float y = rsqrtf(d);
          const float2 rk =
              lane == kk ? make_float2(d * y, 0.f) : (lane > kk ? cscale(c[0], y) : make_float2(0.f, 0.f));
          dn = c[1].x - (rk.x * rk.x + rk.y * rk.y);
          if (col < BW) Gl[k * CQ_RS + col] = rk;  // row k of R (zeros left of the diagonal)
          if (lane == 0) Ry[k] = y;
#pragma unroll
          for (int r = 1; r < 8; r++) {
            float2 rkr;  // R[k][k + r] from lane kk + r (slots past the block are discarded)
            rkr.x = __shfl_sync(0xffffffffu, rk.x, min(kk + r, 31));
            rkr.y = __shfl_sync(0xffffffffu, rk.y, min(kk + r, 31));
            c[r - 1] = csub(c[r], cmul(cconj(rkr), rk));
          }
        }
      }
    }
    __syncthreads();
    // trailing upper triangle: warp w the rows k0 + 8 + w, + 16, ...;
    // lane j column j (two partial sums)
    for (int i = k0 + 8 + w; i < BW; i += 8) {
      if (lane >= i) {
        float2 v0 = Gl[i * CQ_RS + lane], v1 = make_float2(0.f, 0.f);
#pragma unroll
        for (int q = 0; q < 8; q += 2) {
          v0 = csub(v0, cmul(cconj(Gl[(k0 + q) * CQ_RS + i]), Gl[(k0 + q) * CQ_RS + lane]));
          v1 = csub(v1, cmul(cconj(Gl[(k0 + q + 1) * CQ_RS + i]), Gl[(k0 + q + 1) * CQ_RS + lane]));
        }
        Gl[i * CQ_RS + lane] = cadd(v0, v1);
      }
    }
    __syncthreads();
  }
  // diagonal blocks of X; the blocks below the diagonal are zero
  if (w < 4 && lane < 8) {
    const int k0 = 8 * w;
    float2 x[8];
#pragma unroll
    for (int r = 0; r < 8; r++) x[r] = make_float2(r == lane ? 1.f : 0.f, 0.f);
#pragma unroll
    for (int kk = 7; kk >= 0; kk--) {
      x[kk] = cscale(x[kk], Ry[k0 + kk]);
#pragma unroll
      for (int i = 0; i < kk; i++) x[i] = csub(x[i], cmul(Gl[(k0 + i) * CQ_RS + k0 + kk], x[kk]));
    }
#pragma unroll
    for (int r = 0; r < 8; r++) Xs[(k0 + r) * BW + k0 + lane] = x[r];
  }
  for (int e = t; e < BW * BW; e += 256)
    if ((e / BW) / 8 > (e % BW) / 8) Xs[e] = make_float2(0.f, 0.f);
  __syncthreads();
  for (int d = 1; d < 4; d++) {
    const int bi = t / 64, a = (t / 8) % 8, cc = t % 8, bj = bi + d, i = 8 * bi + a, j = 8 * bj + cc;
    if (bj < 4) {
      float2 v = make_float2(0.f, 0.f);
      for (int l = 8 * (bi + 1); l < 8 * (bj + 1); l++) cfma(v, Gl[i * CQ_RS + l], Xs[l * BW + j]);
      Tb[t] = v;
    }
    __syncthreads();
    if (bj < 4) {
      float2 v = make_float2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < 8; q++) cfma(v, Xs[i * BW + 8 * bi + q], Tb[64 * bi + 8 * q + cc]);
      Xs[i * BW + j] = make_float2(-v.x, -v.y);
    }
    __syncthreads();
  }
}

// CholeskyQR passes of one FP32 block (m x b, b <= 32) in one launch: a
// thread-block cluster of CS CTAs holds the block's rows in shared memory
// (CTA q: rows 32 NRB q .. 32 NRB (q+1) - 1, zero-padded), and each pass
//   (A) forms the CTA's partial Gram: thread (row group g, upper 4 x 4 tile)
//       sums its rows g, g + 7, ... in FP32 (about 37 products per entry);
//   (B) adds the row groups in order in float-float;
//   (C) reduce-scatter over the cluster through distributed shared memory:
//       CTA q owns the entries e = q (mod CS) and adds the ranks in order;
//   (D) every CTA gathers the summed Gram;
//   (E) G (+ shift trace(G) on the diagonal) = R^H R and X = R^{-1} in FP32,
//       blocked by 8 columns -- every CTA computes the same R and X from the
//       same Gram;
//   (F) the rows are replaced by rows X (X upper triangular).
// The loops that carry shared-memory loads have no data-dependent exits, so
// the loads of a step issue together.  The rows go back to global memory
// after the last pass.  Every CTA passes the same cluster barriers (two per
// pass and one before leaving, so that no CTA exits while another may still
// read its shared memory).
template <int NRB, int CS>
__global__ void __launch_bounds__(256, 1) cholqr_cluster_kernel(float2* __restrict__ Y, int64_t m, int b, int npass,
                                                            double shift0, int* __restrict__ flags,
                                                            unsigned long long* __restrict__ phase_ns) {
  constexpr int ROWS = 32 * NRB, AROWS = cq_alloc_rows(NRB), GROWS = AROWS / CQ_GROUPS;
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = (int)cluster.block_rank();
  unsigned long long tp = 0;
  auto phase = [&](int ph) {  // optional diagnostics: CTA 0's SM cycles per phase into phase_ns[ph - 1]
    if (phase_ns && crank == 0 && threadIdx.x == 0) {
      const unsigned long long tn = (unsigned long long)clock64();
      if (ph > 0) atomicAdd(&phase_ns[ph - 1], tn - tp);
      tp = tn;
    }
  };
  phase(0);
  extern __shared__ __align__(16) unsigned char cq_smem[];
  float2* Ys = (float2*)cq_smem;                                  // [AROWS][CQ_LDY]
  float4* Gt = (float4*)(cq_smem + (size_t)AROWS * CQ_LDY * sizeof(float2));  // [CQ_GROUPS][CQ_E]
  float4* Gp = Gt + CQ_GROUPS * CQ_E;                             // [2][CQ_E] partial of this CTA
  float4* Gr = Gp + 2 * CQ_E;                                     // [CQ_E] cluster sums owned here
  float2* Gl = (float2*)(Gr + CQ_E);                              // [BW][CQ_RS] the Gram in FP32, then R
  float2* Xs = Gl + BW * CQ_RS;                                   // [BW][BW] R^{-1}
  double* Gd = (double*)(Xs + BW * BW);                           // [BW] diagonal of the Gram
  float* Ry = (float*)(Gd + BW);                                  // [BW] 1 / R[k][k], then the tiny pivot
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int64_t r0 = (int64_t)crank * ROWS;
  // stage: warp w loads columns 4w .. 4w+3, lane l the rows l + 32 u
  {
    float2 v[4][NRB];
#pragma unroll
    for (int cc = 0; cc < 4; cc++)
#pragma unroll
      for (int u = 0; u < NRB; u++) {
        const int c = 4 * w + cc;
        const int64_t r = r0 + lane + 32 * u;
        v[cc][u] = (r < m && c < b) ? Y[r + m * (int64_t)c] : make_float2(0.f, 0.f);
      }
#pragma unroll
    for (int cc = 0; cc < 4; cc++)
#pragma unroll
      for (int u = 0; u < NRB; u++) Ys[(lane + 32 * u) * CQ_LDY + 4 * w + cc] = v[cc][u];
    for (int e = t; e < (AROWS - ROWS) * CQ_LDY; e += 256) Ys[ROWS * CQ_LDY + e] = make_float2(0.f, 0.f);
  }
  const int g = t / CQ_TILES, T = t % CQ_TILES;
  int ti, tj;
  cq_tile(T, ti, tj);
  __syncthreads();
  phase(1);  // staging
  for (int p = 0; p < npass; p++) {
    // (A) partial Gram of the rows g, g + 7, g + 14, ... for one upper tile
    if (g < CQ_GROUPS) {
      float2 acc[16];
#pragma unroll
      for (int k = 0; k < 16; k++) acc[k] = make_float2(0.f, 0.f);
#pragma unroll 4
      for (int q = 0; q < GROWS; q++) {
        const float4* row = (const float4*)(Ys + (g + CQ_GROUPS * q) * CQ_LDY);
        const float4 a01 = row[2 * ti], a23 = row[2 * ti + 1], b01 = row[2 * tj], b23 = row[2 * tj + 1];
        const float2 av[4] = {make_float2(a01.x, a01.y), make_float2(a01.z, a01.w), make_float2(a23.x, a23.y),
                              make_float2(a23.z, a23.w)};
        const float2 bv[4] = {make_float2(b01.x, b01.y), make_float2(b01.z, b01.w), make_float2(b23.x, b23.y),
                              make_float2(b23.z, b23.w)};
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int c = 0; c < 4; c++) cfma_conj(acc[4 * a + c], av[a], bv[c]);
      }
#pragma unroll
      for (int k = 0; k < 16; k++) Gt[g * CQ_E + k * CQ_TILES + T] = make_float4(acc[k].x, 0.f, acc[k].y, 0.f);
    }
    __syncthreads();
    phase(2);  // Gram
    // (B) the row groups in order
    float4* gp = Gp + (p & 1) * CQ_E;
    for (int e = t; e < CQ_E; e += 256) {
      float4 v = Gt[e];
#pragma unroll
      for (int gg = 1; gg < CQ_GROUPS; gg++) v = ff4_add(v, Gt[gg * CQ_E + e]);
      gp[e] = v;
    }
    cluster.sync();
    phase(3);  // row groups + barrier
    // (C) this CTA's entries summed over the cluster in rank order
    if (crank + CS * t < CQ_E) {
      const int e = crank + CS * t;
      float4 v[CS];
#pragma unroll
      for (int q = 0; q < CS; q++) v[q] = cluster.map_shared_rank(gp, q)[e];
#pragma unroll
      for (int q = 1; q < CS; q++) v[0] = ff4_add(v[0], v[q]);
      Gr[e] = v[0];
    }
    cluster.sync();
    phase(4);  // reduce-scatter + barrier
    // (D) the whole Gram, rounded to FP32 (the diagonal kept in FP64 too)
    {
      float4 v[3];
#pragma unroll
      for (int u = 0; u < 3; u++) {
        const int e = t + 256 * u;
        if (e < CQ_E) v[u] = cluster.map_shared_rank(Gr, e % CS)[e];
      }
#pragma unroll
      for (int u = 0; u < 3; u++) {
        const int e = t + 256 * u;
        if (e < CQ_E) {
          int ei, ej;
          cq_tile(e % CQ_TILES, ei, ej);
          const int k = e / CQ_TILES, i = 4 * ei + (k >> 2), j = 4 * ej + (k & 3);
          Gl[i * CQ_RS + j] = make_float2(v[u].x + v[u].y, v[u].z + v[u].w);
          if (i == j) Gd[i] = (double)v[u].x + (double)v[u].y;
        }
      }
    }
    __syncthreads();
    phase(5);  // gather
    // (E) R = chol(G + shift trace(G) I) and X = R^{-1}, the same in every CTA
    cq_factor(Gl, Gd, Ry, Xs, (float2*)Gt, b, p == 0 ? shift0 : 0.0, flags, crank == 0);
    phase(6);  // Cholesky + inverse
    // (F) rows <- rows X: warp w owns columns 4 cg .. 4 cg + 3 (warps w and
    // w + 4 share a scheduler and take column groups w and 7 - w, which
    // balances the triangle), lane l the rows l + 32 rb
    {
      const int cgp = w < 4 ? w : 11 - w, j0 = 4 * cgp, kend = min(j0 + 4, b);
      float2 acc[NRB][4];
#pragma unroll
      for (int rb = 0; rb < NRB; rb++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[rb][c] = make_float2(0.f, 0.f);
      for (int k = 0; k < kend; k += 2) {
        const float4 xa = *(const float4*)(Xs + k * BW + j0), xb = *(const float4*)(Xs + k * BW + j0 + 2);
        const float4 xc = *(const float4*)(Xs + (k + 1) * BW + j0), xd = *(const float4*)(Xs + (k + 1) * BW + j0 + 2);
        const float2 x0[4] = {make_float2(xa.x, xa.y), make_float2(xa.z, xa.w), make_float2(xb.x, xb.y),
                              make_float2(xb.z, xb.w)};
        const float2 x1[4] = {make_float2(xc.x, xc.y), make_float2(xc.z, xc.w), make_float2(xd.x, xd.y),
                              make_float2(xd.z, xd.w)};
        float4 y[NRB];
#pragma unroll
        for (int rb = 0; rb < NRB; rb++) y[rb] = *(const float4*)(Ys + (rb * 32 + lane) * CQ_LDY + k);
#pragma unroll
        for (int rb = 0; rb < NRB; rb++) {
          const float2 y0 = make_float2(y[rb].x, y[rb].y), y1 = make_float2(y[rb].z, y[rb].w);
#pragma unroll
          for (int c = 0; c < 4; c++) {
            cfma(acc[rb][c], y0, x0[c]);
            cfma(acc[rb][c], y1, x1[c]);
          }
        }
      }
      __syncthreads();  // every row has been read
#pragma unroll
      for (int rb = 0; rb < NRB; rb++)
#pragma unroll
        for (int c = 0; c < 4; c++)
          if (j0 + c < b) Ys[(rb * 32 + lane) * CQ_LDY + j0 + c] = acc[rb][c];
      __syncthreads();
    }
    phase(7);  // update
  }
#pragma unroll
  for (int cc = 0; cc < 4; cc++)
#pragma unroll
    for (int u = 0; u < NRB; u++) {
      const int c = 4 * w + cc;
      const int64_t r = r0 + lane + 32 * u;
      if (r < m && c < b) Y[r + m * (int64_t)c] = Ys[(lane + 32 * u) * CQ_LDY + c];
    }
  cluster.sync();  // no CTA leaves while another may still read its shared memory
  phase(8);  // write-back + barrier
}

typedef void (*cq_kernel_t)(float2*, int64_t, int, int, double, int*, unsigned long long*);
cq_kernel_t cq_kernel(int nrb, int cs) {
  if (cs == 16) {
    switch (nrb) {
      case 1: return cholqr_cluster_kernel<1, 16>;
      case 2: return cholqr_cluster_kernel<2, 16>;
      case 4: return cholqr_cluster_kernel<4, 16>;
      default: return cholqr_cluster_kernel<8, 16>;
    }
  }
  switch (nrb) {
    case 1: return cholqr_cluster_kernel<1, 8>;
    case 2: return cholqr_cluster_kernel<2, 8>;
    case 4: return cholqr_cluster_kernel<4, 8>;
    default: return cholqr_cluster_kernel<8, 8>;
  }
}

cudaLaunchConfig_t cq_config(int nrb, int cs, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(cs);
  lc.blockDim = dim3(256);
  lc.dynamicSmemBytes = cq_smem_bytes(nrb);
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return lc;
}

// Shape of the cluster CholeskyQR for m rows: *cs CTAs of 32 nrb rows, the
// largest cluster the GPU schedules (16, else 8) for m > 256, then the fewest
// rows per CTA; nrb = 0 when the block does not fit (m > 16 * 256, or no
// cluster launch) and the four-kernel passes are used.  QT_CHOLQR_CLUSTER=0
// disables it, QT_CHOLQR_CLUSTER=8 keeps clusters of 8.
int cq_shape(int64_t m, int* cs) {
  static int ok[2] = {-1, -1};  // cluster sizes 8 and 16 launchable for every nrb
  if (ok[0] < 0) {
    for (int ci = 0; ci < 2; ci++) {
      const int c = ci ? 16 : 8;
      ok[ci] = 1;
      for (int nrb = 1; nrb <= 8 && ok[ci]; nrb *= 2) {
        ok[ci] = 0;
        cq_kernel_t k = cq_kernel(nrb, c);
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cq_smem_bytes(nrb)) !=
            cudaSuccess)
          continue;
        if (c == 16 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
          continue;
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t lc = cq_config(nrb, c, attr);
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, k, &lc) == cudaSuccess && nc > 0) ok[ci] = 1;
      }
      cudaGetLastError();
    }
  }
  const char* env = std::getenv("QT_CHOLQR_CLUSTER");
  if (env && env[0] == '0') return 0;
  const bool keep8 = env && env[0] == '8';
  *cs = (ok[1] && !keep8 && m > 256) ? 16 : (ok[0] ? 8 : 0);
  if (*cs == 0) return 0;
  for (int nrb = 1; nrb <= 8; nrb *= 2)
    if ((int64_t)(*cs) * 32 * nrb >= m) return nrb;
  return 0;
}

int block_cholqr_cluster(qt_handle* h, float2* Yb, int64_t m, int b, int nrb, int cs, int npass, bool shifted,
                         unsigned long long* phase_ns) {
  const double shift = shifted ? 11.0 * ((double)m * b + (double)b * (b + 1)) * 5.96e-8 : 0.0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t lc = cq_config(nrb, cs, attr);
  lc.stream = h->stream;
  if (h->prof) qt_prof_before(h, "cholqr_cluster_kernel");
  const cudaError_t e =
      cudaLaunchKernelEx(&lc, cq_kernel(nrb, cs), Yb, m, b, npass, shift, h->d_flags, phase_ns);
  if (h->prof) qt_prof_after(h);
  h->launches++;
  if (e != cudaSuccess) return qt_fail(h, QT_ECUDA, std::string("launch cholqr_cluster_kernel: ") + cudaGetErrorString(e));
  return QT_OK;
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

// ---------------------------------------------------------------------------
// The whole orthonormalisation of an FP32 basis in one cooperative launch.
// CTA c keeps rows 16 c .. 16 c + 15 of Y (all l columns, zero-padded) in
// shared memory from start to end, and the steps of the block Gram-Schmidt
// above (project, shifted CholeskyQR, project, CholeskyQR, CholeskyQR per
// 32-column block; three CholeskyQR passes for the first block; fewer
// passes for the lighter uses, OrthArgs::light) become phases between grid
// barriers:
//   projection of block j0 .. j0 + 31 against the j0 columns before it:
//     (1) the CTA's partial coefficients Y[rows, :j0]^H Y[rows, block] in
//         FP32 over its 16 rows, to part[c];                      barrier
//     (2) CTA c adds the partials of its slice of the j0 x 32 coefficients
//         in a fixed order (warp w over CTAs w S .. w S + S - 1, then the
//         eight warp sums), to coef;                              barrier
//     (3) every CTA subtracts Y[rows, :j0] coef from its rows of the block,
//         the coefficients streamed through a six-chunk ring of 32 rows;
//   CholeskyQR pass:
//     (1) the CTA's partial Gram of the block (FP32 over its rows) to
//         gpart[c];                                               barrier
//     (2) CTA c adds its slice of the 32 x 32 entries over the CTAs in
//         float-float, CTAs in order, to gsum;                    barrier
//     (3) every CTA reads the summed Gram, forms the same R and R^{-1}
//         (cq_factor) and replaces its rows of the block by rows R^{-1}.
// The rows go back to global memory once, at the end.  Sums run in a fixed
// order, so the result is reproducible for a given m.  The barrier is a
// monotone arrival counter whose last arriving CTA publishes the barrier's
// number; every wait is bounded, and a wait that gives up sets an abort
// word (ending the other CTAs' waits) and the handle's sticky device status
// (2).  Data written by other CTAs is read past L1 (ld.global.cg /
// cp.async.cg).
// ---------------------------------------------------------------------------
constexpr int OP_NT = 256;     // threads per CTA
constexpr int OP_R = 16;       // rows per CTA
constexpr int OP_KC = 32;      // coefficient rows per staged chunk
constexpr int OP_NBUF = 6;     // staged chunks in the ring (five in flight)
constexpr int OP_CLD = BW + 2; // row stride of a staged chunk (float2): 272 B, conflict-free float4 reads
constexpr int OP_SPIN = 1 << 22;  // polls of a barrier wait before it gives up
constexpr int OP_MAXCTA = 152;    // CTAs at most (one per SM)

struct OrthArgs {
  float2* Y;
  int64_t m;
  int l, ldy;     // columns; row stride of the staged rows (float2)
  float2* part;   // [ncta][l][BW] coefficient partials
  float2* coef;   // [l][BW] summed coefficients
  float2* gpart;  // [ncta][BW * BW] Gram partials
  float4* gsum;   // [BW * BW] summed Gram (re hi, re lo, im hi, im lo)
  int* bar;       // [0] arrivals, [1] abort word, [2] the last completed barrier, [3] the test hook's word
  int* flags;     // QT_FLAG_CHOL
  int* status;    // sticky device status
  int spin;
  int light;      // 0: as above; 1: no third CholeskyQR pass; 2: also one projection only
  int stall;      // test hook: CTA 0 first waits this many polls on a word nothing sets
  unsigned long long* phase_ns;  // optional: CTA 0's time per phase (diagnostics)
};

// diagnostics: CTA 0's thread 0 adds the time since the previous mark
// (kept in a.phase_ns[10]) to a.phase_ns[ph]
__device__ inline void op_mark(const OrthArgs& a, int ph) {
  if (a.phase_ns && blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long tn;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(tn));
    if (ph >= 0) a.phase_ns[ph] += tn - a.phase_ns[10];
    a.phase_ns[10] = tn;
  }
}

__host__ __device__ constexpr size_t op_smem_bytes(int ldy) {
  return (size_t)OP_R * ldy * sizeof(float2) + (size_t)OP_NBUF * OP_KC * OP_CLD * sizeof(float2) +
         (size_t)BW * CQ_RS * sizeof(float2) +
         (size_t)BW * BW * sizeof(float2) + OP_NT * sizeof(float2) + BW * sizeof(double) + (BW + 4) * sizeof(float);
}

__device__ inline int op_ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ inline void op_cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}

// Grid barrier: false (in every thread of the CTA) when a wait gave up.  The
// last CTA to arrive publishes the barrier's number in bar[2]; the others
// poll that word (written once per barrier), not the arrival counter.
__device__ bool op_barrier(const OrthArgs& a, int& epoch) {
  __syncthreads();
  epoch++;
  int ok = 1;
  if (threadIdx.x == 0) {
    __threadfence();
    const int arrived = atomicAdd(a.bar, 1) + 1;
    if (arrived == epoch * (int)gridDim.x) {
      asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(a.bar + 2), "r"(epoch) : "memory");
    } else {
      int it = 0;
      for (; it < a.spin; it++) {
        if (op_ld_acquire(a.bar + 2) >= epoch) break;
        if ((it & 7) == 7 && *(volatile int*)(a.bar + 1)) { it = a.spin; break; }
        __nanosleep(20);
      }
      if (it >= a.spin) {
        ok = 0;
        atomicExch(a.bar + 1, 1);
        atomicExch(a.status, 2);
      }
    }
    __threadfence();
  }
  return __syncthreads_and(ok) != 0;
}

// Projection of the block at column j0 (> 0) against the columns before it.
__device__ bool op_project(const OrthArgs& a, float2* Ys, float2* Cs, int j0, int& epoch) {
  const int t = threadIdx.x, c = blockIdx.x, nc = gridDim.x, L = a.ldy;
  // (1) partials: tile tau = (previous columns 4 kt .. 4 kt + 3, block columns 8 jt .. 8 jt + 7)
  float2* part = a.part + (size_t)c * a.l * BW;
  for (int tau = t; tau < j0; tau += OP_NT) {
    const int kt = tau >> 2, jt = tau & 3;
    float2 acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 8; j++) acc[i][j] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int r = 0; r < OP_R; r++) {
      const float4* q4 = (const float4*)(Ys + r * L + 4 * kt);
      const float4* y4 = (const float4*)(Ys + r * L + j0 + 8 * jt);
      const float4 qa = q4[0], qb = q4[1];
      const float2 q[4] = {make_float2(qa.x, qa.y), make_float2(qa.z, qa.w), make_float2(qb.x, qb.y),
                           make_float2(qb.z, qb.w)};
      float2 y[8];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float4 v = y4[u];
        y[2 * u] = make_float2(v.x, v.y);
        y[2 * u + 1] = make_float2(v.z, v.w);
      }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) cfma_conj(acc[i][j], q[i], y[j]);
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
      float4* dst = (float4*)(part + (size_t)(4 * kt + i) * BW + 8 * jt);
#pragma unroll
      for (int u = 0; u < 4; u++)
        __stcg(dst + u, make_float4(acc[i][2 * u].x, acc[i][2 * u].y, acc[i][2 * u + 1].x, acc[i][2 * u + 1].y));
    }
  }
  op_mark(a, 0);  // coefficient partials
  if (!op_barrier(a, epoch)) return false;
  op_mark(a, 1);  // barrier
  // (2) this CTA's slice of the j0 * BW coefficients, OP_NT entries at a
  // time: warp w adds the CTAs w S .. w S + S - 1 in order for 32
  // consecutive entries at a time (lane = entry: coalesced reads), then the
  // eight warp sums of each entry are added in order through shared memory
  // (the coefficient ring, idle here)
  {
    const int E = j0 * BW, per = (E + nc - 1) / nc, e_lo = c * per, e_hi = min(E, e_lo + per);
    const int w = t >> 5, lane = t & 31, S = (nc + 7) / 8, q0 = w * S, q1 = min(nc, q0 + S);
    const size_t stride = (size_t)a.l * BW;
    float2* ws = Cs;  // [8][OP_NT]
    for (int w0 = e_lo; w0 < e_hi; w0 += OP_NT) {
      for (int g = 0; g < OP_NT; g += 32) {
        const int e = w0 + g + lane;
        float2 sum = make_float2(0.f, 0.f);
        if (e < e_hi) {
#pragma unroll 8
          for (int q = q0; q < q1; q++) sum = cadd(sum, __ldcg(a.part + (size_t)q * stride + e));
        }
        ws[w * OP_NT + g + lane] = sum;
      }
      __syncthreads();
      const int e = w0 + t;
      if (e < e_hi) {
        float2 sum = ws[t];
#pragma unroll
        for (int u = 1; u < 8; u++) sum = cadd(sum, ws[u * OP_NT + t]);
        __stcg(a.coef + e, sum);
      }
      __syncthreads();
    }
  }
  op_mark(a, 2);  // coefficient sums
  if (!op_barrier(a, epoch)) return false;
  op_mark(a, 1);
  // (3) rows -= rows[:, :j0] coef: thread (rows 4 rt .., block columns 4 jt .., previous columns = ks mod 8)
  {
    const int ks = t & 7, jt = (t >> 3) & 7, rt = t >> 6;
    float2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = make_float2(0.f, 0.f);
    // the coefficients stream through a ring of OP_NBUF chunks of OP_KC
    // rows, OP_NBUF - 1 chunks in flight; every step commits one copy group
    // (empty past the last chunk), so waiting for all but the newest
    // OP_NBUF - 1 groups means chunk ch has landed
    const int nch = (j0 + OP_KC - 1) / OP_KC;  // j0 is a multiple of BW = OP_KC
    auto stage = [&](int ch) {
      if (ch < nch) {
        const float2* src = a.coef + (size_t)ch * OP_KC * BW;
        float2* dst = Cs + (ch % OP_NBUF) * OP_KC * OP_CLD;
        for (int p = t; p < OP_KC * BW / 2; p += OP_NT) {
          const int row = p / (BW / 2), c2 = p % (BW / 2);
          op_cp_async16(dst + row * OP_CLD + 2 * c2, src + row * BW + 2 * c2);
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
#pragma unroll 1
    for (int c = 0; c < OP_NBUF - 1; c++) stage(c);
    for (int ch = 0; ch < nch; ch++) {
      stage(ch + OP_NBUF - 1);  // into the buffer read in step ch - 1
      asm volatile("cp.async.wait_group %0;" ::"n"(OP_NBUF - 1) : "memory");
      __syncthreads();
      const float2* cs = Cs + (ch % OP_NBUF) * OP_KC * OP_CLD;
      const int k0 = ch * OP_KC;
#pragma unroll
      for (int kk = ks; kk < OP_KC; kk += 8) {
        float2 q[4];
#pragma unroll
        for (int i = 0; i < 4; i++) q[i] = Ys[(4 * rt + i) * L + k0 + kk];
        const float4 ca = *(const float4*)(cs + kk * OP_CLD + 4 * jt),
                     cb = *(const float4*)(cs + kk * OP_CLD + 4 * jt + 2);
        const float2 cv[4] = {make_float2(ca.x, ca.y), make_float2(ca.z, ca.w), make_float2(cb.x, cb.y),
                              make_float2(cb.z, cb.w)};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) cfma(acc[i][j], q[i], cv[j]);
      }
      __syncthreads();  // the buffer is restaged in the next step
    }
    // the eight previous-column slices added in order (Cs reused: 8 x 16 x 32 entries)
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) Cs[ks * (OP_R * BW) + (4 * rt + i) * BW + 4 * jt + j] = acc[i][j];
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int o = t + OP_NT * h, r = o / BW, j = o % BW;
      float2 v = Cs[o];
#pragma unroll
      for (int q = 1; q < 8; q++) v = cadd(v, Cs[q * (OP_R * BW) + o]);
      Ys[r * L + j0 + j] = csub(Ys[r * L + j0 + j], v);
    }
    __syncthreads();
  }
  op_mark(a, 3);  // projection update
  return true;
}

// One CholeskyQR pass of the block at column j0 (b columns).
__device__ bool op_cholqr(const OrthArgs& a, float2* Ys, float2* Gl, float2* Xs, float2* Tb, double* Gd, float* Ry,
                          int j0, int b, double shift, int& epoch) {
  const int t = threadIdx.x, c = blockIdx.x, nc = gridDim.x, L = a.ldy;
  // (1) partial Gram: thread (i = t mod 32, j = t / 32 + 8 u)
  {
    const int i = t & 31, jq = t >> 5;
    float2 g[4];
#pragma unroll
    for (int u = 0; u < 4; u++) g[u] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int r = 0; r < OP_R; r++) {
      const float2 yi = Ys[r * L + j0 + i];
#pragma unroll
      for (int u = 0; u < 4; u++) cfma_conj(g[u], yi, Ys[r * L + j0 + jq + 8 * u]);
    }
    float2* gp = a.gpart + (size_t)c * BW * BW;
#pragma unroll
    for (int u = 0; u < 4; u++) __stcg(gp + i + BW * (jq + 8 * u), g[u]);
  }
  op_mark(a, 4);  // Gram partials
  if (!op_barrier(a, epoch)) return false;
  op_mark(a, 1);
  // (2) this CTA's slice of the entries: warp w the entries e_lo + w + 8 v,
  // lane l the CTAs l, l + 32, ... in float-float, then a fixed shuffle tree
  {
    const int per = (BW * BW + nc - 1) / nc, e_lo = c * per, e_hi = min(BW * BW, e_lo + per);
    const int w = t >> 5, lane = t & 31;
    for (int e = e_lo + w; e < e_hi; e += OP_NT / 32) {
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int q = lane; q < nc; q += 32) {
        const float2 x = __ldcg(a.gpart + (size_t)q * BW * BW + e);
        v = ff4_add(v, make_float4(x.x, 0.f, x.y, 0.f));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        float4 u;
        u.x = __shfl_xor_sync(0xffffffffu, v.x, o);
        u.y = __shfl_xor_sync(0xffffffffu, v.y, o);
        u.z = __shfl_xor_sync(0xffffffffu, v.z, o);
        u.w = __shfl_xor_sync(0xffffffffu, v.w, o);
        v = ff4_add(v, u);
      }
      if (lane == 0) __stcg(a.gsum + e, v);
    }
  }
  op_mark(a, 5);  // Gram sums
  if (!op_barrier(a, epoch)) return false;
  op_mark(a, 1);
  // (3) the Gram in FP32 (diagonal in FP64), R, R^{-1}, rows <- rows R^{-1}
  for (int e = t; e < BW * BW; e += OP_NT) {
    const int i = e % BW, j = e / BW;
    if (i <= j) {
      const float4 v = __ldcg(a.gsum + e);
      Gl[i * CQ_RS + j] = make_float2(v.x + v.y, v.z + v.w);
      if (i == j) Gd[i] = (double)v.x + (double)v.y;
    }
  }
  __syncthreads();
  op_mark(a, 6);  // Gram gather
  cq_factor(Gl, Gd, Ry, Xs, Tb, b, shift, a.flags, c == 0);
  op_mark(a, 7);  // Cholesky + inverse
  {
    const int r = t >> 4, jc = 2 * (t & 15);
    float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll 8
    for (int k = 0; k < BW; k++) {
      const float2 y = Ys[r * L + j0 + k];
      if (k <= jc) cfma(a0, y, Xs[k * BW + jc]);
      if (k <= jc + 1) cfma(a1, y, Xs[k * BW + jc + 1]);
    }
    __syncthreads();  // every row of the block has been read
    Ys[r * L + j0 + jc] = a0;
    Ys[r * L + j0 + jc + 1] = a1;
    __syncthreads();
  }
  op_mark(a, 8);  // block update
  return true;
}

__global__ void __launch_bounds__(OP_NT, 1) orth_one_launch_kernel(OrthArgs a) {
  extern __shared__ __align__(16) unsigned char op_smem[];
  const int t = threadIdx.x, L = a.ldy;
  op_mark(a, -1);
  float2* Ys = (float2*)op_smem;          // [OP_R][L]
  float2* Cs = Ys + (size_t)OP_R * L;     // [OP_NBUF][OP_KC][OP_CLD]
  float2* Gl = Cs + OP_NBUF * OP_KC * OP_CLD;  // [BW][CQ_RS]
  float2* Xs = Gl + BW * CQ_RS;           // [BW][BW]
  float2* Tb = Xs + BW * BW;              // [OP_NT] scratch of the factor
  double* Gd = (double*)(Tb + OP_NT);     // [BW]
  float* Ry = (float*)(Gd + BW);          // [BW + 1]
  const int64_t r0 = (int64_t)blockIdx.x * OP_R;
  for (int e = t; e < OP_R * L; e += OP_NT) {
    const int rr = e % OP_R, cc = e / OP_R;
    const int64_t r = r0 + rr;
    Ys[rr * L + cc] = (r < a.m && cc < a.l) ? a.Y[r + a.m * (int64_t)cc] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  op_mark(a, 9);  // staging (the mark before it is the kernel start)
  if (a.stall > 0) {
    // test hook (QT_ORTH_STALL_TEST): CTA 0 waits a bounded number of polls
    // on bar[3], which nothing sets, then gives up like a barrier wait; the
    // other CTAs leave their first barrier through the abort word
    int gave = 0;
    if (blockIdx.x == 0 && t == 0) {
      int it = 0;
      for (; it < a.stall; it++) {
        if (op_ld_acquire(a.bar + 3) != 0) break;
        __nanosleep(20);
      }
      if (it >= a.stall) {
        gave = 1;
        atomicExch(a.bar + 1, 1);
        atomicExch(a.status, 2);
      }
    }
    if (__syncthreads_or(gave)) return;
  }
  int epoch = 0;
  for (int j0 = 0; j0 < a.l; j0 += BW) {
    const int b = min(BW, a.l - j0);
    const double shift = 11.0 * ((double)a.m * b + (double)b * (b + 1)) * 5.96e-8;
    if (j0 > 0) {
      if (!op_project(a, Ys, Cs, j0, epoch)) return;
      if (!op_cholqr(a, Ys, Gl, Xs, Tb, Gd, Ry, j0, b, shift, epoch)) return;
      if (a.light < 2 && !op_project(a, Ys, Cs, j0, epoch)) return;
      if (!op_cholqr(a, Ys, Gl, Xs, Tb, Gd, Ry, j0, b, 0.0, epoch)) return;
    } else {
      if (!op_cholqr(a, Ys, Gl, Xs, Tb, Gd, Ry, j0, b, shift, epoch)) return;
      if (!op_cholqr(a, Ys, Gl, Xs, Tb, Gd, Ry, j0, b, 0.0, epoch)) return;
    }
    if (a.light == 0 && !op_cholqr(a, Ys, Gl, Xs, Tb, Gd, Ry, j0, b, 0.0, epoch)) return;
  }
  for (int e = t; e < OP_R * a.l; e += OP_NT) {
    const int rr = e % OP_R, cc = e / OP_R;
    const int64_t r = r0 + rr;
    if (r < a.m) a.Y[r + a.m * (int64_t)cc] = Ys[rr * L + cc];
  }
}

// CTAs and row stride of the one-launch orthonormalisation of an m x l FP32
// basis; 0 when it does not apply (QT_ORTH_ONE_LAUNCH=0, no cooperative
// launch, the rows' columns beyond shared memory, or more CTAs than fit).
int op_shape(int64_t m, int64_t l, int* ldy, size_t* smem) {
  static int sms = -1, max_smem = 0;
  if (sms < 0) {
    int dev = 0, coop = 0;
    cudaFuncAttributes fa;
    sms = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop &&
        cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess &&
        cudaFuncGetAttributes(&fa, orth_one_launch_kernel) == cudaSuccess) {
      max_smem -= (int)fa.sharedSizeBytes;  // the dynamic part's limit
      if (cudaFuncSetAttribute(orth_one_launch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem) ==
          cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    cudaGetLastError();
  }
  const char* env = std::getenv("QT_ORTH_ONE_LAUNCH");
  if ((env && env[0] == '0') || sms <= 0) return 0;
  *ldy = (int)((l + BW - 1) / BW * BW + 2);
  *smem = op_smem_bytes(*ldy);
  if (*smem > (size_t)max_smem) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, orth_one_launch_kernel, OP_NT, *smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int64_t ncta = (m + OP_R - 1) / OP_R;
  return (ncta <= (int64_t)per_sm * sms && ncta <= OP_MAXCTA) ? (int)ncta : 0;
}

int orth_one_launch(qt_handle* h, float2* Y, int64_t m, int64_t l, int ncta, int ldy, size_t smem, int light) {
  qt_scratch s(h);
  OrthArgs a;
  a.Y = Y;
  a.m = m;
  a.l = (int)l;
  a.ldy = ldy;
  QT_TRY(s.get(&a.part, (size_t)ncta * l * BW));
  QT_TRY(s.get(&a.coef, (size_t)l * BW));
  QT_TRY(s.get(&a.gpart, (size_t)ncta * BW * BW));
  QT_TRY(s.get(&a.gsum, (size_t)BW * BW));
  QT_TRY(s.get(&a.bar, 4));
  a.flags = h->d_flags;
  a.status = h->d_status;
  if (!a.status) QT_TRY(s.get(&a.status, 1));
  a.spin = OP_SPIN;
  a.light = light;
  // QT_ORTH_STALL_TEST=N (tests only): CTA 0 gives up a wait after N polls
  a.stall = std::getenv("QT_ORTH_STALL_TEST") ? std::atoi(std::getenv("QT_ORTH_STALL_TEST")) : 0;
  a.phase_ns = nullptr;
  // QT_ORTH_PHASES=1 prints CTA 0's time per phase after each launch
  static const bool phases = std::getenv("QT_ORTH_PHASES") != nullptr;
  if (phases && h->pool) {
    QT_TRY(s.get(&a.phase_ns, 11));
    QT_CHECK_CUDA(h, cudaMemsetAsync(a.phase_ns, 0, 11 * sizeof(unsigned long long), h->stream));
  }
  QT_CHECK_CUDA(h, cudaMemsetAsync(a.bar, 0, 4 * sizeof(int), h->stream));
  if (a.status != h->d_status) QT_CHECK_CUDA(h, cudaMemsetAsync(a.status, 0, sizeof(int), h->stream));
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)ncta);
  lc.blockDim = dim3(OP_NT);
  lc.dynamicSmemBytes = smem;
  lc.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  if (h->prof) qt_prof_before(h, "orth_one_launch_kernel");
  const cudaError_t e = cudaLaunchKernelEx(&lc, orth_one_launch_kernel, a);
  if (h->prof) qt_prof_after(h);
  h->launches++;
  if (e != cudaSuccess)
    return qt_fail(h, QT_ECUDA, std::string("launch orth_one_launch_kernel: ") + cudaGetErrorString(e));
  if (a.status != h->d_status) {  // a handle without a status word: check here
    int hs = 0;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(&hs, a.status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hs) return qt_fail(h, QT_ETIMEOUT, "orthonormalize: a grid barrier wait timed out");
  }
  if (a.phase_ns) {
    unsigned long long hp[10];
    QT_CHECK_CUDA(h, cudaMemcpyAsync(hp, a.phase_ns, sizeof(hp), cudaMemcpyDeviceToHost, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    const char* nm[10] = {"coef partials", "barriers", "coef sums", "projection update", "Gram partials",
                          "Gram sums", "Gram gather", "Cholesky+inverse", "block update", "staging"};
    std::fprintf(stderr, "one-launch orthonormalisation %lldx%lld (%d CTAs), us per launch:", (long long)m,
                 (long long)l, ncta);
    for (int i = 0; i < 10; i++) std::fprintf(stderr, " %s %.1f", nm[i], hp[i] * 1e-3);
    std::fprintf(stderr, "\n");
  }
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
int qt_orthonormalize(qt_handle* h, C* Y, int64_t m, int64_t l, int use) {
  if (l > m) return qt_fail(h, QT_EINVAL, "orthonormalize: more columns than rows");
  if constexpr (std::is_same<C, float2>::value) {
    int ldy = 0;
    size_t smem = 0;
    const int ncta = op_shape(m, l, &ldy, &smem);
    // A basis that only carries a range to the next product of a power
    // iteration needs to be well conditioned, not orthonormal to rounding:
    // one projection and two CholeskyQR passes per block (QT_ORTH_RANGE=2,
    // the default; 1 keeps both projections, 0 all three passes).  At the
    // chi = 1024 bench bond that leaves the truncation error unchanged
    // (1.00014 of the exact split with a three-pass final basis) and saves
    // 4.8 ms per update.  The final basis of a sketch keeps both
    // projections and drops the third pass (QT_ORTH_FINAL=1, the default; 0
    // restores it): a second CholeskyQR after the shifted one already leaves
    // the block orthonormal to a few u, and the split that follows projects
    // theta' exactly (B' = A'^H theta').  A basis kept as such (an MPS site)
    // takes all passes.
    const char* env = std::getenv("QT_ORTH_RANGE");
    const char* fenv = std::getenv("QT_ORTH_FINAL");
    const int light = use == QT_ORTH_USE_RANGE ? (env ? std::atoi(env) : 2)
                      : use == QT_ORTH_USE_SKETCH ? (fenv ? std::atoi(fenv) : 1) : 0;
    if (ncta > 0) return orth_one_launch(h, Y, m, l, ncta, ldy, smem, std::min(2, std::max(0, light)));
  }
  qt_scratch s(h);
  double2* dG;
  C *coef, *part;
  const int64_t nchunk = (m + PJ_ROWS - 1) / PJ_ROWS, lpad = (l + PJ_K - 1) / PJ_K * PJ_K;
  QT_TRY(s.get(&dG, 2 * BW * BW));
  QT_TRY(s.get(&coef, (size_t)l * BW));
  QT_TRY(s.get(&part, (size_t)nchunk * lpad * BW));
  int nrb = 0, cs = 0;
  unsigned long long* phase_ns = nullptr;
  // QT_CHOLQR_PHASES=1 prints the average SM cycles per phase of the
  // cluster CholeskyQR (CTA 0's clock) after each orthonormalisation
  static const bool phases = std::getenv("QT_CHOLQR_PHASES") != nullptr;
  if constexpr (std::is_same<C, float2>::value) {
    nrb = cq_shape(m, &cs);
    if (nrb > 0 && phases) {
      QT_TRY(s.get(&phase_ns, 16));
      QT_CHECK_CUDA(h, cudaMemsetAsync(phase_ns, 0, 16 * sizeof(unsigned long long), h->stream));
    }
  }
  int cq_launches = 0, cq_passes = 0;
  for (int64_t j0 = 0; j0 < l; j0 += BW) {
    const int b = (int)std::min<int64_t>(BW, l - j0);
    C* Yb = Y + m * j0;
    if constexpr (std::is_same<C, float2>::value) {
      if (nrb > 0) {
        // the same passes as below with each run of CholeskyQR passes in one
        // cluster launch: shifted, (projection,) plain, plain
        if (j0 > 0) {
          QT_TRY(block_project<C>(h, Y, m, (int)j0, Yb, b, part, coef));
          QT_TRY(block_cholqr_cluster(h, Yb, m, b, nrb, cs, 1, true, phase_ns));
          QT_TRY(block_project<C>(h, Y, m, (int)j0, Yb, b, part, coef));
          QT_TRY(block_cholqr_cluster(h, Yb, m, b, nrb, cs, 2, false, phase_ns));
          cq_launches += 2;
          cq_passes += 3;
        } else {
          QT_TRY(block_cholqr_cluster(h, Yb, m, b, nrb, cs, 3, true, phase_ns));
          cq_launches += 1;
          cq_passes += 3;
        }
        continue;
      }
    }
    for (int pass = 0; pass < 2; pass++) {
      if (j0 > 0) QT_TRY(block_project<C>(h, Y, m, (int)j0, Yb, b, part, coef));
      QT_TRY(block_cholqr<C>(h, Yb, m, b, pass == 0, dG));
    }
    // one more CholeskyQR (shifted CholeskyQR3): after a shifted pass with
    // the FP32 shift the block is only well conditioned, not orthonormal
    if (sizeof(typename real_of<C>::type) == 4) QT_TRY(block_cholqr<C>(h, Yb, m, b, false, dG));
  }
  if (phase_ns && cq_launches > 0) {
    unsigned long long hp[8];
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    QT_CHECK_CUDA(h, cudaMemcpy(hp, phase_ns, sizeof(hp), cudaMemcpyDeviceToHost));
    const char* nm[8] = {"stage", "gram", "groups+barrier", "scatter+barrier", "gather", "cholesky+inverse",
                         "update", "writeback+barrier"};
    std::fprintf(stderr, "cluster CholeskyQR (%d CTAs of %d rows), %d launches, %d passes; SM kilocycles per "
                 "launch (stage, writeback) or pass:", cs, 32 * nrb, cq_launches, cq_passes);
    for (int i = 0; i < 8; i++)
      std::fprintf(stderr, " %s %.2f", nm[i], hp[i] * 1e-3 / (i == 0 || i == 7 ? cq_launches : cq_passes));
    std::fprintf(stderr, "\n");
  }
  return QT_OK;
}
template int qt_orthonormalize<float2>(qt_handle*, float2*, int64_t, int64_t, int);
template int qt_orthonormalize<double2>(qt_handle*, double2*, int64_t, int64_t, int);
