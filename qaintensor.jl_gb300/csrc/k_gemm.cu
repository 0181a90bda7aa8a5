// Contraction kernels: the two-site theta formation with the gate folded into
// the epilogue, a generic column-major complex GEMM, and element helpers.
//
// theta = A_mat (2chiL x chiM) . B_mat (chiM x 2chiR) is the pairwise ncon
// step of src/contract.jl:257,263 for two neighbouring MPS sites (the two-site
// contraction of src/switch.jl:26).  The gate acts on the input
// legs, G[o1 + 2 o2, i1 + 2 i2] (src/decompose.jl:16-31, src/mpo.jl:41-57).
#include <cuda_runtime.h>

#include "qt_internal.cuh"

namespace {

struct GateParam {
  double2 g[16];  // column-major 4x4: g[row + 4 * col]
};

// Each CTA owns a block of TA values of a and TB values of b and computes all
// four (s1, s2) combinations for them, so the 4x4 gate mixes values that sit
// in one thread's registers.  Thread (tx, ty) owns a = a0 + tx + 16 i,
// b = b0 + ty + 16 j.  Accumulation in R (double or float).
template <typename TI, typename R, typename TO, int RA, int RB>
__global__ void __launch_bounds__(256)
theta_gate_kernel(const TI* __restrict__ A, const TI* __restrict__ B, int chil, int chim, int chir,
                  GateParam gp, TO* __restrict__ out) {
  typedef typename cplx_of<R>::type CR;
  constexpr int TA = 16 * RA, TB = 16 * RB, KC = 16;
  __shared__ CR As[2][KC][TA];
  __shared__ CR Bs[2][KC][TB + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int a0 = blockIdx.x * TA, b0 = blockIdx.y * TB;
  CR acc[RA][RB][2][2];
#pragma unroll
  for (int i = 0; i < RA; i++)
#pragma unroll
    for (int j = 0; j < RB; j++)
#pragma unroll
      for (int s = 0; s < 4; s++) acc[i][j][s >> 1][s & 1] = czero<CR>();

  for (int k0 = 0; k0 < chim; k0 += KC) {
    for (int idx = threadIdx.x; idx < 2 * KC * TA; idx += 256) {
      const int a = idx % TA, k = (idx / TA) % KC, s = idx / (TA * KC);
      const int ga = a0 + a, gk = k0 + k;
      CR v = czero<CR>();
      if (ga < chil && gk < chim) v = ccast<CR>(A[ga + (int64_t)chil * (s + 2 * (int64_t)gk)]);
      As[s][k][a] = v;
    }
    for (int idx = threadIdx.x; idx < 2 * KC * TB; idx += 256) {
      const int k = idx % KC, b = (idx / KC) % TB, s = idx / (KC * TB);
      const int gb = b0 + b, gk = k0 + k;
      CR v = czero<CR>();
      if (gb < chir && gk < chim) v = ccast<CR>(B[gk + (int64_t)chim * (s + 2 * (int64_t)gb)]);
      Bs[s][k][b] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < KC; k++) {
      CR av[RA][2], bv[RB][2];
#pragma unroll
      for (int i = 0; i < RA; i++) {
        av[i][0] = As[0][k][tx + 16 * i];
        av[i][1] = As[1][k][tx + 16 * i];
      }
#pragma unroll
      for (int j = 0; j < RB; j++) {
        bv[j][0] = Bs[0][k][ty + 16 * j];
        bv[j][1] = Bs[1][k][ty + 16 * j];
      }
#pragma unroll
      for (int i = 0; i < RA; i++)
#pragma unroll
        for (int j = 0; j < RB; j++)
#pragma unroll
          for (int s = 0; s < 4; s++) cfma(acc[i][j][s >> 1][s & 1], av[i][s >> 1], bv[j][s & 1]);
    }
    __syncthreads();
  }

  CR g[16];
#pragma unroll
  for (int e = 0; e < 16; e++) g[e] = ccast<CR>(gp.g[e]);
  const int64_t ldo = 2 * (int64_t)chil;
#pragma unroll
  for (int i = 0; i < RA; i++) {
    const int a = a0 + tx + 16 * i;
    if (a >= chil) continue;
#pragma unroll
    for (int j = 0; j < RB; j++) {
      const int b = b0 + ty + 16 * j;
      if (b >= chir) continue;
#pragma unroll
      for (int o = 0; o < 4; o++) {
        const int o1 = o & 1, o2 = o >> 1;
        CR v = czero<CR>();
#pragma unroll
        for (int q = 0; q < 4; q++) cfma(v, g[o + 4 * q], acc[i][j][q & 1][q >> 1]);
        out[(a + (int64_t)chil * o1) + ldo * (o2 + 2 * (int64_t)b)] = ccast<TO>(v);
      }
    }
  }
}

// Generic complex GEMM, 64x64 output tile, 16-deep K slices, 4x4 per thread.
template <typename C>
__global__ void __launch_bounds__(256)
cgemm_kernel(int opA, int opB, int M, int N, int K, C alpha, const C* __restrict__ A, int64_t lda,
             const C* __restrict__ B, int64_t ldb, C beta, C* __restrict__ Cm, int64_t ldc) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ C As[BK][BM + 1];
  __shared__ C Bs[BK][BN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  C acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = czero<C>();

  for (int k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int idx = threadIdx.x + 256 * r;
      int m, k;
      if (opA == QT_OP_N) { m = idx % BM; k = idx / BM; } else { k = idx % BK; m = idx / BK; }
      const int gm = m0 + m, gk = k0 + k;
      C v = czero<C>();
      if (gm < M && gk < K) {
        if (opA == QT_OP_N) v = A[gm + lda * gk];
        else { v = A[gk + lda * gm]; if (opA == QT_OP_C) v = cconj(v); }
      }
      As[k][m] = v;
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int idx = threadIdx.x + 256 * r;
      int n, k;
      if (opB == QT_OP_N) { k = idx % BK; n = idx / BK; } else { n = idx % BN; k = idx / BN; }
      const int gn = n0 + n, gk = k0 + k;
      C v = czero<C>();
      if (gn < N && gk < K) {
        if (opB == QT_OP_N) v = B[gk + ldb * gn];
        else { v = B[gn + ldb * gk]; if (opB == QT_OP_C) v = cconj(v); }
      }
      Bs[k][n] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < BK; k++) {
      C a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[k][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[k][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) cfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  const bool use_beta = (beta.x != 0 || beta.y != 0);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int m = m0 + tx + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int n = n0 + ty + 16 * j;
      if (n >= N) continue;
      C v = cmul(alpha, acc[i][j]);
      if (use_beta) v = cadd(v, cmul(beta, Cm[m + ldc * n]));
      Cm[m + ldc * n] = v;
    }
  }
}

template <typename S, typename D>
__global__ void convert_kernel(const S* __restrict__ src, D* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = ccast<D>(src[i]);
}

// dst (n x m) = src^H, src (m x n); 32x32 tiles through shared memory.
template <typename C>
__global__ void adjoint_kernel(const C* __restrict__ src, int64_t m, int64_t n, int64_t lds, C* __restrict__ dst,
                               int64_t ldd) {
  __shared__ C tile[32][33];
  const int64_t i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int64_t i = i0 + threadIdx.x, j = j0 + r;
    if (i < m && j < n) tile[r][threadIdx.x] = src[i + lds * j];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int64_t j = j0 + threadIdx.x, i = i0 + r;
    if (i < m && j < n) dst[j + ldd * i] = cconj(tile[threadIdx.x][r]);
  }
}

template <typename C>
__global__ void identity_kernel(C* V, int64_t n, int64_t ld) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n * n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % n, j = idx / n;
    C v = czero<C>();
    if (i == j) v.x = 1;
    V[i + ld * j] = v;
  }
}

template <typename C>
__global__ void norm2_kernel(const C* __restrict__ x, int64_t n, double* out) {
  double s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double re = x[i].x, im = x[i].y;
    s = fma(re, re, s);
    s = fma(im, im, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(out, s);
  }
}

// theta'(a,o1,o2,b) = sum G[o1+2o2, i1+2i2] theta(a,i1,i2,b), in place; one
// thread per (a, b) owns the four physical values.
__global__ void gate_inplace_kernel(float2* __restrict__ th, int chil, int chir, GateParam gp) {
  const int64_t ldo = 2 * (int64_t)chil;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)chil * chir;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = idx % chil, b = idx / chil;
    float2 v[4];
#pragma unroll
    for (int q = 0; q < 4; q++) v[q] = th[(a + chil * (q & 1)) + ldo * ((q >> 1) + 2 * b)];
#pragma unroll
    for (int o = 0; o < 4; o++) {
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < 4; q++) cfma(acc, ccast<float2>(gp.g[o + 4 * q]), v[q]);
      th[(a + chil * (o & 1)) + ldo * ((o >> 1) + 2 * b)] = acc;
    }
  }
}

inline int grid1d(int64_t n, int block = 256) {
  int64_t g = (n + block - 1) / block;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

int qt_theta_gate(qt_handle* h, int dtype_in, const void* A, const void* B, int64_t chil, int64_t chim,
                  int64_t chir, const double* G, int prec, void* theta_out) {
  GateParam gp;
  for (int e = 0; e < 16; e++) gp.g[e] = make_double2(G[2 * e], G[2 * e + 1]);
  if (chil <= 0 || chim <= 0 || chir <= 0) return qt_fail(h, QT_EINVAL, "theta: empty bond");
  if (prec == 0) {
    dim3 grid((unsigned)((chil + 15) / 16), (unsigned)((chir + 15) / 16));
    if (dtype_in == QT_C128)
      QT_LAUNCH(h, (theta_gate_kernel<double2, double, double2, 1, 1>), grid, 256, 0, (const double2*)A,
                (const double2*)B, (int)chil, (int)chim, (int)chir, gp, (double2*)theta_out);
    else
      QT_LAUNCH(h, (theta_gate_kernel<float2, double, double2, 1, 1>), grid, 256, 0, (const float2*)A,
                (const float2*)B, (int)chil, (int)chim, (int)chir, gp, (double2*)theta_out);
  } else {
    dim3 grid((unsigned)((chil + 31) / 32), (unsigned)((chir + 31) / 32));
    if (dtype_in == QT_C128)
      QT_LAUNCH(h, (theta_gate_kernel<double2, float, float2, 2, 2>), grid, 256, 0, (const double2*)A,
                (const double2*)B, (int)chil, (int)chim, (int)chir, gp, (float2*)theta_out);
    else
      QT_LAUNCH(h, (theta_gate_kernel<float2, float, float2, 2, 2>), grid, 256, 0, (const float2*)A,
                (const float2*)B, (int)chil, (int)chim, (int)chir, gp, (float2*)theta_out);
  }
  return QT_OK;
}

int qt_apply_gate_inplace(qt_handle* h, float2* theta, int64_t chil, int64_t chir, const double* G) {
  GateParam gp;
  for (int e = 0; e < 16; e++) gp.g[e] = make_double2(G[2 * e], G[2 * e + 1]);
  QT_LAUNCH(h, gate_inplace_kernel, grid1d(chil * chir), 256, 0, theta, (int)chil, (int)chir, gp);
  return QT_OK;
}

template <typename C>
int qt_cgemm(qt_handle* h, int opA, int opB, int64_t M, int64_t N, int64_t K, C alpha, const C* A, int64_t lda,
             const C* B, int64_t ldb, C beta, C* Cm, int64_t ldc) {
  if (M <= 0 || N <= 0) return QT_OK;
  dim3 grid((unsigned)((M + 63) / 64), (unsigned)((N + 63) / 64));
  QT_LAUNCH(h, cgemm_kernel<C>, grid, 256, 0, opA, opB, (int)M, (int)N, (int)K, alpha, A, lda, B, ldb, beta, Cm,
            ldc);
  return QT_OK;
}
template int qt_cgemm<float2>(qt_handle*, int, int, int64_t, int64_t, int64_t, float2, const float2*, int64_t,
                              const float2*, int64_t, float2, float2*, int64_t);
template int qt_cgemm<double2>(qt_handle*, int, int, int64_t, int64_t, int64_t, double2, const double2*, int64_t,
                               const double2*, int64_t, double2, double2*, int64_t);

int qt_convert(qt_handle* h, const void* src, int sd, void* dst, int dd, int64_t n) {
  if (n <= 0) return QT_OK;
  const int g = grid1d(n);
  if (sd == QT_C64 && dd == QT_C128) QT_LAUNCH(h, (convert_kernel<float2, double2>), g, 256, 0, (const float2*)src, (double2*)dst, n);
  else if (sd == QT_C128 && dd == QT_C64) QT_LAUNCH(h, (convert_kernel<double2, float2>), g, 256, 0, (const double2*)src, (float2*)dst, n);
  else if (sd == QT_C64) QT_LAUNCH(h, (convert_kernel<float2, float2>), g, 256, 0, (const float2*)src, (float2*)dst, n);
  else QT_LAUNCH(h, (convert_kernel<double2, double2>), g, 256, 0, (const double2*)src, (double2*)dst, n);
  return QT_OK;
}

template <typename C>
int qt_adjoint_copy(qt_handle* h, const C* src, int64_t m, int64_t n, int64_t lds, C* dst, int64_t ldd) {
  dim3 grid((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
  QT_LAUNCH(h, adjoint_kernel<C>, grid, dim3(32, 8), 0, src, m, n, lds, dst, ldd);
  return QT_OK;
}
template int qt_adjoint_copy<float2>(qt_handle*, const float2*, int64_t, int64_t, int64_t, float2*, int64_t);
template int qt_adjoint_copy<double2>(qt_handle*, const double2*, int64_t, int64_t, int64_t, double2*, int64_t);

template <typename C>
int qt_set_identity(qt_handle* h, C* V, int64_t n, int64_t ld) {
  QT_LAUNCH(h, identity_kernel<C>, grid1d(n * n), 256, 0, V, n, ld);
  return QT_OK;
}
template int qt_set_identity<float2>(qt_handle*, float2*, int64_t, int64_t);
template int qt_set_identity<double2>(qt_handle*, double2*, int64_t, int64_t);

template <typename C>
int qt_norm2(qt_handle* h, const C* x, int64_t n, double* d_out) {
  QT_CHECK_CUDA(h, cudaMemsetAsync(d_out, 0, sizeof(double), h->stream));
  QT_LAUNCH(h, norm2_kernel<C>, grid1d(n), 256, 0, x, n, d_out);
  return QT_OK;
}
template int qt_norm2<float2>(qt_handle*, const float2*, int64_t, double*);
template int qt_norm2<double2>(qt_handle*, const double2*, int64_t, double*);
