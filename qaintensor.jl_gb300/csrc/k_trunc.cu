// Truncation and split: singular values from converged Jacobi columns, the
// absolute tail-norm rank rule of src/svd.jl:29-33, and the split of
// src/switch.jl:42-53: U[:, 1:k] -> left site, diag(S) V'[1:k, :]
// -> right site.
#include <cuda_runtime.h>

#include <cmath>

#include "qt_internal.cuh"

namespace {

// sigma_j = ||x_j|| in FP64, one CTA per column.
template <typename TS>
__global__ void column_norms_kernel(const TS* __restrict__ X, int64_t mm, int64_t ldx, double* __restrict__ sig) {
  const int64_t j = blockIdx.x;
  double s = 0;
  for (int64_t i = threadIdx.x; i < mm; i += blockDim.x) {
    const double re = X[i + ldx * j].x, im = X[i + ldx * j].y;
    s = fma(re, re, s);
    s = fma(im, im, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
    sig[j] = sqrt(tot);
  }
}

// Single-CTA bitonic sort, descending by value, of up to 8192 (value, index).
__global__ void sort_desc_kernel(double* __restrict__ val, int* __restrict__ idx, int n, int npow2) {
  extern __shared__ unsigned char smem[];
  double* v = reinterpret_cast<double*>(smem);
  int* ix = reinterpret_cast<int*>(v + npow2);
  for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
    v[i] = (i < n) ? val[i] : -1.0;
    ix[i] = i;
  }
  __syncthreads();
  for (int k = 2; k <= npow2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const bool desc = ((i & k) == 0);
          const double a = v[i], b = v[l];
          // descending blocks keep the larger value first; ties by index
          const bool swap = desc ? (a < b || (a == b && ix[i] > ix[l])) : (a > b || (a == b && ix[i] < ix[l]));
          if (swap) {
            v[i] = b; v[l] = a;
            const int t = ix[i]; ix[i] = ix[l]; ix[l] = t;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    val[i] = v[i];
    idx[i] = ix[i];
  }
}

// Left site A' (m x k): column j is the unit vector belonging to the j-th
// largest singular value.  Not transposed: X[:, perm j] / sigma_j.
// Transposed (X holds theta^H): the V factor's column perm j.
template <typename TS, typename TO>
__global__ void absorb_left_kernel(int transposed, const TS* __restrict__ X, int64_t ldx, const TS* __restrict__ Vx,
                                   int64_t ldv, const double* __restrict__ sig, const int* __restrict__ perm,
                                   int64_t m, int k, TO* __restrict__ A) {
  const int j = blockIdx.y;
  const int pj = perm[j];
  const double s = sig[j];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    double2 v;
    if (!transposed) {
      v = ccast<double2>(X[i + ldx * pj]);
      const double inv = (s > 0) ? 1.0 / s : 0.0;
      v.x *= inv; v.y *= inv;
    } else {
      v = ccast<double2>(Vx[i + ldv * pj]);
    }
    A[i + m * (int64_t)j] = ccast<TO>(v);
  }
}

// Right site B' (k x n): row j = sscale * sigma_j * V[:, perm j]^H (not
// transposed) or sscale * X[:, perm j]^H (transposed).  32x32 tiles.
template <typename TS, typename TO>
__global__ void absorb_right_kernel(int transposed, const TS* __restrict__ X, int64_t ldx, const TS* __restrict__ Vx,
                                    int64_t ldv, const double* __restrict__ sig, const int* __restrict__ perm,
                                    int64_t n, int k, double sscale, TO* __restrict__ B) {
  __shared__ double2 tile[32][33];
  const int64_t c0 = blockIdx.x * 32;
  const int j0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int j = j0 + r;
    const int64_t c = c0 + threadIdx.x;
    double2 v = make_double2(0, 0);
    if (j < k && c < n) {
      const int pj = perm[j];
      if (!transposed) {
        v = ccast<double2>(Vx[c + ldv * pj]);
        const double f = sscale * sig[j];
        v.x *= f; v.y *= -f;
      } else {
        v = ccast<double2>(X[c + ldx * pj]);
        v.x *= sscale; v.y *= -sscale;
      }
    }
    tile[r][threadIdx.x] = v;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int64_t c = c0 + r;
    const int j = j0 + threadIdx.x;
    if (j < k && c < n) B[j + (int64_t)k * c] = ccast<TO>(tile[threadIdx.x][r]);
  }
}

}  // namespace

template <typename TS>
int qt_sorted_column_norms(qt_handle* h, const TS* X, int64_t mm, int64_t nn, int64_t ldx, double* d_sigma,
                           int* d_perm) {
  if (nn > 8192) return qt_fail(h, QT_ENOTSUP, "sort: more than 8192 singular values");
  QT_LAUNCH(h, column_norms_kernel<TS>, (unsigned)nn, 256, 0, X, mm, ldx, d_sigma);
  int np2 = 1;
  while (np2 < nn) np2 <<= 1;
  const size_t smem = (size_t)np2 * (sizeof(double) + sizeof(int));
  if (smem > 48 * 1024) QT_CHECK_CUDA(h, cudaFuncSetAttribute(sort_desc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  QT_LAUNCH(h, sort_desc_kernel, 1, 1024, smem, d_sigma, d_perm, (int)nn, np2);
  return QT_OK;
}
template int qt_sorted_column_norms<double2>(qt_handle*, const double2*, int64_t, int64_t, int64_t, double*, int*);
template int qt_sorted_column_norms<float2>(qt_handle*, const float2*, int64_t, int64_t, int64_t, double*, int*);

// src/svd.jl:29-33 on a descending spectrum: the cumulative sum of squares
// runs from the smallest value upward, sequentially, exactly as Julia's (and
// numpy's) cumsum does; k = smallest count with sqrt(tail) <= cutoff.  When
// no tail exceeds the cutoff the reference throws; the engine keeps k = 1.
int qt_tail_rule_host(const std::vector<double>& s, double cutoff, int* k_cutoff) {
  const int n = (int)s.size();
  double acc = 0.0;
  int k = 1;
  for (int i = n - 1; i >= 0; i--) {
    acc = acc + s[i] * s[i];
    if (std::sqrt(acc) > cutoff) { k = i + 1; break; }
  }
  *k_cutoff = k;
  return k;
}

template <typename TS, typename TO>
int qt_absorb(qt_handle* h, int transposed, const TS* X, int64_t ldx, const TS* Vx, int64_t ldv, const double* d_sigma,
              const int* d_perm, int64_t m, int64_t n, int k, double sscale, TO* Aout, TO* Bout) {
  if (m > 0) {
    dim3 gl((unsigned)((m + 255) / 256), (unsigned)k);
    QT_LAUNCH(h, (absorb_left_kernel<TS, TO>), gl, 256, 0, transposed, X, ldx, Vx, ldv, d_sigma, d_perm, m, k, Aout);
  }
  dim3 gr((unsigned)((n + 31) / 32), (unsigned)((k + 31) / 32));
  QT_LAUNCH(h, (absorb_right_kernel<TS, TO>), gr, dim3(32, 8), 0, transposed, X, ldx, Vx, ldv, d_sigma, d_perm, n, k,
            sscale, Bout);
  return QT_OK;
}
template int qt_absorb<double2, double2>(qt_handle*, int, const double2*, int64_t, const double2*, int64_t,
                                         const double*, const int*, int64_t, int64_t, int, double, double2*, double2*);
template int qt_absorb<double2, float2>(qt_handle*, int, const double2*, int64_t, const double2*, int64_t,
                                        const double*, const int*, int64_t, int64_t, int, double, float2*, float2*);
template int qt_absorb<float2, float2>(qt_handle*, int, const float2*, int64_t, const float2*, int64_t, const double*,
                                       const int*, int64_t, int64_t, int, double, float2*, float2*);
template int qt_absorb<float2, double2>(qt_handle*, int, const float2*, int64_t, const float2*, int64_t,
                                        const double*, const int*, int64_t, int64_t, int, double, double2*, double2*);
