// Truncated SVD for callers that cannot allocate device memory.
//
// Some callers own every byte of device memory themselves -- an embedding
// framework with a fixed memory budget or its own arena, or code running
// where a cudaMalloc would synchronise the device or is not permitted -- and
// can hand the library only the input and output buffers.  This entry point
// serves them: its scratch (the working copy of the matrix, the Jacobi
// rotations, the partial Grams, the singular values and status words) lives
// in one file-scope __device__ array of fixed size, so it calls no
// cudaMalloc, cudaFree or allocating library routine.
//
// Limits and rules:
//   * m, n <= 256; larger sizes are rejected with QT_ENOTSUP.  The array
//     (NA_BYTES, about 2.6 MB: 1 MiB each for the working matrix and the
//     rotations, 516 KiB of Jacobi workspace, the values and status words)
//     stays allocated on every device that loads the library until the
//     process exits.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, that device current); make that
//     first call before any stream capture.  The address is kept for the
//     life of the process: after a cudaDeviceReset the library must be
//     reloaded before this entry point is used again on that device.
//   * Failures come back as the status code only (there is no handle to
//     carry a message).  The Jacobi phase counters of QT_JACOBI_PHASES are
//     not collected here, since they would need an allocation.
//   * All calls share the one array and each call leaves its contents
//     behind; calls that overlap on the GPU (different streams or threads)
//     race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "qt_internal.cuh"

namespace {

constexpr int64_t NA_MAX = 256;
constexpr size_t NA_X = (size_t)NA_MAX * NA_MAX;           // working matrix (max(m,n) x min(m,n))
constexpr size_t NA_V = (size_t)NA_MAX * NA_MAX;           // accumulated rotations
constexpr size_t NA_PARTS = 16 * 8 * 256 + 256;            // Jacobi workspace (partial Grams, pair unitaries, flags)
constexpr size_t NA_SIG = NA_MAX;                          // singular values
constexpr size_t NA_BYTES = sizeof(double2) * (NA_X + NA_V + NA_PARTS) + sizeof(double) * NA_SIG +
                            sizeof(int) * (NA_MAX + QT_FLAG_COUNT) + 256;
static_assert(NA_BYTES > 2600000 && NA_BYTES < 2700000, "the documented size of the scratch array is about 2.6 MB");

__device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

std::mutex g_na_mutex;
void* g_na_addr[64] = {};

__global__ void scale_rows_inv_kernel(double2* Vh, int k, int64_t n, const double* sig) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)k * n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(idx % k);
    const double s = sig[j];
    const double f = s > 0 ? 1.0 / s : 0.0;
    Vh[idx] = cscale(Vh[idx], f);
  }
}

}  // namespace

extern "C" int qt_truncated_svd_noalloc(int64_t m, int64_t n, const void* dM, double cutoff, int chi_max, void* dU,
                                        double* dS, void* dVh, int* k_out, void* stream_ptr) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
  if (!dM || !dU || !dS || !dVh || !k_out) return QT_EINVAL;
  if (!(cutoff >= 0)) return QT_EINVAL_ERR_NEG;
  if (m < 1 || n < 1 || m > NA_MAX || n > NA_MAX) return QT_ENOTSUP;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return QT_ECUDA;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mutex);
    if (!g_na_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return QT_ECUDA;
      g_na_addr[dev] = p;
    }
    base = g_na_addr[dev];
  }
  // carve the array: X | V | parts | sigma | perm | flags
  double2* X = static_cast<double2*>(base);
  double2* V = X + NA_X;
  double2* parts = V + NA_V;
  double* sig = reinterpret_cast<double*>(parts + NA_PARTS);
  int* perm = reinterpret_cast<int*>(sig + NA_SIG);
  int* flags = perm + NA_MAX;

  qt_handle h;  // a stack handle on the caller's stream: no pool, no allocation
  qt_config_default(&h.cfg);
  h.device = dev;
  h.stream = stream;
  int hflags[QT_FLAG_COUNT] = {0};
  h.d_flags = flags;
  h.h_flags = hflags;

  const bool tr = m < n;
  const int64_t mm = tr ? n : m, nn = tr ? m : n;
  int nb = 0, chunks = 0;
  if ((size_t)qt_jacobi_layout(mm, nn, &nb, &chunks) > NA_PARTS) return QT_ENOTSUP;
  // the matrix is copied into the scratch (the caller's input is not modified)
  if (tr) {
    QT_TRY(qt_adjoint_copy<double2>(&h, static_cast<const double2*>(dM), m, n, m, X, mm));
  } else {
    QT_CHECK_CUDA(&h, cudaMemcpyAsync(X, dM, sizeof(double2) * m * n, cudaMemcpyDeviceToDevice, stream));
  }
  int sweeps = 0;
  const double tol = 16.0 * std::sqrt((double)std::max<int64_t>(mm, 16)) * 1.11e-16;
  QT_TRY(qt_jacobi_svd_ws<double2>(&h, X, mm, nn, mm, V, nn, tol, h.cfg.max_sweeps, &sweeps, parts));
  QT_TRY(qt_sorted_column_norms<double2>(&h, X, mm, nn, mm, sig, perm));
  std::vector<double> s((size_t)nn);
  QT_CHECK_CUDA(&h, cudaMemcpyAsync(s.data(), sig, sizeof(double) * nn, cudaMemcpyDeviceToHost, stream));
  QT_CHECK_CUDA(&h, cudaStreamSynchronize(stream));
  int kc = 1;
  qt_tail_rule_host(s, cutoff, &kc);
  const int k = chi_max > 0 ? std::min(kc, chi_max) : kc;
  // U (m x k) and diag(S) Vh (k x n), then Vh = rows divided by S
  QT_TRY((qt_absorb<double2, double2>(&h, tr ? 1 : 0, X, mm, V, nn, sig, perm, m, n, k, 1.0,
                                       static_cast<double2*>(dU), static_cast<double2*>(dVh))));
  scale_rows_inv_kernel<<<64, 256, 0, stream>>>(static_cast<double2*>(dVh), k, n, sig);
  QT_CHECK_CUDA(&h, cudaGetLastError());
  QT_CHECK_CUDA(&h, cudaMemcpyAsync(dS, sig, sizeof(double) * k, cudaMemcpyDeviceToDevice, stream));
  QT_CHECK_CUDA(&h, cudaStreamSynchronize(stream));
  *k_out = k;
  return QT_OK;
}
