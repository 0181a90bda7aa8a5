// Device-resident tensors and the pairwise steps of ncon on the GPU.
//
// TensorOperations.ncon, which src/contract.jl:257,263 calls, contracts a
// network one pair of tensors at a time: each step permutes its operands to
// [free, contracted] x [contracted, free], multiplies them with a BLAS gemm
// and keeps the result's legs as A's free legs followed by B's.  Here the
// tensors stay in HBM between steps (qt_tensor), and the permutes never
// produce a permuted copy: every operand is read through two offset tables
// -- one over the legs that become matrix rows, one over the legs that
// become columns, in element strides of the source tensor -- so element
// (r, c) of the GEMM operand is src[row[r] + col[c]].  For complex64 the
// tables drive the tensor-core operand gather (split-TF32 planes,
// k_tcgemm.cu); otherwise one tiled gather kernel writes the operand matrix
// for the SIMT GEMM.  A label repeated on one tensor is traced on the
// device; the final leg order is a device permute.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "qt_internal.cuh"

struct qt_tensor {
  int dtype = QT_C128;
  std::vector<int64_t> dims;
  void* data = nullptr;
  int64_t count = 1;
};

namespace {

constexpr int MAX_LEGS = 24;

size_t esize(int dtype) { return dtype == QT_C64 ? sizeof(float2) : sizeof(double2); }

// Column-major element strides of a tensor.
std::vector<int64_t> strides_of(const std::vector<int64_t>& dims) {
  std::vector<int64_t> st(dims.size(), 1);
  for (size_t i = 1; i < dims.size(); i++) st[i] = st[i - 1] * dims[i - 1];
  return st;
}

// Offsets of the multi-index over `legs` (first leg fastest) in a tensor
// with strides `st`: table[i] = sum_j idx_j st[legs[j]].
std::vector<int64_t> offset_table(const std::vector<int64_t>& dims, const std::vector<int64_t>& st,
                                  const std::vector<int>& legs) {
  int64_t n = 1;
  for (int l : legs) n *= dims[l];
  std::vector<int64_t> t((size_t)n, 0);
  int64_t span = 1;
  for (int l : legs) {
    const int64_t d = dims[l];
    for (int64_t i = span; i < span * d; i++) t[(size_t)i] = t[(size_t)(i % span)] + (i / span) * st[l];
    span *= d;
  }
  return t;
}

// dst (R x Cn, column-major) = src[row[r] + col[c]]; a 32 x 32 tile through
// shared memory so that the writes (along r) and the reads (along r when the
// source's unit-stride leg is a row leg, else along c) are both coalesced.
template <typename C>
__global__ void gather_matrix_kernel(const C* __restrict__ src, const int64_t* __restrict__ row,
                                     const int64_t* __restrict__ col, int rows_fast, int64_t R, int64_t Cn,
                                     C* __restrict__ dst) {
  __shared__ C tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.x * 32, c0 = (int64_t)blockIdx.y * 32;
  for (int q = threadIdx.y; q < 32; q += 8) {
    if (rows_fast) {
      const int64_t r = r0 + threadIdx.x, c = c0 + q;
      if (r < R && c < Cn) tile[threadIdx.x][q] = src[row[r] + col[c]];
    } else {
      const int64_t r = r0 + q, c = c0 + threadIdx.x;
      if (r < R && c < Cn) tile[q][threadIdx.x] = src[row[r] + col[c]];
    }
  }
  __syncthreads();
  for (int q = threadIdx.y; q < 32; q += 8) {
    const int64_t r = r0 + threadIdx.x, c = c0 + q;
    if (r < R && c < Cn) dst[r + R * c] = tile[threadIdx.x][q];
  }
}

// out[f] = sum_j src[row[f] + j * dstride], j < n (a partial trace).
template <typename C>
__global__ void trace_kernel(const C* __restrict__ src, const int64_t* __restrict__ row, int64_t F, int64_t dstride,
                             int64_t n, C* __restrict__ out) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < F; f += (int64_t)gridDim.x * blockDim.x) {
    C acc = czero<C>();
    for (int64_t j = 0; j < n; j++) acc = cadd(acc, src[row[f] + j * dstride]);
    out[f] = acc;
  }
}

int check_tensor(qt_handle* h, const qt_tensor* t) {
  if (!t || !t->data) return qt_fail(h, QT_EINVAL, "tensor: null tensor");
  return QT_OK;
}

int new_tensor(qt_handle* h, int dtype, const std::vector<int64_t>& dims, qt_tensor** out) {
  qt_tensor* t = new qt_tensor();
  t->dtype = dtype;
  t->dims = dims;
  t->count = 1;
  for (int64_t d : dims) t->count *= d;
  const int rc = qt_dmalloc(h, &t->data, esize(dtype) * (size_t)std::max<int64_t>(t->count, 1));
  if (rc != QT_OK) {
    delete t;
    return rc;
  }
  *out = t;
  return QT_OK;
}

void drop_tensor(qt_handle* h, qt_tensor** t) {
  if (*t) {
    qt_dfree(h, (*t)->data);
    delete *t;
    *t = nullptr;
  }
}

// Upload an offset table into pool scratch.  A copy from pageable host
// memory has read its source when cudaMemcpyAsync returns, so the vector may
// go out of scope afterwards.
int upload_table(qt_handle* h, qt_scratch& s, const std::vector<int64_t>& t, int64_t** d) {
  QT_TRY(s.get(d, std::max<size_t>(t.size(), 1)));
  if (!t.empty())
    QT_CHECK_CUDA(h, cudaMemcpyAsync(*d, t.data(), sizeof(int64_t) * t.size(), cudaMemcpyHostToDevice, h->stream));
  return QT_OK;
}

// Rows are fast when the source's unit-stride leg (leg 0) is a row leg.
bool leg0_in(const std::vector<int>& legs) { return std::find(legs.begin(), legs.end(), 0) != legs.end(); }

// dst = the operand matrix of tensor t with rows over `rlegs`, columns over
// `clegs`, written into `into` when given, else into pool scratch.
template <typename C>
int gather_matrix(qt_handle* h, qt_scratch& s, const qt_tensor* t, const std::vector<int>& rlegs,
                  const std::vector<int>& clegs, C** dst, C* into = nullptr) {
  const std::vector<int64_t> st = strides_of(t->dims);
  const std::vector<int64_t> trow = offset_table(t->dims, st, rlegs), tcol = offset_table(t->dims, st, clegs);
  const int64_t R = (int64_t)trow.size(), Cn = (int64_t)tcol.size();
  int64_t *drow, *dcol;
  QT_TRY(upload_table(h, s, trow, &drow));
  QT_TRY(upload_table(h, s, tcol, &dcol));
  if (into) *dst = into;
  else QT_TRY(s.get(dst, (size_t)std::max<int64_t>(R * Cn, 1)));
  if (R == 0 || Cn == 0) return QT_OK;
  dim3 grid((unsigned)((R + 31) / 32), (unsigned)((Cn + 31) / 32));
  QT_LAUNCH(h, gather_matrix_kernel<C>, grid, dim3(32, 8), 0, (const C*)t->data, drow, dcol, leg0_in(rlegs) ? 1 : 0,
            R, Cn, *dst);
  return QT_OK;
}

// The pairwise step: result legs = A's free legs (in order) then B's.
int contract_device(qt_handle* h, const qt_tensor* A, const qt_tensor* B, int nc, const int* axA, const int* axB,
                    qt_tensor** out) {
  const int ndA = (int)A->dims.size(), ndB = (int)B->dims.size();
  std::vector<char> ca(ndA, 0), cb(ndB, 0);
  for (int i = 0; i < nc; i++) {
    if (axA[i] < 0 || axA[i] >= ndA || axB[i] < 0 || axB[i] >= ndB || ca[axA[i]] || cb[axB[i]])
      return qt_fail(h, QT_EINVAL, "contract_pair: bad axis");
    if (A->dims[axA[i]] != B->dims[axB[i]])
      return qt_fail(h, QT_EDIM_MISMATCH, "Dimensions of contraction legs do not match");
    ca[axA[i]] = 1;
    cb[axB[i]] = 1;
  }
  std::vector<int> afree, acon(axA, axA + nc), bcon(axB, axB + nc), bfree;
  std::vector<int64_t> odims;
  for (int i = 0; i < ndA; i++)
    if (!ca[i]) { afree.push_back(i); odims.push_back(A->dims[i]); }
  for (int i = 0; i < ndB; i++)
    if (!cb[i]) { bfree.push_back(i); odims.push_back(B->dims[i]); }
  if ((int)odims.size() > MAX_LEGS) return qt_fail(h, QT_ENOTSUP, "contract_pair: too many legs");
  QT_TRY(new_tensor(h, A->dtype, odims, out));
  qt_tensor* Ct = *out;
  int rc = QT_OK;
  {
    qt_scratch s(h);
    const std::vector<int64_t> sa = strides_of(A->dims), sb = strides_of(B->dims);
    const std::vector<int64_t> tab[4] = {offset_table(A->dims, sa, afree), offset_table(A->dims, sa, acon),
                                         offset_table(B->dims, sb, bcon), offset_table(B->dims, sb, bfree)};
    const int64_t M = (int64_t)tab[0].size(), K = (int64_t)tab[1].size(), N = (int64_t)tab[3].size();
    if (A->dtype == QT_C64 && h->cfg.tc_gemm && M >= 64 && N >= 32 && K >= 32) {
      int64_t* d[4];
      for (int i = 0; i < 4 && rc == QT_OK; i++) rc = upload_table(h, s, tab[i], &d[i]);
      if (rc == QT_OK)
        rc = qt_cgemm_tc_mapped(h, M, N, K, (const float2*)A->data, d[0], d[1], leg0_in(afree) ? 1 : 0,
                                (const float2*)B->data, d[2], d[3], leg0_in(bcon) ? 1 : 0, (float2*)Ct->data);
    } else if (A->dtype == QT_C64) {
      float2 *Am = nullptr, *Bm = nullptr;
      rc = gather_matrix<float2>(h, s, A, afree, acon, &Am);
      if (rc == QT_OK) rc = gather_matrix<float2>(h, s, B, bcon, bfree, &Bm);
      if (rc == QT_OK)
        rc = qt_cgemm_c64(h, QT_OP_N, QT_OP_N, M, N, K, make_float2(1, 0), Am, M, Bm, K, make_float2(0, 0),
                          (float2*)Ct->data, M);
    } else {
      double2 *Am = nullptr, *Bm = nullptr;
      rc = gather_matrix<double2>(h, s, A, afree, acon, &Am);
      if (rc == QT_OK) rc = gather_matrix<double2>(h, s, B, bcon, bfree, &Bm);
      if (rc == QT_OK)
        rc = qt_cgemm<double2>(h, QT_OP_N, QT_OP_N, M, N, K, make_double2(1, 0), Am, M, Bm, K, make_double2(0, 0),
                               (double2*)Ct->data, M);
    }
    {
      const int st = qt_check_status(h);  // a timed-out device wait is the cause of what followed
      if (st != QT_OK) rc = st;
    }
    if (rc == QT_OK && cudaStreamSynchronize(h->stream) != cudaSuccess)
      rc = qt_fail(h, QT_ECUDA, "contract_pair: device error");
  }
  if (rc != QT_OK) drop_tensor(h, out);
  return rc;
}

// out = the legs of A in the order perm (out leg i = A leg perm[i]).
int permute_device(qt_handle* h, const qt_tensor* A, const int* perm, qt_tensor** out) {
  const int nd = (int)A->dims.size();
  std::vector<char> seen(nd, 0);
  std::vector<int> legs(perm, perm + nd);
  std::vector<int64_t> odims;
  for (int l : legs) {
    if (l < 0 || l >= nd || seen[l]) return qt_fail(h, QT_EINVAL, "permute: not a permutation");
    seen[l] = 1;
    odims.push_back(A->dims[l]);
  }
  QT_TRY(new_tensor(h, A->dtype, odims, out));
  if (A->count == 0) return QT_OK;
  int rc = QT_OK;
  {
    // a gather with the output's first leg as rows and the others as columns
    qt_scratch s(h);
    std::vector<int> rl, cl;
    if (nd > 0) rl.push_back(legs[0]);
    for (int i = 1; i < nd; i++) cl.push_back(legs[i]);
    if (A->dtype == QT_C64) {
      float2* dst = nullptr;
      rc = gather_matrix<float2>(h, s, A, rl, cl, &dst, (float2*)(*out)->data);
    } else {
      double2* dst = nullptr;
      rc = gather_matrix<double2>(h, s, A, rl, cl, &dst, (double2*)(*out)->data);
    }
    if (rc == QT_OK && cudaStreamSynchronize(h->stream) != cudaSuccess)
      rc = qt_fail(h, QT_ECUDA, "permute: device error");
  }
  if (rc != QT_OK) drop_tensor(h, out);
  return rc;
}

}  // namespace

void* qt_tensor_data(const qt_tensor* t) { return t ? t->data : nullptr; }

extern "C" int qt_tensor_create(qt_handle* h, int dtype, int nd, const int64_t* dims, const void* host,
                                qt_tensor** out) {
  if (!h || !out || nd < 0 || nd > MAX_LEGS || (nd > 0 && !dims)) return qt_fail(h, QT_EINVAL, "tensor: bad argument");
  if (dtype != QT_C64 && dtype != QT_C128) return qt_fail(h, QT_EINVAL, "tensor: bad dtype");
  std::vector<int64_t> d(dims, dims + nd);
  for (int64_t v : d)
    if (v < 0) return qt_fail(h, QT_EINVAL, "tensor: negative dimension");
  cudaSetDevice(h->device);
  QT_TRY(new_tensor(h, dtype, d, out));
  const size_t bytes = esize(dtype) * (size_t)(*out)->count;
  if (bytes) {
    cudaError_t e = host ? cudaMemcpyAsync((*out)->data, host, bytes, cudaMemcpyHostToDevice, h->stream)
                         : cudaMemsetAsync((*out)->data, 0, bytes, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
      drop_tensor(h, out);
      return qt_fail(h, QT_ECUDA, std::string("tensor upload: ") + cudaGetErrorString(e));
    }
  }
  return QT_OK;
}

extern "C" int qt_tensor_free(qt_handle* h, qt_tensor* t) {
  if (!t) return QT_OK;
  if (h) qt_dfree(h, t->data);
  delete t;
  return QT_OK;
}

extern "C" int qt_tensor_ndims(const qt_tensor* t) { return t ? (int)t->dims.size() : -1; }

extern "C" int qt_tensor_dims(const qt_tensor* t, int64_t* dims) {
  if (!t || !dims) return QT_EINVAL;
  std::copy(t->dims.begin(), t->dims.end(), dims);
  return QT_OK;
}

extern "C" int qt_tensor_download(qt_handle* h, const qt_tensor* t, void* host) {
  if (!h || !host) return qt_fail(h, QT_EINVAL, "tensor download: null argument");
  QT_TRY(check_tensor(h, t));
  cudaSetDevice(h->device);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(host, t->data, esize(t->dtype) * (size_t)t->count, cudaMemcpyDeviceToHost,
                                   h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

extern "C" int qt_tensor_contract(qt_handle* h, const qt_tensor* A, const qt_tensor* B, int ncontract,
                                  const int* axesA, const int* axesB, const int* out_perm, qt_tensor** out) {
  if (!h || !out || ncontract < 0 || (ncontract > 0 && (!axesA || !axesB)))
    return qt_fail(h, QT_EINVAL, "contract_pair: bad argument");
  QT_TRY(check_tensor(h, A));
  QT_TRY(check_tensor(h, B));
  if (A->dtype != B->dtype) return qt_fail(h, QT_EINVAL, "contract_pair: operands of different dtype");
  cudaSetDevice(h->device);
  qt_tensor* C = nullptr;
  QT_TRY(contract_device(h, A, B, ncontract, axesA, axesB, &C));
  if (!out_perm) {
    *out = C;
    return QT_OK;
  }
  const int rc = permute_device(h, C, out_perm, out);
  qt_tensor_free(h, C);
  return rc;
}

extern "C" int qt_tensor_permute(qt_handle* h, const qt_tensor* A, const int* perm, qt_tensor** out) {
  if (!h || !out) return qt_fail(h, QT_EINVAL, "permute: bad argument");
  QT_TRY(check_tensor(h, A));
  if (!perm && !A->dims.empty()) return qt_fail(h, QT_EINVAL, "permute: null permutation");
  cudaSetDevice(h->device);
  return permute_device(h, A, perm, out);
}

extern "C" int qt_tensor_trace(qt_handle* h, const qt_tensor* A, int ax1, int ax2, qt_tensor** out) {
  if (!h || !out) return qt_fail(h, QT_EINVAL, "trace: bad argument");
  QT_TRY(check_tensor(h, A));
  const int nd = (int)A->dims.size();
  if (ax1 < 0 || ax2 < 0 || ax1 >= nd || ax2 >= nd || ax1 == ax2) return qt_fail(h, QT_EINVAL, "trace: bad axes");
  if (A->dims[ax1] != A->dims[ax2]) return qt_fail(h, QT_EDIM_MISMATCH, "Dimensions of contraction legs do not match");
  cudaSetDevice(h->device);
  std::vector<int> free;
  std::vector<int64_t> odims;
  for (int i = 0; i < nd; i++)
    if (i != ax1 && i != ax2) { free.push_back(i); odims.push_back(A->dims[i]); }
  QT_TRY(new_tensor(h, A->dtype, odims, out));
  int rc = QT_OK;
  {
    qt_scratch s(h);
    const std::vector<int64_t> st = strides_of(A->dims);
    const std::vector<int64_t> row = offset_table(A->dims, st, free);
    int64_t* drow = nullptr;
    rc = upload_table(h, s, row, &drow);
    const int64_t F = (int64_t)row.size();
    if (rc == QT_OK && F > 0) {
      const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((F + 255) / 256, 4096));
      if (A->dtype == QT_C64) {
        QT_LAUNCH(h, trace_kernel<float2>, grid, 256, 0, (const float2*)A->data, drow, F, st[ax1] + st[ax2],
                  A->dims[ax1], (float2*)(*out)->data);
      } else {
        QT_LAUNCH(h, trace_kernel<double2>, grid, 256, 0, (const double2*)A->data, drow, F, st[ax1] + st[ax2],
                  A->dims[ax1], (double2*)(*out)->data);
      }
    }
    if (rc == QT_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = qt_fail(h, QT_ECUDA, "trace: device error");
  }
  if (rc != QT_OK) drop_tensor(h, out);
  return rc;
}

// The host-buffer pairwise contraction: upload, the device step, download.
extern "C" int qt_contract_pair(qt_handle* h, int dtype, int ndA, const int64_t* dimsA, const void* A, int ndB,
                                const int64_t* dimsB, const void* B, int ncontract, const int* axesA,
                                const int* axesB, void* C) {
  if (!h || !A || !B || !C || (ndA > 0 && !dimsA) || (ndB > 0 && !dimsB))
    return qt_fail(h, QT_EINVAL, "contract_pair: null argument");
  if (dtype != QT_C64 && dtype != QT_C128) return qt_fail(h, QT_EINVAL, "contract_pair: bad dtype");
  qt_tensor *ta = nullptr, *tb = nullptr, *tc = nullptr;
  int rc = qt_tensor_create(h, dtype, ndA, dimsA, A, &ta);
  if (rc == QT_OK) rc = qt_tensor_create(h, dtype, ndB, dimsB, B, &tb);
  if (rc == QT_OK) rc = qt_tensor_contract(h, ta, tb, ncontract, axesA, axesB, nullptr, &tc);
  if (rc == QT_OK) rc = qt_tensor_download(h, tc, C);
  qt_tensor_free(h, ta);
  qt_tensor_free(h, tb);
  qt_tensor_free(h, tc);
  return rc;
}
