// C ABI of the engine: handle, device-resident MPS, the two-qubit gate +
// truncated-SVD update in its three modes, and the dense primitives that sit
// behind contract / contract_svd / svd of the reference.
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>

#include "qt_internal.cuh"
#include "qt_rank_model.h"

// ---------------------------------------------------------------------------
// basics
// ---------------------------------------------------------------------------

int qt_fail(qt_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int qt_check_status(qt_handle* h) {
  if (!h->d_status) return QT_OK;
  int hs = 0;
  QT_CHECK_CUDA(h, cudaMemcpyAsync(&hs, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  if (!hs) return QT_OK;
  QT_CHECK_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
  return qt_fail(h, QT_ETIMEOUT, hs == 2 ? "orthonormalize: a grid barrier wait timed out"
                                          : "tc gemm: a pipeline wait timed out");
}

int qt_dmalloc(qt_handle* h, void** p, size_t bytes) {
  cudaError_t e = cudaMallocFromPoolAsync(p, bytes ? bytes : 16, h->pool, h->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return qt_fail(h, QT_ENOMEM, std::string("device allocation of ") + std::to_string(bytes) +
                                     " bytes failed: " + cudaGetErrorString(e));
  }
  return QT_OK;
}

void qt_dfree(qt_handle* h, void* p) {
  if (p) cudaFreeAsync(p, h->stream);
}

static size_t elem_size(int dtype) { return dtype == QT_C64 ? sizeof(float2) : sizeof(double2); }

extern "C" int qt_abi_version(void) { return QT_ABI_VERSION; }

extern "C" int qt_cert_counters(const qt_handle* h, int64_t* out) {
  if (!h || !out) return QT_EINVAL;
  for (int i = 0; i < QT_CERT_SLOTS; i++) out[i] = h->cert_count[i];
  return QT_OK;
}

extern "C" int qt_work_counters(const qt_handle* h, double* out) {
  if (!h || !out) return QT_EINVAL;
  out[0] = h->work_jacobi_bytes;
  out[1] = h->work_jacobi_rounds;
  out[2] = h->work_tc_flops;
  out[3] = h->work_tc_launches;
  out[4] = h->work_jacobi_pairs;
  out[5] = h->work_jacobi_inner;
  out[6] = h->work_jacobi_gram_bytes;
  out[7] = h->work_jacobi_rot_bytes;
  return QT_OK;
}

extern "C" int qt_config_default(qt_config* cfg) {
  if (!cfg) return QT_EINVAL;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->device = 0;
  cfg->mode = QT_MODE_PLAIN;
  cfg->cutoff = 0.0;
  cfg->chi_max = 0;
  cfg->oversample = 16;
  cfg->power_iters = 1;
  cfg->renormalize = 0;
  cfg->use_rank_model = 1;
  cfg->max_sweeps = 80;
  cfg->jacobi_tol = 0.0;     // 0: sqrt(rows) * unit roundoff of the storage type
  cfg->noise_floor = 0.0;    // 0: 4 * 2^-23 (FP32-level products)
  cfg->seed = 0x5eed5eedull;
  cfg->tc_gemm = 0;
  cfg->jacobi_kernel = 0;
  cfg->cap_sketch = 0.0;     // 0: 1.125 chi_max
  return QT_OK;
}

extern "C" int qt_create(qt_handle** out, const qt_config* cfg) {
  if (!out) return QT_EINVAL;
  *out = nullptr;
  qt_handle* h = new qt_handle();
  if (cfg) h->cfg = *cfg; else qt_config_default(&h->cfg);
  h->device = h->cfg.device;
  int rc = QT_OK;
  do {
    if (cudaSetDevice(h->device) != cudaSuccess) { rc = QT_ECUDA; break; }
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) { rc = QT_ECUDA; break; }
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = h->device;
    if (cudaMemPoolCreate(&h->pool, &props) != cudaSuccess) { rc = QT_ECUDA; break; }
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(h->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    if (cudaMalloc(&h->d_flags, sizeof(int) * QT_FLAG_COUNT) != cudaSuccess) { rc = QT_ENOMEM; break; }
    if (cudaMallocHost(&h->h_flags, sizeof(int) * QT_FLAG_COUNT) != cudaSuccess) { rc = QT_ENOMEM; break; }
    cudaMemset(h->d_flags, 0, sizeof(int) * QT_FLAG_COUNT);
    if (cudaMalloc(&h->d_status, sizeof(int)) != cudaSuccess) { rc = QT_ENOMEM; break; }
    cudaMemset(h->d_status, 0, sizeof(int));
    h->rank_model = qt_rank_model_create();
  } while (0);
  if (rc != QT_OK) {
    cudaGetLastError();
    qt_destroy(h);
    return rc;
  }
  *out = h;
  return QT_OK;
}

extern "C" int qt_destroy(qt_handle* h) {
  if (!h) return QT_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  qt_rank_model_destroy(h->rank_model);
  for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : h->timers)
    if (e) cudaEventDestroy(e);
  if (h->d_flags) cudaFree(h->d_flags);
  if (h->d_status) cudaFree(h->d_status);
  if (h->h_flags) cudaFreeHost(h->h_flags);
  if (h->pool) cudaMemPoolDestroy(h->pool);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return QT_OK;
}

extern "C" const char* qt_last_error(const qt_handle* h) { return h ? h->err.c_str() : "null handle"; }

// ---------------------------------------------------------------------------
// timing and profiling
// ---------------------------------------------------------------------------

static cudaEvent_t pool_event(qt_handle* h) {
  if (h->event_next == h->event_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    h->event_pool.push_back(e);
  }
  return h->event_pool[h->event_next++];
}

void qt_prof_before(qt_handle* h, const char* name) {
  qt_profile_rec r;
  r.name = name;
  r.start = pool_event(h);
  r.stop = pool_event(h);
  cudaEventRecord(r.start, h->stream);
  h->prof_recs.push_back(r);
}

void qt_prof_after(qt_handle* h) { cudaEventRecord(h->prof_recs.back().stop, h->stream); }

struct prof_agg {
  std::string name;
  int64_t launches = 0;
  double ms = 0;
};
static std::vector<prof_agg> g_prof_view;  // last qt_profile_collect result

extern "C" int qt_profile_enable(qt_handle* h, int on) {
  if (!h) return QT_EINVAL;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  h->prof = on != 0;
  h->prof_recs.clear();
  h->event_next = 0;
  return QT_OK;
}

// Aggregate the recorded launches by kernel name; returns the number of kernels.
extern "C" int qt_profile_collect(qt_handle* h) {
  if (!h) return QT_EINVAL;
  cudaSetDevice(h->device);
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  g_prof_view.clear();
  for (const auto& r : h->prof_recs) {
    float ms = 0;
    cudaEventElapsedTime(&ms, r.start, r.stop);
    auto it = std::find_if(g_prof_view.begin(), g_prof_view.end(), [&](const prof_agg& a) { return a.name == r.name; });
    if (it == g_prof_view.end()) {
      g_prof_view.push_back(prof_agg());
      it = g_prof_view.end() - 1;
      it->name = r.name;
    }
    it->launches++;
    it->ms += ms;
  }
  return (int)g_prof_view.size();
}

extern "C" int qt_profile_get(int idx, char* name, int namelen, int64_t* launches, double* total_ms) {
  if (idx < 0 || idx >= (int)g_prof_view.size() || !name || namelen < 1) return QT_EINVAL;
  std::strncpy(name, g_prof_view[idx].name.c_str(), (size_t)namelen - 1);
  name[namelen - 1] = 0;
  if (launches) *launches = g_prof_view[idx].launches;
  if (total_ms) *total_ms = g_prof_view[idx].ms;
  return QT_OK;
}

extern "C" int qt_timer_record(qt_handle* h, int slot) {
  if (!h || slot < 0 || slot >= 8) return QT_EINVAL;
  cudaSetDevice(h->device);
  if (!h->timers[slot]) QT_CHECK_CUDA(h, cudaEventCreate(&h->timers[slot]));
  QT_CHECK_CUDA(h, cudaEventRecord(h->timers[slot], h->stream));
  return QT_OK;
}

extern "C" int qt_timer_elapsed(qt_handle* h, int a, int b, double* ms) {
  if (!h || !ms || a < 0 || b < 0 || a >= 8 || b >= 8 || !h->timers[a] || !h->timers[b]) return QT_EINVAL;
  QT_CHECK_CUDA(h, cudaEventSynchronize(h->timers[b]));
  float f = 0;
  QT_CHECK_CUDA(h, cudaEventElapsedTime(&f, h->timers[a], h->timers[b]));
  *ms = f;
  return QT_OK;
}

extern "C" int qt_sync(qt_handle* h) {
  if (!h) return QT_EINVAL;
  cudaSetDevice(h->device);
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

// Write a 256 MiB device buffer (larger than the 129 MB L2) on the handle's
// stream so the next step starts from a cold L2.
extern "C" int qt_l2_flush(qt_handle* h) {
  if (!h) return QT_EINVAL;
  cudaSetDevice(h->device);
  const size_t bytes = (size_t)256 << 20;
  void* p = nullptr;
  QT_TRY(qt_dmalloc(h, &p, bytes));
  QT_CHECK_CUDA(h, cudaMemsetAsync(p, (int)(h->launches & 0xff), bytes, h->stream));
  qt_dfree(h, p);
  return QT_OK;
}

extern "C" void* qt_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
  return p;
}

extern "C" int qt_host_free(void* p) {
  if (p) cudaFreeHost(p);
  return QT_OK;
}
extern "C" int64_t qt_launch_count(const qt_handle* h) { return h ? h->launches : 0; }

// ---------------------------------------------------------------------------
// MPS objects
// ---------------------------------------------------------------------------

extern "C" int qt_mps_create(qt_handle* h, int nsites, const int64_t* dims, const void* const* host_sites, int dtype,
                             qt_mps** out) {
  if (!h || !out || !dims) return qt_fail(h, QT_EINVAL, "mps_create: null argument");
  *out = nullptr;
  if (nsites < 1) return qt_fail(h, QT_EINVAL, "mps_create: need at least one site");
  if (dtype != QT_C64 && dtype != QT_C128) return qt_fail(h, QT_EINVAL, "mps_create: dtype must be QT_C64 or QT_C128");
  for (int i = 0; i < nsites; i++) {
    if (dims[3 * i] < 1 || dims[3 * i + 1] != 2 || dims[3 * i + 2] < 1)
      return qt_fail(h, QT_EINVAL, "Each site must have dims (chiL, 2, chiR)");
    if (i > 0 && dims[3 * i] != dims[3 * i - 1])
      return qt_fail(h, QT_EDIM_MISMATCH, "Dimensions of contraction legs do not match");
    if (!host_sites && (dims[3 * i] != 1 || dims[3 * i + 2] != 1))
      return qt_fail(h, QT_EINVAL, "mps_create: the product state needs bond dimension 1");
  }
  cudaSetDevice(h->device);
  qt_mps* m = new qt_mps();
  m->nsites = nsites;
  m->dtype = dtype;
  m->spectrum.resize(nsites > 1 ? nsites - 1 : 0);
  m->bond_updates.assign(nsites > 1 ? nsites - 1 : 0, 0);
  const size_t es = elem_size(dtype);
  for (int i = 0; i < nsites; i++) {
    m->chil.push_back(dims[3 * i]);
    m->chir.push_back(dims[3 * i + 2]);
    const size_t bytes = (size_t)dims[3 * i] * 2 * dims[3 * i + 2] * es;
    void* p = nullptr;
    int rc = qt_dmalloc(h, &p, bytes);
    if (rc != QT_OK) { qt_mps_free(h, m); return rc; }
    m->site.push_back(p);
    m->cap.push_back(bytes);
    if (host_sites) {
      if (!host_sites[i]) { qt_mps_free(h, m); return qt_fail(h, QT_EINVAL, "mps_create: null site pointer"); }
      cudaMemcpyAsync(p, host_sites[i], bytes, cudaMemcpyHostToDevice, h->stream);
    } else {
      double2 z[2] = {make_double2(1, 0), make_double2(0, 0)};
      float2 zf[2] = {make_float2(1, 0), make_float2(0, 0)};
      cudaMemcpyAsync(p, dtype == QT_C128 ? (const void*)z : (const void*)zf, bytes, cudaMemcpyHostToDevice,
                      h->stream);
    }
  }
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  *out = m;
  return QT_OK;
}

extern "C" int qt_mps_free(qt_handle* h, qt_mps* m) {
  if (!m) return QT_OK;
  if (h) {
    cudaSetDevice(h->device);
    for (void* p : m->site) qt_dfree(h, p);
    cudaStreamSynchronize(h->stream);
  }
  delete m;
  return QT_OK;
}

extern "C" int qt_mps_clone(qt_handle* h, const qt_mps* src, qt_mps** out) {
  if (!h || !src || !out) return qt_fail(h, QT_EINVAL, "mps_clone: null argument");
  *out = nullptr;
  cudaSetDevice(h->device);
  qt_mps* m = new qt_mps(*src);
  for (int i = 0; i < src->nsites; i++) {
    const size_t bytes = (size_t)src->chil[i] * 2 * src->chir[i] * elem_size(src->dtype);
    void* p = nullptr;
    int rc = qt_dmalloc(h, &p, bytes);
    if (rc != QT_OK) {
      for (int j = 0; j < i; j++) qt_dfree(h, m->site[j]);
      delete m;
      return rc;
    }
    m->site[i] = p;
    m->cap[i] = bytes;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(p, src->site[i], bytes, cudaMemcpyDeviceToDevice, h->stream));
  }
  *out = m;
  return QT_OK;
}

extern "C" int qt_mps_nsites(const qt_mps* m) { return m ? m->nsites : 0; }

extern "C" int qt_mps_site_dims(const qt_mps* m, int site, int64_t* d) {
  if (!m || !d) return QT_EINVAL;
  if (site < 0 || site >= m->nsites) return QT_EBOUNDS;
  d[0] = m->chil[site];
  d[1] = 2;
  d[2] = m->chir[site];
  return QT_OK;
}

extern "C" int qt_mps_download(qt_handle* h, const qt_mps* m, int site, void* host) {
  if (!h || !m || !host) return qt_fail(h, QT_EINVAL, "mps_download: null argument");
  if (site < 0 || site >= m->nsites) return qt_fail(h, QT_EBOUNDS, "mps_download: site out of range");
  cudaSetDevice(h->device);
  const size_t bytes = (size_t)m->chil[site] * 2 * m->chir[site] * elem_size(m->dtype);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(host, m->site[site], bytes, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

static int replace_site(qt_handle* h, qt_mps* m, int site, int64_t cl, int64_t cr, void* buf, size_t bytes) {
  qt_dfree(h, m->site[site]);
  m->site[site] = buf;
  m->cap[site] = bytes;
  m->chil[site] = cl;
  m->chir[site] = cr;
  return QT_OK;
}

extern "C" int qt_mps_upload_site(qt_handle* h, qt_mps* m, int site, const int64_t* d, const void* host) {
  if (!h || !m || !d || !host) return qt_fail(h, QT_EINVAL, "mps_upload_site: null argument");
  if (site < 0 || site >= m->nsites) return qt_fail(h, QT_EBOUNDS, "mps_upload_site: site out of range");
  if (d[1] != 2 || d[0] < 1 || d[2] < 1) return qt_fail(h, QT_EINVAL, "Each site must have dims (chiL, 2, chiR)");
  if ((site > 0 && d[0] != m->chir[site - 1]) || (site + 1 < m->nsites && d[2] != m->chil[site + 1]))
    return qt_fail(h, QT_EDIM_MISMATCH, "Dimensions of contraction legs do not match");
  cudaSetDevice(h->device);
  const size_t bytes = (size_t)d[0] * 2 * d[2] * elem_size(m->dtype);
  void* p = nullptr;
  QT_TRY(qt_dmalloc(h, &p, bytes));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, h->stream));
  replace_site(h, m, site, d[0], d[2], p, bytes);
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

// ---------------------------------------------------------------------------
// truncated SVD of a device matrix (shared by every mode)
// ---------------------------------------------------------------------------

namespace {

struct SvdOut {
  int k = 0, k_cut = 0, sweeps = 0;
  double norm2 = 0, discarded = 0;
  std::vector<double> s;  // full computed spectrum, descending
};

// Relative orthogonality threshold of the one-sided Jacobi.  The Gram entries
// of a freshly rotated pair carry rounding noise of about sqrt(rows) u, so
// the threshold sits a factor 16 above it; the singular values depend on the
// remaining non-orthogonality only to second order.
double auto_tol(const qt_handle* h, int64_t rows, bool fp32) {
  if (h->cfg.jacobi_tol > 0) return h->cfg.jacobi_tol;
  const double u = fp32 ? 5.96e-8 : 1.11e-16;
  return 16.0 * std::sqrt((double)std::max<int64_t>(rows, 16)) * u;
}

int choose_rank(const qt_handle* h, const std::vector<double>& s, double cutoff, int chi_max, SvdOut* o) {
  int kc = 1;
  if (cutoff < 0) kc = (int)s.size();  // no truncation (switch!)
  else qt_tail_rule_host(s, cutoff, &kc);
  int k = kc;
  if (chi_max > 0) k = std::min(k, chi_max);
  o->k = k;
  o->k_cut = kc;
  o->norm2 = 0;
  o->discarded = 0;
  for (size_t i = 0; i < s.size(); i++) {
    o->norm2 += s[i] * s[i];
    if ((int)i >= k) o->discarded += s[i] * s[i];
  }
  (void)h;
  return QT_OK;
}

// Chosen-mode rank certification.  The FP32-level split resolves singular
// values and tail norms only down to eta (a few units of FP32 rounding of
// ||theta'||_F).  The tail rule of src/svd.jl:29-33 at a cutoff below eta is
// still decided exactly when
//   - the cutoff is at or above eta (resolved), or
//   - the chi_max cap binds with margin: the computed tail beyond chi_max
//     exceeds cutoff + eta, so the exact tail does too and k = chi_max, or
//   - exactly struct_rank values lie above eta, where struct_rank bounds the
//     rank in exact arithmetic (the gate's operator-Schmidt rank times the
//     inner bond, the Hilbert-space dimensions of the two sides): the values
//     below eta are then exact zeros, which the rule drops at any cutoff,
//     while every value above eta exceeds the cutoff.
// Any other decision is left to the exact FP64 split (fallback 4).
struct RankCert {
  double eta = -1.0;        // absolute resolution of the computed spectrum
  int64_t struct_rank = 0;  // exact-arithmetic rank bound (0: unknown)
  int how = 0;              // out: QT_CERT_*
};

bool certify_rank(const std::vector<double>& s, double extra_tail, double cutoff, int chi_max, RankCert* c,
                  SvdOut* o) {
  if (cutoff >= c->eta) {
    c->how = QT_CERT_RESOLVED;
    return true;
  }
  if (chi_max > 0 && o->k_cut > chi_max && (int64_t)s.size() >= chi_max) {
    double t2 = extra_tail > 0 ? extra_tail * extra_tail : 0.0;
    for (size_t i = s.size(); i-- > (size_t)chi_max;) t2 += s[i] * s[i];
    if (std::sqrt(t2) > cutoff + c->eta) {
      c->how = QT_CERT_CAP;
      return true;
    }
  }
  if (c->struct_rank > 0 && c->struct_rank <= (int64_t)s.size() && !(extra_tail > c->eta)) {
    int64_t kr = 0;
    while (kr < (int64_t)s.size() && s[kr] > c->eta) kr++;
    if (kr == c->struct_rank) {
      const int kc = (int)kr;
      o->k_cut = kc;
      o->k = chi_max > 0 ? std::min(kc, chi_max) : kc;
      o->discarded = extra_tail > 0 ? extra_tail * extra_tail : 0.0;
      for (size_t i = (size_t)o->k; i < s.size(); i++) o->discarded += s[i] * s[i];
      c->how = QT_CERT_STRUCT;
      return true;
    }
  }
  c->how = QT_CERT_NONE;
  return false;
}

double renorm_scale(const qt_handle* h, const SvdOut& o) {
  if (!h->cfg.renormalize) return 1.0;
  const double kept = o.norm2 - o.discarded;
  return kept > 0 ? std::sqrt(o.norm2 / kept) : 1.0;
}

template <typename C>
__global__ void gather_cols_kernel(const C* __restrict__ V, int64_t rows, int64_t ldv, const int* __restrict__ perm,
                                   int k, C* __restrict__ out) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < rows * k;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    out[i + rows * j] = V[i + ldv * perm[j]];
  }
}

template <typename S, typename D>
__global__ void convert_scale_kernel(const S* __restrict__ src, D* __restrict__ dst, int64_t n, double scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    D v;
    v.x = src[i].x * scale;
    v.y = src[i].y * scale;
    dst[i] = v;
  }
}

template <typename C>
C cone() { C c; c.x = 1; c.y = 0; return c; }
template <typename C>
C czr() { C c; c.x = 0; c.y = 0; return c; }

// Truncated SVD split of M (m x n, ld m, element TS): M ~ A' B' with A' (m x k)
// orthonormal and B' = diag(S_k) V'[:k, :] (k x n).  QR-preconditioned
// one-sided Jacobi (Drmac and Veselic): a wide M is first reduced by a QR of
// M^H (M = M1 Q1^H, M1 = M Q1 square), then M1 = Q2 R2 and the block Jacobi
// runs on Y = R2^H, whose rows are graded, with the rotations V accumulated:
// M1 = Q2 V Y_f^H.  So A' = Q2 V[:, perm] and B' = (Q1 Y_f[:, perm])^H --
// neither needs a division by a singular value.  The QRs are the BCGS2 +
// shifted CholeskyQR2 of qt_orthonormalize with R = Q^H M by GEMM.  M is not
// modified.  Outputs are allocated in element TO.
template <typename TS, typename TO>
int svd_split_jacobi(qt_handle* h, TS* M, int64_t m, int64_t n, double cutoff, int chi_max, bool fp32_storage,
                     TO** Aout, TO** Bout, SvdOut* o, double extra_tail = -1.0) {
  qt_scratch s(h);
  const TS one = cone<TS>(), zero = czr<TS>();
  const bool wide = m < n;
  const int64_t r = std::min(m, n);
  TS *Q1 = nullptr, *M1 = M;
  if (wide) {
    QT_TRY(s.get(&Q1, (size_t)n * m));
    QT_TRY(qt_adjoint_copy<TS>(h, M, m, n, m, Q1, n));
    QT_TRY(qt_orthonormalize<TS>(h, Q1, n, m));
    QT_TRY(s.get(&M1, (size_t)m * m));
    QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, m, m, n, one, M, m, Q1, n, zero, M1, m));  // R1^H = M Q1
  }
  TS *Q2, *Y, *V;
  QT_TRY(s.get(&Q2, (size_t)m * r));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(Q2, M1, sizeof(TS) * m * r, cudaMemcpyDeviceToDevice, h->stream));
  QT_TRY(qt_orthonormalize<TS>(h, Q2, m, r));
  QT_TRY(s.get(&Y, (size_t)r * r));
  QT_TRY(qt_gemm_any(h, QT_OP_C, QT_OP_N, r, r, m, one, M1, m, Q2, m, zero, Y, r));  // R2^H = M1^H Q2
  QT_TRY(s.get(&V, (size_t)r * r));
  double* sig;
  int* perm;
  QT_TRY(s.get(&sig, (size_t)r));
  QT_TRY(s.get(&perm, (size_t)r));
  QT_TRY(qt_jacobi_svd<TS>(h, Y, r, r, r, V, r, auto_tol(h, r, fp32_storage), h->cfg.max_sweeps, &o->sweeps));
  QT_TRY(qt_sorted_column_norms<TS>(h, Y, r, r, r, sig, perm));
  o->s.resize(r);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(o->s.data(), sig, sizeof(double) * r, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  if (extra_tail >= 0) {
    // a weight outside this factorisation (a sketch's residual) counts as
    // the smallest tail value
    std::vector<double> sx = o->s;
    sx.push_back(extra_tail);
    QT_TRY(choose_rank(h, sx, cutoff, chi_max, o));
    if (o->k > (int)r) o->k = (int)r;
  } else {
    QT_TRY(choose_rank(h, o->s, cutoff, chi_max, o));
  }
  const int k = o->k;
  const double sc = renorm_scale(h, *o);
  // A' = Q2 V[:, perm[:k]]
  TS *Vk, *At, *Bt;
  QT_TRY(s.get(&Vk, (size_t)r * k));
  QT_LAUNCH(h, gather_cols_kernel<TS>, 256, 256, 0, V, r, r, perm, k, Vk);
  QT_TRY(s.get(&At, (size_t)m * k));
  QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, m, k, r, one, Q2, m, Vk, r, zero, At, m));
  // B' = Y_f[:, perm]^H (tall) or (Q1 Y_f[:, perm])^H (wide)
  TS* Yk;
  QT_TRY(s.get(&Yk, (size_t)r * k));
  QT_LAUNCH(h, gather_cols_kernel<TS>, 256, 256, 0, Y, r, r, perm, k, Yk);
  QT_TRY(s.get(&Bt, (size_t)k * n));
  if (wide) {
    TS* Z;
    QT_TRY(s.get(&Z, (size_t)n * k));
    QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, n, k, m, one, Q1, n, Yk, m, zero, Z, n));
    QT_TRY(qt_adjoint_copy<TS>(h, Z, n, k, n, Bt, k));
  } else {
    QT_TRY(qt_adjoint_copy<TS>(h, Yk, r, k, r, Bt, k));
  }
  QT_TRY(qt_dmalloc(h, (void**)Aout, sizeof(TO) * m * k));
  QT_TRY(qt_dmalloc(h, (void**)Bout, sizeof(TO) * k * n));
  QT_LAUNCH(h, (convert_scale_kernel<TS, TO>), 256, 256, 0, At, *Aout, (int64_t)m * k, 1.0);
  QT_LAUNCH(h, (convert_scale_kernel<TS, TO>), 256, 256, 0, Bt, *Bout, (int64_t)k * n, sc);
  return QT_OK;
}

// out[:, j] = X[:, perm[j]] / sigma_j (zero columns stay zero).
template <typename C>
__global__ void gather_unit_cols_kernel(const C* __restrict__ X, int64_t rows, int64_t ldx, const int* __restrict__ perm,
                                        const double* __restrict__ sig, int k, C* __restrict__ out) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < rows * k;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    const double s = sig[j];
    const typename real_of<C>::type inv = (typename real_of<C>::type)(s > 0 ? 1.0 / s : 0.0);
    out[i + rows * j] = cscale(X[i + ldx * perm[j]], inv);
  }
}

// out[j] = ||row j of B|| (B: k x n, ld k) in FP64, one CTA per row.
__global__ void row_norms_kernel(const float2* __restrict__ B, int k, int64_t n, double* __restrict__ out) {
  const int j = blockIdx.x;
  double s = 0;
  for (int64_t c = threadIdx.x; c < n; c += blockDim.x) {
    const float2 v = B[j + (int64_t)k * c];
    s = fma((double)v.x, (double)v.x, s);
    s = fma((double)v.y, (double)v.y, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
    out[j] = sqrt(tot);
  }
}

// W = 1.5 I - 0.5 G (k x k): one Newton-Schulz step towards G^{-1/2}.
__global__ void newton_schulz_kernel(const float2* __restrict__ G, int k, float2* __restrict__ W) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)k * k;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % k, j = idx / k;
    const float2 g = G[idx];
    W[idx] = make_float2((i == j ? 1.5f : 0.f) - 0.5f * g.x, -0.5f * g.y);
  }
}

// Chosen-mode noise floor: singular values whose tail lies below
// floor_rel ||theta'||_F are rounding noise of complex64 storage and of the
// FP32-level (split-TF32x3) products: 4 sqrt(max(m, n)) u_fp32.
double fp32_floor_rel(const qt_handle* h, int64_t m, int64_t n) {
  return h->cfg.noise_floor > 0 ? h->cfg.noise_floor : 4.0 * std::sqrt((double)std::max(m, n)) * 5.96e-8;
}

// Columns frozen at sqrt(rows) u ||theta|| hold up to ~0.35 min(m,n) u
// ||theta|| of weight in total; a cutoff above 1.2 min(m,n) u ||theta||
// leaves them inside the tail with room to spare.
bool fast_freeze_ok(int64_t m, int64_t n, double eff_cut, double theta_norm) {
  return eff_cut >= 1.2 * (double)std::min(m, n) * 5.96e-8 * theta_norm;
}

// In-place scaling of n complex values by a power of two (exact).
template <typename C>
__global__ void scale_pow2_kernel(C* x, int64_t n, double scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    C v = x[i];
    v.x *= scale;
    v.y *= scale;
    x[i] = v;
  }
}

// FP32 storage keeps squared column norms and Gram entries in FP32: a matrix
// far from unit norm (an unnormalised state after repeated operator
// applications reaches |psi|^2 ~ 1e38, the FP32 limit) is scaled by 2^-e
// first -- exact -- and the results scaled back.  Returns e (0 when
// ||M||_F^2 lies within 2^+-64).
int fp32_scale_exponent(double norm2) {
  if (!(norm2 > 0) || !std::isfinite(norm2)) return 0;
  const int e2 = std::ilogb(norm2);
  return (e2 > 64 || e2 < -64) ? e2 / 2 : 0;
}

// FP32-storage truncated split of theta (m x n, ld m, not modified): the
// one-sided block Jacobi runs on theta itself (tall or square) or on
// theta^H (wide), with no QR preconditioning -- theta' may be numerically
// rank-deficient at FP32 resolution, where a Cholesky-based QR breaks down
// while Jacobi only stops rotating the noise-level columns.
//   tall/square: X = theta V (V not accumulated); A' = unit columns of X for
//     the k largest norms;
//   wide: X = theta^H V, V (m x m) accumulated; A' = V[:, perm].
// Either A' is orthonormal only to the Jacobi tolerance (FP32: ~1e-5); one
// Newton-Schulz step A' <- A' (1.5 I - 0.5 A'^H A') makes it orthonormal to
// FP32 rounding, and B' = A'^H theta is the exact projection onto it (both
// tensor-core GEMMs), so A' B' carries no error beyond the truncation.
// `extra_tail` (>= 0) is a weight outside this factorisation (a sketch's
// residual), counted as the smallest tail value of the rank rule.
// `fast_freeze`: the rank is decided far above the FP32 rounding level (a
// chi_max cap, or a cutoff well above the noise floor), so the Jacobi may
// freeze columns below sqrt(rows) u ||theta||_F and skip the sweeps that only
// rotate rounding noise.
// `keep_hint` > 0: the rank is pinned at that cap, so the Jacobi may stop once
// the columns at and above the cut have converged.
// `proj` (m x proj_n, ld m), when given: B' is the projection A'^H proj of
// that matrix instead of A'^H theta (a sketch theta = proj Y with orthonormal
// Y: the exact projection of the full matrix), scaled by `out_scale`.
template <typename TO>
int svd_split_direct32(qt_handle* h, const float2* theta, int64_t m, int64_t n, double cutoff, int chi_max,
                       TO** Aout, TO** Bout, SvdOut* o, double extra_tail = -1.0, bool fast_freeze = false,
                       int keep_hint = 0, const float2* proj = nullptr, int64_t proj_n = 0, double out_scale = 1.0,
                       RankCert* cert = nullptr) {
  qt_scratch s(h);
  const bool wide = m < n;
  const int64_t rows = wide ? n : m, cols = wide ? m : n;
  float2 *X, *V = nullptr;
  double* dn;
  QT_TRY(s.get(&X, (size_t)rows * cols));
  QT_TRY(s.get(&dn, 1));
  QT_TRY(qt_norm2<float2>(h, theta, m * n, dn));
  if (wide) {
    QT_TRY(qt_adjoint_copy<float2>(h, theta, m, n, m, X, n));
    QT_TRY(s.get(&V, (size_t)cols * cols));
  } else {
    QT_CHECK_CUDA(h, cudaMemcpyAsync(X, theta, sizeof(float2) * m * n, cudaMemcpyDeviceToDevice, h->stream));
  }
  double tn2 = 0;
  QT_CHECK_CUDA(h, cudaMemcpyAsync(&tn2, dn, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  // the Jacobi works on X = theta 2^-e; the unit left factor and the
  // projection B' = A'^H theta (from theta itself) need no correction
  const int e = fp32_scale_exponent(tn2);
  if (e) QT_LAUNCH(h, scale_pow2_kernel<float2>, 256, 256, 0, X, rows * cols, std::ldexp(1.0, -e));
  // QT_JACOBI_FREEZE scales the fast freeze threshold (tuning)
  static const double freeze_scale =
      std::getenv("QT_JACOBI_FREEZE") ? std::atof(std::getenv("QT_JACOBI_FREEZE")) : 1.0;
  QT_TRY(qt_jacobi_svd<float2>(h, X, rows, cols, rows, V, cols, auto_tol(h, rows, true), h->cfg.max_sweeps,
                               &o->sweeps, fast_freeze ? freeze_scale * std::sqrt((double)rows) * 5.96e-8 : -1.0,
                               keep_hint));
  double* sig;
  int* perm;
  QT_TRY(s.get(&sig, (size_t)cols));
  QT_TRY(s.get(&perm, (size_t)cols));
  QT_TRY(qt_sorted_column_norms<float2>(h, X, rows, cols, rows, sig, perm));
  o->s.resize(cols);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(o->s.data(), sig, sizeof(double) * cols, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  if (e)
    for (double& v : o->s) v = std::ldexp(v, e);
  if (extra_tail >= 0) {
    std::vector<double> sx = o->s;
    sx.push_back(extra_tail);
    QT_TRY(choose_rank(h, sx, cutoff, chi_max, o));
    if (o->k > (int)cols) o->k = (int)cols;
  } else {
    QT_TRY(choose_rank(h, o->s, cutoff, chi_max, o));
  }
  // a rank decision below the FP32 resolution that nothing certifies is
  // left to the caller's exact FP64 split
  if (cert && !certify_rank(o->s, extra_tail, cutoff, chi_max, cert, o)) return QT_UNCERTIFIED;
  const int k = o->k;
  const double sc = renorm_scale(h, *o) * out_scale;
  const float2 one = make_float2(1, 0), zero = make_float2(0, 0);
  const float2* psrc = proj ? proj : theta;
  const int64_t pn = proj ? proj_n : n;
  float2 *At, *Bt;
  QT_TRY(s.get(&At, (size_t)m * k));
  QT_TRY(s.get(&Bt, (size_t)k * pn));
  float2 *A0, *G, *W;
  QT_TRY(s.get(&A0, (size_t)m * k));
  QT_TRY(s.get(&G, (size_t)k * k));
  QT_TRY(s.get(&W, (size_t)k * k));
  if (!wide) QT_LAUNCH(h, gather_unit_cols_kernel<float2>, 256, 256, 0, X, m, m, perm, sig, k, A0);
  else QT_LAUNCH(h, gather_cols_kernel<float2>, 256, 256, 0, V, m, m, perm, k, A0);
  QT_TRY(qt_gemm_any(h, QT_OP_C, QT_OP_N, k, k, m, one, A0, m, A0, m, zero, G, k));
  QT_LAUNCH(h, newton_schulz_kernel, 256, 256, 0, G, k, W);
  QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, m, k, k, one, A0, m, W, k, zero, At, m));
  QT_TRY(qt_gemm_any(h, QT_OP_C, QT_OP_N, k, pn, m, one, At, m, psrc, m, zero, Bt, k));
  {
    // the kept values as reported: norms of the rows of B' = A'^H theta (an
    // exact projection, free of the small drift of the Jacobi column norms)
    QT_LAUNCH(h, row_norms_kernel, (unsigned)k, 256, 0, Bt, k, pn, sig);
    QT_CHECK_CUDA(h, cudaMemcpyAsync(o->s.data(), sig, sizeof(double) * k, cudaMemcpyDeviceToHost, h->stream));
  }
  QT_TRY(qt_dmalloc(h, (void**)Aout, sizeof(TO) * m * k));
  QT_TRY(qt_dmalloc(h, (void**)Bout, sizeof(TO) * k * pn));
  QT_LAUNCH(h, (convert_scale_kernel<float2, TO>), 256, 256, 0, At, *Aout, (int64_t)m * k, 1.0);
  QT_LAUNCH(h, (convert_scale_kernel<float2, TO>), 256, 256, 0, Bt, *Bout, (int64_t)k * pn, sc);
  return QT_OK;
}

__global__ void scale_columns_kernel(double2* X, int64_t rows, int64_t cols, int64_t ld, const double* s) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < rows * cols;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % rows, j = idx / rows;
    X[i + ld * j] = cscale(X[i + ld * j], s[j]);
  }
}

__global__ void iota_kernel(int* p, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

// Cross-check path: cuSOLVER zgesvd (library) on theta, same rank rule and split.
template <typename TO>
int svd_split_cusolver(qt_handle* h, double2* theta, int64_t m, int64_t n, double cutoff, int chi_max, TO** Aout,
                       TO** Bout, SvdOut* o) {
  qt_scratch s(h);
  const bool tr = m < n;
  const int64_t mm = tr ? n : m, nn = tr ? m : n;  // gesvd needs rows >= cols
  double2* X = theta;
  if (tr) {
    QT_TRY(s.get(&X, (size_t)mm * nn));
    QT_TRY(qt_adjoint_copy<double2>(h, theta, m, n, m, X, mm));
  }
  double2 *U, *VT, *work;
  double *S, *rwork;
  int *info, *perm;
  QT_TRY(s.get(&U, (size_t)mm * nn));
  QT_TRY(s.get(&VT, (size_t)nn * nn));
  QT_TRY(s.get(&S, (size_t)nn));
  QT_TRY(s.get(&rwork, (size_t)nn * 5));
  QT_TRY(s.get(&info, 1));
  QT_TRY(s.get(&perm, (size_t)nn));
  cusolverDnHandle_t cs;
  if (cusolverDnCreate(&cs) != CUSOLVER_STATUS_SUCCESS) return qt_fail(h, QT_ECUDA, "cusolverDnCreate failed");
  cusolverDnSetStream(cs, h->stream);
  int lwork = 0;
  cusolverDnZgesvd_bufferSize(cs, (int)mm, (int)nn, &lwork);
  int rc = s.get(&work, (size_t)lwork);
  if (rc == QT_OK) {
    if (cusolverDnZgesvd(cs, 'S', 'S', (int)mm, (int)nn, (cuDoubleComplex*)X, (int)mm, S, (cuDoubleComplex*)U,
                         (int)mm, (cuDoubleComplex*)VT, (int)nn, (cuDoubleComplex*)work, lwork, rwork,
                         info) != CUSOLVER_STATUS_SUCCESS)
      rc = qt_fail(h, QT_ECUDA, "cusolverDnZgesvd failed");
  }
  h->launches++;
  cusolverDnDestroy(cs);
  QT_TRY(rc);
  // As the transposed split: "Vx" holds unit vectors of the left factor and
  // "X" holds (right factor) x diag(S).  gesvd: X = U S VT.
  //   not transposed: theta = U S VT  -> left = U,          right^H = VT^H S
  //   transposed:     theta = VT^H S U^H -> left = VT^H,     right^H = U S
  double2 *L, *Rh;
  QT_TRY(s.get(&L, (size_t)std::max(mm, nn) * nn));
  QT_TRY(s.get(&Rh, (size_t)std::max(mm, nn) * nn));
  if (!tr) {
    QT_CHECK_CUDA(h, cudaMemcpyAsync(L, U, sizeof(double2) * m * nn, cudaMemcpyDeviceToDevice, h->stream));
    QT_TRY(qt_adjoint_copy<double2>(h, VT, nn, n, nn, Rh, n));
  } else {
    QT_TRY(qt_adjoint_copy<double2>(h, VT, nn, m, nn, L, m));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(Rh, U, sizeof(double2) * n * nn, cudaMemcpyDeviceToDevice, h->stream));
  }
  QT_LAUNCH(h, scale_columns_kernel, 256, 256, 0, Rh, n, nn, n, (const double*)S);
  QT_LAUNCH(h, iota_kernel, 8, 256, 0, perm, (int)nn);
  o->s.resize(nn);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(o->s.data(), S, sizeof(double) * nn, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  QT_TRY(choose_rank(h, o->s, cutoff, chi_max, o));
  QT_TRY(qt_dmalloc(h, (void**)Aout, sizeof(TO) * m * o->k));
  QT_TRY(qt_dmalloc(h, (void**)Bout, sizeof(TO) * o->k * n));
  QT_TRY((qt_absorb<double2, TO>(h, 1, Rh, n, L, m, S, perm, m, n, o->k, renorm_scale(h, *o), *Aout, *Bout)));
  return QT_OK;
}


// The exact FP64 split that decides where the chosen mode's FP32 split
// cannot (an uncertified rank, an unsettled Jacobi, a sketch that lost
// rank).  M (an FP64 copy) is overwritten.  For min(m, n) >= 512 it is
// cuSOLVER's zgesvd (1.76 s against 7.2 s for the engine's FP64 Jacobi at
// 2048 x 2048 on GB300, where FP64 runs at 1/64 of the FP32 rate); below,
// the FP64 Jacobi.  QT_FALLBACK_JACOBI=1 keeps the Jacobi at every size.
template <typename TO>
int svd_split_exact64(qt_handle* h, double2* M, int64_t m, int64_t n, double cutoff, int chi_max, TO** A, TO** B,
                      SvdOut* o) {
  static const bool jacobi_only = std::getenv("QT_FALLBACK_JACOBI") && std::atoi(std::getenv("QT_FALLBACK_JACOBI"));
  if (!jacobi_only && std::min(m, n) >= 512) return svd_split_cusolver<TO>(h, M, m, n, cutoff, chi_max, A, B, o);
  return svd_split_jacobi<double2, TO>(h, M, m, n, cutoff, chi_max, false, A, B, o);
}

// Chosen mode: FP32-level products, randomized range finder sized by the
// predicted rank, FP32-storage one-sided Jacobi on the small projected matrix
// (FP64 Gram/angles); exact FP64 SVD as fallback when the tail rule needs
// more values than the sketch holds, when the sketch basis lost rank, or when
// the Jacobi does not settle.  theta is m x n float2 (ld m); it is
// overwritten by the sketch residual.
// struct_rank bounds theta's rank in exact arithmetic (0: unknown); with it a
// cutoff below the FP32 resolution is still decided exactly when theta has
// no values between the cutoff and that resolution (certify_rank).
template <typename TO>
int svd_split_chosen(qt_handle* h, float2* theta, int64_t m, int64_t n, double cutoff, int chi_max, int kpred,
                     TO** Aout, TO** Bout, SvdOut* o, int* sketch, int* fallback, double* residual,
                     int64_t struct_rank = 0) {
  qt_scratch s(h);
  const int64_t kmin = std::min(m, n);
  double* dn;
  QT_TRY(s.get(&dn, 1));
  QT_TRY(qt_norm2<float2>(h, theta, m * n, dn));
  double tn2 = 0;
  QT_CHECK_CUDA(h, cudaMemcpyAsync(&tn2, dn, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  // the rule runs at the caller's cutoff; eta is the FP32 resolution below
  // which the decision needs a certificate or the exact split
  const double eta = fp32_floor_rel(h, m, n) * std::sqrt(tn2);
  RankCert cert;
  cert.eta = eta;
  cert.struct_rank = struct_rank;
  int64_t l = (kpred > 0 ? kpred : kmin) + std::max(0, h->cfg.oversample);
  // A rank predicted at the chi_max cap is pinned there by a spectrum that
  // is still decaying slowly at the cap; a sketch of cap + oversample then
  // misses the kept space by far more than the exact truncation does, so the
  // sketch is widened to 1.125 x the cap.  With one power iteration that keeps
  // the truncation error within 1.0001 of the exact split at chi = 1024
  // (1152 columns: 1.00008; 1216: 1.00006; 1280: 1.00005; no power
  // iteration at 1280: 1.10), and the Jacobi on the sketched matrix, free of
  // the FP32 noise columns of theta', settles in 5 sweeps instead of ~20 on
  // the whole theta'.
  const bool cap_bound = chi_max > 0 && chi_max < kmin && kpred > 0 && kpred + h->cfg.oversample >= 0.9 * chi_max;
  // (cfg.cap_sketch sets the factor, as the autotuner chooses it; QT_CAP_SKETCH
  // overrides the default when it is unset)
  static const double cap_env = std::getenv("QT_CAP_SKETCH") ? std::atof(std::getenv("QT_CAP_SKETCH")) : 1.125;
  const double cap_mult = h->cfg.cap_sketch > 0 ? h->cfg.cap_sketch : cap_env;
  // (and by at least 64 columns: at chi = 64 a sketch of 80 left 1.006 x)
  if (cap_bound) l = std::max<int64_t>(l, std::max<int64_t>((int64_t)(cap_mult * chi_max), chi_max + 64));
  l = ((l + 7) / 8) * 8;
  *fallback = 0;
  *residual = 0;
  // A sketch of three quarters of the matrix or more saves less in the small
  // SVD than its range finder and orthogonalisation cost: factor theta'
  // directly.
  // freezing columns below sqrt(rows) u ||theta|| leaves every value above
  // eta intact, which is all a certificate below eta looks at
  const bool fast = cap_bound || cutoff < eta || fast_freeze_ok(m, n, cutoff, std::sqrt(tn2));
  if (4 * l >= 3 * kmin || kmin <= 32) {
    *sketch = 0;
    const int rc = svd_split_direct32<TO>(h, theta, m, n, cutoff, chi_max, Aout, Bout, o, -1.0, fast,
                                          cap_bound ? chi_max : 0, nullptr, 0, 1.0, &cert);
    h->cert_count[cert.how]++;
    if (rc == QT_ENUMERIC || rc == QT_UNCERTIFIED) {  // no settled Jacobi / no certified rank: exact FP64 path
      qt_dfree(h, *Aout);
      qt_dfree(h, *Bout);
      *Aout = *Bout = nullptr;
      *fallback = rc == QT_ENUMERIC ? 2 : 4;
      return QT_OK;
    }
    return rc;
  }
  *sketch = (int)l;
  // the range finder's Gram matrices are FP32: work on theta 2^-e (theta is
  // this function's to overwrite) and scale the results back at the end
  const int e = fp32_scale_exponent(tn2);
  const double up = std::ldexp(1.0, e);
  if (e) QT_LAUNCH(h, scale_pow2_kernel<float2>, 256, 256, 0, theta, m * n, 1.0 / up);
  const double cut_s = e ? cutoff / up : cutoff;
  cert.eta = e ? eta / up : eta;
  const float2 one = make_float2(1, 0), zero = make_float2(0, 0), mone = make_float2(-1, 0);
  // The sketch spans theta's row space: Y (n x l) orthonormal, C = theta Y
  // (m x l) tall, so its one-sided Jacobi carries no V; A' comes from C and
  // B' = A'^H theta is the exact projection of the whole matrix.
  float2 *om, *Y, *Z, *Cm, *Rm;
  QT_TRY(s.get(&om, (size_t)m * l));
  QT_TRY(s.get(&Y, (size_t)n * l));
  QT_TRY(s.get(&Z, (size_t)m * l));
  QT_TRY(s.get(&Cm, (size_t)m * l));
  QT_TRY(s.get(&Rm, (size_t)m * n));
  QT_CHECK_CUDA(h, cudaMemsetAsync(h->d_flags + QT_FLAG_CHOL, 0, sizeof(int), h->stream));
  // range finder: Y = theta^H Omega, q rounds of subspace iteration
  QT_TRY(qt_gaussian<float2>(h, om, m, l, m, h->cfg.seed + 0x9E37ull * (++h->sketch_counter)));
  QT_TRY(qt_gemm_any(h, QT_OP_C, QT_OP_N, n, l, m, one, theta, m, om, m, zero, Y, n));
  QT_TRY(qt_orthonormalize<float2>(h, Y, n, l, h->cfg.power_iters > 0 ? QT_ORTH_USE_RANGE : QT_ORTH_USE_SKETCH));
  for (int q = 0; q < h->cfg.power_iters; q++) {
    QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, m, l, n, one, theta, m, Y, n, zero, Z, m));
    QT_TRY(qt_orthonormalize<float2>(h, Z, m, l, QT_ORTH_USE_RANGE));
    QT_TRY(qt_gemm_any(h, QT_OP_C, QT_OP_N, n, l, m, one, theta, m, Z, m, zero, Y, n));
    QT_TRY(qt_orthonormalize<float2>(h, Y, n, l, q + 1 < h->cfg.power_iters ? QT_ORTH_USE_RANGE : QT_ORTH_USE_SKETCH));
  }
  {
    // a Cholesky pivot that vanished means the sketch held fewer than l
    // numerically independent directions: the basis is not trustworthy
    int chol = 0;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(&chol, h->d_flags + QT_FLAG_CHOL, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (chol) {
      *fallback = 3;
      return QT_OK;
    }
  }
  // C = theta Y; residual theta - C Y^H (its weight is a tail value of the rule)
  QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, m, l, n, one, theta, m, Y, n, zero, Cm, m));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(Rm, theta, sizeof(float2) * m * n, cudaMemcpyDeviceToDevice, h->stream));
  QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_C, m, n, l, mone, Cm, m, Y, n, one, Rm, m));
  QT_TRY(qt_norm2<float2>(h, Rm, m * n, dn));
  double res2 = 0;
  QT_CHECK_CUDA(h, cudaMemcpyAsync(&res2, dn, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  *residual = std::sqrt(res2);
  // the split of the tall C (m x l): A' from its Jacobi, B' = A'^H theta
  {
    const int rc = svd_split_direct32<TO>(h, Cm, m, l, cut_s, chi_max, Aout, Bout, o, *residual, fast,
                                          cap_bound ? chi_max : 0, theta, n, up, &cert);
    h->cert_count[cert.how]++;
    if (rc == QT_ENUMERIC || rc == QT_UNCERTIFIED) {  // no settled small SVD / no certified rank: exact FP64 path
      qt_dfree(h, *Aout);
      qt_dfree(h, *Bout);
      *Aout = *Bout = nullptr;
      *fallback = rc == QT_ENUMERIC ? 2 : 4;
      return QT_OK;
    }
    QT_TRY(rc);
  }
  const bool held_by_cap = chi_max > 0 && chi_max + std::max(0, h->cfg.oversample) <= l;
  if (o->k_cut > (int)l && !held_by_cap) {  // the cutoff needs more than the sketch holds
    qt_dfree(h, *Aout);
    qt_dfree(h, *Bout);
    *Aout = *Bout = nullptr;
    *fallback = 1;
    return QT_OK;
  }
  if (e) {  // back to theta's scale: the values, the weights, the residual (B' is scaled already)
    for (double& v : o->s) v *= up;
    o->norm2 *= up * up;
    o->discarded *= up * up;
    *residual *= up;
  }
  return QT_OK;
}

}  // namespace

// Truncated split M (m x n, device, element of `dtype`) ~ A (m x k) B (k x n),
// A orthonormal, B = diag(S) V^H; A, B are pool allocations the caller frees.
// Plain mode runs the exact FP64 path; chosen mode on complex64 keeps FP32
// storage.
int qt_split_device(qt_handle* h, int dtype, const void* M, int64_t m, int64_t n, double cutoff, int chi_max, int mode,
                    void** A, void** B, int* k, double* discarded, int64_t struct_rank) {
  SvdOut o;
  *A = *B = nullptr;
  int rc;
  if (dtype == QT_C128) {
    qt_scratch s(h);
    double2* Mc;
    QT_TRY(s.get(&Mc, (size_t)m * n));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(Mc, M, sizeof(double2) * m * n, cudaMemcpyDeviceToDevice, h->stream));
    if (mode == QT_MODE_CUSOLVER)
      rc = svd_split_cusolver<double2>(h, Mc, m, n, cutoff, chi_max, (double2**)A, (double2**)B, &o);
    else
      rc = svd_split_jacobi<double2, double2>(h, Mc, m, n, cutoff, chi_max, false, (double2**)A, (double2**)B, &o);
  } else if (mode == QT_MODE_CHOSEN) {
    qt_scratch s(h);
    double* dn;
    QT_TRY(s.get(&dn, 1));
    QT_TRY(qt_norm2<float2>(h, (const float2*)M, m * n, dn));
    double n2 = 0;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(&n2, dn, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    RankCert cert;
    cert.eta = fp32_floor_rel(h, m, n) * std::sqrt(n2);
    cert.struct_rank = struct_rank;
    rc = svd_split_direct32<float2>(h, (const float2*)M, m, n, cutoff, chi_max, (float2**)A, (float2**)B, &o, -1.0,
                                    cutoff < cert.eta || fast_freeze_ok(m, n, cutoff, std::sqrt(n2)), 0, nullptr, 0,
                                    1.0, &cert);
    h->cert_count[cert.how]++;
    if (rc == QT_UNCERTIFIED || rc == QT_ENUMERIC) {  // the exact FP64 split decides
      qt_dfree(h, *A);
      qt_dfree(h, *B);
      *A = *B = nullptr;
      double2* Mc;
      QT_TRY(s.get(&Mc, (size_t)m * n));
      QT_TRY(qt_convert(h, M, QT_C64, Mc, QT_C128, m * n));
      o = SvdOut();
      rc = svd_split_exact64<float2>(h, Mc, m, n, cutoff, chi_max, (float2**)A, (float2**)B, &o);
      if (rc != QT_OK) rc = QT_EFALLBACK_FAILED;
    }
  } else {
    qt_scratch s(h);
    double2* Mc;
    QT_TRY(s.get(&Mc, (size_t)m * n));
    QT_TRY(qt_convert(h, M, QT_C64, Mc, QT_C128, m * n));
    if (mode == QT_MODE_CUSOLVER)
      rc = svd_split_cusolver<float2>(h, Mc, m, n, cutoff, chi_max, (float2**)A, (float2**)B, &o);
    else
      rc = svd_split_jacobi<double2, float2>(h, Mc, m, n, cutoff, chi_max, false, (float2**)A, (float2**)B, &o);
  }
  {
    // a bounded device wait that gave up is the cause of whatever followed it
    const int st = qt_check_status(h);
    if (st != QT_OK) rc = st;
  }
  if (rc != QT_OK) {
    qt_dfree(h, *A);
    qt_dfree(h, *B);
    *A = *B = nullptr;
    return rc;
  }
  *k = o.k;
  if (discarded) *discarded = o.discarded;
  return QT_OK;
}

// ---------------------------------------------------------------------------
// the update
// ---------------------------------------------------------------------------

static bool finite_gate(const double* G) {
  for (int i = 0; i < 32; i++)
    if (!std::isfinite(G[i])) return false;
  return true;
}

template <typename TO>
static int update_impl(qt_handle* h, qt_mps* mps, int site, const double* G, double cutoff, int chi_max, int mode,
                       qt_update_stats* st) {
  const int64_t cl = mps->chil[site], cm = mps->chir[site], cr = mps->chir[site + 1];
  const int64_t m = 2 * cl, n = 2 * cr;
  SvdOut o;
  TO *An = nullptr, *Bn = nullptr;
  int sketch = 0, fallback = 0, kpred = -1;
  double residual = 0;
  int rc = QT_OK;
  float feat[QT_MLP_IN];
  const int kmax = qt_rank_kmax(mps, site, chi_max);
  qt_rank_features(mps, site, G, cutoff < 0 ? 0.0 : cutoff, chi_max, feat);
  {
    qt_scratch s(h);
    if (mode == QT_MODE_CHOSEN) {
      float2* th;
      QT_TRY(s.get(&th, (size_t)m * n));
      if (h->cfg.tc_gemm && mps->dtype == QT_C64 && m >= 64 && n >= 32 && cm >= 32) {
        // theta = A_mat (2chiL x chiM) . B_mat (chiM x 2chiR) on the tensor cores, then the gate
        const float2 one = make_float2(1.f, 0.f), zero = make_float2(0.f, 0.f);
        QT_TRY(qt_cgemm_tc(h, QT_OP_N, QT_OP_N, m, n, cm, one, (const float2*)mps->site[site], m,
                           (const float2*)mps->site[site + 1], cm, zero, th, m));
        QT_TRY(qt_apply_gate_inplace(h, th, cl, cr, G));
      } else {
        QT_TRY(qt_theta_gate(h, mps->dtype, mps->site[site], mps->site[site + 1], cl, cm, cr, G, 1, th));
      }
      kpred = qt_rank_model_predict(h, feat, kmax);
      // exact-arithmetic rank bound of theta' = G (A B): the gate's
      // operator-Schmidt rank times the inner bond, and the Hilbert-space
      // dimensions of the qubits left and right of the bond
      int64_t srank = std::min<int64_t>(std::min(m, n), (int64_t)qt_gate_schmidt_rank(G) * cm);
      if (site + 1 < 40) srank = std::min<int64_t>(srank, (int64_t)1 << (site + 1));
      if (mps->nsites - site - 1 < 40) srank = std::min<int64_t>(srank, (int64_t)1 << (mps->nsites - site - 1));
      rc = svd_split_chosen<TO>(h, th, m, n, cutoff, chi_max, kpred, &An, &Bn, &o, &sketch, &fallback, &residual,
                                srank);
      if (rc == QT_OK && fallback) {
        qt_dfree(h, An);
        qt_dfree(h, Bn);
        An = Bn = nullptr;
        double2* th64;
        QT_TRY(s.get(&th64, (size_t)m * n));
        QT_TRY(qt_theta_gate(h, mps->dtype, mps->site[site], mps->site[site + 1], cl, cm, cr, G, 0, th64));
        rc = svd_split_exact64<TO>(h, th64, m, n, cutoff, chi_max, &An, &Bn, &o);
        if (rc != QT_OK) rc = QT_EFALLBACK_FAILED;
      }
    } else {
      double2* th;
      QT_TRY(s.get(&th, (size_t)m * n));
      QT_TRY(qt_theta_gate(h, mps->dtype, mps->site[site], mps->site[site + 1], cl, cm, cr, G, 0, th));
      if (mode == QT_MODE_CUSOLVER) rc = svd_split_cusolver<TO>(h, th, m, n, cutoff, chi_max, &An, &Bn, &o);
      else rc = svd_split_jacobi<double2, TO>(h, th, m, n, cutoff, chi_max, false, &An, &Bn, &o);
    }
  }
  {
    // a bounded device wait that gave up is the cause of whatever followed it
    const int st = qt_check_status(h);
    if (st != QT_OK) rc = st;
  }
  if (rc != QT_OK) {
    qt_dfree(h, An);
    qt_dfree(h, Bn);
    cudaStreamSynchronize(h->stream);
    return rc;
  }
  const int k = o.k;
  replace_site(h, mps, site, cl, k, An, sizeof(TO) * m * k);
  replace_site(h, mps, site + 1, k, cr, Bn, sizeof(TO) * k * n);
  mps->spectrum[site].assign(o.s.begin(), o.s.begin() + std::min<size_t>(o.s.size(), (size_t)k));
  mps->bond_updates[site]++;
  // the rank model learns from exact FP64 splits (the engine's Jacobi or cuSOLVER)
  if ((mode == QT_MODE_PLAIN || mode == QT_MODE_CUSOLVER) && cutoff >= 0) qt_rank_model_log(h, feat, o.k, kmax);
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  if (st) {
    st->rank = k;
    st->rank_cutoff = o.k_cut;
    st->predicted_rank = kpred;
    st->sketch_size = sketch;
    st->fallback = fallback;
    st->sweeps = o.sweeps;
    st->discarded_weight = o.discarded;
    st->norm2 = o.norm2;
    st->residual = residual;
  }
  return QT_OK;
}

extern "C" int qt_apply_2q(qt_handle* h, qt_mps* mps, int site, const double* G, double cutoff, int chi_max, int mode,
                           qt_update_stats* st) {
  if (!h || !mps || !G) return qt_fail(h, QT_EINVAL, "apply_2q: null argument");
  if (site < 0 || site + 1 >= mps->nsites) return qt_fail(h, QT_EBOUNDS, "apply_2q: site out of range");
  if (cutoff < 0) cutoff = h->cfg.cutoff;
  if (chi_max < 0) chi_max = h->cfg.chi_max;
  if (mode < 0) mode = h->cfg.mode;
  if (!(cutoff >= 0)) return qt_fail(h, QT_EINVAL_ERR_NEG, "Error must be positive");
  if (mode != QT_MODE_PLAIN && mode != QT_MODE_CHOSEN && mode != QT_MODE_CUSOLVER)
    return qt_fail(h, QT_EINVAL, "apply_2q: unknown mode");
  if (!finite_gate(G)) return qt_fail(h, QT_ENUMERIC, "apply_2q: non-finite gate entry");
  cudaSetDevice(h->device);
  if (mps->dtype == QT_C128) return update_impl<double2>(h, mps, site, G, cutoff, chi_max, mode, st);
  return update_impl<float2>(h, mps, site, G, cutoff, chi_max, mode, st);
}

extern "C" int qt_switch(qt_handle* h, qt_mps* mps, int site) {
  // switch!(mps, i): the swap gate with no truncation, the plain FP64 path
  if (!h || !mps) return qt_fail(h, QT_EINVAL, "switch: null argument");
  if (site < 0 || site + 1 >= mps->nsites) return qt_fail(h, QT_EBOUNDS, "switch: site out of range");
  // the SWAP gate, column-major interleaved: e0->e0, e1->e2, e2->e1, e3->e3
  double G[32];
  std::memset(G, 0, sizeof(G));
  G[2 * (0 + 4 * 0)] = 1;
  G[2 * (2 + 4 * 1)] = 1;
  G[2 * (1 + 4 * 2)] = 1;
  G[2 * (3 + 4 * 3)] = 1;
  cudaSetDevice(h->device);
  // no truncation at all: the reference keeps bond_dim = length(S)
  if (mps->dtype == QT_C128) return update_impl<double2>(h, mps, site, G, -1.0, 0, QT_MODE_PLAIN, nullptr);
  return update_impl<float2>(h, mps, site, G, -1.0, 0, QT_MODE_PLAIN, nullptr);
}

extern "C" int qt_expect_z(qt_handle* h, const qt_mps* mps, int site, double* out) {
  if (!h || !mps || !out) return qt_fail(h, QT_EINVAL, "expect_z: null argument");
  double num = 0, den = 0;
  QT_TRY(qt_mps_expect(h, mps, site, 1, &num));
  QT_TRY(qt_mps_expect(h, mps, 0, 0, &den));
  *out = num / den;
  return QT_OK;
}

extern "C" int qt_expect_zz(qt_handle* h, const qt_mps* mps, int site, double* out) {
  if (!h || !mps || !out) return qt_fail(h, QT_EINVAL, "expect_zz: null argument");
  double num = 0, den = 0;
  QT_TRY(qt_mps_expect(h, mps, site, 2, &num));
  QT_TRY(qt_mps_expect(h, mps, 0, 0, &den));
  *out = num / den;
  return QT_OK;
}

extern "C" int qt_mps_norm2(qt_handle* h, const qt_mps* mps, double* out) {
  if (!h || !mps || !out) return qt_fail(h, QT_EINVAL, "mps_norm2: null argument");
  return qt_mps_expect(h, mps, 0, 0, out);
}

// ---------------------------------------------------------------------------
// dense primitives on host buffers
// ---------------------------------------------------------------------------

// (qt_contract_pair, the ncon pairwise step on host buffers, is in k_ncon.cu
// with the device-resident tensors it runs on.)

extern "C" int qt_gemm(qt_handle* h, int dtype, int opA, int opB, int64_t M, int64_t N, int64_t K,
                       const double* alpha, const void* A, int64_t lda, const void* B, int64_t ldb,
                       const double* beta, void* C, int64_t ldc) {
  if (!h || !alpha || !beta || !A || !B || !C) return qt_fail(h, QT_EINVAL, "gemm: null argument");
  if (M < 1 || N < 1 || K < 1) return qt_fail(h, QT_EINVAL, "gemm: empty operand");
  if ((opA != QT_OP_N && opA != QT_OP_C) || (opB != QT_OP_N && opB != QT_OP_C))
    return qt_fail(h, QT_EINVAL, "gemm: op must be N or C");
  if (dtype != QT_C64 && dtype != QT_C128) return qt_fail(h, QT_EINVAL, "gemm: bad dtype");
  const int64_t ar = opA == QT_OP_N ? M : K, ac = opA == QT_OP_N ? K : M;
  const int64_t br = opB == QT_OP_N ? K : N, bc = opB == QT_OP_N ? N : K;
  if (lda < ar || ldb < br || ldc < M) return qt_fail(h, QT_EINVAL, "gemm: leading dimension too small");
  cudaSetDevice(h->device);
  const size_t es = dtype == QT_C64 ? sizeof(float2) : sizeof(double2);
  qt_scratch s(h);
  unsigned char *dA, *dB, *dC;
  QT_TRY(s.get(&dA, es * lda * ac));
  QT_TRY(s.get(&dB, es * ldb * bc));
  QT_TRY(s.get(&dC, es * ldc * N));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dA, A, es * lda * ac, cudaMemcpyHostToDevice, h->stream));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dB, B, es * ldb * bc, cudaMemcpyHostToDevice, h->stream));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dC, C, es * ldc * N, cudaMemcpyHostToDevice, h->stream));
  if (dtype == QT_C64) {
    QT_TRY(qt_cgemm_c64(h, opA, opB, M, N, K, make_float2((float)alpha[0], (float)alpha[1]), (const float2*)dA, lda,
                        (const float2*)dB, ldb, make_float2((float)beta[0], (float)beta[1]), (float2*)dC, ldc));
  } else {
    QT_TRY(qt_cgemm<double2>(h, opA, opB, M, N, K, make_double2(alpha[0], alpha[1]), (const double2*)dA, lda,
                             (const double2*)dB, ldb, make_double2(beta[0], beta[1]), (double2*)dC, ldc));
  }
  QT_TRY(qt_check_status(h));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(C, dC, es * ldc * N, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}


namespace {

// Host-facing truncated SVD, results in FP64.  M64 (FP64 copy of the input)
// feeds the exact paths; M32 (the complex64 input itself, chosen mode) feeds
// the FP32-storage Jacobi, whose rank decision at a cutoff below its
// resolution 4 sqrt(max(m, n)) u_fp32 ||M||_F is certified by the chi_max cap
// or left to the exact FP64 split of M64.
int host_truncated_svd64(qt_handle* h, const double2* M64, const float2* M32, int64_t m, int64_t n, double cutoff,
                         int chi_max, int mode, std::vector<double2>* U, std::vector<double>* S,
                         std::vector<double2>* Vh, int* k, double* disc) {
  qt_scratch s(h);
  SvdOut o;
  double2 *A = nullptr, *B = nullptr;
  int rc;
  if (M32) {
    float2* dM;
    QT_TRY(s.get(&dM, (size_t)m * n));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(dM, M32, sizeof(float2) * m * n, cudaMemcpyHostToDevice, h->stream));
    double* dn;
    QT_TRY(s.get(&dn, 1));
    QT_TRY(qt_norm2<float2>(h, dM, m * n, dn));
    double n2 = 0;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(&n2, dn, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    RankCert cert;
    cert.eta = fp32_floor_rel(h, m, n) * std::sqrt(n2);
    rc = svd_split_direct32<double2>(h, dM, m, n, cutoff, chi_max, &A, &B, &o, -1.0,
                                     cutoff < cert.eta || fast_freeze_ok(m, n, cutoff, std::sqrt(n2)), 0, nullptr, 0,
                                     1.0, &cert);
    h->cert_count[cert.how]++;
    if (rc == QT_UNCERTIFIED || rc == QT_ENUMERIC) {  // the exact FP64 split decides
      qt_dfree(h, A);
      qt_dfree(h, B);
      A = B = nullptr;
      double2* dM64;
      QT_TRY(s.get(&dM64, (size_t)m * n));
      QT_CHECK_CUDA(h, cudaMemcpyAsync(dM64, M64, sizeof(double2) * m * n, cudaMemcpyHostToDevice, h->stream));
      o = SvdOut();
      rc = svd_split_exact64<double2>(h, dM64, m, n, cutoff, chi_max, &A, &B, &o);
      if (rc != QT_OK) rc = QT_EFALLBACK_FAILED;
    }
  } else {
    double2* dM;
    QT_TRY(s.get(&dM, (size_t)m * n));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(dM, M64, sizeof(double2) * m * n, cudaMemcpyHostToDevice, h->stream));
    rc = (mode == QT_MODE_CUSOLVER) ? svd_split_cusolver<double2>(h, dM, m, n, cutoff, chi_max, &A, &B, &o)
                                    : svd_split_jacobi<double2, double2>(h, dM, m, n, cutoff, chi_max, false, &A, &B, &o);
  }
  {
    // a bounded device wait that gave up is the cause of whatever followed it
    const int st = qt_check_status(h);
    if (st != QT_OK) rc = st;
  }
  if (rc == QT_OK) {
    U->resize((size_t)m * o.k);
    Vh->resize((size_t)o.k * n);
    cudaMemcpyAsync(U->data(), A, sizeof(double2) * m * o.k, cudaMemcpyDeviceToHost, h->stream);
    cudaMemcpyAsync(Vh->data(), B, sizeof(double2) * o.k * n, cudaMemcpyDeviceToHost, h->stream);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) rc = qt_fail(h, QT_ECUDA, "svd download failed");
    S->assign(o.s.begin(), o.s.begin() + o.k);
    // B = diag(S) Vh: divide the rows back out (exact zeros keep zero rows)
    for (int j = 0; j < o.k; j++) {
      const double sj = (*S)[j];
      const double sc = renorm_scale(h, o);
      for (int64_t c = 0; c < n; c++) {
        double2& v = (*Vh)[j + (size_t)o.k * c];
        const double f = (sj > 0) ? 1.0 / (sj * sc) : 0.0;
        v.x *= f;
        v.y *= f;
      }
    }
    *k = o.k;
    *disc = o.discarded;
  }
  qt_dfree(h, A);
  qt_dfree(h, B);
  return rc;
}

}  // namespace

extern "C" int qt_truncated_svd(qt_handle* h, int dtype, int64_t m, int64_t n, const void* M, double cutoff,
                                int chi_max, int mode, void* U, double* S, void* Vh, int* k, double* discarded) {
  if (!h || !M || !U || !S || !Vh || !k) return qt_fail(h, QT_EINVAL, "truncated_svd: null argument");
  if (!(cutoff >= 0)) return qt_fail(h, QT_EINVAL_ERR_NEG, "Error must be positive");
  if (m < 1 || n < 1) return qt_fail(h, QT_EINVAL, "truncated_svd: empty matrix");
  cudaSetDevice(h->device);
  if (mode < 0) mode = QT_MODE_PLAIN;
  const int64_t kcap = std::min(m, n);
  std::vector<double2> M64((size_t)m * n), u, vh;
  std::vector<double> s;
  for (int64_t i = 0; i < m * n; i++)
    M64[i] = (dtype == QT_C64) ? make_double2(((const float2*)M)[i].x, ((const float2*)M)[i].y) : ((const double2*)M)[i];
  int kk = 0;
  double disc = 0;
  const bool fp32 = dtype == QT_C64 && mode == QT_MODE_CHOSEN;
  QT_TRY(host_truncated_svd64(h, M64.data(), fp32 ? (const float2*)M : nullptr, m, n, cutoff, chi_max,
                              mode == QT_MODE_CUSOLVER ? mode : QT_MODE_PLAIN, &u, &s, &vh, &kk, &disc));
  for (int j = 0; j < kk; j++) S[j] = s[j];
  for (int64_t j = 0; j < kcap; j++)
    for (int64_t i = 0; i < m; i++) {
      const double2 v = (j < kk) ? u[i + (size_t)m * j] : make_double2(0, 0);
      if (dtype == QT_C64) ((float2*)U)[i + m * j] = make_float2((float)v.x, (float)v.y);
      else ((double2*)U)[i + m * j] = v;
    }
  for (int64_t c = 0; c < n; c++)
    for (int64_t j = 0; j < kcap; j++) {
      const double2 v = (j < kk) ? vh[j + (size_t)kk * c] : make_double2(0, 0);
      if (dtype == QT_C64) ((float2*)Vh)[j + kcap * c] = make_float2((float)v.x, (float)v.y);
      else ((double2*)Vh)[j + kcap * c] = v;
    }
  *k = kk;
  if (discarded) *discarded = disc;
  return QT_OK;
}

extern "C" int qt_contract_svd(qt_handle* h, int dtype, int nd1, const int64_t* dims1, const void* T1, int nd2,
                               const int64_t* dims2, const void* T2, int i1, int i2, double er, void* out) {
  // src/svd.jl:7-38.  Argument checks in the reference's order.
  if (!h || !dims1 || !dims2 || !T1 || !T2 || !out) return qt_fail(h, QT_EINVAL, "contract_svd: null argument");
  if (!(er >= 0)) return qt_fail(h, QT_EINVAL_ERR_NEG, "Error must be positive");
  if (i1 < 1 || i2 < 1) return qt_fail(h, QT_EINVAL, "contract_svd: leg numbers are 1-based");
  const int64_t D1 = (i1 <= nd1) ? dims1[i1 - 1] : 1, D2 = (i2 <= nd2) ? dims2[i2 - 1] : 1;
  if (D1 != D2) return qt_fail(h, QT_EDIM_MISMATCH, "Dimensions of contraction legs do not match");
  if (i1 > nd1 || i2 > nd2) return qt_fail(h, QT_ENOTSUP, "contract_svd: trailing singleton legs");
  if (dtype != QT_C64 && dtype != QT_C128) return qt_fail(h, QT_EINVAL, "contract_svd: bad dtype");
  cudaSetDevice(h->device);
  // the operands on the device in FP64 (the plain path of the reference's svd)
  int64_t n1 = 1, n2 = 1;
  for (int i = 0; i < nd1; i++) n1 *= dims1[i];
  for (int i = 0; i < nd2; i++) n2 *= dims2[i];
  std::vector<double2> t1((size_t)n1), t2((size_t)n2);
  for (int64_t i = 0; i < n1; i++)
    t1[i] = (dtype == QT_C64) ? make_double2(((const float2*)T1)[i].x, ((const float2*)T1)[i].y) : ((const double2*)T1)[i];
  for (int64_t i = 0; i < n2; i++)
    t2[i] = (dtype == QT_C64) ? make_double2(((const float2*)T2)[i].x, ((const float2*)T2)[i].y) : ((const double2*)T2)[i];
  // T1p = permutedims(T1, [rest..., i1]) as (:, D1); T2p = permutedims(T2, [i2, rest...]) as (D1, :)
  // (src/svd.jl:20-24), permuted on the device
  std::vector<int> p1, p2;
  for (int i = 0; i < nd1; i++) if (i != i1 - 1) p1.push_back(i);
  p1.push_back(i1 - 1);
  p2.push_back(i2 - 1);
  for (int i = 0; i < nd2; i++) if (i != i2 - 1) p2.push_back(i);
  qt_tensor *a0 = nullptr, *b0 = nullptr, *a = nullptr, *b = nullptr;
  int rc = qt_tensor_create(h, QT_C128, nd1, dims1, t1.data(), &a0);
  if (rc == QT_OK) rc = qt_tensor_create(h, QT_C128, nd2, dims2, t2.data(), &b0);
  if (rc == QT_OK) rc = qt_tensor_permute(h, a0, p1.data(), &a);
  if (rc == QT_OK) rc = qt_tensor_permute(h, b0, p2.data(), &b);
  qt_tensor_free(h, a0);
  qt_tensor_free(h, b0);
  const int64_t m1 = n1 / D1, m2 = n2 / D1;
  // two truncated splits (src/svd.jl:26-33): T1p ~ A1 (diag(S1) V1'), T2p ~ A2 (diag(S2) V2'),
  // then the product chain of :35, U1 S1 V1' U2 S2 V2', as ((A1 B1) A2) B2
  void *A1 = nullptr, *B1 = nullptr, *A2 = nullptr, *B2 = nullptr;
  int k1 = 0, k2 = 0;
  double dd = 0;
  if (rc == QT_OK)
    rc = qt_split_device(h, QT_C128, qt_tensor_data(a), m1, D1, er, 0, QT_MODE_PLAIN, &A1, &B1, &k1, &dd, 0);
  if (rc == QT_OK)
    rc = qt_split_device(h, QT_C128, qt_tensor_data(b), D1, m2, er, 0, QT_MODE_PLAIN, &A2, &B2, &k2, &dd, 0);
  qt_tensor_free(h, a);
  qt_tensor_free(h, b);
  std::vector<double2> res((size_t)m1 * m2);
  if (rc == QT_OK) {
    qt_scratch s(h);
    double2 *L = nullptr, *LA = nullptr, *T = nullptr;
    const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
    rc = s.get(&L, (size_t)m1 * D1);
    if (rc == QT_OK) rc = s.get(&LA, (size_t)m1 * k2);
    if (rc == QT_OK) rc = s.get(&T, (size_t)m1 * m2);
    if (rc == QT_OK)
      rc = qt_cgemm<double2>(h, QT_OP_N, QT_OP_N, m1, D1, k1, one, (const double2*)A1, m1, (const double2*)B1, k1,
                             zero, L, m1);
    if (rc == QT_OK)
      rc = qt_cgemm<double2>(h, QT_OP_N, QT_OP_N, m1, k2, D1, one, L, m1, (const double2*)A2, D1, zero, LA, m1);
    if (rc == QT_OK)
      rc = qt_cgemm<double2>(h, QT_OP_N, QT_OP_N, m1, m2, k2, one, LA, m1, (const double2*)B2, k2, zero, T, m1);
    if (rc == QT_OK && (cudaMemcpyAsync(res.data(), T, sizeof(double2) * m1 * m2, cudaMemcpyDeviceToHost,
                                        h->stream) != cudaSuccess ||
                        cudaStreamSynchronize(h->stream) != cudaSuccess))
      rc = qt_fail(h, QT_ECUDA, "contract_svd: download failed");
  }
  qt_dfree(h, A1);
  qt_dfree(h, B1);
  qt_dfree(h, A2);
  qt_dfree(h, B2);
  QT_TRY(rc);
  for (int64_t i = 0; i < m1 * m2; i++) {
    if (dtype == QT_C64) ((float2*)out)[i] = make_float2((float)res[i].x, (float)res[i].y);
    else ((double2*)out)[i] = res[i];
  }
  return QT_OK;
}
