// Batched two-qubit gate + truncated-SVD updates over many independent
// circuits (uneven qubit counts, bond caps and depths).
//
// Storage: every circuit c owns nsites(c) site slots of cap(c) x 2 x cap(c)
// complex64 (cap = its chi_max) in one device buffer, and a bond-dimension
// array bonds[c][0..n] on the device (site i is (bonds[i], 2, bonds[i+1])).
//
// One launch per circuit layer: a persistent kernel whose CTAs take
// (circuit, site) tasks from an atomic counter and run a whole update each:
//   theta' = G (A B)            FP32, gate folded per (a, b), kept in a per-CTA slab
//   one-sided Jacobi on theta'  FP32 columns, warps on disjoint column pairs of a
//                               round-robin round, rotation angles in FP64
//   sigma_j = ||x_j||           FP64, bitonic sort, tail rule (FP64, sequential),
//                               effective cutoff max(cutoff, floor ||theta'||), cap
//   A' = x_perm(j) / sigma_j    written into site slot w
//   B' = A'^H theta'            written into site slot w+1 (no V accumulation)
//   bonds[w+1] = k
// Tasks of one brickwork layer touch disjoint sites, so CTAs never race.  A
// whole program (every layer) is a fixed sequence of (counter reset, kernel)
// pairs that the host captures once in a CUDA graph.  There are no waits on
// other CTAs: a CTA stops when the counter passes the task count.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "qt_internal.cuh"

namespace {

constexpr int BT = 256;            // threads per CTA
constexpr int BWARPS = BT / 32;
constexpr int MAXN = 256;          // largest 2 * cap handled (cap <= 128)

struct BatchArgs {
  float2* sites;
  const int64_t* site_off;   // per circuit: float2 offset of site 0
  const int* cap;            // per circuit: chi_max
  int* bonds;                // bond dims, bond_off[c] + i, i = 0..n
  const int* bond_off;
  const int* task_circ;
  const int* task_site;
  const double2* task_gate;  // 16 per task, column-major
  int task_begin, task_end;
  int* counter;
  float2* slab;              // per CTA: 2 * slab_elems
  int slab_elems;
  double cutoff;
  double floor_rel;
  float tol;
  int max_sweeps;
  int* task_rank;
  int* task_sweeps;
  float* task_discarded;
};

__device__ inline void tourney(int r, int q, int n, int& a, int& b) {
  if (q == 0) { a = r % (n - 1); b = n - 1; }
  else { a = (r + q) % (n - 1); b = (r - q + (n - 1)) % (n - 1); }
}

__device__ inline float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(BT) batch_layer_kernel(BatchArgs p) {
  __shared__ int s_task, s_rot, s_k;
  __shared__ float2 g[16];
  __shared__ double s_sig[MAXN];
  __shared__ int s_perm[MAXN];
  __shared__ double s_red[BWARPS];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float2* X = p.slab + (size_t)blockIdx.x * 2 * p.slab_elems;
  float2* T = X + p.slab_elems;

  for (;;) {
    if (tid == 0) s_task = p.task_begin + atomicAdd(p.counter, 1);
    __syncthreads();
    const int task = s_task;
    if (task >= p.task_end) break;
    const int c = p.task_circ[task], w = p.task_site[task];
    int* bond = p.bonds + p.bond_off[c];
    const int chil = bond[w], chim = bond[w + 1], chir = bond[w + 2];
    const int cap = p.cap[c];
    const size_t slot = (size_t)cap * 2 * cap;
    float2* A = p.sites + p.site_off[c] + (size_t)w * slot;
    float2* B = A + slot;
    const int m = 2 * chil, n = 2 * chir;
    if (tid < 16) {
      const double2 v = p.task_gate[(size_t)task * 16 + tid];
      g[tid] = make_float2((float)v.x, (float)v.y);
    }
    __syncthreads();

    // 1. theta' = G (A B), one thread per (a, b) owning the four physical values
    for (int idx = tid; idx < chil * chir; idx += BT) {
      const int a = idx % chil, b = idx / chil;
      float2 acc[4] = {make_float2(0, 0), make_float2(0, 0), make_float2(0, 0), make_float2(0, 0)};
      for (int k = 0; k < chim; k++) {
        const float2 a0 = A[a + chil * (2 * k)], a1 = A[a + chil * (2 * k + 1)];
        const float2 b0 = B[k + chim * (2 * b)], b1 = B[k + chim * (2 * b + 1)];
        cfma(acc[0], a0, b0);
        cfma(acc[1], a1, b0);
        cfma(acc[2], a0, b1);
        cfma(acc[3], a1, b1);
      }
#pragma unroll
      for (int o = 0; o < 4; o++) {
        float2 v = make_float2(0, 0);
#pragma unroll
        for (int q = 0; q < 4; q++) cfma(v, g[o + 4 * q], acc[q]);
        const int r = a + chil * (o & 1), col = (o >> 1) + 2 * b;
        X[r + m * col] = v;
        T[r + m * col] = v;
      }
    }
    __syncthreads();

    // ||theta'||_F^2 in FP64 (sets the rounding floor)
    double part = 0;
    for (int i = tid; i < m * n; i += BT) part += (double)X[i].x * X[i].x + (double)X[i].y * X[i].y;
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) s_red[warp] = part;
    __syncthreads();
    double fro2 = 0;
    for (int i = 0; i < BWARPS; i++) fro2 += s_red[i];
    const double nu = 4.0 * sqrt((double)max(m, 16)) * 5.96e-8;
    const float nu2 = (float)(nu * nu * fro2);

    // 2. one-sided Jacobi on the n columns of X (m rows)
    int sweeps = 0;
    if (n > 1) {
      for (int sweep = 0; sweep < p.max_sweeps; sweep++) {
        __syncthreads();  // every thread has read s_rot of the previous sweep
        if (tid == 0) s_rot = 0;
        __syncthreads();
        for (int r = 0; r < n - 1; r++) {
          for (int q = warp; q < n / 2; q += BWARPS) {
            int pc, qc;
            tourney(r, q, n, pc, qc);
            float2* xp = X + (size_t)m * pc;
            float2* xq = X + (size_t)m * qc;
            float aa = 0, bb = 0, gr = 0, gi = 0;
            for (int i = lane; i < m; i += 32) {
              const float2 u = xp[i], v = xq[i];
              aa = fmaf(u.x, u.x, fmaf(u.y, u.y, aa));
              bb = fmaf(v.x, v.x, fmaf(v.y, v.y, bb));
              gr = fmaf(u.x, v.x, fmaf(u.y, v.y, gr));
              gi = fmaf(u.x, v.y, fmaf(-u.y, v.x, gi));
            }
            aa = warp_sum(aa);
            bb = warp_sum(bb);
            gr = warp_sum(gr);
            gi = warp_sum(gi);
            const double ag = sqrt((double)gr * gr + (double)gi * gi);
            if (aa > nu2 && bb > nu2 && ag > (double)p.tol * sqrt((double)aa * bb)) {
              const double zeta = ((double)bb - aa) / (2.0 * ag);
              const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
              const double cs = 1.0 / sqrt(1.0 + t * t);
              const float c = (float)cs, s = (float)(cs * t);
              const float er = (float)(gr / ag), ei = (float)(gi / ag);
              for (int i = lane; i < m; i += 32) {
                const float2 u = xp[i], v = xq[i];
                // x_p' = c x_p - s e^{-i phi} x_q ;  x_q' = s e^{i phi} x_p + c x_q
                xp[i] = make_float2(c * u.x - s * (er * v.x + ei * v.y), c * u.y - s * (er * v.y - ei * v.x));
                xq[i] = make_float2(s * (er * u.x - ei * u.y) + c * v.x, s * (er * u.y + ei * u.x) + c * v.y);
              }
              if (lane == 0) s_rot = 1;
            }
          }
          __syncthreads();
        }
        sweeps = sweep + 1;
        const int again = s_rot;  // read after the round's closing barrier
        if (!again) break;
      }
    }

    // 3. singular values (FP64 norms), sorted descending
    int np2 = 1;
    while (np2 < n) np2 <<= 1;
    for (int j = tid; j < np2; j += BT) {
      double s = -1.0;
      if (j < n) {
        s = 0;
        for (int i = 0; i < m; i++) {
          const float2 v = X[i + (size_t)m * j];
          s += (double)v.x * v.x + (double)v.y * v.y;
        }
        s = sqrt(s);
      }
      s_sig[j] = s;
      s_perm[j] = j;
    }
    __syncthreads();
    for (int k2 = 2; k2 <= np2; k2 <<= 1)
      for (int j2 = k2 >> 1; j2 > 0; j2 >>= 1) {
        for (int i = tid; i < np2; i += BT) {
          const int l = i ^ j2;
          if (l > i) {
            const bool desc = ((i & k2) == 0);
            const double x = s_sig[i], y = s_sig[l];
            const bool sw = desc ? (x < y || (x == y && s_perm[i] > s_perm[l]))
                                 : (x > y || (x == y && s_perm[i] < s_perm[l]));
            if (sw) {
              s_sig[i] = y; s_sig[l] = x;
              const int tp = s_perm[i]; s_perm[i] = s_perm[l]; s_perm[l] = tp;
            }
          }
        }
        __syncthreads();
      }

    // 4. the tail rule (sequential, from the smallest value), then the cap
    if (tid == 0) {
      const double eff = fmax(p.cutoff, p.floor_rel * sqrt(fro2));
      double acc = 0;
      int k = 1;
      for (int i = n - 1; i >= 0; i--) {
        acc += s_sig[i] * s_sig[i];
        if (sqrt(acc) > eff) { k = i + 1; break; }
      }
      k = min(k, min(cap, min(m, n)));
      double disc = 0;
      for (int i = k; i < n; i++) disc += s_sig[i] * s_sig[i];
      s_k = k;
      p.task_rank[task] = k;
      p.task_sweeps[task] = sweeps;
      p.task_discarded[task] = (float)disc;
    }
    __syncthreads();
    const int k = s_k;

    // 5. A' (chil, 2, k) = unit columns, into site slot w
    for (int idx = tid; idx < m * k; idx += BT) {
      const int r = idx % m, j = idx / m;
      const double s = s_sig[j];
      const float inv = s > 0 ? (float)(1.0 / s) : 0.f;
      const float2 v = X[r + (size_t)m * s_perm[j]];
      A[r + (size_t)m * j] = make_float2(v.x * inv, v.y * inv);
    }
    __syncthreads();
    // 6. B' (k, 2, chir) = A'^H theta', into site slot w+1
    for (int idx = tid; idx < k * n; idx += BT) {
      const int j = idx % k, col = idx / k;
      float2 acc = make_float2(0, 0);
      for (int r = 0; r < m; r++) cfma_conj(acc, A[r + (size_t)m * j], T[r + (size_t)m * col]);
      B[j + (size_t)k * col] = acc;
    }
    if (tid == 0) bond[w + 1] = k;
    __syncthreads();
  }
}

// <Z_site> per circuit: a left-to-right transfer sweep in FP32 with the
// environment in a per-CTA slab; one CTA per circuit (grid-stride).
__global__ void __launch_bounds__(BT)
batch_expect_kernel(const float2* sites, const int64_t* site_off, const int* cap, const int* nsites, const int* bonds,
                    const int* bond_off, int ncirc, int site, float2* slab, int slab_elems, double* out) {
  float2* E = slab + (size_t)blockIdx.x * 3 * slab_elems;
  float2* E2 = E + slab_elems;
  float2* Tm = E2 + slab_elems;
  __shared__ double s_red[BWARPS];
  for (int c = blockIdx.x; c < ncirc; c += gridDim.x) {
    const int n = nsites[c];
    const int* bd = bonds + bond_off[c];
    const size_t slot = (size_t)cap[c] * 2 * cap[c];
    double res[2];
    for (int pass = 0; pass < 2; pass++) {  // pass 0: <psi|psi>, pass 1: <psi|Z|psi>
      const int c0 = bd[0];
      for (int i = threadIdx.x; i < c0 * c0; i += BT) E[i] = make_float2((i % c0) == (i / c0) ? 1.f : 0.f, 0.f);
      __syncthreads();
      for (int st = 0; st < n; st++) {
        const float2* Aq = sites + site_off[c] + (size_t)st * slot;
        const int cl = bd[st], cr = bd[st + 1];
        for (int i = threadIdx.x; i < cr * cr; i += BT) E2[i] = make_float2(0, 0);
        __syncthreads();
        for (int s = 0; s < 2; s++) {
          const float wgt = (pass == 1 && st == site && s == 1) ? -1.f : 1.f;
          // Tm (cl x cr) = E (cl x cl) A_s
          for (int idx = threadIdx.x; idx < cl * cr; idx += BT) {
            const int i = idx % cl, j = idx / cl;
            float2 acc = make_float2(0, 0);
            for (int q = 0; q < cl; q++) cfma(acc, E[i + cl * q], Aq[q + cl * (s + 2 * j)]);
            Tm[idx] = acc;
          }
          __syncthreads();
          // E2 (cr x cr) += w A_s^H Tm
          for (int idx = threadIdx.x; idx < cr * cr; idx += BT) {
            const int i = idx % cr, j = idx / cr;
            float2 acc = make_float2(0, 0);
            for (int q = 0; q < cl; q++) cfma_conj(acc, Aq[q + cl * (s + 2 * i)], Tm[q + cl * j]);
            E2[idx].x += wgt * acc.x;
            E2[idx].y += wgt * acc.y;
          }
          __syncthreads();
        }
        for (int i = threadIdx.x; i < cr * cr; i += BT) E[i] = E2[i];
        __syncthreads();
      }
      const int cn = bd[n];
      double tr = 0;
      for (int i = threadIdx.x; i < cn; i += BT) tr += E[i + cn * i].x;
      for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
      if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = tr;
      __syncthreads();
      double tot = 0;
      for (int i = 0; i < BWARPS; i++) tot += s_red[i];
      res[pass] = tot;
      __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = res[1] / res[0];
    __syncthreads();
  }
}

__global__ void batch_init_kernel(float2* sites, const int64_t* site_off, const int* cap, const int* nsites, int ncirc) {
  for (int c = blockIdx.x; c < ncirc; c += gridDim.x) {
    const size_t slot = (size_t)cap[c] * 2 * cap[c];
    for (int i = threadIdx.x; i < nsites[c]; i += blockDim.x) {
      float2* s = sites + site_off[c] + (size_t)i * slot;
      s[0] = make_float2(1.f, 0.f);  // (1,2,1): |0>
      s[1] = make_float2(0.f, 0.f);
    }
  }
}

}  // namespace

struct qt_batch {
  int ncirc = 0, capmax = 0;
  std::vector<int> nsites, cap;
  std::vector<int64_t> site_off;
  std::vector<int> bond_off;
  float2* d_sites = nullptr;
  int64_t* d_site_off = nullptr;
  int *d_cap = nullptr, *d_nsites = nullptr, *d_bonds = nullptr, *d_bond_off = nullptr;
  float2* d_slab = nullptr;
  int ctas = 0, slab_elems = 0;
  int* d_counter = nullptr;  // one counter per layer
  int counter_cap = 0;
  // the last program (device copies) and its captured graph
  int* d_tc = nullptr;
  int* d_ts = nullptr;
  double2* d_tg = nullptr;
  int* d_rank = nullptr;
  int* d_sweeps = nullptr;
  float* d_disc = nullptr;
  int ntask_cap = 0;
  cudaGraphExec_t graph = nullptr;
};

static void batch_free_program(qt_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  cudaFree(b->d_tc); cudaFree(b->d_ts); cudaFree(b->d_tg);
  cudaFree(b->d_rank); cudaFree(b->d_sweeps); cudaFree(b->d_disc);
  b->d_tc = b->d_ts = nullptr; b->d_tg = nullptr; b->d_rank = b->d_sweeps = nullptr; b->d_disc = nullptr;
  b->ntask_cap = 0;
}

extern "C" int qt_batch_create(qt_handle* h, int ncirc, const int* nqubits, const int* chi_max, qt_batch** out) {
  if (!h || !nqubits || !chi_max || !out || ncirc < 1) return qt_fail(h, QT_EINVAL, "batch_create: bad argument");
  *out = nullptr;
  cudaSetDevice(h->device);
  qt_batch* b = new qt_batch();
  b->ncirc = ncirc;
  int64_t off = 0;
  int boff = 0;
  for (int c = 0; c < ncirc; c++) {
    if (nqubits[c] < 2 || chi_max[c] < 1 || chi_max[c] > MAXN / 2) {
      delete b;
      return qt_fail(h, QT_ENOTSUP, "batch_create: needs >= 2 qubits and 1 <= chi_max <= 128");
    }
    b->nsites.push_back(nqubits[c]);
    b->cap.push_back(chi_max[c]);
    b->site_off.push_back(off);
    b->bond_off.push_back(boff);
    off += (int64_t)nqubits[c] * chi_max[c] * 2 * chi_max[c];
    boff += nqubits[c] + 1;
    b->capmax = std::max(b->capmax, chi_max[c]);
  }
  int dev_sms = 152;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, h->device);
  b->ctas = dev_sms;
  b->slab_elems = (2 * b->capmax) * (2 * b->capmax);
  std::vector<int> bonds(boff, 1);
  bool ok = cudaMalloc(&b->d_sites, sizeof(float2) * off) == cudaSuccess &&
            cudaMalloc(&b->d_site_off, sizeof(int64_t) * ncirc) == cudaSuccess &&
            cudaMalloc(&b->d_cap, sizeof(int) * ncirc) == cudaSuccess &&
            cudaMalloc(&b->d_nsites, sizeof(int) * ncirc) == cudaSuccess &&
            cudaMalloc(&b->d_bonds, sizeof(int) * boff) == cudaSuccess &&
            cudaMalloc(&b->d_bond_off, sizeof(int) * ncirc) == cudaSuccess &&
            cudaMalloc(&b->d_slab, sizeof(float2) * 3 * (size_t)b->slab_elems * b->ctas) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    qt_batch_free(h, b);
    return qt_fail(h, QT_ENOMEM, "batch_create: device allocation failed");
  }
  cudaMemcpy(b->d_site_off, b->site_off.data(), sizeof(int64_t) * ncirc, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_cap, b->cap.data(), sizeof(int) * ncirc, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_nsites, b->nsites.data(), sizeof(int) * ncirc, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_bonds, bonds.data(), sizeof(int) * boff, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_bond_off, b->bond_off.data(), sizeof(int) * ncirc, cudaMemcpyHostToDevice);
  batch_init_kernel<<<std::min(ncirc, 1024), 128, 0, h->stream>>>(b->d_sites, b->d_site_off, b->d_cap, b->d_nsites,
                                                                    ncirc);
  h->launches++;
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  *out = b;
  return QT_OK;
}

extern "C" int qt_batch_free(qt_handle* h, qt_batch* b) {
  if (!b) return QT_OK;
  if (h) {
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
  }
  batch_free_program(b);
  cudaFree(b->d_sites); cudaFree(b->d_site_off); cudaFree(b->d_cap); cudaFree(b->d_nsites);
  cudaFree(b->d_bonds); cudaFree(b->d_bond_off); cudaFree(b->d_slab); cudaFree(b->d_counter);
  delete b;
  return QT_OK;
}

// Run a whole program: layers [layer_start[l], layer_start[l+1]) of tasks
// (circuit, site 0-based, gate); tasks of one layer must touch disjoint
// sites.  With use_graph the launch sequence is captured once and replayed.
extern "C" int qt_batch_run(qt_handle* h, qt_batch* b, int nlayers, const int* layer_start, const int* circ,
                            const int* site, const double* gates, double cutoff, int use_graph) {
  if (!h || !b || nlayers < 0 || !layer_start) return qt_fail(h, QT_EINVAL, "batch_run: bad argument");
  if (!(cutoff >= 0)) return qt_fail(h, QT_EINVAL_ERR_NEG, "Error must be positive");
  cudaSetDevice(h->device);
  const int ntask = layer_start[nlayers];
  for (int t = 0; t < ntask; t++) {
    if (circ[t] < 0 || circ[t] >= b->ncirc || site[t] < 0 || site[t] + 1 >= b->nsites[circ[t]])
      return qt_fail(h, QT_EBOUNDS, "batch_run: task site out of range");
  }
  batch_free_program(b);
  if (ntask > 0) {
    bool ok = cudaMalloc(&b->d_tc, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_ts, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_tg, sizeof(double2) * 16 * (size_t)ntask) == cudaSuccess &&
              cudaMalloc(&b->d_rank, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_sweeps, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_disc, sizeof(float) * ntask) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      return qt_fail(h, QT_ENOMEM, "batch_run: device allocation failed");
    }
    b->ntask_cap = ntask;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(b->d_tc, circ, sizeof(int) * ntask, cudaMemcpyHostToDevice, h->stream));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(b->d_ts, site, sizeof(int) * ntask, cudaMemcpyHostToDevice, h->stream));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(b->d_tg, gates, sizeof(double2) * 16 * ntask, cudaMemcpyHostToDevice, h->stream));
  }
  if (b->counter_cap < nlayers) {
    cudaFree(b->d_counter);
    if (cudaMalloc(&b->d_counter, sizeof(int) * std::max(nlayers, 1)) != cudaSuccess)
      return qt_fail(h, QT_ENOMEM, "batch_run: counter allocation failed");
    b->counter_cap = nlayers;
  }
  BatchArgs a;
  a.sites = b->d_sites; a.site_off = b->d_site_off; a.cap = b->d_cap; a.bonds = b->d_bonds;
  a.bond_off = b->d_bond_off; a.task_circ = b->d_tc; a.task_site = b->d_ts; a.task_gate = b->d_tg;
  a.slab = b->d_slab; a.slab_elems = b->slab_elems; a.cutoff = cutoff;
  a.floor_rel = h->cfg.noise_floor > 0 ? h->cfg.noise_floor : 4.0 * std::sqrt(2.0 * b->capmax) * 5.96e-8;
  a.tol = (float)(16.0 * std::sqrt(2.0 * b->capmax) * 5.96e-8);
  a.max_sweeps = std::max(4, h->cfg.max_sweeps);
  a.task_rank = b->d_rank; a.task_sweeps = b->d_sweeps; a.task_discarded = b->d_disc;
  auto launch_all = [&]() -> int {
    QT_CHECK_CUDA(h, cudaMemsetAsync(b->d_counter, 0, sizeof(int) * std::max(nlayers, 1), h->stream));
    for (int l = 0; l < nlayers; l++) {
      if (layer_start[l + 1] <= layer_start[l]) continue;
      BatchArgs al = a;
      al.task_begin = layer_start[l];
      al.task_end = layer_start[l + 1];
      al.counter = b->d_counter + l;
      const int grid = std::min(b->ctas, layer_start[l + 1] - layer_start[l]);
      QT_LAUNCH(h, batch_layer_kernel, grid, BT, 0, al);
    }
    return QT_OK;
  };
  if (use_graph) {
    cudaGraph_t g;
    QT_CHECK_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = launch_all();
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc != QT_OK) return rc;
    if (e != cudaSuccess) return qt_fail(h, QT_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return qt_fail(h, QT_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    QT_CHECK_CUDA(h, cudaGraphLaunch(b->graph, h->stream));
  } else {
    QT_TRY(launch_all());
  }
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

// Replay the last captured program (fresh state needs qt_batch_reset first).
extern "C" int qt_batch_replay(qt_handle* h, qt_batch* b) {
  if (!h || !b || !b->graph) return qt_fail(h, QT_EINVAL, "batch_replay: no captured program");
  cudaSetDevice(h->device);
  QT_CHECK_CUDA(h, cudaGraphLaunch(b->graph, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

// Back to |0...0> on every circuit.
extern "C" int qt_batch_reset(qt_handle* h, qt_batch* b) {
  if (!h || !b) return qt_fail(h, QT_EINVAL, "batch_reset: bad argument");
  cudaSetDevice(h->device);
  std::vector<int> bonds(b->bond_off.back() + b->nsites.back() + 1, 1);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(b->d_bonds, bonds.data(), sizeof(int) * bonds.size(), cudaMemcpyHostToDevice,
                                   h->stream));
  QT_LAUNCH(h, batch_init_kernel, std::min(b->ncirc, 1024), 128, 0, b->d_sites, b->d_site_off, b->d_cap, b->d_nsites,
            b->ncirc);
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

extern "C" int qt_batch_task_stats(qt_handle* h, const qt_batch* b, int* rank, int* sweeps, float* discarded) {
  if (!h || !b) return qt_fail(h, QT_EINVAL, "batch_task_stats: bad argument");
  const int n = b->ntask_cap;
  if (n == 0) return QT_OK;
  if (rank) QT_CHECK_CUDA(h, cudaMemcpy(rank, b->d_rank, sizeof(int) * n, cudaMemcpyDeviceToHost));
  if (sweeps) QT_CHECK_CUDA(h, cudaMemcpy(sweeps, b->d_sweeps, sizeof(int) * n, cudaMemcpyDeviceToHost));
  if (discarded) QT_CHECK_CUDA(h, cudaMemcpy(discarded, b->d_disc, sizeof(float) * n, cudaMemcpyDeviceToHost));
  return QT_OK;
}

extern "C" int qt_batch_bond_dims(qt_handle* h, const qt_batch* b, int c, int* dims) {
  if (!h || !b || !dims || c < 0 || c >= b->ncirc) return qt_fail(h, QT_EINVAL, "batch_bond_dims: bad argument");
  QT_CHECK_CUDA(h, cudaMemcpy(dims, b->d_bonds + b->bond_off[c], sizeof(int) * (b->nsites[c] + 1),
                              cudaMemcpyDeviceToHost));
  return QT_OK;
}

// Site (0-based) of circuit c as a compact (chiL, 2, chiR) complex64 array.
extern "C" int qt_batch_download_site(qt_handle* h, const qt_batch* b, int c, int s, void* host) {
  if (!h || !b || !host || c < 0 || c >= b->ncirc || s < 0 || s >= b->nsites[c])
    return qt_fail(h, QT_EINVAL, "batch_download_site: bad argument");
  int d[2];
  QT_CHECK_CUDA(h, cudaMemcpy(d, b->d_bonds + b->bond_off[c] + s, sizeof(int) * 2, cudaMemcpyDeviceToHost));
  const size_t slot = (size_t)b->cap[c] * 2 * b->cap[c];
  QT_CHECK_CUDA(h, cudaMemcpy(host, b->d_sites + b->site_off[c] + (size_t)s * slot, sizeof(float2) * d[0] * 2 * d[1],
                              cudaMemcpyDeviceToHost));
  return QT_OK;
}

extern "C" int qt_batch_expect_z(qt_handle* h, qt_batch* b, int site, double* out) {
  if (!h || !b || !out) return qt_fail(h, QT_EINVAL, "batch_expect_z: bad argument");
  for (int c = 0; c < b->ncirc; c++)
    if (site < 0 || site >= b->nsites[c]) return qt_fail(h, QT_EBOUNDS, "batch_expect_z: site out of range");
  cudaSetDevice(h->device);
  double* d_out;
  QT_CHECK_CUDA(h, cudaMalloc(&d_out, sizeof(double) * b->ncirc));
  const int grid = std::min(b->ncirc, b->ctas);
  // the slab holds 2 * slab_elems per CTA for the update; the sweep needs 3 (cap^2 each fits in one)
  batch_expect_kernel<<<grid, BT, 0, h->stream>>>(b->d_sites, b->d_site_off, b->d_cap, b->d_nsites, b->d_bonds,
                                                   b->d_bond_off, b->ncirc, site, b->d_slab, b->slab_elems / 4 + 1,
                                                   d_out);
  h->launches++;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, sizeof(double) * b->ncirc, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d_out);
  if (e != cudaSuccess) return qt_fail(h, QT_ECUDA, std::string("batch_expect_z: ") + cudaGetErrorString(e));
  return QT_OK;
}
