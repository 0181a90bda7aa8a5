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
//   sigma_j = ||x_j||           FP64, bitonic sort, tail rule (FP64, sequential) at
//                               the caller's cutoff, cap; a decision below the FP32
//                               resolution without a certificate (cap or exact rank
//                               bound) is redone as an FP64 split in the same CTA
//   A' = x_perm(j) / sigma_j    written into site slot w
//   B' = A'^H theta'            written into site slot w+1 (no V accumulation)
//   bonds[w+1] = k
// Tasks of one brickwork layer touch disjoint sites, so CTAs never race.  A
// whole program (every layer) is a fixed sequence of (counter reset, kernel)
// pairs that the host captures once in a CUDA graph.  There are no waits on
// other CTAs: a CTA stops when the counter passes the task count.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "qt_internal.cuh"
#include "qt_rank_model.h"

namespace {

constexpr int BT = 256;            // threads per CTA
constexpr int BWARPS = BT / 32;
constexpr int MAXN = 256;          // largest 2 * cap handled (cap <= 128)

struct BatchArgs {
  float2* sites;
  const int64_t* site_off;   // per circuit: float2 offset of site 0
  const int* cap;            // per circuit: chi_max
  const int* nsites;         // per circuit: qubits
  int* bonds;                // bond dims, bond_off[c] + i, i = 0..n
  const int* bond_off;
  const int* task_circ;
  const int* task_site;
  const double2* task_gate;  // 16 per task, column-major
  const int* task_grank;     // per task: the gate's operator-Schmidt rank
  int task_begin, task_end;
  int* counter;
  float2* slab;              // per CTA: 4 * slab_elems float2 (FP32 X, T; or the FP64 X, T of a fallback)
  int slab_elems;
  double cutoff;
  double floor_rel;          // FP32 resolution relative to ||theta'||_F (<= 0: 4 sqrt(max(m, n)) u)
  float tol;                 // FP32 Jacobi tolerance (relative off-diagonal)
  int max_sweeps;
  int* task_rank;
  int* task_sweeps;
  float* task_discarded;
  int* task_cert;            // QT_CERT_* of the rank decision (QT_CERT_NONE: the FP64 split decided)
};

__device__ inline void tourney(int r, int q, int n, int& a, int& b) {
  if (q == 0) { a = r % (n - 1); b = n - 1; }
  else { a = (r + q) % (n - 1); b = (r - q + (n - 1)) % (n - 1); }
}

template <typename R>
__device__ inline R warp_sum(R v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// theta' = G (A B) into X and T (m x n, ld m), one thread per (a, b) owning
// the four physical values; C = float2 (FP32 products) or double2 (FP64).
template <int NT, typename C>
__device__ void form_theta(const float2* A, const float2* B, int chil, int chim, int chir, const C* g, C* X, C* T) {
  const int m = 2 * chil;
  for (int idx = threadIdx.x; idx < chil * chir; idx += NT) {
    const int a = idx % chil, b = idx / chil;
    C acc[4] = {czero<C>(), czero<C>(), czero<C>(), czero<C>()};
    for (int k = 0; k < chim; k++) {
      const C a0 = ccast<C>(A[a + chil * (2 * k)]), a1 = ccast<C>(A[a + chil * (2 * k + 1)]);
      const C b0 = ccast<C>(B[k + chim * (2 * b)]), b1 = ccast<C>(B[k + chim * (2 * b + 1)]);
      cfma(acc[0], a0, b0);
      cfma(acc[1], a1, b0);
      cfma(acc[2], a0, b1);
      cfma(acc[3], a1, b1);
    }
#pragma unroll
    for (int o = 0; o < 4; o++) {
      C v = czero<C>();
#pragma unroll
      for (int q = 0; q < 4; q++) cfma(v, g[o + 4 * q], acc[q]);
      const int r = a + chil * (o & 1), col = (o >> 1) + 2 * b;
      X[r + m * col] = v;
      T[r + m * col] = v;
    }
  }
}

// ||X||_F^2 in FP64 over the CTA.
template <int NT, typename C>
__device__ double fro2_of(const C* X, int cnt, double* s_red) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double part = 0;
  for (int i = threadIdx.x; i < cnt; i += NT) part += (double)X[i].x * X[i].x + (double)X[i].y * X[i].y;
  part = warp_sum(part);
  __syncthreads();
  if (lane == 0) s_red[warp] = part;
  __syncthreads();
  double fro2 = 0;
  for (int i = 0; i < NT / 32; i++) fro2 += s_red[i];
  return fro2;
}

// One-sided Jacobi on the n columns of X (m rows): warps on disjoint column
// pairs of a round-robin round, rotation angles in FP64.  Columns with
// |x|^2 <= nu2 are frozen.  Returns the sweeps run.
template <int NT, typename C>
__device__ int jacobi_columns(C* X, int m, int n, double tol, double nu2, int max_sweeps, int* s_rot) {
  typedef typename real_of<C>::type R;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int sweeps = 0;
  if (n < 2) return 0;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    __syncthreads();  // every thread has read s_rot of the previous sweep
    if (threadIdx.x == 0) *s_rot = 0;
    __syncthreads();
    for (int r = 0; r < n - 1; r++) {
      for (int q = warp; q < n / 2; q += NT / 32) {
        int pc, qc;
        tourney(r, q, n, pc, qc);
        C* xp = X + (size_t)m * pc;
        C* xq = X + (size_t)m * qc;
        R aa = 0, bb = 0, gr = 0, gi = 0;
        for (int i = lane; i < m; i += 32) {
          const C u = xp[i], v = xq[i];
          aa = fma(u.x, u.x, fma(u.y, u.y, aa));
          bb = fma(v.x, v.x, fma(v.y, v.y, bb));
          gr = fma(u.x, v.x, fma(u.y, v.y, gr));
          gi = fma(u.x, v.y, fma(-u.y, v.x, gi));
        }
        aa = warp_sum(aa);
        bb = warp_sum(bb);
        gr = warp_sum(gr);
        gi = warp_sum(gi);
        const double ag = sqrt((double)gr * gr + (double)gi * gi);
        if ((double)aa > nu2 && (double)bb > nu2 && ag > tol * sqrt((double)aa * bb)) {
          const double zeta = ((double)bb - aa) / (2.0 * ag);
          const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          const double cs = 1.0 / sqrt(1.0 + t * t);
          const R c = (R)cs, s = (R)(cs * t);
          const R er = (R)(gr / ag), ei = (R)(gi / ag);
          for (int i = lane; i < m; i += 32) {
            const C u = xp[i], v = xq[i];
            // x_p' = c x_p - s e^{-i phi} x_q ;  x_q' = s e^{i phi} x_p + c x_q
            xp[i] = mk(c * u.x - s * (er * v.x + ei * v.y), c * u.y - s * (er * v.y - ei * v.x));
            xq[i] = mk(s * (er * u.x - ei * u.y) + c * v.x, s * (er * u.y + ei * u.x) + c * v.y);
          }
          if (lane == 0) *s_rot = 1;
        }
      }
      __syncthreads();
    }
    sweeps = sweep + 1;
    const int again = *s_rot;  // read after the round's closing barrier
    if (!again) break;
  }
  return sweeps;
}

// Column norms of X in FP64, sorted descending into s_sig / s_perm (bitonic).
template <int NT, typename C>
__device__ void sorted_norms(const C* X, int m, int n, double* s_sig, int* s_perm) {
  int np2 = 1;
  while (np2 < n) np2 <<= 1;
  for (int j = threadIdx.x; j < np2; j += NT) {
    double s = -1.0;
    if (j < n) {
      s = 0;
      for (int i = 0; i < m; i++) {
        const C v = X[i + (size_t)m * j];
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
      for (int i = threadIdx.x; i < np2; i += NT) {
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
}

// The tail rule of src/svd.jl:29-33 (sequential from the smallest value,
// strict >, k >= 1) on the n sorted values.
__device__ int tail_rule(const double* s, int n, double cutoff) {
  double acc = 0;
  for (int i = n - 1; i >= 0; i--) {
    acc += s[i] * s[i];
    if (sqrt(acc) > cutoff) return i + 1;
  }
  return 1;
}

template <int NT>
__global__ void __launch_bounds__(NT) batch_layer_kernel(BatchArgs p) {
  __shared__ int s_task, s_rot, s_k, s_fb;
  __shared__ float2 g[16];
  __shared__ double2 g64[16];
  __shared__ double s_sig[MAXN];
  __shared__ int s_perm[MAXN];
  __shared__ double s_red[NT / 32];
  const int tid = threadIdx.x;
  float2* X = p.slab + (size_t)blockIdx.x * 4 * p.slab_elems;
  float2* T = X + p.slab_elems;

  for (;;) {
    if (tid == 0) s_task = p.task_begin + atomicAdd(p.counter, 1);
    __syncthreads();
    const int task = s_task;
    if (task >= p.task_end) break;
    const int c = p.task_circ[task], w = p.task_site[task];
    int* bond = p.bonds + p.bond_off[c];
    const int chil = bond[w], chim = bond[w + 1], chir = bond[w + 2];
    const int cap = p.cap[c], nq = p.nsites[c];
    const size_t slot = (size_t)cap * 2 * cap;
    float2* A = p.sites + p.site_off[c] + (size_t)w * slot;
    float2* B = A + slot;
    const int m = 2 * chil, n = 2 * chir;
    if (tid < 16) {
      const double2 v = p.task_gate[(size_t)task * 16 + tid];
      g[tid] = make_float2((float)v.x, (float)v.y);
      g64[tid] = v;
    }
    __syncthreads();

    // 1. theta' = G (A B) in FP32
    form_theta<NT, float2>(A, B, chil, chim, chir, g, X, T);
    __syncthreads();
    const double fro2 = fro2_of<NT>(X, m * n, s_red);
    const double nu = 4.0 * sqrt((double)max(m, 16)) * 5.96e-8;

    // 2. one-sided Jacobi on the columns of X, 3. sorted FP64 norms
    int sweeps = jacobi_columns<NT, float2>(X, m, n, (double)p.tol, nu * nu * fro2, p.max_sweeps, &s_rot);
    sorted_norms<NT, float2>(X, m, n, s_sig, s_perm);

    // 4. the tail rule at the caller's cutoff, then the cap.  Below the FP32
    // resolution eta the decision needs a certificate: the cap binding with
    // margin, or exactly as many values above eta as the exact rank bound
    // allows (the gate's operator-Schmidt rank times the inner bond, the
    // Hilbert-space dimensions of the two sides).  Otherwise the FP64 split
    // below decides.
    const int kcap = min(cap, min(m, n));
    if (tid == 0) {
      const double eta = (p.floor_rel > 0 ? p.floor_rel : 4.0 * sqrt((double)max(m, n)) * 5.96e-8) * sqrt(fro2);
      int kc = tail_rule(s_sig, n, p.cutoff);
      int cert = QT_CERT_NONE;
      if (p.cutoff >= eta) {
        cert = QT_CERT_RESOLVED;
      } else if (cap < min(m, n) && kc > cap) {
        double t2 = 0;
        for (int i = n - 1; i >= cap; i--) t2 += s_sig[i] * s_sig[i];
        if (sqrt(t2) > p.cutoff + eta) cert = QT_CERT_CAP;
      }
      if (cert == QT_CERT_NONE) {
        int srank = min(min(m, n), p.task_grank[task] * chim);
        if (w + 1 < 30) srank = min(srank, 1 << (w + 1));
        if (nq - w - 1 < 30) srank = min(srank, 1 << (nq - w - 1));
        int kr = 0;
        while (kr < n && s_sig[kr] > eta) kr++;
        if (kr == srank) {
          kc = srank;
          cert = QT_CERT_STRUCT;
        }
      }
      const int k = min(kc, kcap);
      double disc = 0;
      for (int i = k; i < n; i++) disc += s_sig[i] * s_sig[i];
      s_k = k;
      s_fb = cert == QT_CERT_NONE;
      p.task_rank[task] = k;
      p.task_sweeps[task] = sweeps;
      p.task_discarded[task] = (float)disc;
      p.task_cert[task] = cert;
    }
    __syncthreads();

    if (!s_fb) {
      const int k = s_k;
      // 5. A' (chil, 2, k) = unit columns, into site slot w
      for (int idx = tid; idx < m * k; idx += NT) {
        const int r = idx % m, j = idx / m;
        const double s = s_sig[j];
        const float inv = s > 0 ? (float)(1.0 / s) : 0.f;
        const float2 v = X[r + (size_t)m * s_perm[j]];
        A[r + (size_t)m * j] = make_float2(v.x * inv, v.y * inv);
      }
      __syncthreads();
      // 6. B' (k, 2, chir) = A'^H theta', into site slot w+1
      for (int idx = tid; idx < k * n; idx += NT) {
        const int j = idx % k, col = idx / k;
        float2 acc = make_float2(0, 0);
        for (int r = 0; r < m; r++) cfma_conj(acc, A[r + (size_t)m * j], T[r + (size_t)m * col]);
        B[j + (size_t)k * col] = acc;
      }
    } else {
      // The exact FP64 split: theta' from the complex64 sites in FP64, FP64
      // Jacobi (tolerance and freeze at FP64 rounding), the rule at the
      // caller's cutoff; the FP64 X and T take the whole slab.
      double2* X64 = reinterpret_cast<double2*>(X);
      double2* T64 = X64 + p.slab_elems;
      __syncthreads();
      form_theta<NT, double2>(A, B, chil, chim, chir, g64, X64, T64);
      __syncthreads();
      const double f64 = fro2_of<NT>(X64, m * n, s_red);
      const double nu64 = 4.0 * sqrt((double)max(m, 16)) * 1.11e-16;
      sweeps += jacobi_columns<NT, double2>(X64, m, n, 16.0 * sqrt((double)max(m, 16)) * 1.11e-16,
                                            nu64 * nu64 * f64, p.max_sweeps, &s_rot);
      sorted_norms<NT, double2>(X64, m, n, s_sig, s_perm);
      if (tid == 0) {
        const int k = min(tail_rule(s_sig, n, p.cutoff), kcap);
        double disc = 0;
        for (int i = k; i < n; i++) disc += s_sig[i] * s_sig[i];
        s_k = k;
        p.task_rank[task] = k;
        p.task_sweeps[task] = sweeps;
        p.task_discarded[task] = (float)disc;
      }
      __syncthreads();
      const int k = s_k;
      // B' = A'^H theta' from the FP64 columns (before A is overwritten: B
      // reads only X64 and T64), then A' = unit columns
      for (int idx = tid; idx < k * n; idx += NT) {
        const int j = idx % k, col = idx / k;
        const double s = s_sig[j];
        const double inv = s > 0 ? 1.0 / s : 0.0;
        const double2* xj = X64 + (size_t)m * s_perm[j];
        double2 acc = make_double2(0, 0);
        for (int r = 0; r < m; r++) cfma_conj(acc, xj[r], T64[r + (size_t)m * col]);
        B[j + (size_t)k * col] = make_float2((float)(acc.x * inv), (float)(acc.y * inv));
      }
      for (int idx = tid; idx < m * k; idx += NT) {
        const int r = idx % m, j = idx / m;
        const double s = s_sig[j];
        const double inv = s > 0 ? 1.0 / s : 0.0;
        const double2 v = X64[r + (size_t)m * s_perm[j]];
        A[r + (size_t)m * j] = make_float2((float)(v.x * inv), (float)(v.y * inv));
      }
    }
    if (tid == 0) bond[w + 1] = s_k;
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
  int* d_grank = nullptr;
  int* d_cert = nullptr;
  float* d_disc = nullptr;
  int ntask_cap = 0;
  std::vector<int> order;    // device task index -> the caller's task index
  cudaGraphExec_t graph = nullptr;
  // launch shape per bond-cap bucket (caps <= 16, 32, 64, 128): threads per
  // CTA and CTAs per SM of the persistent layer kernel (qt_batch_set_launch)
  int threads[4] = {256, 256, 256, 256};
  int cps[4] = {1, 1, 1, 1};
  int slab_ctas = 0;         // CTAs the slab holds
};

namespace {

int bucket_of(int cap) { return cap <= 16 ? 0 : cap <= 32 ? 1 : cap <= 64 ? 2 : 3; }

}  // namespace

static void batch_free_program(qt_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  cudaFree(b->d_tc); cudaFree(b->d_ts); cudaFree(b->d_tg);
  cudaFree(b->d_rank); cudaFree(b->d_sweeps); cudaFree(b->d_disc); cudaFree(b->d_grank); cudaFree(b->d_cert);
  b->d_tc = b->d_ts = nullptr; b->d_tg = nullptr; b->d_rank = b->d_sweeps = nullptr; b->d_disc = nullptr;
  b->d_grank = b->d_cert = nullptr;
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
            cudaMalloc(&b->d_slab, sizeof(float2) * 4 * (size_t)b->slab_elems * b->ctas) == cudaSuccess;
  b->slab_ctas = b->ctas;
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
  // tasks of each layer grouped by the bucket of their circuit's cap (stable):
  // one launch per (layer, bucket) with that bucket's launch shape
  std::vector<int> order;
  std::vector<int> seg_begin, seg_end, seg_bucket;
  order.reserve(ntask);
  for (int l = 0; l < nlayers; l++) {
    for (int bk = 0; bk < 4; bk++) {
      const int start = (int)order.size();
      for (int t = layer_start[l]; t < layer_start[l + 1]; t++)
        if (bucket_of(b->cap[circ[t]]) == bk) order.push_back(t);
      if ((int)order.size() > start) {
        seg_begin.push_back(start);
        seg_end.push_back((int)order.size());
        seg_bucket.push_back(bk);
      }
    }
  }
  const int nseg = (int)seg_begin.size();
  std::vector<int> oc(ntask), os(ntask);
  std::vector<double> og((size_t)32 * ntask);
  for (int i = 0; i < ntask; i++) {
    oc[i] = circ[order[i]];
    os[i] = site[order[i]];
    std::memcpy(&og[(size_t)32 * i], gates + (size_t)32 * order[i], sizeof(double) * 32);
  }
  b->order = order;
  // the slab holds one 4-unit block per CTA of the widest launch
  const int dev_sms = b->ctas;
  int need = 0;
  for (int bk = 0; bk < 4; bk++) need = std::max(need, dev_sms * b->cps[bk]);
  if (need > b->slab_ctas) {
    cudaFree(b->d_slab);
    b->d_slab = nullptr;
    if (cudaMalloc(&b->d_slab, sizeof(float2) * 4 * (size_t)b->slab_elems * need) != cudaSuccess) {
      cudaGetLastError();
      b->slab_ctas = 0;
      return qt_fail(h, QT_ENOMEM, "batch_run: slab allocation failed");
    }
    b->slab_ctas = need;
  }
  if (ntask > 0) {
    bool ok = cudaMalloc(&b->d_tc, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_ts, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_tg, sizeof(double2) * 16 * (size_t)ntask) == cudaSuccess &&
              cudaMalloc(&b->d_rank, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_sweeps, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_disc, sizeof(float) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_grank, sizeof(int) * ntask) == cudaSuccess &&
              cudaMalloc(&b->d_cert, sizeof(int) * ntask) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      return qt_fail(h, QT_ENOMEM, "batch_run: device allocation failed");
    }
    b->ntask_cap = ntask;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(b->d_tc, oc.data(), sizeof(int) * ntask, cudaMemcpyHostToDevice, h->stream));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(b->d_ts, os.data(), sizeof(int) * ntask, cudaMemcpyHostToDevice, h->stream));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(b->d_tg, og.data(), sizeof(double2) * 16 * ntask, cudaMemcpyHostToDevice,
                                     h->stream));
    std::vector<int> grank(ntask);
    for (int t = 0; t < ntask; t++) grank[t] = qt_gate_schmidt_rank(og.data() + 32 * (size_t)t);
    QT_CHECK_CUDA(h, cudaMemcpyAsync(b->d_grank, grank.data(), sizeof(int) * ntask, cudaMemcpyHostToDevice,
                                     h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  if (b->counter_cap < nseg) {
    cudaFree(b->d_counter);
    if (cudaMalloc(&b->d_counter, sizeof(int) * std::max(nseg, 1)) != cudaSuccess)
      return qt_fail(h, QT_ENOMEM, "batch_run: counter allocation failed");
    b->counter_cap = nseg;
  }
  BatchArgs a;
  a.sites = b->d_sites; a.site_off = b->d_site_off; a.cap = b->d_cap; a.nsites = b->d_nsites; a.bonds = b->d_bonds;
  a.task_grank = b->d_grank; a.task_cert = b->d_cert;
  a.bond_off = b->d_bond_off; a.task_circ = b->d_tc; a.task_site = b->d_ts; a.task_gate = b->d_tg;
  a.slab = b->d_slab; a.slab_elems = b->slab_elems; a.cutoff = cutoff;
  a.floor_rel = h->cfg.noise_floor;  // <= 0: the default resolution of each task's shape
  // FP32 Jacobi tolerance: a pair is rotated while its relative
  // off-diagonal exceeds 16 u (u = 2^-24).  The FP32 Gram of a converged pair
  // is accurate to a few u at these sizes (m <= 256), so the sweeps still end,
  // one or two after a tolerance of 16 sqrt(m) u would; the truncated state,
  // whose error at a cap inside a dense spectrum grows with the tolerance over
  // the gap at the cut, comes out about 10x closer to the exact split's
  // (a simulated FP32 Jacobi on 256 x 256 Haar-circuit bonds: 6.6e-5 -> 6e-6)
  a.tol = (float)(h->cfg.jacobi_tol > 0 ? h->cfg.jacobi_tol : 16.0 * 5.96e-8);
  a.max_sweeps = std::max(4, h->cfg.max_sweeps);
  a.task_rank = b->d_rank; a.task_sweeps = b->d_sweeps; a.task_discarded = b->d_disc;
  auto launch_all = [&]() -> int {
    QT_CHECK_CUDA(h, cudaMemsetAsync(b->d_counter, 0, sizeof(int) * std::max(nseg, 1), h->stream));
    for (int sg = 0; sg < nseg; sg++) {
      const int bk = seg_bucket[sg];
      BatchArgs al = a;
      al.task_begin = seg_begin[sg];
      al.task_end = seg_end[sg];
      al.counter = b->d_counter + sg;
      const int grid = std::min(dev_sms * b->cps[bk], seg_end[sg] - seg_begin[sg]);
      switch (b->threads[bk]) {
        case 128: QT_LAUNCH(h, batch_layer_kernel<128>, grid, 128, 0, al); break;
        case 512: QT_LAUNCH(h, batch_layer_kernel<512>, grid, 512, 0, al); break;
        case 1024: QT_LAUNCH(h, batch_layer_kernel<1024>, grid, 1024, 0, al); break;
        default: QT_LAUNCH(h, batch_layer_kernel<256>, grid, 256, 0, al); break;
      }
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
  // device order -> the caller's task order
  std::vector<int> ri(n), si(n);
  std::vector<float> di(n);
  QT_CHECK_CUDA(h, cudaMemcpy(ri.data(), b->d_rank, sizeof(int) * n, cudaMemcpyDeviceToHost));
  QT_CHECK_CUDA(h, cudaMemcpy(si.data(), b->d_sweeps, sizeof(int) * n, cudaMemcpyDeviceToHost));
  QT_CHECK_CUDA(h, cudaMemcpy(di.data(), b->d_disc, sizeof(float) * n, cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; i++) {
    const int t = b->order[i];
    if (rank) rank[t] = ri[i];
    if (sweeps) sweeps[t] = si[i];
    if (discarded) discarded[t] = di[i];
  }
  return QT_OK;
}

extern "C" int qt_batch_set_launch(qt_handle* h, qt_batch* b, int bucket_cap, int threads, int ctas_per_sm) {
  if (!h || !b) return qt_fail(h, QT_EINVAL, "batch_set_launch: bad argument");
  if (bucket_cap != 16 && bucket_cap != 32 && bucket_cap != 64 && bucket_cap != 128)
    return qt_fail(h, QT_EINVAL, "batch_set_launch: bucket_cap must be 16, 32, 64 or 128");
  if (threads != 128 && threads != 256 && threads != 512 && threads != 1024)
    return qt_fail(h, QT_EINVAL, "batch_set_launch: threads must be 128, 256, 512 or 1024");
  if (ctas_per_sm < 1 || ctas_per_sm > 4) return qt_fail(h, QT_EINVAL, "batch_set_launch: ctas_per_sm must be 1..4");
  const int bk = bucket_of(bucket_cap);
  b->threads[bk] = threads;
  b->cps[bk] = ctas_per_sm;
  return QT_OK;
}

extern "C" int qt_batch_get_launch(const qt_batch* b, int bucket_cap, int* threads, int* ctas_per_sm) {
  if (!b || !threads || !ctas_per_sm) return QT_EINVAL;
  const int bk = bucket_of(bucket_cap);
  *threads = b->threads[bk];
  *ctas_per_sm = b->cps[bk];
  return QT_OK;
}

extern "C" int qt_batch_cert_counts(qt_handle* h, const qt_batch* b, int64_t* out) {
  if (!h || !b || !out) return qt_fail(h, QT_EINVAL, "batch_cert_counts: bad argument");
  for (int i = 0; i < QT_CERT_SLOTS; i++) out[i] = 0;
  const int n = b->ntask_cap;
  if (n == 0) return QT_OK;
  std::vector<int> cert(n);
  QT_CHECK_CUDA(h, cudaMemcpy(cert.data(), b->d_cert, sizeof(int) * n, cudaMemcpyDeviceToHost));
  for (int c : cert) out[(c >= 0 && c < QT_CERT_SLOTS) ? c : QT_CERT_NONE]++;
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
  // the slab holds 4 * slab_elems per CTA for the update; the sweep needs 3 (cap^2 each fits in one)
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
