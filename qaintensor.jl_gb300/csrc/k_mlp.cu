// The learned-rank MLP: hand-written forward, backward and Adam kernels, the
// bond-update features, and the logging of exact kept ranks as training data.
// (No counterpart in the reference, whose only rank rule is the tail rule of
// src/svd.jl:29-33; the predicted rank only sizes the randomized sketch.)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>

#include "qt_rank_model.h"

namespace {

constexpr int H = QT_MLP_H, IN = QT_MLP_IN, NP = QT_MLP_NPARAM;

// One CTA of 64 threads walks a slice of the samples; thread j owns hidden
// unit j of both layers.  With do_bwd the mean-squared-error gradients are
// accumulated per thread and added to grad with atomics; the summed squared
// error goes to *loss.
__global__ void __launch_bounds__(64)
mlp_kernel(const float* __restrict__ P, const float* __restrict__ X, const float* __restrict__ Y,
           const int* __restrict__ idx, int n, int per, float inv_n, int do_bwd, float* __restrict__ grad,
           float* __restrict__ loss, float* __restrict__ pred) {
  __shared__ float sP[NP];
  __shared__ float x[IN], h1[H], z1[H], h2[H], z2[H], dz2[H], red[2];
  const int j = threadIdx.x;
  for (int e = j; e < NP; e += 64) sP[e] = P[e];
  float gW1[IN], gW2[H], gb1 = 0, gb2 = 0, gW3 = 0, gb3 = 0, lsum = 0;
#pragma unroll
  for (int i = 0; i < IN; i++) gW1[i] = 0;
#pragma unroll
  for (int k = 0; k < H; k++) gW2[k] = 0;
  __syncthreads();
  const float* W1 = sP + QT_MLP_OFF_W1;
  const float* b1 = sP + QT_MLP_OFF_B1;
  const float* W2 = sP + QT_MLP_OFF_W2;
  const float* b2 = sP + QT_MLP_OFF_B2;
  const float* W3 = sP + QT_MLP_OFF_W3;
  const float b3 = sP[QT_MLP_OFF_B3];
  const int s0 = blockIdx.x * per, s1 = min(n, s0 + per);
  for (int s = s0; s < s1; s++) {
    const int row = idx ? idx[s] : s;
    if (j < IN) x[j] = X[(size_t)row * IN + j];
    __syncthreads();
    float z = b1[j];
#pragma unroll
    for (int i = 0; i < IN; i++) z = fmaf(W1[j * IN + i], x[i], z);
    z1[j] = z;
    h1[j] = fmaxf(z, 0.f);
    __syncthreads();
    z = b2[j];
#pragma unroll 16
    for (int k = 0; k < H; k++) z = fmaf(W2[j * H + k], h1[k], z);
    z2[j] = z;
    h2[j] = fmaxf(z, 0.f);
    float part = W3[j] * h2[j];
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((j & 31) == 0) red[j >> 5] = part;
    __syncthreads();
    const float y = b3 + red[0] + red[1];
    if (pred && j == 0) pred[s] = y;
    if (do_bwd) {
      const float t = Y[row];
      const float dy = 2.f * (y - t) * inv_n;
      if (j == 0) { lsum += (y - t) * (y - t); gb3 += dy; }
      gW3 = fmaf(dy, h2[j], gW3);
      const float d2 = (z2[j] > 0.f) ? dy * W3[j] : 0.f;
      dz2[j] = d2;
      gb2 += d2;
#pragma unroll
      for (int k = 0; k < H; k++) gW2[k] = fmaf(d2, h1[k], gW2[k]);
      __syncthreads();
      float dh1 = 0.f;
#pragma unroll 16
      for (int i = 0; i < H; i++) dh1 = fmaf(W2[i * H + j], dz2[i], dh1);
      const float d1 = (z1[j] > 0.f) ? dh1 : 0.f;
      gb1 += d1;
#pragma unroll
      for (int i = 0; i < IN; i++) gW1[i] = fmaf(d1, x[i], gW1[i]);
    }
    __syncthreads();
  }
  if (do_bwd && s1 > s0) {
#pragma unroll
    for (int i = 0; i < IN; i++) atomicAdd(&grad[QT_MLP_OFF_W1 + j * IN + i], gW1[i]);
    atomicAdd(&grad[QT_MLP_OFF_B1 + j], gb1);
#pragma unroll
    for (int k = 0; k < H; k++) atomicAdd(&grad[QT_MLP_OFF_W2 + j * H + k], gW2[k]);
    atomicAdd(&grad[QT_MLP_OFF_B2 + j], gb2);
    atomicAdd(&grad[QT_MLP_OFF_W3 + j], gW3);
    if (j == 0) {
      atomicAdd(&grad[QT_MLP_OFF_B3], gb3);
      atomicAdd(loss, lsum);
    }
  }
}

__global__ void adam_kernel(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Singular values of a 4x4 complex matrix: eigenvalues of M^H M by cyclic
// Jacobi in FP64 (host; 4x4 only).
void singular_values_4x4(const double* m /* col-major interleaved */, double* sv) {
  double a[4][4][2];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      double re = 0, im = 0;
      for (int k = 0; k < 4; k++) {
        const double ar = m[2 * (k + 4 * i)], ai = -m[2 * (k + 4 * i) + 1];  // conj(M[k,i])
        const double br = m[2 * (k + 4 * j)], bi = m[2 * (k + 4 * j) + 1];
        re += ar * br - ai * bi;
        im += ar * bi + ai * br;
      }
      a[i][j][0] = re;
      a[i][j][1] = im;
    }
  for (int sweep = 0; sweep < 30; sweep++) {
    double off = 0;
    for (int p = 0; p < 4; p++)
      for (int q = p + 1; q < 4; q++) off += a[p][q][0] * a[p][q][0] + a[p][q][1] * a[p][q][1];
    if (off < 1e-30) break;
    for (int p = 0; p < 4; p++)
      for (int q = p + 1; q < 4; q++) {
        const double gr = a[p][q][0], gi = a[p][q][1];
        const double ag = std::sqrt(gr * gr + gi * gi);
        if (ag < 1e-300) continue;
        const double zeta = (a[q][q][0] - a[p][p][0]) / (2 * ag);
        const double t = std::copysign(1.0, zeta) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
        const double c = 1 / std::sqrt(1 + t * t), s = c * t;
        const double er = gr / ag, ei = gi / ag;
        // columns: x_p' = c x_p - s e^{-i phi} x_q ; x_q' = s e^{i phi} x_p + c x_q
        for (int r = 0; r < 4; r++) {
          const double xpr = a[r][p][0], xpi = a[r][p][1], xqr = a[r][q][0], xqi = a[r][q][1];
          a[r][p][0] = c * xpr - s * (er * xqr + ei * xqi);
          a[r][p][1] = c * xpi - s * (er * xqi - ei * xqr);
          a[r][q][0] = s * (er * xpr - ei * xpi) + c * xqr;
          a[r][q][1] = s * (er * xpi + ei * xpr) + c * xqi;
        }
        // rows: g_p' = c g_p - s e^{i phi} g_q ; g_q' = s e^{-i phi} g_p + c g_q
        for (int r = 0; r < 4; r++) {
          const double gpr = a[p][r][0], gpi = a[p][r][1], gqr = a[q][r][0], gqi = a[q][r][1];
          a[p][r][0] = c * gpr - s * (er * gqr - ei * gqi);
          a[p][r][1] = c * gpi - s * (er * gqi + ei * gqr);
          a[q][r][0] = s * (er * gpr + ei * gpi) + c * gqr;
          a[q][r][1] = s * (er * gpi - ei * gpr) + c * gqi;
        }
      }
  }
  for (int i = 0; i < 4; i++) sv[i] = std::sqrt(std::max(0.0, a[i][i][0]));
  std::sort(sv, sv + 4, [](double x, double y) { return x > y; });
}

}  // namespace

qt_rank_model* qt_rank_model_create() { return new qt_rank_model(); }

void qt_rank_model_destroy(qt_rank_model* m) {
  if (!m) return;
  if (m->d_params) cudaFree(m->d_params);
  delete m;
}

int qt_rank_kmax(const qt_mps* mps, int site, int chi_max) {
  const int64_t a = 2 * mps->chil[site], b = 2 * mps->chir[site + 1];
  int64_t k = std::min(a, b);
  if (chi_max > 0) k = std::min<int64_t>(k, chi_max);
  return (int)k;
}

void qt_rank_features(const qt_mps* mps, int site, const double* G, double cutoff, int chi_max, float* f) {
  const int kmax = qt_rank_kmax(mps, site, chi_max);
  std::vector<double> s = mps->spectrum[site];
  if (s.empty()) s.assign((size_t)mps->chir[site], 1.0);  // unknown: flat over the bond
  double nrm = 0;
  for (double v : s) nrm += v * v;
  nrm = nrm > 0 ? std::sqrt(nrm) : 1.0;
  f[0] = (float)((double)s.size() / kmax);
  for (int j = 1; j <= 8; j++) {
    const double th = std::pow(10.0, -j);
    int c = 0;
    for (double v : s) c += (v / nrm > th) ? 1 : 0;
    f[j] = (float)((double)c / kmax);
  }
  // operator-Schmidt values: SVD of the interleaved (o1 i1) x (o2 i2) reshape
  // (the 4x4 SVD of src/decompose.jl:16-26 for M = 2)
  double r[32];
  for (int o1 = 0; o1 < 2; o1++)
    for (int o2 = 0; o2 < 2; o2++)
      for (int i1 = 0; i1 < 2; i1++)
        for (int i2 = 0; i2 < 2; i2++) {
          const int gi = (o1 + 2 * o2) + 4 * (i1 + 2 * i2);
          const int row = o1 + 2 * i1, col = o2 + 2 * i2;
          r[2 * (row + 4 * col)] = G[2 * gi];
          r[2 * (row + 4 * col) + 1] = G[2 * gi + 1];
        }
  double sv[4];
  singular_values_4x4(r, sv);
  for (int i = 0; i < 4; i++) f[9 + i] = (float)(sv[i] / 2.0);
  f[13] = (float)((double)site / std::max(1, mps->nsites));
  const double depth = mps->circuit_depth > 0 ? mps->circuit_depth : 1;
  f[14] = (float)(mps->circuit_layer / depth);
  f[15] = (float)(-std::log10(std::max(cutoff, 1e-300)) / 16.0);
}

int qt_gate_schmidt_rank(const double* G) {
  double r[32];
  for (int o1 = 0; o1 < 2; o1++)
    for (int o2 = 0; o2 < 2; o2++)
      for (int i1 = 0; i1 < 2; i1++)
        for (int i2 = 0; i2 < 2; i2++) {
          const int gi = (o1 + 2 * o2) + 4 * (i1 + 2 * i2);
          const int row = o1 + 2 * i1, col = o2 + 2 * i2;
          r[2 * (row + 4 * col)] = G[2 * gi];
          r[2 * (row + 4 * col) + 1] = G[2 * gi + 1];
        }
  double sv[4];
  singular_values_4x4(r, sv);
  int k = 0;
  for (int i = 0; i < 4; i++) k += (sv[i] > 1e-12 * sv[0]) ? 1 : 0;
  return std::max(k, 1);
}

int qt_rank_model_predict(qt_handle* h, const float* feat, int kmax) {
  qt_rank_model* m = h->rank_model;
  if (!m || !m->trained || !h->cfg.use_rank_model || !m->d_params) return -1;
  qt_scratch s(h);
  float *dx, *dp;
  if (s.get(&dx, IN) != QT_OK || s.get(&dp, 1) != QT_OK) return -1;
  cudaMemcpyAsync(dx, feat, sizeof(float) * IN, cudaMemcpyHostToDevice, h->stream);
  mlp_kernel<<<1, 64, 0, h->stream>>>(m->d_params, dx, nullptr, nullptr, 1, 1, 1.f, 0, nullptr, nullptr, dp);
  h->launches++;
  float y = 0;
  cudaMemcpyAsync(&y, dp, sizeof(float), cudaMemcpyDeviceToHost, h->stream);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return -1;
  double frac = std::min(1.0, std::max(0.0, (double)y)) * (1.0 + m->margin);
  int k = (int)std::ceil(frac * kmax);
  return std::max(1, std::min(k, kmax));
}

void qt_rank_model_log(qt_handle* h, const float* feat, int k, int kmax) {
  qt_rank_model* m = h->rank_model;
  if (!m || !m->logging) return;
  m->log_x.insert(m->log_x.end(), feat, feat + IN);
  m->log_y.push_back((float)k / (float)kmax);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

int qt_rank_model_set_logging(qt_handle* h, int on) {
  if (!h) return QT_EINVAL;
  h->rank_model->logging = on != 0;
  return QT_OK;
}

int64_t qt_rank_model_log_size(const qt_handle* h) { return h ? (int64_t)h->rank_model->log_y.size() : 0; }

int qt_rank_model_get_log(const qt_handle* h, float* X, float* Y) {
  if (!h || !X || !Y) return QT_EINVAL;
  std::memcpy(X, h->rank_model->log_x.data(), sizeof(float) * h->rank_model->log_x.size());
  std::memcpy(Y, h->rank_model->log_y.data(), sizeof(float) * h->rank_model->log_y.size());
  return QT_OK;
}

int qt_rank_model_clear_log(qt_handle* h) {
  if (!h) return QT_EINVAL;
  h->rank_model->log_x.clear();
  h->rank_model->log_y.clear();
  return QT_OK;
}

int qt_rank_model_set_params(qt_handle* h, const float* p, int nparam, int enable) {
  if (!h || !p) return QT_EINVAL;
  if (nparam != NP) return qt_fail(h, QT_EINVAL, "rank model: wrong parameter count");
  cudaSetDevice(h->device);
  qt_rank_model* m = h->rank_model;
  m->params.assign(p, p + NP);
  if (!m->d_params) QT_CHECK_CUDA(h, cudaMalloc(&m->d_params, sizeof(float) * NP));
  QT_CHECK_CUDA(h, cudaMemcpy(m->d_params, p, sizeof(float) * NP, cudaMemcpyHostToDevice));
  m->trained = enable != 0;
  return QT_OK;
}

int qt_rank_model_get_params(const qt_handle* h, float* p, int nparam) {
  if (!h || !p || nparam != NP || h->rank_model->params.empty()) return QT_EINVAL;
  std::memcpy(p, h->rank_model->params.data(), sizeof(float) * NP);
  return QT_OK;
}

int qt_rank_model_enable(qt_handle* h, int on) {
  if (!h) return QT_EINVAL;
  if (on && !h->rank_model->d_params) return qt_fail(h, QT_EINVAL, "rank model: no parameters");
  h->rank_model->trained = on != 0;
  return QT_OK;
}

int qt_rank_model_set_margin(qt_handle* h, double margin) {
  if (!h || !(margin >= 0)) return QT_EINVAL;
  h->rank_model->margin = margin;
  return QT_OK;
}

int qt_rank_model_nparams(void) { return NP; }

// Forward pass of the current parameters on n samples (row-major n x 16).
int qt_mlp_forward(qt_handle* h, int64_t n, const float* X, float* out) {
  if (!h || !X || !out || n < 1) return qt_fail(h, QT_EINVAL, "mlp_forward: bad argument");
  qt_rank_model* m = h->rank_model;
  if (!m->d_params) return qt_fail(h, QT_EINVAL, "mlp_forward: no parameters");
  cudaSetDevice(h->device);
  qt_scratch s(h);
  float *dx, *dy;
  QT_TRY(s.get(&dx, (size_t)n * IN));
  QT_TRY(s.get(&dy, (size_t)n));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dx, X, sizeof(float) * n * IN, cudaMemcpyHostToDevice, h->stream));
  const int per = 32;
  QT_LAUNCH(h, mlp_kernel, (unsigned)((n + per - 1) / per), 64, 0, m->d_params, dx, nullptr, nullptr, (int)n, per, 1.f,
            0, nullptr, nullptr, dy);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(out, dy, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

// Mean-squared-error loss and its gradient for the given parameters.
int qt_mlp_loss_grad(qt_handle* h, int64_t n, const float* X, const float* Y, const float* params, float* grad,
                     double* loss) {
  if (!h || !X || !Y || !params || !grad || !loss || n < 1) return qt_fail(h, QT_EINVAL, "mlp_loss_grad: bad argument");
  cudaSetDevice(h->device);
  qt_scratch s(h);
  float *dx, *dy, *dp, *dg, *dl;
  QT_TRY(s.get(&dx, (size_t)n * IN));
  QT_TRY(s.get(&dy, (size_t)n));
  QT_TRY(s.get(&dp, NP));
  QT_TRY(s.get(&dg, NP));
  QT_TRY(s.get(&dl, 1));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dx, X, sizeof(float) * n * IN, cudaMemcpyHostToDevice, h->stream));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dy, Y, sizeof(float) * n, cudaMemcpyHostToDevice, h->stream));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dp, params, sizeof(float) * NP, cudaMemcpyHostToDevice, h->stream));
  QT_CHECK_CUDA(h, cudaMemsetAsync(dg, 0, sizeof(float) * NP, h->stream));
  QT_CHECK_CUDA(h, cudaMemsetAsync(dl, 0, sizeof(float), h->stream));
  const int per = 32;
  QT_LAUNCH(h, mlp_kernel, (unsigned)((n + per - 1) / per), 64, 0, dp, dx, dy, nullptr, (int)n, per, 1.f / (float)n, 1,
            dg, dl, nullptr);
  float lf = 0;
  QT_CHECK_CUDA(h, cudaMemcpyAsync(grad, dg, sizeof(float) * NP, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(&lf, dl, sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  *loss = lf / (double)n;
  return QT_OK;
}

// Train from the given parameters (or a seeded He initialisation when
// init == NULL) with Adam on minibatches; the result becomes the active model.
int qt_rank_model_train(qt_handle* h, int64_t n, const float* X, const float* Y, const float* init, int epochs,
                        int batch, double lr, uint64_t seed, double* final_loss) {
  if (!h || !X || !Y || n < 1 || epochs < 1 || batch < 1) return qt_fail(h, QT_EINVAL, "rank_model_train: bad argument");
  cudaSetDevice(h->device);
  std::vector<float> p(NP, 0.f);
  std::mt19937_64 rng(seed);
  if (init) {
    std::memcpy(p.data(), init, sizeof(float) * NP);
  } else {
    std::normal_distribution<float> nd(0.f, 1.f);
    for (int i = 0; i < H * IN; i++) p[QT_MLP_OFF_W1 + i] = nd(rng) * std::sqrt(2.f / IN);
    for (int i = 0; i < H * H; i++) p[QT_MLP_OFF_W2 + i] = nd(rng) * std::sqrt(2.f / H);
    for (int i = 0; i < H; i++) p[QT_MLP_OFF_W3 + i] = nd(rng) * std::sqrt(2.f / H);
  }
  qt_scratch s(h);
  float *dx, *dy, *dp, *dg, *dm, *dv, *dl;
  int* didx;
  QT_TRY(s.get(&dx, (size_t)n * IN));
  QT_TRY(s.get(&dy, (size_t)n));
  QT_TRY(s.get(&didx, (size_t)n));
  QT_TRY(s.get(&dp, NP));
  QT_TRY(s.get(&dg, NP));
  QT_TRY(s.get(&dm, NP));
  QT_TRY(s.get(&dv, NP));
  QT_TRY(s.get(&dl, 1));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dx, X, sizeof(float) * n * IN, cudaMemcpyHostToDevice, h->stream));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dy, Y, sizeof(float) * n, cudaMemcpyHostToDevice, h->stream));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(dp, p.data(), sizeof(float) * NP, cudaMemcpyHostToDevice, h->stream));
  QT_CHECK_CUDA(h, cudaMemsetAsync(dm, 0, sizeof(float) * NP, h->stream));
  QT_CHECK_CUDA(h, cudaMemsetAsync(dv, 0, sizeof(float) * NP, h->stream));
  std::vector<int> order((size_t)n);
  std::iota(order.begin(), order.end(), 0);
  int step = 0;
  const float b1 = 0.9f, b2 = 0.999f;
  for (int ep = 0; ep < epochs; ep++) {
    std::shuffle(order.begin(), order.end(), rng);
    QT_CHECK_CUDA(h, cudaMemcpyAsync(didx, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));  // order is reshuffled next epoch
    for (int64_t b0 = 0; b0 < n; b0 += batch) {
      const int nb = (int)std::min<int64_t>(batch, n - b0);
      QT_CHECK_CUDA(h, cudaMemsetAsync(dg, 0, sizeof(float) * NP, h->stream));
      const int per = 16;
      QT_LAUNCH(h, mlp_kernel, (unsigned)((nb + per - 1) / per), 64, 0, dp, dx, dy, didx + b0, nb, per,
                1.f / (float)nb, 1, dg, dl, nullptr);
      step++;
      const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
      QT_LAUNCH(h, adam_kernel, (NP + 255) / 256, 256, 0, dp, dg, dm, dv, NP, (float)lr, b1, b2, 1e-8f, c1, c2);
    }
  }
  // final full-data loss
  QT_CHECK_CUDA(h, cudaMemsetAsync(dg, 0, sizeof(float) * NP, h->stream));
  QT_CHECK_CUDA(h, cudaMemsetAsync(dl, 0, sizeof(float), h->stream));
  QT_LAUNCH(h, mlp_kernel, (unsigned)((n + 31) / 32), 64, 0, dp, dx, dy, nullptr, (int)n, 32, 1.f / (float)n, 1, dg, dl,
            nullptr);
  float lf = 0;
  QT_CHECK_CUDA(h, cudaMemcpyAsync(p.data(), dp, sizeof(float) * NP, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaMemcpyAsync(&lf, dl, sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  if (final_loss) *final_loss = lf / (double)n;
  return qt_rank_model_set_params(h, p.data(), NP, 1);
}

int qt_rank_features_of(const qt_mps* mps, int site, const double* G, double cutoff, int chi_max, float* f) {
  if (!mps || !G || !f || site < 0 || site + 1 >= mps->nsites) return QT_EINVAL;
  qt_rank_features(mps, site, G, cutoff, chi_max, f);
  return QT_OK;
}

int qt_mps_set_bond_spectrum(qt_mps* mps, int bond, const double* s, int n) {
  if (!mps || bond < 0 || bond + 1 >= mps->nsites || n < 0 || (n > 0 && !s)) return QT_EINVAL;
  mps->spectrum[bond].assign(s, s + n);
  return QT_OK;
}

int qt_mps_set_circuit_position(qt_mps* mps, int layer, int depth) {
  if (!mps || depth < 0) return QT_EINVAL;
  mps->circuit_layer = layer;
  mps->circuit_depth = depth;
  return QT_OK;
}

}  // extern "C"
