// MPO application, SVD compression sweep and MPO expectation on a
// device-resident MPS.
//
// The reference applies an MPO lazily by wiring it into a network
// (apply_MPO, src/mpo.jl:184-216) and contracts everything exactly; its MPO
// sites are (b, out, in, b') (src/mpo.jl:66).  Here the MPO is applied site
// by site into the MPS (bond chi*b), then a compression sweep brings the
// bond back under chi_max with the tail rule of src/svd.jl:29-33:
//   left to right:  site = Q (orthonormalised), R absorbed into the next site;
//   right to left:  the truncated split of site^H = A'' B'' gives the new site
//                   A''^H (exact isometry) and B''^H absorbed into the left one.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "qt_internal.cuh"

namespace {

// N[(a + chiL al), o, (b + chiR be)] = sum_i W[al, o, i, be] A[a, i, b]
template <typename C>
__global__ void mpo_site_kernel(const C* __restrict__ A, int cl, int cr, const double2* __restrict__ W, int bl, int br,
                                C* __restrict__ N) {
  const int64_t ncl = (int64_t)cl * bl, ncr = (int64_t)cr * br;
  const int64_t total = ncl * 2 * ncr;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = idx % ncl, rest = idx / ncl;
    const int o = (int)(rest % 2);
    const int64_t col = rest / 2;
    const int a = (int)(row % cl), al = (int)(row / cl);
    const int b = (int)(col % cr), be = (int)(col / cr);
    double2 acc = make_double2(0, 0);
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const double2 w = W[al + bl * (o + 2 * (i + 2 * (int64_t)be))];
      cfma(acc, w, ccast<double2>(A[a + (int64_t)cl * (i + 2 * (int64_t)b)]));
    }
    N[idx] = ccast<C>(acc);
  }
}

// T2[(a + chiL s), (be + br d)] = sum_{al, t} W[al, s, t, be] T1[(a + chiL al), (t + 2 d)]
__global__ void mpo_env_mid_kernel(const double2* __restrict__ T1, int cl, int bl, int cr, const double2* __restrict__ W,
                                   int br, double2* __restrict__ T2) {
  const int64_t rows = 2 * (int64_t)cl, cols = (int64_t)br * cr;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < rows * cols;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx % rows, c = idx / rows;
    const int a = (int)(r % cl), s = (int)(r / cl);
    const int be = (int)(c % br), d = (int)(c / br);
    double2 acc = make_double2(0, 0);
    for (int al = 0; al < bl; al++)
      for (int t = 0; t < 2; t++) {
        const double2 w = W[al + bl * (s + 2 * (t + 2 * (int64_t)be))];
        cfma(acc, w, T1[(a + (int64_t)cl * al) + (int64_t)cl * bl * (t + 2 * (int64_t)d)]);
      }
    T2[idx] = acc;
  }
}

inline int g1(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 152 * 16); }

template <typename C>
int apply_mpo_t(qt_handle* h, qt_mps* mps, const double2* const* dW, const int* bl, const int* br) {
  for (int i = 0; i < mps->nsites; i++) {
    const int64_t cl = mps->chil[i], cr = mps->chir[i];
    const int64_t ncl = cl * bl[i], ncr = cr * br[i];
    void* p = nullptr;
    QT_TRY(qt_dmalloc(h, &p, sizeof(C) * ncl * 2 * ncr));
    QT_LAUNCH(h, mpo_site_kernel<C>, g1(ncl * 2 * ncr), 256, 0, (const C*)mps->site[i], (int)cl, (int)cr, dW[i], bl[i],
              br[i], (C*)p);
    qt_dfree(h, mps->site[i]);
    mps->site[i] = p;
    mps->cap[i] = sizeof(C) * ncl * 2 * ncr;
    mps->chil[i] = ncl;
    mps->chir[i] = ncr;
  }
  for (auto& s : mps->spectrum) s.clear();
  return QT_OK;
}

}  // namespace


extern "C" int qt_mps_apply_mpo(qt_handle* h, qt_mps* mps, const double* const* W, const int64_t* dims) {
  // W[i]: (bl, 2, 2, br) complex128 column-major interleaved; dims 4 per site
  if (!h || !mps || !W || !dims) return qt_fail(h, QT_EINVAL, "apply_mpo: null argument");
  cudaSetDevice(h->device);
  const int n = mps->nsites;
  std::vector<int> bl(n), br(n);
  for (int i = 0; i < n; i++) {
    if (dims[4 * i + 1] != 2 || dims[4 * i + 2] != 2 || dims[4 * i] < 1 || dims[4 * i + 3] < 1)
      return qt_fail(h, QT_EINVAL, "apply_mpo: MPO sites must be (b, 2, 2, b')");
    if (i > 0 && dims[4 * i] != dims[4 * i - 1])
      return qt_fail(h, QT_EDIM_MISMATCH, "Dimensions of contraction legs do not match");
    bl[i] = (int)dims[4 * i];
    br[i] = (int)dims[4 * i + 3];
  }
  qt_scratch s(h);
  std::vector<double2*> dW(n);
  for (int i = 0; i < n; i++) {
    const size_t cnt = (size_t)bl[i] * 4 * br[i];
    QT_TRY(s.get(&dW[i], cnt));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(dW[i], W[i], sizeof(double2) * cnt, cudaMemcpyHostToDevice, h->stream));
  }
  if (mps->dtype == QT_C128) QT_TRY(apply_mpo_t<double2>(h, mps, dW.data(), bl.data(), br.data()));
  else QT_TRY(apply_mpo_t<float2>(h, mps, dW.data(), bl.data(), br.data()));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

// Left-canonicalise with QRs, optionally normalise, then truncate right to
// left by the tail rule and chi_max.  ranks/discarded: nsites-1 entries (bond i).
extern "C" int qt_mps_compress(qt_handle* h, qt_mps* mps, double cutoff, int chi_max, int mode, int normalize,
                               int* ranks, double* discarded) {
  if (!h || !mps) return qt_fail(h, QT_EINVAL, "compress: null argument");
  if (!(cutoff >= 0)) return qt_fail(h, QT_EINVAL_ERR_NEG, "Error must be positive");
  cudaSetDevice(h->device);
  const int n = mps->nsites;
  const bool c64 = mps->dtype == QT_C64;
  const size_t es = c64 ? sizeof(float2) : sizeof(double2);
  // left to right: site = Q, next = R next  (R = Q^H site)
  for (int i = 0; i + 1 < n; i++) {
    const int64_t cl = mps->chil[i], cr = mps->chir[i];
    const int64_t rows = 2 * cl;
    const int64_t k = std::min(rows, cr);
    qt_scratch s(h);
    void *Q, *R, *nx;
    QT_TRY(s.get((char**)&Q, es * rows * k));
    QT_TRY(s.get((char**)&R, es * k * cr));
    const int64_t ncr = mps->chir[i + 1];
    QT_CHECK_CUDA(h, cudaMemcpyAsync(Q, mps->site[i], es * rows * k, cudaMemcpyDeviceToDevice, h->stream));
    if (c64) {
      const float2 one = make_float2(1, 0), zero = make_float2(0, 0);
      QT_TRY(qt_orthonormalize<float2>(h, (float2*)Q, rows, k));
      QT_TRY(qt_gemm_any(h, QT_OP_C, QT_OP_N, k, cr, rows, one, (float2*)Q, rows, (const float2*)mps->site[i], rows,
                         zero, (float2*)R, k));
      QT_TRY(qt_dmalloc(h, &nx, es * k * 2 * ncr));
      QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, k, 2 * ncr, cr, one, (float2*)R, k, (const float2*)mps->site[i + 1], cr,
                         zero, (float2*)nx, k));
    } else {
      const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
      QT_TRY(qt_orthonormalize<double2>(h, (double2*)Q, rows, k));
      QT_TRY(qt_gemm_any(h, QT_OP_C, QT_OP_N, k, cr, rows, one, (double2*)Q, rows, (const double2*)mps->site[i], rows,
                         zero, (double2*)R, k));
      QT_TRY(qt_dmalloc(h, &nx, es * k * 2 * ncr));
      QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_N, k, 2 * ncr, cr, one, (double2*)R, k, (const double2*)mps->site[i + 1],
                         cr, zero, (double2*)nx, k));
    }
    void* q_site = nullptr;
    QT_TRY(qt_dmalloc(h, &q_site, es * rows * k));
    QT_CHECK_CUDA(h, cudaMemcpyAsync(q_site, Q, es * rows * k, cudaMemcpyDeviceToDevice, h->stream));
    qt_dfree(h, mps->site[i]);
    mps->site[i] = q_site;
    mps->chir[i] = k;
    qt_dfree(h, mps->site[i + 1]);
    mps->site[i + 1] = nx;
    mps->chil[i + 1] = k;
  }
  if (normalize) {
    double* dn;
    qt_scratch s(h);
    QT_TRY(s.get(&dn, 1));
    const int64_t cnt = mps->chil[n - 1] * 2 * mps->chir[n - 1];
    if (c64) QT_TRY(qt_norm2<float2>(h, (const float2*)mps->site[n - 1], cnt, dn));
    else QT_TRY(qt_norm2<double2>(h, (const double2*)mps->site[n - 1], cnt, dn));
    double nrm2 = 0;
    QT_CHECK_CUDA(h, cudaMemcpyAsync(&nrm2, dn, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (nrm2 > 0) {
      // scale by converting the last site through the split helper's convert-scale
      const double f = 1.0 / std::sqrt(nrm2);
      std::vector<char> host((size_t)cnt * es);
      QT_CHECK_CUDA(h, cudaMemcpy(host.data(), mps->site[n - 1], host.size(), cudaMemcpyDeviceToHost));
      if (c64) {
        float2* v = (float2*)host.data();
        for (int64_t j = 0; j < cnt; j++) { v[j].x = (float)(v[j].x * f); v[j].y = (float)(v[j].y * f); }
      } else {
        double2* v = (double2*)host.data();
        for (int64_t j = 0; j < cnt; j++) { v[j].x *= f; v[j].y *= f; }
      }
      QT_CHECK_CUDA(h, cudaMemcpy(mps->site[n - 1], host.data(), host.size(), cudaMemcpyHostToDevice));
    }
  }
  // right to left: site^H (2 chiR x chiL) = A'' B''; site <- A''^H, left <- left B''^H
  for (int i = n - 1; i > 0; i--) {
    const int64_t cl = mps->chil[i], cr = mps->chir[i];
    qt_scratch s(h);
    void* Mh;
    QT_TRY(s.get((char**)&Mh, es * cl * 2 * cr));
    if (c64) QT_TRY(qt_adjoint_copy<float2>(h, (const float2*)mps->site[i], cl, 2 * cr, cl, (float2*)Mh, 2 * cr));
    else QT_TRY(qt_adjoint_copy<double2>(h, (const double2*)mps->site[i], cl, 2 * cr, cl, (double2*)Mh, 2 * cr));
    void *Ah = nullptr, *Bh = nullptr;
    int k = 0;
    double disc = 0;
    // exact rank bound: the Hilbert-space dimensions of the i qubits left of
    // the bond and the n - i right of it
    int64_t srank = std::min<int64_t>(2 * cr, cl);
    if (i < 40) srank = std::min<int64_t>(srank, (int64_t)1 << i);
    if (n - i < 40) srank = std::min<int64_t>(srank, (int64_t)1 << (n - i));
    QT_TRY(qt_split_device(h, mps->dtype, Mh, 2 * cr, cl, cutoff, chi_max, mode, &Ah, &Bh, &k, &disc, srank));
    // new site = Ah^H (k x 2cr); left site (pl, 2, cl) <- left . Bh^H (cl x k)
    void *ns = nullptr, *nl = nullptr;
    QT_TRY(qt_dmalloc(h, &ns, es * k * 2 * cr));
    const int64_t pl = mps->chil[i - 1];
    QT_TRY(qt_dmalloc(h, &nl, es * pl * 2 * k));
    if (c64) {
      const float2 one = make_float2(1, 0), zero = make_float2(0, 0);
      QT_TRY(qt_adjoint_copy<float2>(h, (const float2*)Ah, 2 * cr, k, 2 * cr, (float2*)ns, k));
      QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_C, 2 * pl, k, cl, one, (const float2*)mps->site[i - 1], 2 * pl,
                         (const float2*)Bh, k, zero, (float2*)nl, 2 * pl));
    } else {
      const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
      QT_TRY(qt_adjoint_copy<double2>(h, (const double2*)Ah, 2 * cr, k, 2 * cr, (double2*)ns, k));
      QT_TRY(qt_gemm_any(h, QT_OP_N, QT_OP_C, 2 * pl, k, cl, one, (const double2*)mps->site[i - 1], 2 * pl,
                         (const double2*)Bh, k, zero, (double2*)nl, 2 * pl));
    }
    qt_dfree(h, Ah);
    qt_dfree(h, Bh);
    qt_dfree(h, mps->site[i]);
    qt_dfree(h, mps->site[i - 1]);
    mps->site[i] = ns;
    mps->chil[i] = k;
    mps->site[i - 1] = nl;
    mps->chir[i - 1] = k;
    if (ranks) ranks[i - 1] = k;
    if (discarded) discarded[i - 1] = disc;
  }
  for (auto& sp : mps->spectrum) sp.clear();
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  return QT_OK;
}

// <psi|H|psi> / <psi|psi> for an MPO H with sites (bl, 2, 2, br), FP64 sweep.
extern "C" int qt_mps_expect_mpo(qt_handle* h, const qt_mps* mps, const double* const* W, const int64_t* dims,
                                 double* out) {
  if (!h || !mps || !W || !dims || !out) return qt_fail(h, QT_EINVAL, "expect_mpo: null argument");
  cudaSetDevice(h->device);
  const int n = mps->nsites;
  int64_t maxchi = 1, maxb = 1, maxsite = 1;
  for (int i = 0; i < n; i++) {
    maxchi = std::max(maxchi, std::max(mps->chil[i], mps->chir[i]));
    maxb = std::max<int64_t>(maxb, std::max(dims[4 * i], dims[4 * i + 3]));
    maxsite = std::max(maxsite, mps->chil[i] * 2 * mps->chir[i]);
  }
  qt_scratch s(h);
  double2 *E, *T1, *T2, *A64, *Wd;
  QT_TRY(s.get(&E, (size_t)maxchi * maxb * maxchi));
  QT_TRY(s.get(&T1, (size_t)maxchi * maxb * 2 * maxchi));
  QT_TRY(s.get(&T2, (size_t)2 * maxchi * maxb * maxchi));
  QT_TRY(s.get(&A64, (size_t)maxsite));
  QT_TRY(s.get(&Wd, (size_t)maxb * 4 * maxb));
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  // E[(a + chiL al), b] starts as the identity over the open left leg (bl = 1)
  const int64_t c0 = mps->chil[0];
  QT_TRY(qt_set_identity<double2>(h, E, c0, c0));
  for (int i = 0; i < n; i++) {
    const int64_t cl = mps->chil[i], cr = mps->chir[i];
    const int bl = (int)dims[4 * i], br = (int)dims[4 * i + 3];
    const double2* A = (const double2*)mps->site[i];
    if (mps->dtype == QT_C64) {
      QT_TRY(qt_convert(h, mps->site[i], QT_C64, A64, QT_C128, cl * 2 * cr));
      A = A64;
    }
    QT_CHECK_CUDA(h, cudaMemcpyAsync(Wd, W[i], sizeof(double2) * bl * 4 * br, cudaMemcpyHostToDevice, h->stream));
    // T1 ((cl bl) x (2 cr)) = E ((cl bl) x cl) . A (cl x 2cr)
    QT_TRY(qt_cgemm<double2>(h, QT_OP_N, QT_OP_N, cl * bl, 2 * cr, cl, one, E, cl * bl, A, cl, zero, T1, cl * bl));
    QT_LAUNCH(h, mpo_env_mid_kernel, g1(2 * cl * br * cr), 256, 0, T1, (int)cl, bl, (int)cr, Wd, br, T2);
    // E' (cr x (br cr)) = A_mat^H ((2cl) x cr)^H . T2 ((2cl) x (br cr))
    QT_TRY(qt_cgemm<double2>(h, QT_OP_C, QT_OP_N, cr, br * cr, 2 * cl, one, A, 2 * cl, T2, 2 * cl, zero, E, cr));
    // E' is laid out (c, be, d): the next step reads it as ((c + cr be) x d)
  }
  // trace over the open right leg with br = 1
  const int64_t cn = mps->chir[n - 1];
  std::vector<double2> hv((size_t)cn * cn);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(hv.data(), E, sizeof(double2) * cn * cn, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  double num = 0;
  for (int64_t i = 0; i < cn; i++) num += hv[i + cn * i].x;
  double den = 0;
  QT_TRY(qt_mps_expect(h, mps, 0, 0, &den));
  *out = num / den;
  return QT_OK;
}
