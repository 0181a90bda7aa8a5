// Expectation values by a left-to-right transfer sweep in FP64:
// E <- sum_s w_s A_s^H E A_s with A_s = A[:, s, :] (ld 2 chiL), w_s = 1 or the
// eigenvalue of Z (+1, -1) on the measured sites.  The reference has no
// observable routine; its closure-network pattern is the expectation_value
// cell of examples/expectation_value_optimization_example.ipynb.
#include <cuda_runtime.h>

#include "qt_internal.cuh"

int qt_mps_expect(qt_handle* h, const qt_mps* mps, int site, int nops, double* out) {
  const int n = mps->nsites;
  if (nops > 0 && (site < 0 || site + nops > n)) return qt_fail(h, QT_EBOUNDS, "expectation: site out of range");
  int64_t maxchi = 1, maxsite = 1;
  for (int i = 0; i < n; i++) {
    maxchi = std::max(maxchi, std::max(mps->chil[i], mps->chir[i]));
    maxsite = std::max(maxsite, mps->chil[i] * 2 * mps->chir[i]);
  }
  qt_scratch s(h);
  double2 *env, *env2, *tmp, *site64;
  QT_TRY(s.get(&env, (size_t)maxchi * maxchi));
  QT_TRY(s.get(&env2, (size_t)maxchi * maxchi));
  QT_TRY(s.get(&tmp, (size_t)maxchi * maxchi));
  QT_TRY(s.get(&site64, (size_t)maxsite));
  // E = ones(chiL0, chiL0) contracted with the open left leg: the identity on
  // that leg (an open chain's boundary legs are traced, as <psi|psi> does).
  const int64_t c0 = mps->chil[0];
  QT_TRY(qt_set_identity<double2>(h, env, c0, c0));
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  for (int i = 0; i < n; i++) {
    const int64_t cl = mps->chil[i], cr = mps->chir[i];
    const double2* A;
    if (mps->dtype == QT_C128) {
      A = (const double2*)mps->site[i];
    } else {
      QT_TRY(qt_convert(h, mps->site[i], QT_C64, site64, QT_C128, cl * 2 * cr));
      A = site64;
    }
    const bool measured = nops > 0 && i >= site && i < site + nops;
    for (int sidx = 0; sidx < 2; sidx++) {
      const double w = (measured && sidx == 1) ? -1.0 : 1.0;
      const double2* As = A + cl * sidx;
      // tmp (cl x cr) = env (cl x cl) . A_s
      QT_TRY(qt_cgemm<double2>(h, QT_OP_N, QT_OP_N, cl, cr, cl, one, env, cl, As, 2 * cl, zero, tmp, cl));
      // env2 (cr x cr) (+)= w A_s^H tmp
      QT_TRY(qt_cgemm<double2>(h, QT_OP_C, QT_OP_N, cr, cr, cl, make_double2(w, 0), As, 2 * cl, tmp, cl,
                               sidx == 0 ? zero : one, env2, cr));
    }
    std::swap(env, env2);
  }
  // trace over the open right leg
  const int64_t cn = mps->chir[n - 1];
  std::vector<double2> hv((size_t)cn * cn);
  QT_CHECK_CUDA(h, cudaMemcpyAsync(hv.data(), env, sizeof(double2) * cn * cn, cudaMemcpyDeviceToHost, h->stream));
  QT_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
  double tr = 0;
  for (int64_t i = 0; i < cn; i++) tr += hv[i + cn * i].x;
  *out = tr;
  return QT_OK;
}
