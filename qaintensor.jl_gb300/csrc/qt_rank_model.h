// Learned-rank model: a 16-64-64-1 ReLU MLP that predicts the kept rank of a
// bond update (as a fraction of k_max = min(2 chiL, 2 chiR, chi_max)) from
// the bond's previous spectrum, the gate's operator-Schmidt values, the site
// and the circuit position.  Training data are (features, exact kept rank)
// pairs logged from updates whose rank came from an exact SVD.
#pragma once

#include <vector>

#include "qt_internal.cuh"

constexpr int QT_MLP_IN = 16;
constexpr int QT_MLP_H = 64;
// packed parameter layout: W1 (64x16, row-major), b1 (64), W2 (64x64), b2 (64), W3 (64), b3 (1)
constexpr int QT_MLP_OFF_W1 = 0;
constexpr int QT_MLP_OFF_B1 = QT_MLP_OFF_W1 + QT_MLP_H * QT_MLP_IN;
constexpr int QT_MLP_OFF_W2 = QT_MLP_OFF_B1 + QT_MLP_H;
constexpr int QT_MLP_OFF_B2 = QT_MLP_OFF_W2 + QT_MLP_H * QT_MLP_H;
constexpr int QT_MLP_OFF_W3 = QT_MLP_OFF_B2 + QT_MLP_H;
constexpr int QT_MLP_OFF_B3 = QT_MLP_OFF_W3 + QT_MLP_H;
constexpr int QT_MLP_NPARAM = QT_MLP_OFF_B3 + 1;

struct qt_rank_model {
  bool trained = false;
  bool logging = false;
  float* d_params = nullptr;        // device copy of the packed parameters
  std::vector<float> params;        // host copy
  std::vector<float> log_x, log_y;  // logged features / targets (k / k_max)
  double margin = 0.10;             // predicted fraction is inflated by this
};

qt_rank_model* qt_rank_model_create();
void qt_rank_model_destroy(qt_rank_model* m);

// 16 features of the update on bond (site, site+1) of mps with gate G.
void qt_rank_features(const qt_mps* mps, int site, const double* G, double cutoff, int chi_max, float* f);
int qt_rank_kmax(const qt_mps* mps, int site, int chi_max);
// Operator-Schmidt rank of a 4x4 gate (complex128, column-major): the number
// of its operator-Schmidt values above 1e-12 of the largest (1 for a product
// of one-qubit gates, 2 for CNOT, 4 for SWAP and generic gates).
int qt_gate_schmidt_rank(const double* G);

// Predicted kept rank (>= 1), or -1 when no trained model is active.
int qt_rank_model_predict(qt_handle* h, const float* feat, int kmax);
// Record (features, k / kmax) when logging is on.
void qt_rank_model_log(qt_handle* h, const float* feat, int k, int kmax);
