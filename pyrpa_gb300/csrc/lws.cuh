// Learned warm start: a small network that refines the coarse-mesh seed of
// the FLEX loop before the fine-mesh iterations start.
//
// One row per fine irreducible k, Matsubara index n and band pair (i, j):
// 16 features of the interpolated coarse Sigma in the band basis
// U(k)^dagger Sigma U(k), the band energies, w_n against the coarse cutoff
// and the model's descriptors -> 64 -> 64 -> 2 (tanh), the band-basis
// correction of Sigma in units of max |Sigma_seed|.  FP32 weights, inputs and
// activations stored as bf16 (rounded to nearest even), FP32 gradients, Adam.
// Parameters are one flat float vector: W1 [64][16], b1 [64], W2 [64][64],
// b2 [64], W3 [2][64], b3 [2].
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace pgb {

constexpr int kLwsNF = 16, kLwsNH = 64, kLwsNO = 2;
constexpr int kLwsOffB1 = kLwsNH * kLwsNF;
constexpr int kLwsOffW2 = kLwsOffB1 + kLwsNH;
constexpr int kLwsOffB2 = kLwsOffW2 + kLwsNH * kLwsNH;
constexpr int kLwsOffW3 = kLwsOffB2 + kLwsNH;
constexpr int kLwsOffB3 = kLwsOffW3 + kLwsNO * kLwsNH;
constexpr int kLwsNParam = kLwsOffB3 + kLwsNO;  // 5378

// Per-solution scalars, in the order of the C ABI's desc[9]: the Hubbard U
// and J, temperature, electrons per spin, Stoner factor and mu of the coarse
// solve, band width W of the fine mesh, s_scale = max |Sigma_seed|, Norb.
struct LwsDesc {
  double U, J, T, fill, stoner, mu_c, W, s_scale, Norb;
};

struct LwsNet {
  DBuf<float> theta, m, v;      // parameters and Adam moments
  DBuf<__nv_bfloat16> X;        // training rows [cap][16]
  DBuf<float> T;                // targets [cap][2]
  long long M = 0, cap = 0;     // rows held, rows allocated
  long long step = 0;           // Adam steps taken
};

int64_t lws_create();
void lws_destroy(int64_t h);
LwsNet& lws_get(int64_t h);

void lws_set_params(LwsNet& net, const float* host, long long n);
void lws_get_params(LwsNet& net, float* host, long long n);

// Host arrays in the C-ABI layouts: sigma (Nk,Nw,Norb,Norb), uni
// (Norb,Norb,Nk), eig (Norb,Nk) Fortran order; kn [P][2] = (k, n), 0-based.
// Appends P * Norb^2 rows of features and targets to the training set.
void lws_add_samples(LwsNet& net, const double2* sig_seed, const double2* sig_fine, const double2* uni,
                     const double* eig, const int64_t* kn, long long P, int Nk, int Nw, int Nw_c, int No,
                     const LwsDesc& d);
void lws_clear_samples(LwsNet& net);

// Features and targets of the given pairs, as float (the stored bf16
// features widened), without adding them to a training set; for checks.
void lws_features_host(float* x, float* t, const double2* sig_seed, const double2* sig_fine, const double2* uni,
                       const double* eig, const int64_t* kn, long long P, int Nk, int Nw, int Nw_c, int No,
                       const LwsDesc& d);

// y [M][2] of rows x [M][16] (rounded to bf16 on the way in).
void lws_forward_host(LwsNet& net, const float* x, long long M, float* y);

// Mean-square loss over the whole training set and its gradient (host).
double lws_loss_grad(LwsNet& net, float* grad);

// One Adam step with the gradient of the whole training set; its loss.
void lws_step_full(LwsNet& net, double lr, double beta1, double beta2, double eps, double* loss);

// `steps` Adam steps on batches of `batch` rows drawn uniformly with
// replacement (std::mt19937_64 seeded with `seed`); loss of each batch.
void lws_train(LwsNet& net, long long steps, long long batch, double lr, double beta1, double beta2, double eps,
               uint64_t seed, double* loss_out);

// Sigma (host, in place) += U (s_scale * y) U^dagger at every (k, n).
void lws_apply(LwsNet& net, double2* sigma, const double2* uni, const double* eig, int Nk, int Nw, int Nw_c, int No,
               const LwsDesc& d);

}  // namespace pgb
