// mlp.cuh — launchers of the learned-correction network (mlp.cu).
//
// Weight vector (FP32, the nn.Linear convention W[out][in]):
//     W1[64][9] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]
#pragma once

#include "learn.cuh"

namespace geon {

constexpr int MLP_NPARAM = LH * LF + LH + LH * LH + LH + LO * LH + LO;   // 4930

// Y[n][2] = net(X[n][9]) with device arrays.
void mlp_forward(const float* W, const float* X, int n, float* Y, int* err, cudaStream_t st, LaunchCounter& lc);

// Adds m_i * (M s^2 / r_e^4) * net(features) to S.force for every recorded (cell,
// target) pair; `npairs` is the number of valid entries of `pairs`.
void mlp_correct(const DevParams& P, const DevState& S, const TreeBufs& T, const float* W, const LearnPair* pairs,
                 int npairs, int* err, cudaStream_t st, LaunchCounter& lc);

// Accumulates into `grad` (MLP_NPARAM floats, zeroed by the caller) the
// gradient of  L = (1/B) * sum_s wt_s * |net(x_s) - t_s|^2  over a batch of B
// samples, and adds L to *loss.  With seed == 0 the batch is samples 0..B-1
// of the data; otherwise sample j of step `step` is drawn uniformly from the
// n_data samples by a counter-based hash of (seed, step, j).  `wt` may be null
// (all weights 1).
// The sum over the CTAs is taken in a fixed order from per-CTA slots in
// `part` (mlp_grad_scratch_floats() floats) and `loss_part`
// (mlp_grad_scratch_ctas() doubles), so the result does not depend on timing.
void mlp_grad(const float* W, const float* X, const float* T, const float* wt, int n_data, int batch, uint64_t seed,
              int step, float* grad, double* loss, float* part, double* loss_part, int* err, cudaStream_t st,
              LaunchCounter& lc);
size_t mlp_grad_scratch_floats();
int mlp_grad_scratch_ctas();

// One Adam update of W from `grad` (then zeroed); m and v are the moment
// vectors, t the 1-based step number.
void mlp_adam(float* W, float* grad, float* m, float* v, float lr, float beta1, float beta2, float eps, int t,
              cudaStream_t st, LaunchCounter& lc);

}  // namespace geon
