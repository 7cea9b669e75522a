// mlp.cuh — launchers of the learned-correction network (mlp.cu).
//
// Weight vector (FP32, the nn.Linear convention W[out][in]):
//     mu[14] isd[14] W1[64][14] b1[64] W2[64][64] b2[64] W3[6][64] b3[6]
// mu, isd normalise the features, x' = (x - mu) * isd, in FP32 before they
// are rounded to BF16; training leaves them as they are.
#pragma once

#include "learn.cuh"

namespace geon {

constexpr int MLP_NPARAM = 2 * LF + LH * LF + LH + LH * LH + LH + LO * LH + LO;   // 5538

// Y[n][6] = net(X[n][14]) with device arrays.
void mlp_forward(const float* W, const float* X, int n, float* Y, int* err, cudaStream_t st, LaunchCounter& lc);

// Adds the learned correction of every record of the last walk (recs,
// rec_cnt, gcen, rec_cap; learn.cuh) to S.force of the ngroups groups'
// targets.  off[ngroups] is the exclusive prefix of the groups' counts and
// total their sum; expo (total x 16 floats), flags (total), net_list
// (total), net_count (1) and group_queue (1) are scratch.  With yext the
// network is not run: a record e (in group order) it applies to takes its
// outputs from yext[e * 6 ...] instead.
void learn_correct(const DevParams& P, const DevState& S, const TreeBufs& T, const FrameCtl* ctl, const float* W,
                   const uint2* recs, const int* rec_cnt, const float4* gcen, int rec_cap, int ngroups, const int* off,
                   int total, const float* yext, float4* expo, uint2* flags, int* net_list, int* net_count,
                   unsigned* group_queue, int* err, cudaStream_t st, LaunchCounter& lc);

// Accumulates into `grad` (MLP_NPARAM floats, zeroed by the caller) the
// gradient of  L = (1/B) sum_s wt_s sum_c (y_sc - y*_sc)^T A_sc (y_sc - y*_sc)
// over a batch of B samples and adds L to *loss.  T holds per sample
// y*[6] then the two quadratic forms A_c (A00 A11 A22 A01 A02 A12 each).
// With seed == 0 the batch is samples 0..B-1 of the data; otherwise sample j
// of step `step` is drawn uniformly from the n_data samples by a
// counter-based hash of (seed, step, j).  `wt` may be null (all weights 1).
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
