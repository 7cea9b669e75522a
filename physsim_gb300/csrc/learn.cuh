// learn.cuh — learned far-field correction: features of a (cell, target)
// pair and the launchers of learn.cu / mlp.cu.
//
// For a Barnes-Hut interaction in which target i accepts cell c as one
// aggregate (src/forces.js:680-685), the force is the monopole term at the
// cell's centre of mass.  The correction adds
//     m_i * (M s^2 / r_e^4) * g(x_mass)
// where g is a small MLP (9 -> 64 -> 64 -> 2, GELU) of dimensionless features
// of the cell seen from the target, M the cell mass, s the cell size and
// r_e^2 = |d|^2 + softening^2: the mass-sourced field (gravity and Yukawa).
// The dataset also carries charge-net features with the scale S / r_e^2
// (S = sum |q|) for the Coulomb field; measured, a charge net gains nothing
// on the configurations here, so the force pass applies g only.
#pragma once

#include "state.cuh"

namespace geon {

constexpr int LF = 9;          // features per net
constexpr int LH = 64;         // hidden width
constexpr int LO = 2;          // outputs per net

// d = cell COM - target position; size = 2 * half-size of the cell.
__device__ __forceinline__ void pair_features(const DevParams& P, float dx, float dy, float size, float M, float Q,
                                              const float4& m1, const float4& m2, const float4& m3,
                                              float* fm, float* fc, float& scale_m, float& scale_c) {
    const float r2 = dx * dx + dy * dy;
    const float re2 = r2 + P.softSq;
    const float inv = rsqrtf(re2);
    const float inv2 = inv * inv;
    const float ux = dx * inv, uy = dy * inv;
    const float sz = size * inv, so = P.soft * inv;
    fm[0] = ux; fm[1] = uy; fm[2] = sz; fm[3] = so;
    // second moments per unit mass in units of the cell size squared, and a
    // scale with the quadrupole's fall-off M s^2 / r_e^4, so that features and
    // targets stay O(1) from the largest to the smallest accepted cells
    const float s2 = size * size;
    const float iMs = (M > 0.f && s2 > 0.f) ? 1.f / (M * s2) : 0.f;
    fm[4] = m1.x * iMs; fm[5] = m1.y * iMs; fm[6] = m1.z * iMs;
    fm[7] = P.yukOn ? P.yukMu * (re2 * inv) * (1.f / 6.f) : 0.f;
    fm[8] = P.yukOn ? r2 / P.yukCutSq : 0.f;
    scale_m = M * s2 * inv2 * inv2;
    const float S = m1.w;
    const float iS = S > 0.f ? 1.f / S : 0.f;
    fc[0] = ux; fc[1] = uy; fc[2] = sz; fc[3] = so;
    fc[4] = Q * iS;
    fc[5] = m2.x * iS * inv; fc[6] = m2.y * iS * inv;
    fc[7] = (m2.z - m3.x) * iS * inv2; fc[8] = 2.f * m2.w * iS * inv2;
    scale_c = S * inv2;
}

// Per-pair record of the inference path: the cell (internal node index) and
// the target particle.
struct LearnPair { int node; int target; };

// learn.cu
// Collects the (cell, target) aggregate interactions of a Barnes-Hut walk for
// the listed targets (device arrays), then computes features and the exact
// member-sum residuals.  Returns the pair count through *d_count (64-bit:
// at small theta a million targets accept more than 2^31 cells); pairs at
// positions >= cap are counted but not stored.
void learn_collect_pairs(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                         const int* d_targets, int k, LearnPair* pairs, long long cap, unsigned long long* d_count,
                         cudaStream_t st, LaunchCounter& lc);
// Writes the first min(*d_count, cap) pairs to `out` in (target, node)
// order (so that datasets do not depend on the collection's timing); *d_n
// receives their number.  `scratch` holds learn_sort_scratch_bytes(cap).
size_t learn_sort_scratch_bytes(int cap);
void learn_sort_pairs(const LearnPair* pairs, const unsigned long long* d_count, int cap, LearnPair* out, int* d_n,
                      void* scratch, cudaStream_t st, LaunchCounter& lc);
void learn_residuals(const DevParams& P, const DevState& S, const TreeBufs& T, const LearnPair* pairs,
                     const unsigned long long* d_count,
                     int cap, float* feat_m, float* feat_c, float* target, float* scales, cudaStream_t st,
                     LaunchCounter& lc);

}  // namespace geon
