// boson.cuh — walks over the boson tree (boson.cu).
#pragma once

#include "state.cuh"

namespace geon {

constexpr float BOSON_SOFTENING_SQ = 4.f;   // src/config.js:48

// The boson pool's tree: the buffers of the handle that holds the pool as
// particles (position, mass = _srcMass, charge = _srcCharge).
struct BosonTree {
    TreeBufs T;
    const FrameCtl* ctl;    // node counts of that build
    const int* d_root;
    DevState S;             // the pool itself (targets of the kicks)
    const float2* kind;     // [n] kind (0 photon, 1 massive), v^2
    const double* iq;       // [cap_int] exact charge of each internal node
    const double* lq;       // [cap_pts] exact charge of each leaf
    int n;
};

// Exact (FP64) charge sums of the pool's nodes: the Coulomb walk skips a node
// whose charge is exactly zero (forces.js:864), so the sums of FP32 charges
// must be exact, as the reference's FP64 sums of the same values are.
void boson_charges(const BosonTree& B, double* iq, double* lq, cudaStream_t st, LaunchCounter& lc);

// computeBosonGravity (src/forces.js:788-804) on every particle of the force
// pass just run (targets from `tgt_list` when not null, else the particle
// tree's order TP.tgt, whose tree must be current),
// added to force and the gravity breakdown rows; then the planner maxima of
// that pass are recomputed from the updated forces.
void boson_gravity(const DevParams& P, const DevState& S, const TreeBufs& TP, FrameCtl* ctl, const BosonTree& B,
                   const int* tgt_list, int tgt_count, bool brk, int n_cap, cudaStream_t st, LaunchCounter& lc);

// The kicks of applyBosonBosonGravity (what & 1; src/forces.js:812-856) and
// applyPionPionCoulomb (what & 2; src/forces.js:878-901) on every boson of
// the pool, into out[n] (device).  `massive` counts the pions and leptons.
void boson_kicks(const DevParams& P, const BosonTree& B, float dt, unsigned what, int massive, float2* out,
                 cudaStream_t st, LaunchCounter& lc);

}  // namespace geon
