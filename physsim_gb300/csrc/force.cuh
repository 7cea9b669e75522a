// force.cuh — declarations shared by the force kernels (force.cu) and the
// frame driver (capi.cu).
#pragma once

#include "state.cuh"

namespace geon {

// Per-pass context for the force kernels.
struct ForceCtx {
    double simTime;
    const double* hist_t;     // [256] sample times (ring, shared by all particles)
    const float* hist_age;    // [256] simTime - t[slot]
    const float* hist_segdt;  // [256] t[slot+1] - t[slot]
    int hist_head;            // next ring slot to be written
    int pe;                   // accumulate potential energy
    int brk;                  // keep per-type vectors
    int bounce;               // boundary == BOUNCE (wall forces)
    // batched handles (all null for one system)
    const int* tgt_list;      // targets, each system's run padded to whole warps (-1 = padding)
    int tgt_count;
    const int* roots;         // root of each system
    const double* sys_dt;     // substep of each system; systems with dt <= 0 sit this pass out
    unsigned long long* sys_accel;   // per-system planner maxima (double bits)
    unsigned long long* sys_cyc;
    // learned correction: each warp of the walk (a group of 32 consecutive
    // targets in walk order) records every cell some of its targets accept as
    // one aggregate, as (node, mask of accepting lanes), into its own segment
    // recs[group * rec_cap ...]; rec_cnt[group] receives the count (records
    // beyond rec_cap are counted, not stored), rec_max the largest count and
    // rec_total their sum
    uint2* recs;
    int rec_cap;
    int* rec_cnt;
    unsigned* rec_max;
    unsigned long long* rec_total;
    float4* gcen;                // per group: centre of the targets' box (x, y), radius bound
    // pairwise sum split over source slices (direct_plan): scratch of partial
    // sums, null or dslices <= 1 for one pass over all sources
    float* dpart;
    int dslices;
    // split walk (walkc_body with SPLIT warps per target group): nodes at
    // levels up to split_level are evaluated by one warp each (node index
    // modulo SPLIT), and a node at split_level is opened only by that warp
    int split_level;
    // walk shape of the launch-per-phase force pass (batched handles): walk_split
    // selects four warps per group of 32 targets (plain forces only), walk_ctas
    // > 0 caps the resident walk CTAs per SM by padding their shared memory
    int walk_split;
    int walk_ctas;
    // walk_chunk > 0: the grouped walk runs as persistent CTAs (as many as fit
    // the GPU at once) that take walk blocks walk_chunk at a time from the
    // counters walk_queue[2] (zero between launches); plain forces only
    int walk_chunk;
    unsigned* walk_queue;
};

// How the pairwise sum over n_cap targets is split: the number of source
// slices that fills whole waves of the GPU (1 when the targets alone do) and
// the scratch floats they need.
struct DirectPlan { int slices; size_t floats; };
DirectPlan direct_plan(const DevParams& P, bool brk, int n_cap);
DirectPlan direct1pn_plan(int n_cap);   // the same for the 1PN-only pairwise pass
DirectPlan direct_subset_plan(const DevParams& P, int k);   // and for direct_subset over k targets

// Force pass: resetForces + computeAllForces (+ external fields, bounce
// walls) for every particle, with the max-acceleration / cyclotron
// reductions for the substep planner.  `bh` selects the tree walk (tree must
// be built) or the pairwise sum.
// Potential heat map on a G x G grid of cell centres (heatmap.js:152-206):
// tree walk (useTree, tree built) or pairwise sum; optional 3 x 3 box blur
// of each computed field (tmp: G*G floats).  Device outputs of G*G floats.
// The pairwise sum runs split over source slices (part: their partial sums).
void heatmap_pass(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                  const ForceCtx& C, double left, double top, double cw, double ch, int G, bool doG, bool doE, bool doY,
                  bool useTree, bool blur, float* g, float* e, float* y, float* tmp, float* part, int slices,
                  cudaStream_t st, LaunchCounter& lc);
// Source slices of the pairwise heat map (1 in tree mode); `part` for
// heatmap_pass then holds slices * 6 * G * G floats.
int heatmap_slices(const DevParams& P, int G, bool useTree);

// clear = false keeps the planner reductions and the interaction counter of
// earlier passes (a force pass split over target chunks).
// Prepares the work-queue walk (ForceCtx::walk_chunk) on the current device:
// its shared-memory limit and resident CTAs per SM, looked up outside any
// graph capture.
void walk_queue_setup();

void force_pass(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                const ForceCtx& C, bool bh, int n_cap, cudaStream_t st, LaunchCounter& lc, bool clear = true);

// Pairwise forces (fx, fy) on the listed particles from all particles, into
// separate outputs (device arrays of k floats); the state is not changed.
void direct_subset(const DevParams& P, const DevState& S, const FrameCtl* ctl, const ForceCtx& C, const int* idx,
                   int k, float* fx, float* fy, cudaStream_t st, LaunchCounter& lc);

// 1PN-only pass (forces.js:578-610): writes S.f1pn.
void onepn_pass(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                const ForceCtx& C, bool bh, int n_cap, cudaStream_t st, LaunchCounter& lc);

}  // namespace geon
