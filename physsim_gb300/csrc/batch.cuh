// batch.cuh — many independent systems in one handle: device-side substep
// planner, per-system reductions and warp-aligned target lists (batch.cu).
//
// Every system of a batched handle runs Physics.update's adaptive substep
// loop (src/integrator.js:810-875) with its own dt schedule; the planner
// that the single-system driver runs on the host in FP64 runs here on the
// device, one thread per system, with the same formulas, so that a frame
// needs no host round trip and can be captured in a CUDA graph.
#pragma once

#include "state.cuh"

namespace geon {

struct SysPlan {
    double dtRemain;       // time left in the frame
    double curAccel;       // max |a|^2 of the current forces
    double curCyc;         // max cyclotron frequency of the current forces
    double lastKick;       // curAccel of the forces used by the previous kick (integrator.js:881-928)
    double simTime;
    int steps;             // substeps taken in this frame
    int pending;           // a force pass ran since the last planning step
};

// Device arrays of a batched handle.
struct BatchDev {
    int nsys;
    SysPlan* plan;         // [nsys]
    double* sys_dt;        // [nsys] substep of the current pass (<= 0: not stepping)
    unsigned long long* sys_accel;   // [nsys] planner maxima written by the force pass (double bits)
    unsigned long long* sys_cyc;
    const int* sys_off;    // [nsys + 1] first particle of each system
    const int* pad_off;    // [nsys] first walk slot of each system (multiples of 32)
    int* tgt_pad;          // [n_slots] walk order, -1 in padding slots
    int* any_active;       // set by the planner: some system takes another substep
    double* frame_dt;      // dt of the frame being run
};

// Frame start: per-system maxima of the forces in place (integrator.js:813-836)
// and the planner state for a frame of length *frame_dt.
void batch_frame_start(const DevParams& P, const DevState& S, const BatchDev& B, int n, cudaStream_t st,
                       LaunchCounter& lc);
// Planning step: reads the maxima of the force pass just run, then decides
// each system's next substep (sys_dt) and whether any system continues.
// `cond` (when non-zero) is the graph conditional handle the decision also
// sets.
void batch_plan(const DevParams& P, const BatchDev& B, double softening, int max_substeps,
                unsigned long long cond, cudaStream_t st, LaunchCounter& lc);
// Warp-aligned walk order from the tree's target order T.tgt.
void batch_targets(const DevState& S, const TreeBufs& T, FrameCtl* ctl, const BatchDev& B, int n, cudaStream_t st,
                   LaunchCounter& lc);

}  // namespace geon
