// frame.cuh — the whole frame of a small open system in one launch (frame.cu).
#pragma once

#include "force.cuh"
#include "push.cuh"

namespace geon {

// Largest system the frame kernel takes: its sort ranks every point against
// all points held in shared memory.
constexpr int FRAME_MAX_POINTS = 4096;

// Phase boundaries recorded by block 0 (globaltimer ns): launch, then the end
// of the frame-start scan, and of the first substep's push + keys, sort,
// gather, scans, emit, link, aggregation and walk, then the end of the frame.
constexpr int FRAME_STAMPS = 11;

// Device-side state of one frame launch: the grid barrier, the frame-start
// planner maxima and the frame's results.  count, abort and the maxima are
// zero between launches; gen only grows.
struct FrameRun {
    unsigned count;                  // blocks arrived at the current barrier
    unsigned gen;                    // barriers completed
    int abort;                       // a block's wait ran out: every block returns
    int substeps;                    // substeps the frame took
    int removed;                     // particles the boundary removed (already compacted into S2)
    int pad;
    double simTime;                  // simulation time at the end of the frame
    unsigned long long scanAccel;    // frame-start max |F|^2 / m^2 (double bits)
    unsigned long long scanCyc;      // frame-start max cyclotron frequency (double bits)
    unsigned long long stamp[FRAME_STAMPS];   // phase boundaries of the last frame (block 0's clock)
    int valid[2];                    // points inside the root box, by substep parity
};

struct FrameArgs {
    double dt;              // frame length
    double simTime;         // simulation time at the start
    double softening;       // planner: dtSafe = sqrt(softening / aMax)
    int maxSub;             // substep cap
    PushFlags F;
    int recordHist;         // sample the history at the end of the frame
    int histSlot;           // ring slot of that sample
    double* hist_t;         // [HIST_LEN] sample times
    float* hist_age;        // [HIST_LEN] scratch: simTime - t[slot]
    float* hist_segdt;      // [HIST_LEN] scratch: t[slot + 1] - t[slot]
    int* keep;              // [n] boundary keep flags
    int* dst;               // [n] compaction targets
    int slots;              // row stride of the force-breakdown rows
    int withHist;           // history rings allocated (compaction copies them)
    long long waitNs;       // a barrier gives up after this many nanoseconds
    int extraArrivals;      // blocks a barrier waits for beyond the grid (0; more only to test the time-out)
};

// Whether a system of n points (no ghosts) fits the frame kernel.
inline bool frame_fits(int n) { return n > 0 && n <= FRAME_MAX_POINTS; }

// Launches the frame: frame-start planner scan, the adaptive substeps (push,
// tree build, signal-delay tables, Barnes-Hut walk, planner) and the frame end
// (history sample, boundary, compaction into S2), all in one cooperative
// launch of frame_blocks(n) CTAs.  REL selects the signal-delayed walk.
// Returns the launch error (cudaErrorCooperativeLaunchTooLarge when the grid
// cannot be co-resident).
cudaError_t frame_launch(bool rel, const DevParams& P, const DevState& S, const DevState& S2, const TreeBufs& T,
                         int* d_root, FrameCtl* ctl, const ForceCtx& C, const FrameArgs& A, FrameRun* run, int n,
                         cudaStream_t st, LaunchCounter& lc);
int frame_blocks(int n);

}  // namespace geon
