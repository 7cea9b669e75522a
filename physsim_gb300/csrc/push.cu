// push.cu — the per-particle parts of the substep and of the frame:
//   frame-start planner scan       src/integrator.js:813-836
//   Boris kick / rotate / kick     src/integrator.js:884-928
//   spin-orbit + torques           src/integrator.js:930-982
//   drift                          src/integrator.js:1269-1278
//   1PN velocity-Verlet kick       src/integrator.js:1311-1317
//   history sampling               src/integrator.js:1549-1565
//   boundary + compaction          src/integrator.js:1798-1824, topology.js:81-135
//   conserved quantities (FP64)    src/energy.js:11-62
// One thread per particle; every loop of the reference over particles is a
// grid-stride loop here.  Positions are compensated pairs (pos + pos_lo), so
// the small drift increments are not lost against large coordinates.
#include "push_dev.cuh"

namespace geon {

static inline int grid_for(int n, int threads) {
    int b = (n + threads - 1) / threads;
    return std::max(1, std::min(b, device_sms() * 16));
}

__global__ void scan_forces_kernel(DevParams P, DevState S, FrameCtl* ctl) {
    scan_forces_body(P, S, ctl, &ctl->maxAccelSqBits, &ctl->maxCycBits, blockIdx.x, gridDim.x);
}
__global__ void clear_planner_kernel(FrameCtl* ctl) { clear_planner_body(ctl, blockIdx.x, gridDim.x); }
__global__ void push_kernel(DevParams P, DevState S, const FrameCtl* ctl, float dtSub0, PushFlags F,
                            const double* __restrict__ sys_dt) { push_body(P, S, ctl, dtSub0, F, sys_dt, blockIdx.x, gridDim.x); }
__global__ void vv_kick_kernel(DevParams P, DevState S, const FrameCtl* ctl, float halfDt) { vv_kick_body(P, S, ctl, halfDt, blockIdx.x, gridDim.x); }
__global__ void hist_tables_kernel(const double* __restrict__ hist_t, double simTime, float* age, float* segdt) { hist_tables_body(hist_t, simTime, age, segdt, blockIdx.x, gridDim.x); }
__global__ void record_history_kernel(DevState S, const FrameCtl* ctl, double* hist_t, int slot, double simTime) { record_history_body(S, ctl, hist_t, slot, simTime, blockIdx.x, gridDim.x); }
__global__ void boundary_kernel(DevParams P, DevState S, FrameCtl* ctl, int* keep) { boundary_body(P, S, ctl, keep, blockIdx.x, gridDim.x); }
__global__ void compact_kernel(DevState S, DevState D, const int* keep, const int* dst, int n, int n_cap,
                               int with_hist, int with_brk) { compact_body(S, D, keep, dst, n, n_cap, with_hist, with_brk, blockIdx.x, gridDim.x); }
__global__ void stats_pass1_kernel(DevParams P, DevState S, const FrameCtl* ctl, double* out) { stats_pass1_body(P, S, ctl, out, blockIdx.x, gridDim.x); }
__global__ void stats_pass2_kernel(DevParams P, DevState S, const FrameCtl* ctl, double* out) { stats_pass2_body(P, S, ctl, out, blockIdx.x, gridDim.x); }

void launch_frame_scan(const DevParams& P, const DevState& S, FrameCtl* ctl, int n_cap, cudaStream_t st, LaunchCounter& lc) {
    clear_planner_kernel<<<1, 1, 0, st>>>(ctl);
    scan_forces_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(P, S, ctl);
    lc.add(2);
}
void launch_push(const DevParams& P, const DevState& S, const FrameCtl* ctl, float dtSub, const PushFlags& F,
                 int n_cap, cudaStream_t st, LaunchCounter& lc, const double* sys_dt) {
    push_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(P, S, ctl, dtSub, F, sys_dt);
    lc.add(1);
}
void launch_vv_kick(const DevParams& P, const DevState& S, const FrameCtl* ctl, float halfDt, int n_cap,
                    cudaStream_t st, LaunchCounter& lc) {
    vv_kick_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(P, S, ctl, halfDt);
    lc.add(1);
}
void launch_hist_tables(const double* hist_t, double simTime, float* age, float* segdt, cudaStream_t st, LaunchCounter& lc) {
    hist_tables_kernel<<<1, HIST_LEN, 0, st>>>(hist_t, simTime, age, segdt);
    lc.add(1);
}
void launch_record_history(const DevState& S, const FrameCtl* ctl, double* hist_t, int slot, double simTime,
                           int n_cap, cudaStream_t st, LaunchCounter& lc) {
    record_history_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(S, ctl, hist_t, slot, simTime);
    lc.add(1);
}
void launch_boundary(const DevParams& P, const DevState& S, FrameCtl* ctl, int* keep, int n_cap, cudaStream_t st,
                     LaunchCounter& lc) {
    boundary_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(P, S, ctl, keep);
    lc.add(1);
}
void launch_compact(const DevState& S, const DevState& D, const int* keep, const int* dst, int n, int n_cap,
                    bool with_hist, bool with_brk, cudaStream_t st, LaunchCounter& lc) {
    compact_kernel<<<grid_for(std::max(n, 1), 256), 256, 0, st>>>(S, D, keep, dst, n, n_cap, with_hist ? 1 : 0, with_brk ? 1 : 0);
    lc.add(1);
}
void launch_stats(const DevParams& P, const DevState& S, const FrameCtl* ctl, double* out, int n_cap, cudaStream_t st,
                  LaunchCounter& lc) {
    cudaMemsetAsync(out, 0, 10 * sizeof(double), st);
    stats_pass1_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(P, S, ctl, out);
    stats_pass2_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(P, S, ctl, out);
    lc.add(2);
}

}  // namespace geon
