// push.cuh — launchers of the per-particle substep and frame kernels (push.cu).
#pragma once

#include "state.cuh"

namespace geon {

struct PushFlags {
    int has1PN;          // save force1PN before the kick (integrator.js:890-893)
    int needBoris;       // magnetic || gravitomagnetic || external Bz
    int needSpinOrbit;   // spinOrbitEnabled && (magnetic || gravitomagnetic)
    int needTorques;     // (gravitomagnetic && relativity) || gravity
};

void launch_frame_scan(const DevParams& P, const DevState& S, FrameCtl* ctl, int n_cap, cudaStream_t st, LaunchCounter& lc);
// sys_dt (batched handles): per-system substep; particles of systems with
// dt <= 0 are left alone.  Null: every particle advances by dtSub.
void launch_push(const DevParams& P, const DevState& S, const FrameCtl* ctl, float dtSub, const PushFlags& F,
                 int n_cap, cudaStream_t st, LaunchCounter& lc, const double* sys_dt = nullptr);
void launch_vv_kick(const DevParams& P, const DevState& S, const FrameCtl* ctl, float halfDt, int n_cap,
                    cudaStream_t st, LaunchCounter& lc);
void launch_hist_tables(const double* hist_t, double simTime, float* age, float* segdt, cudaStream_t st, LaunchCounter& lc);
void launch_record_history(const DevState& S, const FrameCtl* ctl, double* hist_t, int slot, double simTime,
                           int n_cap, cudaStream_t st, LaunchCounter& lc);
void launch_boundary(const DevParams& P, const DevState& S, FrameCtl* ctl, int* keep, int n_cap, cudaStream_t st,
                     LaunchCounter& lc);
void launch_compact(const DevState& S, const DevState& D, const int* keep, const int* dst, int n, int n_cap,
                    bool with_hist, bool with_brk, cudaStream_t st, LaunchCounter& lc);
void launch_stats(const DevParams& P, const DevState& S, const FrameCtl* ctl, double* out, int n_cap, cudaStream_t st,
                  LaunchCounter& lc);

}  // namespace geon
