// batch.cu — planner, reductions and target lists of batched handles.
#include "batch.cuh"

namespace geon {

static inline int grid_for(int n, int threads) {
    const int b = (n + threads - 1) / threads;
    return b < 1 ? 1 : (b > device_sms() * 16 ? device_sms() * 16 : b);
}
__device__ __forceinline__ bool on(const DevParams& P, uint32_t bit) { return (P.toggles & bit) != 0; }

// ---- frame start ---------------------------------------------------------------------
__global__ void batch_clear_kernel(BatchDev B) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < B.nsys; s += gridDim.x * blockDim.x) {
        B.sys_accel[s] = 0ull;
        B.sys_cyc[s] = 0ull;
    }
}

// Per-system maxima of |F|^2/m^2 and of the cyclotron frequency over the
// forces in place (the scan of integrator.js:813-836, per system).  Particles
// are stored system by system, so a warp usually spans one system and
// reduces in registers first.
__global__ void batch_scan_kernel(DevParams P, DevState S, BatchDev B, int n) {
    const int stride = gridDim.x * blockDim.x;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int iters = (n + stride - 1) / stride;
    for (int it = 0; it < iters; it++) {
        const int i = i0 + it * stride;
        double aSq = 0.0, wc = 0.0;
        int sys = -1;
        if (i < n) {
            sys = S.sys[i];
            const float4 f = S.force[i];
            const double im = (double)S.spin[i].w;
            aSq = ((double)f.x * f.x + (double)f.y * f.y) * im * im;
            if (on(P, GEON_MAGNETIC) || P.extBz != 0.f) {
                const double absBz = fabs((double)f.z);
                if (absBz > 0) wc = fmax(wc, fabs((double)S.pos[i].w) * absBz * im);
            }
            if (on(P, GEON_GRAVITOMAG)) {
                const double absBgz = fabs((double)f.w);
                if (absBgz > 0) wc = fmax(wc, 4.0 * absBgz);
            }
            if (!(aSq == aSq)) aSq = 0.0;
            if (!(wc == wc)) wc = 0.0;
        }
        const int s0 = __shfl_sync(0xffffffffu, sys, 0);
        const bool uniform = __all_sync(0xffffffffu, sys == s0);
        if (uniform) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                aSq = fmax(aSq, __shfl_xor_sync(0xffffffffu, aSq, o));
                wc = fmax(wc, __shfl_xor_sync(0xffffffffu, wc, o));
            }
            if ((threadIdx.x & 31) == 0 && s0 >= 0) {
                atomic_max_pos_double(&B.sys_accel[s0], aSq);
                atomic_max_pos_double(&B.sys_cyc[s0], wc);
            }
        } else if (sys >= 0) {
            atomic_max_pos_double(&B.sys_accel[sys], aSq);
            atomic_max_pos_double(&B.sys_cyc[sys], wc);
        }
    }
}

__global__ void batch_init_kernel(BatchDev B) {
    const double dt = *B.frame_dt;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < B.nsys; s += gridDim.x * blockDim.x) {
        SysPlan q = B.plan[s];
        q.dtRemain = dt;
        q.curAccel = __longlong_as_double((long long)B.sys_accel[s]);
        q.curCyc = __longlong_as_double((long long)B.sys_cyc[s]);
        q.lastKick = 0.0;
        q.steps = 0;
        q.pending = 0;
        B.plan[s] = q;
        B.sys_dt[s] = 0.0;
    }
}

// ---- planning step (integrator.js:810-875, one thread per system) -------------------------
// One block: the "any system continues" decision is a block-wide OR.
__global__ void batch_plan_kernel(BatchDev B, double softening, int maxSub, unsigned long long cond) {
    const double EPS = 1e-12;
    int act_any = 0;
    for (int s = threadIdx.x; s < B.nsys; s += blockDim.x) {
        SysPlan q = B.plan[s];
        if (q.pending) {                       // forces of the substep just run (integrator.js:1336-1348)
            q.curAccel = __longlong_as_double((long long)B.sys_accel[s]);
            q.curCyc = __longlong_as_double((long long)B.sys_cyc[s]);
            q.pending = 0;
        }
        double dtSub = 0.0;
        if (q.dtRemain > EPS && q.steps < maxSub) {
            const double useAccel = q.steps == 0 ? q.curAccel : q.lastKick;
            double aMax = sqrt(useAccel);
            if (aMax != aMax) aMax = 0;
            double dtSafe = aMax > EPS ? sqrt(softening / aMax) : q.dtRemain;
            if (q.curCyc > 0) {
                const double dtCyc = 0.7853981633974483 / q.curCyc;
                if (dtCyc < dtSafe) dtSafe = dtCyc;
            }
            const double need = ceil(q.dtRemain / dtSafe);
            const double stepsNeeded = fmin(need, (double)(maxSub - q.steps));
            dtSub = q.dtRemain / stepsNeeded;
            q.steps++;
            q.dtRemain -= dtSub;
            q.lastKick = q.curAccel;
            q.simTime += dtSub;
            q.pending = 1;
            B.sys_accel[s] = 0ull;
            B.sys_cyc[s] = 0ull;
            act_any = 1;
        }
        B.sys_dt[s] = dtSub;
        B.plan[s] = q;
    }
    act_any = __syncthreads_or(act_any);
    if (threadIdx.x == 0) {
        *B.any_active = act_any;
        if (cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, act_any ? 1u : 0u);
    }
}

// ---- warp-aligned walk order ----------------------------------------------------------------
// T.tgt lists the particles in key order, which is system by system; slot
// pad_off[s] + r of the padded list gets the r-th target of system s.
__global__ void batch_targets_kernel(DevState S, TreeBufs T, FrameCtl* ctl, BatchDev B, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = T.tgt[k];
        if (i < 0 || i >= n) { atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
        const int s = S.sys[i];
        const int r = k - B.sys_off[s];
        if (s < 0 || s >= B.nsys || r < 0 || r >= B.sys_off[s + 1] - B.sys_off[s]) {
            atomicOr(&ctl->err, ERR_BAD_INDEX);
            continue;
        }
        B.tgt_pad[B.pad_off[s] + r] = i;
    }
}

// ---- launchers ------------------------------------------------------------------------------
void batch_frame_start(const DevParams& P, const DevState& S, const BatchDev& B, int n, cudaStream_t st,
                       LaunchCounter& lc) {
    batch_clear_kernel<<<(B.nsys + 255) / 256, 256, 0, st>>>(B);
    batch_scan_kernel<<<grid_for(std::max(n, 1), 256), 256, 0, st>>>(P, S, B, n);
    batch_init_kernel<<<(B.nsys + 255) / 256, 256, 0, st>>>(B);
    lc.add(3);
}

void batch_plan(const DevParams& P, const BatchDev& B, double softening, int max_substeps,
                unsigned long long cond, cudaStream_t st, LaunchCounter& lc) {
    (void)P;
    batch_plan_kernel<<<1, 512, 0, st>>>(B, softening, max_substeps, cond);
    lc.add(1);
}

void batch_targets(const DevState& S, const TreeBufs& T, FrameCtl* ctl, const BatchDev& B, int n, cudaStream_t st,
                   LaunchCounter& lc) {
    batch_targets_kernel<<<grid_for(std::max(n, 1), 256), 256, 0, st>>>(S, T, ctl, B, n);
    lc.add(1);
}

}  // namespace geon
