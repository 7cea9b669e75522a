// frame.cu — one frame of a small open system (no periodic ghosts, at most
// FRAME_MAX_POINTS particles) in a single cooperative launch.
//
// Physics.update (src/integrator.js:726-1825), the part geon_update runs,
// with every phase a body shared with the separate-launch path:
//   frame-start planner scan       integrator.js:813-836    scan_forces_body (push_dev.cuh)
//   substep planner (lagged aMax)  integrator.js:810-875    frame_kernel below, in FP64 on every thread
//   Boris kick / rotate / drift    integrator.js:884-982, 1269-1278   push_body
//   tree build                     quadtree.js:98-318       tree_dev.cuh bodies; the sort ranks keys here
//   force recompute (BH walk)      forces.js:622-694        walkc_body (walk_dev.cuh)
//   signal-delay tables            signal-delay.js:16-221   hist_tables_body
//   history sample                 integrator.js:1549-1565  record_history_body
//   boundary + compaction          integrator.js:1798-1824  boundary_body, compact_body
//
// The planner runs redundantly on every thread from the same device values
// (the maxima the walk leaves), so every block takes the same substeps and
// nothing goes back to the host until the frame is over.  Phases are
// separated by a grid-wide barrier whose wait is bounded in time: a block
// that gives up raises ERR_FRAME_TIMEOUT and the abort flag, and every block
// returns.  The cooperative launch guarantees that all blocks are resident.
#include "walk_dev.cuh"
#include "tree_dev.cuh"
#include "push_dev.cuh"
#include "frame.cuh"

namespace geon {

constexpr int FR_THREADS = WC_THREADS;   // one walk CTA (four target groups of 32) per block and pass

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier over `expect` arrivals.  The last block to arrive resets
// the count and advances the generation; the others poll the generation until
// it moves, the abort flag is set or waitNs nanoseconds (or 2^28 polls) pass.
// Returns false for every thread of the block when the block has to return.
__device__ __forceinline__ bool frame_barrier(FrameRun* R, unsigned expect, long long waitNs, FrameCtl* ctl, int* s_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &R->gen;
        volatile int* vabort = &R->abort;
        const unsigned g = *vgen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(&R->count, 1u) + 1u == expect) {
            atomicExch(&R->count, 0u);
            __threadfence();
            atomicAdd(&R->gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            unsigned polls = 0;
            while (*vgen == g) {
                if (*vabort) { ok = 0; break; }
                ++polls;
                if (polls > (1u << 28) || ((polls & 31u) == 0 && global_ns() - t0 > (unsigned long long)waitNs)) {
                    atomicOr(&ctl->err, ERR_FRAME_TIMEOUT);
                    atomicExch(&R->abort, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// Exclusive scan of in[0, n) into out by one CTA; *total (optional) gets the sum.
__device__ __forceinline__ void cta_excl_scan(const int* in, int* out, int n, int* total, int* s_warp) {
    const int per = (n + (int)blockDim.x - 1) / (int)blockDim.x;
    const int i0 = (int)threadIdx.x * per;
    int s = 0;
    for (int k = 0; k < per; k++) {
        const int i = i0 + k;
        if (i < n) s += __ldcg(&in[i]);
    }
    const int incl = warp_incl_scan_i(s);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    int off = 0, tot = 0;
    for (int j = 0; j < (int)(blockDim.x >> 5); j++) {
        const int v = s_warp[j];
        if (j < w) off += v;
        tot += v;
    }
    int ex = off + incl - s;
    for (int k = 0; k < per; k++) {
        const int i = i0 + k;
        if (i < n) {
            const int v = __ldcg(&in[i]);
            out[i] = ex;
            ex += v;
        }
    }
    if (threadIdx.x == 0 && total) *total = tot;
    __syncthreads();
}

// Stable sort of the n keys by rank: point p goes to slot
// #{q : key_q < key_p} + #{q < p : key_q == key_p}, the order of a stable
// radix sort of (key, p) pairs.  Every block holding points loads all keys
// into shared memory; a warp's own 32 keys are the only ones that need the
// index tie-break.
__device__ __forceinline__ void rank_sort(const uint64_t* keys, uint64_t* okeys, uint32_t* ovals, int n, int b, int G) {
    if (b * (int)blockDim.x >= n) return;                      // uniform over the block
    uint64_t* sk = reinterpret_cast<uint64_t*>(geon_dsmem);
    for (int i = threadIdx.x; i < n; i += blockDim.x) sk[i] = __ldcg(&keys[i]);
    __syncthreads();
    for (int base = b * (int)blockDim.x; base < n; base += G * (int)blockDim.x) {
        const int p = base + (int)threadIdx.x;
        const int w0 = base + (int)(threadIdx.x & ~31u);
        if (w0 >= n) continue;
        const uint64_t kp = p < n ? sk[p] : 0ull;
        int r0 = 0, r1 = 0, r2 = 0, r3 = 0;
        int q = 0;
        for (; q + 4 <= w0; q += 4) {                          // q < p: equal keys come first
            r0 += sk[q] <= kp; r1 += sk[q + 1] <= kp; r2 += sk[q + 2] <= kp; r3 += sk[q + 3] <= kp;
        }
        for (; q < w0; q++) r0 += sk[q] <= kp;
        const int w1 = min(w0 + 32, n);
        for (q = w0; q < w1; q++) {
            const uint64_t kq = sk[q];
            r0 += (kq < kp) || (kq == kp && q < p);
        }
        q = w1;
        for (; q + 4 <= n; q += 4) {                           // q > p: equal keys come after
            r0 += sk[q] < kp; r1 += sk[q + 1] < kp; r2 += sk[q + 2] < kp; r3 += sk[q + 3] < kp;
        }
        for (; q < n; q++) r0 += sk[q] < kp;
        if (p < n) {
            const int r = r0 + r1 + r2 + r3;
            okeys[r] = kp;
            ovals[r] = (uint32_t)p;
        }
    }
}

__device__ __forceinline__ double bits_double(const unsigned long long* a) {
    return __longlong_as_double((long long)__ldcg(a));
}

template <bool REL>
__global__ void __launch_bounds__(FR_THREADS, 1)
frame_kernel(DevParams P, DevState S, DevState S2, TreeBufs T, int* d_root, FrameCtl* ctl, ForceCtx C, FrameArgs A,
             FrameRun* R) {
    __shared__ int s_ok;
    __shared__ int s_warp[FR_THREADS / 32 + 1];
    const int G = gridDim.x, b = blockIdx.x;
    const unsigned expect = (unsigned)(G + A.extraArrivals);
    const bool lead = b == 0 && threadIdx.x == 0;
    const int n = __ldcg(&ctl->n);
    T.skey = T.key_alt;                                                   // the rank sort's output
    T.sidx = T.idx_alt;
    auto sync = [&]() { return frame_barrier(R, expect, A.waitNs, ctl, &s_ok); };

    // frame start: planner maxima of the current forces
    if (lead) ctl->nRemoved = 0;
    scan_forces_body(P, S, ctl, &R->scanAccel, &R->scanCyc, b, G);
    if (!sync()) return;
    double curAccel = bits_double(&R->scanAccel), curCyc = bits_double(&R->scanCyc);
    double lastKick = 0.0, dtRemain = A.dt, simTime = A.simTime;
    int total = 0;
    const double EPS = 1e-12;
    const int nWalk = (n + FR_THREADS - 1) / FR_THREADS;
    while (dtRemain > EPS && total < A.maxSub) {                          // integrator.js:810
        const double useAccel = total == 0 ? curAccel : lastKick;
        double aMax = sqrt(useAccel);
        if (aMax != aMax) aMax = 0;
        double dtSafe = aMax > EPS ? sqrt(A.softening / aMax) : dtRemain;
        if (curCyc > 0) {
            const double dtCyc = 0.7853981633974483 / curCyc;
            if (dtCyc < dtSafe) dtSafe = dtCyc;
        }
        const double need = ceil(dtRemain / dtSafe);
        const double stepsNeeded = fmin(need, (double)(A.maxSub - total));
        const double dtSub = dtRemain / stepsNeeded;
        total++;
        dtRemain -= dtSub;
        lastKick = curAccel;
        simTime += dtSub;

        // push, and the tree counters for the rebuild
        push_body(P, S, ctl, (float)dtSub, A.F, nullptr, b, G);
        if (lead) {
            tree_reset_body(ctl, 0, 1);
            ctl->nGhost = 0;
            ctl->nPts = n;
        }
        if (!sync()) return;
        // the planner maxima were read before the barrier: clear them for the walk
        if (lead) { ctl->maxAccelSqBits = 0ull; ctl->maxCycBits = 0ull; ctl->interactions = 0ull; }
        if (REL) hist_tables_body(A.hist_t, simTime, A.hist_age, A.hist_segdt, b, G);
        {                                                                 // point references and keys
            int valid = 0;
            for (int p = b * blockDim.x + threadIdx.x; p < n; p += G * blockDim.x) {
                const uint32_t ref = make_ref((uint32_t)p, CODE_IDENTITY);
                uint64_t key;
                valid += point_key(P, S, ref, p, key) ? 1 : 0;
                T.pt_ref[p] = ref;
                T.key[p] = key;
                T.idx[p] = (uint32_t)p;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) valid += __shfl_xor_sync(0xffffffffu, valid, o);
            if ((threadIdx.x & 31) == 0 && valid) atomicAdd(&ctl->nValid, valid);
        }
        if (!sync()) return;
        rank_sort(T.key, T.skey, T.sidx, n, b, G);
        if (!sync()) return;
        gather_body(P, S, T, ctl, b, G);
        if (!sync()) return;
        for (int k = b; k < 3; k += G) {
            if (k == 0) cta_excl_scan(T.int_cnt, T.int_base, n, &ctl->nInternal, s_warp);
            else if (k == 1) cta_excl_scan(T.leaf_flag, T.leaf_base, n, &ctl->nLeaves, s_warp);
            else cta_excl_scan(T.real_flag, T.tgt_base, n, nullptr, s_warp);
        }
        if (!sync()) return;
        emit_body(P, T, ctl, b, G);
        if (!sync()) return;
        link_body(P, T, ctl, d_root, b, G);
        if (!sync()) return;
        aggregate_body(P, S, T, ctl, b, G);
        if (!sync()) return;
        for (int vb = b; vb < nWalk; vb += G) {                              // forces.js:622-694
            walkc_body<false, REL, false, false, true, false>(P, S, T, d_root, ctl, C, vb);
            __syncthreads();
        }
        if (!sync()) return;
        curAccel = bits_double(&ctl->maxAccelSqBits);
        curCyc = bits_double(&ctl->maxCycBits);
    }

    // frame end: history sample (before the boundary moves anything), boundary
    if (A.recordHist) record_history_body(S, ctl, A.hist_t, A.histSlot, simTime, b, G);
    boundary_body(P, S, ctl, A.keep, b, G);
    if (!sync()) return;
    const int removed = __ldcg(&ctl->nRemoved);
    if (removed > 0) {
        if (b == 0) cta_excl_scan(A.keep, A.dst, n, nullptr, s_warp);
        if (!sync()) return;
        compact_body(S, S2, A.keep, A.dst, n, A.slots, A.withHist, 1, b, G);
        if (lead) ctl->n = n - removed;
    }
    if (lead) {
        R->substeps = total;
        R->simTime = simTime;
        R->removed = removed;
        R->scanAccel = 0ull;
        R->scanCyc = 0ull;
    }
}

int frame_blocks(int n) {
    return std::max(1, std::min((n + FR_THREADS - 1) / FR_THREADS, FRAME_MAX_POINTS / FR_THREADS));
}

template <bool REL>
static cudaError_t launch_frame_t(const DevParams& P, const DevState& S, const DevState& S2, const TreeBufs& T,
                                  int* d_root, FrameCtl* ctl, const ForceCtx& C, const FrameArgs& A, FrameRun* run,
                                  int n, cudaStream_t st, LaunchCounter& lc) {
    constexpr size_t walk_smem = wc_smem_bytes<false, REL, false, false, true>();
    constexpr size_t sort_smem = (size_t)FRAME_MAX_POINTS * sizeof(uint64_t);
    constexpr size_t smem = walk_smem > sort_smem ? walk_smem : sort_smem;
    static_assert(smem <= 200 * 1024, "frame kernel shared memory");
    static int attr_dev = -1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (attr_dev != dev) {
        cudaError_t e = cudaFuncSetAttribute(frame_kernel<REL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_dev = dev;
    }
    const int G = frame_blocks(n);
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, frame_kernel<REL>, FR_THREADS, smem);
    if (e != cudaSuccess) return e;
    if ((long long)per_sm * device_sms() < G) return cudaErrorCooperativeLaunchTooLarge;
    DevParams p = P;
    DevState s = S, s2 = S2;
    TreeBufs t = T;
    ForceCtx c = C;
    FrameArgs a = A;
    void* args[] = { &p, &s, &s2, &t, &d_root, &ctl, &c, &a, &run };
    e = cudaLaunchCooperativeKernel((const void*)frame_kernel<REL>, dim3(G), dim3(FR_THREADS), args, smem, st);
    lc.add(1);
    return e;
}

cudaError_t frame_launch(bool rel, const DevParams& P, const DevState& S, const DevState& S2, const TreeBufs& T,
                         int* d_root, FrameCtl* ctl, const ForceCtx& C, const FrameArgs& A, FrameRun* run, int n,
                         cudaStream_t st, LaunchCounter& lc) {
    if (!frame_fits(n)) return cudaErrorInvalidValue;
    return rel ? launch_frame_t<true>(P, S, S2, T, d_root, ctl, C, A, run, n, st, lc)
               : launch_frame_t<false>(P, S, S2, T, d_root, ctl, C, A, run, n, st, lc);
}

}  // namespace geon
