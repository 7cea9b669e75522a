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

constexpr int FR_THREADS = 2 * WC_THREADS;   // one block per group of 32 targets: its eight warps share the walk

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier over `expect` arrivals.  A block arrives with an
// acquire-release addition to the count; the last one resets the count and
// publishes the next generation with a release addition; the others poll the
// generation (tightly at first, then with short sleeps) until it moves, the
// abort flag is set or waitNs nanoseconds (or 2^28 polls) pass.  Returns
// false for every thread of the block when the block has to return.
__device__ __forceinline__ bool frame_barrier(FrameRun* R, unsigned expect, long long waitNs, FrameCtl* ctl, int* s_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned g, arrived;
        asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(&R->gen) : "memory");
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(arrived) : "l"(&R->count) : "memory");
        int ok = 1;
        if (arrived + 1u == expect) {
            asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" :: "l"(&R->count) : "memory");
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" :: "l"(&R->gen) : "memory");
        } else {
            const unsigned long long t0 = global_ns();
            unsigned polls = 0;
            for (;;) {
                unsigned cur;
                int ab;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(&R->gen) : "memory");
                if (cur != g) break;
                asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(ab) : "l"(&R->abort) : "memory");
                if (ab) { ok = 0; break; }
                ++polls;
                if (polls > (1u << 28) || ((polls & 31u) == 0 && global_ns() - t0 > (unsigned long long)waitNs)) {
                    atomicOr(&ctl->err, ERR_FRAME_TIMEOUT);
                    atomicExch(&R->abort, 1);
                    ok = 0;
                    break;
                }
                if (polls > 256) __nanosleep(32);
            }
        }
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

constexpr int FR_SCAN_ITEMS = FRAME_MAX_POINTS / FR_THREADS;   // items per thread of a one-block scan
static_assert(FR_SCAN_ITEMS * FR_THREADS >= FRAME_MAX_POINTS, "one-block scan covers the largest system");

// Exclusive scan of in[0, n) (n <= FRAME_MAX_POINTS) into out by one CTA of
// FR_THREADS threads, each holding a contiguous run of items in registers;
// *total (optional) gets the sum.
__device__ __forceinline__ void cta_excl_scan(const int* in, int* out, int n, int* total, int* s_warp) {
    const int per = (n + FR_THREADS - 1) / FR_THREADS;
    const int i0 = (int)threadIdx.x * per;
    int v[FR_SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < FR_SCAN_ITEMS; k++) {
        const int i = i0 + k;
        v[k] = (k < per && i < n) ? __ldcg(&in[i]) : 0;
        s += v[k];
    }
    const int incl = warp_incl_scan_i(s);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    int off = 0, tot = 0;
#pragma unroll
    for (int j = 0; j < FR_THREADS / 32; j++) {
        const int x = s_warp[j];
        if (j < w) off += x;
        tot += x;
    }
    int ex = off + incl - s;
#pragma unroll
    for (int k = 0; k < FR_SCAN_ITEMS; k++) {
        const int i = i0 + k;
        if (k < per && i < n) out[i] = ex;
        ex += v[k];
    }
    if (threadIdx.x == 0 && total) *total = tot;
    __syncthreads();
}

// #{q in [lo, hi) : sk[q] <= kp} (LE) or #{... : sk[q] < kp}, two keys per shared-memory load.
template <bool LE>
__device__ __forceinline__ int count_below(const uint64_t* sk, int lo, int hi, uint64_t kp) {
    int r0 = 0, r1 = 0, r2 = 0, r3 = 0;
    int q = lo;
    if ((q & 1) && q < hi) { r0 += LE ? sk[q] <= kp : sk[q] < kp; q++; }
    const ulonglong2* s2 = reinterpret_cast<const ulonglong2*>(sk);
    for (; q + 4 <= hi; q += 4) {
        const ulonglong2 a = s2[q >> 1], c = s2[(q >> 1) + 1];
        if (LE) { r0 += a.x <= kp; r1 += a.y <= kp; r2 += c.x <= kp; r3 += c.y <= kp; }
        else    { r0 += a.x < kp;  r1 += a.y < kp;  r2 += c.x < kp;  r3 += c.y < kp; }
    }
    for (; q < hi; q++) r0 += LE ? sk[q] <= kp : sk[q] < kp;
    return r0 + r1 + r2 + r3;
}

// Stable sort of the n keys by rank: point p goes to slot
// #{q : key_q < key_p} + #{q < p : key_q == key_p}, the order of a stable
// radix sort of (key, p) pairs.  Chunks of 32 keys go to the blocks in turn;
// a block's warps rank the chunk against an equal share of all keys each
// (held in shared memory) and warp 0 adds their counts.
__device__ __forceinline__ void rank_sort(const uint64_t* keys, uint64_t* okeys, uint32_t* ovals, int n, int b, int G,
                                          int (*s_part)[32]) {
    const int nch = (n + 31) / 32;
    if (b >= nch) return;                                      // uniform over the block
    uint64_t* sk = reinterpret_cast<uint64_t*>(geon_dsmem);
    for (int i = threadIdx.x; i < n; i += blockDim.x) sk[i] = __ldcg(&keys[i]);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int per = (((n + nw - 1) / nw) + 1) & ~1;            // even: the pair loads stay aligned
    const int qa = min(n, warp * per), qb = min(n, qa + per);
    for (int c = b; c < nch; c += G) {
        const int w0 = c * 32, w1 = min(w0 + 32, n);
        const int p = w0 + lane;
        const uint64_t kp = p < n ? sk[p] : 0ull;
        int r = count_below<true>(sk, qa, min(qb, w0), kp);            // before the chunk: ties come first
        for (int q = max(qa, w0); q < min(qb, w1); q++) {              // the chunk itself
            const uint64_t kq = sk[q];
            r += (kq < kp) || (kq == kp && q < p);
        }
        r += count_below<false>(sk, max(qa, w1), qb, kp);              // after it: ties come after
        s_part[warp][lane] = r;
        __syncthreads();
        if (warp == 0 && p < n) {
            int rr = 0;
            for (int w = 0; w < nw; w++) rr += s_part[w][lane];
            okeys[rr] = kp;
            ovals[rr] = (uint32_t)p;
        }
        __syncthreads();
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
    __shared__ int s_part[FR_THREADS / 32][32];
    const int G = gridDim.x, b = blockIdx.x;
    const unsigned expect = (unsigned)(G + A.extraArrivals);
    const bool lead = b == 0 && threadIdx.x == 0;
    const int n = __ldcg(&ctl->n);
    T.skey = T.key_alt;                                                   // the rank sort's output
    T.sidx = T.idx_alt;
    auto sync = [&]() { return frame_barrier(R, expect, A.waitNs, ctl, &s_ok); };
    auto mark = [&](int i) { if (lead) R->stamp[i] = global_ns(); };
    if (lead)
        for (int i = 1; i < FRAME_STAMPS; i++) R->stamp[i] = 0ull;         // phases this frame does not reach stay 0
    mark(0);

    // frame start: planner maxima of the current forces
    if (lead) { ctl->nRemoved = 0; R->valid[1] = 0; }
    scan_forces_body(P, S, ctl, &R->scanAccel, &R->scanCyc, b, G);
    if (!sync()) return;
    mark(1);
    double curAccel = bits_double(&R->scanAccel), curCyc = bits_double(&R->scanCyc);
    double lastKick = 0.0, dtRemain = A.dt, simTime = A.simTime;
    int total = 0;
    const double EPS = 1e-12;
    const int nGroups = (n + 31) / 32;
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

        // push, then each particle's reference and key by the thread that
        // pushed it (same index, so no barrier between them)
        push_body(P, S, ctl, (float)dtSub, A.F, nullptr, b, G);
        {
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
            if ((threadIdx.x & 31) == 0 && valid) atomicAdd(&R->valid[total & 1], valid);
        }
        if (lead) {                                                       // tree counters of this rebuild
            R->valid[(total + 1) & 1] = 0;
            ctl->nBucket = 0;
            ctl->maxLevel = 0;
            ctl->nGhost = 0;
            ctl->nPts = n;
        }
        if (!sync()) return;
        if (total == 1) mark(2);
        // every thread read the planner maxima before the barrier: clear them for the walk
        if (lead) {
            ctl->nValid = __ldcg(&R->valid[total & 1]);
            ctl->maxAccelSqBits = 0ull;
            ctl->maxCycBits = 0ull;
            ctl->interactions = 0ull;
        }
        if (REL) hist_tables_body(A.hist_t, simTime, A.hist_age, A.hist_segdt, b, G);
        rank_sort(T.key, T.skey, T.sidx, n, b, G, s_part);
        if (!sync()) return;
        if (total == 1) mark(3);
        // the sorted keys in shared memory for gather, emit and link (read-only there)
        TreeBufs Ts = T;
        {
            uint64_t* ks = reinterpret_cast<uint64_t*>(geon_dsmem);
            for (int i = threadIdx.x; i < n; i += blockDim.x) ks[i] = __ldcg(&T.skey[i]);
            __syncthreads();
            Ts.skey = ks;
        }
        gather_body(P, S, Ts, ctl, b, G);
        if (!sync()) return;
        if (total == 1) mark(4);
        for (int k = b; k < 3; k += G) {
            if (k == 0) cta_excl_scan(T.int_cnt, T.int_base, n, &ctl->nInternal, s_warp);
            else if (k == 1) cta_excl_scan(T.leaf_flag, T.leaf_base, n, &ctl->nLeaves, s_warp);
            else cta_excl_scan(T.real_flag, T.tgt_base, n, nullptr, s_warp);
        }
        if (!sync()) return;
        if (total == 1) mark(5);
        emit_body(P, Ts, ctl, b, G);
        if (!sync()) return;
        if (total == 1) mark(6);
        link_body(P, Ts, ctl, d_root, b, G);
        if (!sync()) return;
        if (total == 1) mark(7);
        aggregate_body(P, S, T, ctl, b, G);
        if (!sync()) return;
        if (total == 1) mark(8);
        for (int vb = b; vb < nGroups; vb += G) {                            // forces.js:622-694
            walkc_body<false, REL, false, false, true, false, FR_THREADS / 32>(P, S, T, d_root, ctl, C, vb);
            __syncthreads();
        }
        if (!sync()) return;
        if (total == 1) mark(9);
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
    mark(FRAME_STAMPS - 1);
    if (lead) {
        R->substeps = total;
        R->simTime = simTime;
        R->removed = removed;
        R->scanAccel = 0ull;
        R->scanCyc = 0ull;
    }
}

// One block per group of 32 targets: the walk's eight warps share a group.
int frame_blocks(int n) {
    return std::max(1, std::min((n + 31) / 32, FRAME_MAX_POINTS / 32));
}

template <bool REL>
static cudaError_t launch_frame_t(const DevParams& P, const DevState& S, const DevState& S2, const TreeBufs& T,
                                  int* d_root, FrameCtl* ctl, const ForceCtx& C, const FrameArgs& A, FrameRun* run,
                                  int n, cudaStream_t st, LaunchCounter& lc) {
    constexpr size_t walk_smem = wc_smem_bytes<false, REL, false, false, true, FR_THREADS / 32>();
    constexpr size_t sort_smem = (size_t)FRAME_MAX_POINTS * sizeof(uint64_t);
    constexpr size_t smem = walk_smem > sort_smem ? walk_smem : sort_smem;
    static_assert(smem <= 200 * 1024, "frame kernel shared memory");
    // per device: the shared-memory attribute and the resident blocks it allows
    static int attr_dev = -1, per_sm = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if (attr_dev != dev) {
        cudaError_t e = cudaFuncSetAttribute(frame_kernel<REL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, frame_kernel<REL>, FR_THREADS, smem);
        if (e != cudaSuccess) return e;
        attr_dev = dev;
    }
    const int G = frame_blocks(n);
    if ((long long)per_sm * device_sms() < G) return cudaErrorCooperativeLaunchTooLarge;
    cudaError_t e;
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
