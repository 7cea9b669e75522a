// force.cu — pairwise force accumulation: Barnes-Hut walk, O(N^2) pairwise
// sum, and the 1PN-only passes used by the velocity-Verlet correction.
//
// Physics restated from the reference CPU path:
//   pairForce          src/forces.js:163-442
//   computeAllForces   src/forces.js:61-154 (moment caching :71-76, Yukawa
//                      cutoff :82-83, pairwise loop :94-125)
//   calculateForce     src/forces.js:622-694 (BH walk)
//   _accum1PN / _compute1PNTreeWalk / compute1PN   src/forces.js:445-610
//   getDelayedState    src/signal-delay.js:16-221
//   external fields    src/integrator.js:563-593
//   bounce walls       src/integrator.js:607-668
//
// Arithmetic is FP32.  Per-particle sums use partial sums flushed every 16
// terms into compensated (hi, lo) accumulators.  Decisions that switch terms
// on or off -- the opening test size^2 < theta^2 d^2 and the Yukawa cutoff
// r^2 < (6/mu)^2 -- are re-evaluated in FP64 from the exact inputs when the
// FP32 margin is within rounding, so the set of interactions matches the
// FP64 reference.
//
// Walk: one warp per 32 particles taken in Morton order.  The warp shares a
// stack of (node, lane mask) entries in shared memory; each lane applies its
// own opening test and a ballot splits the mask into lanes that accept the
// aggregate and lanes that descend, so every particle sees exactly the
// interaction list of the reference's per-particle walk while node records
// are fetched once per warp.
#include "walk_dev.cuh"

namespace geon {

// Shared memory of a walk launch: the kernel's own, or padded so that at most
// C.walk_ctas CTAs fit an SM (228 KB of shared memory, 1 KB reserved per CTA).
constexpr size_t WC_SMEM_LIMIT = 227 * 1024;
static size_t walk_dyn_smem(size_t smem, const ForceCtx& C) {
    if (C.walk_ctas <= 0) return smem;
    const size_t per = (size_t)228 * 1024 / (size_t)C.walk_ctas;
    const size_t want = per > 1024 ? per - 1024 : smem;
    return std::min(std::max(smem, want), WC_SMEM_LIMIT);
}

template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE = false, bool EMIT = false, bool YUK = true>
static void launch_walkc(int blocks, const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root,
                         FrameCtl* ctl, const ForceCtx& C, cudaStream_t st) {
    constexpr size_t smem = wc_smem_bytes<MAGGM, REL, BRK, PER, NOPE>();
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(walkc_kernel<MAGGM, REL, BRK, PER, NOPE, EMIT, YUK>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WC_SMEM_LIMIT);
        attr = true;
    }
    walkc_kernel<MAGGM, REL, BRK, PER, NOPE, EMIT, YUK><<<blocks, WC_THREADS, walk_dyn_smem(smem, C), st>>>(
        P, S, T, d_root, ctl, C);
}

// The split walk: one CTA per group of 32 targets, its four warps sharing the
// group's subtrees (walkc_body with SPLIT = WC_WARPS).
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool YUK = true>
__global__ void __launch_bounds__(WC_THREADS, wc_min_blocks<MAGGM, REL, BRK, PER, NOPE>())
walkc_split_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root, FrameCtl* ctl, ForceCtx C) {
    walkc_body<MAGGM, REL, BRK, PER, NOPE, false, WC_WARPS, WC_STACK, YUK>(P, S, T, d_root, ctl, C, blockIdx.x);
}

// The short-stack walk (a batched walk shape): a 288-entry stack takes the
// plain walk's shared memory to 31 KB per CTA and its registers to 72, so
// seven CTAs fit an SM instead of six.  Only shallow walks gain: at small
// opening angles the stack runs deep and the walk falls back to single pops.
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool YUK = true>
__global__ void __launch_bounds__(WC_THREADS, 7)
walkc_short_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root, FrameCtl* ctl, ForceCtx C) {
    walkc_body<MAGGM, REL, BRK, PER, NOPE, false, 1, WC_STACK_SHORT, YUK>(P, S, T, d_root, ctl, C, blockIdx.x);
}

template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool YUK = true>
static void launch_walkc_short(int blocks, const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root,
                               FrameCtl* ctl, const ForceCtx& C, cudaStream_t st) {
    constexpr size_t smem = wc_smem_bytes<MAGGM, REL, BRK, PER, NOPE, WC_WARPS, WC_STACK_SHORT>();
    walkc_short_kernel<MAGGM, REL, BRK, PER, NOPE, YUK><<<blocks, WC_THREADS, smem, st>>>(P, S, T, d_root, ctl, C);
}

// The grouped walk from a work queue: persistent CTAs take walk blocks (four
// groups of 32 targets each) C.walk_chunk at a time from C.walk_queue[0];
// C.walk_queue[1] counts the CTAs that are done.  Both are zero before a
// launch and after it.  Every group's walk is the same code on the same data
// whichever CTA runs it, so the results do not depend on the order.
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool YUK = true>
__global__ void __launch_bounds__(WC_THREADS, wc_min_blocks<MAGGM, REL, BRK, PER, NOPE>())
walkc_queue_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root, FrameCtl* ctl, ForceCtx C,
                   int nblocks) {
    __shared__ int s_base;
    for (;;) {
        if (threadIdx.x == 0) s_base = (int)atomicAdd(C.walk_queue, (unsigned)C.walk_chunk);
        __syncthreads();
        const int base = s_base;
        __syncthreads();                                   // all have read it before thread 0 takes the next
        if (base >= nblocks) break;
        const int end = min(base + C.walk_chunk, nblocks);
        for (int vb = base; vb < end; vb++) {
            walkc_body<MAGGM, REL, BRK, PER, NOPE, false, 1, WC_STACK, YUK>(P, S, T, d_root, ctl, C, vb);
            __syncthreads();
        }
    }
    // the last CTA out leaves both counters at zero for the next launch (no
    // other CTA takes blocks any more)
    if (threadIdx.x == 0 && atomicAdd(C.walk_queue + 1, 1u) + 1u == gridDim.x) {
        atomicExch(C.walk_queue, 0u);
        atomicExch(C.walk_queue + 1, 0u);
    }
}

// Resident CTAs per SM of the work-queue walk, looked up once per device.
// The lookup is not a stream operation: walk_queue_setup() makes it outside
// any graph capture (geon_batch_set_shape calls it).
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool YUK>
static int& walk_queue_per_sm(int dev) {
    static int cache[64] = { 0 };
    return cache[dev >= 0 && dev < 64 ? dev : 0];
}

template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool YUK>
static int walk_queue_prepare() {
    int dev = 0;
    cudaGetDevice(&dev);
    int& per_sm = walk_queue_per_sm<MAGGM, REL, BRK, PER, NOPE, YUK>(dev);
    if (per_sm <= 0) {
        constexpr size_t smem = wc_smem_bytes<MAGGM, REL, BRK, PER, NOPE>();
        cudaFuncSetAttribute(walkc_queue_kernel<MAGGM, REL, BRK, PER, NOPE, YUK>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, walkc_queue_kernel<MAGGM, REL, BRK, PER, NOPE, YUK>, WC_THREADS,
                                                      smem);
        per_sm = std::max(v, 1);
    }
    return per_sm;
}

void walk_queue_setup() {
    walk_queue_prepare<false, false, false, 2, true, true>();
    walk_queue_prepare<false, false, false, 2, true, false>();
}

template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool YUK = true>
static void launch_walkc_queue(int blocks, const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root,
                               FrameCtl* ctl, const ForceCtx& C, cudaStream_t st) {
    constexpr size_t smem = wc_smem_bytes<MAGGM, REL, BRK, PER, NOPE>();
    const int per_sm = walk_queue_prepare<MAGGM, REL, BRK, PER, NOPE, YUK>();
    const int grid = std::max(1, std::min(blocks, per_sm * device_sms()));
    walkc_queue_kernel<MAGGM, REL, BRK, PER, NOPE, YUK><<<grid, WC_THREADS, smem, st>>>(P, S, T, d_root, ctl, C, blocks);
}

template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool YUK = true>
static void launch_walkc_split(int slots, const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root,
                               FrameCtl* ctl, const ForceCtx& C, cudaStream_t st) {
    constexpr size_t smem = wc_smem_bytes<MAGGM, REL, BRK, PER, NOPE>();
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(walkc_split_kernel<MAGGM, REL, BRK, PER, NOPE, YUK>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WC_SMEM_LIMIT);
        attr = true;
    }
    const int blocks = std::max(1, (slots + 31) / 32);
    walkc_split_kernel<MAGGM, REL, BRK, PER, NOPE, YUK><<<blocks, WC_THREADS, walk_dyn_smem(smem, C), st>>>(
        P, S, T, d_root, ctl, C);
}

// The plain torus walk without energy sums in the shape the batch chose:
// four warps per group, a work queue, the short stack, or one warp per group.
template <bool YUK>
static void launch_lean_torus(int slots, int blocks, const DevParams& P, const DevState& S, const TreeBufs& T,
                              const int* d_root, FrameCtl* ctl, const ForceCtx& C, cudaStream_t st) {
    if (C.walk_split) launch_walkc_split<false, false, false, 2, true, YUK>(slots, P, S, T, d_root, ctl, C, st);
    else if (C.walk_chunk > 0 && C.walk_queue) launch_walkc_queue<false, false, false, 2, true, YUK>(blocks, P, S, T, d_root, ctl, C, st);
    else if (C.walk_ctas == 7) launch_walkc_short<false, false, false, 2, true, YUK>(blocks, P, S, T, d_root, ctl, C, st);
    else launch_walkc<false, false, false, 2, true, false, YUK>(blocks, P, S, T, d_root, ctl, C, st);
}

// ---- pairwise O(N^2) sum (forces.js:94-125) -------------------------------------------------
constexpr int DIRECT_THREADS = 256;

// Partial sums of one source slice: hi and lo of every accumulated quantity,
// then the interaction count, each a row of (gridDim.x * DIRECT_THREADS) floats.
template <bool MAGGM, bool BRK>
__host__ __device__ constexpr int direct_part_rows() { return 2 * Acc<MAGGM, BRK>::NQ + 1; }

// blockIdx.y selects a slice of the source tiles (gridDim.y slices).  With
// one slice the kernel finishes each target itself; with more it writes the
// slice's partial sums to C.dpart and direct_combine_kernel finishes.
template <bool MAGGM, bool REL, bool BRK>
__global__ void __launch_bounds__(DIRECT_THREADS, (MAGGM || REL || BRK) ? 2 : 3)
direct_kernel(DevParams P, DevState S, FrameCtl* ctl, ForceCtx C) {
    __shared__ float4 s_pos[DIRECT_THREADS];
    __shared__ float4 s_vel[DIRECT_THREADS];   // vx, vy, angVel, radius^2
    __shared__ float2 s_lo[DIRECT_THREADS];
    __shared__ float s_age[REL ? HIST_LEN : 1], s_segdt[REL ? HIST_LEN : 1];
    if (REL) load_hist_tables(C, s_age, s_segdt);
    const int n = ctl->n;
    const int i = blockIdx.x * DIRECT_THREADS + threadIdx.x;
    const bool valid = i < n;
    Tgt t;
    if (valid) { t = load_target(S, i); target_coupling(P, t); }
    else { t = Tgt{}; t.idx = -1; }
    Acc<MAGGM, BRK> A;
    A.init();
    unsigned inter = 0;
    const bool pe = C.pe != 0;
    const int ntile = (n + DIRECT_THREADS - 1) / DIRECT_THREADS;
    const int tile0 = (int)((long long)ntile * blockIdx.y / gridDim.y);
    const int tile1 = (int)((long long)ntile * (blockIdx.y + 1) / gridDim.y);
    for (int base = tile0 * DIRECT_THREADS; base < tile1 * DIRECT_THREADS; base += DIRECT_THREADS) {
        const int j = base + threadIdx.x;
        __syncthreads();
        if (j < n) {
            const float4 sv = S.vel[j], ss = S.spin[j];
            s_pos[threadIdx.x] = S.pos[j];
            s_lo[threadIdx.x] = S.pos_lo[j];
            s_vel[threadIdx.x] = make_float4(sv.z, sv.w, ss.y, ss.z * ss.z);
        }
        __syncthreads();
        const int cnt = min(DIRECT_THREADS, n - base);
        if (!valid) continue;
        for (int jj = 0; jj < cnt; jj++) {
            const int jg = base + jj;
            if (jg == i) continue;
            const float4 sp = s_pos[jj];
            const float4 sv = s_vel[jj];
            float rx, ry;
            SPos spos;
            float svx, svy, sAng;
            bool dl = false;
            if (REL) {
                Delayed d;
                if (!delayed_state(P, S, C, s_age, s_segdt, jg, t, d)) continue;
                spos = SPos{ d.x, 0.f, d.y, 0.f };
                rx = d.rx; ry = d.ry;
                svx = d.vx; svy = d.vy;
                sAng = d.angw * rsqrtf(1.f + d.angw * d.angw * sv.w);
                dl = true;
            } else {
                const float2 sl = s_lo[jj];
                spos = SPos{ sp.x, sl.x, sp.y, sl.y };
                displacement(P, t.x, t.y, sp.x, sl.x - t.xlo, sp.y, sl.y - t.ylo, rx, ry);
                svx = sv.x; svy = sv.y; sAng = sv.z;
            }
            const float sMu = MAG_MOMENT_K * sp.w * sAng * sv.w;
            const float sL = INERTIA_K * sp.z * sAng * sv.w;
            const bool yk = yukawa_in(P, rx, ry, spos, t);
            pair_force<MAGGM, BRK>(P, t, rx, ry, svx, svy, sp.z, sp.w, sAng, sMu, sL, dl, yk, pe, A);
            A.tick();
            inter++;
        }
    }
    if (gridDim.y == 1) {
        finalize_target<MAGGM, BRK>(P, S, C, ctl, t, valid, A, inter);
        return;
    }
    A.flush();
    if (valid) {
        constexpr int NQ = Acc<MAGGM, BRK>::NQ;
        const size_t stride = (size_t)gridDim.x * DIRECT_THREADS;
        float* part = C.dpart + (size_t)blockIdx.y * direct_part_rows<MAGGM, BRK>() * stride + i;
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            part[(size_t)q * stride] = A.hi(q);
            part[(size_t)(NQ + q) * stride] = A.lo(q);
        }
        part[(size_t)(2 * NQ) * stride] = __uint_as_float(inter);
    }
}

// Adds the slices' partial sums in slice order through the same compensated
// accumulator, then runs the per-particle epilogue of the pairwise sum.
template <bool MAGGM, bool BRK>
__global__ void __launch_bounds__(DIRECT_THREADS)
direct_combine_kernel(DevParams P, DevState S, FrameCtl* ctl, ForceCtx C, int slices) {
    const int n = ctl->n;
    const int i = blockIdx.x * DIRECT_THREADS + threadIdx.x;
    const bool valid = i < n;
    Tgt t;
    if (valid) { t = load_target(S, i); target_coupling(P, t); }
    else { t = Tgt{}; t.idx = -1; }
    Acc<MAGGM, BRK> A;
    A.init();
    unsigned inter = 0;
    if (valid) {
        constexpr int NQ = Acc<MAGGM, BRK>::NQ;
        const size_t stride = (size_t)gridDim.x * DIRECT_THREADS;
        for (int y = 0; y < slices; y++) {
            const float* part = C.dpart + (size_t)y * direct_part_rows<MAGGM, BRK>() * stride + i;
#pragma unroll
            for (int q = 0; q < NQ; q++) A.part[q] = part[(size_t)q * stride];
            A.flush();
#pragma unroll
            for (int q = 0; q < NQ; q++) A.part[q] = part[(size_t)(NQ + q) * stride];
            A.flush();
            inter += __float_as_uint(part[(size_t)(2 * NQ) * stride]);
        }
    }
    finalize_target<MAGGM, BRK>(P, S, C, ctl, t, valid, A, inter);
}

// Source slices for a pairwise sum over n_cap targets with `slots` resident
// CTAs: each added slice must raise the CTAs' wave efficiency (CTAs over
// whole waves of slots) by 2 %; at most 16 slices and 8 waves.
static int slice_count(long long blocks, long long slots) {
    auto eff = [&](int s) {
        const long long c = blocks * s;
        return (double)c / (double)(((c + slots - 1) / slots) * slots);
    };
    int best = 1;
    double bestEff = eff(1);
    for (int s = 2; s <= 16 && blocks * s <= 8 * slots; s++) {
        const double e = eff(s);
        if (e > bestEff + 0.02) { best = s; bestEff = e; }
    }
    return best;
}

static int direct_slice_count(int n_cap, long long slots) {
    return slice_count(std::max(1, (n_cap + DIRECT_THREADS - 1) / DIRECT_THREADS), slots);
}

template <bool MAGGM, bool REL, bool BRK>
static DirectPlan direct_plan_t(int n_cap) {
    static int occ = 0, sms = 0;
    if (!occ) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, direct_kernel<MAGGM, REL, BRK>, DIRECT_THREADS, 0);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (occ < 1) occ = 1;
        if (sms < 1) sms = 1;
    }
    const int best = direct_slice_count(n_cap, (long long)occ * sms);
    const long long blocks = std::max(1, (n_cap + DIRECT_THREADS - 1) / DIRECT_THREADS);
    const size_t floats = best > 1 ? (size_t)best * direct_part_rows<MAGGM, BRK>() * blocks * DIRECT_THREADS : 0;
    return DirectPlan{ best, floats };
}

DirectPlan direct_plan(const DevParams& P, bool brk, int n_cap) {
    const bool maggm = (P.toggles & (GEON_MAGNETIC | GEON_GRAVITOMAG | GEON_ONE_PN)) != 0;
    const bool rel = P.rel != 0;
    if (maggm) {
        if (rel) return brk ? direct_plan_t<true, true, true>(n_cap) : direct_plan_t<true, true, false>(n_cap);
        return brk ? direct_plan_t<true, false, true>(n_cap) : direct_plan_t<true, false, false>(n_cap);
    }
    if (rel) return brk ? direct_plan_t<false, true, true>(n_cap) : direct_plan_t<false, true, false>(n_cap);
    return brk ? direct_plan_t<false, false, true>(n_cap) : direct_plan_t<false, false, false>(n_cap);
}

// ---- pairwise forces for a subset of targets (no state change) -----------------------------
// The O(N^2) sum of forces.js:94-125 evaluated for the listed particles only
// and written to separate outputs: the exact reference against which the
// Barnes-Hut force error is measured.
template <bool MAGGM, bool REL>
__global__ void __launch_bounds__(DIRECT_THREADS)
direct_subset_kernel(DevParams P, DevState S, const FrameCtl* ctl, ForceCtx C, const int* __restrict__ idx, int k,
                     float* __restrict__ out_fx, float* __restrict__ out_fy) {
    __shared__ float4 s_pos[DIRECT_THREADS];
    __shared__ float4 s_vel[DIRECT_THREADS];
    __shared__ float2 s_lo[DIRECT_THREADS];
    __shared__ float s_age[REL ? HIST_LEN : 1], s_segdt[REL ? HIST_LEN : 1];
    if (REL) load_hist_tables(C, s_age, s_segdt);
    const int n = ctl->n;
    const int ti = blockIdx.x * DIRECT_THREADS + threadIdx.x;
    const bool valid = ti < k && idx[ti] >= 0 && idx[ti] < n;
    const int i = valid ? idx[ti] : -1;
    Tgt t;
    if (valid) { t = load_target(S, i); target_coupling(P, t); }
    else { t = Tgt{}; t.idx = -1; }
    Acc<MAGGM, false> A;
    A.init();
    const int ntile = (n + DIRECT_THREADS - 1) / DIRECT_THREADS;       // blockIdx.y: a slice of the source tiles
    const int tile0 = (int)((long long)ntile * blockIdx.y / gridDim.y);
    const int tile1 = (int)((long long)ntile * (blockIdx.y + 1) / gridDim.y);
    for (int base = tile0 * DIRECT_THREADS; base < tile1 * DIRECT_THREADS; base += DIRECT_THREADS) {
        const int j = base + threadIdx.x;
        __syncthreads();
        if (j < n) {
            const float4 sv = S.vel[j], ss = S.spin[j];
            s_pos[threadIdx.x] = S.pos[j];
            s_lo[threadIdx.x] = S.pos_lo[j];
            s_vel[threadIdx.x] = make_float4(sv.z, sv.w, ss.y, ss.z * ss.z);
        }
        __syncthreads();
        if (!valid) continue;
        const int cnt = min(DIRECT_THREADS, n - base);
        for (int jj = 0; jj < cnt; jj++) {
            const int jg = base + jj;
            if (jg == i) continue;
            const float4 sp = s_pos[jj];
            const float4 sv = s_vel[jj];
            float rx, ry, svx, svy, sAng;
            SPos spos;
            bool dl = false;
            if (REL) {
                Delayed d;
                if (!delayed_state(P, S, C, s_age, s_segdt, jg, t, d)) continue;
                spos = SPos{ d.x, 0.f, d.y, 0.f };
                rx = d.rx; ry = d.ry; svx = d.vx; svy = d.vy;
                sAng = d.angw * rsqrtf(1.f + d.angw * d.angw * sv.w);
                dl = true;
            } else {
                const float2 sl = s_lo[jj];
                spos = SPos{ sp.x, sl.x, sp.y, sl.y };
                displacement(P, t.x, t.y, sp.x, sl.x - t.xlo, sp.y, sl.y - t.ylo, rx, ry);
                svx = sv.x; svy = sv.y; sAng = sv.z;
            }
            const float sMu = MAG_MOMENT_K * sp.w * sAng * sv.w;
            const float sL = INERTIA_K * sp.z * sAng * sv.w;
            const bool yk = yukawa_in(P, rx, ry, spos, t);
            pair_force<MAGGM, false>(P, t, rx, ry, svx, svy, sp.z, sp.w, sAng, sMu, sL, dl, yk, false, A);
            A.tick();
        }
    }
    A.flush();
    if (!valid) return;
    if (gridDim.y == 1) { out_fx[ti] = A.get(Q_FX); out_fy[ti] = A.get(Q_FY); return; }
    const size_t stride = (size_t)gridDim.x * DIRECT_THREADS;
    float* q = C.dpart + (size_t)blockIdx.y * 4 * stride + ti;       // the slice's fx, fy as (hi, lo)
    q[0] = A.hi(Q_FX); q[stride] = A.lo(Q_FX);
    q[2 * stride] = A.hi(Q_FY); q[3 * stride] = A.lo(Q_FY);
}

__global__ void __launch_bounds__(DIRECT_THREADS)
direct_subset_combine_kernel(ForceCtx C, const int* __restrict__ idx, int k, const FrameCtl* ctl, int slices,
                             float* __restrict__ out_fx, float* __restrict__ out_fy) {
    const int ti = blockIdx.x * DIRECT_THREADS + threadIdx.x;
    if (ti >= k || idx[ti] < 0 || idx[ti] >= ctl->n) return;
    const size_t stride = (size_t)gridDim.x * DIRECT_THREADS;
    CAcc x, y;
    x.init();
    y.init();
    for (int s = 0; s < slices; s++) {
        const float* q = C.dpart + (size_t)s * 4 * stride + ti;
        x.add(q[0]); x.add(q[stride]);
        y.add(q[2 * stride]); y.add(q[3 * stride]);
    }
    out_fx[ti] = x.value();
    out_fy[ti] = y.value();
}

DirectPlan direct_subset_plan(const DevParams& P, int k) {
    static int occ[4] = { 0, 0, 0, 0 }, sms = 0;
    const bool maggm = (P.toggles & (GEON_MAGNETIC | GEON_GRAVITOMAG | GEON_ONE_PN)) != 0;
    const int v = (maggm ? 2 : 0) + (P.rel ? 1 : 0);
    if (!occ[v]) {
        switch (v) {
            case 3: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[v], direct_subset_kernel<true, true>, DIRECT_THREADS, 0); break;
            case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[v], direct_subset_kernel<true, false>, DIRECT_THREADS, 0); break;
            case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[v], direct_subset_kernel<false, true>, DIRECT_THREADS, 0); break;
            default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[v], direct_subset_kernel<false, false>, DIRECT_THREADS, 0); break;
        }
        if (occ[v] < 1) occ[v] = 1;
    }
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms < 1) sms = 1;
    }
    const int best = direct_slice_count(k, (long long)occ[v] * sms);
    const long long blocks = std::max(1, (k + DIRECT_THREADS - 1) / DIRECT_THREADS);
    return DirectPlan{ best, best > 1 ? (size_t)best * 4 * blocks * DIRECT_THREADS : 0 };
}



void direct_subset(const DevParams& P, const DevState& S, const FrameCtl* ctl, const ForceCtx& C, const int* idx,
                   int k, float* fx, float* fy, cudaStream_t st, LaunchCounter& lc) {
    const bool maggm = (P.toggles & (GEON_MAGNETIC | GEON_GRAVITOMAG | GEON_ONE_PN)) != 0;
    const int blocks = std::max(1, (k + DIRECT_THREADS - 1) / DIRECT_THREADS);
    const int slices = (C.dpart && C.dslices > 1) ? C.dslices : 1;
    const dim3 grid(blocks, slices);
    if (maggm) {
        if (P.rel) direct_subset_kernel<true, true><<<grid, DIRECT_THREADS, 0, st>>>(P, S, ctl, C, idx, k, fx, fy);
        else direct_subset_kernel<true, false><<<grid, DIRECT_THREADS, 0, st>>>(P, S, ctl, C, idx, k, fx, fy);
    } else {
        if (P.rel) direct_subset_kernel<false, true><<<grid, DIRECT_THREADS, 0, st>>>(P, S, ctl, C, idx, k, fx, fy);
        else direct_subset_kernel<false, false><<<grid, DIRECT_THREADS, 0, st>>>(P, S, ctl, C, idx, k, fx, fy);
    }
    lc.add(1);
    if (slices > 1) {
        direct_subset_combine_kernel<<<blocks, DIRECT_THREADS, 0, st>>>(C, idx, k, ctl, slices, fx, fy);
        lc.add(1);
    }
}

// ---- potential heat map (heatmap.js:38-101, 152-206) ---------------------------------------------
// One thread per grid point.  Tree mode follows treePotential: a node is
// skipped only when both its mass and charge are zero; aggregates use the
// centre of mass without minimum image; leaves evaluate their real points
// (ghosts are skipped), signal-delayed when relativity is on; no Yukawa
// cutoff.  Pairwise mode follows the grid loop's direct branch: minimum
// image, Yukawa cutoff on r^2 + softening^2 < (6/mu)^2.
constexpr int HM_THREADS = 128;
constexpr int HM_STACK = 128;       // depth 31 needs at most 3 * 31 + 4 entries

__device__ __forceinline__ void potential_terms(const DevParams& P, float rx, float ry, float m, float q,
                                                bool doG, bool doE, bool doY, bool cut, CAcc& g, CAcc& e, CAcc& y) {
    const float rSq = __fmaf_rn(rx, rx, ry * ry) + P.softSq;
    const float invR = rsqrtf(rSq);
    if (doG) g.add(-m * invR);
    if (doE) e.add(q * invR);
    if (doY) {
        bool in = true;
        if (cut) {                                          // heatmap.js:185 (pairwise branch only)
            const float c = P.yukCutSq;
            in = fabsf(rSq - c) > 1e-6f * c ? rSq < c
                                            : ((double)rx * rx + (double)ry * ry + (double)P.softSq < P.yukCutSqD);
        }
        if (in) {
            const float r = rSq * invR;
            y.add(-YUKAWA_COUPLING * m * __expf(-P.yukMu * r) * invR);
        }
    }
}

template <bool REL>
__global__ void __launch_bounds__(HM_THREADS)
heatmap_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root, FrameCtl* ctl, ForceCtx C,
               double left, double top, double cw, double chh, int G, int doG_, int doE_, int doY_, int useTree,
               float* __restrict__ gOut, float* __restrict__ eOut, float* __restrict__ yOut, float* __restrict__ part) {
    __shared__ float s_age[REL ? HIST_LEN : 1], s_segdt[REL ? HIST_LEN : 1];
    if (REL) load_hist_tables(C, s_age, s_segdt);
    const bool doG = doG_ != 0, doE = doE_ != 0, doY = doY_ != 0;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G * G) return;
    const int gy = idx / G, gx = idx % G;
    const double wy = top + (gy + 0.5) * chh, wx = left + (gx + 0.5) * cw;
    Tgt o{};
    o.x = (float)wx; o.xlo = (float)(wx - (double)o.x);
    o.y = (float)wy; o.ylo = (float)(wy - (double)o.y);
    o.idx = -1;
    CAcc g, e, y;
    g.init(); e.init(); y.init();
    const int n = ctl->n;
    if (useTree) {
        int stack[HM_STACK];
        int sp = 0;
        const int root = *d_root;
        const int nInt = ctl->nInternal, nLeaf = ctl->nLeaves, nValid = ctl->nValid;
        if (root != ROOT_NONE && !(ctl->err & (ERR_NODE_OVERFLOW | ERR_BAD_INDEX))) stack[sp++] = root;
        while (sp > 0) {
            const int node = stack[--sp];
            if (node & LEAF_REF) {
                const int li = node & ~LEAF_REF;
                if (li < 0 || li >= nLeaf) { atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
                const float4 la = T.leaf_a[li];
                if (la.z == 0.f && la.w == 0.f) continue;
                const int4 lm = T.leaf_meta[li];
                if (lm.x < 0 || lm.x + lm.y > nValid) { atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
                for (int q = lm.x; q < lm.x + lm.y; q++) {
                    const uint32_t ref = __float_as_uint(T.ps_c[q].w);
                    if (ref_code(ref) != CODE_IDENTITY) continue;            // heatmap.js:60
                    const float4 pa = T.ps_a[q];
                    float rx, ry;
                    if (REL) {
                        const int j = (int)ref_index(ref);
                        Delayed d;
                        if (!delayed_state(P, S, C, s_age, s_segdt, j, o, d)) continue;
                        rx = d.rx; ry = d.ry;
                    } else {
                        const float4 pb = T.ps_b[q];
                        rx = __fadd_rn(__fsub_rn(pa.x, o.x), pb.x - o.xlo);
                        ry = __fadd_rn(__fsub_rn(pa.y, o.y), pb.y - o.ylo);
                    }
                    potential_terms(P, rx, ry, pa.z, pa.w, doG, doE, doY, false, g, e, y);
                }
            } else {
                if (node < 0 || node >= nInt) { atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
                const float4 a = T.int_a[node];
                if (a.z == 0.f && a.w == 0.f) continue;
                const float4 c = T.int_c[node];
                const float dx = __fadd_rn(__fsub_rn(a.x, o.x), c.x - o.xlo);
                const float dy = __fadd_rn(__fsub_rn(a.y, o.y), c.y - o.ylo);
                const float rhs = P.thetaSq * __fmaf_rn(dx, dx, dy * dy);
                bool accept = c.z < rhs;
                if (fabsf(rhs - c.z) <= 1e-6f * c.z) {
                    const double ddx = ((double)a.x + (double)c.x) - wx, ddy = ((double)a.y + (double)c.y) - wy;
                    const double size = 2.0 * ldexp(P.rootW, -(int)c.w);
                    accept = size * size < P.thetaSqD * (ddx * ddx + ddy * ddy);
                }
                if (accept) {
                    potential_terms(P, dx, dy, a.z, a.w, doG, doE, doY, false, g, e, y);
                } else {
                    const int4 ch = T.int_child[node];
                    if (sp + 4 > HM_STACK) { atomicOr(&ctl->err, ERR_STACK_OVERFLOW); break; }
                    if (ch.x >= 0) stack[sp++] = ch.x;
                    if (ch.y >= 0) stack[sp++] = ch.y;
                    if (ch.z >= 0) stack[sp++] = ch.z;
                    if (ch.w >= 0) stack[sp++] = ch.w;
                }
            }
        }
    } else {
        // pairwise: blockIdx.y selects a slice of the sources (gridDim.y slices)
        const int i0 = (int)((long long)n * blockIdx.y / gridDim.y);
        const int i1 = (int)((long long)n * (blockIdx.y + 1) / gridDim.y);
        for (int i = i0; i < i1; i++) {
            float rx, ry;
            const float4 p = S.pos[i];
            if (REL) {
                Delayed d;
                if (!delayed_state(P, S, C, s_age, s_segdt, i, o, d)) continue;
                rx = d.rx; ry = d.ry;
            } else {
                const float2 pl = S.pos_lo[i];
                displacement(P, o.x, o.y, p.x, pl.x - o.xlo, p.y, pl.y - o.ylo, rx, ry);
            }
            potential_terms(P, rx, ry, p.z, p.w, doG, doE, doY, true, g, e, y);
        }
    }
    if (gridDim.y == 1) {
        gOut[idx] = g.value();
        eOut[idx] = e.value();
        yOut[idx] = y.value();
        return;
    }
    const size_t gg = (size_t)G * G;
    float* q = part + (size_t)blockIdx.y * 6 * gg + idx;    // the slice's (hi, lo) per field
    q[0] = g.hi; q[gg] = g.lo;
    q[2 * gg] = e.hi; q[3 * gg] = e.lo;
    q[4 * gg] = y.hi; q[5 * gg] = y.lo;
}

// Adds the pairwise heat map's slices in slice order (compensated).
__global__ void __launch_bounds__(HM_THREADS)
heatmap_combine_kernel(const float* __restrict__ part, int slices, int G, float* __restrict__ gOut,
                       float* __restrict__ eOut, float* __restrict__ yOut) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t gg = (size_t)G * G;
    if (idx >= (int)gg) return;
    CAcc g, e, y;
    g.init(); e.init(); y.init();
    for (int k = 0; k < slices; k++) {
        const float* q = part + (size_t)k * 6 * gg + idx;
        g.add(q[0]); g.add(q[gg]);
        e.add(q[2 * gg]); e.add(q[3 * gg]);
        y.add(q[4 * gg]); y.add(q[5 * gg]);
    }
    gOut[idx] = g.value();
    eOut[idx] = e.value();
    yOut[idx] = y.value();
}

int heatmap_slices(const DevParams& P, int G, bool useTree) {
    if (useTree) return 1;
    static int occ[2] = { 0, 0 }, sms = 0;
    const int r = P.rel ? 1 : 0;
    if (!occ[r]) {
        if (r) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[r], heatmap_kernel<true>, HM_THREADS, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[r], heatmap_kernel<false>, HM_THREADS, 0);
        if (occ[r] < 1) occ[r] = 1;
    }
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms < 1) sms = 1;
    }
    return slice_count(((long long)G * G + HM_THREADS - 1) / HM_THREADS, (long long)occ[r] * sms);
}

// Heatmap._blur (heatmap.js:278-302): 3 x 3 box blur, clamp to edge, as two passes.
__global__ void blur_kernel(const float* __restrict__ in, float* __restrict__ out, int G, int horizontal) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G * G) return;
    const int yy = idx / G, xx = idx % G;
    float a, b, c;
    if (horizontal) {
        a = in[yy * G + max(xx - 1, 0)]; b = in[idx]; c = in[yy * G + min(xx + 1, G - 1)];
    } else {
        a = in[max(yy - 1, 0) * G + xx]; b = in[idx]; c = in[min(yy + 1, G - 1) * G + xx];
    }
    out[idx] = (a + b + c) * (1.f / 3.f);
}

void heatmap_pass(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                  const ForceCtx& C, double left, double top, double cw, double ch, int G, bool doG, bool doE, bool doY,
                  bool useTree, bool blur, float* g, float* e, float* y, float* tmp, float* part, int slices,
                  cudaStream_t st, LaunchCounter& lc) {
    const int blocks = (G * G + HM_THREADS - 1) / HM_THREADS;
    if (useTree || !part) slices = 1;
    const dim3 grid(blocks, std::max(slices, 1));
    if (P.rel) heatmap_kernel<true><<<grid, HM_THREADS, 0, st>>>(P, S, T, d_root, ctl, C, left, top, cw, ch, G, doG, doE, doY, useTree, g, e, y, part);
    else heatmap_kernel<false><<<grid, HM_THREADS, 0, st>>>(P, S, T, d_root, ctl, C, left, top, cw, ch, G, doG, doE, doY, useTree, g, e, y, part);
    lc.add(1);
    if (slices > 1) {
        heatmap_combine_kernel<<<blocks, HM_THREADS, 0, st>>>(part, slices, G, g, e, y);
        lc.add(1);
    }
    if (blur) {
        float* fields[3] = { g, e, y };
        const bool on3[3] = { doG, doE, doY };
        for (int f = 0; f < 3; f++) {
            if (!on3[f]) continue;
            blur_kernel<<<blocks, HM_THREADS, 0, st>>>(fields[f], tmp, G, 1);
            blur_kernel<<<blocks, HM_THREADS, 0, st>>>(tmp, fields[f], G, 0);
            lc.add(2);
        }
    }
}

// ---- 1PN-only passes (forces.js:445-610) ----------------------------------------------------
__device__ __forceinline__ void accum_1pn(const DevParams& P, const Tgt& t, float rx, float ry, float svx, float svy,
                                          float sm, float sq, float& ox, float& oy) {
    const float rSq = __fmaf_rn(rx, rx, ry * ry) + P.softSq;
    const float invR = rsqrtf(rSq);
    const float invRSq = invR * invR;
    const float r = rSq * invR;
    const float nx = rx * invR, ny = ry * invR;
    const bool gm = on(P, GEON_GRAVITOMAG), mag = on(P, GEON_MAGNETIC);
    if (gm) {
        const float v1Sq = t.vx * t.vx + t.vy * t.vy, v2Sq = svx * svx + svy * svy;
        const float nDotV1 = nx * t.vx + ny * t.vy, nDotV2 = nx * svx + ny * svy;
        const float radial = -v1Sq - 2.f * v2Sq + 1.5f * nDotV2 * nDotV2 + 5.f * t.m * invR + 4.f * sm * invR;
        const float v1Coeff = 4.f * nDotV1 - 3.f * nDotV2, v2Coeff = 3.f * nDotV2;
        const float base = t.m * sm * invRSq * invR;
        ox += base * (rx * radial + (t.vx * v1Coeff + svx * v2Coeff) * r);
        oy += base * (ry * radial + (t.vy * v1Coeff + svy * v2Coeff) * r);
    }
    if (mag) {
        const float v2DotN = svx * nx + svy * ny, v1DotN = t.vx * nx + t.vy * ny;
        const float coeff = 0.5f * t.q * sq * invRSq;
        ox += coeff * (t.vx * v2DotN - 3.f * nx * v1DotN * v2DotN);
        oy += coeff * (t.vy * v2DotN - 3.f * ny * v1DotN * v2DotN);
    }
    if (gm && mag) {
        const float crossCoeff = t.q * sq * (t.m + sm) - (t.q * t.q * sm + sq * sq * t.m);
        const float fDir = crossCoeff * invRSq * invRSq;
        ox += rx * fDir; oy += ry * fDir;
    }
    if (on(P, GEON_YUKAWA)) {                                        // no cutoff in the 1PN pass
        const float mu = P.yukMu;
        const float expMuR = __expf(-mu * r);
        const float nDotV1 = nx * t.vx + ny * t.vy, nDotV2 = nx * svx + ny * svy;
        const float v1DotV2 = t.vx * svx + t.vy * svy;
        const float alpha = 1.f + mu * r;
        const float beta = 0.5f * YUKAWA_COUPLING * t.m * sm * expMuR * invRSq;
        const float radial = -(alpha * v1DotV2 + (alpha * alpha + alpha + 1.f) * nDotV1 * nDotV2);
        ox += beta * (radial * nx + alpha * (nDotV2 * t.vx + nDotV1 * svx));
        oy += beta * (radial * ny + alpha * (nDotV2 * t.vy + nDotV1 * svy));
    }
}

struct Acc2 {
    float px, py; CAcc x, y; int cnt;
    __device__ __forceinline__ void init() { px = py = 0.f; x.init(); y.init(); cnt = 0; }
    __device__ __forceinline__ void flush() { x.add(px); y.add(py); px = py = 0.f; }
    __device__ __forceinline__ void tick() { if (++cnt >= FLUSH_EVERY) { flush(); cnt = 0; } }
};

__global__ void __launch_bounds__(WALK_THREADS)
walk1pn_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root, FrameCtl* ctl, ForceCtx C) {
    __shared__ int s_node[WALK_WARPS][WALK_STACK];
    __shared__ unsigned s_mask[WALK_WARPS][WALK_STACK];
    __shared__ float s_age[HIST_LEN], s_segdt[HIST_LEN];
    load_hist_tables(C, s_age, s_segdt);
    const int n = ctl->n;
    const int warp = threadIdx.x >> 5;
    const unsigned lane = threadIdx.x & 31;
    const int k = (blockIdx.x * WALK_WARPS + warp) * 32 + (int)lane;
    const bool valid = k < n;
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    if (active == 0) return;
    Tgt t;
    if (valid) t = load_target(S, T.tgt[k]);
    else { t = Tgt{}; t.idx = -1; }
    Acc2 A; A.init();
    const int root = *d_root;
    const bool treeOk = (ctl->err & (ERR_NODE_OVERFLOW | ERR_BAD_INDEX)) == 0;
    const int nIntW = ctl->nInternal, nLeafW = ctl->nLeaves, nValidW = ctl->nValid;
    int top = 0;
    if (root != ROOT_NONE && treeOk) {
        if (lane == 0) { s_node[warp][0] = root; s_mask[warp][0] = active; }
        top = 1;
    }
    __syncwarp();
    while (top > 0) {
        top--;
        const int node = s_node[warp][top];
        const unsigned mask = s_mask[warp][top];
        __syncwarp();
        const bool in = (mask >> lane) & 1u;
        if (node & LEAF_REF) {
            const int li = node & ~LEAF_REF;
            if (li >= nLeafW) { if (lane == 0) atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
            if (T.leaf_a[li].z < EPS_F) continue;
            const int4 lm = T.leaf_meta[li];
            if (lm.x < 0 || lm.x + lm.y > nValidW) { if (lane == 0) atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
            for (int q = lm.x; q < lm.x + lm.y; q++) {               // forces.js:534-554
                const float4 pa = T.ps_a[q];
                const float4 pb = T.ps_b[q];
                const uint32_t ref = __float_as_uint(T.ps_c[q].w);
                const int j = (int)ref_index(ref);
                const uint32_t code = ref_code(ref);
                if (!in || j == t.idx) continue;
                float rx, ry, svx, svy;
                if (code == CODE_IDENTITY) {
                    Delayed d;
                    if (!delayed_state(P, S, C, s_age, s_segdt, j, t, d)) continue;
                    rx = d.rx; ry = d.ry;
                    svx = d.vx; svy = d.vy;
                } else {
                    displacement(P, t.x, t.y, pa.x, pb.x - t.xlo, pa.y, pb.y - t.ylo, rx, ry);
                    svx = pb.z; svy = pb.w;
                }
                accum_1pn(P, t, rx, ry, svx, svy, pa.z, pa.w, A.px, A.py);
                A.tick();
            }
        } else {
            if (node < 0 || node >= nIntW) { if (lane == 0) atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
            const float4 a = T.int_a[node];
            if (a.z < EPS_F) continue;
            const float4 c = T.int_c[node];
            bool accept = false;
            float rx = 0.f, ry = 0.f;
            if (in) {
                displacement(P, t.x, t.y, a.x, c.x - t.xlo, a.y, c.y - t.ylo, rx, ry);
                const float dSq = __fmaf_rn(rx, rx, ry * ry);
                const float rhs = P.thetaSq * dSq;
                accept = c.z < rhs;
                if (fabsf(rhs - c.z) <= 1e-6f * c.z) {
                    double dx, dy;
                    exact_disp(P, t.xd(), t.yd(), (double)a.x + (double)c.x, (double)a.y + (double)c.y, dx, dy);
                    const double size = 2.0 * ldexp(P.rootW, -(int)c.w);
                    accept = size * size < P.thetaSqD * (dx * dx + dy * dy);
                }
            }
            const unsigned acc = __ballot_sync(0xffffffffu, accept);
            const unsigned open = mask & ~acc;
            if (accept) {
                const float4 b = T.int_b[node];
                accum_1pn(P, t, rx, ry, b.x, b.y, a.z, a.w, A.px, A.py);
                A.tick();
            }
            if (open) {
                const int4 ch = T.int_child[node];
                const int np = (ch.x >= 0) + (ch.y >= 0) + (ch.z >= 0) + (ch.w >= 0);
                if (top + np > WALK_STACK) {
                    if (lane == 0) atomicOr(&ctl->err, ERR_STACK_OVERFLOW);
                } else {
                    if (lane == 0) {
                        int tp = top;
                        if (ch.x >= 0) { s_node[warp][tp] = ch.x; s_mask[warp][tp++] = open; }
                        if (ch.y >= 0) { s_node[warp][tp] = ch.y; s_mask[warp][tp++] = open; }
                        if (ch.z >= 0) { s_node[warp][tp] = ch.z; s_mask[warp][tp++] = open; }
                        if (ch.w >= 0) { s_node[warp][tp] = ch.w; s_mask[warp][tp++] = open; }
                    }
                    top += np;
                }
                __syncwarp();
            }
        }
    }
    A.flush();
    if (valid) S.f1pn[t.idx] = make_float2(A.x.value(), A.y.value());
}

// blockIdx.y selects a slice of the source tiles, as in direct_kernel; with
// more than one slice the partial sums (x hi, x lo, y hi, y lo) go to C.dpart
// and direct1pn_combine_kernel finishes.
__global__ void __launch_bounds__(DIRECT_THREADS)
direct1pn_kernel(DevParams P, DevState S, FrameCtl* ctl, ForceCtx C) {
    __shared__ float4 s_pos[DIRECT_THREADS];
    __shared__ float s_age[HIST_LEN], s_segdt[HIST_LEN];
    load_hist_tables(C, s_age, s_segdt);
    const int n = ctl->n;
    const int i = blockIdx.x * DIRECT_THREADS + threadIdx.x;
    const bool valid = i < n;
    Tgt t;
    if (valid) t = load_target(S, i);
    else { t = Tgt{}; t.idx = -1; }
    Acc2 A; A.init();
    const int ntile = (n + DIRECT_THREADS - 1) / DIRECT_THREADS;
    const int tile0 = (int)((long long)ntile * blockIdx.y / gridDim.y);
    const int tile1 = (int)((long long)ntile * (blockIdx.y + 1) / gridDim.y);
    for (int base = tile0 * DIRECT_THREADS; base < tile1 * DIRECT_THREADS; base += DIRECT_THREADS) {
        const int j = base + threadIdx.x;
        __syncthreads();
        if (j < n) s_pos[threadIdx.x] = S.pos[j];
        __syncthreads();
        if (!valid) continue;
        const int cnt = min(DIRECT_THREADS, n - base);
        for (int jj = 0; jj < cnt; jj++) {                           // forces.js:592-608
            const int jg = base + jj;
            if (jg == i) continue;
            Delayed d;
            if (!delayed_state(P, S, C, s_age, s_segdt, jg, t, d)) continue;
            const float rx = d.rx, ry = d.ry;
            const float4 sp = s_pos[jj];
            accum_1pn(P, t, rx, ry, d.vx, d.vy, sp.z, sp.w, A.px, A.py);
            A.tick();
        }
    }
    A.flush();
    if (!valid) return;
    if (gridDim.y == 1) {
        S.f1pn[i] = make_float2(A.x.value(), A.y.value());
        return;
    }
    const size_t stride = (size_t)gridDim.x * DIRECT_THREADS;
    float* part = C.dpart + (size_t)blockIdx.y * 4 * stride + i;
    part[0] = A.x.hi;
    part[stride] = A.x.lo;
    part[2 * stride] = A.y.hi;
    part[3 * stride] = A.y.lo;
}

__global__ void __launch_bounds__(DIRECT_THREADS)
direct1pn_combine_kernel(DevState S, const FrameCtl* ctl, ForceCtx C, int slices) {
    const int i = blockIdx.x * DIRECT_THREADS + threadIdx.x;
    if (i >= ctl->n) return;
    const size_t stride = (size_t)gridDim.x * DIRECT_THREADS;
    CAcc x, y;
    x.init();
    y.init();
    for (int k = 0; k < slices; k++) {
        const float* part = C.dpart + (size_t)k * 4 * stride + i;
        x.add(part[0]);
        x.add(part[stride]);
        y.add(part[2 * stride]);
        y.add(part[3 * stride]);
    }
    S.f1pn[i] = make_float2(x.value(), y.value());
}

DirectPlan direct1pn_plan(int n_cap) {
    static int occ = 0, sms = 0;
    if (!occ) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, direct1pn_kernel, DIRECT_THREADS, 0);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (occ < 1) occ = 1;
        if (sms < 1) sms = 1;
    }
    const int best = direct_slice_count(n_cap, (long long)occ * sms);
    const long long blocks = std::max(1, (n_cap + DIRECT_THREADS - 1) / DIRECT_THREADS);
    return DirectPlan{ best, best > 1 ? (size_t)best * 4 * blocks * DIRECT_THREADS : 0 };
}

// ---- dispatch ---------------------------------------------------------------------------------
__global__ void clear_reductions_kernel(FrameCtl* ctl) {
    ctl->maxAccelSqBits = 0ull;
    ctl->maxCycBits = 0ull;
    ctl->interactions = 0ull;
}

template <bool MAGGM, bool REL, bool BRK>
static void launch_force(bool bh, const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root,
                         FrameCtl* ctl, const ForceCtx& C, int n_cap, cudaStream_t st) {
    const int slots = C.tgt_list ? C.tgt_count : n_cap;      // walk slots (batched: padded per system)
    if (bh && (P.flags & GEON_FLAG_SIMPLE_WALK)) {
        const int blocks = std::max(1, (slots + WALK_THREADS - 1) / WALK_THREADS);
        walk_kernel<MAGGM, REL, BRK><<<blocks, WALK_THREADS, 0, st>>>(P, S, T, d_root, ctl, C);
    } else if (bh) {
        constexpr bool PLAIN = !MAGGM && !REL && !BRK;
        const int blocks = std::max(1, (slots + WC_THREADS - 1) / WC_THREADS);
        const bool lean = PLAIN && !C.pe;
        if (PLAIN && C.recs) {                     // learned correction (plain forces only)
            if (P.periodic) {
                if (lean) launch_walkc<false, false, false, 1, true, true>(blocks, P, S, T, d_root, ctl, C, st);
                else launch_walkc<false, false, false, 1, false, true>(blocks, P, S, T, d_root, ctl, C, st);
            } else {
                if (lean) launch_walkc<false, false, false, 0, true, true>(blocks, P, S, T, d_root, ctl, C, st);
                else launch_walkc<false, false, false, 0, false, true>(blocks, P, S, T, d_root, ctl, C, st);
            }
        } else if (P.periodic) {
            // the torus walks of the ensemble (plain forces) and of the full
            // force set with relativity carry the torus wrap alone
            const bool torus = P.topology == GEON_TORUS;
            if constexpr (PLAIN) {
                if (lean && torus) {
                    // without the Yukawa term its cutoff guard and force leave the loop
                    if (P.yukOn) launch_lean_torus<true>(slots, blocks, P, S, T, d_root, ctl, C, st);
                    else launch_lean_torus<false>(slots, blocks, P, S, T, d_root, ctl, C, st);
                    return;
                }
                if (lean) {
                    launch_walkc<false, false, false, 1, true>(blocks, P, S, T, d_root, ctl, C, st);
                    return;
                }
            }
            if constexpr (MAGGM && REL && !BRK) {
                if (torus) { launch_walkc<MAGGM, REL, BRK, 2>(blocks, P, S, T, d_root, ctl, C, st); return; }
            }
            launch_walkc<MAGGM, REL, BRK, 1>(blocks, P, S, T, d_root, ctl, C, st);
        } else {
            if constexpr (PLAIN) {
                if (lean && C.walk_split) {
                    launch_walkc_split<false, false, false, 0, true>(slots, P, S, T, d_root, ctl, C, st);
                    return;
                }
            }
            if (lean) launch_walkc<MAGGM, REL, BRK, 0, PLAIN>(blocks, P, S, T, d_root, ctl, C, st);
            else launch_walkc<MAGGM, REL, BRK, 0>(blocks, P, S, T, d_root, ctl, C, st);
        }
    } else {
        const int blocks = std::max(1, (n_cap + DIRECT_THREADS - 1) / DIRECT_THREADS);
        const int slices = (C.dpart && C.dslices > 1) ? C.dslices : 1;
        direct_kernel<MAGGM, REL, BRK><<<dim3(blocks, slices), DIRECT_THREADS, 0, st>>>(P, S, ctl, C);
        if (slices > 1) direct_combine_kernel<MAGGM, BRK><<<blocks, DIRECT_THREADS, 0, st>>>(P, S, ctl, C, slices);
    }
}

void force_pass(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                const ForceCtx& C, bool bh, int n_cap, cudaStream_t st, LaunchCounter& lc, bool clear) {
    if (clear) clear_reductions_kernel<<<1, 1, 0, st>>>(ctl);
    const bool maggm = (P.toggles & (GEON_MAGNETIC | GEON_GRAVITOMAG | GEON_ONE_PN)) != 0;
    const bool rel = P.rel != 0;
    const bool brk = C.brk != 0;
    if (maggm) {
        if (rel) { if (brk) launch_force<true, true, true>(bh, P, S, T, d_root, ctl, C, n_cap, st); else launch_force<true, true, false>(bh, P, S, T, d_root, ctl, C, n_cap, st); }
        else     { if (brk) launch_force<true, false, true>(bh, P, S, T, d_root, ctl, C, n_cap, st); else launch_force<true, false, false>(bh, P, S, T, d_root, ctl, C, n_cap, st); }
    } else {
        if (rel) { if (brk) launch_force<false, true, true>(bh, P, S, T, d_root, ctl, C, n_cap, st); else launch_force<false, true, false>(bh, P, S, T, d_root, ctl, C, n_cap, st); }
        else     { if (brk) launch_force<false, false, true>(bh, P, S, T, d_root, ctl, C, n_cap, st); else launch_force<false, false, false>(bh, P, S, T, d_root, ctl, C, n_cap, st); }
    }
    lc.add((clear ? 2 : 1) + ((!bh && C.dpart && C.dslices > 1) ? 1 : 0));
}

void onepn_pass(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                const ForceCtx& C, bool bh, int n_cap, cudaStream_t st, LaunchCounter& lc) {
    if (bh) {
        const int blocks = std::max(1, (n_cap + WALK_THREADS - 1) / WALK_THREADS);
        walk1pn_kernel<<<blocks, WALK_THREADS, 0, st>>>(P, S, T, d_root, ctl, C);
    } else {
        const int blocks = std::max(1, (n_cap + DIRECT_THREADS - 1) / DIRECT_THREADS);
        const int slices = (C.dpart && C.dslices > 1) ? C.dslices : 1;
        direct1pn_kernel<<<dim3(blocks, slices), DIRECT_THREADS, 0, st>>>(P, S, ctl, C);
        if (slices > 1) { direct1pn_combine_kernel<<<blocks, DIRECT_THREADS, 0, st>>>(S, ctl, C, slices); lc.add(1); }
    }
    lc.add(1);
}

}  // namespace geon
