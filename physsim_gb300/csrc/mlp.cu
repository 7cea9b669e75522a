// mlp.cu — the learned-correction network on fifth-generation tensor cores.
//
// Network (learn.cuh): 14 -> 64 -> 64 -> 6 with GELU (tanh form) after the two
// hidden layers; BF16 weights and activations, FP32 accumulation in TMEM, the
// same roundings in inference and in training.
// A CTA of 128 threads (one warpgroup) processes tiles of 128 samples: thread
// t owns sample row t, which is TMEM lane t.  Per layer the epilogue of the
// previous layer writes BF16 activations to shared memory in the canonical
// K-major layout (tc.cuh); thread 0 issues the tcgen05.mma chain and commits
// it to an mbarrier; all threads wait (bounded) and read their accumulator
// row back with tcgen05.ld.
//
// Training runs the same forward pass and then the backward pass on the
// tensor cores too:
//     dH2 = dY W3,   dZ2 = dH2 * gelu'(Z2),   dH1 = dZ2 W2,   dZ1 = dH1 * gelu'(Z1)
// and the weight gradients as two GEMMs over the 128 samples of a tile
// (K = samples), accumulated in TMEM across every tile a CTA processes:
//     GA = [dZ2^T ; dZ1^T] [H1^T ; X'^T]^T     (128 x 80)
//     GB = [H2^T ; 1]      [dY^T]^T            (128 x 16)
// X' is the feature row with a constant 1 in column 14, so GA column 64+14
// holds the bias gradients db2 (rows 0..63) and db1 (rows 64..127); the ones
// row of GB gives db3.  The epilogues write the transposed operands with
// scattered 2-byte stores.
//
// Loss of a training sample: its 6 outputs y against the least-squares
// targets y* of its record and the record's quadratic form, per component c
// (the parallel and the perpendicular one),
//     L_s = wt_s sum_c (y_c - y*_c)^T A_c (y_c - y*_c),   y_c = y[3c .. 3c+2],
// the squared relative force error its output error causes at the targets
// of the record (learn.cuh).
#include "mlp.cuh"
#include "tc.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>

namespace geon {

using namespace tc;

constexpr int MT = 128;          // samples per tile = threads per CTA = TMEM lanes
constexpr int K1 = 16;           // layer-1 K: 14 features, a constant 1, zeros
constexpr int N3 = 16;           // layer-3 N: 6 outputs, zeros
static_assert(LF + 1 <= K1 && LO <= N3, "layer shapes");
constexpr int NGA = LH + K1;     // N of the GA gradient GEMM
constexpr float GELU_C = 0.7978845608028654f;   // sqrt(2/pi)
constexpr float GELU_A = 0.044715f;

constexpr int OFF_MU = 0;                 // input normalisation x' = (x - mu) * isd (FP32, not trained)
constexpr int OFF_ISD = OFF_MU + LF;
constexpr int OFF_W1 = OFF_ISD + LF;
constexpr int OFF_B1 = OFF_W1 + LH * LF;
constexpr int OFF_W2 = OFF_B1 + LH;
constexpr int OFF_B2 = OFF_W2 + LH * LH;
constexpr int OFF_W3 = OFF_B2 + LH;
constexpr int OFF_B3 = OFF_W3 + LO * LH;
static_assert(OFF_B3 + LO == MLP_NPARAM, "weight layout");

// TMEM columns of the training CTA (512 allocated).
constexpr uint32_t TC_Z1 = 0, TC_Z2 = 64, TC_Y = 128, TC_DH2 = 160, TC_DH1 = 224, TC_GA = 288, TC_GB = 384;
static_assert(TC_GA + NGA <= TC_GB && TC_GB + N3 <= 512, "TMEM plan");

__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu(float x) {
    const float u = GELU_C * fmaf(GELU_A * x, x * x, x);
    return 0.5f * x * (1.f + tanh_approx(u));
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float x2 = x * x;
    const float t = tanh_approx(GELU_C * fmaf(GELU_A * x, x2, x));
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * GELU_C * fmaf(3.f * GELU_A, x2, 1.f);
}

// Forward operands, biases and the MMA barrier (every kernel of this file).
struct NetSmem {
    __align__(128) uint8_t w1[LH * K1 * 2];     // B of Z1 (N 64, K 16)
    __align__(128) uint8_t w2[LH * LH * 2];     // B of Z2 (N 64, K 64)
    __align__(128) uint8_t w3[N3 * LH * 2];     // B of Y  (N 16, K 64)
    __align__(128) uint8_t x[MT * K1 * 2];      // A of Z1
    __align__(128) uint8_t h1[MT * LH * 2];     // A of Z2
    __align__(128) uint8_t h2[MT * LH * 2];     // A of Y
    float b1[LH], b2[LH], b3[LO];
    float nmu[LF], nisd[LF];
    float red[MT / 32];
    uint64_t bar;
    uint32_t tmem;
};
// Inference CTA: the second hidden layer reuses the first layer's activation
// buffer and accumulator columns (GEMM 2 has consumed layer 1 before the
// epilogue overwrites it), so the network needs 33 KB of shared memory and 64
// TMEM columns per CTA.
struct InfSmem {
    __align__(128) uint8_t w1[LH * K1 * 2];
    __align__(128) uint8_t w2[LH * LH * 2];
    __align__(128) uint8_t w3[N3 * LH * 2];
    __align__(128) uint8_t x[MT * K1 * 2];
    __align__(128) uint8_t h[MT * LH * 2];      // A of Z2, then A of Y
    float b1[LH], b2[LH], b3[LO];
    float nmu[LF], nisd[LF];
    uint64_t bar;
    uint32_t tmem;
};
constexpr uint32_t INF_COLS = 64;

// Training adds the backward operands.
struct TrainSmem {
    NetSmem f;
    __align__(128) uint8_t w2t[LH * LH * 2];    // B of dH1 (N 64, K 64): W2^T
    __align__(128) uint8_t w3t[LH * N3 * 2];    // B of dH2 (N 64, K 16): W3^T
    __align__(128) uint8_t dy[MT * N3 * 2];     // A of dH2
    __align__(128) uint8_t dz2[MT * LH * 2];    // A of dH1
    __align__(128) uint8_t aga[MT * MT * 2];    // A of GA (128 rows, K = samples)
    __align__(128) uint8_t bga[NGA * MT * 2];   // B of GA
    __align__(128) uint8_t agb[MT * MT * 2];    // A of GB
    __align__(128) uint8_t bgb[N3 * MT * 2];    // B of GB
};

__device__ __forceinline__ void put_bf16(uint8_t* buf, int r, int k, int K, float v) {
    *reinterpret_cast<__nv_bfloat16*>(buf + kmajor_offset(r, k, K)) = __float2bfloat16_rn(v);
}
// Stores 8 consecutive values (k0 a multiple of 8) of row r as one 16-byte chunk.
__device__ __forceinline__ void put8(uint8_t* buf, int r, int k0, int K, const float* v) {
    uint4 u;
    __nv_bfloat162 p;
    p = __floats2bfloat162_rn(v[0], v[1]); u.x = *reinterpret_cast<uint32_t*>(&p);
    p = __floats2bfloat162_rn(v[2], v[3]); u.y = *reinterpret_cast<uint32_t*>(&p);
    p = __floats2bfloat162_rn(v[4], v[5]); u.z = *reinterpret_cast<uint32_t*>(&p);
    p = __floats2bfloat162_rn(v[6], v[7]); u.w = *reinterpret_cast<uint32_t*>(&p);
    *reinterpret_cast<uint4*>(buf + kmajor_offset(r, k0, K)) = u;
}

// Stages the FP32 weights as BF16 operands (zero padded) and FP32 biases.
template <class SM>
__device__ void stage_forward(SM& s, const float* __restrict__ W) {
    for (int i = threadIdx.x; i < LH * K1; i += blockDim.x) {
        const int r = i / K1, k = i % K1;
        put_bf16(s.w1, r, k, K1, k < LF ? W[OFF_W1 + r * LF + k] : 0.f);
    }
    for (int i = threadIdx.x; i < LH * LH; i += blockDim.x) put_bf16(s.w2, i / LH, i % LH, LH, W[OFF_W2 + i]);
    for (int i = threadIdx.x; i < N3 * LH; i += blockDim.x) {
        const int r = i / LH, k = i % LH;
        put_bf16(s.w3, r, k, LH, r < LO ? W[OFF_W3 + r * LH + k] : 0.f);
    }
    for (int i = threadIdx.x; i < LH; i += blockDim.x) { s.b1[i] = W[OFF_B1 + i]; s.b2[i] = W[OFF_B2 + i]; }
    if (threadIdx.x < LO) s.b3[threadIdx.x] = W[OFF_B3 + threadIdx.x];
    if (threadIdx.x < LF) { s.nmu[threadIdx.x] = W[OFF_MU + threadIdx.x]; s.nisd[threadIdx.x] = W[OFF_ISD + threadIdx.x]; }
}

// Input normalisation in FP32, before the features are rounded to BF16.
template <class SM>
__device__ __forceinline__ void normalise(const SM& s, float* x) {
#pragma unroll
    for (int k = 0; k < LF; k++) x[k] = (x[k] - s.nmu[k]) * s.nisd[k];
}

__device__ void stage_backward(TrainSmem& s, const float* __restrict__ W) {
    for (int i = threadIdx.x; i < LH * LH; i += blockDim.x) {
        const int n = i / LH, k = i % LH;                       // W2^T[n][k] = W2[k][n]
        put_bf16(s.w2t, n, k, LH, W[OFF_W2 + k * LH + n]);
    }
    for (int i = threadIdx.x; i < LH * N3; i += blockDim.x) {
        const int n = i / N3, k = i % N3;                       // W3^T[n][k] = W3[k][n]
        put_bf16(s.w3t, n, k, N3, k < LO ? W[OFF_W3 + k * LH + n] : 0.f);
    }
    // constant rows: GB's A operand has a row of ones (row 64) and zeros below;
    // GB's B operand rows 2..15 stay zero
    for (int i = threadIdx.x; i < (MT - LH) * MT; i += blockDim.x) {
        const int r = LH + i / MT, k = i % MT;
        put_bf16(s.agb, r, k, MT, r == LH ? 1.f : 0.f);
    }
    for (int i = threadIdx.x; i < (N3 - LO) * MT; i += blockDim.x) put_bf16(s.bgb, LO + i / MT, i % MT, MT, 0.f);
}

template <class SM>
__device__ __forceinline__ void net_setup(SM& s, uint32_t ncols) {
    if (threadIdx.x == 0) {
        mbar_init(&s.bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < 32) tmem_alloc(&s.tmem, ncols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
}

// Makes this CTA's shared-memory writes visible to the tensor core, lets
// thread 0 issue `issue()` and commit it, and waits for completion.  Returns
// false (uniformly across the CTA) if `ok` was false or the wait timed out;
// `phase` advances only on success so that a timed-out phase can be drained.
template <class SM, class F>
__device__ __forceinline__ bool mma_step(SM& s, uint32_t& phase, bool ok, F&& issue) {
    fence_proxy_async();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (!ok) return false;
    if (threadIdx.x == 0) {
        issue();
        commit(&s.bar);
    }
    const bool done = mbar_wait(&s.bar, phase);
    const bool all = __syncthreads_and(done) != 0;
    if (all) phase ^= 1u;
    fence_after_sync();
    return all;
}

template <class SM>
__device__ __forceinline__ void net_teardown(SM& s, bool ok, uint32_t phase, int* err, uint32_t ncols) {
    if (!ok) {
        if (threadIdx.x == 0) atomicOr(err, ERR_MMA_TIMEOUT);
        mbar_wait(&s.bar, phase);          // drain the MMA still in flight before the columns are released
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (threadIdx.x < 32) tmem_dealloc(s.tmem, ncols);
}

// GELU epilogue of a 64-column accumulator into the next layer's A operand
// (and, when training, into rows rowT0.. of a transposed operand).
template <bool TR>
__device__ __forceinline__ void hidden_epilogue(uint32_t tmem, uint32_t col, const float* bias, uint8_t* out,
                                                uint8_t* outT, int rowT0) {
    const int warp = threadIdx.x >> 5;
    const int row = threadIdx.x;
#pragma unroll
    for (int c0 = 0; c0 < LH; c0 += 16) {
        float v[16];
        tmem_ld16(tmem_addr(tmem, warp, col + c0), v);
#pragma unroll
        for (int i = 0; i < 16; i++) v[i] = gelu(v[i] + bias[c0 + i]);
        put8(out, row, c0, LH, v);
        put8(out, row, c0 + 8, LH, v + 8);
        if (TR) {
#pragma unroll
            for (int i = 0; i < 16; i++) put_bf16(outT, rowT0 + c0 + i, row, MT, v[i]);
        }
    }
}

template <class SM>
__device__ __forceinline__ void stage_x(SM& s, const float* f) {
    put8(s.x, threadIdx.x, 0, K1, f);
    put8(s.x, threadIdx.x, 8, K1, f + 8);
}

// ---- inference ---------------------------------------------------------------------
// Two GELUs (tanh form) in packed FP16 arithmetic, returned as the BF16 pair
// of the next layer's operand.  FP16 keeps 11 significant bits against the
// 8 of the BF16 result, so the result is the FP32 GELU's rounding to BF16
// up to an occasional last-place difference, at half the instructions.
__device__ __forceinline__ uint32_t gelu2_bf16(float x0, float x1) {
    const __half2 x = __floats2half2_rn(x0, x1);
    const __half2 x2 = __hmul2(x, x);
    const __half2 pq = __hfma2(x2, __float2half2_rn(GELU_C * GELU_A), __float2half2_rn(GELU_C));
    const __half2 u = __hmul2(pq, x);
    uint32_t ui = *reinterpret_cast<const uint32_t*>(&u), ti;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(ti) : "r"(ui));
    const __half2 t = *reinterpret_cast<const __half2*>(&ti);
    const __half2 hx = __hmul2(x, __float2half2_rn(0.5f));
    const float2 g = __half22float2(__hfma2(t, hx, hx));
    const __nv_bfloat162 b = __floats2bfloat162_rn(g.x, g.y);
    return *reinterpret_cast<const uint32_t*>(&b);
}

// GELU epilogue of a 64-column accumulator at column 0 into the next layer's
// A operand (BF16, as in training).
__device__ __forceinline__ void hidden_epilogue_inf(uint32_t tmem, const float* bias, uint8_t* out) {
    const int warp = threadIdx.x >> 5;
    const int row = threadIdx.x;
#pragma unroll
    for (int c0 = 0; c0 < LH; c0 += 16) {
        float v[16];
        tmem_ld16(tmem_addr(tmem, warp, c0), v);
        uint32_t g[8];
#pragma unroll
        for (int i = 0; i < 8; i++) g[i] = gelu2_bf16(v[2 * i] + bias[c0 + 2 * i], v[2 * i + 1] + bias[c0 + 2 * i + 1]);
        *reinterpret_cast<uint4*>(out + kmajor_offset(row, c0, LH)) = make_uint4(g[0], g[1], g[2], g[3]);
        *reinterpret_cast<uint4*>(out + kmajor_offset(row, c0 + 8, LH)) = make_uint4(g[4], g[5], g[6], g[7]);
    }
}

// Forward pass of the tile staged in s.x (64 TMEM columns, reused by every
// layer); y[LO] receives this thread's outputs.
__device__ __forceinline__ bool tile_forward(InfSmem& s, uint32_t& phase, bool ok, float* y) {
    const int warp = threadIdx.x >> 5;
    ok = mma_step(s, phase, ok, [&] { gemm(s.tmem + 0, s.x, s.w1, LH, K1, false); });
    hidden_epilogue_inf(s.tmem, s.b1, s.h);
    ok = mma_step(s, phase, ok, [&] { gemm(s.tmem + 0, s.h, s.w2, LH, LH, false); });
    hidden_epilogue_inf(s.tmem, s.b2, s.h);
    ok = mma_step(s, phase, ok, [&] { gemm(s.tmem + 0, s.h, s.w3, N3, LH, false); });
    float v[16];
    tmem_ld16(tmem_addr(s.tmem, warp, 0), v);
#pragma unroll
    for (int o = 0; o < LO; o++) y[o] = v[o] + s.b3[o];
    return ok;
}

__global__ void __launch_bounds__(MT)
mlp_forward_kernel(const float* __restrict__ W, const float* __restrict__ X, int n, float* __restrict__ Y, int* err) {
    extern __shared__ __align__(1024) uint8_t fwd_smem_raw[];
    InfSmem& s = *reinterpret_cast<InfSmem*>(fwd_smem_raw);
    stage_forward(s, W);
    net_setup(s, INF_COLS);
    uint32_t phase = 0;
    bool ok = true;
    const int ntiles = (n + MT - 1) / MT;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int i = tile * MT + threadIdx.x;
        float f[16];
#pragma unroll
        for (int k = 0; k < 16; k++) f[k] = (i < n && k < LF) ? X[(size_t)i * LF + k] : 0.f;
        normalise(s, f);
        f[LF] = 1.f;
        stage_x(s, f);
        float y[LO];
        ok = tile_forward(s, phase, ok, y);
        if (ok && i < n)
#pragma unroll
            for (int o = 0; o < LO; o++) Y[(size_t)i * LO + o] = y[o];
    }
    net_teardown(s, ok, phase, err, INF_COLS);
}

// ---- the correction inside the force pass -------------------------------------------
// Phase A1 (learn_geo_kernel) streams over the records of all groups in
// group order and writes each record's flags and analytic expansion
// (learn.cuh), listing the records near the Yukawa cutoff that the network
// applies to.  Phase A2 (learn_net_kernel) runs the network on that list in
// tiles of 128 on the tensor cores (several CTAs per SM hide one another's
// MMA waits) and adds its residual to the records' expansions.  Phase B
// (learn_apply_kernel) gives each group to one warp, lane l its target l:
// the warp runs through the group's records in order, and every accepting
// lane adds V + J (x - g), the exact analytic term for wide groups, and the
// Yukawa swap near the cutoff.  A warp owns its targets' forces, so the
// result does not depend on timing.
// Record layout of phase A's output: 3 float4 per record (48 bytes, so a
// warp's records fill whole sectors),
//   compact group: Gm.v, Gm.j, Ec.v, Ec.j (12 floats);
//   wide group:    (M, Ixx, Ixy, Iyy), (Dx, Dy, -, -), -;
// then, in a second region of one float4 per record written only for wide
// groups and records near the cutoff, the COM as (hi x, hi y, lo x, lo y);
// plus the cell mass for the Yukawa swap and the flags (uint32, mass as a
// float in the upper word of a uint2).  The buffer holds total x 16 floats:
// the expansions at expo, the COMs at expo + 3 total.
constexpr int EXP_F4 = 3;

// Largest g with off[g] <= e (off: exclusive prefix of the groups' counts).
__device__ __forceinline__ int group_of(const int* __restrict__ off, int ngroups, int e) {
    int lo = 0, hi = ngroups - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= e) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Phase A1: every record's geometry, flags and analytic expansion; the
// records the network applies to (REC_NET) are listed in net_list (in no
// fixed order: each list entry only adds to its own record, so the result
// does not depend on it).
constexpr int LG_THREADS = 256;
constexpr int LG_WARPS = LG_THREADS / 32;
__global__ void __launch_bounds__(LG_THREADS)
learn_geo_kernel(DevParams P, TreeBufs T, const uint2* __restrict__ recs, const int* __restrict__ rec_cnt,
                 const float4* __restrict__ gcen, int rec_cap, const int* __restrict__ off, int ngroups,
                 float4* __restrict__ expo, float4* __restrict__ cms, uint2* __restrict__ flags, int* __restrict__ net_list,
                 int* __restrict__ net_count, unsigned* __restrict__ queue) {
    const int lane = threadIdx.x & 31;
    // one warp per group, taken from *queue (zero at launch): its records
    // r = lane, lane + 32, ...; every record's outputs go to its own slots
    for (;;) {
        int g = 0;
        if (lane == 0) g = (int)atomicAdd(queue, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= ngroups) break;
        const int cnt = min(rec_cnt[g], rec_cap);
        const int base = off[g];
        const float4 gc = gcen[g];
        const int nround = (cnt + 31) & ~31;
        for (int r = lane; r < nround; r += 32) {
            const bool live = r < cnt;
            const int e = base + r;
            uint32_t fl = 0;
            if (live) {
                const uint2 rc = recs[(size_t)g * rec_cap + r];
                RecGeo R;
                float f[LF];
                record_geo(P, T, (int)rc.x, gc.x, gc.y, R, f);
                fl = record_flags(P, R, gc.z);
                float4* o = expo + (size_t)e * EXP_F4;
                if (fl & REC_EXACT) {
                    // wide groups: no expansion (phase B takes the analytic term per target)
                    o[0] = make_float4(R.M, R.ixx, R.ixy, R.iyy);
                    o[1] = make_float4(R.Dx, R.Dy, 0.f, 0.f);
                } else {
                    Lin Gm, Ec;
                    record_expansion(P, R, nullptr, false, Gm, Ec);
                    o[0] = make_float4(Gm.v[0], Gm.v[1], Gm.j[0], Gm.j[1]);
                    o[1] = make_float4(Gm.j[2], Gm.j[3], Ec.v[0], Ec.v[1]);
                    o[2] = make_float4(Ec.j[0], Ec.j[1], Ec.j[2], Ec.j[3]);
                }
                if (fl & (REC_EXACT | REC_NEAR_CUT)) {
                    const float4 na = T.int_a[rc.x], nc = T.int_c[rc.x];
                    cms[e] = make_float4(na.x, na.y, nc.x, nc.y);
                }
                flags[e] = make_uint2(fl, __float_as_uint(R.M));
            }
            const bool net = live && (fl & REC_NET);
            const unsigned bal = __ballot_sync(0xffffffffu, net);
            if (bal) {
                int b0 = 0;
                if (lane == 0) b0 = atomicAdd(net_count, __popc(bal));
                b0 = __shfl_sync(0xffffffffu, b0, 0);
                if (net) net_list[b0 + __popc(bal & lanemask_lt())] = e;
            }
        }
    }
}

// Phase A2: the network on the listed records, in tiles of 128 (thread t of
// a tile forms the features of its record, the tensor cores run the tile),
// its residual added to the record's mass-field expansion.  With EXT the
// outputs come from yext[e * 6 ...] instead.
template <bool EXT>
__global__ void __launch_bounds__(MT)
learn_net_kernel(DevParams P, TreeBufs T, const float* __restrict__ W, const uint2* __restrict__ recs,
                 const float4* __restrict__ gcen, int rec_cap, const int* __restrict__ off, int ngroups,
                 const int* __restrict__ net_list, const int* __restrict__ net_count, const float* __restrict__ yext,
                 float4* __restrict__ expo, int* err) {
    extern __shared__ __align__(1024) uint8_t ln_smem_raw[];
    InfSmem& s = *reinterpret_cast<InfSmem*>(ln_smem_raw);
    const int cnt = *net_count;
    const int ntiles = (cnt + MT - 1) / MT;
    if ((int)blockIdx.x >= ntiles) return;                 // uniform: no TMEM taken
    if (!EXT) stage_forward(s, W);
    net_setup(s, INF_COLS);
    uint32_t phase = 0;
    bool ok = true;
    const int tid = threadIdx.x;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int i = tile * MT + tid;
        const bool live = i < cnt;
        RecGeo R;
        float f[16];
#pragma unroll
        for (int c = 0; c < 16; c++) f[c] = 0.f;
        int e = 0;
        if (live) {
            e = net_list[i];
            const int g = group_of(off, ngroups, e);
            const uint2 rc = recs[(size_t)g * rec_cap + (e - off[g])];
            const float4 gc = gcen[g];
            record_geo(P, T, (int)rc.x, gc.x, gc.y, R, f);
        }
        float y[LO];
        if (EXT) {
#pragma unroll
            for (int o = 0; o < LO; o++) y[o] = live ? yext[(size_t)e * LO + o] : 0.f;
        } else {
            normalise(s, f);
            f[LF] = 1.f;
            stage_x(s, f);
            ok = tile_forward(s, phase, ok, y);
        }
        if (live && ok) {
            float4* o = expo + (size_t)e * EXP_F4;
            const float4 a0 = o[0], a1 = o[1];
            Lin Gm{ { a0.x, a0.y }, { a0.z, a0.w, a1.x, a1.y } };
            add_net_expansion(R, y, Gm);
            o[0] = make_float4(Gm.v[0], Gm.v[1], Gm.j[0], Gm.j[1]);
            o[1] = make_float4(Gm.j[2], Gm.j[3], a1.z, a1.w);
        }
    }
    net_teardown(s, ok, phase, err, INF_COLS);
}

__device__ __forceinline__ void yuk_unit_field(const DevParams& P, float rx, float ry, float& gx, float& gy) {
    const float rSq = __fmaf_rn(rx, rx, ry * ry) + P.softSq;
    const float invR = rsqrtf(rSq);
    const float r = rSq * invR;
    const float f = YUKAWA_COUPLING * __expf(-P.yukMu * r) * (invR * invR + P.yukMu * invR) * invR;
    gx = rx * f;
    gy = ry * f;
}

// The walk's own Yukawa decision for an aggregate source (force.cu
// yukawa_in): FP32 test, re-done in FP64 inside the guard band.
__device__ __forceinline__ bool walk_yukawa_in(const DevParams& P, float rx, float ry, float sx, float sxl, float sy,
                                               float syl, double tx, double ty) {
    const float rr = __fmaf_rn(rx, rx, ry * ry);
    const float cut = P.yukCutSq;
    if (fabsf(rr - cut) > 1e-6f * cut) return rr < cut;
    const double dx = ((double)sx + (double)sxl) - tx, dy = ((double)sy + (double)syl) - ty;
    return dx * dx + dy * dy < P.yukCutSqD;
}

constexpr int LA_THREADS = 256;
constexpr int LA_WARPS = LA_THREADS / 32;

// Phase B.  One warp per group, lane l its target l.  Records every target
// of the group accepts, and that need nothing per target, add the same
// expansion to all of them: the lanes sum those records (lane l takes
// records l, l + 32, ...) and a butterfly gives every lane the sums, so each
// target adds sum V + (sum J)(x - g).  The other records (some targets only,
// wide groups, near the cutoff) are staged 32 at a time in shared memory
// (coalesced loads, all in flight together) and read back in order as
// broadcasts by every lane.  Everything a record needs is in its phase-A
// output: no tree node is read here.  The summation order is fixed.  Warps
// take groups one at a time from *queue (zero at launch), so a warp that
// drew groups with many records does not hold up the end of the launch;
// which warp applies a group does not change its sums.
__global__ void __launch_bounds__(LA_THREADS)
learn_apply_kernel(DevParams P, DevState S, TreeBufs T, const FrameCtl* __restrict__ ctl, const uint2* __restrict__ recs,
                   const int* __restrict__ rec_cnt, const float4* __restrict__ gcen, int rec_cap, const int* __restrict__ off,
                   const float4* __restrict__ expo, const float4* __restrict__ cms, const uint2* __restrict__ flags,
                   unsigned* __restrict__ queue) {
    __shared__ float4 st[LA_WARPS][32][5];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = ctl->n;
    const int ngroups = (n + 31) / 32;
    for (;;) {
        int g = 0;
        if (lane == 0) g = (int)atomicAdd(queue, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= ngroups) break;
        const int k = g * 32 + lane;
        int ti = k < n ? T.tgt[k] : -1;
        if (ti >= n) ti = -1;
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 pl = make_float2(0.f, 0.f);
        if (ti >= 0) { p = S.pos[ti]; pl = S.pos_lo[ti]; }
        const float4 gc = gcen[g];
        const float ox = __fadd_rn(__fsub_rn(p.x, gc.x), pl.x), oy = __fadd_rn(__fsub_rn(p.y, gc.y), pl.y);
        const double txd = (double)p.x + (double)pl.x, tyd = (double)p.y + (double)pl.y;
        const unsigned bit = ti >= 0 ? (1u << lane) : 0u;
        const unsigned active = __ballot_sync(0xffffffffu, ti >= 0);
        const int cnt = min(rec_cnt[g], rec_cap);
        const int base = off[g];
        // records shared by the whole group: lane sums, then a butterfly
        float sv[12];
#pragma unroll
        for (int c = 0; c < 12; c++) sv[c] = 0.f;
        const int nround = (cnt + 31) & ~31;
        float G0 = 0.f, G1 = 0.f, E0 = 0.f, E1 = 0.f;
        for (int c0 = 0; c0 < nround; c0 += 32) {
            const int r = c0 + lane;
            uint32_t mask = 0u;
            uint2 fm = make_uint2(0u, 0u);
            const float4* o = expo + (size_t)(base + r) * EXP_F4;
            if (r < cnt) {
                mask = recs[(size_t)g * rec_cap + r].y;
                fm = flags[base + r];
            }
            const bool shared = r < cnt && mask == active && !(fm.x & (REC_EXACT | REC_NEAR_CUT));
            if (shared) {
                const float4 a0 = o[0], a1 = o[1], a2 = o[2];
                sv[0] += a0.x; sv[1] += a0.y; sv[2] += a0.z; sv[3] += a0.w;
                sv[4] += a1.x; sv[5] += a1.y; sv[6] += a1.z; sv[7] += a1.w;
                sv[8] += a2.x; sv[9] += a2.y; sv[10] += a2.z; sv[11] += a2.w;
            }
            // the rest, compacted into shared memory in record order
            const bool own = r < cnt && !shared && mask != 0u;
            const unsigned ob = __ballot_sync(0xffffffffu, own);
            if (own) {
                const int q = __popc(ob & lanemask_lt());
                st[w][q][0] = o[0];
                st[w][q][1] = o[1];
                st[w][q][2] = o[2];
                if (fm.x & (REC_EXACT | REC_NEAR_CUT)) st[w][q][3] = cms[base + r];
                st[w][q][4] = make_float4(__uint_as_float(mask), __uint_as_float(fm.x), __uint_as_float(fm.y), 0.f);
            }
            __syncwarp();
            const int m = __popc(ob);
            for (int j = 0; j < m; j++) {
                const float4 meta = st[w][j][4];
                if (!(__float_as_uint(meta.x) & bit)) continue;
                const uint32_t fl = __float_as_uint(meta.y);
                const float4 a0 = st[w][j][0], a1 = st[w][j][1];
                if (!(fl & REC_EXACT)) {
                    const float4 a2 = st[w][j][2];
                    G0 += a0.x + a0.z * ox + a0.w * oy;
                    G1 += a0.y + a1.x * ox + a1.y * oy;
                    E0 += a1.z + a2.x * ox + a2.y * oy;
                    E1 += a1.w + a2.z * ox + a2.w * oy;
                }
                if (fl & (REC_EXACT | REC_NEAR_CUT)) {
                    const float4 cm = st[w][j][3];
                    const float rx = __fadd_rn(__fsub_rn(cm.x, p.x), cm.z - pl.x);
                    const float ry = __fadd_rn(__fsub_rn(cm.y, p.y), cm.w - pl.y);
                    const bool ownY = P.yukOn && walk_yukawa_in(P, rx, ry, cm.x, cm.z, cm.y, cm.w, txd, tyd);
                    if (fl & REC_EXACT) {
                        // wide group: the analytic term at this target with its own
                        // Yukawa decision (the one its monopole took), no network
                        RecGeo R;
                        R.ixx = a0.y; R.ixy = a0.z; R.iyy = a0.w; R.Dx = a1.x; R.Dy = a1.y; R.yg = ownY;
                        float gx, gy, ex, ey;
                        analytic_at(P, R, rx, ry, gx, gy, ex, ey);
                        G0 += gx; G1 += gy; E0 += ex; E1 += ey;
                    } else {
                        // near the cutoff: the group's Yukawa decision, formed as record_geo forms it
                        const float gdx = __fadd_rn(__fsub_rn(cm.x, gc.x), cm.z), gdy = __fadd_rn(__fsub_rn(cm.y, gc.y), cm.w);
                        const bool yg = P.yukOn && gdx * gdx + gdy * gdy < P.yukCutSq;
                        if (ownY != yg) {
                            float yx, yy;
                            yuk_unit_field(P, rx, ry, yx, yy);
                            const float M = meta.z;
                            const float sg = ownY ? -M : M;
                            G0 += sg * yx;
                            G1 += sg * yy;
                        }
                    }
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int c = 0; c < 12; c++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sv[c] += __shfl_xor_sync(0xffffffffu, sv[c], o);
        G0 += sv[0] + sv[2] * ox + sv[3] * oy;
        G1 += sv[1] + sv[4] * ox + sv[5] * oy;
        E0 += sv[6] + sv[8] * ox + sv[9] * oy;
        E1 += sv[7] + sv[10] * ox + sv[11] * oy;
        if (ti >= 0) {
            float4 F = S.force[ti];
            F.x += p.z * G0 + p.w * E0;
            F.y += p.z * G1 + p.w * E1;
            S.force[ti] = F;
        }
    }
}

// SplitMix64 finaliser (Steele, Lea, Flood 2014) of a (seed, step, j) counter,
// mapped to [0, n) by a 32 x 32 -> 64-bit multiply.
__device__ __forceinline__ int draw_sample(uint64_t seed, int step, int j, int n) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (((uint64_t)(uint32_t)step << 32) + (uint64_t)(uint32_t)j + 1ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (int)(((z >> 32) * (uint64_t)(uint32_t)n) >> 32);
}

__global__ void __launch_bounds__(MT, 1)
mlp_train_kernel(const float* __restrict__ W, const float* __restrict__ X, const float* __restrict__ Tg,
                 const float* __restrict__ wt, int n_data, int batch, uint64_t seed, int step,
                 float* __restrict__ part_all, double* __restrict__ loss_part, int* err) {
    // this CTA's gradient slot: every element is written exactly once (summed
    // over the CTAs in a fixed order afterwards, so training is reproducible)
    float* __restrict__ grad = part_all + (size_t)blockIdx.x * MLP_NPARAM;
    extern __shared__ __align__(1024) uint8_t tr_smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(tr_smem_raw);
    NetSmem& f = s.f;
    stage_forward(f, W);
    stage_backward(s, W);
    net_setup(f, 512);
    const int warp = threadIdx.x >> 5;
    const int row = threadIdx.x;
    const float invB = 1.f / (float)batch;
    uint32_t phase = 0;
    bool ok = true, first = true;
    float lsum = 0.f;
    const int ntiles = (batch + MT - 1) / MT;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int j = tile * MT + row;
        const bool live = j < batch;
        const int smp = !live ? -1 : (seed ? draw_sample(seed, step, j, n_data) : j);
        float x[16];
#pragma unroll
        for (int k = 0; k < 16; k++) x[k] = 0.f;
        float tg[LT], w = 0.f;
#pragma unroll
        for (int k = 0; k < LT; k++) tg[k] = 0.f;
        if (smp >= 0) {
#pragma unroll
            for (int k = 0; k < LF; k++) x[k] = X[(size_t)smp * LF + k];
#pragma unroll
            for (int k = 0; k < LT; k++) tg[k] = Tg[(size_t)smp * LT + k];
            w = wt ? wt[smp] : 1.f;
        }
        normalise(f, x);
        x[LF] = 1.f;
        stage_x(f, x);
#pragma unroll
        for (int k = 0; k < K1; k++) put_bf16(s.bga, LH + k, row, MT, x[k]);
        // forward
        ok = mma_step(f, phase, ok, [&] { gemm(f.tmem + TC_Z1, f.x, f.w1, LH, K1, false); });
        hidden_epilogue<true>(f.tmem, TC_Z1, f.b1, f.h1, s.bga, 0);
        ok = mma_step(f, phase, ok, [&] { gemm(f.tmem + TC_Z2, f.h1, f.w2, LH, LH, false); });
        hidden_epilogue<true>(f.tmem, TC_Z2, f.b2, f.h2, s.agb, 0);
        ok = mma_step(f, phase, ok, [&] { gemm(f.tmem + TC_Y, f.h2, f.w3, N3, LH, false); });
        {
            float v[16];
            tmem_ld16(tmem_addr(f.tmem, warp, TC_Y), v);
            // per component c: e = y_c - y*_c, loss e^T A_c e, gradient 2 A_c e
            const float g = 2.f * w * invB;
            float d[16];
#pragma unroll
            for (int k = 0; k < 16; k++) d[k] = 0.f;
#pragma unroll
            for (int c = 0; c < 2; c++) {
                const float e0 = v[3 * c] + f.b3[3 * c] - tg[3 * c];
                const float e1 = v[3 * c + 1] + f.b3[3 * c + 1] - tg[3 * c + 1];
                const float e2 = v[3 * c + 2] + f.b3[3 * c + 2] - tg[3 * c + 2];
                const float* A = tg + LO + 6 * c;           // A00 A11 A22 A01 A02 A12
                const float a0 = A[0] * e0 + A[3] * e1 + A[4] * e2;
                const float a1 = A[3] * e0 + A[1] * e1 + A[5] * e2;
                const float a2 = A[4] * e0 + A[5] * e1 + A[2] * e2;
                lsum += w * (e0 * a0 + e1 * a1 + e2 * a2);
                d[3 * c] = g * a0;
                d[3 * c + 1] = g * a1;
                d[3 * c + 2] = g * a2;
            }
            put8(s.dy, row, 0, N3, d);
            put8(s.dy, row, 8, N3, d + 8);
#pragma unroll
            for (int o = 0; o < LO; o++) put_bf16(s.bgb, o, row, MT, d[o]);
        }
        // backward through layer 3 and the second GELU
        ok = mma_step(f, phase, ok, [&] { gemm(f.tmem + TC_DH2, s.dy, s.w3t, LH, N3, false); });
#pragma unroll
        for (int c0 = 0; c0 < LH; c0 += 16) {
            float dh[16], z[16];
            tmem_ld16(tmem_addr(f.tmem, warp, TC_DH2 + c0), dh);
            tmem_ld16(tmem_addr(f.tmem, warp, TC_Z2 + c0), z);
#pragma unroll
            for (int i = 0; i < 16; i++) dh[i] *= gelu_grad(z[i] + f.b2[c0 + i]);
            put8(s.dz2, row, c0, LH, dh);
            put8(s.dz2, row, c0 + 8, LH, dh + 8);
#pragma unroll
            for (int i = 0; i < 16; i++) put_bf16(s.aga, c0 + i, row, MT, dh[i]);
        }
        // backward through layer 2 and the first GELU
        ok = mma_step(f, phase, ok, [&] { gemm(f.tmem + TC_DH1, s.dz2, s.w2t, LH, LH, false); });
#pragma unroll
        for (int c0 = 0; c0 < LH; c0 += 16) {
            float dh[16], z[16];
            tmem_ld16(tmem_addr(f.tmem, warp, TC_DH1 + c0), dh);
            tmem_ld16(tmem_addr(f.tmem, warp, TC_Z1 + c0), z);
#pragma unroll
            for (int i = 0; i < 16; i++) put_bf16(s.aga, LH + c0 + i, row, MT, dh[i] * gelu_grad(z[i] + f.b1[c0 + i]));
        }
        // weight gradients of this tile, accumulated in TMEM
        const bool acc = !first;
        ok = mma_step(f, phase, ok, [&] {
            gemm(f.tmem + TC_GA, s.aga, s.bga, NGA, MT, acc);
            gemm(f.tmem + TC_GB, s.agb, s.bgb, N3, MT, acc);
        });
        first = false;
    }
    // loss
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((row & 31) == 0) f.red[warp] = lsum;
    __syncthreads();
    if (row == 0) loss_part[blockIdx.x] = ok ? (double)(f.red[0] + f.red[1] + f.red[2] + f.red[3]) * (double)invB : 0.0;
    // gradients: TMEM lane r holds row r of GA and of GB
    for (int i = row; i < OFF_W1; i += MT) grad[i] = 0.f;      // the normalisation is not trained
    if (!ok || first) {
        for (int i = row; i < MLP_NPARAM; i += MT) grad[i] = 0.f;
    } else {
        const bool top = row < LH;
        const int o = top ? row : row - LH;
#pragma unroll
        for (int c0 = 0; c0 < LH; c0 += 16) {
            float v[16];
            tmem_ld16(tmem_addr(f.tmem, warp, TC_GA + c0), v);
            if (top) {
#pragma unroll
                for (int i = 0; i < 16; i++) grad[OFF_W2 + o * LH + c0 + i] = v[i];
            }
        }
        {
            float v[16];
            tmem_ld16(tmem_addr(f.tmem, warp, TC_GA + LH), v);
            if (top) {
                grad[OFF_B2 + o] = v[LF];
            } else {
#pragma unroll
                for (int k = 0; k < LF; k++) grad[OFF_W1 + o * LF + k] = v[k];
                grad[OFF_B1 + o] = v[LF];
            }
        }
        {
            float v[16];
            tmem_ld16(tmem_addr(f.tmem, warp, TC_GB), v);
            if (top) {
#pragma unroll
                for (int o = 0; o < LO; o++) grad[OFF_W3 + o * LH + row] = v[o];
            } else if (row == LH) {
#pragma unroll
                for (int o = 0; o < LO; o++) grad[OFF_B3 + o] = v[o];
            }
        }
    }
    net_teardown(f, ok, phase, err, 512);
}

// grad += sum over the CTAs of their slots, loss += sum of their losses, in CTA order.
__global__ void mlp_reduce_kernel(const float* __restrict__ part, const double* __restrict__ loss_part, int nb,
                                  float* __restrict__ grad, double* loss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < MLP_NPARAM) {
        float acc = 0.f;
        for (int b = 0; b < nb; b++) acc += part[(size_t)b * MLP_NPARAM + i];
        grad[i] += acc;
    }
    if (i == 0) {
        double l = 0.0;
        for (int b = 0; b < nb; b++) l += loss_part[b];
        *loss += l;
    }
}

__global__ void mlp_adam_kernel(float* W, float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                                float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_NPARAM) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    W[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    g[i] = 0.f;
}

// ---- launchers ------------------------------------------------------------------
static int sm_count() { return device_sms(); }

template <class K>
static void allow_smem(K kernel, size_t bytes, bool& done) {
    if (!done) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        done = true;
    }
}

constexpr size_t NET_SMEM = sizeof(InfSmem) + 1024;
constexpr size_t TRAIN_SMEM = sizeof(TrainSmem) + 1024;
static_assert(TRAIN_SMEM <= 227 * 1024, "training CTA exceeds shared memory");
// one training CTA per SM: its 512 TMEM columns are the whole TMEM of the SM
static_assert(2 * TRAIN_SMEM > 228 * 1024, "training CTAs must not share an SM");
// at most eight inference CTAs per SM: 8 x 64 TMEM columns
static_assert(9 * NET_SMEM > 228 * 1024, "inference CTAs would oversubscribe TMEM");

void mlp_forward(const float* W, const float* X, int n, float* Y, int* err, cudaStream_t st, LaunchCounter& lc) {
    static bool attr = false;
    allow_smem(mlp_forward_kernel, NET_SMEM, attr);
    if (n <= 0) return;
    const int tiles = (n + MT - 1) / MT;
    const int blocks = std::max(1, std::min(tiles, sm_count() * 6));
    mlp_forward_kernel<<<blocks, MT, NET_SMEM, st>>>(W, X, n, Y, err);
    lc.add(1);
}

void learn_correct(const DevParams& P, const DevState& S, const TreeBufs& T, const FrameCtl* ctl, const float* W,
                   const uint2* recs, const int* rec_cnt, const float4* gcen, int rec_cap, int ngroups, const int* off,
                   int total, const float* yext, float4* expo, uint2* flags, int* net_list, int* net_count,
                   unsigned* group_queue, int* err, cudaStream_t st, LaunchCounter& lc) {
    static bool a0 = false, a1 = false;
    allow_smem(learn_net_kernel<false>, NET_SMEM, a0);
    allow_smem(learn_net_kernel<true>, NET_SMEM, a1);
    if (ngroups <= 0) return;
    if (total > 0) {
        cudaMemsetAsync(net_count, 0, sizeof(int), st);
        const int gblocks = std::max(1, std::min((ngroups + LG_WARPS - 1) / LG_WARPS, sm_count() * 8));
        cudaMemsetAsync(group_queue, 0, sizeof(unsigned), st);
        learn_geo_kernel<<<gblocks, LG_THREADS, 0, st>>>(P, T, recs, rec_cnt, gcen, rec_cap, off, ngroups, expo,
                                                         expo + (size_t)EXP_F4 * total, flags, net_list, net_count,
                                                         group_queue);
        // the network's CTAs: enough for every listed record (the count is read on the device)
        const int tiles = (total + MT - 1) / MT;
        const int blocks = std::max(1, std::min(tiles, sm_count() * 6));
        if (yext) learn_net_kernel<true><<<blocks, MT, NET_SMEM, st>>>(P, T, W, recs, gcen, rec_cap, off, ngroups,
                                                                       net_list, net_count, yext, expo, err);
        else learn_net_kernel<false><<<blocks, MT, NET_SMEM, st>>>(P, T, W, recs, gcen, rec_cap, off, ngroups, net_list,
                                                                    net_count, nullptr, expo, err);
        lc.add(2);
    }
    const int blocks = std::max(1, std::min((ngroups + LA_WARPS - 1) / LA_WARPS, sm_count() * 8));
    cudaMemsetAsync(group_queue, 0, sizeof(unsigned), st);
    learn_apply_kernel<<<blocks, LA_THREADS, 0, st>>>(P, S, T, ctl, recs, rec_cnt, gcen, rec_cap, off, expo,
                                                      expo + (size_t)EXP_F4 * std::max(total, 0), flags, group_queue);
    lc.add(1);
}

size_t mlp_grad_scratch_floats() { return (size_t)sm_count() * MLP_NPARAM; }
int mlp_grad_scratch_ctas() { return sm_count(); }

void mlp_grad(const float* W, const float* X, const float* T, const float* wt, int n_data, int batch, uint64_t seed,
              int step, float* grad, double* loss, float* part, double* loss_part, int* err, cudaStream_t st,
              LaunchCounter& lc) {
    static bool attr = false;
    allow_smem(mlp_train_kernel, TRAIN_SMEM, attr);
    if (batch <= 0 || n_data <= 0) return;
    const int tiles = (batch + MT - 1) / MT;
    const int blocks = std::max(1, std::min(tiles, sm_count()));
    mlp_train_kernel<<<blocks, MT, TRAIN_SMEM, st>>>(W, X, T, wt, n_data, batch, seed, step, part, loss_part, err);
    mlp_reduce_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(part, loss_part, blocks, grad, loss);
    lc.add(2);
}

void mlp_adam(float* W, float* grad, float* m, float* v, float lr, float beta1, float beta2, float eps, int t,
              cudaStream_t st, LaunchCounter& lc) {
    const float c1 = (float)(1.0 - std::pow((double)beta1, (double)t));
    const float c2 = (float)(1.0 - std::pow((double)beta2, (double)t));
    mlp_adam_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(W, grad, m, v, lr, beta1, beta2, eps, c1, c2);
    lc.add(1);
}

}  // namespace geon
