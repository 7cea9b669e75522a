// common.cuh — device-side definitions shared by every translation unit of
// libgeon_cuda.so: physics constants (src/config.js), the launch parameter
// block, compensated-FP32 ("df64") arithmetic and the minimum-image helpers
// (src/topology.js).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/geon.h"

namespace geon {

// ---- physics constants (src/config.js) ------------------------------------
constexpr float  EPS_F = 1e-12f;           // EPSILON, config.js:30
constexpr double EPS_D = 1e-12;
constexpr float  INERTIA_K = 0.4f;         // config.js:52
constexpr float  MAG_MOMENT_K = 0.2f;      // config.js:53
constexpr float  TIDAL_STRENGTH = 64.f;    // config.js:54
constexpr float  YUKAWA_COUPLING = 14.f;   // config.js:80
constexpr int    LEAF_CAP = 4;             // QUADTREE_CAPACITY, config.js:59
constexpr int    HIST_LEN = 256;           // HISTORY_SIZE, config.js:120
constexpr int    HIST_MASK = 255;
constexpr int    HIST_STRIDE = 64;         // config.js:122
constexpr double DESPAWN_MARGIN = 64.0;    // config.js:138
constexpr int    KEY_LEVELS = 31;          // Morton levels kept in a 62-bit key
constexpr uint64_t KEY_INVALID = 1ull << 63;   // point outside the closed root box
constexpr int    MAX_GHOSTS_PER_PARTICLE = 8;
constexpr int    WALK_STACK = 128;         // per-warp stack entries (depth 31 needs <= 97)

// ---- error flags raised on the device --------------------------------------
constexpr int ERR_STACK_OVERFLOW = 1;
constexpr int ERR_NODE_OVERFLOW = 2;
constexpr int ERR_AGG_TIMEOUT = 4;
constexpr int ERR_BAD_INDEX = 8;        // an index failed its bounds check (access skipped)
constexpr int ERR_MMA_TIMEOUT = 16;     // a tensor-core completion wait ran out (kernel returned early)
constexpr int ERR_FRAME_TIMEOUT = 32;   // a grid-wide barrier of the frame kernel ran out (kernel returned early)

// ---- point references: particle index + periodic image code ----------------
// code bits: [0,1] sx+1, [2,3] sy+1, [4] mirror x (x -> W - x), [5] mirror y,
// [6] flip vx, [7] flip vy.  A ghost (integrator.js:176-244) is its original
// particle seen through one of these transforms.
constexpr int REF_SHIFT = 24;
constexpr uint32_t REF_INDEX_MASK = (1u << REF_SHIFT) - 1;
__host__ __device__ inline uint32_t make_ref(uint32_t idx, uint32_t code) { return idx | (code << REF_SHIFT); }
__host__ __device__ inline uint32_t ref_index(uint32_t r) { return r & REF_INDEX_MASK; }
__host__ __device__ inline uint32_t ref_code(uint32_t r) { return r >> REF_SHIFT; }
__host__ __device__ inline int code_sx(uint32_t c) { return (int)(c & 3u) - 1; }
__host__ __device__ inline int code_sy(uint32_t c) { return (int)((c >> 2) & 3u) - 1; }
__host__ __device__ inline bool code_mx(uint32_t c) { return (c >> 4) & 1u; }
__host__ __device__ inline bool code_my(uint32_t c) { return (c >> 5) & 1u; }
__host__ __device__ inline bool code_fvx(uint32_t c) { return (c >> 6) & 1u; }
__host__ __device__ inline bool code_fvy(uint32_t c) { return (c >> 7) & 1u; }
constexpr uint32_t CODE_IDENTITY = 1u | (1u << 2);   // sx = sy = 0, no mirror, no flip

// ---- launch parameter block (passed by value) ----------------------------------
struct DevParams {
    uint32_t toggles, flags;
    int boundary, topology;
    int periodic;          // boundary == LOOP
    int ghosts;            // periodic and ghosts enabled
    int rel;               // relativity on
    int n_cap;             // particle capacity
    // domain
    double Wd, Hd, offXd, offYd;
    float W, H, halfW, halfH;
    float W_lo, H_lo;      // W - (float)W, for compensated shifts
    // root box (integrator.js:727-730) and key quantisation
    double rootX, rootY, rootW, rootH;
    int exact_grid;        // 1 when every node centre down to KEY_LEVELS is exact in FP64
    // forces
    float softSq, soft;
    float thetaSq;
    double thetaSqD, thetaD;
    float yukMu;
    float yukCutSq;        // (6/mu)^2, forces.js:82-83
    double yukCutSqD;
    int yukOn;
    // external fields (integrator.js:553-593)
    float extGx, extGy, extEx, extEy, extBz;
    float friction;
    // batched systems: nsys > 0 when one handle holds several independent
    // systems; tree keys are then (system << 54) | 27-level Morton code
    int nsys;
    int keyTop;            // key bits above the Morton code (2: invalid flag + spare; 10 batched)
    int keyLevels;         // Morton levels in a key (31; 27 batched)
};

constexpr int BATCH_MAX_SYSTEMS = 512;   // 9 system bits above a 54-bit Morton code
constexpr int BATCH_KEY_LEVELS = 27;

// ---- frame control block in device memory --------------------------------------
struct FrameCtl {
    unsigned long long maxAccelSqBits;  // max |F|^2/m^2 over the current forces (double bits)
    unsigned long long maxCycBits;      // max cyclotron frequency (double bits)
    unsigned long long interactions;    // walk interaction counter
    int n;                 // alive particles
    int nGhost;            // ghosts of the current tree
    int nPts;              // n + nGhost
    int nValid;            // points inside the root box
    int nInternal;         // divided nodes
    int nLeaves;           // non-empty leaves
    int nBucket;           // leaves at KEY_LEVELS holding more than LEAF_CAP points
    int maxLevel;
    int err;               // ERR_* bits
    int nRemoved;          // despawned this frame
    int histCount;         // samples recorded so far (saturates at 2^30)
    int pad;
};

// ---- df64: unevaluated sum hi + lo of two floats -----------------------------------
struct df { float hi, lo; };

__device__ __forceinline__ df two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return { s, err };
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {   // |a| >= |b|
    float s = __fadd_rn(a, b);
    float err = __fsub_rn(b, __fsub_rn(s, a));
    return { s, err };
}
__device__ __forceinline__ df two_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    float err = __fmaf_rn(a, b, -p);
    return { p, err };
}
__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    df t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
    df p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_div_f(df a, float b) {
    float q1 = __fdiv_rn(a.hi, b);
    df p = two_prod(q1, b);
    float r = __fsub_rn(__fsub_rn(a.hi, p.hi), p.lo);
    r = __fadd_rn(r, a.lo);
    float q2 = __fdiv_rn(r, b);
    return fast_two_sum(q1, q2);
}
__device__ __forceinline__ df df_from_double(double v) {
    float hi = (float)v;
    float lo = (float)(v - (double)hi);
    return { hi, lo };
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

// Compensated accumulator: partial FP32 sums are flushed into (hi, lo) pairs.
struct CAcc {
    float hi, lo;
    __device__ __forceinline__ void init() { hi = 0.f; lo = 0.f; }
    __device__ __forceinline__ void add(float v) {
        df s = two_sum(hi, v);
        hi = s.hi; lo = __fadd_rn(lo, s.lo);
    }
    __device__ __forceinline__ float value() const { return __fadd_rn(hi, lo); }
};

// ---- minimum image (topology.js:9-76) in FP32 with compensated wrap ---------------------
__device__ __forceinline__ float torus_wrap_f(float d, float full, float half) {   // topology.js:9-12
    if (d > half) d -= full; else if (d < -half) d += full;
    return d;
}

// Exact-rounded displacement along one periodic axis: a - b + k*L, where
// (a - b) is formed error-free and k in {-1, 0, 1} is chosen by the wrap.
__device__ __forceinline__ float wrap_axis_comp(float a, float b, float a_lo, float L, float L_lo, float half) {
    df d = two_sum(a, -b);
    d.lo = __fadd_rn(d.lo, a_lo);
    float approx = __fadd_rn(d.hi, d.lo);
    float k = 0.f;
    if (approx > half) k = -1.f; else if (approx < -half) k = 1.f;
    if (k == 0.f) return approx;
    df s = two_sum(d.hi, k * L);
    return __fadd_rn(s.hi, __fadd_rn(s.lo, __fadd_rn(d.lo, k * L_lo)));
}

// FP64 minimum image, used for Klein / RP^2 and for guard-band re-tests.
__device__ __forceinline__ double torus_wrap_d(double d, double full, double half) {
    if (d > half) d -= full; else if (d < -half) d += full;
    return d;
}
// FP64 minimum image on the torus (the torus case of min_image_d).
__device__ __forceinline__ void torus_image_d(double ox, double oy, double sx, double sy, double W, double H,
                                              double& rx, double& ry) {
    rx = torus_wrap_d(sx - ox, W, W * 0.5);
    ry = torus_wrap_d(sy - oy, H, H * 0.5);
}
__device__ inline void min_image_d(double ox, double oy, double sx, double sy, int topology,
                                   double W, double H, double& rx, double& ry) {
    if (topology == GEON_TORUS) { torus_image_d(ox, oy, sx, sy, W, H, rx, ry); return; }
    const double halfW = W * 0.5;
    auto tw = [](double d, double full, double half) { return torus_wrap_d(d, full, half); };
    double dx = sx - ox, dy = sy - oy;
    const double doubleH = 2 * H;
    if (topology == GEON_KLEIN) {
        double bx = tw(dx, W, halfW), by = dy;
        double bestDx = bx, bestDy = by, bestSq = bx * bx + by * by;
        double cx = tw((W - sx) - ox, W, halfW), cy = tw((sy + H) - oy, doubleH, H);
        double sq = cx * cx + cy * cy;
        if (sq < bestSq) { bestDx = cx; bestDy = cy; }
        rx = bestDx; ry = bestDy; return;
    }
    const double doubleW = 2 * W;
    double bestDx = dx, bestDy = dy, bestSq = dx * dx + dy * dy;
    double cx = (W - sx) - ox, cy = tw((sy + H) - oy, doubleH, H);
    double sq = cx * cx + cy * cy;
    if (sq < bestSq) { bestDx = cx; bestDy = cy; bestSq = sq; }
    cx = tw((sx + W) - ox, doubleW, W); cy = (H - sy) - oy;
    sq = cx * cx + cy * cy;
    if (sq < bestSq) { bestDx = cx; bestDy = cy; bestSq = sq; }
    cx = tw((2 * W - sx) - ox, doubleW, W); cy = tw((2 * H - sy) - oy, doubleH, H);
    sq = cx * cx + cy * cy;
    if (sq < bestSq) { bestDx = cx; bestDy = cy; }
    rx = bestDx; ry = bestDy;
}

// Displacement from observer (ox, oy) to a source whose position is the
// unevaluated sum (sx + sx_lo, sy + sy_lo): plain difference, torus wrap with
// compensation, or the FP64 path for the non-orientable topologies.
__device__ __forceinline__ void displacement(const DevParams& P, float ox, float oy,
                                             float sx, float sx_lo, float sy, float sy_lo,
                                             float& rx, float& ry) {
    if (!P.periodic) {
        rx = __fadd_rn(__fsub_rn(sx, ox), sx_lo);
        ry = __fadd_rn(__fsub_rn(sy, oy), sy_lo);
    } else if (P.topology == GEON_TORUS) {
        rx = wrap_axis_comp(sx, ox, sx_lo, P.W, P.W_lo, P.halfW);
        ry = wrap_axis_comp(sy, oy, sy_lo, P.H, P.H_lo, P.halfH);
    } else {
        double dx, dy;
        min_image_d((double)ox, (double)oy, (double)sx + (double)sx_lo, (double)sy + (double)sy_lo,
                    P.topology, P.Wd, P.Hd, dx, dy);
        rx = (float)dx; ry = (float)dy;
    }
}

// Image position of particle (x, y) under a point code, in FP64 with the
// reference's evaluation order (integrator.js:214-241: "W - x + W" is
// (W - x) + W).
__host__ __device__ inline void image_pos_d(double x, double y, uint32_t code, double W, double H,
                                            double& gx, double& gy) {
    const int sx = code_sx(code), sy = code_sy(code);
    double bx = code_mx(code) ? (W - x) : x;
    double by = code_my(code) ? (H - y) : y;
    gx = sx == 0 ? bx : (sx > 0 ? bx + W : bx - W);
    gy = sy == 0 ? by : (sy > 0 ? by + H : by - H);
}

// Image position of particle (x + xlo, y + ylo) under a point code, as
// compensated pairs (ghost shifts and mirrors, integrator.js:176-244).
__device__ __forceinline__ void point_image(const DevParams& P, float x, float y, float xlo, float ylo, uint32_t code,
                                            float& ix, float& ixlo, float& iy, float& iylo) {
    if (code == CODE_IDENTITY) { ix = x; ixlo = xlo; iy = y; iylo = ylo; return; }
    df a = code_mx(code) ? df_add(df{ P.W, P.W_lo }, df{ -x, -xlo }) : df{ x, xlo };
    df b = code_my(code) ? df_add(df{ P.H, P.H_lo }, df{ -y, -ylo }) : df{ y, ylo };
    const int sx = code_sx(code), sy = code_sy(code);
    if (sx) a = df_add(a, df{ sx * P.W, sx * P.W_lo });
    if (sy) b = df_add(b, df{ sy * P.H, sy * P.H_lo });
    ix = a.hi; ixlo = a.lo; iy = b.hi; iylo = b.lo;
}

// Warp helpers
__device__ __forceinline__ unsigned lane_id() { unsigned r; asm volatile("mov.u32 %0, %%laneid;" : "=r"(r)); return r; }
__device__ __forceinline__ unsigned lanemask_lt() { unsigned r; asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(r)); return r; }

// Atomic max on non-negative doubles through their bit patterns.
// Release + acquire fence at GPU scope.  Paired with a relaxed atomic it
// forms the release (writes, fence, atomic) and acquire (atomic, fence,
// reads) patterns of the PTX memory model, without the extra ordering of a
// sequentially consistent fence (__threadfence).
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// atomicAdd with acquire-release semantics at GPU scope: the caller's earlier
// writes are visible to whoever observes the new value, and the caller sees
// the writes of everyone whose addition it observes.
__device__ __forceinline__ int atomic_add_acq_rel_gpu(int* p, int v) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ void atomic_max_pos_double(unsigned long long* addr, double v) {
    if (!(v > 0.0)) return;   // skips NaN and zero
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

}  // namespace geon
