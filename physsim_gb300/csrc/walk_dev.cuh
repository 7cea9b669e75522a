// walk_dev.cuh — device code of the force passes (force.cu): the pair force,
// the accumulators, the signal-delay solve and the Barnes-Hut walks.  The
// batched walk is a body taking its virtual block index, so walkc_kernel
// (force.cu) and the persistent frame kernel (frame.cu) run the same code.
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
#pragma once

#include "force.cuh"

namespace geon {

constexpr int WALK_THREADS = 128;
constexpr int WALK_WARPS = WALK_THREADS / 32;
constexpr int FLUSH_EVERY = 16;

// ---- accumulators -----------------------------------------------------------
enum { Q_FX = 0, Q_FY, Q_TID, Q_PE, Q_NBASE };
enum { M_BZ = 0, M_BGZ, M_DBZX, M_DBZY, M_DBGZX, M_DBGZY, M_FD, M_F1X, M_F1Y, M_N };
enum { K_GX = 0, K_GY, K_CX, K_CY, K_MX, K_MY, K_GMX, K_GMY, K_YX, K_YY, K_N };

// SH: the compensated (hi, lo) sums live in rows of shared memory at the
// start of the dynamic buffer, [2 * NQ][ACC_SH_THREADS] with one column per
// thread, instead of registers.  They are touched only every FLUSH_EVERY
// terms; the registers they free let the plain Barnes-Hut walk without
// energy sums run six CTAs per SM instead of five (the dipole / 1PN walks:
// four instead of three).
extern __shared__ __align__(16) unsigned char geon_dsmem[];
constexpr int ACC_SH_THREADS = 128;
template <bool MAGGM, bool BRK, bool SH = false>
struct Acc {
    static constexpr int QM = Q_NBASE;
    static constexpr int QK = Q_NBASE + (MAGGM ? M_N : 0);
    static constexpr int NQ = QK + (BRK ? K_N : 0);
    static constexpr size_t SH_BYTES = SH ? (size_t)2 * NQ * ACC_SH_THREADS * sizeof(float) : 0;
    float part[NQ], hi_[SH ? 1 : NQ], lo_[SH ? 1 : NQ];
    int cnt;
    __device__ __forceinline__ static float* row(int q) {
        return reinterpret_cast<float*>(geon_dsmem) + q * ACC_SH_THREADS + threadIdx.x;
    }
    __device__ __forceinline__ float& hi(int q) { if constexpr (SH) return *row(q); else return hi_[q]; }
    __device__ __forceinline__ float& lo(int q) { if constexpr (SH) return *row(NQ + q); else return lo_[q]; }
    __device__ __forceinline__ void init() {
#pragma unroll
        for (int q = 0; q < NQ; q++) { part[q] = 0.f; hi(q) = 0.f; lo(q) = 0.f; }
        cnt = 0;
    }
    __device__ __forceinline__ void flush() {
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            df s = two_sum(hi(q), part[q]);
            hi(q) = s.hi;
            lo(q) = __fadd_rn(lo(q), s.lo);
            part[q] = 0.f;
        }
    }
    __device__ __forceinline__ void tick() {
        if (++cnt >= FLUSH_EVERY) { flush(); cnt = 0; }
    }
    __device__ __forceinline__ float get(int q) { return __fadd_rn(hi(q), lo(q)); }
    __device__ __forceinline__ void add(int q, float v) { part[q] = __fadd_rn(part[q], v); }
    __device__ __forceinline__ void fma(int q, float a, float b) { part[q] = __fmaf_rn(a, b, part[q]); }
    __device__ __forceinline__ void addm(int q, float v) { if (MAGGM) add(QM + q, v); }
    __device__ __forceinline__ void addk(int q, float v) { if (BRK) add(QK + q, v); }
};

// ---- target particle ---------------------------------------------------------------
struct Tgt {
    float x, y, xlo, ylo, vx, vy, m, q, angVel, mu, L, r, r2;
    float qm;       // q/m for the Coulomb share of the tidal coupling (forces.js:436), 0 when unused
    float tk;       // -TIDAL_STRENGTH * bodyRadius^5 (forces.js:437-440)
    int idx;
    __device__ __forceinline__ double xd() const { return (double)x + (double)xlo; }
    __device__ __forceinline__ double yd() const { return (double)y + (double)ylo; }
};

__device__ __forceinline__ Tgt load_target(const DevState& S, int i) {
    Tgt t;
    const float4 p = S.pos[i], v = S.vel[i], s = S.spin[i];
    const float2 lo = S.pos_lo[i];
    t.x = p.x; t.y = p.y; t.xlo = lo.x; t.ylo = lo.y; t.m = p.z; t.q = p.w;
    t.vx = v.z; t.vy = v.w;
    t.angVel = s.y;
    t.r = s.z;
    t.r2 = s.z * s.z;                                   // bodyRadiusSq
    t.mu = MAG_MOMENT_K * t.q * t.angVel * t.r2;        // forces.js:74
    t.L = INERTIA_K * t.m * t.angVel * t.r2;            // forces.js:75
    t.tk = -TIDAL_STRENGTH * (t.r2 * t.r2 * sqrtf(t.r2));
    t.qm = 0.f;
    t.idx = i;
    return t;
}

__device__ __forceinline__ void target_coupling(const DevParams& P, Tgt& t) {
    t.qm = ((P.toggles & GEON_COULOMB) && t.m > EPS_F) ? t.q / t.m : 0.f;
}

__device__ __forceinline__ bool on(const DevParams& P, uint32_t bit) { return (P.toggles & bit) != 0; }

// ---- pairForce (forces.js:163-442) ----------------------------------------------------
template <bool MAGGM, bool BRK, class ACC>
__device__ __forceinline__ void pair_force(const DevParams& P, const Tgt& t, float rx, float ry,
                                           float svx, float svy, float sm, float sq, float sAngVel,
                                           float sMu, float sL, bool delayed, bool yukIn, bool pe,
                                           ACC& A) {
    const float rawRSq = __fmaf_rn(rx, rx, ry * ry);
    const float rSq = rawRSq + P.softSq;
    const float invR = rsqrtf(rSq);
    const float invRSq = invR * invR;
    const float invR3 = invR * invRSq;
    const float invR5 = invR3 * invRSq;
    float aberr = 1.f;
    if (delayed) {                                                   // forces.js:182-187
        const float nDotV = -(rx * svx + ry * svy) * invR;
        const float denom = fmaxf(1.f - nDotV, 0.01f);
        aberr = fminf(1.f / (denom * denom * denom), 100.f);
    }
    const float invR3a = invR3 * aberr;
    const float invR5a = invR5 * aberr;
    const bool grav = on(P, GEON_GRAVITY), coul = on(P, GEON_COULOMB);
    float fr = 0.f;                                                  // sum of the radial (r-parallel) terms

    if (!BRK && grav && coul) {                                      // forces.js:205-240, one radial coefficient
        fr = __fmaf_rn(t.m, sm, -(t.q * sq)) * invR3a;
        if (pe) { A.add(Q_PE, -(t.m * sm) * invR); A.add(Q_PE, t.q * sq * invR); }
    } else {
        if (grav) {                                                  // forces.js:205-220
            const float k = t.m * sm;
            const float fDir = k * invR3a;
            fr += fDir;
            A.addk(K_GX, rx * fDir); A.addk(K_GY, ry * fDir);
            if (pe) A.add(Q_PE, -k * invR);
        }
        if (coul) {                                                  // forces.js:225-240
            const float k = -(t.q * sq);
            const float fDir = k * invR3a;
            fr += fDir;
            A.addk(K_CX, rx * fDir); A.addk(K_CY, ry * fDir);
            if (pe) A.add(Q_PE, t.q * sq * invR);
        }
    }
    if (MAGGM) {
        const bool mag = on(P, GEON_MAGNETIC), gm = on(P, GEON_GRAVITOMAG), pn = on(P, GEON_ONE_PN);
        const float crossSV = svx * ry - svy * rx;
        if (pn && (gm || mag)) {                                     // forces.js:242-298
            const float r = rSq * invR;
            const float nx = rx * invR, ny = ry * invR;
            const float v1DotV2 = t.vx * svx + t.vy * svy;
            if (gm) {
                const float v1Sq = t.vx * t.vx + t.vy * t.vy, v2Sq = svx * svx + svy * svy;
                const float nDotV1 = nx * t.vx + ny * t.vy, nDotV2 = nx * svx + ny * svy;
                const float radial = -v1Sq - 2.f * v2Sq + 1.5f * nDotV2 * nDotV2 + 5.f * t.m * invR + 4.f * sm * invR;
                const float v1Coeff = 4.f * nDotV1 - 3.f * nDotV2, v2Coeff = 3.f * nDotV2;
                const float base = t.m * sm * invR3;
                const float fx = base * (rx * radial + (t.vx * v1Coeff + svx * v2Coeff) * r);
                const float fy = base * (ry * radial + (t.vy * v1Coeff + svy * v2Coeff) * r);
                A.add(Q_FX, fx); A.add(Q_FY, fy);
                A.addm(M_F1X, fx); A.addm(M_F1Y, fy);
                if (pe) A.add(Q_PE, -t.m * sm * invR * (1.5f * (v1Sq + v2Sq) - 3.5f * v1DotV2 - 0.5f * nDotV1 * nDotV2
                                                        + t.m * invR + sm * invR));
            }
            if (mag) {
                const float v2DotN = svx * nx + svy * ny, v1DotN = t.vx * nx + t.vy * ny;
                const float coeff = 0.5f * t.q * sq * invRSq;
                const float symX = coeff * (t.vx * v2DotN - 3.f * nx * v1DotN * v2DotN);
                const float symY = coeff * (t.vy * v2DotN - 3.f * ny * v1DotN * v2DotN);
                A.add(Q_FX, symX); A.add(Q_FY, symY);
                A.addm(M_F1X, symX); A.addm(M_F1Y, symY);
                if (pe) A.add(Q_PE, -0.5f * t.q * sq * invR * (v1DotV2 + v1DotN * v2DotN));
            }
        }
        if (pn && gm && mag) {                                       // forces.js:300-316
            const float crossCoeff = t.q * sq * (t.m + sm) - (t.q * t.q * sm + sq * sq * t.m);
            const float fDir = crossCoeff * invRSq * invRSq;
            fr += fDir;
            A.addm(M_F1X, rx * fDir); A.addm(M_F1Y, ry * fDir);
            if (pe) A.add(Q_PE, 0.5f * crossCoeff * invRSq);
        }
        if (mag) {                                                   // forces.js:318-349
            const float fDir = -3.f * (t.mu * sMu) * invR5a;
            fr += fDir;
            A.addk(K_MX, rx * fDir); A.addk(K_MY, ry * fDir);
            if (pe) A.add(Q_PE, (t.mu * sMu) * invR3);
            const float BzMoving = sq * crossSV * invR3;
            A.addm(M_BZ, BzMoving - sMu * invR3);
            A.addm(M_DBZX, 3.f * BzMoving * rx * invRSq + sq * svy * invR3 - 3.f * sMu * rx * invR5);
            A.addm(M_DBZY, 3.f * BzMoving * ry * invRSq - sq * svx * invR3 - 3.f * sMu * ry * invR5);
        }
        if (gm) {                                                    // forces.js:351-384
            const float fDir = 3.f * (t.L * sL) * invR5a;
            fr += fDir;
            A.addk(K_GMX, rx * fDir); A.addk(K_GMY, ry * fDir);
            if (pe) A.add(Q_PE, -(t.L * sL) * invR3);
            const float BgzMoving = -sm * crossSV * invR3;
            A.addm(M_BGZ, BgzMoving - 2.f * sL * invR3);
            A.addm(M_DBGZX, 3.f * BgzMoving * rx * invRSq - sm * svy * invR3 - 6.f * sL * rx * invR5);
            A.addm(M_DBGZY, 3.f * BgzMoving * ry * invRSq + sm * svx * invR3 - 6.f * sL * ry * invR5);
            A.addm(M_FD, 2.f * sL * (sAngVel - t.angVel) * invR3);
        }
    }
    if (yukIn) {                                                     // forces.js:387-426
        const float mu = P.yukMu;
        const float r = rSq * invR;
        const float expMuR = __expf(-mu * r);
        const float g = YUKAWA_COUPLING * t.m * sm * expMuR;
        const float fDir = g * (invRSq + mu * invR) * (invR * aberr);
        fr += fDir;
        A.addk(K_YX, rx * fDir); A.addk(K_YY, ry * fDir);
        if (pe) A.add(Q_PE, -g * invR);
        if (MAGGM && on(P, GEON_ONE_PN)) {
            const float nx = rx * invR, ny = ry * invR;
            const float nDotV1 = nx * t.vx + ny * t.vy, nDotV2 = nx * svx + ny * svy;
            const float v1DotV2 = t.vx * svx + t.vy * svy;
            const float alpha = 1.f + mu * r;
            const float beta = 0.5f * g * invRSq;
            const float radial = -(alpha * v1DotV2 + (alpha * alpha + alpha + 1.f) * nDotV1 * nDotV2);
            const float fx = beta * (radial * nx + alpha * (nDotV2 * t.vx + nDotV1 * svx));
            const float fy = beta * (radial * ny + alpha * (nDotV2 * t.vy + nDotV1 * svy));
            A.add(Q_FX, fx); A.add(Q_FY, fy);
            A.addm(M_F1X, fx); A.addm(M_F1Y, fy);
            if (pe) A.add(Q_PE, 0.5f * g * invR * (v1DotV2 + nDotV1 * nDotV2 * alpha));
        }
    }
    A.fma(Q_FX, rx, fr);
    A.fma(Q_FY, ry, fr);
    if (grav) {                                                      // forces.js:428-441
        const float crossRV = rx * (svy - t.vy) - ry * (svx - t.vx);
        const float dw = __fmaf_rn(-crossRV, invRSq, t.angVel);
        const float coupling = __fmaf_rn(t.qm, sq, sm);
        const float invR6 = invRSq * invRSq * invRSq;
        A.add(Q_TID, t.tk * (coupling * coupling) * invR6 * dw);
    }
}

// ---- exact (FP64) displacement helpers for guard-band re-tests --------------------------
// Every FP64 operation sits behind a guard that is taken only when an FP32
// margin is within rounding: FP64 runs at a small fraction of the FP32 rate.
// PER: the topology class of a walk fixed at compile time, 0 the open box,
// 1 any topology (decided at run time), 2 the torus only.  The walks that
// know their class carry no code for the others.
template <int PER = 1>
__device__ __forceinline__ void exact_disp(const DevParams& P, double ox, double oy, double sx, double sy,
                                           double& rx, double& ry) {
    if (PER == 0) { rx = sx - ox; ry = sy - oy; }
    else if (PER == 2) torus_image_d(ox, oy, sx, sy, P.Wd, P.Hd, rx, ry);
    else if (P.periodic) min_image_d(ox, oy, sx, sy, P.topology, P.Wd, P.Hd, rx, ry);
    else { rx = sx - ox; ry = sy - oy; }
}

// A source position as unevaluated (hi, lo) pairs, converted to FP64 only in guard paths.
struct SPos { float x, xlo, y, ylo; };

// FP64 re-test of the Yukawa cutoff inside the FP32 guard band (rarely taken).
template <int PER = 1>
__device__ __forceinline__ bool yukawa_in_exact(const DevParams& P, const SPos& sp, double tx, double ty) {
    double dx, dy;
    exact_disp<PER>(P, tx, ty, (double)sp.x + (double)sp.xlo, (double)sp.y + (double)sp.ylo, dx, dy);
    return dx * dx + dy * dy < P.yukCutSqD;
}

template <int PER = 1>
__device__ __forceinline__ bool yukawa_in(const DevParams& P, float rx, float ry, const SPos& sp, const Tgt& t) {
    if (!P.yukOn) return false;
    const float rr = __fmaf_rn(rx, rx, ry * ry);
    const float cut = P.yukCutSq;
    if (fabsf(rr - cut) > 1e-6f * cut) return rr < cut;
    return yukawa_in_exact<PER>(P, sp, t.xd(), t.yd());
}

// Displacement with the topology class fixed at compile time (PER as for
// exact_disp): no wrap code for the open box, the torus wrap alone for the
// torus, the run-time choice otherwise.
template <int PER>
__device__ __forceinline__ void displacement_p(const DevParams& P, float ox, float oy, float sx, float sx_lo,
                                               float sy, float sy_lo, float& rx, float& ry) {
    if (PER == 0) {
        rx = __fadd_rn(__fsub_rn(sx, ox), sx_lo);
        ry = __fadd_rn(__fsub_rn(sy, oy), sy_lo);
    } else if (PER == 2) {
        rx = wrap_axis_comp(sx, ox, sx_lo, P.W, P.W_lo, P.halfW);
        ry = wrap_axis_comp(sy, oy, sy_lo, P.H, P.H_lo, P.halfH);
    } else {
        displacement(P, ox, oy, sx, sx_lo, sy, sy_lo, rx, ry);
    }
}

// ---- signal delay (signal-delay.js:16-221) ----------------------------------------------
// Returns the retarded source state.  The position comes back as the
// displacement (rx, ry) from the target, formed as (sample - target) + frac *
// segment so that FP32 rounding is relative to the separation, not to the
// absolute coordinate; (x, y) is the absolute position for guard paths.
struct Delayed { float rx, ry, x, y, vx, vy, angw; };

// Displacement from target t to the point base + step (base a history sample).
__device__ __forceinline__ void retarded_disp(const DevParams& P, const Tgt& t, float bx, float by, float stx, float sty,
                                              float& rx, float& ry) {
    if (!P.periodic) {
        rx = __fsub_rn(__fadd_rn(__fsub_rn(bx, t.x), stx), t.xlo);
        ry = __fsub_rn(__fadd_rn(__fsub_rn(by, t.y), sty), t.ylo);
    } else if (P.topology == GEON_TORUS) {
        const float dx0 = wrap_axis_comp(bx, t.x, -t.xlo, P.W, P.W_lo, P.halfW);
        const float dy0 = wrap_axis_comp(by, t.y, -t.ylo, P.H, P.H_lo, P.halfH);
        rx = torus_wrap_f(dx0 + stx, P.W, P.halfW);
        ry = torus_wrap_f(dy0 + sty, P.H, P.halfH);
    } else {
        double dx, dy;
        min_image_d(t.xd(), t.yd(), (double)bx + (double)stx, (double)by + (double)sty, P.topology, P.Wd, P.Hd, dx, dy);
        rx = (float)dx; ry = (float)dy;
    }
}

static __device__ bool delayed_state(const DevParams& P, const DevState& S, const ForceCtx& C, const float* s_age,
                              const float* s_segdt, int j, const Tgt& t, Delayed& out) {
    const float ox = t.x, oy = t.y;
    const int count = S.hist_cnt[j];
    if (count < 2) return false;
    const int start = (C.hist_head - count) & HIST_MASK;
    const int newest = (C.hist_head - 1) & HIST_MASK;
    const float timeSpan = s_age[start];
    if (timeSpan < EPS_F) return false;
    const float4* H = S.hist + (size_t)j * HIST_LEN;
    const float* HA = S.hist_angw + (size_t)j * HIST_LEN;
    float cdx, cdy;
    {
        const float4 hn = H[newest];
        displacement(P, ox, oy, hn.x, 0.f, hn.y, 0.f, cdx, cdy);
    }
    const float distSq = cdx * cdx + cdy * cdy;
    if (!(distSq > 4.f * timeSpan * timeSpan)) {
        int lo = 0, hi = count - 2;
        while (lo < hi) {                                            // :55-75
            const int mid = (lo + hi) >> 1;
            const int midIdx = (start + mid + 1) & HIST_MASK;
            const float4 hm = H[midIdx];
            float bx, by;
            displacement(P, ox, oy, hm.x, 0.f, hm.y, 0.f, bx, by);
            const float g = sqrtf(bx * bx + by * by) - s_age[midIdx];
            if (g < 0.f) lo = mid + 1; else hi = mid;
        }
        const int center = lo;
        for (int off = 0; off <= 1; off++) {                         // :80-159
            for (int dir = (off == 0 ? 1 : -1); dir <= 1; dir += 2) {
                const int k = center + off * dir;
                if (k < 0 || k > count - 2) continue;
                const int loIdx = (start + k) & HIST_MASK;
                const int hiIdx = (loIdx + 1) & HIST_MASK;
                const float segDt = s_segdt[loIdx];
                if (segDt < EPS_F) continue;
                const float4 hl = H[loIdx], hh = H[hiIdx];
                float dx, dy, sgx, sgy;
                displacement(P, ox, oy, hl.x, 0.f, hl.y, 0.f, dx, dy);
                if (P.periodic) displacement(P, hl.x, hl.y, hh.x, 0.f, hh.y, 0.f, sgx, sgy);
                else { sgx = hh.x - hl.x; sgy = hh.y - hl.y; }
                const float vx = sgx / segDt, vy = sgy / segDt;
                const float rSq = dx * dx + dy * dy, vSq = vx * vx + vy * vy, dDotV = dx * vx + dy * vy;
                const float T = s_age[loIdx];
                const float a = vSq - 1.f, h = dDotV + T, c = rSq - T * T;
                const float disc = h * h - a * c;
                if (!(disc >= 0.f)) continue;
                const float sqrtDisc = sqrtf(disc);
                float s;
                if (fabsf(a) < EPS_F) {
                    if (fabsf(h) < EPS_F) continue;
                    s = -c / (2.f * h);
                } else {
                    const float s1 = (-h + sqrtDisc) / a, s2 = (-h - sqrtDisc) / a;
                    const bool ok1 = s1 >= -EPS_F && s1 <= segDt + EPS_F;
                    const bool ok2 = s2 >= -EPS_F && s2 <= segDt + EPS_F;
                    if (ok1 && ok2) s = fmaxf(s1, s2);
                    else if (ok1) s = s1;
                    else if (ok2) s = s2;
                    else continue;
                }
                if (s < 0.f) s = 0.f; else if (s > segDt) s = segDt;
                const float frac = s / segDt;
                retarded_disp(P, t, hl.x, hl.y, frac * sgx, frac * sgy, out.rx, out.ry);
                out.x = hl.x + frac * sgx;
                out.y = hl.y + frac * sgy;
                out.vx = hl.z + frac * (hh.z - hl.z);
                out.vy = hl.w + frac * (hh.w - hl.w);
                const float al = HA[loIdx];
                out.angw = al + frac * (HA[hiIdx] - al);
                return true;
            }
        }
    }
    {                                                                // :166-220
        const float4 hs = H[start];
        float dx, dy;
        displacement(P, ox, oy, hs.x, 0.f, hs.y, 0.f, dx, dy);
        const float vx = hs.z, vy = hs.w;
        const float rSq = dx * dx + dy * dy, vSq = vx * vx + vy * vy, dDotV = dx * vx + dy * vy;
        const float T = timeSpan;
        const float a = vSq - 1.f, h = dDotV + T, c = rSq - T * T;
        const float disc = h * h - a * c;
        if (!(disc >= 0.f)) return false;
        const float sqrtDisc = sqrtf(disc);
        float s;
        if (fabsf(a) < EPS_F) {
            if (fabsf(h) < EPS_F) return false;
            s = -c / (2.f * h);
        } else {
            const float s1 = (-h + sqrtDisc) / a, s2 = (-h - sqrtDisc) / a;
            const bool ok1 = s1 <= EPS_F, ok2 = s2 <= EPS_F;
            if (ok1 && ok2) s = fmaxf(s1, s2);
            else if (ok1) s = s1;
            else if (ok2) s = s2;
            else return false;
        }
        if (s > 0.f) s = 0.f;
        if (C.hist_t[start] + (double)s < S.ctime[j]) return false;   // particle did not exist yet
        retarded_disp(P, t, hs.x, hs.y, vx * s, vy * s, out.rx, out.ry);
        out.x = hs.x + vx * s;
        out.y = hs.y + vy * s;
        out.vx = vx; out.vy = vy;
        out.angw = HA[start];
        return true;
    }
}

// Displacement to a delayed source.  Ghosts add their current image offset
// (forces.js:656-661); on the torus that offset is a whole period and the
// minimum image removes it, on Klein / RP^2 it is formed in FP64.
__device__ __forceinline__ void delayed_disp(const DevParams& P, const Tgt& t, const Delayed& d,
                                             float xj, float yj, uint32_t code, float& rx, float& ry, SPos& sp) {
    sp = SPos{ d.x, 0.f, d.y, 0.f };
    if (code == CODE_IDENTITY || (!code_mx(code) && !code_my(code) && P.topology == GEON_TORUS)) {
        rx = d.rx; ry = d.ry;
        return;
    }
    double gx, gy;
    image_pos_d((double)xj, (double)yj, code, P.Wd, P.Hd, gx, gy);
    const double sxd = (double)d.x + (gx - (double)xj);
    const double syd = (double)d.y + (gy - (double)yj);
    double dx, dy;
    exact_disp(P, t.xd(), t.yd(), sxd, syd, dx, dy);
    rx = (float)dx; ry = (float)dy;
    sp = SPos{ (float)sxd, (float)(sxd - (double)(float)sxd), (float)syd, (float)(syd - (double)(float)syd) };
}

// ---- epilogue: outputs, external fields, walls, planner reductions -------------------------
template <bool MAGGM, bool BRK, class ACC>
__device__ __forceinline__ void finalize_target(const DevParams& P, const DevState& S, const ForceCtx& C,
                                                FrameCtl* ctl, const Tgt& t, bool valid, ACC& A,
                                                unsigned inter32, int sysId = -1) {
    // padding lanes evaluate the warp's shared entries too: only real targets count
    unsigned long long inter = valid ? inter32 : 0ull;
    A.flush();
    double aSq = 0.0, wc = 0.0;
    if (valid) {
        float fx = A.get(Q_FX), fy = A.get(Q_FY);
        float Bz = MAGGM ? A.get(A.QM + M_BZ) : 0.f, Bgz = MAGGM ? A.get(A.QM + M_BGZ) : 0.f;
        float ex = 0.f, ey = 0.f, contact = 0.f;
        if (P.extGx != 0.f || P.extGy != 0.f) { ex += t.m * P.extGx; ey += t.m * P.extGy; }   // integrator.js:575-581
        if (P.extEx != 0.f || P.extEy != 0.f) { ex += t.q * P.extEx; ey += t.q * P.extEy; }
        if (P.extBz != 0.f) Bz += P.extBz;
        if (C.bounce) {                                              // integrator.js:607-668
            const float r = S.spin[t.idx].z, fr = P.friction;   // reloaded: not kept live through the walk
            const float left = (float)P.offXd, top = (float)P.offYd;
            const float right = (float)(P.offXd + P.Wd), bottom = (float)(P.offYd + P.Hd);
            auto clamp1 = [](float v) { return fminf(1.f, fmaxf(-1.f, v)); };
            float delta = r - (t.x - left);
            if (delta > 0.f) {
                const float Fn = delta * sqrtf(delta);
                ex += Fn;
                if (fr > 0.f) { const float Ft = -fr * Fn * clamp1((t.vy + t.angVel * r) * 10.f); fy += Ft; contact += r * Ft; }
            }
            delta = r - (right - t.x);
            if (delta > 0.f) {
                const float Fn = delta * sqrtf(delta);
                ex -= Fn;
                if (fr > 0.f) { const float Ft = -fr * Fn * clamp1((-t.vy - t.angVel * r) * 10.f); fy -= Ft; contact -= r * Ft; }
            }
            delta = r - (t.y - top);
            if (delta > 0.f) {
                const float Fn = delta * sqrtf(delta);
                ey += Fn;
                if (fr > 0.f) { const float Ft = -fr * Fn * clamp1((-t.vx + t.angVel * r) * 10.f); fx -= Ft; contact += r * Ft; }
            }
            delta = r - (bottom - t.y);
            if (delta > 0.f) {
                const float Fn = delta * sqrtf(delta);
                ey -= Fn;
                if (fr > 0.f) { const float Ft = -fr * Fn * clamp1((t.vx - t.angVel * r) * 10.f); fx += Ft; contact -= r * Ft; }
            }
        }
        fx += ex; fy += ey;
        const int i = t.idx;
        S.force[i] = make_float4(fx, fy, Bz, Bgz);
        if (MAGGM) {
            S.grad[i] = make_float4(A.get(A.QM + M_DBZX), A.get(A.QM + M_DBZY), A.get(A.QM + M_DBGZX), A.get(A.QM + M_DBGZY));
            S.f1pn[i] = make_float2(A.get(A.QM + M_F1X), A.get(A.QM + M_F1Y));
        } else {
            S.grad[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            S.f1pn[i] = make_float2(0.f, 0.f);
        }
        S.torque[i] = make_float4(A.get(Q_TID), MAGGM ? A.get(A.QM + M_FD) : 0.f, contact, A.get(Q_PE));
        S.mom[i] = make_float2(t.mu, t.L);
        if (BRK) {
            const int cap = P.n_cap;
            float* b = S.brk;
#pragma unroll
            for (int q = 0; q < K_N; q++) b[(size_t)q * cap + i] = A.get(A.QK + q);
            b[(size_t)K_N * cap + i] = ex;
            b[(size_t)(K_N + 1) * cap + i] = ey;
        } else if (S.brk) {
            const int cap = P.n_cap;
            S.brk[(size_t)K_N * cap + i] = ex;
            S.brk[(size_t)(K_N + 1) * cap + i] = ey;
        }
        // planner reductions (integrator.js:816-836)
        const double im = (double)S.spin[i].w;
        aSq = ((double)fx * fx + (double)fy * fy) * im * im;
        if (on(P, GEON_MAGNETIC) || P.extBz != 0.f) {
            const double absBz = fabs((double)Bz);
            if (absBz > 0) wc = fmax(wc, fabs((double)t.q) * absBz * im);
        }
        if (on(P, GEON_GRAVITOMAG)) {
            const double absBgz = fabs((double)Bgz);
            if (absBgz > 0) wc = fmax(wc, 4.0 * absBgz);
        }
        if (!(aSq == aSq)) aSq = 0.0;
        if (!(wc == wc)) wc = 0.0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        aSq = fmax(aSq, __shfl_xor_sync(0xffffffffu, aSq, o));
        wc = fmax(wc, __shfl_xor_sync(0xffffffffu, wc, o));
        inter += __shfl_xor_sync(0xffffffffu, inter, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (C.sys_accel && sysId >= 0) {       // batched: the warp's targets are one system
            atomic_max_pos_double(&C.sys_accel[sysId], aSq);
            atomic_max_pos_double(&C.sys_cyc[sysId], wc);
        } else {
            atomic_max_pos_double(&ctl->maxAccelSqBits, aSq);
            atomic_max_pos_double(&ctl->maxCycBits, wc);
        }
        if (inter) atomicAdd(&ctl->interactions, inter);
    }
}

__device__ __forceinline__ void load_hist_tables(const ForceCtx& C, float* s_age, float* s_segdt) {
    for (int k = threadIdx.x; k < HIST_LEN; k += blockDim.x) {
        s_age[k] = C.hist_age[k];
        s_segdt[k] = C.hist_segdt[k];
    }
    __syncthreads();
}

// Target in slot k of the walk order: T.tgt[k] (k < n) for one system.  For
// batched handles the slots come from the per-system list padded to whole
// warps, and systems whose substep is over sit the pass out.  Returns -1 for
// an empty slot; sysId receives the system (batched) or -1.
__device__ __forceinline__ int walk_target(const DevState& S, const TreeBufs& T, const FrameCtl* ctl,
                                           const ForceCtx& C, int k, int& sysId) {
    sysId = -1;
    if (!C.tgt_list) return k < ctl->n ? T.tgt[k] : -1;
    if (k >= C.tgt_count) return -1;
    const int i = C.tgt_list[k];
    if (i < 0) return -1;
    sysId = S.sys ? S.sys[i] : -1;
    if (C.sys_dt && !(C.sys_dt[sysId] > 0.0)) return -1;
    return i;
}

// ---- Barnes-Hut walk (forces.js:622-694) -----------------------------------------------------
template <bool MAGGM, bool REL, bool BRK>
__global__ void __launch_bounds__(WALK_THREADS)
walk_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root, FrameCtl* ctl, ForceCtx C) {
    __shared__ int s_node[WALK_WARPS][WALK_STACK];
    __shared__ unsigned s_mask[WALK_WARPS][WALK_STACK];
    __shared__ float s_age[REL ? HIST_LEN : 1], s_segdt[REL ? HIST_LEN : 1];
    if (REL) load_hist_tables(C, s_age, s_segdt);
    const int warp = threadIdx.x >> 5;
    const unsigned lane = threadIdx.x & 31;
    const int k = (blockIdx.x * WALK_WARPS + warp) * 32 + (int)lane;
    int sysId;
    const int ti = walk_target(S, T, ctl, C, k, sysId);
    const bool valid = ti >= 0;
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    if (active == 0) return;
    if (C.roots) sysId = __shfl_sync(0xffffffffu, sysId, __ffs(active) - 1);
    Tgt t;
    if (valid) { t = load_target(S, ti); target_coupling(P, t); }
    else { t = Tgt{}; t.idx = -1; }
    Acc<MAGGM, BRK> A;
    A.init();
    unsigned inter = 0;
    const bool pe = C.pe != 0;
    const int root = C.roots ? C.roots[sysId] : *d_root;
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
            const float lmass = T.leaf_a[li].z;
            if (lmass < EPS_F) continue;                             // forces.js:630
            const int4 lm = T.leaf_meta[li];
            if (lm.x < 0 || lm.x + lm.y > nValidW) { if (lane == 0) atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
            for (int q = lm.x; q < lm.x + lm.y; q++) {               // forces.js:643-679
                const float4 pa = T.ps_a[q];
                const float4 pb = T.ps_b[q];
                const float4 pc = T.ps_c[q];
                const uint32_t ref = __float_as_uint(pc.w);
                const int j = (int)ref_index(ref);
                const uint32_t code = ref_code(ref);
                if (!in || j == t.idx) continue;
                float rx, ry;
                SPos sp{ pa.x, pb.x, pa.y, pb.y };
                float svx, svy, sAng, sMu, sL;
                bool dl = false;
                if (REL) {
                    Delayed d;
                    if (!delayed_state(P, S, C, s_age, s_segdt, j, t, d)) continue;
                    float xj = 0.f, yj = 0.f;
                    if (code != CODE_IDENTITY && (code_mx(code) || code_my(code) || P.topology != GEON_TORUS)) {
                        const float4 pj = S.pos[j];
                        xj = pj.x; yj = pj.y;
                    }
                    delayed_disp(P, t, d, xj, yj, code, rx, ry, sp);
                    svx = d.vx; svy = d.vy;
                    const float rj = S.spin[j].z, rj2 = rj * rj;
                    sAng = d.angw * rsqrtf(1.f + d.angw * d.angw * rj2);
                    sMu = MAG_MOMENT_K * pa.w * sAng * rj2;
                    sL = INERTIA_K * pa.z * sAng * rj2;
                    dl = true;
                } else {
                    displacement(P, t.x, t.y, pa.x, pb.x - t.xlo, pa.y, pb.y - t.ylo, rx, ry);
                    svx = pb.z; svy = pb.w; sAng = pc.x; sMu = pc.y; sL = pc.z;
                }
                const bool yk = yukawa_in(P, rx, ry, sp, t);
                pair_force<MAGGM, BRK>(P, t, rx, ry, svx, svy, pa.z, pa.w, sAng, sMu, sL, dl, yk, pe, A);
                A.tick();
                inter++;
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
                accept = c.z < rhs;                                  // forces.js:680
                if (fabsf(rhs - c.z) <= 1e-6f * c.z) {
                    double dx, dy;
                    exact_disp(P, t.xd(), t.yd(), (double)a.x + (double)c.x, (double)a.y + (double)c.y, dx, dy);
                    const double size = 2.0 * ldexp(P.rootW, -(int)c.w);
                    accept = size * size < P.thetaSqD * (dx * dx + dy * dy);
                }
            }
            const unsigned acc = __ballot_sync(0xffffffffu, accept);
            const unsigned open = mask & ~acc;
            if (accept) {                                            // forces.js:682-685
                const float4 b = T.int_b[node];
                const bool yk = yukawa_in(P, rx, ry, SPos{ a.x, c.x, a.y, c.y }, t);
                pair_force<MAGGM, BRK>(P, t, rx, ry, b.x, b.y, a.z, a.w, 0.f, b.z, b.w, false, yk, pe, A);
                A.tick();
                inter++;
            }
            if (open) {                                              // forces.js:686-692
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
    finalize_target<MAGGM, BRK>(P, S, C, ctl, t, valid, A, inter, sysId);
}

// ---- batched Barnes-Hut walk ----------------------------------------------------------------
// Same interaction lists as walk_kernel, restructured for throughput:
//  * each iteration pops up to WC_POP stack entries, one per lane, so the node
//    records arrive with one wide load;
//  * a lane first tests its node against the bounding box of the warp's 32
//    particles: if every particle accepts the node, or every particle opens
//    it, no per-particle test is needed; only the remaining ("mixed") nodes
//    get the per-lane test, from shuffled registers, with a ballot;
//  * accepted aggregates and the points of reached leaves are staged in a
//    per-warp pool in shared memory.  Entries every particle needs fill the
//    pool from the bottom, in order, and are evaluated by position with
//    broadcast reads; entries only some particles need fill it from the top
//    and go to per-lane index lists, evaluated transposed so that no lane
//    idles on another lane's sources.
constexpr int WC_THREADS = 128;
constexpr int WC_WARPS = WC_THREADS / 32;
constexpr int WC_STACK = 448;
constexpr int WC_STACK_SHORT = 288;   // the short-stack plain walk (seven CTAs per SM; a batched walk shape)
constexpr int WC_RESERVE = 3 * KEY_LEVELS + 3 * 16 + 4;   // growth a depth-first tail can still need
constexpr int WC_POOL_SHF = 64;    // the walks in shared-memory form (below)
constexpr int WC_POOL_WIDE = 96;   // the others: fewer, fuller flushes
constexpr int WC_POP = 16;
// one pop step stages at most WC_POP leaves of LEAF_CAP points (or one
// aggregate per lane) and a bucket chunk 32 points, each after a flush
static_assert(WC_POOL_SHF >= WC_POP * LEAF_CAP && WC_POOL_SHF >= 32, "source pool smaller than one step's staging");
static_assert(WC_POOL_WIDE >= WC_POOL_SHF && WC_POOL_WIDE <= 255, "pool indices are bytes");
static_assert(WC_POP * LEAF_CAP < 256, "a pop step's entry counts share one prefix sum, 8 bits apiece");
constexpr uint32_t AGG_REF = 0xffffffffu;

template <bool NEEDC, int POOL, int STACK = WC_STACK>
struct WcSmem {
    static constexpr int kPool = POOL;
    static constexpr int kStack = STACK;
    int stk_node[STACK];
    unsigned stk_mask[STACK];
    float4 a[POOL];                    // x (hi), y (hi), mass, charge
    float4 b[POOL];                    // x (lo), y (lo), vx, vy
    float4 c[NEEDC ? POOL : 1];        // angVel, magMoment, angMomentum, -
    uint32_t ref[POOL];                // particle ref, AGG_REF for aggregates
    uint8_t lst[POOL][32];             // per-lane lists (column = lane) of partial entries
    // read at each node classification, kept here rather than in registers
    float gbox[4];                     // the warp's target box: centre x, y, half-widths x, y
    int counts[3];                     // internal nodes, leaves, valid points of the tree
};

__device__ __forceinline__ int warp_incl_scan_i(int v) {
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    return v;
}
__device__ __forceinline__ float warp_min_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max_i(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// YUK false: the Yukawa term is off at compile time (the lean torus walks
// carry no cutoff guard or Yukawa force code when the term is off).
template <bool MAGGM, bool REL, bool BRK, int PER, bool YUK, class ACC, class WS>
__device__ __forceinline__ void eval_entry(const DevParams& P, const DevState& S, const ForceCtx& C,
                                           const float* s_age, const float* s_segdt, const WS& W,
                                           int e, const Tgt& t, ACC& A, unsigned& inter, bool pe) {
    const float4 a = W.a[e];
    const float4 b = W.b[e];
    const uint32_t ref = W.ref[e];
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (MAGGM || REL) c = W.c[e];
    float rx, ry, svx = b.z, svy = b.w, sAng = c.x, sMu = c.y, sL = c.z;
    SPos sp{ a.x, b.x, a.y, b.y };
    bool dl = false;
    // inter counted this entry when the pool was flushed: an entry that is
    // not evaluated takes it back
    if (!REL) {
        // self and own ghosts (forces.js:648-649); an aggregate's index field
        // (REF_INDEX_MASK) lies above every particle index, so the one test
        // covers points and aggregates alike
        if ((int)ref_index(ref) == t.idx) { inter--; return; }
        displacement_p<PER>(P, t.x, t.y, a.x, b.x - t.xlo, a.y, b.y - t.ylo, rx, ry);
    } else if (ref != AGG_REF) {
        const int j = (int)ref_index(ref);
        if (j == t.idx) { inter--; return; }                         // self and own ghosts (forces.js:648-649)
        {                                                             // forces.js:652-672
            Delayed d;
            if (!delayed_state(P, S, C, s_age, s_segdt, j, t, d)) { inter--; return; }
            const uint32_t code = ref_code(ref);
            float xj = 0.f, yj = 0.f;
            if (code != CODE_IDENTITY && (code_mx(code) || code_my(code) || P.topology != GEON_TORUS)) {
                const float4 pj = S.pos[j];
                xj = pj.x; yj = pj.y;
            }
            delayed_disp(P, t, d, xj, yj, code, rx, ry, sp);
            svx = d.vx; svy = d.vy;
            const float rj = S.spin[j].z, rj2 = rj * rj;
            sAng = d.angw * rsqrtf(1.f + d.angw * d.angw * rj2);
            sMu = MAG_MOMENT_K * a.w * sAng * rj2;
            sL = INERTIA_K * a.z * sAng * rj2;
            dl = true;
        }
    } else {
        displacement_p<PER>(P, t.x, t.y, a.x, b.x - t.xlo, a.y, b.y - t.ylo, rx, ry);
    }
    const bool yk = YUK && yukawa_in<PER>(P, rx, ry, sp, t);
    pair_force<MAGGM, BRK>(P, t, rx, ry, svx, svy, a.z, a.w, sAng, sMu, sL, dl, yk, pe, A);
}

template <bool MAGGM, bool REL, bool BRK, int PER, bool YUK, class ACC, class WS>
__device__ __forceinline__ void flush_pool(const DevParams& P, const DevState& S, const ForceCtx& C,
                                           const float* s_age, const float* s_segdt, WS& W,
                                           int& nfull, int& lcnt, int& npart, const Tgt& t, ACC& A,
                                           unsigned& inter, bool pe) {
    __syncwarp();
    const unsigned lane = threadIdx.x & 31;
    const int total = nfull + warp_max_i(lcnt);
    inter += (unsigned)(nfull + lcnt);                               // the entries this lane evaluates
    // full entries first (pool slots 0 .. nfull - 1, broadcast reads), then
    // this lane's own list
    if (MAGGM) {
        // one entry per iteration: the dipole / 1PN pair force (with the
        // light-cone solve when relativity is on) is large enough that a
        // second inlined copy costs more in instruction fetch than its
        // parallelism gains (torus N = 65,536, full force set: 22.9 -> 14.8
        // ms per force pass; the relativistic walk without dipoles is
        // faster with two)
        for (int i = 0; i < total; i++) {
            const int l0 = i - nfull;
            const int e0 = l0 < 0 ? i : (l0 < lcnt ? W.lst[l0][lane] : -1);
            if (e0 >= 0) eval_entry<MAGGM, REL, BRK, PER, YUK>(P, S, C, s_age, s_segdt, W, e0, t, A, inter, pe);
            if (i & 1) A.tick();
        }
    } else {
        // two independent entries per iteration for instruction-level parallelism
        for (int i = 0; i < total; i += 2) {
            const int l0 = i - nfull, l1 = i + 1 - nfull;
            const int e0 = l0 < 0 ? i : (l0 < lcnt ? W.lst[l0][lane] : -1);
            const int e1 = (i + 1 >= total) ? -1 : (l1 < 0 ? i + 1 : (l1 < lcnt ? W.lst[l1][lane] : -1));
            if (e0 >= 0) eval_entry<MAGGM, REL, BRK, PER, YUK>(P, S, C, s_age, s_segdt, W, e0, t, A, inter, pe);
            if (e1 >= 0) eval_entry<MAGGM, REL, BRK, PER, YUK>(P, S, C, s_age, s_segdt, W, e1, t, A, inter, pe);
            A.tick();
        }
    }
    __syncwarp();
    nfull = 0; lcnt = 0; npart = 0;
}

template <bool NEEDC, class WS>
__device__ __forceinline__ void stage_point(const TreeBufs& T, WS& W, int e, int q) {
    W.a[e] = T.ps_a[q];
    W.b[e] = T.ps_b[q];
    if (NEEDC) {
        const float4 pc = T.ps_c[q];
        W.c[e] = pc;
        W.ref[e] = __float_as_uint(pc.w);
    } else {
        W.ref[e] = __float_as_uint(reinterpret_cast<const float*>(T.ps_c + q)[3]);
    }
}

// FP64 opening test (forces.js:680) inside the FP32 guard band (rarely taken).
template <int PER = 1>
__device__ __forceinline__ bool accept_exact(const DevParams& P, double tx, double ty, double sx, double sy, float lvl) {
    double dx, dy;
    exact_disp<PER>(P, tx, ty, sx, sy, dx, dy);
    const double size = 2.0 * ldexp(P.rootW, -(int)lvl);
    return size * size < P.thetaSqD * (dx * dx + dy * dy);
}

// Appends the pool slots first .. first + cnt - 1 to the lists of the lanes in m.
template <class WS>
__device__ __forceinline__ void list_add(WS& W, unsigned m, int first, int cnt, int& lcnt) {
    const unsigned lane = threadIdx.x & 31;
    if ((m >> lane) & 1u) {
        for (int q = 0; q < cnt; q++) W.lst[lcnt + q][lane] = (uint8_t)(first + q);
        lcnt += cnt;
    }
}

// NOPE: the potential-energy sums are off at compile time (the common case
// of a force pass that only integrates), which keeps their code out of the
// evaluation loop.  EMIT: record the accepted (cell, group) pairs for the
// learned correction.  The plain walk without energy sums keeps its
// compensated sums, group box and node counts in shared memory and runs six
// CTAs per SM (80 registers, no spills); the other forms keep them in
// registers.
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE>
__host__ __device__ constexpr bool wc_six() { return !MAGGM && !REL && !BRK && NOPE; }
// The walks with dipole / 1PN terms and without breakdown rows take the same
// shared-memory form and run four CTAs per SM instead of three (torus
// N = 65,536 with the full force set: 12 % faster).  The relativistic walk
// without them keeps the register form: on small systems, which a single
// wave covers, the shared-memory form only adds work (N = 2,048: 6 % slower).
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE>
__host__ __device__ constexpr bool wc_four() { return MAGGM && !BRK; }
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE>
__host__ __device__ constexpr bool wc_sh() { return wc_six<MAGGM, REL, BRK, PER, NOPE>() || wc_four<MAGGM, REL, BRK, PER, NOPE>(); }
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE>
__host__ __device__ constexpr int wc_min_blocks() {
    return wc_six<MAGGM, REL, BRK, PER, NOPE>() ? 6 : wc_four<MAGGM, REL, BRK, PER, NOPE>() ? 4 : (MAGGM || REL || BRK) ? 3 : 5;
}

// One CTA of the walk: warps vb * WC_WARPS .. + WC_WARPS - 1 of the target
// order, with WC_THREADS threads and wc_smem_bytes() of dynamic shared memory.
// SPLIT > 1 (WC_WARPS, or 2 WC_WARPS in a CTA of that many warps, whose
// accumulators then stay in registers): the CTA's SPLIT warps walk the same
// group vb of 32 targets.  Every warp descends the levels above C.split_level; a node at
// or above it is evaluated (aggregate or leaf points) only by warp
// (index mod SPLIT), and a node at split_level is opened only by that warp,
// so each subtree below it is walked once.  The warps' compensated partial
// sums are then added in warp order by warp 0, which writes the target.
// The interaction list of every target is the one of the plain walk; only
// the order of the sums differs.
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, bool EMIT, int SPLIT = 1, int STACK = WC_STACK,
          bool YUK = true>
__device__ __forceinline__ void walkc_body(const DevParams& P, const DevState& S, const TreeBufs& T,
                                           const int* d_root, FrameCtl* ctl, const ForceCtx& C, int vb) {
    static_assert(SPLIT == 1 || ((SPLIT == WC_WARPS || SPLIT == 2 * WC_WARPS) && !EMIT),
                  "split walk: one group per CTA of SPLIT warps, no records");
    constexpr bool NEEDC = MAGGM || REL;
    constexpr int NWARPS = SPLIT > WC_WARPS ? SPLIT : WC_WARPS;         // warps of the CTA
    // shared-memory form (six or four CTAs per SM); its rows hold ACC_SH_THREADS columns
    constexpr bool SHF = NWARPS == WC_WARPS && wc_sh<MAGGM, REL, BRK, PER, NOPE>();
    using AccT = Acc<MAGGM, BRK, SHF>;
    using WS = WcSmem<NEEDC, SHF ? WC_POOL_SHF : WC_POOL_WIDE, STACK>;
    unsigned char* wc_smem = geon_dsmem + AccT::SH_BYTES;
    WS* Wall = reinterpret_cast<WS*>(wc_smem);
    float* s_age = reinterpret_cast<float*>(Wall + NWARPS);
    float* s_segdt = s_age + HIST_LEN;
    if (REL) load_hist_tables(C, s_age, s_segdt);
    const int warp = threadIdx.x >> 5;
    const unsigned lane = threadIdx.x & 31;
    WS& W = Wall[warp];
    const int k0 = (SPLIT > 1 ? vb * 32 : (vb * WC_WARPS + warp) * 32) + (int)lane;
    int sysId;
    const int ti = walk_target(S, T, ctl, C, k0, sysId);
    const bool valid = ti >= 0;
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    if (active == 0) return;
    if (C.roots) sysId = __shfl_sync(0xffffffffu, sysId, __ffs(active) - 1);
    Tgt t;
    if (valid) { t = load_target(S, ti); target_coupling(P, t); }
    else { t = Tgt{}; t.idx = -1; }
    AccT A;
    A.init();
    unsigned inter = 0;
    const bool pe = NOPE ? false : (C.pe != 0);
    // bounding box of the warp's particles (padded beyond the rounding of hi + lo)
    const float bx0 = warp_min_f(valid ? t.x : 3.0e38f), bx1 = warp_max_f(valid ? t.x : -3.0e38f);
    const float by0 = warp_min_f(valid ? t.y : 3.0e38f), by1 = warp_max_f(valid ? t.y : -3.0e38f);
    const float gcx0 = 0.5f * (bx0 + bx1), gcy0 = 0.5f * (by0 + by1);
    const float ghx0 = 0.5f * (bx1 - bx0) * (1.f + 1e-6f) + 1e-6f * fabsf(gcx0) + 1e-30f;
    const float ghy0 = 0.5f * (by1 - by0) * (1.f + 1e-6f) + 1e-6f * fabsf(gcy0) + 1e-30f;
    if (SHF && lane == 0) { W.gbox[0] = gcx0; W.gbox[1] = gcy0; W.gbox[2] = ghx0; W.gbox[3] = ghy0; }
    const bool groupTests = !P.periodic || P.topology == GEON_TORUS;

    const int root = C.roots ? C.roots[sysId] : *d_root;
    const bool treeOk = (ctl->err & (ERR_NODE_OVERFLOW | ERR_BAD_INDEX)) == 0;
    const int nInt0 = ctl->nInternal, nLeaf0 = ctl->nLeaves, nValid0 = ctl->nValid;
    if (SHF && lane == 0) { W.counts[0] = nInt0; W.counts[1] = nLeaf0; W.counts[2] = nValid0; }
    int top = 0, npart = 0, nfull = 0, lcnt = 0;   // pool: nfull slots from the bottom, npart from the top
    int rcnt = 0;                                                     // EMIT: records of this warp
    const int grp = SPLIT > 1 ? vb : vb * WC_WARPS + warp;
    if (root != ROOT_NONE && treeOk) {
        if (lane == 0) { W.stk_node[0] = root; W.stk_mask[0] = active; }
        top = 1;
    }
    __syncwarp();
    while (top > 0) {
        // wide pops while the stack has room; single pops (depth first) near the limit
        int k = min(min(WC_POP, top), (STACK - WC_RESERVE - top) / 3);
        if (k < 1) k = 1;
        if (top + 3 > STACK) { if (lane == 0) atomicOr(&ctl->err, ERR_STACK_OVERFLOW); break; }
        int node = -1;
        unsigned mask = 0;
        if ((int)lane < k) { node = W.stk_node[top - k + lane]; mask = W.stk_mask[top - k + lane]; }
        __syncwarp();
        top -= k;
        // node records, one per lane; classification against the group box
        int kind = 0;                          // 0 none, 1 leaf, 2 all accept, 3 all open, 4 mixed
        float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nc = make_float4(0.f, 0.f, 0.f, 0.f);
        int4 lm = make_int4(0, 0, 0, 0);
        if (node >= 0) {
            if (node & LEAF_REF) {
                const int li = node & ~LEAF_REF;
                if (li < (SHF ? W.counts[1] : nLeaf0)) {
                    lm = T.leaf_meta[li];
                    const float lmass = T.leaf_a[li].z;
                    if (lmass >= EPS_F && lm.x >= 0 && lm.x + lm.y <= (SHF ? W.counts[2] : nValid0)) kind = 1;   // forces.js:630,643
                } else atomicOr(&ctl->err, ERR_BAD_INDEX);
            } else if (node < (SHF ? W.counts[0] : nInt0)) {
                na = T.int_a[node];
                nc = T.int_c[node];
                if (na.z >= EPS_F) {
                    kind = 4;
                    if (groupTests) {
                        const float gcx = SHF ? W.gbox[0] : gcx0, gcy = SHF ? W.gbox[1] : gcy0;
                        const float ghx = SHF ? W.gbox[2] : ghx0, ghy = SHF ? W.gbox[3] : ghy0;
                        float dx, dy;
                        if (PER && P.periodic) {
                            dx = wrap_axis_comp(na.x, gcx, nc.x, P.W, P.W_lo, P.halfW);
                            dy = wrap_axis_comp(na.y, gcy, nc.y, P.H, P.H_lo, P.halfH);
                        } else {
                            dx = __fadd_rn(__fsub_rn(na.x, gcx), nc.x);
                            dy = __fadd_rn(__fsub_rn(na.y, gcy), nc.y);
                        }
                        const float ax = fabsf(dx), ay = fabsf(dy);
                        const bool wrapSafe = !PER || !P.periodic || (ax + ghx < 0.999f * P.halfW && ay + ghy < 0.999f * P.halfH);
                        if (wrapSafe) {
                            const float mnx = fmaxf(ax - ghx, 0.f), mny = fmaxf(ay - ghy, 0.f);
                            const float mxx = ax + ghx, mxy = ay + ghy;
                            const float dmin2 = mnx * mnx + mny * mny, dmax2 = mxx * mxx + mxy * mxy;
                            if (nc.z < P.thetaSq * dmin2 * (1.f - 1e-5f)) kind = 2;
                            else if (nc.z >= P.thetaSq * dmax2 * (1.f + 1e-5f)) kind = 3;
                        }
                    }
                }
            } else atomicOr(&ctl->err, ERR_BAD_INDEX);
        }
        unsigned myAcc = kind == 2 ? mask : 0u, myOpen = kind == 3 ? mask : 0u;
        for (unsigned tm = __ballot_sync(0xffffffffu, kind == 4); tm; tm &= tm - 1) {   // forces.js:680
            const int jj = __ffs(tm) - 1;
            const float cx = __shfl_sync(0xffffffffu, na.x, jj), cy = __shfl_sync(0xffffffffu, na.y, jj);
            const float clx = __shfl_sync(0xffffffffu, nc.x, jj), cly = __shfl_sync(0xffffffffu, nc.y, jj);
            const float s2 = __shfl_sync(0xffffffffu, nc.z, jj), lvl = __shfl_sync(0xffffffffu, nc.w, jj);
            const unsigned msk = __shfl_sync(0xffffffffu, mask, jj);
            bool accept = false;
            if ((msk >> lane) & 1u) {
                float rx, ry;
                displacement_p<PER>(P, t.x, t.y, cx, clx - t.xlo, cy, cly - t.ylo, rx, ry);
                const float rhs = P.thetaSq * __fmaf_rn(rx, rx, ry * ry);
                accept = s2 < rhs;
                if (fabsf(rhs - s2) <= 1e-6f * s2)
                    accept = accept_exact<PER>(P, t.xd(), t.yd(), (double)cx + (double)clx, (double)cy + (double)cly, lvl);
            }
            const unsigned acc = __ballot_sync(0xffffffffu, accept);
            if ((int)lane == jj) { myAcc = acc & msk; myOpen = msk & ~acc; }
        }
        if (SPLIT > 1 && node >= 0 && kind != 0) {                   // split walk: this warp's share
            const bool isLeaf = (node & LEAF_REF) != 0;
            const int lvl = isLeaf ? lm.z : (int)nc.w;
            if (lvl <= C.split_level) {
                const unsigned id = isLeaf ? (unsigned)(node & ~LEAF_REF) : (unsigned)node;
                if ((int)(id % (unsigned)SPLIT) != warp) {
                    myAcc = 0u;
                    if (lvl == C.split_level) myOpen = 0u;
                    if (kind == 1) kind = 0;
                }
            }
        }
        if (EMIT) {                                                   // learned correction: (cell, group) records
            // one record per accepted cell: the node and the lanes that accept
            // it, in this warp's own segment, in walk order
            const bool mine = myAcc != 0;
            const unsigned rb = __ballot_sync(0xffffffffu, mine);
            if (mine) {
                const int slot = rcnt + __popc(rb & lanemask_lt());
                if (slot < C.rec_cap) C.recs[(size_t)grp * C.rec_cap + slot] = make_uint2((uint32_t)node, myAcc);
            }
            rcnt += __popc(rb);
        }
        const unsigned leafMask = kind == 1 ? mask : 0u;
        const bool bucket = leafMask && lm.y > LEAF_CAP;
        const int myPts = (leafMask && !bucket) ? lm.y : 0;
        // a lane holds one node: its entries (an aggregate, or a leaf's
        // points) are all taken by every lane or all by some.  Entries every
        // lane takes fill the pool from the bottom, in lane order, and are
        // evaluated by position; the others fill it from the top, each lane's
        // block in ascending slots, and then go, source by source, to the
        // lists of the lanes that take them
        const bool accFull = myAcc != 0 && myAcc == active;
        const bool ptsFull = myPts > 0 && leafMask == active;
        const bool isFull = accFull || ptsFull;
        const int myEnt = (myAcc ? 1 : 0) + myPts;
        const int myFull = isFull ? myEnt : 0;
        // one prefix sum for both counts, 8 bits apiece (each totals at most 64)
        const int sc = warp_incl_scan_i(myEnt | (myFull << 8));
        const int scTot = __shfl_sync(0xffffffffu, sc, 31);
        const int incl = sc & 0xff, fincl = sc >> 8;
        const int tot = scTot & 0xff, ftot = scTot >> 8;
        if (nfull + npart + tot > WS::kPool)
            flush_pool<MAGGM, REL, BRK, PER, YUK>(P, S, C, s_age, s_segdt, W, nfull, lcnt, npart, t, A, inter, pe);
        const int e0 = isFull ? nfull + fincl - myFull : WS::kPool - (npart + incl - fincl);
        if (myAcc) {                                                  // forces.js:682-685
            const float4 nb = T.int_b[node];
            W.a[e0] = na;
            W.b[e0] = make_float4(nc.x, nc.y, nb.x, nb.y);
            if (NEEDC) W.c[e0] = make_float4(0.f, nb.z, nb.w, 0.f);
            W.ref[e0] = AGG_REF;
        }
        for (int q = 0; q < myPts; q++) stage_point<NEEDC>(T, W, e0 + q, lm.x + q);   // forces.js:643-679
        nfull += ftot;
        npart += tot - ftot;
        __syncwarp();
        for (unsigned gm = __ballot_sync(0xffffffffu, myAcc != 0 && !accFull); gm; gm &= gm - 1) {
            const int jj = __ffs(gm) - 1;
            list_add(W, __shfl_sync(0xffffffffu, myAcc, jj), __shfl_sync(0xffffffffu, e0, jj), 1, lcnt);
        }
        for (unsigned gm = __ballot_sync(0xffffffffu, myPts > 0 && !ptsFull); gm; gm &= gm - 1) {
            const int jj = __ffs(gm) - 1;
            list_add(W, __shfl_sync(0xffffffffu, leafMask, jj), __shfl_sync(0xffffffffu, e0, jj),
                     __shfl_sync(0xffffffffu, myPts, jj), lcnt);
        }
        // leaves holding more than LEAF_CAP points (level-31 buckets)
        for (unsigned bk = __ballot_sync(0xffffffffu, bucket); bk; bk &= bk - 1) {
            const int jj = __ffs(bk) - 1;
            const int bstart = __shfl_sync(0xffffffffu, lm.x, jj), bcount = __shfl_sync(0xffffffffu, lm.y, jj);
            const unsigned bmask = __shfl_sync(0xffffffffu, leafMask, jj);
            const bool bfull = bmask == active;
            for (int b0 = 0; b0 < bcount; b0 += 32) {
                const int chunk = min(32, bcount - b0);
                if (nfull + npart + chunk > WS::kPool)
                    flush_pool<MAGGM, REL, BRK, PER, YUK>(P, S, C, s_age, s_segdt, W, nfull, lcnt, npart, t, A, inter, pe);
                const int first = bfull ? nfull : WS::kPool - npart - chunk;
                if ((int)lane < chunk) stage_point<NEEDC>(T, W, first + lane, bstart + b0 + lane);
                __syncwarp();
                if (bfull) nfull += chunk;
                else { list_add(W, bmask, first, chunk, lcnt); npart += chunk; }
            }
        }
        // children of nodes some lanes open (forces.js:686-692)
        int4 ch = make_int4(-1, -1, -1, -1);
        int myCh = 0;
        if (myOpen) {
            ch = T.int_child[node];
            myCh = (ch.x >= 0) + (ch.y >= 0) + (ch.z >= 0) + (ch.w >= 0);
        }
        const int chIncl = warp_incl_scan_i(myCh);
        const int chTot = __shfl_sync(0xffffffffu, chIncl, 31);
        if (myCh) {
            int pos = top + chIncl - myCh;
            if (ch.x >= 0) { W.stk_node[pos] = ch.x; W.stk_mask[pos++] = myOpen; }
            if (ch.y >= 0) { W.stk_node[pos] = ch.y; W.stk_mask[pos++] = myOpen; }
            if (ch.z >= 0) { W.stk_node[pos] = ch.z; W.stk_mask[pos++] = myOpen; }
            if (ch.w >= 0) { W.stk_node[pos] = ch.w; W.stk_mask[pos++] = myOpen; }
        }
        top += chTot;
        __syncwarp();
    }
    flush_pool<MAGGM, REL, BRK, PER, YUK>(P, S, C, s_age, s_segdt, W, nfull, lcnt, npart, t, A, inter, pe);
    if constexpr (SPLIT > 1) {
        // partial sums of warps 1.. through their (now unused) stacks; warp 0 adds them in order
        constexpr int NQ = AccT::NQ;
        static_assert((2 * NQ + 1) * 32 * sizeof(float) <= sizeof(W.stk_node) + sizeof(W.stk_mask),
                      "split walk exchange area");
        A.flush();
        if (warp > 0) {
            float* xw = reinterpret_cast<float*>(W.stk_node);
#pragma unroll
            for (int q = 0; q < NQ; q++) { xw[q * 32 + lane] = A.hi(q); xw[(NQ + q) * 32 + lane] = A.lo(q); }
            reinterpret_cast<unsigned*>(xw)[2 * NQ * 32 + lane] = inter;
        }
        __syncthreads();
        if (warp > 0) return;
        for (int k = 1; k < SPLIT; k++) {
            const float* xk = reinterpret_cast<const float*>(Wall[k].stk_node);
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const df s2 = two_sum(A.hi(q), xk[q * 32 + lane]);
                A.hi(q) = s2.hi;
                A.lo(q) = __fadd_rn(__fadd_rn(A.lo(q), xk[(NQ + q) * 32 + lane]), s2.lo);
            }
            inter += reinterpret_cast<const unsigned*>(xk)[2 * NQ * 32 + lane];
        }
    }
    if (EMIT && lane == 0) {
        const float cx = SHF ? W.gbox[0] : gcx0, cy = SHF ? W.gbox[1] : gcy0;
        const float hx = SHF ? W.gbox[2] : ghx0, hy = SHF ? W.gbox[3] : ghy0;
        C.gcen[grp] = make_float4(cx, cy, sqrtf(hx * hx + hy * hy) * (1.f + 1e-5f), 0.f);
        C.rec_cnt[grp] = rcnt;
        atomicMax(C.rec_max, (unsigned)rcnt);
        atomicAdd(C.rec_total, (unsigned long long)rcnt);
    }
    finalize_target<MAGGM, BRK>(P, S, C, ctl, t, valid, A, inter, sysId);
}

template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE = false, bool EMIT = false, bool YUK = true>
__global__ void __launch_bounds__(WC_THREADS, wc_min_blocks<MAGGM, REL, BRK, PER, NOPE>())
walkc_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root, FrameCtl* ctl, ForceCtx C) {
    walkc_body<MAGGM, REL, BRK, PER, NOPE, EMIT, 1, WC_STACK, YUK>(P, S, T, d_root, ctl, C, blockIdx.x);
}

// Dynamic shared memory of one walk CTA: accumulator rows (six-CTA form),
// the four warps' stacks and source pools, and the history tables when
// relativity is on.
template <bool MAGGM, bool REL, bool BRK, int PER, bool NOPE, int NWARPS = WC_WARPS, int STACK = WC_STACK>
constexpr size_t wc_smem_bytes() {
    constexpr bool SHF = NWARPS == WC_WARPS && wc_sh<MAGGM, REL, BRK, PER, NOPE>();
    return Acc<MAGGM, BRK, SHF>::SH_BYTES + sizeof(WcSmem<MAGGM || REL, SHF ? WC_POOL_SHF : WC_POOL_WIDE, STACK>) * NWARPS +
           (REL ? 2 * HIST_LEN * sizeof(float) : 0);
}
static_assert(7 * (wc_smem_bytes<false, false, false, 2, true, WC_WARPS, WC_STACK_SHORT>() + 1024) <= 228 * 1024,
              "seven short-stack torus plain walk CTAs per SM must fit in shared memory");
static_assert(6 * (wc_smem_bytes<false, false, false, false, true>() + 1024) <= 228 * 1024,
              "six plain walk CTAs per SM must fit in shared memory");
static_assert(6 * (wc_smem_bytes<false, false, false, true, true>() + 1024) <= 228 * 1024,
              "six periodic plain walk CTAs per SM must fit in shared memory");
static_assert(4 * (wc_smem_bytes<true, true, false, true, false>() + 1024) <= 228 * 1024,
              "four dipole / 1PN walk CTAs per SM must fit in shared memory");
static_assert(5 * (wc_smem_bytes<false, false, false, true, false>() + 1024) <= 228 * 1024,
              "five walk CTAs per SM must fit in shared memory");

}  // namespace geon
