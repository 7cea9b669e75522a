// push_dev.cuh — device code of the per-particle passes (push.cu).  A body
// takes the virtual block index and block count of its grid-stride loop, so
// the kernels of push.cu and the persistent frame kernel (force.cu) run the
// same code.
#pragma once

#include "push.cuh"

namespace geon {

__device__ __forceinline__ bool push_on(const DevParams& P, uint32_t bit) { return (P.toggles & bit) != 0; }

__device__ __forceinline__ void warp_max_atomic(unsigned long long* accBits, unsigned long long* cycBits, double aSq,
                                                double wc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        aSq = fmax(aSq, __shfl_xor_sync(0xffffffffu, aSq, o));
        wc = fmax(wc, __shfl_xor_sync(0xffffffffu, wc, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_pos_double(accBits, aSq);
        atomic_max_pos_double(cycBits, wc);
    }
}

// ---- frame-start scan ----------------------------------------------------------------
// Planner maxima of the current forces (integrator.js:813-836) into the two
// accumulators (double bits, zero beforehand).
__device__ __forceinline__ void scan_forces_body(DevParams P, DevState S, const FrameCtl* ctl, unsigned long long* accBits,
                                                 unsigned long long* cycBits, int vb, int nvb) {
    const int n = ctl->n;
    const int stride = nvb * blockDim.x;
    const int i0 = vb * blockDim.x + threadIdx.x;
    const int iters = (n + stride - 1) / stride;
    for (int it = 0; it < iters; it++) {
        const int i = i0 + it * stride;
        double aSq = 0.0, wc = 0.0;
        if (i < n) {
            const float4 f = S.force[i];
            const double im = (double)S.spin[i].w;
            aSq = ((double)f.x * f.x + (double)f.y * f.y) * im * im;
            if (push_on(P, GEON_MAGNETIC) || P.extBz != 0.f) {
                const double absBz = fabs((double)f.z);
                if (absBz > 0) wc = fmax(wc, fabs((double)S.pos[i].w) * absBz * im);
            }
            if (push_on(P, GEON_GRAVITOMAG)) {
                const double absBgz = fabs((double)f.w);
                if (absBgz > 0) wc = fmax(wc, 4.0 * absBgz);
            }
            if (!(aSq == aSq)) aSq = 0.0;
            if (!(wc == wc)) wc = 0.0;
        }
        warp_max_atomic(accBits, cycBits, aSq, wc);
    }
}

__device__ __forceinline__ void clear_planner_body(FrameCtl* ctl, int vb, int nvb) {
    ctl->maxAccelSqBits = 0ull;
    ctl->maxCycBits = 0ull;
}

// ---- substep push -----------------------------------------------------------------------
__device__ __forceinline__ void push_body(DevParams P, DevState S, const FrameCtl* ctl, float dtSub0, PushFlags F,
                            const double* __restrict__ sys_dt, int vb, int nvb) {
    const int n = ctl->n;
    const bool rel = P.rel != 0;
    const bool mag = push_on(P, GEON_MAGNETIC), gm = push_on(P, GEON_GRAVITOMAG), grav = push_on(P, GEON_GRAVITY);
    const bool hasExtBz = P.extBz != 0.f;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        float dtSub = dtSub0;
        if (sys_dt) {                           // batched: the substep of this particle's system
            const double d = sys_dt[S.sys[i]];
            if (!(d > 0.0)) continue;
            dtSub = (float)d;
        }
        const float halfDt = dtSub * 0.5f;
        float4 pos = S.pos[i];
        float2 plo = S.pos_lo[i];
        float4 vel = S.vel[i];                  // wx, wy, vx, vy
        float4 spn = S.spin[i];                 // angw, angVel, radius, invMass
        const float4 f = S.force[i];
        const float invM = spn.w;
        if (F.has1PN) S.f1pnOld[i] = S.f1pn[i];
        const float halfDtOverM = halfDt * invM;
        float wx = vel.x, wy = vel.y;
        wx += f.x * halfDtOverM; wy += f.y * halfDtOverM;          // half-kick 1
        if (F.needBoris) {                                           // Boris rotation
            float t = 0.f;
            if (mag || hasExtBz) t += (pos.w * 0.5f * invM) * f.z;
            if (gm) t += 2.f * f.w;
            if (t != 0.f) {
                const float gamma = rel ? sqrtf(1.f + wx * wx + wy * wy) : 1.f;
                t *= dtSub / gamma;
                const float s = 2.f * t / (1.f + t * t);
                const float wpx = wx + wy * t, wpy = wy - wx * t;
                wx = wx + wpy * s;
                wy = wy - wpx * s;
            }
        }
        wx += f.x * halfDtOverM; wy += f.y * halfDtOverM;          // half-kick 2
        if (wx != wx || wy != wy) { wx = 0.f; wy = 0.f; vel.z = 0.f; vel.w = 0.f; }
        float angw = spn.x, angVel = spn.y;
        const float radius = spn.z;
        if (F.needSpinOrbit && fabsf(angVel) >= EPS_F) {            // integrator.js:937-963
            const float2 mm = S.mom[i];
            const float IxOmega = mm.y;
            if (fabsf(IxOmega) >= EPS_F) {
                const float4 g = S.grad[i];
                const float dtOverM = dtSub * invM;
                if (mag && fabsf(pos.w) > EPS_F) {
                    const float mu = mm.x;
                    angw -= mu * (vel.z * g.x + vel.w * g.y) * dtSub / IxOmega;
                    wx += mu * g.x * dtOverM; wy += mu * g.y * dtOverM;
                }
                if (gm) {
                    const float L = mm.y;
                    angw -= L * (vel.z * g.z + vel.w * g.w) * dtSub / IxOmega;
                    wx -= L * g.z * dtOverM; wy -= L * g.w * dtOverM;
                }
                if (angw != angw) angw = 0.f;
                const float sr = angw * radius;
                angVel = rel ? angw / sqrtf(1.f + sr * sr) : angw;
            }
        }
        if (F.needTorques) {                                         // integrator.js:966-980
            const float4 tq = S.torque[i];
            float torque = 0.f;
            if (gm && rel) torque += tq.y;
            if (grav) torque += tq.x;
            torque += tq.z;
            if (torque != 0.f) {
                const float I = INERTIA_K * pos.z * radius * radius;
                if (I >= EPS_F) {
                    angw += torque * dtSub / I;
                    if (angw != angw) angw = 0.f;
                    const float sr = angw * radius;
                    angVel = rel ? angw / sqrtf(1.f + sr * sr) : angw;
                }
            }
        }
        // drift (integrator.js:1270-1278)
        const float invG = rel ? 1.f / sqrtf(1.f + wx * wx + wy * wy) : 1.f;
        const float vx = wx * invG, vy = wy * invG;
        angVel = rel ? angw / sqrtf(1.f + angw * angw * radius * radius) : angw;
        {
            df sx = two_sum(pos.x, vx * dtSub);
            sx.lo = __fadd_rn(sx.lo, plo.x);
            sx = fast_two_sum(sx.hi, sx.lo);
            df sy = two_sum(pos.y, vy * dtSub);
            sy.lo = __fadd_rn(sy.lo, plo.y);
            sy = fast_two_sum(sy.hi, sy.lo);
            pos.x = sx.hi; plo.x = sx.lo;
            pos.y = sy.hi; plo.y = sy.lo;
        }
        S.pos[i] = pos;
        S.pos_lo[i] = plo;
        S.vel[i] = make_float4(wx, wy, vx, vy);
        spn.x = angw; spn.y = angVel;
        S.spin[i] = spn;
    }
}

__device__ __forceinline__ void vv_kick_body(DevParams P, DevState S, const FrameCtl* ctl, float halfDt, int vb, int nvb) {
    const int n = ctl->n;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        const float invM = S.spin[i].w;
        const float2 fn = S.f1pn[i], fo = S.f1pnOld[i];
        float4 v = S.vel[i];
        const float h = halfDt * invM;
        v.x += (fn.x - fo.x) * h;
        v.y += (fn.y - fo.y) * h;
        if (v.x != v.x || v.y != v.y) { v.x = 0.f; v.y = 0.f; v.z = 0.f; v.w = 0.f; }
        S.vel[i] = v;
    }
}

// ---- history (integrator.js:1549-1565; signal-delay tables) ----------------------------
__device__ __forceinline__ void hist_tables_body(const double* hist_t, double simTime, float* age, float* segdt, int vb, int nvb) {
    for (int k = vb * blockDim.x + threadIdx.x; k < HIST_LEN; k += nvb * blockDim.x) {
        age[k] = (float)(simTime - hist_t[k]);
        segdt[k] = (float)(hist_t[(k + 1) & HIST_MASK] - hist_t[k]);
    }
}

__device__ __forceinline__ void record_history_body(DevState S, const FrameCtl* ctl, double* hist_t, int slot, double simTime, int vb, int nvb) {
    const int n = ctl->n;
    if (vb == 0 && threadIdx.x == 0) hist_t[slot] = simTime;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        const float4 p = S.pos[i];
        const float2 pl = S.pos_lo[i];
        const float4 v = S.vel[i];
        S.hist[(size_t)i * HIST_LEN + slot] = make_float4(p.x + pl.x, p.y + pl.y, v.z, v.w);
        S.hist_angw[(size_t)i * HIST_LEN + slot] = S.spin[i].x;
        const int c = S.hist_cnt[i];
        if (c < HIST_LEN) S.hist_cnt[i] = c + 1;
    }
}

// ---- boundary (integrator.js:1798-1824) --------------------------------------------------
__device__ __forceinline__ void shift_comp(float& hi, float& lo, float L, float L_lo, float sign) {
    df s = two_sum(hi, sign * L);
    s.lo = __fadd_rn(s.lo, __fadd_rn(lo, sign * L_lo));
    s = fast_two_sum(s.hi, s.lo);
    hi = s.hi; lo = s.lo;
}
__device__ __forceinline__ void mirror_comp(float& hi, float& lo, float L, float L_lo) {   // v -> L - v
    df s = two_sum(L, -hi);
    s.lo = __fadd_rn(s.lo, __fsub_rn(L_lo, lo));
    s = fast_two_sum(s.hi, s.lo);
    hi = s.hi; lo = s.lo;
}

__device__ __forceinline__ void boundary_body(DevParams P, DevState S, FrameCtl* ctl, int* keep, int vb, int nvb) {
    const int n = ctl->n;
    int removed = 0;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        float4 pos = S.pos[i];
        float2 pl = S.pos_lo[i];
        int k = 1;
        const double x = (double)pos.x + pl.x, y = (double)pos.y + pl.y;
        const double left = P.offXd, top = P.offYd, right = P.offXd + P.Wd, bottom = P.offYd + P.Hd;
        if (P.boundary == GEON_BOUND_DESPAWN) {
            if (x < left - DESPAWN_MARGIN || x > right + DESPAWN_MARGIN ||
                y < top - DESPAWN_MARGIN || y > bottom + DESPAWN_MARGIN) k = 0;
        } else if (P.boundary == GEON_BOUND_LOOP) {                 // topology.js:81-135
            float4 v = S.vel[i];
            float4 sp = S.spin[i];
            const float W = P.W, H = P.H;
            auto X = [&]() { return (double)pos.x + pl.x; };
            auto Y = [&]() { return (double)pos.y + pl.y; };
            if (P.topology == GEON_TORUS) {
                if (X() < 0) shift_comp(pos.x, pl.x, W, P.W_lo, 1.f);
                else if (X() > P.Wd) shift_comp(pos.x, pl.x, W, P.W_lo, -1.f);
                if (Y() < 0) shift_comp(pos.y, pl.y, H, P.H_lo, 1.f);
                else if (Y() > P.Hd) shift_comp(pos.y, pl.y, H, P.H_lo, -1.f);
            } else if (P.topology == GEON_KLEIN) {
                if (X() < 0) shift_comp(pos.x, pl.x, W, P.W_lo, 1.f);
                else if (X() > P.Wd) shift_comp(pos.x, pl.x, W, P.W_lo, -1.f);
                if (Y() < 0 || Y() > P.Hd) {
                    shift_comp(pos.y, pl.y, H, P.H_lo, Y() < 0 ? 1.f : -1.f);
                    mirror_comp(pos.x, pl.x, W, P.W_lo);
                    v.x = -v.x; v.z = -v.z; sp.x = -sp.x; sp.y = -sp.y;
                }
            } else {
                for (int it = 0; it < 2; it++) {
                    bool wrapped = false;
                    if (X() < 0 || X() > P.Wd) {
                        shift_comp(pos.x, pl.x, W, P.W_lo, X() < 0 ? 1.f : -1.f);
                        mirror_comp(pos.y, pl.y, H, P.H_lo);
                        v.y = -v.y; v.w = -v.w; sp.x = -sp.x; sp.y = -sp.y;
                        wrapped = true;
                    }
                    if (Y() < 0 || Y() > P.Hd) {
                        shift_comp(pos.y, pl.y, H, P.H_lo, Y() < 0 ? 1.f : -1.f);
                        mirror_comp(pos.x, pl.x, W, P.W_lo);
                        v.x = -v.x; v.z = -v.z; sp.x = -sp.x; sp.y = -sp.y;
                        wrapped = true;
                    }
                    if (!wrapped) break;
                }
            }
            S.pos[i] = pos; S.pos_lo[i] = pl;
            S.vel[i] = v; S.spin[i] = sp;
        } else if (P.boundary == GEON_BOUND_BOUNCE) {
            if (x < left) { pos.x = (float)left; pl.x = (float)(left - (double)pos.x); }
            else if (x > right) { pos.x = (float)right; pl.x = (float)(right - (double)pos.x); }
            if (y < top) { pos.y = (float)top; pl.y = (float)(top - (double)pos.y); }
            else if (y > bottom) { pos.y = (float)bottom; pl.y = (float)(bottom - (double)pos.y); }
            S.pos[i] = pos; S.pos_lo[i] = pl;
        }
        keep[i] = k;
        removed += 1 - k;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) removed += __shfl_xor_sync(0xffffffffu, removed, o);
    if ((threadIdx.x & 31) == 0 && removed) atomicAdd(&ctl->nRemoved, removed);
}

// Stable compaction: particle i moves to slot dst[i] when keep[i].  `n_cap`
// is the row stride of the force-breakdown rows.  History rings are copied
// only for particles holding samples (a ring without samples is never read),
// so slots beyond the ring capacity (merge spawns) are never touched there.
__device__ __forceinline__ void compact_body(DevState S, DevState D, const int* keep, const int* dst, int n, int n_cap,
                               int with_hist, int with_brk, int vb, int nvb) {
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        if (!keep[i]) continue;
        const int d = dst[i];
        D.pos[d] = S.pos[i]; D.pos_lo[d] = S.pos_lo[i]; D.vel[d] = S.vel[i]; D.spin[d] = S.spin[i];
        D.mom[d] = S.mom[i]; D.force[d] = S.force[i]; D.grad[d] = S.grad[i]; D.torque[d] = S.torque[i];
        D.f1pn[d] = S.f1pn[i]; D.f1pnOld[d] = S.f1pnOld[i]; D.ctime[d] = S.ctime[i]; D.id[d] = S.id[i];
        D.matter[d] = S.matter[i];
        const int hc = S.hist_cnt[i];
        D.hist_cnt[d] = hc;
        if (with_brk) {
            for (int r = 0; r < 12; r++) D.brk[(size_t)r * n_cap + d] = S.brk[(size_t)r * n_cap + i];
        }
        if (with_hist && hc > 0) {
            const float4* hs = S.hist + (size_t)i * HIST_LEN;
            float4* hd = D.hist + (size_t)d * HIST_LEN;
            for (int k = 0; k < HIST_LEN; k++) hd[k] = hs[k];
            const float* as = S.hist_angw + (size_t)i * HIST_LEN;
            float* ad = D.hist_angw + (size_t)d * HIST_LEN;
            for (int k = 0; k < HIST_LEN; k++) ad[k] = as[k];
        }
    }
}

// ---- conserved quantities (energy.js:11-62) in FP64 ---------------------------------------
__device__ __forceinline__ double block_sum_d(double v, double* sm) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sm[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sm[k];
    return r;
}

// out[0..9]: linearKE, spinKE, px, py, totalMass, sum m x, sum m y, pe*2, orbital, spin
__device__ __forceinline__ void stats_pass1_body(DevParams P, DevState S, const FrameCtl* ctl, double* out, int vb, int nvb) {
    __shared__ double sm[32];
    const int n = ctl->n;
    const bool rel = P.rel != 0;
    double acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        const float4 p = S.pos[i];
        const float2 pl = S.pos_lo[i];
        const float4 v = S.vel[i];
        const float4 s = S.spin[i];
        const double pm = p.z, rSq = (double)s.z * s.z;
        const double wx = v.x, wy = v.y;
        if (rel) {
            const double wSq = wx * wx + wy * wy;
            const double gamma = sqrt(1 + wSq);
            acc[0] += wSq / (gamma + 1) * pm;
            const double srSq = (double)s.x * s.x * rSq;
            acc[1] += INERTIA_K * pm * srSq / (sqrt(1 + srSq) + 1);
        } else {
            const double spSq = (double)v.z * v.z + (double)v.w * v.w;
            acc[0] += 0.5 * pm * spSq;
            acc[1] += 0.5 * (double)INERTIA_K * pm * rSq * (double)s.y * s.y;
        }
        acc[2] += pm * wx; acc[3] += pm * wy;
        acc[4] += pm;
        acc[5] += pm * ((double)p.x + pl.x);
        acc[6] += pm * ((double)p.y + pl.y);
        acc[7] += (double)S.torque[i].w;
    }
    for (int k = 0; k < 8; k++) {
        const double r = block_sum_d(acc[k], sm);
        if (threadIdx.x == 0) atomicAdd(&out[k], r);
    }
}

__device__ __forceinline__ void stats_pass2_body(DevParams P, DevState S, const FrameCtl* ctl, double* out, int vb, int nvb) {
    __shared__ double sm[32];
    const int n = ctl->n;
    const double M = out[4];
    if (!(M > 0)) return;
    const double cx = out[5] / M, cy = out[6] / M;
    double orb = 0, spin = 0;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        const float4 p = S.pos[i];
        const float2 pl = S.pos_lo[i];
        const float4 v = S.vel[i];
        const float4 s = S.spin[i];
        const double pm = p.z;
        const double dx = (double)p.x + pl.x - cx, dy = (double)p.y + pl.y - cy;
        orb += dx * (pm * v.y) - dy * (pm * v.x);
        spin += (double)INERTIA_K * pm * ((double)s.z * s.z) * (double)s.x;
    }
    const double r0 = block_sum_d(orb, sm);
    if (threadIdx.x == 0) atomicAdd(&out[8], r0);
    const double r1 = block_sum_d(spin, sm);
    if (threadIdx.x == 0) atomicAdd(&out[9], r1);
}

// ---- launchers ------------------------------------------------------------------------

}  // namespace geon
