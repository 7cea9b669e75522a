// learn.cuh — learned far-field correction: what the network sees of a
// (cell, group) pair, the analytic second-order term, and the launchers of
// learn.cu / mlp.cu.
//
// The reference's far field is the monopole: an accepted cell acts through
// pairForce at its centre of mass with the cell's mass and charge
// (src/forces.js:680-685).  The walk of this project keeps that term for
// every target exactly.  The correction is applied once per (cell, group),
// where a group is the 32 consecutive targets of one warp of the walk and the
// cell is one some of them accept, as a linear expansion about the group's
// centre g (the centre of the bounding box of its positions):
//
//     dG(x) = V + J (x - g)
//
// of the mass-sourced field (gravity + Yukawa, per unit target mass), and
// the same for the charge-sourced field (Coulomb, per unit target charge).
// V and J sum two parts:
//   * the analytic second-order term: the mass quadrupole through the
//     softened gravity (+ Yukawa) kernel and the charge dipole through the
//     Coulomb kernel, about the centre of mass, with the Yukawa part present
//     when the cell's centre of mass lies within the Yukawa range of g;
//   * the network: 14 features of the cell seen from g -> 64 -> 64 -> 6
//     (GELU), the mass-field residual beyond that term as (value, gradient)
//     of its two components in the frame of d = COM - g.  What it learns is
//     chiefly what no moment expansion carries: the hard Yukawa cutoff
//     (forces.js:387) cutting through the cell.
// Because the group decision of the Yukawa range can differ from a target's
// own (which the walk's monopole used), the correction also swaps the
// monopole's Yukawa term for those targets.
#pragma once

#include "state.cuh"

namespace geon {

constexpr int LF = 14;         // features
constexpr int LH = 64;         // hidden width
constexpr int LO = 6;          // outputs: (value, d/du, d/dv) of the parallel and perpendicular components
constexpr int LQ = 12;         // quadratic-form entries of a training record (2 components x 6)
constexpr int LT = LO + LQ;    // training target floats per record: y* then A

// One-variable Taylor data of the radial mass kernel phi(rho), rho = r^2 + eps^2:
// the field of a unit point mass at displacement r is r * phi(rho).
struct Phi { float f0, f1, f2, f3; };

// Gravity (rho^-3/2) plus, when yk, the Yukawa kernel
// g(R) = 14 e^{-mu R} (R^-3 + mu R^-2), R = sqrt(rho)  (forces.js:205-220, 387-399).
__device__ __forceinline__ Phi mass_kernel(float rho, bool grav, bool yk, float mu) {
    Phi p{ 0.f, 0.f, 0.f, 0.f };
    const float ir = 1.f / rho;
    const float iR = rsqrtf(rho);
    if (grav) {
        const float a = ir * iR;             // rho^-3/2
        p.f0 = a; p.f1 = -1.5f * a * ir; p.f2 = 3.75f * a * ir * ir; p.f3 = -13.125f * a * ir * ir * ir;
    }
    if (yk) {
        const float R = rho * iR, iR2 = ir, iR3 = iR2 * iR, iR4 = iR2 * iR2, iR5 = iR4 * iR, iR6 = iR4 * iR2;
        const float e = YUKAWA_COUPLING * __expf(-mu * R);
        const float m2 = mu * mu, m3 = m2 * mu, m4 = m2 * m2;
        const float g0 = e * (iR3 + mu * iR2);
        const float g1 = -e * (3.f * iR4 + 3.f * mu * iR3 + m2 * iR2);
        const float g2 = e * (12.f * iR4 * iR + 12.f * mu * iR4 + 5.f * m2 * iR3 + m3 * iR2);
        const float g3 = -e * (60.f * iR6 + 60.f * mu * iR5 + 27.f * m2 * iR4 + 7.f * m3 * iR3 + m4 * iR2);
        // d/drho = (1 / 2R) d/dR
        p.f0 += g0;
        p.f1 += g1 * 0.5f * iR;
        p.f2 += (g2 * R - g1) * 0.25f * iR3;
        p.f3 += (g3 * R * R - 3.f * g2 * R + 3.f * g1) * 0.125f * iR5;
    }
    return p;
}

// Linear expansion (value V, Jacobian J with respect to the target position)
// of one field; J row-major (dVx/dx, dVx/dy, dVy/dx, dVy/dy).
struct Lin { float v[2]; float j[4]; };

// Second-order term at d = COM - x: mass quadrupole I = (Ixx, Ixy, Iyy)
// about the COM through phi, Q(d) = 2 (I d) phi' + d tr(I) phi' + 2 d (d.I.d) phi'',
// and its Jacobian in x (= -d/dd).
__device__ __forceinline__ void quad_term(const Phi& p, float dx, float dy, float ixx, float ixy, float iyy, Lin& L) {
    const float Idx = ixx * dx + ixy * dy, Idy = ixy * dx + iyy * dy;
    const float tr = ixx + iyy, dId = dx * Idx + dy * Idy;
    L.v[0] = 2.f * Idx * p.f1 + dx * (tr * p.f1 + 2.f * dId * p.f2);
    L.v[1] = 2.f * Idy * p.f1 + dy * (tr * p.f1 + 2.f * dId * p.f2);
    const float diag = tr * p.f1 + 2.f * dId * p.f2;
    const float c4 = 4.f * p.f2, cdd = 2.f * tr * p.f2 + 4.f * dId * p.f3;
    const float d[2] = { dx, dy }, Id[2] = { Idx, Idy };
    const float I[2][2] = { { ixx, ixy }, { ixy, iyy } };
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const float dd = 2.f * p.f1 * I[i][k] + (i == k ? diag : 0.f) + c4 * (Id[i] * d[k] + d[i] * Id[k]) + cdd * d[i] * d[k];
            L.j[2 * i + k] = -dd;
        }
}

// Charge dipole D about the COM through the Coulomb field E(r) = -r psi(rho),
// psi = rho^-3/2: P(d) = -(D psi + 2 d (d.D) psi'), and its Jacobian in x.
__device__ __forceinline__ void dipole_term(float rho, float dx, float dy, float Dx, float Dy, Lin& L) {
    const float ir = 1.f / rho;
    const float p0 = ir * rsqrtf(rho), p1 = -1.5f * p0 * ir, p2 = 3.75f * p0 * ir * ir;
    const float dD = dx * Dx + dy * Dy;
    L.v[0] = -(Dx * p0 + 2.f * dx * dD * p1);
    L.v[1] = -(Dy * p0 + 2.f * dy * dD * p1);
    const float d[2] = { dx, dy }, D[2] = { Dx, Dy };
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const float dd = -(2.f * D[i] * d[k] * p1 + (i == k ? 2.f * dD * p1 : 0.f) + 2.f * d[i] * D[k] * p1 + 4.f * d[i] * d[k] * dD * p2);
            L.j[2 * i + k] = -dd;
        }
}

// Centre of the cell box of a node from the first key under it and its level
// (keys interleave x in the even and y in the odd bits, level 1 first).
__device__ __forceinline__ uint32_t key_compact(uint64_t k) {
    k &= 0x5555555555555555ull;
    k = (k | (k >> 1)) & 0x3333333333333333ull;
    k = (k | (k >> 2)) & 0x0F0F0F0F0F0F0F0Full;
    k = (k | (k >> 4)) & 0x00FF00FF00FF00FFull;
    k = (k | (k >> 8)) & 0x0000FFFF0000FFFFull;
    k = (k | (k >> 16)) & 0x00000000FFFFFFFFull;
    return (uint32_t)k;
}
__device__ __forceinline__ void cell_centre(const DevParams& P, uint64_t key, int level, float& cx, float& cy) {
    const int sh = KEY_LEVELS - level;
    const uint32_t qx = sh >= 32 ? 0u : key_compact(key) >> sh, qy = sh >= 32 ? 0u : key_compact(key >> 1) >> sh;
    const double w = ldexp(2.0 * P.rootW, -level), hgt = ldexp(2.0 * P.rootH, -level);
    cx = (float)(P.rootX - P.rootW + ((double)qx + 0.5) * w);
    cy = (float)(P.rootY - P.rootH + ((double)qy + 0.5) * hgt);
}

// Everything the correction needs of one (cell, group) record.
struct RecGeo {
    float dx, dy;        // d = COM - g
    float ux, uy;        // d / |d| (1, 0 at d = 0)
    float re2;           // |d|^2 + eps^2
    float s;             // cell size (2 bw)
    float M, Q;
    float ixx, ixy, iyy, Dx, Dy;
    bool yg;             // Yukawa present at the group centre's distance
};

// Geometry of node `node` seen from the group centre (gx, gy) and its 14
// features:
//   0 eps/re, 1 s/re, 2 min(mu re / 6, 2), 3 clamp((|d| - r_Y) / s, -8, 8),
//   4 [|d| < r_Y], 5-6 (cell centre - COM) / s in the frame (u, u_perp),
//   7-8 cos 4phi, sin 4phi of u, 9 area fraction of the cell box within r_Y of
//   g (half-plane model), 10 that fraction minus feature 4, 11-13 the mass
//   quadrupole in the frame (u, u_perp) over M s^2.
// re = sqrt(|d|^2 + eps^2); r_Y = 6 / mu (forces.js:82-83), or 1e30 with
// Yukawa off.
__device__ __forceinline__ void record_geo(const DevParams& P, const TreeBufs& T, int node, float gx, float gy,
                                           RecGeo& R, float* f) {
    const float4 a = T.int_a[node], c = T.int_c[node];
    const float4 m1 = T.int_m1[node], m2 = T.int_m2[node];
    const int4 meta = T.int_meta[node];
    R.dx = __fadd_rn(__fsub_rn(a.x, gx), c.x);
    R.dy = __fadd_rn(__fsub_rn(a.y, gy), c.y);
    const float r2 = R.dx * R.dx + R.dy * R.dy;
    const float r = sqrtf(r2);
    R.re2 = r2 + P.softSq;
    const float re = sqrtf(R.re2);
    R.ux = r > 0.f ? R.dx / r : 1.f;
    R.uy = r > 0.f ? R.dy / r : 0.f;
    R.s = sqrtf(c.z);
    R.M = a.z; R.Q = a.w;
    R.ixx = m1.x; R.ixy = m1.y; R.iyy = m1.z; R.Dx = m2.x; R.Dy = m2.y;
    const float cut = P.yukOn ? sqrtf(P.yukCutSq) : 1e30f;
    R.yg = P.yukOn && r2 < P.yukCutSq;
    const float ux = R.ux, uy = R.uy, s = R.s;
    const float is = s > 0.f ? 1.f / s : 0.f;
    f[0] = P.soft / re;
    f[1] = s / re;
    f[2] = P.yukOn ? fminf(P.yukMu * re * (1.f / 6.f), 2.f) : 2.f;
    f[3] = fminf(fmaxf((r - cut) * is, -8.f), 8.f);
    f[4] = R.yg ? 1.f : 0.f;
    float ccx, ccy;
    cell_centre(P, T.skey[meta.y], meta.x, ccx, ccy);
    const float ox = __fadd_rn(__fsub_rn(ccx, a.x), -c.x), oy = __fadd_rn(__fsub_rn(ccy, a.y), -c.y);
    f[5] = (ox * ux + oy * uy) * is;
    f[6] = (-ox * uy + oy * ux) * is;
    const float c2 = ux * ux - uy * uy, s2 = 2.f * ux * uy;
    f[7] = c2 * c2 - s2 * s2;
    f[8] = 2.f * s2 * c2;
    {
        const float vx = ccx - gx, vy = ccy - gy, rc = sqrtf(vx * vx + vy * vy);
        const float nx = rc > 0.f ? vx / rc : 1.f, ny = rc > 0.f ? vy / rc : 0.f;
        float aa = 0.5f * s * fabsf(nx), bb = 0.5f * s * fabsf(ny);
        if (aa < bb) { const float t = aa; aa = bb; bb = t; }
        const float t = cut - rc, at = fabsf(t);
        float fr;
        if (at >= aa + bb) fr = t > 0.f ? 1.f : 0.f;
        else {
            const float cdf = (bb < 1e-6f * s || at <= aa - bb) ? 0.5f + at / (2.f * aa)
                                                               : 1.f - (aa + bb - at) * (aa + bb - at) / (8.f * aa * bb);
            fr = t >= 0.f ? cdf : 1.f - cdf;
        }
        f[9] = fr;
        f[10] = fr - f[4];
    }
    const float iMs = (R.M > 0.f && s > 0.f) ? 1.f / (R.M * s * s) : 0.f;
    f[11] = (ux * ux * R.ixx + 2.f * ux * uy * R.ixy + uy * uy * R.iyy) * iMs;
    f[12] = ((R.iyy - R.ixx) * ux * uy + R.ixy * (ux * ux - uy * uy)) * iMs;
    f[13] = (uy * uy * R.ixx - 2.f * ux * uy * R.ixy + ux * ux * R.iyy) * iMs;
}

// A group whose targets lie farther than this fraction of |d| (or, within
// the Yukawa range, of 1/mu) from its centre is "wide" for the record: no
// linear expansion over it is accurate (the sparse background's groups span
// tens of units), so the record takes the analytic term exactly at each
// target, with each target's own Yukawa decision, and no network.
constexpr float EXPAND_MAX = 0.1f;
enum { REC_EXACT = 1u, REC_NEAR_CUT = 2u, REC_NET = 4u };

// How the correction treats a record of a group of radius bound `grad`:
//   REC_EXACT     wide group: the analytic term per target, no network;
//   REC_NEAR_CUT  targets may decide the Yukawa range unlike the centre
//                 (|d| - grad <= r_Y <= |d| + grad): the monopole's Yukawa
//                 term is swapped to the group's decision;
//   REC_NET       the Yukawa cutoff can separate a member of the cell from a
//                 target (| |d| - r_Y | <= s sqrt 2 + grad: members lie
//                 within s sqrt 2 of the COM): the network applies.  Away
//                 from the cutoff the analytic expansion is accurate and the
//                 network would only add its output noise.
__device__ __forceinline__ uint32_t record_flags(const DevParams& P, const RecGeo& R, float grad) {
    const float dn = sqrtf(R.dx * R.dx + R.dy * R.dy);
    uint32_t f = 0;
    // the Yukawa factor e^{-mu r} changes over 1/mu: within its range the
    // group must also be small against that
    if (grad > EXPAND_MAX * dn || (R.yg && grad * P.yukMu > EXPAND_MAX)) f |= REC_EXACT;
    if (P.yukOn) {
        const float cut = sqrtf(P.yukCutSq);
        if ((dn - grad) <= cut * (1.f + 1e-5f) && (dn + grad) >= cut * (1.f - 1e-5f)) f |= REC_NEAR_CUT;
        if (!(f & REC_EXACT) && fabsf(dn - cut) <= 1.4143f * R.s + grad) f |= REC_NET;
    }
    return f;
}

// The analytic second-order term's fields at displacement (dx, dy) = COM - x
// (values only): mass quadrupole through the mass kernel with the group's
// Yukawa decision, charge dipole through the Coulomb kernel.
__device__ __forceinline__ void analytic_at(const DevParams& P, const RecGeo& R, float dx, float dy, float& gx, float& gy,
                                            float& ex, float& ey) {
    const float rho = dx * dx + dy * dy + P.softSq;
    const Phi ph = mass_kernel(rho, (P.toggles & GEON_GRAVITY) != 0, R.yg, P.yukMu);
    const float Idx = R.ixx * dx + R.ixy * dy, Idy = R.ixy * dx + R.iyy * dy;
    const float tr = R.ixx + R.iyy, dId = dx * Idx + dy * Idy;
    const float c = tr * ph.f1 + 2.f * dId * ph.f2;
    gx = 2.f * Idx * ph.f1 + dx * c;
    gy = 2.f * Idy * ph.f1 + dy * c;
    if (P.toggles & GEON_COULOMB) {
        const float ir = 1.f / rho;
        const float p0 = ir * rsqrtf(rho), p1 = -1.5f * p0 * ir;
        const float dD = dx * R.Dx + dy * R.Dy;
        ex = -(R.Dx * p0 + 2.f * dx * dD * p1);
        ey = -(R.Dy * p0 + 2.f * dy * dD * p1);
    } else {
        ex = ey = 0.f;
    }
}

// Scales of the network outputs: value s0 = M / re^2, gradient s0 / s.
__device__ __forceinline__ void out_scales(const RecGeo& R, float& s0, float& s1) {
    s0 = R.M / R.re2;
    s1 = R.s > 0.f ? s0 / R.s : 0.f;
}

// Adds the network residual y[6] to the mass-field expansion about g.
__device__ __forceinline__ void add_net_expansion(const RecGeo& R, const float* y, Lin& Gm) {
    float s0, s1;
    out_scales(R, s0, s1);
    const float ux = R.ux, uy = R.uy;
    // value s0 (y0 u + y3 u_perp); gradient s1 [(y1 u + y4 u_perp) u^T + (y2 u + y5 u_perp) u_perp^T]
    Gm.v[0] += s0 * (y[0] * ux - y[3] * uy);
    Gm.v[1] += s0 * (y[0] * uy + y[3] * ux);
    const float ax = y[1] * ux - y[4] * uy, ay = y[1] * uy + y[4] * ux;   // column along u
    const float bx = y[2] * ux - y[5] * uy, by = y[2] * uy + y[5] * ux;   // column along u_perp
    Gm.j[0] += s1 * (ax * ux - bx * uy);
    Gm.j[1] += s1 * (ax * uy + bx * ux);
    Gm.j[2] += s1 * (ay * ux - by * uy);
    Gm.j[3] += s1 * (ay * uy + by * ux);
}

// The record's mass- and charge-field expansions about g: the analytic
// second-order term (unless `exact`: then it is added per target) plus
// (y != null) the network residual y[6].
__device__ __forceinline__ void record_expansion(const DevParams& P, const RecGeo& R, const float* y, bool exact,
                                                 Lin& Gm, Lin& Ec) {
    const bool grav = (P.toggles & GEON_GRAVITY) != 0;
    if (exact) {
        Gm = Lin{ { 0.f, 0.f }, { 0.f, 0.f, 0.f, 0.f } };
        Ec = Lin{ { 0.f, 0.f }, { 0.f, 0.f, 0.f, 0.f } };
    } else {
        const Phi ph = mass_kernel(R.re2, grav, R.yg, P.yukMu);
        quad_term(ph, R.dx, R.dy, R.ixx, R.ixy, R.iyy, Gm);
        if (P.toggles & GEON_COULOMB) dipole_term(R.re2, R.dx, R.dy, R.Dx, R.Dy, Ec);
        else { Ec.v[0] = Ec.v[1] = 0.f; Ec.j[0] = Ec.j[1] = Ec.j[2] = Ec.j[3] = 0.f; }
    }
    if (y) add_net_expansion(R, y, Gm);
}

// learn.cu
// Training records of the learned correction for the groups g = 0, stride,
// 2 stride, ... of the last walk's records (recs, rec_cnt, rec_cap): for each
// record the 14 features, the least-squares expansion y*[6] of the exact
// residual of its accepting targets (the member sum of src/forces.js:94-125
// restricted to the cell, minus the monopole with the group's Yukawa
// decision, minus the analytic term), and the quadratic form A[12] with which
// an output error enters the sum over those targets of the squared force
// error relative to |F| (weights m^2 / max(|F|^2, (m gfloor)^2), |F| from
// S.force).  `off` holds the exclusive prefix of the selected groups'
// counts, written by learn_record_offsets.
void learn_record_offsets(const int* rec_cnt, int rec_cap, int ngroups, int stride, int* off, int* total,
                          void* scan_tmp, cudaStream_t st, LaunchCounter& lc);
void learn_records(const DevParams& P, const DevState& S, const TreeBufs& T, const uint2* recs, const int* rec_cnt,
                   const float4* gcen, int rec_cap, int ngroups, int stride, const int* off, int cap, float gfloor,
                   float* feat, float* target, int* rec_group, const FrameCtl* ctl, cudaStream_t st, LaunchCounter& lc);
size_t learn_offsets_scratch_bytes(int ngroups);

}  // namespace geon
