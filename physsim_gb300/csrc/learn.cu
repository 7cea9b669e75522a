// learn.cu — training records of the learned far-field correction.
//
// The walk with record emission (force.cu, walkc_kernel EMIT) leaves, for
// each group of 32 consecutive targets in walk order, the cells some of its
// targets accepted as one aggregate (src/forces.js:680-685) with the mask of
// those targets.  For a record, learn_records_kernel evaluates at every
// accepting target the exact field of the cell's member particles (the
// pairwise sum of src/forces.js:94-125 restricted to the cell: gravity and
// Yukawa per unit target mass with the per-pair cutoff of forces.js:387,
// Coulomb per unit target charge), subtracts what the correction already has
// without the network (the monopole with the group's Yukawa decision and the
// analytic expansion of learn.cuh), and fits the mass-field residual with the
// network's output form by weighted least squares.
#include "learn.cuh"

namespace geon {

constexpr int LR_THREADS = 128;
constexpr int LR_WARPS = LR_THREADS / 32;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Mass-sourced (gravity + Yukawa) field of a unit-mass-weighted source at
// displacement (rx, ry), with the Yukawa cutoff decided by `yk`.
__device__ __forceinline__ void mass_field(const DevParams& P, float rx, float ry, bool yk, float& gx, float& gy) {
    const float rSq = __fmaf_rn(rx, rx, ry * ry) + P.softSq;
    const float invR = rsqrtf(rSq);
    const float invR3 = invR * invR * invR;
    float f = (P.toggles & GEON_GRAVITY) ? invR3 : 0.f;
    if (yk) {
        const float r = rSq * invR;
        f += YUKAWA_COUPLING * __expf(-P.yukMu * r) * (invR * invR + P.yukMu * invR) * invR;
    }
    gx = rx * f;
    gy = ry * f;
}

__global__ void sel_counts_kernel(const int* __restrict__ rec_cnt, int rec_cap, int nsel, int stride, int* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nsel; i += gridDim.x * blockDim.x)
        out[i] = min(rec_cnt[(size_t)i * stride], rec_cap);
}

__global__ void __launch_bounds__(LR_THREADS)
learn_records_kernel(DevParams P, DevState S, TreeBufs T, const FrameCtl* __restrict__ ctl, const uint2* __restrict__ recs,
                     const int* __restrict__ rec_cnt, const float4* __restrict__ gcen, int rec_cap, int nsel, int stride,
                     const int* __restrict__ off,
                     int cap, float gfloor, float* __restrict__ feat, float* __restrict__ target, int* __restrict__ rec_group) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = ctl->n;
    for (int gi = blockIdx.x; gi < nsel; gi += gridDim.x) {
        const int grp = gi * stride;
        const int kk = grp * 32 + lane;
        int ti = kk < n ? T.tgt[kk] : -1;
        if (ti >= n) ti = -1;
        const float4 gc = gcen[grp];
        const float gx = gc.x, gy = gc.y;
        float tx = 0.f, ty = 0.f, txl = 0.f, tyl = 0.f, w = 0.f;
        if (ti >= 0) {
            const float4 p = S.pos[ti];
            const float2 pl = S.pos_lo[ti];
            const float4 F = S.force[ti];
            tx = p.x; ty = p.y; txl = pl.x; tyl = pl.y;
            const float m2 = p.z * p.z, f2 = F.x * F.x + F.y * F.y;
            w = m2 / fmaxf(fmaxf(f2, m2 * gfloor * gfloor), 1e-30f);
        }
        // offset of this target from the group centre
        const float ox = __fadd_rn(__fsub_rn(tx, gx), txl), oy = __fadd_rn(__fsub_rn(ty, gy), tyl);
        const int cnt = min(rec_cnt[grp], rec_cap);
        const int base = off[gi];
        for (int r = warp; r < cnt; r += LR_WARPS) {
            const int e = base + r;
            if (e >= cap) break;
            const uint2 rc = recs[(size_t)grp * rec_cap + r];
            const int node = (int)rc.x;
            const bool mine = ti >= 0 && ((rc.y >> lane) & 1u);
            RecGeo R;
            float f[LF];
            record_geo(P, T, node, gx, gy, R, f);
            const uint32_t rflags = record_flags(P, R, gc.z);
            const bool exact = (rflags & REC_EXACT) != 0;
            Lin Gm, Ec;
            record_expansion(P, R, nullptr, exact, Gm, Ec);
            if (!(rflags & REC_NET)) {
                // no member sums for a record the network does not see (lane 0 still writes it, without weight)
                if (lane == 0) {
                    float* o = target + (size_t)e * LT;
#pragma unroll
                    for (int c = 0; c < LT; c++) o[c] = 0.f;
                    float* fo = feat + (size_t)e * LF;
#pragma unroll
                    for (int c = 0; c < LF; c++) fo[c] = f[c];
                    if (rec_group) rec_group[e] = grp;
                }
                continue;
            }
            // exact member sum at this target (two-sum compensated)
            const int4 meta = T.int_meta[node];
            float sx = 0.f, sxl = 0.f, sy = 0.f, syl = 0.f;
            for (int q = meta.y; q < meta.z; q++) {
                const float4 pa = T.ps_a[q];
                const float4 pb = T.ps_b[q];
                const int j = (int)ref_index(__float_as_uint(reinterpret_cast<const float*>(T.ps_c + q)[3]));
                if (!mine || j == ti) continue;
                float rx, ry;
                displacement(P, tx, ty, pa.x, pb.x - txl, pa.y, pb.y - tyl, rx, ry);
                float gxv, gyv;
                mass_field(P, rx, ry, P.yukOn && __fmaf_rn(rx, rx, ry * ry) < P.yukCutSq, gxv, gyv);
                const df a1 = two_sum(sx, pa.z * gxv); sx = a1.hi; sxl += a1.lo;
                const df a2 = two_sum(sy, pa.z * gyv); sy = a2.hi; syl += a2.lo;
            }
            float resx = 0.f, resy = 0.f;
            if (mine) {
                // monopole with the group's Yukawa decision and the analytic expansion at this target
                const float dx = R.dx - ox, dy = R.dy - oy;
                float mgx, mgy;
                mass_field(P, dx, dy, R.yg, mgx, mgy);
                const float ax = Gm.v[0] + Gm.j[0] * ox + Gm.j[1] * oy, ay = Gm.v[1] + Gm.j[2] * ox + Gm.j[3] * oy;
                resx = (sx + sxl) - R.M * mgx - ax;
                resy = (sy + syl) - R.M * mgy - ay;
            }
            // weighted least squares in the frame (u, u_perp), basis (s0, s1 e_u, s1 e_v)
            float s0, s1;
            out_scales(R, s0, s1);
            const float eu = ox * R.ux + oy * R.uy, ev = -ox * R.uy + oy * R.ux;
            const float b0 = s0, b1 = s1 * eu, b2 = s1 * ev;
            const float wm = mine ? w : 0.f;
            const float rp = resx * R.ux + resy * R.uy, rq = -resx * R.uy + resy * R.ux;
            const float A00 = warp_sum(wm * b0 * b0), A11 = warp_sum(wm * b1 * b1), A22 = warp_sum(wm * b2 * b2);
            const float A01 = warp_sum(wm * b0 * b1), A02 = warp_sum(wm * b0 * b2), A12 = warp_sum(wm * b1 * b2);
            const float p0 = warp_sum(wm * b0 * rp), p1 = warp_sum(wm * b1 * rp), p2 = warp_sum(wm * b2 * rp);
            const float q0 = warp_sum(wm * b0 * rq), q1 = warp_sum(wm * b1 * rq), q2 = warp_sum(wm * b2 * rq);
            if (lane == 0) {
                // (A + ridge) y = b by Cramer's rule in FP64 (3 x 3)
                const double tr = (double)A00 + A11 + A22, rg = 1e-6 * tr + 1e-30;
                const double m00 = A00 + rg, m11 = A11 + rg, m22 = A22 + rg, m01 = A01, m02 = A02, m12 = A12;
                const double det = m00 * (m11 * m22 - m12 * m12) - m01 * (m01 * m22 - m12 * m02) + m02 * (m01 * m12 - m11 * m02);
                double yp[3] = { 0, 0, 0 }, yq[3] = { 0, 0, 0 };
                if (det != 0.0 && isfinite(det)) {
                    const double id = 1.0 / det;
                    const double c00 = m11 * m22 - m12 * m12, c01 = m02 * m12 - m01 * m22, c02 = m01 * m12 - m02 * m11;
                    const double c11 = m00 * m22 - m02 * m02, c12 = m01 * m02 - m00 * m12, c22 = m00 * m11 - m01 * m01;
                    yp[0] = id * (c00 * p0 + c01 * p1 + c02 * p2);
                    yp[1] = id * (c01 * p0 + c11 * p1 + c12 * p2);
                    yp[2] = id * (c02 * p0 + c12 * p1 + c22 * p2);
                    yq[0] = id * (c00 * q0 + c01 * q1 + c02 * q2);
                    yq[1] = id * (c01 * q0 + c11 * q1 + c12 * q2);
                    yq[2] = id * (c02 * q0 + c12 * q1 + c22 * q2);
                }
                float* o = target + (size_t)e * LT;
                o[0] = (float)yp[0]; o[1] = (float)yp[1]; o[2] = (float)yp[2];
                o[3] = (float)yq[0]; o[4] = (float)yq[1]; o[5] = (float)yq[2];
                // the same quadratic form for both components (the weights do not depend on the component)
                const float Aq[6] = { A00, A11, A22, A01, A02, A12 };
#pragma unroll
                for (int c = 0; c < 6; c++) { o[LO + c] = Aq[c]; o[LO + 6 + c] = Aq[c]; }
                float* fo = feat + (size_t)e * LF;
#pragma unroll
                for (int c = 0; c < LF; c++) fo[c] = f[c];
                if (rec_group) rec_group[e] = grp;
            }
        }
    }
}

size_t learn_offsets_scratch_bytes(int ngroups) {
    return (size_t)(ngroups + 1) * sizeof(int) + scan_temp_ints(std::max(ngroups, 1)) * sizeof(int) + 256;
}

void learn_record_offsets(const int* rec_cnt, int rec_cap, int ngroups, int stride, int* off, int* total,
                          void* scan_tmp, cudaStream_t st, LaunchCounter& lc) {
    const int nsel = (ngroups + stride - 1) / stride;
    int* sel = static_cast<int*>(scan_tmp);
    int* tmp = reinterpret_cast<int*>(reinterpret_cast<char*>(scan_tmp) + (((size_t)(nsel + 1) * sizeof(int) + 255) & ~(size_t)255));
    sel_counts_kernel<<<std::max(1, std::min((nsel + 255) / 256, 1024)), 256, 0, st>>>(rec_cnt, rec_cap, nsel, stride, sel);
    lc.add(1);
    exclusive_scan(sel, off, nsel, nullptr, total, tmp, st, &lc);
}

void learn_records(const DevParams& P, const DevState& S, const TreeBufs& T, const uint2* recs, const int* rec_cnt,
                   const float4* gcen, int rec_cap, int ngroups, int stride, const int* off, int cap, float gfloor,
                   float* feat, float* target, int* rec_group, const FrameCtl* ctl, cudaStream_t st, LaunchCounter& lc) {
    const int nsel = (ngroups + stride - 1) / stride;
    if (nsel <= 0) return;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = std::max(1, std::min(nsel, std::max(sms, 1) * 8));
    learn_records_kernel<<<blocks, LR_THREADS, 0, st>>>(P, S, T, ctl, recs, rec_cnt, gcen, rec_cap, nsel, stride, off, cap,
                                                        gfloor, feat, target, rec_group);
    lc.add(1);
}

}  // namespace geon
