// tree_dev.cuh — device code of the quadtree build (tree.cu): the helpers
// and every phase's body.  A body takes the virtual block index and block
// count of a grid-stride loop, so the kernels of tree.cu (one launch per
// phase) and the persistent frame kernel (force.cu, all phases in one launch)
// run the same code.
#pragma once

#include "state.cuh"

namespace geon {


// Common-prefix length in levels of two valid keys: the Morton code sits
// below `top` bits (the invalid flag, and in batched handles the system id);
// keys that differ above it share no node (-1).
__device__ __forceinline__ int lcp_level(uint64_t a, uint64_t b, int top, int levels) {
    uint64_t x = a ^ b;
    if (x == 0) return levels;
    int lz = __clzll((long long)x);
    if (lz < top) return -1;
    return (lz - top) >> 1;
}
__device__ __forceinline__ int lcp_level(const DevParams& P, uint64_t a, uint64_t b) {
    return lcp_level(a, b, P.keyTop, P.keyLevels);
}

__device__ __forceinline__ uint32_t key_digit(uint64_t k, int level, int levels) {   // level 1..levels
    return (uint32_t)(k >> (2 * (levels - level))) & 3u;
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ void tree_reset_body(FrameCtl* ctl, int vb, int nvb) {
    ctl->nValid = 0;
    ctl->nInternal = 0;
    ctl->nLeaves = 0;
    ctl->nBucket = 0;
    ctl->maxLevel = 0;
}

// Ghost counts per particle (integrator.js:201-244): margin = max(W,H)*theta.
__device__ __forceinline__ void ghost_flags(const DevParams& P, const DevState& S, int i, bool& L, bool& R, bool& T, bool& B) {
    const float4 p = S.pos[i];
    const float2 pl = S.pos_lo[i];
    const double x = (double)p.x + (double)pl.x, y = (double)p.y + (double)pl.y;
    const double margin = fmax(P.Wd, P.Hd) * P.thetaD;
    L = x < margin; R = x > P.Wd - margin;
    T = y < margin; B = y > P.Hd - margin;
}

__device__ __forceinline__ void ghost_count_body(DevParams P, DevState S, TreeBufs T, const FrameCtl* ctl, int vb, int nvb) {
    const int n = ctl->n;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        int c = 0;
        if (P.ghosts) {
            bool L, R, Tp, B;
            ghost_flags(P, S, i, L, R, Tp, B);
            c = (int)L + (int)R + (int)Tp + (int)B + (int)(L && Tp) + (int)(L && B) + (int)(R && Tp) + (int)(R && B);
        }
        T.ghost_cnt[i] = c;
    }
}

__device__ __forceinline__ uint32_t gcode(int sx, int sy, bool mx, bool my, bool fvx, bool fvy) {
    return (uint32_t)(sx + 1) | ((uint32_t)(sy + 1) << 2) | ((uint32_t)mx << 4) | ((uint32_t)my << 5) |
           ((uint32_t)fvx << 6) | ((uint32_t)fvy << 7);
}

__device__ __forceinline__ void point_refs_body(DevParams P, DevState S, TreeBufs T, FrameCtl* ctl, int vb, int nvb) {
    const int n = ctl->n;
    if (vb == 0 && threadIdx.x == 0) ctl->nPts = n + ctl->nGhost;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) {
        T.pt_ref[i] = make_ref(i, CODE_IDENTITY);
        if (!P.ghosts || T.ghost_cnt[i] == 0) continue;
        bool L, R, Tp, B;
        ghost_flags(P, S, i, L, R, Tp, B);
        uint32_t* out = T.pt_ref + n + T.ghost_off[i];
        int k = 0;
        const uint32_t ui = (uint32_t)i;
        if (P.topology == GEON_TORUS) {                       // integrator.js:213-221
            if (L) out[k++] = make_ref(ui, gcode(1, 0, false, false, false, false));
            if (R) out[k++] = make_ref(ui, gcode(-1, 0, false, false, false, false));
            if (Tp) out[k++] = make_ref(ui, gcode(0, 1, false, false, false, false));
            if (B) out[k++] = make_ref(ui, gcode(0, -1, false, false, false, false));
            if (L && Tp) out[k++] = make_ref(ui, gcode(1, 1, false, false, false, false));
            if (L && B) out[k++] = make_ref(ui, gcode(1, -1, false, false, false, false));
            if (R && Tp) out[k++] = make_ref(ui, gcode(-1, 1, false, false, false, false));
            if (R && B) out[k++] = make_ref(ui, gcode(-1, -1, false, false, false, false));
        } else {
            const bool klein = P.topology == GEON_KLEIN;     // integrator.js:222-241
            if (L) out[k++] = make_ref(ui, klein ? gcode(1, 0, false, false, false, false) : gcode(1, 0, false, true, false, true));
            if (R) out[k++] = make_ref(ui, klein ? gcode(-1, 0, false, false, false, false) : gcode(-1, 0, false, true, false, true));
            if (Tp) out[k++] = make_ref(ui, gcode(0, 1, true, false, true, false));
            if (B) out[k++] = make_ref(ui, gcode(0, -1, true, false, true, false));
            if (L && Tp) out[k++] = make_ref(ui, gcode(1, 1, true, false, true, false));
            if (L && B) out[k++] = make_ref(ui, gcode(1, -1, true, false, true, false));
            if (R && Tp) out[k++] = make_ref(ui, gcode(-1, 1, true, false, true, false));
            if (R && B) out[k++] = make_ref(ui, gcode(-1, -1, true, false, true, false));
        }
    }
}

// Quantise one coordinate to the 31-level grid (exact path).  Returns the
// number of grid boundaries lo + j*delta (j = 1 .. 2^31-1) strictly below v,
// which equals the sequence of "v > centre" decisions of the descent.
__device__ __forceinline__ uint32_t quantise_exact(double v, double lo, double delta, double inv_delta) {
    const double qmax = 2147483647.0;
    double u = (v - lo) * inv_delta;
    double q = ceil(u) - 1.0;
    q = fmin(fmax(q, 0.0), qmax);
    // fix-up against the exact boundaries (fma rounds once; boundaries are representable)
    for (int it = 0; it < 3; it++) {
        if (q >= 1.0 && !(fma(q, delta, lo) < v)) { q -= 1.0; continue; }
        if (q < qmax && fma(q + 1.0, delta, lo) < v) { q += 1.0; continue; }
        break;
    }
    return (uint32_t)q;
}

// Morton key of point p (reference ref) in the root box; points outside it
// get KEY_INVALID | p (quadtree.js:106-179).  Returns whether the point is inside.
__device__ __forceinline__ bool point_key(const DevParams& P, const DevState& S, uint32_t ref, int p, uint64_t& key) {
    const double loX = P.rootX - P.rootW, hiX = P.rootX + P.rootW;   // quadtree.js:106-109
    const double loY = P.rootY - P.rootH, hiY = P.rootY + P.rootH;
    const double dX = P.rootW * (1.0 / 1073741824.0), dY = P.rootH * (1.0 / 1073741824.0);   // bw / 2^30
    const double iX = 1.0 / dX, iY = 1.0 / dY;
    const float4 s = S.pos[ref_index(ref)];
    const float2 sl = S.pos_lo[ref_index(ref)];
    double x, y;
    image_pos_d((double)s.x + (double)sl.x, (double)s.y + (double)sl.y, ref_code(ref), P.Wd, P.Hd, x, y);
    if (!(x >= loX && x <= hiX && y >= loY && y <= hiY)) {
        key = KEY_INVALID | (uint64_t)p;
        return false;
    } else {
        uint32_t qx, qy;
        if (P.exact_grid) {
            qx = quantise_exact(x, loX, dX, iX);
            qy = quantise_exact(y, loY, dY, iY);
        } else {
            // the reference's centre recurrence (quadtree.js:119-179)
            double cx = P.rootX, cy = P.rootY, hw = P.rootW, hh = P.rootH;
            qx = 0; qy = 0;
            for (int l = 0; l < KEY_LEVELS; l++) {
                const uint32_t r = x > cx, d = y > cy;
                hw = hw / 2; hh = hh / 2;
                cx = r ? cx + hw : cx - hw;
                cy = d ? cy + hh : cy - hh;
                qx = (qx << 1) | r; qy = (qy << 1) | d;
            }
        }
        uint64_t k = 0;
        for (int b = 0; b < KEY_LEVELS; b++) {
            k |= (uint64_t)((qx >> b) & 1u) << (2 * b);
            k |= (uint64_t)((qy >> b) & 1u) << (2 * b + 1);
        }
        if (P.nsys) {      // batched: the first 27 routing levels below the system id
            k = ((uint64_t)S.sys[ref_index(ref)] << (2 * BATCH_KEY_LEVELS)) |
                (k >> (2 * (KEY_LEVELS - BATCH_KEY_LEVELS)));
        }
        key = k;
        return true;
    }
}

__device__ __forceinline__ void key_body(DevParams P, DevState S, TreeBufs T, FrameCtl* ctl, int vb, int nvb) {
    const int nPts = ctl->nPts;
    int valid = 0;
    for (int p = vb * blockDim.x + threadIdx.x; p < nPts; p += nvb * blockDim.x) {
        uint64_t key;
        valid += point_key(P, S, T.pt_ref[p], p, key) ? 1 : 0;
        T.key[p] = key;
        T.idx[p] = (uint32_t)p;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) valid += __shfl_xor_sync(0xffffffffu, valid, o);
    if ((threadIdx.x & 31) == 0 && valid) atomicAdd(&ctl->nValid, valid);
}

// Gather sorted point data and the per-point LCP quantities.
__device__ __forceinline__ void gather_body(DevParams P, DevState S, TreeBufs T, const FrameCtl* ctl, int vb, int nvb) {
    const int nPts = ctl->nPts, nValid = ctl->nValid;
    const uint64_t* K = T.skey;
    for (int s = vb * blockDim.x + threadIdx.x; s < nPts; s += nvb * blockDim.x) {
        const uint32_t p = T.sidx[s];
        const uint32_t ref = T.pt_ref[p];
        const uint32_t j = ref_index(ref), code = ref_code(ref);
        const float4 pos = S.pos[j];
        const float4 vel = S.vel[j];
        const float4 spn = S.spin[j];
        const bool fvx = code_fvx(code), fvy = code_fvy(code);
        const float sgn = (fvx || fvy) ? -1.f : 1.f;
        const float angVel = sgn * spn.y;
        const float2 plo = S.pos_lo[j];
        float ix, ixlo, iy, iylo;
        point_image(P, pos.x, pos.y, plo.x, plo.y, code, ix, ixlo, iy, iylo);
        const float rsq = spn.z * spn.z;
        T.ps_a[s] = make_float4(ix, iy, pos.z, pos.w);
        T.ps_b[s] = make_float4(ixlo, iylo, fvx ? -vel.z : vel.z, fvy ? -vel.w : vel.w);
        T.ps_c[s] = make_float4(angVel, MAG_MOMENT_K * pos.w * angVel * rsq, INERTIA_K * pos.z * angVel * rsq,
                                __uint_as_float(ref));
        T.real_flag[s] = (code == CODE_IDENTITY) ? 1 : 0;
        int a = -1, c = 0, lf = 0;
        if (s < nValid) {
            const uint64_t k = K[s];
            a = (s == 0) ? -1 : lcp_level(P, K[s - 1], k);
            const int b = (s + 4 < nValid) ? lcp_level(P, k, K[s + 4]) : -1;
            c = max(0, min(b, P.keyLevels - 1) - a);
            int m = -1;
            for (int jj = max(0, s - 4); jj <= s && jj + 4 < nValid; jj++) m = max(m, lcp_level(P, K[jj], K[jj + 4]));
            const int L = min(m + 1, P.keyLevels);
            lf = (a < L) ? 1 : 0;
        }
        T.lcp_a[s] = a;
        T.int_cnt[s] = c;
        T.leaf_flag[s] = lf;
    }
}

__device__ __forceinline__ int leaf_level_of(const DevParams& P, const uint64_t* K, int s, int nValid) {
    int m = -1;
    for (int jj = max(0, s - 4); jj <= s && jj + 4 < nValid; jj++) m = max(m, lcp_level(P, K[jj], K[jj + 4]));
    return min(m + 1, P.keyLevels);
}

__device__ __forceinline__ void emit_body(DevParams P, TreeBufs T, FrameCtl* ctl, int vb, int nvb) {
    const int nPts = ctl->nPts, nValid = ctl->nValid;
    const int nInt = ctl->nInternal;
    const bool ok = nInt <= T.cap_int;
    if (!ok && vb == 0 && threadIdx.x == 0) atomicOr(&ctl->err, ERR_NODE_OVERFLOW);
    const uint64_t* K = T.skey;
    int bucket = 0, maxl = 0;
    for (int s = vb * blockDim.x + threadIdx.x; s < nPts; s += nvb * blockDim.x) {
        if (T.real_flag[s]) T.tgt[T.tgt_base[s]] = (int)ref_index(__float_as_uint(T.ps_c[s].w));
        if (s >= nValid) continue;
        const int a = T.lcp_a[s];
        const int c = T.int_cnt[s];
        if (ok && c > 0) {
            const int base = T.int_base[s];
            for (int k = 0; k < c; k++) T.int_meta[base + k] = make_int4(a + 1 + k, s, 0, -1);
        }
        const int L = leaf_level_of(P, K, s, nValid);
        const int lb = T.leaf_base[s];
        if (T.leaf_flag[s]) {
            int cnt = 1;
            while (s + cnt < nValid && lcp_level(P, K[s], K[s + cnt]) >= L) cnt++;
            T.leaf_meta[lb] = make_int4(s, cnt, L, -1);
            if (cnt > LEAF_CAP) bucket++;
            maxl = max(maxl, L);
            T.leaf_of[s] = lb;
        } else {
            T.leaf_of[s] = lb - 1;
        }
    }
    if (bucket) atomicAdd(&ctl->nBucket, bucket);
    if (maxl) atomicMax(&ctl->maxLevel, maxl);
}

// First index in [lo, hi) whose digit at `level` is >= d (digits non-decreasing there).
__device__ __forceinline__ int lower_digit(const uint64_t* K, int lo, int hi, int level, int levels, uint32_t d) {
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (key_digit(K[mid], level, levels) < d) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void link_body(DevParams P, TreeBufs T, FrameCtl* ctl, int* d_root, int vb, int nvb) {
    const int nValid = ctl->nValid;
    const int nInt = min(ctl->nInternal, T.cap_int);
    const int nLeaves = ctl->nLeaves;
    const uint64_t* K = T.skey;
    if (vb == 0 && threadIdx.x == 0) {
        *d_root = (nValid > LEAF_CAP) ? 0 : (nValid > 0 ? (LEAF_REF | 0) : ROOT_NONE);
    }
    for (int node = vb * blockDim.x + threadIdx.x; node < nInt; node += nvb * blockDim.x) {
        const int4 m = T.int_meta[node];
        const int d = m.x, s = m.y;
        // end of the run sharing the level-d prefix with K[s]
        int lo = s + 1, hi = nValid;
        const uint64_t ks = K[s];
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (lcp_level(P, ks, K[mid]) >= d) lo = mid + 1; else hi = mid;
        }
        const int e = lo;
        const int LV = P.keyLevels;
        const int b1 = lower_digit(K, s, e, d + 1, LV, 1u);
        const int b2 = lower_digit(K, b1, e, d + 1, LV, 2u);
        const int b3 = lower_digit(K, b2, e, d + 1, LV, 3u);
        const int bounds[5] = { s, b1, b2, b3, e };
        int ch[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int cs = bounds[q], ce = bounds[q + 1];
            if (ce <= cs) { ch[q] = -1; continue; }
            if (ce - cs > LEAF_CAP && d + 1 <= LV - 1) {
                const int ci = T.int_base[cs] + (d + 1 - T.lcp_a[cs] - 1);
                if (ci <= node || ci >= nInt) { atomicOr(&ctl->err, ERR_BAD_INDEX); ch[q] = -1; continue; }
                ch[q] = ci;
                T.int_meta[ci].w = node;
            } else {
                const int li = T.leaf_base[cs];
                if (li < 0 || li >= nLeaves) { atomicOr(&ctl->err, ERR_BAD_INDEX); ch[q] = -1; continue; }
                ch[q] = LEAF_REF | li;
                T.leaf_meta[li].w = node;
            }
        }
        T.int_child[node] = make_int4(ch[0], ch[1], ch[2], ch[3]);
        T.int_meta[node].z = e;
        T.int_count[node] = 0;
    }
}

// Batched handles: the root of every system.  The first sorted point of a
// system shares no prefix with its predecessor (lcp -1), so the first node
// it starts is the system's level-0 node; a system of at most 4 points is a
// single leaf.  Systems without points keep ROOT_NONE.
__device__ __forceinline__ void batch_roots_body(DevParams P, TreeBufs T, const FrameCtl* ctl, int vb, int nvb) {
    const int nValid = ctl->nValid;
    const int nInt = min(ctl->nInternal, T.cap_int), nLeaves = ctl->nLeaves;
    for (int s = vb * blockDim.x + threadIdx.x; s < nValid; s += nvb * blockDim.x) {
        if (T.lcp_a[s] != -1) continue;
        const int sys = (int)(T.skey[s] >> (2 * BATCH_KEY_LEVELS));
        if (sys < 0 || sys >= P.nsys) continue;
        int root = ROOT_NONE;
        if (T.int_cnt[s] > 0) {
            const int ni = T.int_base[s];
            if (ni >= 0 && ni < nInt) root = ni;
        } else {
            const int li = T.leaf_base[s];
            if (li >= 0 && li < nLeaves) root = LEAF_REF | li;
        }
        T.roots[sys] = root;
    }
}

// ---- bottom-up aggregation ---------------------------------------------------------
// Aggregate accumulator.  Sums are compensated FP32 pairs; the centre of
// mass is accumulated as mass-weighted offsets from a local origin (the first
// point or child), so rounding of the total mass only perturbs the offset
// (bounded by the node size), never the absolute coordinate.
struct Agg {
    df mass, charge, mu, L, px, py;
    df ox, oy;          // origin
    df sx, sy;          // sum m * (x - origin)
    bool has_origin;
};

__device__ __forceinline__ void agg_zero(Agg& g) {
    g.mass = g.charge = g.mu = g.L = g.px = g.py = g.ox = g.oy = g.sx = g.sy = df{ 0.f, 0.f };
    g.has_origin = false;
}

__device__ __forceinline__ void agg_add_com(Agg& g, df x, df y, float m) {
    if (!g.has_origin) { g.ox = x; g.oy = y; g.has_origin = true; }
    const df dx = df_add(x, df{ -g.ox.hi, -g.ox.lo });
    const df dy = df_add(y, df{ -g.oy.hi, -g.oy.lo });
    g.sx = df_add(g.sx, two_prod(dx.hi + dx.lo, m));
    g.sy = df_add(g.sy, two_prod(dy.hi + dy.lo, m));
}

// Higher moments about the node centre of mass: mass quadrupole I, charge
// dipole D, charge quadrupole J (second moments, not trace-free), sum |q|.
struct Mom {
    float ixx, ixy, iyy, s, dx, dy, jxx, jxy, jyy;
};
__device__ __forceinline__ void mom_zero(Mom& m) { m = Mom{ 0, 0, 0, 0, 0, 0, 0, 0, 0 }; }
__device__ __forceinline__ void mom_point(Mom& M, float m, float q, float dx, float dy) {
    M.ixx += m * dx * dx; M.ixy += m * dx * dy; M.iyy += m * dy * dy;
    M.dx += q * dx; M.dy += q * dy;
    M.jxx += q * dx * dx; M.jxy += q * dx * dy; M.jyy += q * dy * dy;
    M.s += fabsf(q);
}
// Adds a child's moments shifted by dx, dy (child COM minus parent COM).
__device__ __forceinline__ void mom_child(Mom& M, float m, float q, const float4& c1, const float4& c2, const float4& c3,
                                          float dx, float dy) {
    M.ixx += c1.x + m * dx * dx; M.ixy += c1.y + m * dx * dy; M.iyy += c1.z + m * dy * dy;
    M.s += c1.w;
    M.dx += c2.x + q * dx; M.dy += c2.y + q * dy;
    M.jxx += c2.z + 2.f * c2.x * dx + q * dx * dx;
    M.jxy += c2.w + c2.x * dy + c2.y * dx + q * dx * dy;
    M.jyy += c3.x + 2.f * c2.y * dy + q * dy * dy;
}
__device__ __forceinline__ void mom_write(float4* m1, float4* m2, float4* m3, int idx, const Mom& M) {
    m1[idx] = make_float4(M.ixx, M.ixy, M.iyy, M.s);
    m2[idx] = make_float4(M.dx, M.dy, M.jxx, M.jxy);
    m3[idx] = make_float4(M.jyy, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ void agg_com(const Agg& g, df& cx, df& cy) {
    const float m = g.mass.hi + g.mass.lo;
    if (m > 0.f) {
        cx = df_add(g.ox, df{ (g.sx.hi + g.sx.lo) / m, 0.f });
        cy = df_add(g.oy, df{ (g.sy.hi + g.sy.lo) / m, 0.f });
    } else {
        cx = df{ 0.f, 0.f }; cy = df{ 0.f, 0.f };
    }
}

__device__ __forceinline__ void agg_write(float4* A, float4* B, float4* C, int idx, const Agg& g,
                                          float size2, int level) {
    const float m = g.mass.hi + g.mass.lo;
    df cx, cy;
    float vx = 0.f, vy = 0.f;
    if (m > 0.f) {
        cx = df_add(g.ox, df{ (g.sx.hi + g.sx.lo) / m, 0.f });
        cy = df_add(g.oy, df{ (g.sy.hi + g.sy.lo) / m, 0.f });
        vx = (g.px.hi + g.px.lo) / m;
        vy = (g.py.hi + g.py.lo) / m;
    } else {
        cx = df{ 0.f, 0.f }; cy = df{ 0.f, 0.f };
    }
    A[idx] = make_float4(cx.hi, cy.hi, m, g.charge.hi + g.charge.lo);
    B[idx] = make_float4(vx, vy, g.mu.hi + g.mu.lo, g.L.hi + g.L.lo);
    C[idx] = make_float4(cx.lo, cy.lo, size2, (float)level);
}

__device__ __forceinline__ float node_size2(const DevParams& P, int level) {
    const double size = 2.0 * ldexp(P.rootW, -level);   // size = 2 bw (forces.js:641)
    return (float)(size * size);
}

__device__ __forceinline__ void aggregate_body(DevParams P, DevState S, TreeBufs T, FrameCtl* ctl, int vb, int nvb) {
    const int nLeaves = ctl->nLeaves;
    const int nInt = ctl->nInternal;
    const int nValid = ctl->nValid;
    if (nInt > T.cap_int) return;
    for (int leaf = vb * blockDim.x + threadIdx.x; leaf < nLeaves; leaf += nvb * blockDim.x) {
        const int4 lm = T.leaf_meta[leaf];
        Agg g; agg_zero(g);
        if (lm.x < 0 || lm.y < 1 || lm.x + lm.y > nValid || lm.w >= nInt) { atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
        // one point of the leaf (quadtree.js:276-287); wx, wy and mom come from
        // the particle the point refers to
        auto add_point = [&](const float4& pa, const float4& pb, const float4& pc, const float4& vel, float2 mom) {
            const uint32_t code = ref_code(__float_as_uint(pc.w));
            const float m = pa.z;
            const float wx = code_fvx(code) ? -vel.x : vel.x;
            const float wy = code_fvy(code) ? -vel.y : vel.y;
            if (code != CODE_IDENTITY) mom = make_float2(pc.y, pc.z);   // ghosts: formed at ghost creation (integrator.js:193-194)
            g.mass = df_add(g.mass, df{ m, 0.f });
            g.charge = df_add(g.charge, df{ pa.w, 0.f });
            g.mu = df_add(g.mu, df{ mom.x, 0.f });
            g.L = df_add(g.L, df{ mom.y, 0.f });
            g.px = df_add(g.px, two_prod(m, wx));
            g.py = df_add(g.py, two_prod(m, wy));
            agg_add_com(g, df{ pa.x, pb.x }, df{ pa.y, pb.y }, m);
        };
        if (lm.y <= LEAF_CAP) {
            // all loads of the leaf first (two rounds: the point records, then
            // the particles they refer to), then the sums in point order
            float4 pa[LEAF_CAP], pb[LEAF_CAP], pc[LEAF_CAP], vel[LEAF_CAP];
            float2 mom[LEAF_CAP];
#pragma unroll
            for (int k = 0; k < LEAF_CAP; k++) {
                if (k < lm.y) { pa[k] = T.ps_a[lm.x + k]; pb[k] = T.ps_b[lm.x + k]; pc[k] = T.ps_c[lm.x + k]; }
            }
#pragma unroll
            for (int k = 0; k < LEAF_CAP; k++) {
                if (k < lm.y) {
                    const uint32_t j = ref_index(__float_as_uint(pc[k].w));
                    vel[k] = S.vel[j];
                    mom[k] = S.mom[j];                         // cached by the previous force pass
                }
            }
#pragma unroll
            for (int k = 0; k < LEAF_CAP; k++)
                if (k < lm.y) add_point(pa[k], pb[k], pc[k], vel[k], mom[k]);
        } else {
            for (int k = 0; k < lm.y; k++) {                 // a level-31 bucket
                const int s = lm.x + k;
                const float4 pc = T.ps_c[s];
                const uint32_t j = ref_index(__float_as_uint(pc.w));
                add_point(T.ps_a[s], T.ps_b[s], pc, S.vel[j], S.mom[j]);
            }
        }
        agg_write(T.leaf_a, T.leaf_b, T.leaf_c, leaf, g, node_size2(P, lm.z), lm.z);
        if (T.mom_on) {
            df cx, cy;
            agg_com(g, cx, cy);
            Mom M; mom_zero(M);
            for (int k = 0; k < lm.y; k++) {
                const float4 pa = T.ps_a[lm.x + k];
                const float4 pb = T.ps_b[lm.x + k];
                const df ddx = df_add(df{ pa.x, pb.x }, df{ -cx.hi, -cx.lo });
                const df ddy = df_add(df{ pa.y, pb.y }, df{ -cy.hi, -cy.lo });
                mom_point(M, pa.z, pa.w, ddx.hi + ddx.lo, ddy.hi + ddy.lo);
            }
            mom_write(T.leaf_m1, T.leaf_m2, T.leaf_m3, leaf, M);
        }
        // climb
        int node = lm.w;
        int guard = 0;
        while (node >= 0 && node < nInt && guard++ <= KEY_LEVELS) {
            // the last child to arrive aggregates the node: the acquire-release
            // count publishes this child and shows the others
            const int4 ch = T.int_child[node];
            const int4 mm = T.int_meta[node];
            const int prev = atomic_add_acq_rel_gpu(&T.int_count[node], 1);
            const int nch = (ch.x >= 0) + (ch.y >= 0) + (ch.z >= 0) + (ch.w >= 0);
            if (prev != nch - 1) break;
            Agg h; agg_zero(h);
            const int cs[4] = { ch.x, ch.y, ch.z, ch.w };
            // every child's record first (one round of loads), then the sums in child order
            float4 ca[4], cb[4], cc[4];
            bool have[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {                    // quadtree.js:297-309
                const int c = cs[q];
                have[q] = false;
                if (c < 0) continue;
                if (c & LEAF_REF) {
                    const int li = c & ~LEAF_REF;
                    if (li >= nLeaves) { atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
                    ca[q] = __ldcg(&T.leaf_a[li]); cb[q] = __ldcg(&T.leaf_b[li]); cc[q] = __ldcg(&T.leaf_c[li]);
                } else {
                    if (c >= nInt) { atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
                    ca[q] = __ldcg(&T.int_a[c]); cb[q] = __ldcg(&T.int_b[c]); cc[q] = __ldcg(&T.int_c[c]);
                }
                have[q] = true;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (!have[q]) continue;
                const float4 a = ca[q], b = cb[q];
                const float m = a.z;
                h.mass = df_add(h.mass, df{ m, 0.f });
                h.charge = df_add(h.charge, df{ a.w, 0.f });
                h.mu = df_add(h.mu, df{ b.z, 0.f });
                h.L = df_add(h.L, df{ b.w, 0.f });
                h.px = df_add(h.px, two_prod(m, b.x));
                h.py = df_add(h.py, two_prod(m, b.y));
                if (m > 0.f) agg_add_com(h, df{ a.x, cc[q].x }, df{ a.y, cc[q].y }, m);
            }
            agg_write(T.int_a, T.int_b, T.int_c, node, h, node_size2(P, mm.x), mm.x);
            if (T.mom_on) {
                df px, py;
                agg_com(h, px, py);
                Mom M; mom_zero(M);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int c = cs[q];
                    if (c < 0) continue;
                    float4 a, cc, c1, c2, c3;
                    if (c & LEAF_REF) {
                        const int li = c & ~LEAF_REF;
                        if (li >= nLeaves) continue;
                        a = __ldcg(&T.leaf_a[li]); cc = __ldcg(&T.leaf_c[li]);
                        c1 = __ldcg(&T.leaf_m1[li]); c2 = __ldcg(&T.leaf_m2[li]); c3 = __ldcg(&T.leaf_m3[li]);
                    } else {
                        if (c >= nInt) continue;
                        a = __ldcg(&T.int_a[c]); cc = __ldcg(&T.int_c[c]);
                        c1 = __ldcg(&T.int_m1[c]); c2 = __ldcg(&T.int_m2[c]); c3 = __ldcg(&T.int_m3[c]);
                    }
                    if (!(a.z > 0.f)) continue;
                    const df ddx = df_add(df{ a.x, cc.x }, df{ -px.hi, -px.lo });
                    const df ddy = df_add(df{ a.y, cc.y }, df{ -py.hi, -py.lo });
                    mom_child(M, a.z, a.w, c1, c2, c3, ddx.hi + ddx.lo, ddy.hi + ddy.lo);
                }
                mom_write(T.int_m1, T.int_m2, T.int_m3, node, M);
            }
            node = mm.w;
        }
    }
}


}  // namespace geon
