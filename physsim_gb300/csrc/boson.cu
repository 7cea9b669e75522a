// boson.cu — the boson-tree walks (src/forces.js:697-901).
//
// The boson pool (photons, pions, leptons: positions, gravitational source
// mass _srcMass, charge _srcCharge) is held by a second handle as particles,
// so its quadtree is the same Morton-key build as the particles' (root box of
// the domain, capacity 4, no periodic ghosts: integrator.js:263-277) with
// mass, charge and centre-of-mass aggregates (quadtree.js:316-368).  One walk
// serves the three reference functions: a softened monopole sum of the
// pool's mass (or charge) at a target point, leaves point by point, cells
// accepted when size^2 < theta^2 d^2 (forces.js:713-770).  One thread walks
// one target; the pool is small next to the particles, so its tree is
// shallow and stays in L2.
#include "boson.cuh"

namespace geon {

static inline int grid_for(int n, int threads) {
    const int b = (n + threads - 1) / threads;
    return b < 1 ? 1 : (b > device_sms() * 16 ? device_sms() * 16 : b);
}

constexpr int BOSON_STACK = 128;

__device__ __forceinline__ float root_value(const BosonTree& B, int root, bool charge) {
    if (root == ROOT_NONE) return 0.f;
    const float4 a = (root & LEAF_REF) ? B.T.leaf_a[root & ~LEAF_REF] : B.T.int_a[root];
    return charge ? a.w : a.z;
}

// _walkBosonTreeCore for the 32 targets of a warp (lanes with active =
// false take no part): the warp walks the pool's tree once, every stack
// entry carrying the mask of lanes that still need the node, so nodes several
// lanes need are read once (targets come in tree order, so a warp's targets
// are neighbours).  Per lane: scale * sum of val * r / (r^2 + softSq)^(3/2),
// minimum images when periodic; leaves point by point, cells accepted when
// size^2 < theta^2 d^2 (forces.js:754).  The opening test is FP32 with an
// FP64 re-test within 1e-5 of a tie, so it decides as the reference's FP64
// test does.  `stk` / `msk` are the warp's stack in shared memory.
template <bool CHARGE>
__device__ float2 boson_walk(const DevParams& P, const BosonTree& B, int root, int nInt, int nLeaf, int nValid,
                             int* stk, unsigned* msk, bool active, float tx, float txl, float ty, float tyl,
                             float scale, float softSq, bool& ok) {
    float kx = 0.f, ky = 0.f;
    const unsigned lane = threadIdx.x & 31;
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!act || root == ROOT_NONE) return make_float2(0.f, 0.f);
    const TreeBufs& T = B.T;
    const float thetaSq = (float)P.thetaSqD;
    if (lane == 0) { stk[0] = root; msk[0] = act; }
    __syncwarp();
    int top = 1;
    while (top > 0) {
        const int node = stk[top - 1];
        const unsigned mask = msk[top - 1];
        __syncwarp();
        top--;
        const bool mine = (mask >> lane) & 1u;
        if (node & LEAF_REF) {
            const int li = node & ~LEAF_REF;
            if (li < 0 || li >= nLeaf) { ok = false; break; }
            if (CHARGE ? B.lq[li] == 0.0 : T.leaf_a[li].z < EPS_F) continue;   // skipNode
            const int4 lm = T.leaf_meta[li];
            if (lm.x < 0 || lm.x + lm.y > nValid) { ok = false; break; }
            if (mine) {
                for (int q = lm.x; q < lm.x + lm.y; q++) {
                    const float4 pa = T.ps_a[q], pb = T.ps_b[q];
                    const float val = CHARGE ? pa.w : pa.z;
                    if (CHARGE && val == 0.f) continue;                       // skipPoint
                    float rx, ry;
                    displacement(P, tx, ty, pa.x, pb.x - txl, pa.y, pb.y - tyl, rx, ry);
                    const float inv = rsqrtf(rx * rx + ry * ry + softSq);
                    const float f = scale * val * inv * inv * inv;
                    kx += rx * f;
                    ky += ry * f;
                }
            }
            __syncwarp();
            continue;
        }
        if (node < 0 || node >= nInt) { ok = false; break; }
        const float4 a = T.int_a[node];
        if (CHARGE ? B.iq[node] == 0.0 : a.z < EPS_F) continue;
        const float4 c = T.int_c[node];
        bool open = false;
        if (mine) {
            float rx, ry;
            displacement(P, tx, ty, a.x, c.x - txl, a.y, c.y - tyl, rx, ry);
            float dSq = rx * rx + ry * ry;
            const float rhs = thetaSq * dSq;
            bool accept = c.z < rhs;
            if (fabsf(c.z - rhs) <= 1e-5f * fmaxf(c.z, rhs)) {                 // near a tie: decide in FP64
                double dxd, dyd;
                const double txd = (double)tx + txl, tyd = (double)ty + tyl;
                if (P.periodic) min_image_d(txd, tyd, (double)a.x + c.x, (double)a.y + c.y, P.topology, P.Wd, P.Hd, dxd, dyd);
                else { dxd = ((double)a.x + c.x) - txd; dyd = ((double)a.y + c.y) - tyd; }
                const double dSqd = dxd * dxd + dyd * dyd;
                accept = (double)c.z < P.thetaSqD * dSqd;
                dSq = (float)dSqd;
            }
            if (accept) {
                const float inv = rsqrtf(dSq + softSq);
                const float f = scale * (CHARGE ? (float)B.iq[node] : a.z) * inv * inv * inv;
                kx += rx * f;
                ky += ry * f;
            } else {
                open = true;
            }
        }
        const unsigned om = __ballot_sync(0xffffffffu, open);
        if (!om) continue;
        if (top + 4 > BOSON_STACK) { ok = false; break; }
        const int4 ch = T.int_child[node];
        if (lane == 0) {
            int t = top;
            if (ch.x != -1) { stk[t] = ch.x; msk[t++] = om; }
            if (ch.y != -1) { stk[t] = ch.y; msk[t++] = om; }
            if (ch.z != -1) { stk[t] = ch.z; msk[t++] = om; }
            if (ch.w != -1) { stk[t] = ch.w; msk[t++] = om; }
        }
        top += (ch.x != -1) + (ch.y != -1) + (ch.z != -1) + (ch.w != -1);
        __syncwarp();
    }
    return make_float2(kx, ky);
}

__global__ void boson_clear_planner_kernel(FrameCtl* ctl) {
    ctl->maxAccelSqBits = 0ull;
    ctl->maxCycBits = 0ull;
}

constexpr int BOSON_THREADS = 128;

// Targets: the walk list of the force pass (tgt, after merge collisions),
// the particle tree's order TP.tgt (Barnes-Hut: the tree of this pass), or
// the slots in order (pairwise sum); in tree order each warp holds neighbours.
__global__ void __launch_bounds__(BOSON_THREADS)
boson_gravity_kernel(DevParams P, DevState S, TreeBufs TP, FrameCtl* ctl, BosonTree B, const int* tgt, int tgt_count,
                     int brk) {
    __shared__ int s_stk[BOSON_THREADS / 32][BOSON_STACK];
    __shared__ unsigned s_msk[BOSON_THREADS / 32][BOSON_STACK];
    const int warp = threadIdx.x >> 5;
    const int nT = tgt ? tgt_count : ctl->n;
    const int nInt = min(B.ctl->nInternal, B.T.cap_int), nLeaf = B.ctl->nLeaves, nValid = B.ctl->nValid;
    const int root = *B.d_root;
    const bool any = root_value(B, root, false) >= EPS_F;                     // forces.js:791
    const int stride = gridDim.x * blockDim.x;
    const int iters = (nT + stride - 1) / stride;
    bool ok = true;
    for (int it = 0; it < iters; it++) {
        const int k = blockIdx.x * blockDim.x + threadIdx.x + it * stride;
        double aSq = 0.0, wc = 0.0;
        int i = -1;
        if (k < nT) i = tgt ? tgt[k] : (TP.tgt ? TP.tgt[k] : k);
        const bool valid = i >= 0 && i < P.n_cap;
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 pl = make_float2(0.f, 0.f);
        if (valid) { p = S.pos[i]; pl = S.pos_lo[i]; }
        float2 g = make_float2(0.f, 0.f);
        if (any)
            g = boson_walk<false>(P, B, root, nInt, nLeaf, nValid, s_stk[warp], s_msk[warp], valid, p.x, pl.x, p.y, pl.y,
                                  p.z, P.softSq, ok);
        if (valid) {
            float4 f = S.force[i];
            if (any) {
                f.x += g.x;
                f.y += g.y;
                S.force[i] = f;
                if (brk) {                                                   // forceGravity
                    S.brk[i] += g.x;
                    S.brk[(size_t)P.n_cap + i] += g.y;
                }
            }
            // planner maxima from the forces the next kick uses (integrator.js:813-836)
            const double im = (double)S.spin[i].w;
            aSq = ((double)f.x * f.x + (double)f.y * f.y) * im * im;
            if ((P.toggles & GEON_MAGNETIC) || P.extBz != 0.f) {
                const double absBz = fabs((double)f.z);
                if (absBz > 0) wc = fmax(wc, fabs((double)S.pos[i].w) * absBz * im);
            }
            if (P.toggles & GEON_GRAVITOMAG) {
                const double absBgz = fabs((double)f.w);
                if (absBgz > 0) wc = fmax(wc, 4.0 * absBgz);
            }
            if (!(aSq == aSq)) aSq = 0.0;
            if (!(wc == wc)) wc = 0.0;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            aSq = fmax(aSq, __shfl_xor_sync(0xffffffffu, aSq, o));
            wc = fmax(wc, __shfl_xor_sync(0xffffffffu, wc, o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomic_max_pos_double(&ctl->maxAccelSqBits, aSq);
            atomic_max_pos_double(&ctl->maxCycBits, wc);
        }
    }
    if (!ok) atomicOr(&ctl->err, ERR_BAD_INDEX);
}

// Kicks on the pool itself: gravity with the receivers' factors (2 dt for
// photons, (1 + v^2) dt for pions and leptons, forces.js:824-850), Coulomb
// between the charged massive bosons (-q dt, forces.js:887-899).  `massive`
// is the number of pions and leptons (the Coulomb pass needs two).
__global__ void __launch_bounds__(BOSON_THREADS)
boson_kick_kernel(DevParams P, BosonTree B, float dt, unsigned what, int massive, float2* out) {
    __shared__ int s_stk[BOSON_THREADS / 32][BOSON_STACK];
    __shared__ unsigned s_msk[BOSON_THREADS / 32][BOSON_STACK];
    const int warp = threadIdx.x >> 5;
    const int nInt = min(B.ctl->nInternal, B.T.cap_int), nLeaf = B.ctl->nLeaves, nValid = B.ctl->nValid;
    const int root = *B.d_root;
    const bool grav = (what & 1u) && B.n >= 2 && root_value(B, root, false) >= EPS_F;
    const bool coul = (what & 2u) && massive >= 2;
    bool ok = true;
    const int stride = gridDim.x * blockDim.x;
    const int iters = (B.n + stride - 1) / stride;
    for (int it = 0; it < iters; it++) {
        const int k = blockIdx.x * blockDim.x + threadIdx.x + it * stride;
        const int b = k < B.n ? B.T.tgt[k] : -1;                              // the pool's tree order
        const bool valid = b >= 0 && b < B.n;
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 pl = make_float2(0.f, 0.f), kv = make_float2(0.f, 0.f);
        if (valid) { p = B.S.pos[b]; pl = B.S.pos_lo[b]; kv = B.kind[b]; }
        float kx = 0.f, ky = 0.f;
        if (grav) {
            const float scale = kv.x == 0.f ? 2.f * dt : (1.f + kv.y) * dt;
            const float2 g = boson_walk<false>(P, B, root, nInt, nLeaf, nValid, s_stk[warp], s_msk[warp], valid,
                                               p.x, pl.x, p.y, pl.y, scale, BOSON_SOFTENING_SQ, ok);
            kx += g.x; ky += g.y;
        }
        if (coul) {
            const bool mine = valid && kv.x != 0.f && p.w != 0.f;
            const float2 g = boson_walk<true>(P, B, root, nInt, nLeaf, nValid, s_stk[warp], s_msk[warp], mine,
                                              p.x, pl.x, p.y, pl.y, -p.w * dt, BOSON_SOFTENING_SQ, ok);
            kx += g.x; ky += g.y;
        }
        if (valid) out[b] = make_float2(kx, ky);
    }
    (void)ok;
}

__global__ void boson_charge_kernel(BosonTree B) {
    const int nInt = min(B.ctl->nInternal, B.T.cap_int), nLeaf = B.ctl->nLeaves, nValid = B.ctl->nValid;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nInt + nLeaf; t += gridDim.x * blockDim.x) {
        int s0, s1;
        if (t < nInt) { const int4 m = B.T.int_meta[t]; s0 = m.y; s1 = m.z; }
        else { const int4 lm = B.T.leaf_meta[t - nInt]; s0 = lm.x; s1 = lm.x + lm.y; }
        double q = 0.0;
        for (int k = max(s0, 0); k < min(s1, nValid); k++) q += (double)B.T.ps_a[k].w;   // exact for FP32 inputs
        if (t < nInt) const_cast<double*>(B.iq)[t] = q;
        else const_cast<double*>(B.lq)[t - nInt] = q;
    }
}

void boson_charges(const BosonTree& B, double* iq, double* lq, cudaStream_t st, LaunchCounter& lc) {
    BosonTree b = B;
    b.iq = iq;
    b.lq = lq;
    boson_charge_kernel<<<grid_for(std::max(B.T.cap_int + B.T.cap_pts, 1), 256), 256, 0, st>>>(b);
    lc.add(1);
}

void boson_gravity(const DevParams& P, const DevState& S, const TreeBufs& TP, FrameCtl* ctl, const BosonTree& B,
                   const int* tgt_list, int tgt_count, bool brk, int n_cap, cudaStream_t st, LaunchCounter& lc) {
    boson_clear_planner_kernel<<<1, 1, 0, st>>>(ctl);
    const int nT = tgt_list ? tgt_count : n_cap;
    boson_gravity_kernel<<<grid_for(std::max(nT, 1), BOSON_THREADS), BOSON_THREADS, 0, st>>>(P, S, TP, ctl, B, tgt_list,
                                                                                             tgt_count, brk ? 1 : 0);
    lc.add(2);
}

void boson_kicks(const DevParams& P, const BosonTree& B, float dt, unsigned what, int massive, float2* out,
                 cudaStream_t st, LaunchCounter& lc) {
    boson_kick_kernel<<<grid_for(std::max(B.n, 1), BOSON_THREADS), BOSON_THREADS, 0, st>>>(P, B, dt, what, massive, out);
    lc.add(1);
}

}  // namespace geon
