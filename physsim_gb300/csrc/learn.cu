// learn.cu — training data of the learned far-field correction.
//
// learn_collect_pairs walks the tree for a list of target particles with the
// reference's opening rule (src/forces.js:622-694) and records every cell a
// target accepts as an aggregate.  learn_residuals then evaluates, for each
// pair, the exact sum over the cell's member particles (the pairwise sum of
// src/forces.js:94-125 restricted to the cell, excluding the target itself)
// minus the monopole term the walk uses, separately for the mass-sourced
// field (gravity + Yukawa, per unit target mass) and the charge-sourced field
// (Coulomb, per unit target charge), normalised by the scales of learn.cuh.
#include "learn.cuh"

namespace geon {

constexpr int LC_THREADS = 128;
constexpr int LC_WARPS = LC_THREADS / 32;

__global__ void __launch_bounds__(LC_THREADS)
collect_pairs_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root, FrameCtl* ctl,
                     const int* __restrict__ targets, int k, LearnPair* pairs, long long cap,
                     unsigned long long* d_count) {
    __shared__ int s_node[LC_WARPS][WALK_STACK];
    __shared__ unsigned s_mask[LC_WARPS][WALK_STACK];
    const int warp = threadIdx.x >> 5;
    const unsigned lane = threadIdx.x & 31;
    const int ti = (blockIdx.x * LC_WARPS + warp) * 32 + (int)lane;
    const int n = ctl->n;
    const bool valid = ti < k && targets[ti] >= 0 && targets[ti] < n;
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    if (!active) return;
    const int i = valid ? targets[ti] : 0;
    const float4 p = S.pos[i];
    const float2 pl = S.pos_lo[i];
    const int root = *d_root;
    const int nInt = ctl->nInternal, nLeaf = ctl->nLeaves;
    if ((ctl->err & (ERR_NODE_OVERFLOW | ERR_BAD_INDEX)) || root == ROOT_NONE || (root & LEAF_REF)) return;
    int top = 0;
    if (lane == 0) { s_node[warp][0] = root; s_mask[warp][0] = active; }
    top = 1;
    __syncwarp();
    while (top > 0) {
        top--;
        const int node = s_node[warp][top];
        const unsigned mask = s_mask[warp][top];
        __syncwarp();
        if (node & LEAF_REF) continue;                   // leaves are evaluated point by point
        if (node < 0 || node >= nInt) { if (lane == 0) atomicOr(&ctl->err, ERR_BAD_INDEX); continue; }
        const float4 a = T.int_a[node];
        if (a.z < EPS_F) continue;
        const float4 c = T.int_c[node];
        bool accept = false;
        if ((mask >> lane) & 1u) {
            float rx, ry;
            displacement(P, p.x, p.y, a.x, c.x - pl.x, a.y, c.y - pl.y, rx, ry);
            const float rhs = P.thetaSq * __fmaf_rn(rx, rx, ry * ry);
            accept = c.z < rhs;
            if (fabsf(rhs - c.z) <= 1e-6f * c.z) {
                double dx, dy;
                const double ox = (double)p.x + (double)pl.x, oy = (double)p.y + (double)pl.y;
                const double sx = (double)a.x + (double)c.x, sy = (double)a.y + (double)c.y;
                if (P.periodic) min_image_d(ox, oy, sx, sy, P.topology, P.Wd, P.Hd, dx, dy);
                else { dx = sx - ox; dy = sy - oy; }
                const double size = 2.0 * ldexp(P.rootW, -(int)c.w);
                accept = size * size < P.thetaSqD * (dx * dx + dy * dy);
            }
        }
        const unsigned acc = __ballot_sync(0xffffffffu, accept);
        if (acc) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(d_count, (unsigned long long)__popc(acc));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (accept) {
                const unsigned long long pos = base + (unsigned long long)__popc(acc & lanemask_lt());
                if (pos < (unsigned long long)cap) pairs[pos] = LearnPair{ node, i };
            }
        }
        const unsigned open = mask & ~acc;
        if (open) {
            const int4 ch = T.int_child[node];
            const int np = (ch.x >= 0) + (ch.y >= 0) + (ch.z >= 0) + (ch.w >= 0);
            if (top + np > WALK_STACK) { if (lane == 0) atomicOr(&ctl->err, ERR_STACK_OVERFLOW); break; }
            if (lane == 0) {
                int tp = top;
                if (ch.x >= 0) { s_node[warp][tp] = ch.x; s_mask[warp][tp++] = open; }
                if (ch.y >= 0) { s_node[warp][tp] = ch.y; s_mask[warp][tp++] = open; }
                if (ch.z >= 0) { s_node[warp][tp] = ch.z; s_mask[warp][tp++] = open; }
                if (ch.w >= 0) { s_node[warp][tp] = ch.w; s_mask[warp][tp++] = open; }
            }
            top += np;
            __syncwarp();
        }
    }
    (void)nLeaf;
}

// Field of one source (mass m, charge q) at displacement (rx, ry) from the
// target: mass-sourced (gravity + Yukawa) per unit target mass, and
// charge-sourced (Coulomb) per unit target charge (src/forces.js:205-240, 387-399).
__device__ __forceinline__ void source_fields(const DevParams& P, float rx, float ry, float m, float q,
                                              float& gx, float& gy, float& ex, float& ey) {
    const float rawRSq = rx * rx + ry * ry;
    const float rSq = rawRSq + P.softSq;
    const float invR = rsqrtf(rSq);
    const float invRSq = invR * invR;
    const float invR3 = invR * invRSq;
    float fm = (P.toggles & GEON_GRAVITY) ? m * invR3 : 0.f;
    if (P.yukOn && rawRSq < P.yukCutSq) {
        const float r = rSq * invR;
        fm += YUKAWA_COUPLING * m * __expf(-P.yukMu * r) * (invRSq + P.yukMu * invR) * invR;
    }
    const float fc = (P.toggles & GEON_COULOMB) ? -q * invR3 : 0.f;
    gx += rx * fm; gy += ry * fm;
    ex += rx * fc; ey += ry * fc;
}

__global__ void residual_kernel(DevParams P, DevState S, TreeBufs T, const LearnPair* __restrict__ pairs,
                                const unsigned long long* d_count, int cap, float* feat_m, float* feat_c, float* target,
                                float* scales) {
    const int np = (int)min(*d_count, (unsigned long long)cap);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < np; e += gridDim.x * blockDim.x) {
        const LearnPair pr = pairs[e];
        const int node = pr.node, i = pr.target;
        const float4 p = S.pos[i];
        const float2 pl = S.pos_lo[i];
        const float4 a = T.int_a[node], c = T.int_c[node];
        const int4 mm = T.int_meta[node];
        float dx, dy;
        displacement(P, p.x, p.y, a.x, c.x - pl.x, a.y, c.y - pl.y, dx, dy);
        // monopole (forces.js:680-685)
        float mgx = 0.f, mgy = 0.f, mex = 0.f, mey = 0.f;
        source_fields(P, dx, dy, a.z, a.w, mgx, mgy, mex, mey);
        // exact sum over the cell's members
        float gx = 0.f, gy = 0.f, ex = 0.f, ey = 0.f;
        for (int s = mm.y; s < mm.z; s++) {
            const float4 pa = T.ps_a[s];
            const float4 pb = T.ps_b[s];
            if ((int)ref_index(__float_as_uint(T.ps_c[s].w)) == i) continue;
            float rx, ry;
            displacement(P, p.x, p.y, pa.x, pb.x - pl.x, pa.y, pb.y - pl.y, rx, ry);
            source_fields(P, rx, ry, pa.z, pa.w, gx, gy, ex, ey);
        }
        float fm[LF], fc[LF], sm, sc;
        const float size = sqrtf(c.z);
        pair_features(P, dx, dy, size, a.z, a.w, T.int_m1[node], T.int_m2[node], T.int_m3[node], fm, fc, sm, sc);
        for (int f = 0; f < LF; f++) { feat_m[(size_t)e * LF + f] = fm[f]; feat_c[(size_t)e * LF + f] = fc[f]; }
        const float ism = sm > 0.f ? 1.f / sm : 0.f, isc = sc > 0.f ? 1.f / sc : 0.f;
        target[(size_t)e * 4 + 0] = (gx - mgx) * ism;
        target[(size_t)e * 4 + 1] = (gy - mgy) * ism;
        target[(size_t)e * 4 + 2] = (ex - mex) * isc;
        target[(size_t)e * 4 + 3] = (ey - mey) * isc;
        scales[(size_t)e * 2 + 0] = sm;
        scales[(size_t)e * 2 + 1] = sc;
    }
}

// Deterministic order of the collected pairs: (target, node) keys sorted
// with the stable radix sort, then the records permuted.
__global__ void pair_keys_kernel(const LearnPair* __restrict__ pairs, const unsigned long long* d_count, int cap,
                                 int* d_n, uint64_t* keys, uint32_t* vals) {
    const int n = (int)min(*d_count, (unsigned long long)cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_n = n;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const LearnPair p = pairs[e];
        keys[e] = ((uint64_t)(uint32_t)p.target << 32) | (uint64_t)(uint32_t)p.node;
        vals[e] = (uint32_t)e;
    }
}
__global__ void pair_permute_kernel(const LearnPair* __restrict__ in, const uint32_t* __restrict__ order,
                                    const int* d_n, LearnPair* __restrict__ out) {
    const int n = *d_n;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) out[e] = in[order[e]];
}

size_t learn_sort_scratch_bytes(int cap) {
    const size_t c = (size_t)std::max(cap, 1);
    return c * (2 * sizeof(uint64_t) + 2 * sizeof(uint32_t)) + radix_temp_bytes(std::max(cap, 1)) + 256;
}

void learn_sort_pairs(const LearnPair* pairs, const unsigned long long* d_count, int cap, LearnPair* out, int* d_n,
                      void* scratch, cudaStream_t st, LaunchCounter& lc) {
    const size_t c = (size_t)std::max(cap, 1);
    char* p = static_cast<char*>(scratch);
    uint64_t* keys = reinterpret_cast<uint64_t*>(p); p += c * sizeof(uint64_t);
    uint64_t* keys_alt = reinterpret_cast<uint64_t*>(p); p += c * sizeof(uint64_t);
    uint32_t* vals = reinterpret_cast<uint32_t*>(p); p += c * sizeof(uint32_t);
    uint32_t* vals_alt = reinterpret_cast<uint32_t*>(p); p += c * sizeof(uint32_t);
    p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) & ~(uintptr_t)255);
    const int blocks = 152 * 8;
    pair_keys_kernel<<<blocks, 256, 0, st>>>(pairs, d_count, cap, d_n, keys, vals);
    lc.add(1);
    const int which = radix_sort_pairs(keys, vals, keys_alt, vals_alt, (int)c, d_n, 64, p, st, &lc);
    pair_permute_kernel<<<blocks, 256, 0, st>>>(pairs, which ? vals_alt : vals, d_n, out);
    lc.add(1);
}

void learn_collect_pairs(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                         const int* d_targets, int k, LearnPair* pairs, long long cap, unsigned long long* d_count,
                         cudaStream_t st, LaunchCounter& lc) {
    cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), st);
    const int blocks = std::max(1, (k + LC_THREADS - 1) / LC_THREADS);
    collect_pairs_kernel<<<blocks, LC_THREADS, 0, st>>>(P, S, T, d_root, ctl, d_targets, k, pairs, cap, d_count);
    lc.add(1);
}

void learn_residuals(const DevParams& P, const DevState& S, const TreeBufs& T, const LearnPair* pairs,
                     const unsigned long long* d_count,
                     int cap, float* feat_m, float* feat_c, float* target, float* scales, cudaStream_t st,
                     LaunchCounter& lc) {
    residual_kernel<<<152 * 8, 128, 0, st>>>(P, S, T, pairs, d_count, cap, feat_m, feat_c, target, scales);
    lc.add(1);
}

}  // namespace geon
