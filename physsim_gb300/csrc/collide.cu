// collide.cu — merge collisions (src/collisions.js:24-158) on the quadtree of
// the substep, as Physics.update runs them right after the tree rebuild
// (src/integrator.js:1350-1381) when collisionMode is COL_MERGE.
//
// The reference resolves pairs one at a time: particles in array order, each
// particle's candidates in the order QuadTreePool.query reports them
// (quadtree.js:372-404), with masses, radii and base masses changing as it
// goes.  The order matters (a particle that has merged away keeps "merging"
// with its later candidates, annihilation shrinks radii), so the resolution
// itself stays sequential.  What is parallel is everything around it:
//  * detection: one thread per particle runs the box query against the tree
//    and keeps the candidates that can still collide when their turn comes
//    (geometry and id order are fixed; masses and radii only decrease, so the
//    values at the start of the pass bound every later test);
//  * order: the query visits children SE, SW, NE, NW (the stack of
//    quadtree.js:394-398), which in Morton order is descending digit order,
//    and reports a leaf's points in storage order.  Storage order follows the
//    insertion history: a node that receives its fifth point divides, that
//    point descends first and the four stored points follow from the work
//    stack in reverse (quadtree.js:205-232).  So every node's arrival
//    sequence is a prefix of at most five points (the reversed first five of
//    its parent's sequence that fall in it) followed by its other points in
//    insertion order.  A leaf's order is rebuilt from the root down with the
//    five earliest-inserted points of every internal node, computed bottom-up;
//  * the removed particles stay in the tree for the rest of the substep and
//    act as sources with their live fields (mass 0, last cached moments),
//    exactly as the reference's tree keeps pointing at them; their tree
//    records are patched, and the force pass walks a target list without
//    them plus the spawns (which are targets but not tree points).
#include "collide.cuh"

namespace geon {

static inline int grid_for(int n, int threads) {
    const int b = (n + threads - 1) / threads;
    return b < 1 ? 1 : (b > device_sms() * 16 ? device_sms() * 16 : b);
}

// 31-bit grid coordinate of one axis of a Morton key (bit 2b + axis).
__device__ __forceinline__ uint32_t unzip_axis(uint64_t k, int axis) {
    uint64_t v = (k >> axis) & 0x5555555555555555ull;
    v = (v | (v >> 1)) & 0x3333333333333333ull;
    v = (v | (v >> 2)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v >> 4)) & 0x00FF00FF00FF00FFull;
    v = (v | (v >> 8)) & 0x0000FFFF0000FFFFull;
    v = (v | (v >> 16)) & 0x00000000FFFFFFFFull;
    return (uint32_t)v;
}

__device__ __forceinline__ double point_x(const TreeBufs& T, int q) { return (double)T.ps_a[q].x + (double)T.ps_b[q].x; }
__device__ __forceinline__ double point_y(const TreeBufs& T, int q) { return (double)T.ps_a[q].y + (double)T.ps_b[q].y; }

// Region of the node at `level` holding key K: the closed box of the grid
// cells sharing K's first `level` digits (centre +/- bw of quadtree.js:52-76,
// exact on the quantisation grid).
struct Region { double x0, x1, y0, y1; };
__device__ __forceinline__ Region node_region(const DevParams& P, uint64_t K, int level) {
    const int sh = KEY_LEVELS - level;
    const double dX = P.rootW * (1.0 / 1073741824.0), dY = P.rootH * (1.0 / 1073741824.0);
    const double span = ldexp(1.0, sh);
    Region R;
    R.x0 = (P.rootX - P.rootW) + (double)((unzip_axis(K, 0) >> sh) << sh) * dX;
    R.y0 = (P.rootY - P.rootH) + (double)((unzip_axis(K, 1) >> sh) << sh) * dY;
    R.x1 = R.x0 + span * dX;
    R.y1 = R.y0 + span * dY;
    return R;
}

// Query of one particle: centre (compensated pair), half-size of the box
// (queryReuse(root, x, y, 2r, 2r)), radius, index and id.  Detection works in
// FP32 with slack and keeps a superset of the candidates (GB300's FP64 rate is
// a small fraction of its FP32 rate); the resolution re-tests every candidate
// exactly in FP64.
struct QueryP { float xh, xl, yh, yl, r, rad, slack; int i, id; };

__device__ __forceinline__ bool load_query(const DevState& S, int i, QueryP& Q) {
    const float4 p = S.pos[i];
    if (p.z == 0.f) return false;
    const float2 pl = S.pos_lo[i];
    Q.xh = p.x; Q.xl = pl.x; Q.yh = p.y; Q.yl = pl.y;
    Q.rad = S.spin[i].z;
    Q.r = 2.f * Q.rad;
    Q.slack = 1e-5f * Q.r + 1e-6f * (fabsf(p.x) + fabsf(p.y)) + 1e-30f;
    Q.i = i;
    Q.id = S.id[i];
    return true;
}

// Depth-first box query (quadtree.js:372-404) from node `start`: internal
// nodes whose box meets the query box are opened, children pushed NW, NE, SW,
// SE; `leaf(li)` is called for every leaf reached, in the reference's visiting
// order.  Boxes are widened by COL_TOL of the root size: a node visited in
// excess only costs time, its points are tested one by one.  Starting below
// the root at a node whose box holds the whole query box visits the same
// leaves in the same order.
template <class F>
__device__ bool query_leaves(const TreeBufs& T, const CollBufs& B, int start, int nInt, int nLeaf, float tol,
                             const QueryP& Q, F&& leaf) {
    if (start == ROOT_NONE) return true;
    int stack[COL_STACK];
    int top = 0;
    stack[top++] = start;
    const float r = Q.r + tol;
    while (top > 0) {
        const int node = stack[--top];
        if (node & LEAF_REF) {
            const int li = node & ~LEAF_REF;
            if (li < 0 || li >= nLeaf) return false;
            leaf(li);
            continue;
        }
        if (node < 0 || node >= nInt) return false;
        const float4 b = B.ibox[node];
        if (Q.xh - r > b.z || Q.xh + r < b.x || Q.yh - r > b.w || Q.yh + r < b.y) continue;
        if (top + 4 > COL_STACK) return false;
        const int4 c = T.int_child[node];
        if (c.x != -1) stack[top++] = c.x;
        if (c.y != -1) stack[top++] = c.y;
        if (c.z != -1) stack[top++] = c.z;
        if (c.w != -1) stack[top++] = c.w;
    }
    return true;
}

// Candidate test of tree point q for the query of particle i: inside the box,
// another particle, alive, later id, and overlapping at the start-of-pass
// radii (collisions.js:37-57) -- each test widened by the query's slack.
__device__ __forceinline__ bool candidate(const DevParams& P, const DevState& S, const TreeBufs& T, const QueryP& Q,
                                          int q, int n) {
    const float4 pa = T.ps_a[q], pb = T.ps_b[q];
    float dx = __fadd_rn(__fsub_rn(pa.x, Q.xh), __fsub_rn(pb.x, Q.xl));
    float dy = __fadd_rn(__fsub_rn(pa.y, Q.yh), __fsub_rn(pb.y, Q.yl));
    const float lim = Q.r + Q.slack;
    if (fabsf(dx) > lim || fabsf(dy) > lim) return false;
    const int j = (int)ref_index(__float_as_uint(T.ps_c[q].w));
    if (j == Q.i || j < 0 || j >= n) return false;
    if (S.pos[j].z == 0.f) return false;
    if (Q.id >= S.id[j]) return false;
    if (P.periodic) {
        if (P.topology == GEON_TORUS) {
            dx = torus_wrap_f(dx, P.W, P.halfW);
            dy = torus_wrap_f(dy, P.H, P.halfH);
        } else {
            double ddx, ddy;
            min_image_d((double)Q.xh + Q.xl, (double)Q.yh + Q.yl, (double)pa.x + pb.x, (double)pa.y + pb.y,
                        P.topology, P.Wd, P.Hd, ddx, ddy);
            dx = (float)ddx; dy = (float)ddy;
        }
    }
    const float md = (Q.rad + S.spin[j].z) * (1.f + 1e-5f) + Q.slack;
    return dx * dx + dy * dy < md * md;
}

// ---- detection ------------------------------------------------------------------------------
__global__ void col_begin_kernel(CollCtl* cc) {
    cc->total = 0; cc->spawned = 0; cc->merges = 0; cc->annihilations = 0;
    cc->removed = 0; cc->need_order = 0; cc->nlive = 0;
}

__global__ void col_inverse_kernel(TreeBufs T, const FrameCtl* ctl, CollBufs B) {
    const int nValid = ctl->nValid, n = ctl->n;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nValid; s += gridDim.x * blockDim.x) {
        const uint32_t ref = __float_as_uint(T.ps_c[s].w);
        if (ref_code(ref) != CODE_IDENTITY) continue;
        const int j = (int)ref_index(ref);
        if (j < n) B.inv[j] = s;
    }
}

// Node boxes for the detection pass, rounded outward to FP32: internal
// nodes and leaves.  Containment tests shrink them by COL_TOL of the root
// size and intersection tests grow them by it, which covers the rounding.
__global__ void col_geo_kernel(DevParams P, TreeBufs T, const FrameCtl* ctl, CollBufs B) {
    const int nInt = min(ctl->nInternal, T.cap_int), nLeaf = ctl->nLeaves, nValid = ctl->nValid;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nInt + nLeaf; t += gridDim.x * blockDim.x) {
        int start, level;
        if (t < nInt) { const int4 m = T.int_meta[t]; start = m.y; level = m.x; }
        else { const int4 lm = T.leaf_meta[t - nInt]; start = lm.x; level = lm.z; }
        float4 b = make_float4(0.f, 0.f, -1.f, -1.f);
        if (start >= 0 && start < nValid && level >= 0 && level <= KEY_LEVELS) {
            const Region R = node_region(P, T.skey[start], level);
            b = make_float4(__double2float_rd(R.x0), __double2float_rd(R.y0), __double2float_ru(R.x1), __double2float_ru(R.y1));
        }
        if (t < nInt) B.ibox[t] = b; else B.lbox[t - nInt] = b;
    }
}

__device__ __forceinline__ bool box_holds(const float4 b, const QueryP& Q, float tol) {
    const float r = Q.r + tol;
    return Q.xh - r >= b.x && Q.xh + r <= b.z && Q.yh - r >= b.y && Q.yh + r <= b.w;
}

// Smallest node on the path from particle i's own leaf to the root whose box
// holds the query box (the root when i is not in the tree or none does), and
// the run of sorted points it covers.
__device__ int query_node(const TreeBufs& T, const CollBufs& B, const QueryP& Q, int root, int nInt, int nLeaf,
                          int nValid, int nPts, float tol, int& s0, int& s1) {
    s0 = 0;
    s1 = nPts;
    if (root == ROOT_NONE) { s1 = 0; return root; }
    const int s = B.inv[Q.i];
    if (!(root & LEAF_REF) && s >= 0 && s < nValid) {
        const int li = T.leaf_of[s];
        if (li >= 0 && li < nLeaf) {
            const int4 lm = T.leaf_meta[li];
            if (box_holds(B.lbox[li], Q, tol)) { s0 = lm.x; s1 = lm.x + lm.y; return li | LEAF_REF; }
            int node = lm.w;
            for (int guard = 0; guard <= KEY_LEVELS && node >= 0 && node < nInt; guard++) {
                const int4 m = T.int_meta[node];
                if (box_holds(B.ibox[node], Q, tol)) { s0 = m.y; s1 = m.z; return node; }
                node = m.w;
            }
        }
    }
    if (root & LEAF_REF) { const int4 lm = T.leaf_meta[root & ~LEAF_REF]; s0 = lm.x; s1 = lm.x + lm.y; }
    else if (root >= 0 && root < nInt) { const int4 m = T.int_meta[root]; s0 = m.y; s1 = m.z; }
    return root;
}

constexpr int COL_SCAN_MAX = 256;    // node runs scanned point by point; larger ones are walked

// Candidates of each particle.  The points of a node are one run of the sorted
// order, so a small enclosing node is scanned without any traversal; the
// count does not depend on the visiting order.  Threads take particles in
// tree order, so neighbouring threads read neighbouring runs.
__global__ void col_count_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root,
                                 const FrameCtl* ctl, CollBufs B) {
    const int n = ctl->n, nInt = min(ctl->nInternal, T.cap_int), nLeaf = ctl->nLeaves, nValid = ctl->nValid;
    const int root = *d_root;
    const float tol = (float)(COL_TOL * fmax(P.rootW, P.rootH));
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = T.tgt[k];
        if (i < 0 || i >= n) { atomicOr(&B.cc->err, COL_ERR_QUERY); continue; }
        QueryP Q;
        int cnt = 0;
        bool multi = false, ok = true;
        if (load_query(S, i, Q)) {
            int s0, s1;
            const int start = query_node(T, B, Q, root, nInt, nLeaf, nValid, nValid, tol, s0, s1);
            if (s1 - s0 <= COL_SCAN_MAX) {
                int lastLeaf = -1;
                for (int q = max(s0, 0); q < min(s1, nValid); q++) {
                    if (!candidate(P, S, T, Q, q, n)) continue;
                    const int lf = T.leaf_of[q];
                    multi |= lf == lastLeaf;
                    lastLeaf = lf;
                    cnt++;
                }
            } else {
                ok = query_leaves(T, B, start, nInt, nLeaf, tol, Q, [&](int li) {
                    const int4 lm = T.leaf_meta[li];
                    if (lm.x < 0 || lm.x + lm.y > nValid) { ok = false; return; }
                    int here = 0;
                    for (int q = lm.x; q < lm.x + lm.y; q++) here += candidate(P, S, T, Q, q, n) ? 1 : 0;
                    cnt += here;
                    multi |= here > 1;
                });
            }
        }
        B.cnt[i] = cnt;
        if (multi) B.cc->need_order = 1;
        if (!ok) atomicOr(&B.cc->err, COL_ERR_QUERY);
    }
}

// Sorted positions of the five earliest-inserted points (smallest insertion
// index T.sidx) kept ascending.
__device__ __forceinline__ void top5_insert(int* best, uint32_t* key, int q, uint32_t k) {
    if (k >= key[4]) return;
    int p = 4;
    while (p > 0 && key[p - 1] > k) { key[p] = key[p - 1]; best[p] = best[p - 1]; p--; }
    key[p] = k; best[p] = q;
}

// Bottom-up pass with arrival counters: the last child to finish merges the
// lists of its siblings into its parent's and climbs on.  Runs only when some
// query met two candidates in one leaf.
__global__ void col_min5_kernel(TreeBufs T, const FrameCtl* ctl, CollBufs B) {
    if (!B.cc->need_order) return;
    const int nLeaf = ctl->nLeaves, nInt = min(ctl->nInternal, T.cap_int), nValid = ctl->nValid;
    for (int li = blockIdx.x * blockDim.x + threadIdx.x; li < nLeaf; li += gridDim.x * blockDim.x) {
        int node = T.leaf_meta[li].w;
        while (node >= 0 && node < nInt) {
            const int4 c = T.int_child[node];
            const int nch = (c.x != -1) + (c.y != -1) + (c.z != -1) + (c.w != -1);
            __threadfence();
            if (atomicAdd(&B.m5cnt[node], 1) != nch - 1) break;
            __threadfence();
            int best[5] = { -1, -1, -1, -1, -1 };
            uint32_t key[5] = { 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu };
            const int ch[4] = { c.x, c.y, c.z, c.w };
            for (int k = 0; k < 4; k++) {
                const int cc = ch[k];
                if (cc == -1) continue;
                if (cc & LEAF_REF) {
                    if ((cc & ~LEAF_REF) >= nLeaf) continue;
                    const int4 lm = T.leaf_meta[cc & ~LEAF_REF];
                    const int e = min(lm.x + lm.y, nValid);
                    for (int q = max(lm.x, 0); q < e; q++) top5_insert(best, key, q, T.sidx[q]);
                } else if (cc > node && cc < nInt) {
                    for (int t = 0; t < 5; t++) {
                        const int q = __ldcg(&B.min5[(size_t)cc * 5 + t]);
                        if (q < 0 || q >= nValid) break;
                        top5_insert(best, key, q, T.sidx[q]);
                    }
                }
            }
            for (int t = 0; t < 5; t++) B.min5[(size_t)node * 5 + t] = best[t];
            node = T.int_meta[node].w;
        }
    }
}

// Storage order of leaf li (at most LEAF_CAP points): walk from the root,
// carrying the arrival prefix R of each node on the path (see the file
// comment).  Returns false for leaves the rule does not cover.
__device__ bool leaf_storage_order(const TreeBufs& T, const CollBufs& B, int root, int li, int nInt, int nLeaf,
                                   int nValid, int* ord, int& cnt) {
    const int4 lm = T.leaf_meta[li];
    const int ls = lm.x, lc = lm.y;
    if (lc > LEAF_CAP || ls < 0 || ls + lc > nValid) return false;
    int R[5];
    int nR = 0;
    if (!(root & LEAF_REF)) {
        int node = root;
        bool reached = false;
        for (int guard = 0; guard < KEY_LEVELS + 2 && !reached; guard++) {
            if (node < 0 || node >= nInt) return false;
            int F[5];
            int nF = 0;
            for (int k = 0; k < nR; k++) F[nF++] = R[k];
            for (int k = 0; k < 5 && nF < 5; k++) {
                const int q = __ldcg(&B.min5[(size_t)node * 5 + k]);
                if (q < 0) break;
                bool inR = false;
                for (int t = 0; t < nR; t++) inR |= R[t] == q;
                if (!inR) F[nF++] = q;
            }
            const int4 c = T.int_child[node];
            const int ch[4] = { c.x, c.y, c.z, c.w };
            int child = -1, cs = 0, ce = 0;
            for (int k = 0; k < 4; k++) {
                const int cc = ch[k];
                if (cc == -1) continue;
                if (cc & LEAF_REF) {
                    if ((cc & ~LEAF_REF) >= nLeaf) return false;
                    const int4 l2 = T.leaf_meta[cc & ~LEAF_REF];
                    if (l2.x == ls) { child = cc; cs = l2.x; ce = l2.x + l2.y; }
                } else if (cc >= 0 && cc < nInt) {
                    const int4 m2 = T.int_meta[cc];
                    if (m2.y <= ls && ls < m2.z) { child = cc; cs = m2.y; ce = m2.z; }
                }
            }
            if (child == -1) return false;
            nR = 0;
            for (int k = nF - 1; k >= 0; k--) if (F[k] >= cs && F[k] < ce) R[nR++] = F[k];
            if (child & LEAF_REF) reached = (child & ~LEAF_REF) == li;
            else node = child;
            if ((child & LEAF_REF) && !reached) return false;
        }
        if (!reached) return false;
    }
    if (nR > lc) return false;
    cnt = 0;
    for (int k = 0; k < nR; k++) ord[cnt++] = R[k];
    // the leaf's other points in insertion order
    for (int pass = 0; pass < lc && cnt < LEAF_CAP; pass++) {
        int pick = -1;
        uint32_t pk = 0xffffffffu;
        for (int q = ls; q < ls + lc; q++) {
            bool used = false;
            for (int t = 0; t < cnt; t++) used |= ord[t] == q;
            if (!used && T.sidx[q] < pk) { pk = T.sidx[q]; pick = q; }
        }
        if (pick < 0) break;
        ord[cnt++] = pick;
    }
    return cnt == lc;
}

// The candidates themselves, in the reference's visiting order: a depth-first
// walk from the enclosing node (only particles that have candidates).
__global__ void col_fill_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root,
                                const FrameCtl* ctl, CollBufs B) {
    const int n = ctl->n, nInt = min(ctl->nInternal, T.cap_int), nLeaf = ctl->nLeaves, nValid = ctl->nValid;
    const int root = *d_root;
    const float tol = (float)(COL_TOL * fmax(P.rootW, P.rootH));
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = T.tgt[k];
        if (i < 0 || i >= n || B.cnt[i] == 0) continue;
        QueryP Q;
        if (!load_query(S, i, Q)) continue;
        int w = B.off[i];
        const int wend = w + B.cnt[i];
        bool ok = true;
        int s0, s1;
        const int start = query_node(T, B, Q, root, nInt, nLeaf, nValid, nValid, tol, s0, s1);
        ok = query_leaves(T, B, start, nInt, nLeaf, tol, Q, [&](int li) {
            const int4 lm = T.leaf_meta[li];
            if (lm.x < 0 || lm.x + lm.y > nValid) { ok = false; return; }
            int buf[COL_LEAF_BUF];
            int nb = 0;
            bool spill = false;
            for (int q = lm.x; q < lm.x + lm.y; q++) {
                if (!candidate(P, S, T, Q, q, n)) continue;
                if (nb < COL_LEAF_BUF) buf[nb++] = q;
                else spill = true;
            }
            if (nb > 1) {                          // a leaf's points in its storage order
                int ord[LEAF_CAP];
                int oc = 0;
                if (!spill && leaf_storage_order(T, B, root, li, nInt, nLeaf, nValid, ord, oc)) {
                    int sorted[COL_LEAF_BUF];
                    int ns = 0;
                    for (int t = 0; t < oc; t++)
                        for (int u = 0; u < nb; u++) if (buf[u] == ord[t] && ns < COL_LEAF_BUF) sorted[ns++] = buf[u];
                    if (ns == nb) for (int u = 0; u < nb; u++) buf[u] = sorted[u];
                    else atomicOr(&B.cc->err, COL_ERR_ORDER);
                } else {
                    atomicOr(&B.cc->err, COL_ERR_ORDER);
                }
            }
            for (int u = 0; u < nb; u++) {
                if (w < wend && w < B.cap) B.cand[w] = make_int2(i, buf[u]);
                w++;
            }
            if (spill) {                           // bucket leaf beyond the buffer: index order
                int kk = 0;
                for (int q = lm.x; q < lm.x + lm.y; q++) {
                    if (!candidate(P, S, T, Q, q, n)) continue;
                    if (kk++ < COL_LEAF_BUF) continue;
                    if (w < wend && w < B.cap) B.cand[w] = make_int2(i, q);
                    w++;
                }
            }
        });
        if (!ok || w != wend) atomicOr(&B.cc->err, COL_ERR_QUERY);
    }
}

// ---- resolution ------------------------------------------------------------------------------
// Rounded step by step like the reference (no fused multiply-add), so that
// equal inputs give equal energies at every call site: a merge that changes
// no velocity then loses exactly zero kinetic energy and emits no event.
__device__ __forceinline__ double ke_of(double m, double wx, double wy) {        // collisions.js:17-20
    const double w2 = __dadd_rn(__dmul_rn(wx, wx), __dmul_rn(wy, wy));
    return __dmul_rn(__ddiv_rn(w2, __dadd_rn(__dsqrt_rn(__dadd_rn(1.0, w2)), 1.0)), m);
}

// Tree record of particle j after its mass changed.  A particle still in the
// list gets the moments computeAllForces re-caches (forces.js:71-76, new body
// radius); a removed one keeps the moments of the last force pass.
__device__ void patch_record(const DevState& S, const TreeBufs& T, const CollBufs& B, int j, bool removed) {
    const int s = B.inv[j];
    if (s < 0) return;
    const float4 p = S.pos[j];
    float4 a = T.ps_a[s];
    a.z = p.z;
    T.ps_a[s] = a;
    float4 c = T.ps_c[s];
    if (removed) {
        const float2 mo = S.mom[j];
        c.y = mo.x; c.z = mo.y;
    } else {
        const float rad = S.spin[j].z, rsq = rad * rad;
        c.y = MAG_MOMENT_K * p.w * c.x * rsq;
        c.z = INERTIA_K * p.z * c.x * rsq;
    }
    T.ps_c[s] = c;
}

// Particle.updateColor outside black-hole mode (particle.js:110-121): body
// radius from the mass.  A particle at mass 0 leaves the list this substep.
__device__ void set_mass(const DevState& S, int j, double m) {
    float4 p = S.pos[j];
    p.z = (float)m;
    S.pos[j] = p;
    float4 sp = S.spin[j];
    sp.z = (float)cbrt(m);
    sp.w = m > 0 ? (float)(1.0 / m) : 0.f;
    S.spin[j] = sp;
}

// topology.js:81-135 in FP64, with the velocity / spin flips of the
// non-orientable topologies.
__device__ void wrap_d(const DevParams& P, double& x, double& y, double& wx, double& wy, double& vx, double& vy,
                       double& angw, double& angVel) {
    const double W = P.Wd, H = P.Hd;
    if (P.topology == GEON_TORUS) {
        if (x < 0) x += W; else if (x > W) x -= W;
        if (y < 0) y += H; else if (y > H) y -= H;
        return;
    }
    if (P.topology == GEON_KLEIN) {
        if (x < 0) x += W; else if (x > W) x -= W;
        if (y < 0 || y > H) {
            y += (y < 0) ? H : -H;
            x = W - x;
            wx = -wx; vx = -vx; angw = -angw; angVel = -angVel;
        }
        return;
    }
    for (int it = 0; it < 2; it++) {
        bool wrapped = false;
        if (x < 0 || x > W) {
            x += (x < 0) ? W : -W;
            y = H - y;
            wy = -wy; vy = -vy; angw = -angw; angVel = -angVel;
            wrapped = true;
        }
        if (y < 0 || y > H) {
            y += (y < 0) ? H : -H;
            x = W - x;
            wx = -wx; vx = -vx; angw = -angw; angVel = -angVel;
            wrapped = true;
        }
        if (!wrapped) break;
    }
}

// The merged particle, as Simulation.addParticle builds it and the
// integrator then overrides it (main.js:504-523, integrator.js:1363-1381):
// charge rounded to a multiple of BOSON_CHARGE, proper velocity and spin set
// directly, creation time now, no history, zero forces; wrapped when periodic.
__device__ void write_spawn(const DevParams& P, const DevState& S, int slot, double x, double y, double wx, double wy,
                            double M, double base, double q, double angw, bool anti, double ctime, int id) {
    const double r = cbrt(M);
    double angVel = P.rel ? angw / sqrt(1 + angw * angw * r * r) : angw;
    const double invG = P.rel ? 1 / sqrt(1 + wx * wx + wy * wy) : 1.0;
    double vx = wx * invG, vy = wy * invG;
    if (P.periodic) wrap_d(P, x, y, wx, wy, vx, vy, angw, angVel);
    const double cq = q / 0.1;                                   // Math.round(q / BOSON_CHARGE): nearest, ties up
    double rq = floor(cq);
    if (cq - rq >= 0.5) rq += 1;
    const float xh = (float)x, yh = (float)y;
    const float mf = (float)M;
    S.pos[slot] = make_float4(xh, yh, mf, (float)(rq * 0.1));
    S.pos_lo[slot] = make_float2((float)(x - (double)xh), (float)(y - (double)yh));
    S.vel[slot] = make_float4((float)wx, (float)wy, (float)vx, (float)vy);
    S.spin[slot] = make_float4((float)angw, (float)angVel, (float)r, 1.f / mf);
    S.mom[slot] = make_float2(0.f, 0.f);
    S.force[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    S.grad[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    S.torque[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    S.f1pn[slot] = make_float2(0.f, 0.f);
    S.f1pnOld[slot] = make_float2(0.f, 0.f);
    S.ctime[slot] = ctime;
    S.id[slot] = id;
    S.hist_cnt[slot] = 0;
    S.matter[slot] = make_float2((float)base, anti ? 1.f : 0.f);
    for (int rr = 0; rr < 12; rr++) S.brk[(size_t)rr * P.n_cap + slot] = 0.f;
}

// Merged particle of pair (ci, j) (collisions.js:110-158) from the masses,
// base masses and radii the pair had when it was resolved, and the fields no
// collision changes (position, proper velocity, spin, charge, matter type).
struct Merged { double x, y, wx, wy, M, base, q, angw, keLost; bool anti; };
__device__ Merged merged_of(const DevState& S, int ci, int j, double bx, double by, double dx, double dy,
                            const PairRec& R) {
    const float4 v1 = S.vel[ci], v2 = S.vel[j];
    const double m1 = R.m1, m2 = R.m2, r1 = R.r1, r2 = R.r2;
    Merged G;
    G.M = m1 + m2;
    G.wx = (m1 * v1.x + m2 * v2.x) / G.M;
    G.wy = (m1 * v1.y + m2 * v2.y) / G.M;
    const double p2x = bx + dx, p2y = by + dy;
    G.x = (bx * m1 + p2x * m2) / G.M;
    G.y = (by * m1 + p2y * m2) / G.M;
    const double dx1 = bx - G.x, dy1 = by - G.y, dx2 = p2x - G.x, dy2 = p2y - G.y;
    const double lorb = dx1 * (m1 * v1.y) - dy1 * (m1 * v1.x) + dx2 * (m2 * v2.y) - dy2 * (m2 * v2.x);
    const double lspin = 0.4 * m1 * r1 * r1 * S.spin[ci].x + 0.4 * m2 * r2 * r2 * S.spin[j].x;
    const double nr = cbrt(G.M);
    const double nI = 0.4 * G.M * nr * nr;
    G.angw = nI > EPS_D ? (lorb + lspin) / nI : 0.0;
    G.base = (double)R.b1 + (double)R.b2;
    G.q = (double)S.pos[ci].w + (double)S.pos[j].w;
    G.anti = S.matter[ci].y != 0.f;
    G.keLost = fmax(0.0, ke_of(m1, v1.x, v1.y) + ke_of(m2, v2.x, v2.y) - ke_of(G.M, G.wx, G.wy));
    return G;
}

// Geometry of candidate e: the position of particle ci and the minimum-image
// offset to the tree point (a ghost's image position for ghosts).
__device__ __forceinline__ void pair_geometry(const DevParams& P, const DevState& S, const TreeBufs& T, int ci, int q,
                                              double& bx, double& by, double& qx, double& qy, double& dx, double& dy) {
    const float4 p = S.pos[ci];
    const float2 pl = S.pos_lo[ci];
    bx = (double)p.x + pl.x;
    by = (double)p.y + pl.y;
    qx = point_x(T, q);
    qy = point_y(T, q);
    if (P.periodic) min_image_d(bx, by, qx, qy, P.topology, P.Wd, P.Hd, dx, dy);
    else { dx = qx - bx; dy = qy - by; }
}

// ---- components: pairs that share no particle commute -------------------------------------------
__device__ int uf_find(int* par, int x) {
    volatile int* p = par;
    for (int it = 0; it < (1 << 24); it++) {          // a chain is shorter than the particle count
        const int px = p[x];
        if (px == x) return x;
        const int ppx = p[px];
        if (ppx != px) p[x] = ppx;                       // path halving: links only move up
        x = ppx;
    }
    return -1;
}

__global__ void col_uf_init_kernel(CollBufs B, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) B.uf[i] = i;
}

__device__ __forceinline__ int pair_other(const TreeBufs& T, int q) { return (int)ref_index(__float_as_uint(T.ps_c[q].w)); }

__global__ void col_union_kernel(TreeBufs T, CollBufs B, int n, int total) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int2 cd = B.cand[e];
        if (cd.y < 0 || cd.y >= T.cap_pts) continue;
        const int j = pair_other(T, cd.y);
        if (cd.x < 0 || cd.x >= n || j < 0 || j >= n) continue;
        int a = cd.x, b = j;
        for (int it = 0; it < (1 << 20); it++) {
            a = uf_find(B.uf, a);
            b = uf_find(B.uf, b);
            if (a < 0 || b < 0) { atomicOr(&B.cc->err, COL_ERR_QUERY); break; }
            if (a == b) break;
            if (a < b) { const int t = a; a = b; b = t; }   // the larger root goes under the smaller
            if (atomicCAS(&B.uf[a], a, b) == a) break;
        }
    }
}

// Sort keys (component << 32 | e): a stable sort groups each component's
// pairs and keeps them in the sequential order.
__global__ void col_key_kernel(TreeBufs T, CollBufs B, int n, int total, int serial) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        uint32_t comp = 0;
        if (!serial) {
            const int ci = B.cand[e].x;
            const int r = (ci >= 0 && ci < n) ? uf_find(B.uf, ci) : 0;
            comp = (uint32_t)max(r, 0);
        }
        B.skey[e] = ((uint64_t)comp << 32) | (uint32_t)e;
        B.sval[e] = (uint32_t)e;
    }
}

// handleCollisions' loop body (collisions.js:35-92), restricted to one
// component and run by one thread in the sequential order; the outcome of
// every pair is recorded for the ordered output pass.
__global__ void col_resolve_kernel(DevParams P, DevState S, TreeBufs T, const FrameCtl* ctl, CollBufs B,
                                   const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, int n, int total) {
    const int nValid = ctl->nValid;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const uint32_t comp = (uint32_t)(keys[t] >> 32);
        if (t > 0 && (uint32_t)(keys[t - 1] >> 32) == comp) continue;       // not the first pair of a component
        int cur = -1;
        bool skip = true;
        double br = 0;
        for (int u = t; u < total && (uint32_t)(keys[u] >> 32) == comp; u++) {
            const int e = (int)vals[u];
            if (e < 0 || e >= total) continue;
            B.kind[e] = PAIR_NONE;
            B.sflag[e] = 0;
            B.eflag[e] = 0;
            const int2 cd = B.cand[e];
            const int ci = cd.x, q = cd.y;
            if (ci < 0 || ci >= n || q < 0 || q >= nValid) continue;
            if (ci != cur) {                                     // start of particle ci's turn
                cur = ci;
                skip = S.pos[ci].z == 0.f;
                br = 2.0 * (double)S.spin[ci].z;
            }
            if (skip) continue;
            double bx, by, qx, qy, dx, dy;
            pair_geometry(P, S, T, ci, q, bx, by, qx, qy, dx, dy);
            if (qx < bx - br || qx > bx + br || qy < by - br || qy > by + br) continue;
            const int j = pair_other(T, q);
            if (j == ci || j < 0 || j >= n) continue;
            const float4 p1 = S.pos[ci], p2 = S.pos[j];
            if (p2.z == 0.f || S.id[ci] >= S.id[j]) continue;
            const float4 s1 = S.spin[ci], s2 = S.spin[j];
            const double md = (double)s1.z + (double)s2.z;
            if (!(dx * dx + dy * dy < md * md)) continue;
            float2 mt1 = S.matter[ci], mt2 = S.matter[j];
            const PairRec R{ p1.z, p2.z, mt1.x, mt2.x, s1.z, s2.z };
            B.rec[e] = R;
            const double m1 = p1.z, m2 = p2.z;
            if ((mt1.y != 0.f) != (mt2.y != 0.f)) {              // annihilation, collisions.js:60-80
                B.kind[e] = PAIR_ANNIHILATE;
                B.eflag[e] = 1;
                const double a = fmin(m1, m2);
                const double n1 = m1 - a, n2 = m2 - a;
                if (m1 > 0) mt1.x = (float)((double)mt1.x * (n1 / m1));
                if (m2 > 0) mt2.x = (float)((double)mt2.x * (n2 / m2));
                S.matter[ci] = mt1;
                S.matter[j] = mt2;
                set_mass(S, ci, n1);
                set_mass(S, j, n2);
                patch_record(S, T, B, ci, n1 == 0);
                patch_record(S, T, B, j, n2 == 0);
            } else {                                             // merge, collisions.js:81-91
                B.kind[e] = PAIR_MERGE;
                B.sflag[e] = 1;
                B.eflag[e] = merged_of(S, ci, j, bx, by, dx, dy, R).keLost > 0 ? 1 : 0;
                float4 a1 = p1, a2 = p2;
                a1.z = 0.f; a2.z = 0.f;                          // both die; charge, radius, velocity stay
                S.pos[ci] = a1;
                S.pos[j] = a2;
                mt1.x = 0.f; mt2.x = 0.f;
                S.matter[ci] = mt1;
                S.matter[j] = mt2;
                patch_record(S, T, B, ci, true);
                patch_record(S, T, B, j, true);
            }
        }
    }
}

// Ordered output: spawns take slots n + rank and ids id0 + rank, events go
// to the frame's list, both in the sequential order of their pairs.
__global__ void col_emit_kernel(DevParams P, DevState S, TreeBufs T, CollBufs B, int n, int total, int slots,
                                double simTime, int id0) {
    const int base = B.cc->events;
    int ann = 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int kind = B.kind[e];
        if (kind == PAIR_NONE) continue;
        const int2 cd = B.cand[e];
        const int ci = cd.x, q = cd.y, j = pair_other(T, q);
        double bx, by, qx, qy, dx, dy;
        pair_geometry(P, S, T, ci, q, bx, by, qx, qy, dx, dy);
        const PairRec R = B.rec[e];
        const int ev = base + B.epos[e];
        double* o = (B.eflag[e] && ev < COL_EVENT_CAP) ? B.events + (size_t)ev * 6 : nullptr;
        if (kind == PAIR_ANNIHILATE) {
            ann++;
            const float4 v1 = S.vel[ci], v2 = S.vel[j];
            const double m1 = R.m1, m2 = R.m2;
            const double a = fmin(m1, m2);
            const double f1 = a / m1, f2 = a / m2;               // 0/0 for a particle that already merged away
            if (o) {
                o[0] = 1.0; o[1] = bx + dx * 0.5; o[2] = by + dy * 0.5;
                o[3] = 2 * a + (f1 * ke_of(m1, v1.x, v1.y) + f2 * ke_of(m2, v2.x, v2.y));
                o[4] = ((double)v1.x + (double)v2.x) * a; o[5] = ((double)v1.y + (double)v2.y) * a;
            }
        } else {
            const Merged G = merged_of(S, ci, j, bx, by, dx, dy, R);
            const int rank = B.spos[e];
            const int slot = n + rank;
            if (slot >= slots) { atomicOr(&B.cc->err, COL_ERR_SLOTS); continue; }
            write_spawn(P, S, slot, G.x, G.y, G.wx, G.wy, G.M, G.base, G.q, G.angw, G.anti, simTime, id0 + rank);
            if (o) { o[0] = 2.0; o[1] = G.x; o[2] = G.y; o[3] = G.keLost; o[4] = 0.0; o[5] = 0.0; }
        }
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) ann += __shfl_xor_sync(0xffffffffu, ann, s);
    if ((threadIdx.x & 31) == 0 && ann) atomicAdd(&B.cc->annihilations, ann);
}

__global__ void col_finish_kernel(CollBufs B) {
    CollCtl* cc = B.cc;
    cc->spawned = cc->stotal;
    cc->merges = cc->stotal;
    const int e = cc->events + cc->etotal;
    if (e > COL_EVENT_CAP) { cc->events_dropped += e - COL_EVENT_CAP; cc->events = COL_EVENT_CAP; }
    else cc->events = e;
}

// Keep flags for the compaction after the pass (collisions.js:96-104 keeps
// mass != 0) and the spawns; counts the removed particles.
__global__ void col_keep_kernel(DevState S, CollBufs B, int* keep, int n) {
    const int spawned = B.cc->spawned;
    const bool any = spawned + B.cc->annihilations > 0;
    int removed = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n + spawned; i += gridDim.x * blockDim.x) {
        int k = 1;
        if (i < n && any && S.pos[i].z == 0.f) k = 0;
        keep[i] = k;
        removed += 1 - k;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) removed += __shfl_xor_sync(0xffffffffu, removed, o);
    if ((threadIdx.x & 31) == 0 && removed) atomicAdd(&B.cc->removed, removed);
}

// ---- target list for the force pass after the collisions ---------------------------------------
// The walk takes its targets 32 at a time, and a warp is fast when its 32
// particles are neighbours.  So the list keeps the tree order without the
// removed particles, and each spawn takes the place of the particle it
// replaced (the first of its pair, which always dies): the spawns of one
// particle follow each other there in spawn order.
__global__ void col_tflag_kernel(DevState S, TreeBufs T, CollBufs B, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = T.tgt[k];
        const bool okI = i >= 0 && i < n;
        B.tflag[k] = (okI && S.pos[i].z != 0.f) ? 1 : 0;
        if (okI) B.tk[i] = k;
        B.acnt[k] = 0;
        B.amin[k] = 0x7fffffff;
    }
}

__global__ void col_anchor_kernel(CollBufs B, int n, int total) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        if (B.kind[e] != PAIR_MERGE) continue;
        const int ci = B.cand[e].x;
        if (ci < 0 || ci >= n) continue;
        const int a = B.tk[ci], r = B.spos[e];
        if (a < 0 || a >= n || r < 0 || r >= total) continue;
        B.anch[r] = a;
        atomicAdd(&B.acnt[a], 1);
        atomicMin(&B.amin[a], r);
    }
}

__global__ void col_tgt_kernel(TreeBufs T, CollBufs B, int n, int spawned) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n + spawned; k += gridDim.x * blockDim.x) {
        if (k < n) {
            if (B.tflag[k]) B.tgt2[B.tpos[k] + B.abefore[k]] = T.tgt[k];
        } else {
            const int t = k - n, a = B.anch[t];
            if (a < 0 || a >= n) continue;
            const int at = B.tpos[a] + B.abefore[a] + (t - B.amin[a]);
            if (at >= 0 && at < 2 * n) B.tgt2[at] = k;
        }
    }
}

// ---- launchers ------------------------------------------------------------------------------
void collide_detect(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                    const CollBufs& B, int n_cap, cudaStream_t st, LaunchCounter& lc) {
    col_begin_kernel<<<1, 1, 0, st>>>(B.cc);
    cudaMemsetAsync(B.inv, 0xff, (size_t)n_cap * sizeof(int), st);
    cudaMemsetAsync(B.m5cnt, 0, (size_t)T.cap_int * sizeof(int), st);
    col_inverse_kernel<<<grid_for(T.cap_pts, 256), 256, 0, st>>>(T, ctl, B);
    col_geo_kernel<<<grid_for(T.cap_int + T.cap_pts, 256), 256, 0, st>>>(P, T, ctl, B);
    col_count_kernel<<<grid_for(n_cap, 128), 128, 0, st>>>(P, S, T, d_root, ctl, B);
    exclusive_scan(B.cnt, B.off, n_cap, &ctl->n, &B.cc->total, B.scan_tmp, st, &lc);
    col_min5_kernel<<<grid_for(T.cap_pts, 256), 256, 0, st>>>(T, ctl, B);
    col_fill_kernel<<<grid_for(n_cap, 128), 128, 0, st>>>(P, S, T, d_root, ctl, B);
    lc.add(6);
}

void collide_resolve(const DevParams& P, const DevState& S, const TreeBufs& T, const FrameCtl* ctl, const CollBufs& B,
                     int* keep, int n, int total, int slots, double sim_time, int id0, cudaStream_t st, LaunchCounter& lc) {
    if (total > 0) {
        const bool serial = total <= COL_SERIAL_MAX;
        const int g = grid_for(total, 256);
        if (!serial) {
            col_uf_init_kernel<<<grid_for(n, 256), 256, 0, st>>>(B, n);
            col_union_kernel<<<g, 256, 0, st>>>(T, B, n, total);
            lc.add(2);
        }
        col_key_kernel<<<g, 256, 0, st>>>(T, B, n, total, serial ? 1 : 0);
        lc.add(1);
        const uint64_t* keys = B.skey;
        const uint32_t* vals = B.sval;
        if (!serial && radix_sort_pairs(B.skey, B.sval, B.skey_alt, B.sval_alt, total, &B.cc->total, B.sort_bits,
                                        B.sort_tmp, st, &lc)) {
            keys = B.skey_alt;
            vals = B.sval_alt;
        }
        col_resolve_kernel<<<serial ? 1 : grid_for(total, 128), serial ? 32 : 128, 0, st>>>(P, S, T, ctl, B, keys, vals,
                                                                                           n, total);
        exclusive_scan(B.sflag, B.spos, total, nullptr, &B.cc->stotal, B.scan_tmp, st, &lc);
        exclusive_scan(B.eflag, B.epos, total, nullptr, &B.cc->etotal, B.scan_tmp, st, &lc);
        col_emit_kernel<<<g, 256, 0, st>>>(P, S, T, B, n, total, slots, sim_time, id0);
        col_finish_kernel<<<1, 1, 0, st>>>(B);
        lc.add(3);
    }
    col_keep_kernel<<<grid_for(2 * n + 1, 256), 256, 0, st>>>(S, B, keep, n);
    lc.add(1);
}

void collide_targets(const DevState& S, const TreeBufs& T, FrameCtl* ctl, const CollBufs& B, int n, int total,
                     int spawned, int n_cap, cudaStream_t st, LaunchCounter& lc) {
    cudaMemsetAsync(B.anch, 0xff, (size_t)std::max(spawned, 1) * sizeof(int), st);
    col_tflag_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(S, T, B, n);
    col_anchor_kernel<<<grid_for(std::max(total, 1), 256), 256, 0, st>>>(B, n, total);
    exclusive_scan(B.tflag, B.tpos, n_cap, &ctl->n, &B.cc->nlive, B.scan_tmp, st, &lc);
    exclusive_scan(B.acnt, B.abefore, n_cap, &ctl->n, nullptr, B.scan_tmp, st, &lc);
    col_tgt_kernel<<<grid_for(n + spawned, 256), 256, 0, st>>>(T, B, n, spawned);
    lc.add(3);
}

}  // namespace geon
