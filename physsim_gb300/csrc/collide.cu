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
    return b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b);
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

// Depth-first box query (quadtree.js:372-404): internal nodes whose region
// meets the closed box [bx - r, bx + r] x [by - r, by + r] are opened, children
// pushed NW, NE, SW, SE; `leaf(li)` is called for every leaf reached, in the
// reference's visiting order.  Node regions come from the first key of the
// node's run and are widened by 1e-9 of the root size: a node visited in
// excess only costs time, its points are tested one by one.
template <class F>
__device__ bool query_leaves(const DevParams& P, const TreeBufs& T, int root, int nInt, int nLeaf, int nValid,
                             double bx, double by, double r, F&& leaf) {
    if (root == ROOT_NONE) return true;
    int stack[COL_STACK];
    int top = 0;
    stack[top++] = root;
    const double loX = P.rootX - P.rootW, loY = P.rootY - P.rootH;
    const double dX = P.rootW * (1.0 / 1073741824.0), dY = P.rootH * (1.0 / 1073741824.0);
    const double tolX = 1e-9 * P.rootW, tolY = 1e-9 * P.rootH;
    while (top > 0) {
        const int node = stack[--top];
        if (node & LEAF_REF) {
            const int li = node & ~LEAF_REF;
            if (li < 0 || li >= nLeaf) return false;
            leaf(li);
            continue;
        }
        if (node < 0 || node >= nInt) return false;
        const int4 m = T.int_meta[node];
        const int sh = KEY_LEVELS - m.x;
        if (m.x < 0 || sh < 0 || m.y < 0 || m.y >= nValid) return false;
        const uint64_t K = T.skey[m.y];
        const double span = ldexp(1.0, sh);
        const double x0 = loX + (double)((unzip_axis(K, 0) >> sh) << sh) * dX;
        const double y0 = loY + (double)((unzip_axis(K, 1) >> sh) << sh) * dY;
        const double x1 = x0 + span * dX, y1 = y0 + span * dY;
        if (bx - r > x1 + tolX || bx + r < x0 - tolX || by - r > y1 + tolY || by + r < y0 - tolY) continue;
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
// radii (collisions.js:37-57).
struct QueryP { double x, y, r; int i, id; float rad; };

__device__ __forceinline__ bool candidate(const DevParams& P, const DevState& S, const TreeBufs& T, const QueryP& Q,
                                          int q, int n) {
    const double x = point_x(T, q), y = point_y(T, q);
    if (x < Q.x - Q.r || x > Q.x + Q.r || y < Q.y - Q.r || y > Q.y + Q.r) return false;
    const int j = (int)ref_index(__float_as_uint(T.ps_c[q].w));
    if (j == Q.i || j < 0 || j >= n) return false;
    if (S.pos[j].z == 0.f) return false;
    if (Q.id >= S.id[j]) return false;
    double dx, dy;
    if (P.periodic) min_image_d(Q.x, Q.y, x, y, P.topology, P.Wd, P.Hd, dx, dy);
    else { dx = x - Q.x; dy = y - Q.y; }
    const double md = (double)Q.rad + (double)S.spin[j].z;
    return dx * dx + dy * dy < md * md;
}

__device__ __forceinline__ bool load_query(const DevState& S, int i, QueryP& Q) {
    const float4 p = S.pos[i];
    if (p.z == 0.f) return false;
    const float2 pl = S.pos_lo[i];
    Q.x = (double)p.x + pl.x;
    Q.y = (double)p.y + pl.y;
    Q.rad = S.spin[i].z;
    Q.r = 2.0 * (double)Q.rad;                     // queryReuse(root, x, y, 2r, 2r)
    Q.i = i;
    Q.id = S.id[i];
    return true;
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

__global__ void col_count_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root,
                                 const FrameCtl* ctl, CollBufs B) {
    const int n = ctl->n, nInt = min(ctl->nInternal, T.cap_int), nLeaf = ctl->nLeaves, nValid = ctl->nValid;
    const int root = *d_root;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        QueryP Q;
        int cnt = 0;
        bool multi = false, ok = true;
        if (load_query(S, i, Q)) {
            ok = query_leaves(P, T, root, nInt, nLeaf, nValid, Q.x, Q.y, Q.r, [&](int li) {
                const int4 lm = T.leaf_meta[li];
                if (lm.x < 0 || lm.x + lm.y > nValid) { ok = false; return; }
                int here = 0;
                for (int q = lm.x; q < lm.x + lm.y; q++) here += candidate(P, S, T, Q, q, n) ? 1 : 0;
                cnt += here;
                multi |= here > 1;
            });
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

__global__ void col_fill_kernel(DevParams P, DevState S, TreeBufs T, const int* __restrict__ d_root,
                                const FrameCtl* ctl, CollBufs B) {
    const int n = ctl->n, nInt = min(ctl->nInternal, T.cap_int), nLeaf = ctl->nLeaves, nValid = ctl->nValid;
    const int root = *d_root;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (B.cnt[i] == 0) continue;
        QueryP Q;
        if (!load_query(S, i, Q)) continue;
        int w = B.off[i];
        const int wend = w + B.cnt[i];
        bool ok = true;
        ok = query_leaves(P, T, root, nInt, nLeaf, nValid, Q.x, Q.y, Q.r, [&](int li) {
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
            if (nb > 1) {
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
            if (spill) {                       // bucket leaf beyond the buffer: index order
                int k = 0;
                for (int q = lm.x; q < lm.x + lm.y; q++) {
                    if (!candidate(P, S, T, Q, q, n)) continue;
                    if (k++ < COL_LEAF_BUF) continue;
                    if (w < wend && w < B.cap) B.cand[w] = make_int2(i, q);
                    w++;
                }
            }
        });
        if (!ok || w != wend) atomicOr(&B.cc->err, COL_ERR_QUERY);
    }
}

// ---- sequential resolution ------------------------------------------------------------------
// Rounded step by step like the reference (no fused multiply-add), so that
// equal inputs give equal energies at every call site: a merge that changes
// no velocity then loses exactly zero kinetic energy and emits no event.
__device__ __forceinline__ double ke_of(double m, double wx, double wy) {        // collisions.js:17-20
    const double w2 = __dadd_rn(__dmul_rn(wx, wx), __dmul_rn(wy, wy));
    return __dmul_rn(__ddiv_rn(w2, __dadd_rn(__dsqrt_rn(__dadd_rn(1.0, w2)), 1.0)), m);
}

__device__ void put_event(const CollBufs& B, double type, double x, double y, double e, double px, double py) {
    const int k = B.cc->events;
    if (k >= COL_EVENT_CAP) { B.cc->events_dropped++; return; }
    double* o = B.events + (size_t)k * 6;
    o[0] = type; o[1] = x; o[2] = y; o[3] = e; o[4] = px; o[5] = py;
    B.cc->events = k + 1;
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

// One thread walks the candidates in order: collisions.js:35-92.
__global__ void col_resolve_kernel(DevParams P, DevState S, TreeBufs T, const FrameCtl* ctl, CollBufs B, int n,
                                   int slots, double simTime, int id0) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int nValid = ctl->nValid;
    CollCtl* cc = B.cc;
    const int total = cc->total;
    if (total > B.cap) { cc->err |= COL_ERR_CAND_OVERFLOW; return; }
    if (cc->err & COL_ERR_QUERY) return;
    int spawned = 0, merges = 0, ann = 0;
    int cur = -1;
    bool skip = true;
    double bx = 0, by = 0, br = 0;
    for (int e = 0; e < total; e++) {
        const int2 cd = B.cand[e];
        const int ci = cd.x, q = cd.y;
        if (ci < 0 || ci >= n || q < 0 || q >= nValid) continue;
        if (ci != cur) {                                         // start of particle ci's turn
            cur = ci;
            const float4 p = S.pos[ci];
            skip = p.z == 0.f;
            if (!skip) {
                const float2 pl = S.pos_lo[ci];
                bx = (double)p.x + pl.x;
                by = (double)p.y + pl.y;
                br = 2.0 * (double)S.spin[ci].z;
            }
        }
        if (skip) continue;
        const double qx = point_x(T, q), qy = point_y(T, q);
        if (qx < bx - br || qx > bx + br || qy < by - br || qy > by + br) continue;
        const int j = (int)ref_index(__float_as_uint(T.ps_c[q].w));
        if (j == ci || j < 0 || j >= n) continue;
        const float4 p1 = S.pos[ci], p2 = S.pos[j];
        if (p2.z == 0.f || S.id[ci] >= S.id[j]) continue;
        double dx, dy;
        if (P.periodic) min_image_d(bx, by, qx, qy, P.topology, P.Wd, P.Hd, dx, dy);
        else { dx = qx - bx; dy = qy - by; }
        const float4 s1 = S.spin[ci], s2 = S.spin[j];
        const double r1 = s1.z, r2 = s2.z;
        const double md = r1 + r2;
        if (!(dx * dx + dy * dy < md * md)) continue;
        float2 mt1 = S.matter[ci], mt2 = S.matter[j];
        const float4 v1 = S.vel[ci], v2 = S.vel[j];
        const double m1 = p1.z, m2 = p2.z;
        const double ke1 = ke_of(m1, v1.x, v1.y), ke2 = ke_of(m2, v2.x, v2.y);
        if ((mt1.y != 0.f) != (mt2.y != 0.f)) {                  // annihilation, collisions.js:60-80
            const double a = fmin(m1, m2);
            const double f1 = a / m1, f2 = a / m2;
            put_event(B, 1.0, bx + dx * 0.5, by + dy * 0.5, 2 * a + (f1 * ke1 + f2 * ke2),
                      ((double)v1.x + (double)v2.x) * a, ((double)v1.y + (double)v2.y) * a);
            ann++;
            const double n1 = m1 - a, n2 = m2 - a;
            if (m1 > 0) mt1.x = (float)((double)mt1.x * (n1 / m1));
            if (m2 > 0) mt2.x = (float)((double)mt2.x * (n2 / m2));
            S.matter[ci] = mt1;
            S.matter[j] = mt2;
            set_mass(S, ci, n1);
            set_mass(S, j, n2);
            patch_record(S, T, B, ci, n1 == 0);
            patch_record(S, T, B, j, n2 == 0);
        } else {                                                 // merge, collisions.js:81-91, 110-158
            const int slot = n + spawned;
            if (slot >= slots) { cc->err |= COL_ERR_SLOTS; break; }
            const double M = m1 + m2;
            const double nwx = (m1 * v1.x + m2 * v2.x) / M, nwy = (m1 * v1.y + m2 * v2.y) / M;
            const double p2x = bx + dx, p2y = by + dy;
            const double nx = (bx * m1 + p2x * m2) / M, ny = (by * m1 + p2y * m2) / M;
            const double dx1 = bx - nx, dy1 = by - ny, dx2 = p2x - nx, dy2 = p2y - ny;
            const double lorb = dx1 * (m1 * v1.y) - dy1 * (m1 * v1.x) + dx2 * (m2 * v2.y) - dy2 * (m2 * v2.x);
            const double lspin = 0.4 * m1 * r1 * r1 * s1.x + 0.4 * m2 * r2 * r2 * s2.x;
            const double nr = cbrt(M);
            const double nI = 0.4 * M * nr * nr;
            const double nangw = nI > EPS_D ? (lorb + lspin) / nI : 0.0;
            const double keLost = fmax(0.0, ke1 + ke2 - ke_of(M, nwx, nwy));
            if (keLost > 0) put_event(B, 2.0, nx, ny, keLost, 0.0, 0.0);
            const double base = (double)mt1.x + (double)mt2.x;
            const double qsum = (double)p1.w + (double)p2.w;
            const bool anti = mt1.y != 0.f;
            float4 a1 = p1, a2 = p2;
            a1.z = 0.f; a2.z = 0.f;                              // both die; charge, radius, velocity stay
            S.pos[ci] = a1;
            S.pos[j] = a2;
            mt1.x = 0.f; mt2.x = 0.f;
            S.matter[ci] = mt1;
            S.matter[j] = mt2;
            patch_record(S, T, B, ci, true);
            patch_record(S, T, B, j, true);
            write_spawn(P, S, slot, nx, ny, nwx, nwy, M, base, qsum, nangw, anti, simTime, id0 + spawned);
            spawned++;
            merges++;
        }
    }
    cc->spawned = spawned;
    cc->merges = merges;
    cc->annihilations = ann;
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
__global__ void col_tflag_kernel(DevState S, TreeBufs T, CollBufs B, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = T.tgt[k];
        B.tflag[k] = (i >= 0 && i < n && S.pos[i].z != 0.f) ? 1 : 0;
    }
}

__global__ void col_tgt_kernel(TreeBufs T, CollBufs B, int n, int spawned) {
    const int nlive = B.cc->nlive;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n + spawned; k += gridDim.x * blockDim.x) {
        if (k < n) { if (B.tflag[k]) B.tgt2[B.tpos[k]] = T.tgt[k]; }
        else B.tgt2[nlive + (k - n)] = k;
    }
}

// ---- launchers ------------------------------------------------------------------------------
void collide_detect(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                    const CollBufs& B, int n_cap, cudaStream_t st, LaunchCounter& lc) {
    col_begin_kernel<<<1, 1, 0, st>>>(B.cc);
    cudaMemsetAsync(B.inv, 0xff, (size_t)n_cap * sizeof(int), st);
    cudaMemsetAsync(B.m5cnt, 0, (size_t)T.cap_int * sizeof(int), st);
    col_inverse_kernel<<<grid_for(T.cap_pts, 256), 256, 0, st>>>(T, ctl, B);
    col_count_kernel<<<grid_for(n_cap, 128), 128, 0, st>>>(P, S, T, d_root, ctl, B);
    exclusive_scan(B.cnt, B.off, n_cap, &ctl->n, &B.cc->total, B.scan_tmp, st, &lc);
    col_min5_kernel<<<grid_for(T.cap_pts, 256), 256, 0, st>>>(T, ctl, B);
    col_fill_kernel<<<grid_for(n_cap, 128), 128, 0, st>>>(P, S, T, d_root, ctl, B);
    lc.add(5);
}

void collide_resolve(const DevParams& P, const DevState& S, const TreeBufs& T, const FrameCtl* ctl, const CollBufs& B,
                     int* keep, int n, int slots, double sim_time, int id0, int n_cap, cudaStream_t st, LaunchCounter& lc) {
    col_resolve_kernel<<<1, 32, 0, st>>>(P, S, T, ctl, B, n, slots, sim_time, id0);
    col_keep_kernel<<<grid_for(2 * n_cap, 256), 256, 0, st>>>(S, B, keep, n);
    lc.add(2);
}

void collide_targets(const DevState& S, const TreeBufs& T, FrameCtl* ctl, const CollBufs& B, int n, int spawned,
                     int n_cap, cudaStream_t st, LaunchCounter& lc) {
    col_tflag_kernel<<<grid_for(n_cap, 256), 256, 0, st>>>(S, T, B, n);
    exclusive_scan(B.tflag, B.tpos, n_cap, &ctl->n, &B.cc->nlive, B.scan_tmp, st, &lc);
    col_tgt_kernel<<<grid_for(n + spawned, 256), 256, 0, st>>>(T, B, n, spawned);
    lc.add(2);
}

}  // namespace geon
