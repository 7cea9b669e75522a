// tree.cu — quadtree build from radix-sorted Morton keys.
//
// Reproduces the node membership of QuadTreePool (src/quadtree.js:13-312,
// 412-419) built as Physics._buildTree does (src/integrator.js:247-260):
//  * root box centre (offX + W/2, offY + H/2), half-size (2W, 2H)
//    (integrator.js:727-730); points outside the closed box are dropped
//    (quadtree.js:186);
//  * a point goes to child NW/NE/SW/SE by `py <= cy ? (px <= cx ? NW : NE) :
//    (px <= cx ? SW : SE)` (quadtree.js:175-179), with child centres formed as
//    cx +/- bw/2 in FP64 (quadtree.js:119-172);
//  * a node is divided iff more than 4 points reach it (capacity 4,
//    quadtree.js:214-229), which does not depend on insertion order.
//
// Instead of inserting points one by one, every point gets a 62-bit Morton
// key whose 31 two-bit digits are exactly those routing decisions, computed in
// FP64 (an exact integer quantisation when every node centre is representable,
// the reference's centre recurrence otherwise).  After sorting, the points of
// any node are a contiguous run, so each point can find in O(1), from the
// common-prefix lengths (LCP) of its neighbours four places away, the level of
// its leaf and the levels of the internal nodes whose run it starts.  Nodes
// are numbered by exclusive scans, linked by binary search over the run, and
// aggregated bottom-up (mass, charge, magnetic moment, angular momentum,
// momentum, centre of mass; quadtree.js:239-312) with arrival counters.
//
// Aggregates use compensated FP32 (centre of mass as an unevaluated hi+lo
// pair), so the walk can measure distances to a node without the rounding of
// a large absolute coordinate.
//
// Depth: keys keep 31 levels.  A leaf at level 31 holding more than 4 points
// (a "bucket") is reported in GeonTreeInfo.n_bucket; the reference would keep
// subdividing there (and never terminates for 5 coincident points).
#include "tree_dev.cuh"

namespace geon {

__global__ void tree_reset_kernel(FrameCtl* ctl) { tree_reset_body(ctl, blockIdx.x, gridDim.x); }
__global__ void ghost_count_kernel(DevParams P, DevState S, TreeBufs T, const FrameCtl* ctl) { ghost_count_body(P, S, T, ctl, blockIdx.x, gridDim.x); }
__global__ void point_refs_kernel(DevParams P, DevState S, TreeBufs T, FrameCtl* ctl) { point_refs_body(P, S, T, ctl, blockIdx.x, gridDim.x); }
__global__ void key_kernel(DevParams P, DevState S, TreeBufs T, FrameCtl* ctl) { key_body(P, S, T, ctl, blockIdx.x, gridDim.x); }
__global__ void gather_kernel(DevParams P, DevState S, TreeBufs T, const FrameCtl* ctl) { gather_body(P, S, T, ctl, blockIdx.x, gridDim.x); }
__global__ void emit_kernel(DevParams P, TreeBufs T, FrameCtl* ctl) { emit_body(P, T, ctl, blockIdx.x, gridDim.x); }
__global__ void link_kernel(DevParams P, TreeBufs T, FrameCtl* ctl, int* d_root) { link_body(P, T, ctl, d_root, blockIdx.x, gridDim.x); }
__global__ void batch_roots_kernel(DevParams P, TreeBufs T, const FrameCtl* ctl) { batch_roots_body(P, T, ctl, blockIdx.x, gridDim.x); }
__global__ void aggregate_kernel(DevParams P, DevState S, TreeBufs T, FrameCtl* ctl) { aggregate_body(P, S, T, ctl, blockIdx.x, gridDim.x); }

static inline int grid_for(int n, int threads) {
    int b = (n + threads - 1) / threads;
    return std::max(1, std::min(b, device_sms() * 16));
}

void tree_build(const DevParams& P, const DevState& S, TreeBufs& T, FrameCtl* ctl, int* d_root,
                int n_cap, cudaStream_t st, LaunchCounter& lc) {
    const int TH = 256;
    tree_reset_kernel<<<1, 1, 0, st>>>(ctl);
    ghost_count_kernel<<<grid_for(n_cap, TH), TH, 0, st>>>(P, S, T, ctl);
    exclusive_scan(T.ghost_cnt, T.ghost_off, n_cap, &ctl->n, &ctl->nGhost, T.scan_tmp, st, &lc);
    point_refs_kernel<<<grid_for(n_cap, TH), TH, 0, st>>>(P, S, T, ctl);
    key_kernel<<<grid_for(T.cap_pts, TH), TH, 0, st>>>(P, S, T, ctl);
    lc.add(4);
    const int which = radix_sort_pairs(T.key, T.idx, T.key_alt, T.idx_alt, T.cap_pts, &ctl->nPts, 64,
                                       T.sort_tmp, st, &lc);
    T.skey = which ? T.key_alt : T.key;
    T.sidx = which ? T.idx_alt : T.idx;
    gather_kernel<<<grid_for(T.cap_pts, TH), TH, 0, st>>>(P, S, T, ctl);
    lc.add(1);
    exclusive_scan(T.int_cnt, T.int_base, T.cap_pts, &ctl->nPts, &ctl->nInternal, T.scan_tmp, st, &lc);
    exclusive_scan(T.leaf_flag, T.leaf_base, T.cap_pts, &ctl->nPts, &ctl->nLeaves, T.scan_tmp, st, &lc);
    exclusive_scan(T.real_flag, T.tgt_base, T.cap_pts, &ctl->nPts, nullptr, T.scan_tmp, st, &lc);
    emit_kernel<<<grid_for(T.cap_pts, TH), TH, 0, st>>>(P, T, ctl);
    link_kernel<<<grid_for(T.cap_int, TH), TH, 0, st>>>(P, T, ctl, d_root);
    lc.add(2);
    if (P.nsys) {
        cudaMemsetAsync(T.roots, 0xFF, (size_t)P.nsys * sizeof(int), st);      // ROOT_NONE
        batch_roots_kernel<<<grid_for(T.cap_pts, TH), TH, 0, st>>>(P, T, ctl);
        lc.add(1);
    }
    aggregate_kernel<<<grid_for(T.cap_pts, TH), TH, 0, st>>>(P, S, T, ctl);
    lc.add(1);
}

// ---- leaf dump for membership tests ----------------------------------------------------
__global__ void leaf_dump_kernel(DevParams P, TreeBufs T, const FrameCtl* ctl, int* leaf_of_point,
                                 double* bx, double* by, double* bw, int* level, int cap_pts) {
    const int nPts = ctl->nPts, nValid = ctl->nValid, nLeaves = ctl->nLeaves;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nPts; s += gridDim.x * blockDim.x) {
        const uint32_t p = T.sidx[s];
        if ((int)p < cap_pts) leaf_of_point[p] = (s < nValid) ? T.leaf_of[s] : -1;
    }
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nLeaves; l += gridDim.x * blockDim.x) {
        const int4 lm = T.leaf_meta[l];
        const uint64_t k = T.skey[lm.x];
        double cx = P.rootX, cy = P.rootY, hw = P.rootW, hh = P.rootH;
        for (int lv = 1; lv <= lm.z; lv++) {                 // quadtree.js:119-131
            const uint32_t dg = key_digit(k, lv, P.keyLevels);
            hw = hw / 2; hh = hh / 2;
            cx = (dg & 1u) ? cx + hw : cx - hw;
            cy = (dg & 2u) ? cy + hh : cy - hh;
        }
        bx[l] = cx; by[l] = cy; bw[l] = hw; level[l] = lm.z;
    }
}

void tree_leaf_dump(const DevParams& P, const TreeBufs& T, const FrameCtl* ctl, int* d_leaf_of_point,
                    double* d_bx, double* d_by, double* d_bw, int* d_level, int cap_pts, cudaStream_t st,
                    LaunchCounter& lc) {
    leaf_dump_kernel<<<grid_for(T.cap_pts, 256), 256, 0, st>>>(P, T, ctl, d_leaf_of_point, d_bx, d_by, d_bw, d_level, cap_pts);
    lc.add(1);
}

}  // namespace geon
