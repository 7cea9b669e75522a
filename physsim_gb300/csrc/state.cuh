// state.cuh — device buffers of one particle system and of its quadtree,
// and the host-side launchers each translation unit provides.
#pragma once

#include "common.cuh"
#include "prims.cuh"

namespace geon {

// Particle state, SoA, insertion order (the CPU path's array order).
struct DevState {
    float4* pos;      // x, y, mass, charge
    float2* pos_lo;   // low parts of x, y: positions are the unevaluated sums pos + pos_lo
    float4* vel;      // wx, wy (proper velocity), vx, vy (coordinate velocity)
    float4* spin;     // angw, angVel, radius (cbrt m), invMass
    float2* mom;      // magMoment, angMomentum cached by the last force pass (forces.js:71-76)
    float4* force;    // fx, fy, Bz, Bgz
    float4* grad;     // dBzdx, dBzdy, dBgzdx, dBgzdy
    float4* torque;   // _tidalTorque, _frameDragTorque, _contactTorque, pe
    float2* f1pn;     // force1PN
    float2* f1pnOld;  // _f1pnOld
    float*  brk;      // per-type force vectors, 12 rows of n_cap (GEON_OUT_GRAV_X .. EXT_Y)
    double* ctime;    // creationTime
    int*    id;       // stable ids
    float4* hist;     // history ring [n_cap][256]: x, y, vx, vy
    float*  hist_angw;// [n_cap][256]
    int*    hist_cnt; // samples held per particle
    int*    sys;      // system of each particle (batched handles; null otherwise)
    float2* matter;   // baseMass, antimatter (1 or 0) (particle.js:48-50; merge collisions)
};

// Quadtree over particles + ghosts.
struct TreeBufs {
    int cap_pts;        // point capacity
    int cap_int;        // internal-node capacity
    uint32_t* pt_ref;   // [cap_pts] unsorted point refs (particles, then ghosts)
    int* ghost_cnt;     // [n_cap]
    int* ghost_off;     // [n_cap]
    uint64_t* key; uint64_t* key_alt;
    uint32_t* idx; uint32_t* idx_alt;
    void* sort_tmp;
    int* scan_tmp;
    // sorted points
    uint64_t* skey;     // sorted keys (points to key or key_alt)
    uint32_t* sidx;     // sorted point indices
    // sorted point records, ready to stage as force sources
    float4* ps_a;       // image x (hi), image y (hi), mass, charge
    float4* ps_b;       // image x (lo), image y (lo), vx, vy (image flips applied)
    float4* ps_c;       // angVel (flipped), magMoment, angMomentum (current), ref bits
    int* lcp_a;         // lcp level with the previous key (-1 at 0)
    int* int_cnt;       // internal nodes started per point
    int* int_base;
    int* leaf_flag;
    int* leaf_base;
    int* real_flag;     // 1 if sorted point is a particle
    int* tgt_base;
    int* tgt;           // [n_cap] walk order: particle indices by key
    // internal nodes
    float4* int_a;      // com_hi.x, com_hi.y, mass, charge
    float4* int_b;      // vbar.x, vbar.y, sum mu, sum L
    float4* int_c;      // com_lo.x, com_lo.y, size^2, level
    int4*   int_child;  // child refs (LEAF_REF bit for leaves), -1 empty
    int4*   int_meta;   // level, start, end, parent
    int*    int_count;  // arrivals for the bottom-up pass
    // leaves
    float4* leaf_a; float4* leaf_b; float4* leaf_c;
    int4*   leaf_meta;  // start, count, level, parent
    int*    leaf_of;    // [cap_pts] leaf of each sorted point
    // higher moments about each node's centre of mass (learned correction only; null otherwise)
    float4* int_m1; float4* int_m2; float4* int_m3;    // (Ixx, Ixy, Iyy, sum|q|), (Dx, Dy, Jxx, Jxy), (Jyy, -, -, -)
    float4* leaf_m1; float4* leaf_m2; float4* leaf_m3;
    int mom_on;         // compute the moments in this tree build
    int* roots;         // [nsys] root of each system (batched handles; null otherwise)
};

constexpr int LEAF_REF = 1 << 30;
constexpr int ROOT_NONE = -1;

// tree.cu
void tree_build(const DevParams& P, const DevState& S, TreeBufs& T, FrameCtl* ctl, int* d_root,
                int n_cap, cudaStream_t st, LaunchCounter& lc);
void tree_leaf_dump(const DevParams& P, const TreeBufs& T, const FrameCtl* ctl, int* d_leaf_of_point,
                    double* d_bx, double* d_by, double* d_bw, int* d_level, int cap_pts, cudaStream_t st,
                    LaunchCounter& lc);

}  // namespace geon
