// collide.cuh — merge collisions on the substep's quadtree (collide.cu).
#pragma once

#include "state.cuh"

namespace geon {

constexpr int COL_EVENT_CAP = 1 << 16;   // events kept per frame (later ones are counted only)
constexpr int COL_LEAF_BUF = 8;          // candidates of one leaf that are put in storage order
constexpr int COL_STACK = 128;           // query stack (31 levels need <= 97)
constexpr int COL_SERIAL_MAX = 16;       // candidates resolved by one thread without the component sort
constexpr double COL_TOL = 2e-6;         // FP32 node-box slack, relative to the root size

// error bits of CollCtl.err
constexpr int COL_ERR_SLOTS = 2;         // a spawn found no free slot (cannot happen: slots >= 2 * capacity)
constexpr int COL_ERR_ORDER = 4;         // a leaf at the depth cap held > 4 points: its candidates kept index order
constexpr int COL_ERR_QUERY = 8;         // a query stack overflowed or met a bad node index

struct CollCtl {
    int total;           // overlap candidates of this substep
    int spawned;         // merged particles appended this substep
    int merges;
    int annihilations;
    int removed;         // particles whose mass reached zero this substep
    int events;          // events stored this frame
    int events_dropped;  // events beyond COL_EVENT_CAP this frame
    int need_order;      // a query met two or more candidates in one leaf
    int err;             // COL_ERR_* bits
    int nlive;           // targets left after removal (scan total)
    int stotal;          // merges of this substep (scan total)
    int etotal;          // events of this substep (scan total)
    int pad[4];
};

// What the resolution recorded for one candidate pair: masses, base masses
// and radii of the two particles at that moment.
struct PairRec { float m1, m2, b1, b2, r1, r2; };
enum { PAIR_NONE = 0, PAIR_ANNIHILATE = 1, PAIR_MERGE = 2 };

struct CollBufs {
    CollCtl* cc;
    int* cnt;            // [n_cap] candidates per particle
    int* off;            // [n_cap] their exclusive scan
    int2* cand;          // [cap] (particle, sorted tree point) in the reference's visiting order
    int cap;
    int* uf;             // [n_cap] union-find parents: pairs sharing a particle form one component
    uint64_t* skey; uint64_t* skey_alt;   // [cap] component << 32 | pair
    uint32_t* sval; uint32_t* sval_alt;   // [cap]
    void* sort_tmp;
    int sort_bits;
    PairRec* rec;        // [cap]
    int* kind;           // [cap] PAIR_*
    int* sflag; int* spos;   // [cap] merges and their ranks (spawn order)
    int* eflag; int* epos;   // [cap] events and their ranks
    int* inv;            // [n_cap] sorted position of each particle's own tree point (-1: not in the tree)
    float4* ibox;        // [cap_int] internal node boxes (x0, y0, x1, y1), FP32 rounded outward
    float4* lbox;        // [cap_pts] leaf boxes
    int* min5;           // [cap_int * 5] earliest-inserted five points of each internal node (sorted positions)
    int* m5cnt;          // [cap_int] child arrivals of the bottom-up pass
    int* tflag;          // [n_cap] tree targets still alive
    int* tpos;           // [n_cap] their exclusive scan
    int* tk;             // [n_cap] position of each particle in the tree order
    int* acnt;           // [n_cap] spawns anchored at each position of the tree order
    int* abefore;        // [n_cap] their exclusive scan
    int* amin;           // [n_cap] first spawn anchored there
    int* anch;           // [cap] anchor position of each spawn
    int* tgt2;           // [slots] live targets in tree order, then the spawns
    double* events;      // [COL_EVENT_CAP][6]: type (1 annihilation, 2 merge), x, y, energy, px, py
    int* scan_tmp;
};

// Overlap candidates of every particle (a superset of the pairs the
// sequential pass will merge), in the order QuadTreePool.query reports them.
void collide_detect(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                    const CollBufs& B, int n_cap, cudaStream_t st, LaunchCounter& lc);

// The sequential pass of handleCollisions over the `total` candidates: one
// thread per connected component of the pair graph (one thread for all when
// total <= COL_SERIAL_MAX), spawns written to slots n, n+1, ... in order;
// then keep flags for slots [0, n + spawned) and the count of removed particles.
void collide_resolve(const DevParams& P, const DevState& S, const TreeBufs& T, const FrameCtl* ctl, const CollBufs& B,
                     int* keep, int n, int total, int slots, double sim_time, int id0, cudaStream_t st, LaunchCounter& lc);

// Walk target list for the force pass that follows: the tree order without
// the removed particles, each spawn in the place of the particle it replaced
// (B.tgt2, n - removed + spawned entries).
void collide_targets(const DevState& S, const TreeBufs& T, FrameCtl* ctl, const CollBufs& B, int n, int total,
                     int spawned, int n_cap, cudaStream_t st, LaunchCounter& lc);

}  // namespace geon
