// collide.cuh — merge collisions on the substep's quadtree (collide.cu).
#pragma once

#include "state.cuh"

namespace geon {

constexpr int COL_EVENT_CAP = 1 << 16;   // events kept per frame (later ones are counted only)
constexpr int COL_LEAF_BUF = 8;          // candidates of one leaf that are put in storage order
constexpr int COL_STACK = 128;           // query stack (31 levels need <= 97)

// error bits of CollCtl.err
constexpr int COL_ERR_CAND_OVERFLOW = 1; // more overlap candidates than the buffer holds: no collisions resolved
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
    int pad[6];
};

struct CollBufs {
    CollCtl* cc;
    int* cnt;            // [n_cap] candidates per particle
    int* off;            // [n_cap] their exclusive scan
    int2* cand;          // [cap] (particle, sorted tree point) in the reference's visiting order
    int cap;
    int* inv;            // [n_cap] sorted position of each particle's own tree point (-1: not in the tree)
    int* min5;           // [cap_int * 5] earliest-inserted five points of each internal node (sorted positions)
    int* m5cnt;          // [cap_int] child arrivals of the bottom-up pass
    int* tflag;          // [n_cap] tree targets still alive
    int* tpos;           // [n_cap] their exclusive scan
    int* tgt2;           // [slots] live targets in tree order, then the spawns
    double* events;      // [COL_EVENT_CAP][6]: type (1 annihilation, 2 merge), x, y, energy, px, py
    int* scan_tmp;
};

// Overlap candidates of every particle (a superset of the pairs the
// sequential pass will merge), in the order QuadTreePool.query reports them.
void collide_detect(const DevParams& P, const DevState& S, const TreeBufs& T, const int* d_root, FrameCtl* ctl,
                    const CollBufs& B, int n_cap, cudaStream_t st, LaunchCounter& lc);

// The sequential pass of handleCollisions over the candidates (one thread),
// spawns written to slots n, n+1, ...; then keep flags for slots [0, n + spawned)
// and the count of removed particles.
void collide_resolve(const DevParams& P, const DevState& S, const TreeBufs& T, const FrameCtl* ctl, const CollBufs& B,
                     int* keep, int n, int slots, double sim_time, int id0, int n_cap, cudaStream_t st, LaunchCounter& lc);

// Walk target list for the force pass that follows: the tree order without
// the removed particles, then the spawns (B.tgt2, n - removed + spawned entries).
void collide_targets(const DevState& S, const TreeBufs& T, FrameCtl* ctl, const CollBufs& B, int n, int spawned,
                     int n_cap, cudaStream_t st, LaunchCounter& lc);

}  // namespace geon
