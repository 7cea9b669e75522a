// geon_oracle.cpp — FP64 CPU restatement of Geon's particle force-and-push
// path.  TEST INFRASTRUCTURE ONLY: the parity tests, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load this library as the checker.  Nothing
// in the product path (physsim_gb300) links or calls it.
//
// Parity status: unpinned by the reference's own outputs.  The reference
// (a9lim/physsim) is browser JavaScript with no tests, fixtures or golden
// vectors, and no JavaScript engine exists where this repository is built or
// tested, so this restatement cannot be run side by side with it.  It follows
// the reference line by line (citations below, paths relative to the
// reference project) and is anchored by analytic known-answer tests
// (tests/test_oracle_kat.py) and by committed fixtures it generated
// (tests/golden/).
//
// Restated (reference file:line):
//   config.js:28-60,120-122       constants
//   topology.js:9-135             minImage / wrapPosition
//   quadtree.js:13-312,412-419    QuadTreePool (insert order, capacity 4,
//                                 depth guard, post-order aggregation)
//   signal-delay.js:16-221        getDelayedState
//   forces.js:14-154              resetForces / computeAllForces
//   forces.js:163-442             pairForce (radiation jerk omitted: the
//                                 radiation step needs a Simulation object,
//                                 integrator.js:986, which the path runs without)
//   forces.js:445-610             _accum1PN / _compute1PNTreeWalk / compute1PN
//   forces.js:622-694             calculateForce (BH walk)
//   integrator.js:138-260         _syncToggles, ghosts, _buildTree
//   integrator.js:553-660         external fields, bounce-wall forces
//   integrator.js:726-982,1269-1348,1489-1565,1741-1824   Physics.update
//   relativity.js:7-25            angwToAngVel / setVelocity
//   energy.js:11-62               KE, momentum, COM, angular momentum
//
// Everything is double precision.  The per-particle loops of the force pass
// can run on several threads (OpenMP) for the timed CPU baseline; each
// particle's accumulators are written by one thread only, so the numbers do
// not depend on the thread count.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <string>
#include <limits>
#include <algorithm>
#include <array>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/geon.h"

namespace {

// ---- constants (config.js) -------------------------------------------------
constexpr double EPS = 1e-12;                // config.js:30
constexpr double INERTIA_K = 0.4;            // config.js:52
constexpr double MAG_MOMENT_K = 0.2;         // config.js:53
constexpr double TIDAL_STRENGTH = 64;        // config.js:54
constexpr double BOSON_CHARGE = 0.1;         // config.js:75
constexpr double BOSON_SOFTENING_SQ = 4;     // config.js:48
constexpr double YUKAWA_COUPLING = 14;       // config.js:80
constexpr int    QT_CAPACITY = 4;            // config.js:59
constexpr int    HISTORY_SIZE = 256;         // config.js:120
constexpr int    HISTORY_MASK = 255;         // config.js:121
constexpr int    HISTORY_STRIDE = 64;        // config.js:122
constexpr double DESPAWN_MARGIN = 64;        // config.js:138
constexpr double MAX_SPEED_RATIO = 0.999;    // config.js:32
constexpr double INF = std::numeric_limits<double>::infinity();

enum Comp { C_GRAV = 0, C_COUL, C_MAG, C_GM, C_1PN, C_SPINCURV, C_YUK, C_EXT, NCOMP };

struct History {
    std::vector<double> x, y, vx, vy, angw, t;
    int head = 0, count = 0;
    bool alloc = false;
    void init() {                              // particle.js:124-134
        if (alloc) return;
        x.assign(HISTORY_SIZE, 0); y.assign(HISTORY_SIZE, 0);
        vx.assign(HISTORY_SIZE, 0); vy.assign(HISTORY_SIZE, 0);
        angw.assign(HISTORY_SIZE, 0); t.assign(HISTORY_SIZE, 0);
        head = 0; count = 0; alloc = true;
    }
};

struct Particle {                              // particle.js:15-92 (fields on the path)
    int id = 0;
    double x = 0, y = 0, vx = 0, vy = 0, wx = 0, wy = 0;
    double mass = 1, charge = 0, angw = 0, angVel = 0;
    double radius = 1, radiusSq = 1, bodyRadiusSq = 1, invMass = 1;
    double magMoment = 0, angMomentum = 0;
    double fx = 0, fy = 0;
    double comp[NCOMP][2] = {};
    double Bz = 0, Bgz = 0, dBzdx = 0, dBzdy = 0, dBgzdx = 0, dBgzdy = 0;
    double tidal = 0, frameDrag = 0, contact = 0;
    double tqSpinOrbit = 0, tqFrameDrag = 0, tqTidal = 0, tqContact = 0;
    double f1pnOldx = 0, f1pnOldy = 0;
    double creationTime = -INF, deathTime = INF;
    double axMod = 1, yukMod = 1, higgsMod = 1;
    double pe = 0;                             // this particle's share of _peAccum
    double baseMass = 1;                       // particle.js:48 (scaled by annihilation, summed by merges)
    bool antimatter = false;                   // particle.js:50
    bool dead = false;                         // removed by a collision this substep, still a tree source
    History h;

    void setMass(double m) {                   // Particle.updateColor (particle.js:110-121), non-BH
        mass = m;
        double r = std::cbrt(m);
        bodyRadiusSq = r * r;
        radius = r;
        radiusSq = r * r;
        invMass = 1 / m;
    }
};

// Periodic image of a particle (integrator.js:176-198).
struct Ghost {
    double x, y, vx, vy, wx, wy, mass, charge, angVel, angw, magMoment, angMomentum, radius, radiusSq;
    int orig;
};

struct Toggles {                               // integrator.js:114-124,138-150
    bool gravity, coulomb, magnetic, gravitomag, onePN, yukawa, axion, higgs, radiation;
    double yukawaMu, softeningSq;
};

struct Vec { double x, y; };

// ---- topology.js -------------------------------------------------------------
inline double torusWrap(double d, double full, double half) {     // topology.js:9-12
    if (d > half) d -= full; else if (d < -half) d += full;
    return d;
}

inline Vec minImage(double ox, double oy, double sx, double sy, int topology,
                    double W, double H, double halfW, double halfH) {  // topology.js:18-76
    double dx = sx - ox, dy = sy - oy;
    if (topology == GEON_TORUS) return { torusWrap(dx, W, halfW), torusWrap(dy, H, halfH) };
    const double doubleH = 2 * H;
    if (topology == GEON_KLEIN) {
        double bx = torusWrap(dx, W, halfW), by = dy;
        double bestDx = bx, bestDy = by, bestSq = bx * bx + by * by;
        double cx = torusWrap((W - sx) - ox, W, halfW);
        double cy = torusWrap((sy + H) - oy, doubleH, H);
        double sq = cx * cx + cy * cy;
        if (sq < bestSq) { bestDx = cx; bestDy = cy; }
        return { bestDx, bestDy };
    }
    const double doubleW = 2 * W;
    double bestDx = dx, bestDy = dy, bestSq = dx * dx + dy * dy;
    double cx = (W - sx) - ox;
    double cy = torusWrap((sy + H) - oy, doubleH, H);
    double sq = cx * cx + cy * cy;
    if (sq < bestSq) { bestDx = cx; bestDy = cy; bestSq = sq; }
    cx = torusWrap((sx + W) - ox, doubleW, W);
    cy = (H - sy) - oy;
    sq = cx * cx + cy * cy;
    if (sq < bestSq) { bestDx = cx; bestDy = cy; bestSq = sq; }
    cx = torusWrap((2 * W - sx) - ox, doubleW, W);
    cy = torusWrap((2 * H - sy) - oy, doubleH, H);
    sq = cx * cx + cy * cy;
    if (sq < bestSq) { bestDx = cx; bestDy = cy; }
    return { bestDx, bestDy };
}

void wrapPosition(Particle& p, int topology, double W, double H) {   // topology.js:81-135
    if (topology == GEON_TORUS) {
        if (p.x < 0) p.x += W; else if (p.x > W) p.x -= W;
        if (p.y < 0) p.y += H; else if (p.y > H) p.y -= H;
        return;
    }
    if (topology == GEON_KLEIN) {
        if (p.x < 0) p.x += W; else if (p.x > W) p.x -= W;
        if (p.y < 0 || p.y > H) {
            p.y += (p.y < 0) ? H : -H;
            p.x = W - p.x;
            p.wx = -p.wx; p.vx = -p.vx;
            p.angw = -p.angw; p.angVel = -p.angVel;
        }
        return;
    }
    for (int iter = 0; iter < 2; iter++) {
        bool wrapped = false;
        if (p.x < 0 || p.x > W) {
            p.x += (p.x < 0) ? W : -W;
            p.y = H - p.y;
            p.wy = -p.wy; p.vy = -p.vy;
            p.angw = -p.angw; p.angVel = -p.angVel;
            wrapped = true;
        }
        if (p.y < 0 || p.y > H) {
            p.y += (p.y < 0) ? H : -H;
            p.x = W - p.x;
            p.wx = -p.wx; p.vx = -p.vx;
            p.angw = -p.angw; p.angVel = -p.angVel;
            wrapped = true;
        }
        if (!wrapped) break;
    }
}

inline double angwToAngVel(double angw, double radius) {           // relativity.js:7-9
    return angw / std::sqrt(1 + angw * angw * radius * radius);
}

// ---- quadtree.js ------------------------------------------------------------------
// Tree points are integers: 0..nReal-1 are particles, nReal.. are ghosts.
struct QuadTree {
    std::vector<double> bx, by, bw, bh, totalMass, totalCharge, totalMag, totalAngMom, momX, momY, comX, comY;
    std::vector<int32_t> nw, ne, sw, se;
    std::vector<int32_t> points;
    std::vector<uint8_t> pointCount, divided;
    std::vector<int32_t> level;              // depth of each node (root 0); for leaf dumps
    int count = 0;
    bool overflow = false;
    size_t nodeLimit = 0;

    int alloc(double x, double y, double w, double h, int lvl) {     // quadtree.js:52-76
        int idx = count++;
        if ((size_t)count > bx.size()) grow(count);
        bx[idx] = x; by[idx] = y; bw[idx] = w; bh[idx] = h;
        totalMass[idx] = 0; totalCharge[idx] = 0; totalMag[idx] = 0; totalAngMom[idx] = 0;
        momX[idx] = 0; momY[idx] = 0; comX[idx] = x; comY[idx] = y;
        nw[idx] = ne[idx] = sw[idx] = se[idx] = -1;
        pointCount[idx] = 0; divided[idx] = 0; level[idx] = lvl;
        return idx;
    }
    void grow(size_t need) {
        size_t n = std::max<size_t>(need, bx.size() * 2 + 64);
        for (auto* v : { &bx, &by, &bw, &bh, &totalMass, &totalCharge, &totalMag, &totalAngMom,
                         &momX, &momY, &comX, &comY }) v->resize(n);
        for (auto* v : { &nw, &ne, &sw, &se, &level }) v->resize(n, -1);
        pointCount.resize(n); divided.resize(n);
        points.resize(n * QT_CAPACITY, -1);
    }
    bool contains(int idx, double px, double py) const {           // quadtree.js:105-110
        return px >= bx[idx] - bw[idx] && px <= bx[idx] + bw[idx] &&
               py >= by[idx] - bh[idx] && py <= by[idx] + bh[idx];
    }
    void subdivide(int idx) {                                     // quadtree.js:119-172
        double x = bx[idx], y = by[idx];
        double hw = bw[idx] / 2, hh = bh[idx] / 2;
        int lvl = level[idx] + 1;
        int c = alloc(x - hw, y - hh, hw, hh, lvl);     // NW
        alloc(x + hw, y - hh, hw, hh, lvl);             // NE
        alloc(x - hw, y + hh, hw, hh, lvl);             // SW
        alloc(x + hw, y + hh, hw, hh, lvl);             // SE
        nw[idx] = c; ne[idx] = c + 1; sw[idx] = c + 2; se[idx] = c + 3;
        divided[idx] = 1;
    }
    int childFor(int idx, double px, double py) const {           // quadtree.js:175-179
        return py <= by[idx] ? (px <= bx[idx] ? nw[idx] : ne[idx])
                             : (px <= bx[idx] ? sw[idx] : se[idx]);
    }
    template <class PosFn>
    bool insert(int root, int pt, PosFn pos, std::vector<std::pair<int, int>>& work) {  // quadtree.js:185-237
        double px0, py0; pos(pt, px0, py0);
        if (!contains(root, px0, py0)) return false;
        work.clear();
        work.push_back({ root, pt });
        while (!work.empty()) {
            auto [nodeIdx, p] = work.back(); work.pop_back();
            double px, py; pos(p, px, py);
            int depth = 0;
            while (depth <= 48) {
                if (pointCount[nodeIdx] < QT_CAPACITY && !divided[nodeIdx]) {
                    points[nodeIdx * QT_CAPACITY + pointCount[nodeIdx]] = p;
                    pointCount[nodeIdx]++;
                    break;
                }
                if (!divided[nodeIdx]) {
                    if ((size_t)count + 4 > nodeLimit) { overflow = true; return true; }
                    subdivide(nodeIdx);
                    int base = nodeIdx * QT_CAPACITY;
                    for (int i = 0; i < pointCount[nodeIdx]; i++) {
                        int q = points[base + i];
                        double qx, qy; pos(q, qx, qy);
                        work.push_back({ childFor(nodeIdx, qx, qy), q });
                    }
                    pointCount[nodeIdx] = 0;
                }
                nodeIdx = childFor(nodeIdx, px, py);
                depth++;
            }
        }
        return true;
    }
};

struct Sim {
    GeonParams prm{};
    std::vector<Particle> ps;
    std::vector<Ghost> ghosts;
    QuadTree tree;
    int root = -1;
    double simTime = 0;
    bool forcesInit = false;
    int histStride = 0;
    int lastSubsteps = 0;
    double pe = 0;
    int64_t interactions = 0;
    int nextId = 0;
    int nThreads = 1;
    int nTree = 0;                             // particles in the last tree (ghost points start there)
    // collision results of the last update (collisions.js:24-107)
    std::vector<std::array<double, 6>> events; // type (1 annihilation, 2 merge), x, y, energy, px, py
    int nMerges = 0, nAnnihilations = 0, nSpawned = 0, nRemovedCol = 0;
    // boson pool (photons, pions, leptons as the Simulation holds them): the
    // fields the boson tree and its walks read
    struct Boson { double x, y, srcMass, srcCharge, vSq; int kind; };   // kind 0 photon, 1 massive
    std::vector<Boson> bosons;
    QuadTree btree;
    int broot = -1;
    std::string err;

    bool on(uint32_t bit) const { return (prm.toggles & bit) != 0; }
    bool relOn() const { return on(GEON_RELATIVITY); }
    bool periodic() const { return prm.boundary_mode == GEON_BOUND_LOOP; }

    Toggles toggles() const {                                     // integrator.js:138-150
        Toggles t;
        t.gravity = on(GEON_GRAVITY); t.coulomb = on(GEON_COULOMB);
        t.magnetic = on(GEON_MAGNETIC); t.gravitomag = on(GEON_GRAVITOMAG);
        t.onePN = on(GEON_ONE_PN); t.yukawa = on(GEON_YUKAWA);
        t.axion = false; t.higgs = false; t.radiation = false;
        t.yukawaMu = prm.yukawa_mu;
        t.softeningSq = prm.softening * prm.softening;
        return t;
    }

    // tree point accessors
    int nReal() const { return (int)ps.size(); }
    void ptPos(int i, double& x, double& y) const {
        if (i < nTree) { x = ps[i].x; y = ps[i].y; }
        else { x = ghosts[i - nTree].x; y = ghosts[i - nTree].y; }
    }

    // ---- ghosts (integrator.js:176-244) ----
    void addGhost(const Particle& p, int orig, double sx, double sy, bool flipVx, bool flipVy) {
        Ghost g;
        g.x = sx; g.y = sy;
        g.vx = flipVx ? -p.vx : p.vx; g.vy = flipVy ? -p.vy : p.vy;
        g.wx = flipVx ? -p.wx : p.wx; g.wy = flipVy ? -p.wy : p.wy;
        g.mass = p.mass; g.charge = p.charge;
        g.angVel = (flipVx || flipVy) ? -p.angVel : p.angVel;
        g.angw = (flipVx || flipVy) ? -p.angw : p.angw;
        g.radius = p.radius; g.radiusSq = p.radiusSq;
        g.magMoment = MAG_MOMENT_K * g.charge * g.angVel * g.radiusSq;
        g.angMomentum = INERTIA_K * g.mass * g.angVel * g.radiusSq;
        g.orig = orig;
        ghosts.push_back(g);
    }
    void generateGhosts() {
        ghosts.clear();
        const double W = prm.domain_w, H = prm.domain_h;
        const double margin = std::max(W, H) * prm.theta;          // integrator.js:204 (BH_THETA)
        const int topo = prm.topology;
        for (int i = 0; i < nReal(); i++) {
            const Particle& p = ps[i];
            const double x = p.x, y = p.y;
            const bool nearL = x < margin, nearR = x > W - margin;
            const bool nearT = y < margin, nearB = y > H - margin;
            if (topo == GEON_TORUS) {
                if (nearL) addGhost(p, i, x + W, y, false, false);
                if (nearR) addGhost(p, i, x - W, y, false, false);
                if (nearT) addGhost(p, i, x, y + H, false, false);
                if (nearB) addGhost(p, i, x, y - H, false, false);
                if (nearL && nearT) addGhost(p, i, x + W, y + H, false, false);
                if (nearL && nearB) addGhost(p, i, x + W, y - H, false, false);
                if (nearR && nearT) addGhost(p, i, x - W, y + H, false, false);
                if (nearR && nearB) addGhost(p, i, x - W, y - H, false, false);
            } else if (topo == GEON_KLEIN) {
                if (nearL) addGhost(p, i, x + W, y, false, false);
                if (nearR) addGhost(p, i, x - W, y, false, false);
                if (nearT) addGhost(p, i, W - x, y + H, true, false);
                if (nearB) addGhost(p, i, W - x, y - H, true, false);
                if (nearL && nearT) addGhost(p, i, W - x + W, y + H, true, false);
                if (nearL && nearB) addGhost(p, i, W - x + W, y - H, true, false);
                if (nearR && nearT) addGhost(p, i, W - x - W, y + H, true, false);
                if (nearR && nearB) addGhost(p, i, W - x - W, y - H, true, false);
            } else {
                if (nearL) addGhost(p, i, x + W, H - y, false, true);
                if (nearR) addGhost(p, i, x - W, H - y, false, true);
                if (nearT) addGhost(p, i, W - x, y + H, true, false);
                if (nearB) addGhost(p, i, W - x, y - H, true, false);
                if (nearL && nearT) addGhost(p, i, W - x + W, y + H, true, false);
                if (nearL && nearB) addGhost(p, i, W - x + W, y - H, true, false);
                if (nearR && nearT) addGhost(p, i, W - x - W, y + H, true, false);
                if (nearR && nearB) addGhost(p, i, W - x - W, y - H, true, false);
            }
        }
    }

    // ---- tree build (integrator.js:247-260, quadtree.js:412-419) ----
    void calculateMassDistribution(int rootIdx) {                 // quadtree.js:239-312
        QuadTree& t = tree;
        std::vector<int> stack, order;
        stack.push_back(rootIdx);
        while (!stack.empty()) {
            int idx = stack.back(); stack.pop_back();
            order.push_back(idx);
            if (t.divided[idx]) {
                stack.push_back(t.nw[idx]); stack.push_back(t.ne[idx]);
                stack.push_back(t.sw[idx]); stack.push_back(t.se[idx]);
            }
        }
        for (int k = (int)order.size() - 1; k >= 0; k--) {
            int idx = order[k];
            if (!t.divided[idx]) {
                int cnt = t.pointCount[idx];
                if (cnt == 0) continue;
                double mass = 0, charge = 0, magMom = 0, angMom = 0, cx = 0, cy = 0, momX = 0, momY = 0;
                for (int i = 0; i < cnt; i++) {
                    int pt = t.points[idx * QT_CAPACITY + i];
                    double pm, q, mu, L, x, y, wx, wy;
                    if (pt < nTree) {
                        const Particle& p = ps[pt];
                        pm = p.mass; q = p.charge; mu = p.magMoment; L = p.angMomentum;
                        x = p.x; y = p.y; wx = p.wx; wy = p.wy;
                    } else {
                        const Ghost& g = ghosts[pt - nTree];
                        pm = g.mass; q = g.charge; mu = g.magMoment; L = g.angMomentum;
                        x = g.x; y = g.y; wx = g.wx; wy = g.wy;
                    }
                    mass += pm; charge += q; magMom += mu; angMom += L;
                    cx += x * pm; cy += y * pm;
                    momX += pm * wx; momY += pm * wy;
                }
                t.totalMass[idx] = mass; t.totalCharge[idx] = charge;
                t.totalMag[idx] = magMom; t.totalAngMom[idx] = angMom;
                t.momX[idx] = momX; t.momY[idx] = momY;
                if (mass > 0) { t.comX[idx] = cx / mass; t.comY[idx] = cy / mass; }
            } else {
                int c0 = t.nw[idx], c1 = t.ne[idx], c2 = t.sw[idx], c3 = t.se[idx];
                double m0 = t.totalMass[c0], m1 = t.totalMass[c1], m2 = t.totalMass[c2], m3 = t.totalMass[c3];
                double mass = m0 + m1 + m2 + m3;
                t.totalMass[idx] = mass;
                t.totalCharge[idx] = t.totalCharge[c0] + t.totalCharge[c1] + t.totalCharge[c2] + t.totalCharge[c3];
                t.totalMag[idx] = t.totalMag[c0] + t.totalMag[c1] + t.totalMag[c2] + t.totalMag[c3];
                t.totalAngMom[idx] = t.totalAngMom[c0] + t.totalAngMom[c1] + t.totalAngMom[c2] + t.totalAngMom[c3];
                t.momX[idx] = t.momX[c0] + t.momX[c1] + t.momX[c2] + t.momX[c3];
                t.momY[idx] = t.momY[c0] + t.momY[c1] + t.momY[c2] + t.momY[c3];
                if (mass > 0) {
                    t.comX[idx] = (t.comX[c0] * m0 + t.comX[c1] * m1 + t.comX[c2] * m2 + t.comX[c3] * m3) / mass;
                    t.comY[idx] = (t.comY[c0] * m0 + t.comY[c1] * m1 + t.comY[c2] * m2 + t.comY[c3] * m3) / mass;
                }
            }
        }
    }

    int buildTree() {
        nTree = nReal();
        if (periodic() && !(prm.flags & GEON_FLAG_NO_GHOSTS)) generateGhosts(); else ghosts.clear();
        const double bxr = prm.off_x + prm.domain_w / 2, byr = prm.off_y + prm.domain_h / 2;  // integrator.js:727-730
        const double bwr = prm.domain_w * 2, bhr = prm.domain_h * 2;
        int nPts = nTree + (int)ghosts.size();
        tree.count = 0;
        tree.overflow = false;
        // Guard against the reference's unbounded subdivision on >= 5 coincident points.
        tree.nodeLimit = (size_t)64 * (nPts + 16);
        if (tree.bx.size() < (size_t)2 * nPts + 16) tree.grow((size_t)2 * nPts + 16);
        int r = tree.alloc(bxr, byr, bwr, bhr, 0);
        std::vector<std::pair<int, int>> work;
        auto pos = [this](int i, double& x, double& y) { ptPos(i, x, y); };
        for (int i = 0; i < nPts; i++) tree.insert(r, i, pos, work);
        calculateMassDistribution(r);
        root = r;
        return r;
    }

    // ---- QuadTreePool.query (quadtree.js:372-404): points in the closed box
    // (rx +/- rw, ry +/- rh), depth first with children pushed NW, NE, SW, SE.
    void query(double rx, double ry, double rw, double rh, std::vector<int>& found, std::vector<int>& qs) const {
        const QuadTree& t = tree;
        found.clear();
        if (root < 0) return;
        qs.clear();
        qs.push_back(root);
        while (!qs.empty()) {
            const int ni = qs.back(); qs.pop_back();
            if (rx - rw > t.bx[ni] + t.bw[ni] || rx + rw < t.bx[ni] - t.bw[ni] ||     // _intersects, quadtree.js:112-117
                ry - rh > t.by[ni] + t.bh[ni] || ry + rh < t.by[ni] - t.bh[ni]) continue;
            if (!t.divided[ni]) {
                for (int i = 0; i < t.pointCount[ni]; i++) {
                    const int pt = t.points[ni * QT_CAPACITY + i];
                    double x, y; ptPos(pt, x, y);
                    if (x >= rx - rw && x <= rx + rw && y >= ry - rh && y <= ry + rh) found.push_back(pt);
                }
            } else {
                qs.push_back(t.nw[ni]); qs.push_back(t.ne[ni]);
                qs.push_back(t.sw[ni]); qs.push_back(t.se[ni]);
            }
        }
    }

    // ---- merge collisions (collisions.js:24-158, integrator.js:1350-1381) ----
    static double particleKE(const Particle& p) {                 // collisions.js:17-20
        const double wSq = p.wx * p.wx + p.wy * p.wy;
        return wSq / (std::sqrt(1 + wSq) + 1) * p.mass;
    }
    struct Spawn { double x, y, wx, wy, mass, baseMass, charge, angw, ke; bool antimatter; };
    static Spawn resolveMerge(Particle& p1, Particle& p2, double miDx, double miDy) {   // collisions.js:110-158
        Spawn s;
        const double totalMass = p1.mass + p2.mass;
        s.wx = (p1.mass * p1.wx + p2.mass * p2.wx) / totalMass;
        s.wy = (p1.mass * p1.wy + p2.mass * p2.wy) / totalMass;
        const double p2x = p1.x + miDx, p2y = p1.y + miDy;
        s.x = (p1.x * p1.mass + p2x * p2.mass) / totalMass;
        s.y = (p1.y * p1.mass + p2y * p2.mass) / totalMass;
        const double dx1 = p1.x - s.x, dy1 = p1.y - s.y;
        const double dx2 = p2x - s.x, dy2 = p2y - s.y;
        const double Lorb = dx1 * (p1.mass * p1.wy) - dy1 * (p1.mass * p1.wx)
                          + dx2 * (p2.mass * p2.wy) - dy2 * (p2.mass * p2.wx);
        const double Lspin = INERTIA_K * p1.mass * p1.radius * p1.radius * p1.angw
                           + INERTIA_K * p2.mass * p2.radius * p2.radius * p2.angw;
        const double newRadius = std::cbrt(totalMass);
        const double newI = INERTIA_K * totalMass * newRadius * newRadius;
        s.angw = newI > EPS ? (Lorb + Lspin) / newI : 0;
        s.baseMass = p1.baseMass + p2.baseMass;
        s.charge = p1.charge + p2.charge;
        s.antimatter = p1.antimatter;
        s.mass = totalMass;
        const double wSq = s.wx * s.wx + s.wy * s.wy;
        s.ke = wSq / (std::sqrt(1 + wSq) + 1) * totalMass;
        p1.mass = 0; p2.mass = 0;                   // both die; charge, radius, velocity stay as they were
        p1.baseMass = 0; p2.baseMass = 0;
        return s;
    }

    // handleCollisions in COL_MERGE mode over the tree just built.  Removed
    // particles are flagged `dead` and spawns are appended; the particle list is
    // compacted after the substep's force pass (compactDead), which leaves the
    // force pass exactly as the reference runs it: the removed particles are no
    // longer targets but remain in the tree with their live fields, and the
    // spawns are targets but not in the tree.
    void handleCollisions() {
        const bool per = periodic();
        const int topo = prm.topology;
        const double W = prm.domain_w, H = prm.domain_h;
        const int n = nReal();
        std::vector<int> cand, qs;
        std::vector<Spawn> spawns;
        int ann = 0;
        for (int ci = 0; ci < n; ci++) {
            Particle& p1 = ps[ci];
            if (p1.mass == 0) continue;
            query(p1.x, p1.y, p1.radius * 2, p1.radius * 2, cand, qs);
            for (int pt : cand) {
                const bool isGhost = pt >= nTree;
                const int r2 = isGhost ? ghosts[pt - nTree].orig : pt;
                Particle& p2 = ps[r2];
                if (r2 == ci || p2.mass == 0 || p1.id >= p2.id) continue;
                double qx, qy; ptPos(pt, qx, qy);
                double dx, dy;
                if (per) { Vec d = minImage(p1.x, p1.y, qx, qy, topo, W, H, W * 0.5, H * 0.5); dx = d.x; dy = d.y; }
                else { dx = qx - p1.x; dy = qy - p1.y; }
                const double distSq = dx * dx + dy * dy;
                const double minDist = p1.radius + p2.radius;
                if (!(distSq < minDist * minDist)) continue;
                if (p1.antimatter != p2.antimatter) {             // collisions.js:60-80
                    const double a = std::min(p1.mass, p2.mass);
                    const double f1 = a / p1.mass, f2 = a / p2.mass;
                    const double ke = f1 * particleKE(p1) + f2 * particleKE(p2);
                    events.push_back({ 1.0, p1.x + dx * 0.5, p1.y + dy * 0.5, 2 * a + ke,
                                       (p1.wx + p2.wx) * a, (p1.wy + p2.wy) * a });
                    ann++;
                    const double m1 = p1.mass, m2 = p2.mass;
                    p1.mass -= a; p2.mass -= a;
                    if (m1 > 0) p1.baseMass *= p1.mass / m1;
                    if (m2 > 0) p2.baseMass *= p2.mass / m2;
                    p1.setMass(p1.mass);                          // updateColor (particle.js:110-121)
                    p2.setMass(p2.mass);
                } else {                                          // collisions.js:81-91
                    const double keBefore = particleKE(p1) + particleKE(p2);
                    Spawn s = resolveMerge(p1, p2, dx, dy);
                    const double keLost = std::max(0.0, keBefore - s.ke);
                    if (keLost > 0) events.push_back({ 2.0, s.x, s.y, keLost, 0.0, 0.0 });
                    spawns.push_back(s);
                }
            }
        }
        nAnnihilations += ann;
        nMerges += (int)spawns.size();
        if (ann == 0 && spawns.empty()) return;
        for (int i = 0; i < n; i++)                                // collisions.js:96-104
            if (ps[i].mass == 0) { ps[i].dead = true; nRemovedCol++; }
        const bool rel = relOn();
        for (const Spawn& s : spawns) {                            // integrator.js:1363-1381, main.js:504-523
            Particle q;
            q.id = nextId++;
            q.x = s.x; q.y = s.y;
            q.setMass(s.mass);
            q.baseMass = s.baseMass;
            const double cq = s.charge / BOSON_CHARGE;             // Math.round: nearest, ties up
            double rq = std::floor(cq);
            if (cq - rq >= 0.5) rq += 1;
            q.charge = rq * BOSON_CHARGE;
            q.antimatter = s.antimatter;
            q.creationTime = simTime;
            q.wx = s.wx; q.wy = s.wy;
            q.angw = s.angw;
            q.angVel = rel ? angwToAngVel(q.angw, q.radius) : q.angw;
            const double invG = rel ? 1 / std::sqrt(1 + s.wx * s.wx + s.wy * s.wy) : 1;
            q.vx = s.wx * invG; q.vy = s.wy * invG;
            if (per) wrapPosition(q, topo, W, H);
            ps.push_back(q);
            nSpawned++;
        }
    }

    // Drops the particles removed by this substep's collisions, keeping order.
    void compactDead() {
        size_t w = 0;
        for (size_t i = 0; i < ps.size(); i++) {
            if (ps[i].dead) continue;
            if (w != i) ps[w] = std::move(ps[i]);
            w++;
        }
        ps.resize(w);
    }

    // ---- signal-delay.js ----
    struct Delayed { double x, y, vx, vy, angw; };
    bool getDelayedState(const Particle& src, double ox, double oy, Delayed& out) const {   // signal-delay.js:16-221
        const History& H = src.h;
        if (H.count < 2) return false;
        const bool per = periodic();
        const int topo = prm.topology;
        const double W = prm.domain_w, Hh = prm.domain_h, halfW = W * 0.5, halfH = Hh * 0.5;
        const int count = H.count;
        const int start = (H.head - count + HISTORY_SIZE) & HISTORY_MASK;
        const int newest = (H.head - 1 + HISTORY_SIZE) & HISTORY_MASK;
        const double tOldest = H.t[start];
        const double timeSpan = simTime - tOldest;
        if (timeSpan < EPS) return false;
        auto diff = [&](double ax, double ay, double bx, double by) -> Vec {
            if (per) return minImage(ax, ay, bx, by, topo, W, Hh, halfW, halfH);
            return { bx - ax, by - ay };
        };
        Vec cd = diff(ox, oy, H.x[newest], H.y[newest]);
        const double distSq = cd.x * cd.x + cd.y * cd.y;
        if (!(distSq > 4 * timeSpan * timeSpan)) {
            int lo = 0, hi = count - 2;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                int midIdx = (start + mid + 1) & HISTORY_MASK;
                double tMid = H.t[midIdx];
                Vec b = diff(ox, oy, H.x[midIdx], H.y[midIdx]);
                double g = std::sqrt(b.x * b.x + b.y * b.y) - (simTime - tMid);
                if (g < 0) lo = mid + 1; else hi = mid;
            }
            const int center = lo;
            for (int offset = 0; offset <= 1; offset++) {
                for (int dir = (offset == 0 ? 1 : -1); dir <= 1; dir += 2) {
                    int k = center + offset * dir;
                    if (k < 0 || k > count - 2) continue;
                    int loIdx = (start + k) & HISTORY_MASK;
                    int hiIdx = (loIdx + 1) & HISTORY_MASK;
                    double tLo = H.t[loIdx];
                    double segDt = H.t[hiIdx] - tLo;
                    if (segDt < EPS) continue;
                    double xLo = H.x[loIdx], yLo = H.y[loIdx], xHi = H.x[hiIdx], yHi = H.y[hiIdx];
                    double dx, dy, vx, vy;
                    if (per) {
                        Vec d = minImage(ox, oy, xLo, yLo, topo, W, Hh, halfW, halfH);
                        dx = d.x; dy = d.y;
                        Vec s = minImage(xLo, yLo, xHi, yHi, topo, W, Hh, halfW, halfH);
                        vx = s.x / segDt; vy = s.y / segDt;
                    } else {
                        dx = xLo - ox; dy = yLo - oy;
                        vx = (xHi - xLo) / segDt; vy = (yHi - yLo) / segDt;
                    }
                    double rSq = dx * dx + dy * dy, vSq = vx * vx + vy * vy, dDotV = dx * vx + dy * vy;
                    double T = simTime - tLo;
                    double a = vSq - 1, hh = dDotV + T, c = rSq - T * T;
                    double disc = hh * hh - a * c;
                    if (!(disc >= 0)) continue;
                    double sqrtDisc = std::sqrt(disc);
                    double s;
                    if (std::fabs(a) < EPS) {
                        if (std::fabs(hh) < EPS) continue;
                        s = -c / (2 * hh);
                    } else {
                        double s1 = (-hh + sqrtDisc) / a, s2 = (-hh - sqrtDisc) / a;
                        bool ok1 = s1 >= -EPS && s1 <= segDt + EPS;
                        bool ok2 = s2 >= -EPS && s2 <= segDt + EPS;
                        if (ok1 && ok2) s = std::max(s1, s2);
                        else if (ok1) s = s1;
                        else if (ok2) s = s2;
                        else continue;
                    }
                    if (s < 0) s = 0; else if (s > segDt) s = segDt;
                    double frac = s / segDt;
                    if (per) {
                        Vec sd = minImage(xLo, yLo, xHi, yHi, topo, W, Hh, halfW, halfH);
                        out.x = xLo + frac * sd.x; out.y = yLo + frac * sd.y;
                    } else {
                        out.x = xLo + frac * (xHi - xLo); out.y = yLo + frac * (yHi - yLo);
                    }
                    out.vx = H.vx[loIdx] + frac * (H.vx[hiIdx] - H.vx[loIdx]);
                    out.vy = H.vy[loIdx] + frac * (H.vy[hiIdx] - H.vy[loIdx]);
                    out.angw = H.angw[loIdx] + frac * (H.angw[hiIdx] - H.angw[loIdx]);
                    return true;
                }
            }
        }
        if (src.deathTime < INF) return false;
        {
            Vec d = diff(ox, oy, H.x[start], H.y[start]);
            double vx = H.vx[start], vy = H.vy[start];
            double rSq = d.x * d.x + d.y * d.y, vSq = vx * vx + vy * vy, dDotV = d.x * vx + d.y * vy;
            double T = timeSpan;
            double a = vSq - 1, hh = dDotV + T, c = rSq - T * T;
            double disc = hh * hh - a * c;
            if (!(disc >= 0)) return false;
            double sqrtDisc = std::sqrt(disc);
            double s;
            if (std::fabs(a) < EPS) {
                if (std::fabs(hh) < EPS) return false;
                s = -c / (2 * hh);
            } else {
                double s1 = (-hh + sqrtDisc) / a, s2 = (-hh - sqrtDisc) / a;
                bool ok1 = s1 <= EPS, ok2 = s2 <= EPS;
                if (ok1 && ok2) s = std::max(s1, s2);
                else if (ok1) s = s1;
                else if (ok2) s = s2;
                else return false;
            }
            if (s > 0) s = 0;
            if (tOldest + s < src.creationTime) return false;
            out.x = H.x[start] + vx * s; out.y = H.y[start] + vy * s;
            out.vx = vx; out.vy = vy; out.angw = H.angw[start];
            return true;
        }
    }

    // ---- pairForce (forces.js:163-442) ----
    void pairForce(Particle& p, double sx, double sy, double svx, double svy, double sMass, double sCharge,
                   double sAngVel, double sMagMoment, double sAngMomentum, const Toggles& tg,
                   double /*sAxMod*/, double /*sYukMod*/, bool signalDelayed, double /*sHiggsMod*/,
                   double yukawaCutoffSq) const {
        double rx, ry;
        if (periodic()) {
            Vec d = minImage(p.x, p.y, sx, sy, prm.topology, prm.domain_w, prm.domain_h,
                             prm.domain_w * 0.5, prm.domain_h * 0.5);
            rx = d.x; ry = d.y;
        } else { rx = sx - p.x; ry = sy - p.y; }
        const double rawRSq = rx * rx + ry * ry;
        const double rSq = rawRSq + tg.softeningSq;
        const double invRSq = 1 / rSq;
        const double invR = std::sqrt(invRSq);
        const double invR3 = invR * invRSq;
        const double invR5 = invR3 * invRSq;
        double aberr = 1;
        if (signalDelayed) {
            double nDotV = -(rx * svx + ry * svy) * invR;
            double denom = std::max(1 - nDotV, 0.01);
            aberr = std::min(1 / (denom * denom * denom), 100.0);
        }
        const double invR3a = signalDelayed ? invR3 * aberr : invR3;
        const double invR5a = signalDelayed ? invR5 * aberr : invR5;
        const double crossSV = svx * ry - svy * rx;
        const double pMagMoment = p.magMoment, pAngMomentum = p.angMomentum;

        if (tg.gravity) {
            double k = p.mass * sMass;
            double fDir = k * invR3a;
            p.fx += rx * fDir; p.fy += ry * fDir;
            p.comp[C_GRAV][0] += rx * fDir; p.comp[C_GRAV][1] += ry * fDir;
            p.pe -= k * invR;
        }
        const double axModPair = 1;   // axion off (forces.js:223)
        if (tg.coulomb) {
            double k = -(p.charge * sCharge) * axModPair;
            double fDir = k * invR3a;
            p.fx += rx * fDir; p.fy += ry * fDir;
            p.comp[C_COUL][0] += rx * fDir; p.comp[C_COUL][1] += ry * fDir;
            p.pe += p.charge * sCharge * invR * axModPair;
        }
        if (tg.onePN && (tg.gravitomag || tg.magnetic)) {
            const double r = 1 / invR;
            const double nx = rx * invR, ny = ry * invR;
            const double pvx = p.vx, pvy = p.vy;
            const double v1DotV2 = pvx * svx + pvy * svy;
            if (tg.gravitomag) {
                double v1Sq = pvx * pvx + pvy * pvy, v2Sq = svx * svx + svy * svy;
                double nDotV1 = nx * pvx + ny * pvy, nDotV2 = nx * svx + ny * svy;
                double radial = -v1Sq - 2 * v2Sq + 1.5 * nDotV2 * nDotV2 + 5 * p.mass * invR + 4 * sMass * invR;
                double v1Coeff = 4 * nDotV1 - 3 * nDotV2, v2Coeff = 3 * nDotV2;
                double base = p.mass * sMass * invR3;
                double fx = base * (rx * radial + (pvx * v1Coeff + svx * v2Coeff) * r);
                double fy = base * (ry * radial + (pvy * v1Coeff + svy * v2Coeff) * r);
                p.fx += fx; p.fy += fy;
                p.comp[C_1PN][0] += fx; p.comp[C_1PN][1] += fy;
                p.pe -= p.mass * sMass * invR * (1.5 * (v1Sq + v2Sq) - 3.5 * v1DotV2 - 0.5 * nDotV1 * nDotV2
                                                 + p.mass * invR + sMass * invR);
            }
            if (tg.magnetic) {
                double v2DotN = svx * nx + svy * ny, v1DotN = pvx * nx + pvy * ny;
                double coeff = 0.5 * p.charge * sCharge * invRSq;
                double symX = coeff * (pvx * v2DotN - 3 * nx * v1DotN * v2DotN);
                double symY = coeff * (pvy * v2DotN - 3 * ny * v1DotN * v2DotN);
                p.fx += symX; p.fy += symY;
                p.comp[C_1PN][0] += symX; p.comp[C_1PN][1] += symY;
                p.pe -= 0.5 * p.charge * sCharge * invR * (v1DotV2 + v1DotN * v2DotN);
            }
        }
        if (tg.onePN && tg.gravitomag && tg.magnetic) {
            double crossCoeff = p.charge * sCharge * (p.mass + sMass) - (p.charge * p.charge * sMass + sCharge * sCharge * p.mass);
            double fDir = crossCoeff * invRSq * invRSq;
            p.fx += rx * fDir; p.fy += ry * fDir;
            p.comp[C_1PN][0] += rx * fDir; p.comp[C_1PN][1] += ry * fDir;
            p.pe += 0.5 * crossCoeff * invRSq;
        }
        if (tg.magnetic) {
            const double axMod = axModPair;
            double fDir = -3 * (pMagMoment * sMagMoment) * invR5a * axMod;
            p.fx += rx * fDir; p.fy += ry * fDir;
            p.comp[C_MAG][0] += rx * fDir; p.comp[C_MAG][1] += ry * fDir;
            p.pe += (pMagMoment * sMagMoment) * invR3 * axMod;
            double BzMoving = sCharge * crossSV * invR3 * axMod;
            p.Bz += BzMoving;
            p.dBzdx += 3 * BzMoving * rx * invRSq + sCharge * svy * invR3 * axMod;
            p.dBzdy += 3 * BzMoving * ry * invRSq - sCharge * svx * invR3 * axMod;
            p.Bz -= sMagMoment * invR3 * axMod;
            p.dBzdx -= 3 * sMagMoment * rx * invR5 * axMod;
            p.dBzdy -= 3 * sMagMoment * ry * invR5 * axMod;
        }
        if (tg.gravitomag) {
            double fDir = 3 * (pAngMomentum * sAngMomentum) * invR5a;
            p.fx += rx * fDir; p.fy += ry * fDir;
            p.comp[C_GM][0] += rx * fDir; p.comp[C_GM][1] += ry * fDir;
            p.pe -= (pAngMomentum * sAngMomentum) * invR3;
            double BgzMoving = -sMass * crossSV * invR3;
            p.Bgz += BgzMoving;
            p.dBgzdx += 3 * BgzMoving * rx * invRSq - sMass * svy * invR3;
            p.dBgzdy += 3 * BgzMoving * ry * invRSq + sMass * svx * invR3;
            p.Bgz -= 2 * sAngMomentum * invR3;
            p.dBgzdx -= 6 * sAngMomentum * rx * invR5;
            p.dBgzdy -= 6 * sAngMomentum * ry * invR5;
            p.frameDrag += 2 * sAngMomentum * (sAngVel - p.angVel) * invR3;
        }
        if (tg.yukawa && rawRSq < yukawaCutoffSq) {
            const double mu = tg.yukawaMu;   // Higgs off (forces.js:388)
            const double r = 1 / invR;
            const double expMuR = std::exp(-mu * r);
            const double ym = 1;             // axion off (forces.js:391)
            double fDir = YUKAWA_COUPLING * ym * p.mass * sMass * expMuR * (invRSq + mu * invR) * (signalDelayed ? invR * aberr : invR);
            p.fx += rx * fDir; p.fy += ry * fDir;
            p.comp[C_YUK][0] += rx * fDir; p.comp[C_YUK][1] += ry * fDir;
            p.pe -= YUKAWA_COUPLING * ym * p.mass * sMass * expMuR * invR;
            if (tg.onePN) {
                double pvx = p.vx, pvy = p.vy;
                double nx = rx * invR, ny = ry * invR;
                double nDotV1 = nx * pvx + ny * pvy, nDotV2 = nx * svx + ny * svy;
                double v1DotV2 = pvx * svx + pvy * svy;
                double alpha = 1 + mu * r;
                double beta = 0.5 * YUKAWA_COUPLING * ym * p.mass * sMass * expMuR * invRSq;
                double radial = -(alpha * v1DotV2 + (alpha * alpha + alpha + 1) * nDotV1 * nDotV2);
                double fx = beta * (radial * nx + alpha * (nDotV2 * pvx + nDotV1 * svx));
                double fy = beta * (radial * ny + alpha * (nDotV2 * pvy + nDotV1 * svy));
                p.fx += fx; p.fy += fy;
                p.comp[C_1PN][0] += fx; p.comp[C_1PN][1] += fy;
                p.pe += 0.5 * YUKAWA_COUPLING * ym * p.mass * sMass * expMuR * invR * (v1DotV2 + nDotV1 * nDotV2 * alpha);
            }
        }
        if (tg.gravity) {
            double crossRV = rx * (svy - p.vy) - ry * (svx - p.vx);
            double wOrbit = crossRV * invRSq;
            double dw = p.angVel - wOrbit;
            double coupling = sMass;
            if (tg.coulomb && p.mass > EPS) coupling += p.charge * sCharge / p.mass;
            double bodyR = std::sqrt(p.bodyRadiusSq);
            double ri5 = p.bodyRadiusSq * p.bodyRadiusSq * bodyR;
            double invR6 = invRSq * invRSq * invRSq;
            p.tidal -= TIDAL_STRENGTH * coupling * coupling * ri5 * invR6 * dw;
        }
    }

    // ---- calculateForce: BH walk (forces.js:622-694) ----
    void calculateForce(int pi, const Toggles& tg, bool useSignalDelay, double cutSq, std::vector<int>& stack, int64_t& inter) {
        Particle& particle = ps[pi];
        const double px = particle.x, py = particle.y;
        const double thetaSq = prm.theta * prm.theta;
        const QuadTree& t = tree;
        const bool per = periodic();
        stack.clear();
        stack.push_back(root);
        while (!stack.empty()) {
            int nodeIdx = stack.back(); stack.pop_back();
            if (t.totalMass[nodeIdx] < EPS) continue;
            double dx, dy;
            if (per) {
                Vec d = minImage(px, py, t.comX[nodeIdx], t.comY[nodeIdx], prm.topology, prm.domain_w, prm.domain_h,
                                 prm.domain_w * 0.5, prm.domain_h * 0.5);
                dx = d.x; dy = d.y;
            } else { dx = t.comX[nodeIdx] - px; dy = t.comY[nodeIdx] - py; }
            const double dSq = dx * dx + dy * dy;
            const double size = t.bw[nodeIdx] * 2;
            if (!t.divided[nodeIdx] && t.pointCount[nodeIdx] > 0) {
                for (int i = 0; i < t.pointCount[nodeIdx]; i++) {
                    int other = t.points[nodeIdx * QT_CAPACITY + i];
                    if (other == pi) continue;
                    const bool isGhost = other >= nTree;
                    const int realIdx = isGhost ? ghosts[other - nTree].orig : other;
                    if (isGhost && realIdx == pi) continue;
                    const Particle& real = ps[realIdx];
                    double sx, sy, svx, svy, sAngVel, sMag, sAng, oMass, oCharge;
                    bool delayed;
                    if (isGhost) { const Ghost& g = ghosts[other - nTree]; oMass = g.mass; oCharge = g.charge; }
                    else { oMass = real.mass; oCharge = real.charge; }
                    if (useSignalDelay) {
                        if (real.h.count < 2) continue;
                        Delayed ret;
                        if (!getDelayedState(real, px, py, ret)) continue;
                        if (isGhost) {
                            const Ghost& g = ghosts[other - nTree];
                            sx = ret.x + (g.x - real.x); sy = ret.y + (g.y - real.y);
                        } else { sx = ret.x; sy = ret.y; }
                        svx = ret.vx; svy = ret.vy;
                        double retRadiusSq = real.bodyRadiusSq;
                        sAngVel = ret.angw / std::sqrt(1 + ret.angw * ret.angw * retRadiusSq);
                        sMag = MAG_MOMENT_K * oCharge * sAngVel * retRadiusSq;
                        sAng = INERTIA_K * oMass * sAngVel * retRadiusSq;
                        delayed = true;
                    } else {
                        if (isGhost) {
                            const Ghost& g = ghosts[other - nTree];
                            sx = g.x; sy = g.y; svx = g.vx; svy = g.vy;
                            sAngVel = g.angVel; sMag = g.magMoment; sAng = g.angMomentum;
                        } else {
                            sx = real.x; sy = real.y; svx = real.vx; svy = real.vy;
                            sAngVel = real.angVel; sMag = real.magMoment; sAng = real.angMomentum;
                        }
                        delayed = false;
                    }
                    pairForce(particle, sx, sy, svx, svy, oMass, oCharge, sAngVel, sMag, sAng, tg,
                              real.axMod, real.yukMod, delayed, real.higgsMod, cutSq);
                    inter++;
                }
            } else if (t.divided[nodeIdx] && (size * size < thetaSq * dSq)) {
                const double nodeMass = t.totalMass[nodeIdx];
                pairForce(particle, t.comX[nodeIdx], t.comY[nodeIdx], t.momX[nodeIdx] / nodeMass, t.momY[nodeIdx] / nodeMass,
                          nodeMass, t.totalCharge[nodeIdx], 0, t.totalMag[nodeIdx], t.totalAngMom[nodeIdx], tg,
                          1, 1, false, 1, cutSq);
                inter++;
            } else if (t.divided[nodeIdx]) {
                stack.push_back(t.nw[nodeIdx]); stack.push_back(t.ne[nodeIdx]);
                stack.push_back(t.sw[nodeIdx]); stack.push_back(t.se[nodeIdx]);
            }
        }
    }

    // ---- potential heat map (heatmap.js) ----
    // treePotential (heatmap.js:38-101) at (wx, wy): aggregates at the node's
    // centre of mass without minimum image, leaf points skip ghosts and use
    // the signal-delayed position when useDelay; no Yukawa cutoff.
    void treePotential(double wx, double wy, bool doG, bool doE, bool doY, bool useDelay, std::vector<int>& stack,
                       double& g, double& e, double& yk) const {
        const QuadTree& t = tree;
        const double thetaSq = prm.theta * prm.theta;
        const double softSq = prm.softening * prm.softening;
        const double mu = prm.yukawa_mu;
        const bool per = periodic();
        stack.clear();
        stack.push_back(root);
        while (!stack.empty()) {
            const int nodeIdx = stack.back(); stack.pop_back();
            if (t.totalMass[nodeIdx] == 0 && t.totalCharge[nodeIdx] == 0) continue;
            const double dx = t.comX[nodeIdx] - wx, dy = t.comY[nodeIdx] - wy;
            const double dSq = dx * dx + dy * dy;
            const double size = t.bw[nodeIdx] * 2;
            if (!t.divided[nodeIdx] && t.pointCount[nodeIdx] > 0) {
                double gP = 0, eP = 0, yP = 0;
                for (int i = 0; i < t.pointCount[nodeIdx]; i++) {
                    const int other = t.points[nodeIdx * QT_CAPACITY + i];
                    if (other >= nTree) continue;                   // ghosts: periodic images (heatmap.js:60)
                    const Particle& q = ps[other];
                    double pdx, pdy;
                    if (useDelay) {
                        if (q.h.count < 2) continue;
                        Delayed ret;
                        if (!getDelayedState(q, wx, wy, ret)) continue;
                        if (per) {
                            const Vec d = minImage(wx, wy, ret.x, ret.y, prm.topology, prm.domain_w, prm.domain_h,
                                                   prm.domain_w * 0.5, prm.domain_h * 0.5);
                            pdx = d.x; pdy = d.y;
                        } else { pdx = ret.x - wx; pdy = ret.y - wy; }
                    } else { pdx = q.x - wx; pdy = q.y - wy; }
                    const double rSq = pdx * pdx + pdy * pdy + softSq;
                    const double invR = 1 / std::sqrt(rSq);
                    if (doG) gP -= q.mass * invR;
                    if (doE) eP += q.charge * invR;
                    if (doY) { const double r = 1 / invR; yP -= YUKAWA_COUPLING * q.mass * std::exp(-mu * r) * invR; }
                }
                g += gP; e += eP; yk += yP;
            } else if (t.divided[nodeIdx] && (size * size < thetaSq * dSq)) {
                const double invR = 1 / std::sqrt(dSq + softSq);
                if (doG) g -= t.totalMass[nodeIdx] * invR;
                if (doE) e += t.totalCharge[nodeIdx] * invR;
                if (doY) { const double r = 1 / invR; yk -= YUKAWA_COUPLING * t.totalMass[nodeIdx] * std::exp(-mu * r) * invR; }
            } else if (t.divided[nodeIdx]) {
                stack.push_back(t.nw[nodeIdx]); stack.push_back(t.ne[nodeIdx]);
                stack.push_back(t.sw[nodeIdx]); stack.push_back(t.se[nodeIdx]);
            }
        }
    }

    // Heatmap.update's grid loop (heatmap.js:152-206, without dead
    // particles): G x G sample points at cell centres of the view rectangle.
    void heatmap(double left, double top, double cellW, double cellH, int G, bool doG, bool doE, bool doY,
                 double* gOut, double* eOut, double* yOut) {
        const bool useTree = (prm.toggles & GEON_BARNES_HUT) != 0;
        const bool useDelay = (prm.toggles & GEON_RELATIVITY) != 0;
        if (useTree) buildTree();
        const double softSq = prm.softening * prm.softening;
        const double mu = prm.yukawa_mu;
        const double cutSq = doY ? (6 / mu) * (6 / mu) : INF;          // heatmap.js:149
        const bool per = periodic();
        const int n = nReal();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nThreads)
        for (int idx = 0; idx < G * G; idx++) {
            const int gy = idx / G, gx = idx % G;
            const double wy = top + (gy + 0.5) * cellH;
            const double wx = left + (gx + 0.5) * cellW;
            double g = 0, e = 0, yk = 0;
            if (useTree && root >= 0) {
                std::vector<int> stack;
                treePotential(wx, wy, doG, doE, doY, useDelay, stack, g, e, yk);
            } else {
                for (int i = 0; i < n; i++) {
                    const Particle& q = ps[i];
                    double dx, dy;
                    if (useDelay) {
                        if (q.h.count < 2) continue;
                        Delayed ret;
                        if (!getDelayedState(q, wx, wy, ret)) continue;
                        if (per) {
                            const Vec d = minImage(wx, wy, ret.x, ret.y, prm.topology, prm.domain_w, prm.domain_h,
                                                   prm.domain_w * 0.5, prm.domain_h * 0.5);
                            dx = d.x; dy = d.y;
                        } else { dx = ret.x - wx; dy = ret.y - wy; }
                    } else if (per) {
                        const Vec d = minImage(wx, wy, q.x, q.y, prm.topology, prm.domain_w, prm.domain_h,
                                               prm.domain_w * 0.5, prm.domain_h * 0.5);
                        dx = d.x; dy = d.y;
                    } else { dx = q.x - wx; dy = q.y - wy; }
                    const double rSq = dx * dx + dy * dy + softSq;
                    const double invR = 1 / std::sqrt(rSq);
                    if (doG) g -= q.mass * invR;
                    if (doE) e += q.charge * invR;
                    if (doY && rSq < cutSq) { const double r = 1 / invR; yk -= YUKAWA_COUPLING * q.mass * std::exp(-mu * r) * invR; }
                }
            }
            gOut[idx] = g; eOut[idx] = e; yOut[idx] = yk;
        }
    }

    // Heatmap._blur (heatmap.js:278-302): separable 3 x 3 box blur, clamp to edge.
    static void blur(double* arr, int G) {
        std::vector<double> t((size_t)G * G);
        for (int y = 0; y < G; y++) {
            const int row = y * G;
            for (int x = 0; x < G; x++) {
                const double l = x > 0 ? arr[row + x - 1] : arr[row];
                const double r = x < G - 1 ? arr[row + x + 1] : arr[row + G - 1];
                t[row + x] = (l + arr[row + x] + r) * (1.0 / 3);
            }
        }
        const int lastRow = (G - 1) * G;
        for (int y = 0; y < G; y++) {
            const int rA = y > 0 ? (y - 1) * G : 0, rC = y * G, rB = y < G - 1 ? (y + 1) * G : lastRow;
            for (int x = 0; x < G; x++) arr[rC + x] = (t[rA + x] + t[rC + x] + t[rB + x]) * (1.0 / 3);
        }
    }

    // ---- resetForces (forces.js:31-54) ----
    static void resetOne(Particle& p) {
        p.fx = p.fy = 0;
        std::memset(p.comp, 0, sizeof(p.comp));
        p.Bz = p.dBzdx = p.dBzdy = 0;
        p.Bgz = p.dBgzdx = p.dBgzdy = 0;
        p.tqSpinOrbit = 0;
        p.frameDrag = 0; p.tqFrameDrag = 0;
        p.tidal = 0; p.tqTidal = 0;
        p.tqContact = 0; p.contact = 0;
    }
    void resetForces() { for (auto& p : ps) resetOne(p); }

    // ---- computeAllForces (forces.js:61-154) ----
    void computeAllForces() {
        const Toggles tg = toggles();
        const int n = nReal();
        for (auto& p : ps) p.pe = 0;
        // Particles removed by this substep's collisions are no longer in the
        // particle list: they are neither targets nor re-cached, but stay tree
        // sources with their live fields (collisions.js:98-107).
        for (int i = 0; i < n; i++) {                        // forces.js:71-76
            Particle& p = ps[i];
            if (p.dead) continue;
            const double rSq = p.bodyRadiusSq;
            p.magMoment = MAG_MOMENT_K * p.charge * p.angVel * rSq;
            p.angMomentum = INERTIA_K * p.mass * p.angVel * rSq;
        }
        const double muMin = tg.yukawaMu;                   // forces.js:82-83 (Higgs off)
        const double cutSq = tg.yukawa ? (6 / muMin) * (6 / muMin) : INF;
        const bool useSignalDelay = relOn();
        int64_t inter = 0;
        if (on(GEON_BARNES_HUT)) {
            if (root >= 0) {
#pragma omp parallel num_threads(nThreads) reduction(+:inter)
                {
                    std::vector<int> stack;
                    stack.reserve(256);
#pragma omp for schedule(dynamic, 64)
                    for (int i = 0; i < n; i++) if (!ps[i].dead) calculateForce(i, tg, useSignalDelay, cutSq, stack, inter);
                }
            }
        } else {
            const double W = prm.domain_w, H = prm.domain_h;
            (void)W; (void)H;
#pragma omp parallel for num_threads(nThreads) schedule(dynamic, 16) reduction(+:inter)
            for (int i = 0; i < n; i++) {
                Particle& p = ps[i];
                if (p.dead) continue;
                for (int j = 0; j < n; j++) {
                    if (i == j || ps[j].dead) continue;
                    const Particle& o = ps[j];
                    double sx, sy, svx, svy, sAngVel, sMag, sAng;
                    if (useSignalDelay) {
                        if (o.h.count < 2) continue;
                        Delayed ret;
                        if (!getDelayedState(o, p.x, p.y, ret)) continue;
                        sx = ret.x; sy = ret.y; svx = ret.vx; svy = ret.vy;
                        double retRadiusSq = o.bodyRadiusSq;
                        sAngVel = ret.angw / std::sqrt(1 + ret.angw * ret.angw * retRadiusSq);
                        sMag = MAG_MOMENT_K * o.charge * sAngVel * retRadiusSq;
                        sAng = INERTIA_K * o.mass * sAngVel * retRadiusSq;
                    } else {
                        sx = o.x; sy = o.y; svx = o.vx; svy = o.vy;
                        sAngVel = o.angVel; sMag = o.magMoment; sAng = o.angMomentum;
                    }
                    pairForce(p, sx, sy, svx, svy, o.mass, o.charge, sAngVel, sMag, sAng, tg,
                              o.axMod, o.yukMod, useSignalDelay, o.higgsMod, cutSq);
                    inter++;
                }
            }
        }
        interactions = inter;
        double s = 0;
        for (auto& p : ps) if (!p.dead) s += p.pe;
        pe = s * 0.5;                                        // forces.js:26
    }

    // ---- 1PN (forces.js:445-610) ----
    void accum1PN(double px, double py, double pvx, double pvy, double pMass, double pCharge,
                  double sx, double sy, double svx, double svy, double sMass, double sCharge,
                  const Toggles& tg, double& ox, double& oy) const {
        double rx, ry;
        if (periodic()) {
            Vec d = minImage(px, py, sx, sy, prm.topology, prm.domain_w, prm.domain_h, prm.domain_w * 0.5, prm.domain_h * 0.5);
            rx = d.x; ry = d.y;
        } else { rx = sx - px; ry = sy - py; }
        const double rSq = rx * rx + ry * ry + tg.softeningSq;
        const double invRSq = 1 / rSq;
        const double invR = std::sqrt(invRSq);
        const double r = 1 / invR;
        const double nx = rx * invR, ny = ry * invR;
        if (tg.gravitomag) {
            double v1Sq = pvx * pvx + pvy * pvy, v2Sq = svx * svx + svy * svy;
            double nDotV1 = nx * pvx + ny * pvy, nDotV2 = nx * svx + ny * svy;
            double radial = -v1Sq - 2 * v2Sq + 1.5 * nDotV2 * nDotV2 + 5 * pMass * invR + 4 * sMass * invR;
            double v1Coeff = 4 * nDotV1 - 3 * nDotV2, v2Coeff = 3 * nDotV2;
            double base = pMass * sMass * invRSq * invR;
            ox += base * (rx * radial + (pvx * v1Coeff + svx * v2Coeff) * r);
            oy += base * (ry * radial + (pvy * v1Coeff + svy * v2Coeff) * r);
        }
        if (tg.magnetic) {
            double v2DotN = svx * nx + svy * ny, v1DotN = pvx * nx + pvy * ny;
            double coeff = 0.5 * pCharge * sCharge * invRSq;
            ox += coeff * (pvx * v2DotN - 3 * nx * v1DotN * v2DotN);
            oy += coeff * (pvy * v2DotN - 3 * ny * v1DotN * v2DotN);
        }
        if (tg.gravitomag && tg.magnetic) {
            double crossCoeff = pCharge * sCharge * (pMass + sMass) - (pCharge * pCharge * sMass + sCharge * sCharge * pMass);
            double fDir = crossCoeff * invRSq * invRSq;
            ox += rx * fDir; oy += ry * fDir;
        }
        if (tg.yukawa) {                                     // no cutoff here (forces.js:493)
            double mu = tg.yukawaMu;
            double expMuR = std::exp(-mu * r);
            double nDotV1 = nx * pvx + ny * pvy, nDotV2 = nx * svx + ny * svy;
            double v1DotV2 = pvx * svx + pvy * svy;
            double alpha = 1 + mu * r;
            double beta = 0.5 * YUKAWA_COUPLING * 1.0 * pMass * sMass * expMuR * invRSq;
            double radial = -(alpha * v1DotV2 + (alpha * alpha + alpha + 1) * nDotV1 * nDotV2);
            ox += beta * (radial * nx + alpha * (nDotV2 * pvx + nDotV1 * svx));
            oy += beta * (radial * ny + alpha * (nDotV2 * pvy + nDotV1 * svy));
        }
    }

    void compute1PNTreeWalk(int pi, const Toggles& tg, std::vector<int>& stack, double& ox, double& oy) const {  // forces.js:511-571
        const Particle& particle = ps[pi];
        const double px = particle.x, py = particle.y, pvx = particle.vx, pvy = particle.vy;
        const double pMass = particle.mass, pCharge = particle.charge;
        const double thetaSq = prm.theta * prm.theta;
        const QuadTree& t = tree;
        stack.clear();
        stack.push_back(root);
        while (!stack.empty()) {
            int nodeIdx = stack.back(); stack.pop_back();
            if (t.totalMass[nodeIdx] < EPS) continue;
            double dx, dy;
            if (periodic()) {
                Vec d = minImage(px, py, t.comX[nodeIdx], t.comY[nodeIdx], prm.topology, prm.domain_w, prm.domain_h,
                                 prm.domain_w * 0.5, prm.domain_h * 0.5);
                dx = d.x; dy = d.y;
            } else { dx = t.comX[nodeIdx] - px; dy = t.comY[nodeIdx] - py; }
            const double dSq = dx * dx + dy * dy;
            const double size = t.bw[nodeIdx] * 2;
            if (!t.divided[nodeIdx] && t.pointCount[nodeIdx] > 0) {
                for (int i = 0; i < t.pointCount[nodeIdx]; i++) {
                    int other = t.points[nodeIdx * QT_CAPACITY + i];
                    if (other == pi) continue;
                    const bool isGhost = other >= nTree;
                    const int realIdx = isGhost ? ghosts[other - nTree].orig : other;
                    if (isGhost && realIdx == pi) continue;
                    const Particle& real = ps[realIdx];
                    double sx, sy, svx, svy, oMass, oCharge;
                    if (!isGhost) {
                        if (real.h.count < 2) continue;
                        Delayed ret;
                        if (!getDelayedState(real, px, py, ret)) continue;
                        sx = ret.x; sy = ret.y; svx = ret.vx; svy = ret.vy;
                        oMass = real.mass; oCharge = real.charge;
                    } else {
                        const Ghost& g = ghosts[other - nTree];
                        sx = g.x; sy = g.y; svx = g.vx; svy = g.vy;
                        oMass = g.mass; oCharge = g.charge;
                    }
                    accum1PN(px, py, pvx, pvy, pMass, pCharge, sx, sy, svx, svy, oMass, oCharge, tg, ox, oy);
                }
            } else if (t.divided[nodeIdx] && (size * size < thetaSq * dSq)) {
                const double nodeMass = t.totalMass[nodeIdx];
                accum1PN(px, py, pvx, pvy, pMass, pCharge, t.comX[nodeIdx], t.comY[nodeIdx],
                         t.momX[nodeIdx] / nodeMass, t.momY[nodeIdx] / nodeMass, nodeMass, t.totalCharge[nodeIdx], tg, ox, oy);
            } else if (t.divided[nodeIdx]) {
                stack.push_back(t.nw[nodeIdx]); stack.push_back(t.ne[nodeIdx]);
                stack.push_back(t.sw[nodeIdx]); stack.push_back(t.se[nodeIdx]);
            }
        }
    }

    void compute1PN(bool bhOn) {                                     // forces.js:578-610
        const Toggles tg = toggles();
        const int n = nReal();
        for (auto& p : ps) { p.comp[C_1PN][0] = 0; p.comp[C_1PN][1] = 0; }
        if (bhOn && root >= 0) {
#pragma omp parallel num_threads(nThreads)
            {
                std::vector<int> stack;
#pragma omp for schedule(dynamic, 64)
                for (int i = 0; i < n; i++) {
                    double ox = 0, oy = 0;
                    compute1PNTreeWalk(i, tg, stack, ox, oy);
                    ps[i].comp[C_1PN][0] += ox; ps[i].comp[C_1PN][1] += oy;
                }
            }
        } else {
#pragma omp parallel for num_threads(nThreads) schedule(dynamic, 16)
            for (int i = 0; i < n; i++) {
                Particle& p = ps[i];
                double ox = 0, oy = 0;
                for (int j = 0; j < n; j++) {
                    if (i == j) continue;
                    const Particle& o = ps[j];
                    if (o.h.count < 2) continue;
                    Delayed ret;
                    if (!getDelayedState(o, p.x, p.y, ret)) continue;
                    accum1PN(p.x, p.y, p.vx, p.vy, p.mass, p.charge, ret.x, ret.y, ret.vx, ret.vy, o.mass, o.charge, tg, ox, oy);
                }
                p.comp[C_1PN][0] += ox; p.comp[C_1PN][1] += oy;
            }
        }
    }

    // ---- external fields / bounce walls (integrator.js:553-660) ----
    void applyExternalFields() {
        const double g = prm.ext_gravity, E = prm.ext_electric, Bext = prm.ext_bz;
        if (g == 0 && E == 0 && Bext == 0) return;
        const double gx = g * std::cos(prm.ext_gravity_angle), gy = g * std::sin(prm.ext_gravity_angle);
        const double ex = E * std::cos(prm.ext_electric_angle), ey = E * std::sin(prm.ext_electric_angle);
        for (auto& p : ps) {
            if (g != 0) { double fx = p.mass * gx, fy = p.mass * gy; p.fx += fx; p.fy += fy; p.comp[C_EXT][0] += fx; p.comp[C_EXT][1] += fy; }
            if (E != 0) { double fx = p.charge * ex, fy = p.charge * ey; p.fx += fx; p.fy += fy; p.comp[C_EXT][0] += fx; p.comp[C_EXT][1] += fy; }
            if (Bext != 0) p.Bz += Bext;
        }
    }
    void applyBoundaryForces() {
        const double friction = prm.bounce_friction;
        const double left = prm.off_x, top = prm.off_y, right = prm.off_x + prm.domain_w, bottom = prm.off_y + prm.domain_h;
        auto clamp1 = [](double v) { return std::max(-1.0, std::min(1.0, v)); };
        for (auto& p : ps) {
            const double r = p.radius;
            double delta = r - (p.x - left);
            if (delta > 0) {
                double Fn = delta * std::sqrt(delta);
                p.fx += Fn; p.comp[C_EXT][0] += Fn;
                if (friction > 0) { double vt = p.vy + p.angVel * r; double Ft = -friction * Fn * clamp1(vt * 10); p.fy += Ft; p.contact += r * Ft; }
            }
            delta = r - (right - p.x);
            if (delta > 0) {
                double Fn = delta * std::sqrt(delta);
                p.fx -= Fn; p.comp[C_EXT][0] -= Fn;
                if (friction > 0) { double vt = -p.vy - p.angVel * r; double Ft = -friction * Fn * clamp1(vt * 10); p.fy -= Ft; p.contact -= r * Ft; }
            }
            delta = r - (p.y - top);
            if (delta > 0) {
                double Fn = delta * std::sqrt(delta);
                p.fy += Fn; p.comp[C_EXT][1] += Fn;
                if (friction > 0) { double vt = -p.vx + p.angVel * r; double Ft = -friction * Fn * clamp1(vt * 10); p.fx -= Ft; p.contact += r * Ft; }
            }
            delta = r - (bottom - p.y);
            if (delta > 0) {
                double Fn = delta * std::sqrt(delta);
                p.fy -= Fn; p.comp[C_EXT][1] -= Fn;
                if (friction > 0) { double vt = p.vx - p.angVel * r; double Ft = -friction * Fn * clamp1(vt * 10); p.fx += Ft; p.contact -= r * Ft; }
            }
        }
    }

    // One force pass at the current state (integrator.js:754-780 without fields/bosons).
    // ---- boson tree (integrator.js:263-277, quadtree.js:316-368) ----
    void buildBosonTree() {
        broot = -1;
        if (bosons.empty()) return;
        const double bxr = prm.off_x + prm.domain_w / 2, byr = prm.off_y + prm.domain_h / 2;
        const double bwr = prm.domain_w * 2, bhr = prm.domain_h * 2;
        const int nb = (int)bosons.size();
        btree.count = 0;
        btree.overflow = false;
        btree.nodeLimit = (size_t)64 * (nb + 16);
        if (btree.bx.size() < (size_t)2 * nb + 16) btree.grow((size_t)2 * nb + 16);
        const int r = btree.alloc(bxr, byr, bwr, bhr, 0);
        std::vector<std::pair<int, int>> work;
        auto pos = [this](int i, double& x, double& y) { x = bosons[i].x; y = bosons[i].y; };
        for (int i = 0; i < nb; i++) btree.insert(r, i, pos, work);
        // calculateBosonDistribution: post-order sums of _srcMass, _srcCharge, COM by _srcMass
        QuadTree& t = btree;
        std::vector<int> stack, order;
        stack.push_back(r);
        while (!stack.empty()) {
            const int idx = stack.back(); stack.pop_back();
            order.push_back(idx);
            if (t.divided[idx]) { stack.push_back(t.nw[idx]); stack.push_back(t.ne[idx]); stack.push_back(t.sw[idx]); stack.push_back(t.se[idx]); }
        }
        for (int k = (int)order.size() - 1; k >= 0; k--) {
            const int idx = order[k];
            if (!t.divided[idx]) {
                const int cnt = t.pointCount[idx];
                if (cnt == 0) continue;
                double mass = 0, charge = 0, cx = 0, cy = 0;
                for (int i = 0; i < cnt; i++) {
                    const Boson& b = bosons[t.points[idx * QT_CAPACITY + i]];
                    mass += b.srcMass; charge += b.srcCharge;
                    cx += b.x * b.srcMass; cy += b.y * b.srcMass;
                }
                t.totalMass[idx] = mass; t.totalCharge[idx] = charge;
                if (mass > 0) { t.comX[idx] = cx / mass; t.comY[idx] = cy / mass; }
            } else {
                const int c0 = t.nw[idx], c1 = t.ne[idx], c2 = t.sw[idx], c3 = t.se[idx];
                const double m0 = t.totalMass[c0], m1 = t.totalMass[c1], m2 = t.totalMass[c2], m3 = t.totalMass[c3];
                const double mass = m0 + m1 + m2 + m3;
                t.totalMass[idx] = mass;
                t.totalCharge[idx] = t.totalCharge[c0] + t.totalCharge[c1] + t.totalCharge[c2] + t.totalCharge[c3];
                if (mass > 0) {
                    t.comX[idx] = (t.comX[c0] * m0 + t.comX[c1] * m1 + t.comX[c2] * m2 + t.comX[c3] * m3) / mass;
                    t.comY[idx] = (t.comY[c0] * m0 + t.comY[c1] * m1 + t.comY[c2] * m2 + t.comY[c3] * m3) / mass;
                }
            }
        }
        broot = r;
    }

    // _walkBosonTreeCore (forces.js:713-770): softened monopole sum of the
    // boson pool's mass (or charge) at (px, py), times `scale`.
    Vec walkBosonTree(double px, double py, double scale, double softSq, bool byCharge) const {
        const QuadTree& t = btree;
        double kx = 0, ky = 0;
        if (broot < 0) return { 0, 0 };
        const bool per = periodic();
        const double W = prm.domain_w, H = prm.domain_h;
        const double thetaSq = prm.theta * prm.theta;
        std::vector<int> stack;
        stack.push_back(broot);
        while (!stack.empty()) {
            const int idx = stack.back(); stack.pop_back();
            if (byCharge ? t.totalCharge[idx] == 0 : t.totalMass[idx] < EPS) continue;
            double dx, dy;
            if (per) { Vec d = minImage(px, py, t.comX[idx], t.comY[idx], prm.topology, W, H, W * 0.5, H * 0.5); dx = d.x; dy = d.y; }
            else { dx = t.comX[idx] - px; dy = t.comY[idx] - py; }
            const double dSq = dx * dx + dy * dy;
            const double size = t.bw[idx] * 2;
            const int cnt = t.pointCount[idx];
            if (!t.divided[idx] && cnt > 0) {
                for (int k = 0; k < cnt; k++) {
                    const Boson& b = bosons[t.points[idx * QT_CAPACITY + k]];
                    const double val = byCharge ? b.srcCharge : b.srcMass;
                    if (byCharge && val == 0) continue;
                    double bdx, bdy;
                    if (per) { Vec d = minImage(px, py, b.x, b.y, prm.topology, W, H, W * 0.5, H * 0.5); bdx = d.x; bdy = d.y; }
                    else { bdx = b.x - px; bdy = b.y - py; }
                    const double rSq = bdx * bdx + bdy * bdy + softSq;
                    const double invRSq = 1 / rSq;
                    const double f = scale * val * std::sqrt(invRSq) * invRSq;
                    kx += bdx * f; ky += bdy * f;
                }
            } else if (t.divided[idx] && size * size < thetaSq * dSq) {
                const double rSq = dSq + softSq;
                const double invRSq = 1 / rSq;
                const double f = scale * (byCharge ? t.totalCharge[idx] : t.totalMass[idx]) * std::sqrt(invRSq) * invRSq;
                kx += dx * f; ky += dy * f;
            } else if (t.divided[idx]) {
                stack.push_back(t.nw[idx]); stack.push_back(t.ne[idx]);
                stack.push_back(t.sw[idx]); stack.push_back(t.se[idx]);
            }
        }
        return { kx, ky };
    }

    bool bosonsOn() const { return (prm.flags & GEON_FLAG_BOSONS) && !bosons.empty(); }

    // computeBosonGravity (forces.js:788-804): boson mass acting on the particles.
    void bosonGravity() {
        if (!bosonsOn() || !on(GEON_GRAVITY)) return;
        buildBosonTree();
        if (broot < 0 || btree.totalMass[broot] < EPS) return;
        const double softSq = prm.softening * prm.softening;
#pragma omp parallel for num_threads(nThreads) schedule(dynamic, 64)
        for (int i = 0; i < nReal(); i++) {
            Particle& p = ps[i];
            if (p.dead) continue;
            const Vec k = walkBosonTree(p.x, p.y, p.mass, softSq, false);
            p.fx += k.x; p.fy += k.y;
            p.comp[C_GRAV][0] += k.x; p.comp[C_GRAV][1] += k.y;
        }
    }

    // The kicks of applyBosonBosonGravity (forces.js:812-856; photons 2 dt,
    // massive bosons (1 + v^2) dt, before the photons' renormalisation) and
    // applyPionPionCoulomb (forces.js:878-901; -q dt for charged massive bosons).
    void bosonKicks(double dt, unsigned what, double* out) {
        buildBosonTree();
        const int nb = (int)bosons.size();
        int massive = 0;
        for (const Boson& b : bosons) massive += b.kind != 0;
        for (int i = 0; i < nb; i++) {
            const Boson& b = bosons[i];
            double kx = 0, ky = 0;
            if ((what & 1) && broot >= 0 && btree.totalMass[broot] >= EPS && nb >= 2) {
                const double scale = b.kind == 0 ? 2 * dt : (1 + b.vSq) * dt;
                const Vec k = walkBosonTree(b.x, b.y, scale, BOSON_SOFTENING_SQ, false);
                kx += k.x; ky += k.y;
            }
            if ((what & 2) && broot >= 0 && b.kind != 0 && b.srcCharge != 0 && massive >= 2) {   // nPi + nLe >= 2
                const Vec k = walkBosonTree(b.x, b.y, -b.srcCharge * dt, BOSON_SOFTENING_SQ, true);
                kx += k.x; ky += k.y;
            }
            out[2 * i] = kx; out[2 * i + 1] = ky;
        }
    }

    void forcePass(bool rebuild) {
        resetForces();
        if (rebuild) buildTree();
        computeAllForces();
        applyExternalFields();
        bosonGravity();                                          // integrator.js:773-777
        if (prm.boundary_mode == GEON_BOUND_BOUNCE) applyBoundaryForces();
    }

    // ---- Physics.update (integrator.js:726-1825), in-scope part ----
    int update(double dt) {
        events.clear();
        nMerges = nAnnihilations = nSpawned = nRemovedCol = 0;
        const int n0 = nReal();
        const bool relOn_ = relOn();
        const Toggles tg = toggles();
        if (!forcesInit && n0 > 0) {                                 // integrator.js:750-782
            for (auto& p : ps) p.angVel = relOn_ ? angwToAngVel(p.angw, p.radius) : p.angw;
            forcePass(true);
            forcesInit = true;
        }
        int n = nReal();
        const bool hasGrav = on(GEON_GRAVITY), hasMagnetic = on(GEON_MAGNETIC), hasGM = on(GEON_GRAVITOMAG);
        const bool hasExtBz = prm.ext_bz != 0;
        double dtRemain = dt;
        int totalSteps = 0;
        double prevMaxAccelSq = 0;
        const int maxSub = prm.max_substeps > 0 ? prm.max_substeps : 32;
        while (dtRemain > EPS && totalSteps < maxSub) {             // integrator.js:810
            double maxAccelSq = 0, maxCyclotron = 0;
            for (int i = 0; i < n; i++) {
                const Particle& p = ps[i];
                if (totalSteps == 0) {
                    double aSq = (p.fx * p.fx + p.fy * p.fy) * p.invMass * p.invMass;
                    if (aSq > maxAccelSq) maxAccelSq = aSq;
                }
                if (hasMagnetic || hasExtBz) {
                    double absBz = p.Bz > 0 ? p.Bz : -p.Bz;
                    if (absBz > 0) {
                        double absQ = p.charge > 0 ? p.charge : -p.charge;
                        double wc = absQ * absBz * p.invMass;
                        if (wc > maxCyclotron) maxCyclotron = wc;
                    }
                }
                if (hasGM) {
                    double absBgz = p.Bgz > 0 ? p.Bgz : -p.Bgz;
                    if (absBgz > 0) { double wc = 4 * absBgz; if (wc > maxCyclotron) maxCyclotron = wc; }
                }
            }
            if (totalSteps != 0) maxAccelSq = prevMaxAccelSq;
            double aMax = std::sqrt(maxAccelSq);
            if (aMax != aMax) aMax = 0;
            double dtSafe = aMax > EPS ? std::sqrt(prm.softening / aMax) : dtRemain;
            if (maxCyclotron > 0) {
                double dtCyc = 0.7853981633974483 / maxCyclotron;
                if (dtCyc < dtSafe) dtSafe = dtCyc;
            }
            const int budgetLeft = maxSub - totalSteps;
            const double need = std::ceil(dtRemain / dtSafe);
            const double stepsNeeded = std::min(need, (double)budgetLeft);
            const double dtSub = dtRemain / stepsNeeded;
            totalSteps++;
            dtRemain -= dtSub;
            const bool has1PN = tg.onePN;
            const double halfDt = dtSub * 0.5;
            const bool needBoris = hasMagnetic || hasGM || hasExtBz;
            double nextMaxAccelSq = 0;
            for (int i = 0; i < n; i++) {                            // integrator.js:884-927
                Particle& p = ps[i];
                const double invM = p.invMass;
                const double halfDtOverM = halfDt * invM;
                if (has1PN) { p.f1pnOldx = p.comp[C_1PN][0]; p.f1pnOldy = p.comp[C_1PN][1]; }
                const double fx = p.fx, fy = p.fy;
                p.wx += fx * halfDtOverM; p.wy += fy * halfDtOverM;
                if (needBoris) {
                    double t = 0;
                    if (hasMagnetic || hasExtBz) t += (p.charge * 0.5 * invM) * p.Bz;
                    if (hasGM) t += 2 * p.Bgz;
                    if (t != 0) {
                        double gamma = relOn_ ? std::sqrt(1 + p.wx * p.wx + p.wy * p.wy) : 1;
                        t *= dtSub / gamma;
                        double s = 2 * t / (1 + t * t);
                        double wx = p.wx, wy = p.wy;
                        double wpx = wx + wy * t, wpy = wy - wx * t;
                        p.wx = wx + wpy * s; p.wy = wy - wpx * s;
                    }
                }
                p.wx += fx * halfDtOverM; p.wy += fy * halfDtOverM;
                if (p.wx != p.wx || p.wy != p.wy) { p.wx = 0; p.wy = 0; p.vx = 0; p.vy = 0; }
                double aSq = (fx * fx + fy * fy) * invM * invM;
                if (aSq > nextMaxAccelSq) nextMaxAccelSq = aSq;
            }
            prevMaxAccelSq = nextMaxAccelSq;
            const bool needSpinOrbit = on(GEON_SPIN_ORBIT) && (hasMagnetic || hasGM);   // integrator.js:930-982
            const bool needTorques = (hasGM && relOn_) || hasGrav;
            if (needSpinOrbit || needTorques) {
                for (int i = 0; i < n; i++) {
                    Particle& p = ps[i];
                    if (needSpinOrbit && std::fabs(p.angVel) >= EPS) {
                        const double IxOmega = p.angMomentum;
                        if (std::fabs(IxOmega) >= EPS) {
                            const double dtOverM = dtSub * p.invMass;
                            if (hasMagnetic && std::fabs(p.charge) > EPS) {
                                const double mu = p.magMoment;
                                p.angw -= mu * (p.vx * p.dBzdx + p.vy * p.dBzdy) * dtSub / IxOmega;
                                p.wx += mu * p.dBzdx * dtOverM; p.wy += mu * p.dBzdy * dtOverM;
                            }
                            if (hasGM) {
                                const double L = p.angMomentum;
                                p.angw -= L * (p.vx * p.dBgzdx + p.vy * p.dBgzdy) * dtSub / IxOmega;
                                p.wx -= L * p.dBgzdx * dtOverM; p.wy -= L * p.dBgzdy * dtOverM;
                            }
                            if (p.angw != p.angw) p.angw = 0;
                            const double sr = p.angw * p.radius;
                            p.angVel = relOn_ ? p.angw / std::sqrt(1 + sr * sr) : p.angw;
                        }
                    }
                    if (needTorques) {
                        double torque = 0;
                        if (hasGM && relOn_) torque += p.frameDrag;
                        if (hasGrav) torque += p.tidal;
                        torque += p.contact;
                        if (torque != 0) {
                            const double I = INERTIA_K * p.mass * p.radiusSq;
                            if (I >= EPS) {
                                p.angw += torque * dtSub / I;
                                if (p.angw != p.angw) p.angw = 0;
                                const double sr = p.angw * p.radius;
                                p.angVel = relOn_ ? p.angw / std::sqrt(1 + sr * sr) : p.angw;
                            }
                        }
                    }
                }
            }
            for (int i = 0; i < n; i++) {                            // integrator.js:1270-1278
                Particle& p = ps[i];
                const double invG = relOn_ ? 1 / std::sqrt(1 + p.wx * p.wx + p.wy * p.wy) : 1;
                p.vx = p.wx * invG; p.vy = p.wy * invG;
                p.angVel = relOn_ ? angwToAngVel(p.angw, p.radius) : p.angw;
                p.x += p.vx * dtSub; p.y += p.vy * dtSub;
            }
            simTime += dtSub;
            bool haveVVTree = false;
            if (has1PN) {                                            // integrator.js:1297-1318
                const bool bhOn = on(GEON_BARNES_HUT);
                if (bhOn) { buildTree(); haveVVTree = true; }
                compute1PN(bhOn);
                for (int i = 0; i < n; i++) {
                    Particle& p = ps[i];
                    const double halfDtOverM = halfDt * p.invMass;
                    p.wx += (p.comp[C_1PN][0] - p.f1pnOldx) * halfDtOverM;
                    p.wy += (p.comp[C_1PN][1] - p.f1pnOldy) * halfDtOverM;
                    if (p.wx != p.wx || p.wy != p.wy) { p.wx = 0; p.wy = 0; p.vx = 0; p.vy = 0; }
                }
            }
            if (!haveVVTree) buildTree();                            // integrator.js:1340-1347
            const bool merge = prm.collision_mode == GEON_COL_MERGE;
            if (merge) handleCollisions();                           // integrator.js:1350-1381
            resetForces();                                           // integrator.js:1490-1493
            computeAllForces();
            applyExternalFields();
            bosonGravity();                                          // integrator.js:1508-1513
            if (prm.boundary_mode == GEON_BOUND_BOUNCE) applyBoundaryForces();
            if (merge) { compactDead(); n = nReal(); }
        }
        lastSubsteps = totalSteps;
        if (relOn_ && n > 0 && ++histStride >= HISTORY_STRIDE) {    // integrator.js:1550-1565
            histStride -= HISTORY_STRIDE;
            for (auto& p : ps) {
                p.h.init();
                const int hh = p.h.head;
                p.h.x[hh] = p.x; p.h.y[hh] = p.y; p.h.vx[hh] = p.vx; p.h.vy[hh] = p.vy;
                p.h.angw[hh] = p.angw; p.h.t[hh] = simTime;
                p.h.head = (hh + 1) & HISTORY_MASK;
                if (p.h.count < HISTORY_SIZE) p.h.count++;
            }
        }
        // display torques (integrator.js:1788-1790)
        for (auto& p : ps) {
            if (hasGM && relOn_ && p.frameDrag != 0) p.tqFrameDrag = p.frameDrag;
            if (hasGrav && p.tidal != 0) p.tqTidal = p.tidal;
        }
        // boundary (integrator.js:1798-1824)
        size_t write = 0;
        const double left = prm.off_x, top = prm.off_y, right = prm.off_x + prm.domain_w, bottom = prm.off_y + prm.domain_h;
        for (size_t i = 0; i < ps.size(); i++) {
            Particle& p = ps[i];
            if (prm.boundary_mode == GEON_BOUND_DESPAWN) {
                if (p.x < left - DESPAWN_MARGIN || p.x > right + DESPAWN_MARGIN ||
                    p.y < top - DESPAWN_MARGIN || p.y > bottom + DESPAWN_MARGIN) continue;
            } else if (prm.boundary_mode == GEON_BOUND_LOOP) {
                wrapPosition(p, prm.topology, prm.domain_w, prm.domain_h);
            } else if (prm.boundary_mode == GEON_BOUND_BOUNCE) {
                if (p.x < left) p.x = left; else if (p.x > right) p.x = right;
                if (p.y < top) p.y = top; else if (p.y > bottom) p.y = bottom;
            }
            if (write != i) ps[write] = std::move(ps[i]);
            write++;
        }
        ps.resize(write);
        return totalSteps;
    }
};

}  // namespace

// =============================================================================
// C API (ctypes)
// =============================================================================
extern "C" {

void* oracle_create(const GeonParams* prm) {
    if (!prm) return nullptr;
    Sim* s = new Sim();
    s->prm = *prm;
    if (s->prm.theta <= 0) s->prm.theta = 0.5;
    if (s->prm.softening <= 0) s->prm.softening = 8;
    if (s->prm.max_substeps <= 0) s->prm.max_substeps = 32;
    return s;
}
void oracle_destroy(void* h) { delete static_cast<Sim*>(h); }
void oracle_set_params(void* h, const GeonParams* prm) { static_cast<Sim*>(h)->prm = *prm; }
void oracle_set_threads(void* h, int n) { static_cast<Sim*>(h)->nThreads = n > 0 ? n : 1; }
int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Add n particles from raw state (x, y, wx, wy, mass, charge, angw), as the
// library's geon_add_particles does: vel = w/gamma (w when relativity is off),
// angVel from angw, radius = cbrt(mass), creationTime stamp.
int oracle_add_particles(void* h, int n, const double* x, const double* y, const double* wx, const double* wy,
                         const double* mass, const double* charge, const double* angw, double creationTime) {
    Sim* s = static_cast<Sim*>(h);
    const bool rel = s->relOn();
    for (int i = 0; i < n; i++) {
        Particle p;
        p.id = s->nextId++;
        p.x = x[i]; p.y = y[i];
        p.setMass(mass[i]);
        p.baseMass = mass[i];
        p.charge = charge[i];
        p.wx = wx[i]; p.wy = wy[i];
        if (rel) {
            double invG = 1 / std::sqrt(1 + p.wx * p.wx + p.wy * p.wy);
            p.vx = p.wx * invG; p.vy = p.wy * invG;
        } else { p.vx = p.wx; p.vy = p.wy; }
        p.angw = angw[i];
        p.angVel = rel ? angwToAngVel(p.angw, p.radius) : p.angw;
        p.creationTime = creationTime;
        s->ps.push_back(std::move(p));
    }
    return (int)s->ps.size();
}

int oracle_count(void* h) { return (int)static_cast<Sim*>(h)->ps.size(); }

// Boson pool: n rows of 6 doubles (x, y, src_mass, src_charge, kind, vSq);
// kind 0 = photon, 1 = pion or lepton.
void oracle_set_bosons(void* h, int n, const double* rows) {
    Sim* s = static_cast<Sim*>(h);
    s->bosons.resize(n);
    for (int i = 0; i < n; i++) {
        const double* r = rows + (size_t)i * 6;
        s->bosons[i] = { r[0], r[1], r[2], r[3], r[5], (int)r[4] };
    }
}
// Kicks of the boson pool on itself (what: 1 gravity, 2 Coulomb), 2 doubles per boson.
void oracle_boson_kicks(void* h, double dt, unsigned what, double* out) { static_cast<Sim*>(h)->bosonKicks(dt, what, out); }

// Antimatter flags and base masses of the first n particles (null: unchanged).
void oracle_set_matter(void* h, int n, const int* antimatter, const double* base_mass) {
    Sim* s = static_cast<Sim*>(h);
    for (int i = 0; i < n && i < (int)s->ps.size(); i++) {
        if (antimatter) s->ps[i].antimatter = antimatter[i] != 0;
        if (base_mass) s->ps[i].baseMass = base_mass[i];
    }
}
int oracle_get_matter(void* h, int* antimatter, double* base_mass, int cap) {
    Sim* s = static_cast<Sim*>(h);
    const int n = std::min(cap, (int)s->ps.size());
    for (int i = 0; i < n; i++) { antimatter[i] = s->ps[i].antimatter ? 1 : 0; base_mass[i] = s->ps[i].baseMass; }
    return n;
}
// Collision events of the last update, 6 doubles each (type, x, y, energy,
// px, py); returns the number of events (all of them, even beyond cap).
int oracle_collision_events(void* h, double* out, int cap) {
    Sim* s = static_cast<Sim*>(h);
    for (int k = 0; k < (int)s->events.size() && k < cap; k++)
        for (int c = 0; c < 6; c++) out[(size_t)k * 6 + c] = s->events[k][c];
    return (int)s->events.size();
}
// merges, annihilations, spawned particles, removed particles of the last update
void oracle_collision_counts(void* h, int* out) {
    Sim* s = static_cast<Sim*>(h);
    out[0] = s->nMerges; out[1] = s->nAnnihilations; out[2] = s->nSpawned; out[3] = s->nRemovedCol;
}
void oracle_set_sim_time(void* h, double t) { static_cast<Sim*>(h)->simTime = t; }
double oracle_sim_time(void* h) { return static_cast<Sim*>(h)->simTime; }
int oracle_last_substeps(void* h) { return static_cast<Sim*>(h)->lastSubsteps; }
long long oracle_interactions(void* h) { return static_cast<Sim*>(h)->interactions; }
double oracle_pe(void* h) { return static_cast<Sim*>(h)->pe; }
void oracle_set_forces_init(void* h, int v) { static_cast<Sim*>(h)->forcesInit = v != 0; }

int oracle_update(void* h, double dt) { return static_cast<Sim*>(h)->update(dt); }

// Bootstrap-style force pass at the current state (no state change).
void oracle_compute_forces(void* h) {
    Sim* s = static_cast<Sim*>(h);
    s->forcePass(s->on(GEON_BARNES_HUT));
}
// Force pass over the tree built by the last oracle_build_tree (or none for the pairwise sum).
void oracle_compute_forces_no_build(void* h) {
    Sim* s = static_cast<Sim*>(h);
    s->forcePass(false);
}
// computeAllForces restricted to the listed target particles, over the tree
// built by the last oracle_build_tree (BH) or all sources (pairwise): the
// bounded CPU sample of the timed baseline.  Returns the interaction count.
long long oracle_compute_forces_subset(void* h, const int* idx, int k) {
    Sim* s = static_cast<Sim*>(h);
    const Toggles tg = s->toggles();
    for (int i = 0; i < s->nReal(); i++) {
        Particle& p = s->ps[i];
        p.magMoment = MAG_MOMENT_K * p.charge * p.angVel * p.bodyRadiusSq;
        p.angMomentum = INERTIA_K * p.mass * p.angVel * p.bodyRadiusSq;
    }
    const double cutSq = tg.yukawa ? (6 / tg.yukawaMu) * (6 / tg.yukawaMu) : INF;
    int64_t inter = 0;
#pragma omp parallel num_threads(s->nThreads) reduction(+:inter)
    {
        std::vector<int> stack;
#pragma omp for schedule(dynamic, 16)
        for (int t = 0; t < k; t++) {
            const int i = idx[t];
            Sim::resetOne(s->ps[i]);
            s->ps[i].pe = 0;
            if (s->on(GEON_BARNES_HUT)) {
                if (s->root >= 0) s->calculateForce(i, tg, s->relOn(), cutSq, stack, inter);
                continue;
            }
            Particle& p = s->ps[i];                                  // the pairwise branch (forces.js:94-125)
            for (int j = 0; j < s->nReal(); j++) {
                if (j == i) continue;
                const Particle& o = s->ps[j];
                if (s->relOn()) {
                    if (o.h.count < 2) continue;
                    Sim::Delayed ret;
                    if (!s->getDelayedState(o, p.x, p.y, ret)) continue;
                    const double rr = o.bodyRadiusSq;
                    const double av = ret.angw / std::sqrt(1 + ret.angw * ret.angw * rr);
                    s->pairForce(p, ret.x, ret.y, ret.vx, ret.vy, o.mass, o.charge, av, MAG_MOMENT_K * o.charge * av * rr,
                                 INERTIA_K * o.mass * av * rr, tg, o.axMod, o.yukMod, true, o.higgsMod, cutSq);
                } else {
                    s->pairForce(p, o.x, o.y, o.vx, o.vy, o.mass, o.charge, o.angVel, o.magMoment, o.angMomentum, tg,
                                 o.axMod, o.yukMod, false, o.higgsMod, cutSq);
                }
                inter++;
            }
        }
    }
    return inter;
}

// 1PN-only pass (compute1PN) at the current state.
void oracle_compute_1pn(void* h) {
    Sim* s = static_cast<Sim*>(h);
    const bool bh = s->on(GEON_BARNES_HUT);
    if (bh) s->buildTree();
    s->compute1PN(bh);
}

// State rows: x, y, wx, wy, mass, charge, angw, vx, vy, angVel (each n doubles).
int oracle_get_state(void* h, double* out, int cap) {
    Sim* s = static_cast<Sim*>(h);
    int n = (int)s->ps.size();
    if (n > cap) n = cap;
    for (int i = 0; i < n; i++) {
        const Particle& p = s->ps[i];
        double v[10] = { p.x, p.y, p.wx, p.wy, p.mass, p.charge, p.angw, p.vx, p.vy, p.angVel };
        for (int r = 0; r < 10; r++) out[(size_t)r * cap + i] = v[r];
    }
    return n;
}
void oracle_get_ids(void* h, int* ids, int cap) {
    Sim* s = static_cast<Sim*>(h);
    int n = std::min(cap, (int)s->ps.size());
    for (int i = 0; i < n; i++) ids[i] = s->ps[i].id;
}

// Force rows in GEON_OUT_* order.
int oracle_get_forces(void* h, double* out, int cap) {
    Sim* s = static_cast<Sim*>(h);
    int n = std::min(cap, (int)s->ps.size());
    for (int i = 0; i < n; i++) {
        const Particle& p = s->ps[i];
        double v[GEON_OUT_ROWS] = {
            p.fx, p.fy, p.Bz, p.Bgz, p.dBzdx, p.dBzdy, p.dBgzdx, p.dBgzdy, p.tidal, p.frameDrag,
            p.comp[C_1PN][0], p.comp[C_1PN][1], p.pe,
            p.comp[C_GRAV][0], p.comp[C_GRAV][1], p.comp[C_COUL][0], p.comp[C_COUL][1],
            p.comp[C_MAG][0], p.comp[C_MAG][1], p.comp[C_GM][0], p.comp[C_GM][1],
            p.comp[C_YUK][0], p.comp[C_YUK][1], p.comp[C_EXT][0], p.comp[C_EXT][1] };
        for (int r = 0; r < GEON_OUT_ROWS; r++) out[(size_t)r * cap + i] = v[r];
    }
    return n;
}

// Potential heat map (heatmap.js:152-206, 278-302): fields bit 1 gravity,
// 2 electric, 4 Yukawa (each also needs its force toggle); blur != 0 applies
// the 3 x 3 box blur to each computed field.  Outputs G*G doubles each.
void oracle_heatmap(void* h, double left, double top, double cell_w, double cell_h, int G, unsigned fields, int blur,
                    double* g, double* e, double* y) {
    Sim* s = static_cast<Sim*>(h);
    const unsigned tg = s->prm.toggles;
    const bool doG = (fields & 1u) && (tg & GEON_GRAVITY);
    const bool doE = (fields & 2u) && (tg & GEON_COULOMB);
    const bool doY = (fields & 4u) && (tg & GEON_YUKAWA);
    s->heatmap(left, top, cell_w, cell_h, G, doG, doE, doY, g, e, y);
    if (blur) {
        if (doG) Sim::blur(g, G);
        if (doE) Sim::blur(e, G);
        if (doY) Sim::blur(y, G);
    }
}

// Build the tree at the current positions; returns the number of tree points.
int oracle_build_tree(void* h, int* n_nodes) {
    Sim* s = static_cast<Sim*>(h);
    s->buildTree();
    if (n_nodes) *n_nodes = s->tree.count;
    return s->nTree + (int)s->ghosts.size();
}
int oracle_tree_overflow(void* h) { return static_cast<Sim*>(h)->tree.overflow ? 1 : 0; }

// Leaf dump: for each tree point its leaf id (-1 if dropped); per leaf the
// centre, half-size and level.  Returns the number of non-empty leaves.
int oracle_tree_leaves(void* h, int* leaf_of_point, int n_points, double* lbx, double* lby, double* lbw, int* llevel, int cap) {
    Sim* s = static_cast<Sim*>(h);
    const QuadTree& t = s->tree;
    for (int i = 0; i < n_points; i++) leaf_of_point[i] = -1;
    int nl = 0;
    for (int idx = 0; idx < t.count; idx++) {
        if (t.divided[idx] || t.pointCount[idx] == 0) continue;
        if (nl < cap) { lbx[nl] = t.bx[idx]; lby[nl] = t.by[idx]; lbw[nl] = t.bw[idx]; llevel[nl] = t.level[idx]; }
        for (int k = 0; k < t.pointCount[idx]; k++) {
            int pt = t.points[idx * QT_CAPACITY + k];
            if (pt >= 0 && pt < n_points) leaf_of_point[pt] = nl;
        }
        nl++;
    }
    return nl;
}
// Storage slot of each tree point inside its leaf (-1 if dropped): the order
// in which QuadTreePool.query reports a leaf's points (quadtree.js:386-393).
void oracle_tree_leaf_slots(void* h, int* slot_of_point, int n_points) {
    Sim* s = static_cast<Sim*>(h);
    const QuadTree& t = s->tree;
    for (int i = 0; i < n_points; i++) slot_of_point[i] = -1;
    for (int idx = 0; idx < t.count; idx++) {
        if (t.divided[idx]) continue;
        for (int k = 0; k < t.pointCount[idx]; k++) {
            const int pt = t.points[idx * QT_CAPACITY + k];
            if (pt >= 0 && pt < n_points) slot_of_point[pt] = k;
        }
    }
}
// Ghost originals in generation order.
int oracle_ghost_origins(void* h, int* orig, int cap) {
    Sim* s = static_cast<Sim*>(h);
    int n = std::min(cap, (int)s->ghosts.size());
    for (int i = 0; i < n; i++) orig[i] = s->ghosts[i].orig;
    return (int)s->ghosts.size();
}
// Aggregates of the node that holds the most points in the tree, etc.: full node dump.
int oracle_tree_nodes(void* h, double* out /* 12 x cap */, int* meta /* 3 x cap: divided, count, level */, int cap) {
    Sim* s = static_cast<Sim*>(h);
    const QuadTree& t = s->tree;
    int n = std::min(cap, t.count);
    for (int i = 0; i < n; i++) {
        double v[12] = { t.bx[i], t.by[i], t.bw[i], t.totalMass[i], t.totalCharge[i], t.totalMag[i], t.totalAngMom[i],
                         t.momX[i], t.momY[i], t.comX[i], t.comY[i], t.bh[i] };
        for (int r = 0; r < 12; r++) out[(size_t)r * cap + i] = v[r];
        meta[i] = t.divided[i]; meta[cap + i] = t.pointCount[i]; meta[2 * cap + i] = t.level[i];
    }
    return t.count;
}

// History upload: count samples, times shared; samples rows x,y,vx,vy,angw (n*count each, particle-major).
int oracle_upload_history(void* h, int n, int count, const double* times, const double* samples) {
    Sim* s = static_cast<Sim*>(h);
    if (n != (int)s->ps.size() || count < 0 || count > HISTORY_SIZE) return -1;
    const size_t plane = (size_t)n * count;
    for (int i = 0; i < n; i++) {
        History& H = s->ps[i].h;
        H.alloc = false; H.init();
        for (int k = 0; k < count; k++) {
            const size_t o = (size_t)i * count + k;
            H.x[k] = samples[o]; H.y[k] = samples[plane + o];
            H.vx[k] = samples[2 * plane + o]; H.vy[k] = samples[3 * plane + o];
            H.angw[k] = samples[4 * plane + o]; H.t[k] = times[k];
        }
        H.head = count & HISTORY_MASK; H.count = count;
    }
    return 0;
}
void oracle_set_hist_stride(void* h, int v) { static_cast<Sim*>(h)->histStride = v; }

// Stats (energy.js:11-62 passes 1-2) into GeonStats.
void oracle_stats(void* h, GeonStats* st) {
    Sim* s = static_cast<Sim*>(h);
    const bool rel = s->relOn();
    double linearKE = 0, spinKE = 0, totalMass = 0, comX = 0, comY = 0, px = 0, py = 0;
    for (const auto& p : s->ps) {
        const double pm = p.mass, rSq = p.radiusSq;
        if (rel) {
            double wSq = p.wx * p.wx + p.wy * p.wy;
            double gamma = std::sqrt(1 + wSq);
            linearKE += wSq / (gamma + 1) * pm;
            double srSq = p.angw * p.angw * rSq;
            double gammaRot = std::sqrt(1 + srSq);
            spinKE += INERTIA_K * pm * srSq / (gammaRot + 1);
        } else {
            double speedSq = p.vx * p.vx + p.vy * p.vy;
            linearKE += 0.5 * pm * speedSq;
            spinKE += 0.5 * INERTIA_K * pm * rSq * p.angVel * p.angVel;
        }
        px += pm * p.wx; py += pm * p.wy;
        totalMass += pm; comX += pm * p.x; comY += pm * p.y;
    }
    double orb = 0, spin = 0;
    if (totalMass > 0) {
        comX /= totalMass; comY /= totalMass;
        for (const auto& p : s->ps) {
            double dx = p.x - comX, dy = p.y - comY;
            orb += dx * (p.mass * p.wy) - dy * (p.mass * p.wx);
            spin += INERTIA_K * p.mass * p.radiusSq * p.angw;
        }
    }
    st->linear_ke = linearKE; st->spin_ke = spinKE; st->pe = s->pe;
    st->px = px; st->py = py; st->orbital_ang_mom = orb; st->spin_ang_mom = spin;
    st->com_x = comX; st->com_y = comY; st->total_mass = totalMass;
    st->sim_time = s->simTime; st->alive_count = (int)s->ps.size(); st->last_substeps = s->lastSubsteps;
}

// getDelayedState of particle `src` seen from (ox, oy) at the current simTime;
// returns 1 and writes x, y, vx, vy, angw, or 0 when there is no solution.
int oracle_delayed_state(void* h, int src, double ox, double oy, double* out) {
    Sim* s = static_cast<Sim*>(h);
    if (src < 0 || src >= (int)s->ps.size()) return 0;
    Sim::Delayed d;
    if (!s->getDelayedState(s->ps[src], ox, oy, d)) return 0;
    out[0] = d.x; out[1] = d.y; out[2] = d.vx; out[3] = d.vy; out[4] = d.angw;
    return 1;
}

// Free-function kernels used by known-answer tests.
void oracle_min_image(double ox, double oy, double sx, double sy, int topology, double W, double H, double* out) {
    Vec v = minImage(ox, oy, sx, sy, topology, W, H, W * 0.5, H * 0.5);
    out[0] = v.x; out[1] = v.y;
}

}  // extern "C"
