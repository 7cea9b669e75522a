// capi.cu — the C ABI (include/geon.h): handle lifetime, state upload and
// download, and the frame driver that sequences the kernels of one
// Physics.update (src/integrator.js:726-1825, in-scope part).
//
// Substep planning (integrator.js:810-875) runs on the host in FP64 from
// max-reductions that the force pass leaves in device memory: the host reads
// them back once per substep (one small copy), computes dtSub exactly as the
// reference does, and enqueues the next substep.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <climits>
#include <string>
#include <vector>
#include "force.cuh"
#include "push.cuh"
#include "learn.cuh"
#include "mlp.cuh"
#include "batch.cuh"
#include "collide.cuh"
#include "boson.cuh"
#include "frame.cuh"

using namespace geon;

#define GEON_VERSION_STRING "geon-gb300 1.0 (sm_103a)"

namespace {

thread_local std::string g_err;

// Frees every pointer registered with it.
struct DevArena {
    std::vector<void*> ptrs;
    bool failed = false;
    template <class T> T* alloc(size_t count) {
        if (count == 0) count = 1;
        void* p = nullptr;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) { failed = true; return nullptr; }
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    void free_all() {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
    }
};

int lsb_exp(double v) {
    if (v == 0.0) return INT_MAX;
    int e;
    double m = std::frexp(std::fabs(v), &e);
    uint64_t M = (uint64_t)std::ldexp(m, 53);
    return e - 53 + __builtin_ctzll(M);
}

// True when every grid value c - hw + j * hw / 2^30, j = 0 .. 2^31, is an exact
// double, so the reference's centre recurrence never rounds.
bool grid_exact(double c, double hw) {
    if (!(hw > 0)) return false;
    const int e = std::min(lsb_exp(c), lsb_exp(hw) - 30);
    const double maxabs = std::fabs(c) + hw;
    return std::ldexp(maxabs, -e) < 9007199254740992.0;
}

}  // namespace

// Batched handle: device arrays of the per-system planner and the frame
// graph (a WHILE conditional node over the substeps).
struct Batch {
    BatchDev dev{};
    DevArena A;
    std::vector<int> off;           // [nsys + 1] first particle of each system
    std::vector<int> pad;           // [nsys] first walk slot of each system
    int slots = 0;                  // padded walk slots
    int* sys = nullptr;             // [n_cap] system of each particle
    int* roots = nullptr;           // [nsys]
    int* any_h = nullptr;           // pinned copy of dev.any_active
    double* dt_h = nullptr;         // pinned frame dt
    SysPlan* plan_h = nullptr;      // pinned copy of dev.plan
    int use_graph = 1;
    int walk_split = 0;             // walk shape (geon_batch_set_shape): four warps per group
    int split_level = 6;
    int walk_ctas = 0;              // resident walk CTAs per SM (0: as many as fit)
    int walk_chunk = 0;             // > 0: persistent walk CTAs take this many walk blocks at a time
    unsigned* walk_queue = nullptr; // [2] their counters (next block, CTAs done)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long graph_head = 0, graph_body = 0, graph_tail = 0;   // kernels per part of the graph
    uint32_t graph_flags = 0;       // flags the graph was captured with
    int last_max_steps = 0;
};

struct GeonHandle {
    GeonParams prm{};
    DevParams P{};
    int n_cap = 0;
    int slots = 0;          // particle slots of S / S2: n_cap, or 2 n_cap once merge collisions are on
    int n = 0;
    cudaStream_t st = nullptr;
    DevArena arena;         // control
    DevArena state_arena;   // S, S2 and the compaction buffers (reallocated when slots grow)
    DevArena col_arena;     // merge-collision buffers (allocated when the merge mode is first used)
    DevArena tree_arena;    // tree buffers (reallocated when ghost capacity changes)
    DevArena hist_arena;    // history rings (allocated when relativity is first enabled)
    DevArena learn_arena;   // learned-correction weights and record counters
    DevState S{}, S2{};
    TreeBufs T{};
    bool tree_periodic = false;
    bool tree_moments = false;
    bool hist_alloc = false;
    FrameCtl* ctl = nullptr;
    FrameCtl* ctl_h = nullptr;     // pinned
    FrameRun* frun = nullptr;      // one-launch frame: barrier state and results
    FrameRun* frun_h = nullptr;    // pinned
    long long frame_wait_ns = 1000000000LL;   // a frame barrier gives up after this long
    int frame_extra = 0;           // barrier arrivals waited for beyond the grid (time-out test)
    int* d_root = nullptr;
    double* hist_t = nullptr;
    float* hist_age = nullptr;
    float* hist_segdt = nullptr;
    int* keep = nullptr;
    int* dst = nullptr;
    int* cscan_tmp = nullptr;
    float* staging = nullptr;      // GEON_ST_ROWS x n_cap floats
    double* staging_d = nullptr;   // GEON_ST_ROWS x n_cap doubles
    double* stats_d = nullptr;
    double* stats_h = nullptr;     // pinned
    double simTime = 0.0;
    bool forcesInit = false;
    float* dpart = nullptr;          // pairwise-sum slice partials (direct_plan), grown on demand
    size_t dpart_floats = 0;
    int histStride = 0;
    long long histTotal = 0;
    int lastSubsteps = 0;
    int nextId = 0;
    // merge collisions
    CollBufs col{};
    CollCtl* col_h = nullptr;       // pinned copy of col.cc
    int col_cap_int = 0;            // tree node capacity the collision buffers were sized for
    bool col_alloc = false;
    bool col_tgt_active = false;    // the next force pass walks col.tgt2
    int col_tgt_count = 0;
    GeonCollisionInfo col_info{};
    // boson pool: a second handle holds it as particles (its tree is the boson tree)
    GeonHandle* bos = nullptr;
    int nb = 0;                     // bosons of the current pool
    int nb_massive = 0;             // pions and leptons among them
    DevArena boson_arena;
    float2* bkind = nullptr;        // [bos->n_cap] kind, v^2
    float2* bkick = nullptr;        // [bos->n_cap] kicks
    double* biq = nullptr;          // exact node charges of the pool's tree
    double* blq = nullptr;
    // batched systems (nsys > 0)
    int nsys = 0;
    Batch* batch = nullptr;
    // learned correction
    float* learn_w = nullptr;       // [GEON_MLP_NPARAM] device weights (null: correction off)
    float* learn_w_buf = nullptr;   // their buffer, kept when the weights are cleared
    uint2* recs = nullptr;          // (cell, group) records: rec_cap per group of 32 walk slots
    int* rec_cnt = nullptr;         // [rec_groups] records of each group in the last walk
    unsigned* rec_max = nullptr;    // largest count of the last walk (counters: learn_arena)
    unsigned* apply_queue = nullptr;  // the correction's group counter (learn_arena)
    unsigned long long* rec_total = nullptr;
    long long rec_total_h = 0;      // records of the last walk
    int rec_cap = 0;
    int rec_groups = 0;
    float4* gcen = nullptr;         // [rec_groups] group centres and radius bounds
    int* rec_off = nullptr;         // [rec_groups + 1] exclusive prefix of the counts
    void* rec_scan = nullptr;       // scan scratch of learn_record_offsets
    float4* rec_exp = nullptr;      // per record output (4 float4) of the correction's phase A
    uint2* rec_flags = nullptr;     // per record flags and cell mass
    int* rec_net = nullptr;         // records the network applies to (+ 1 count at the end)
    long long rec_exp_cap = 0;
    LaunchCounter lc;
    std::string err;
    // profiling
    bool prof = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_ev;
    std::vector<cudaEvent_t> ev_pool;
    GeonProfile prof_acc{};
};

enum { PH_TREE = 0, PH_FORCE, PH_ONEPN, PH_PUSH, PH_LEARN, PH_COLLIDE };

static cudaEvent_t get_event(GeonHandle* h) {
    if (!h->ev_pool.empty()) { cudaEvent_t e = h->ev_pool.back(); h->ev_pool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// Records a start event for a phase; returns its slot (or -1 when profiling is off).
static int prof_begin(GeonHandle* h, int phase) {
    if (!h->prof) return -1;
    cudaEvent_t a = get_event(h), b = get_event(h);
    cudaEventRecord(a, h->st);
    h->prof_ev.push_back({ phase, { a, b } });
    return (int)h->prof_ev.size() - 1;
}
static void prof_end(GeonHandle* h, int slot) {
    if (slot < 0) return;
    cudaEventRecord(h->prof_ev[slot].second.second, h->st);
}
static void prof_collect(GeonHandle* h) {
    if (h->prof_ev.empty()) return;
    cudaStreamSynchronize(h->st);
    for (auto& pe : h->prof_ev) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pe.second.first, pe.second.second);
        switch (pe.first) {
            case PH_TREE: h->prof_acc.tree_ms += ms; h->prof_acc.tree_count++; break;
            case PH_FORCE: h->prof_acc.force_ms += ms; h->prof_acc.force_count++; break;
            case PH_ONEPN: h->prof_acc.onepn_ms += ms; h->prof_acc.onepn_count++; break;
            case PH_LEARN: h->prof_acc.learn_ms += ms; h->prof_acc.learn_count++; break;
            case PH_COLLIDE: h->prof_acc.collide_ms += ms; h->prof_acc.collide_count++; break;
            default: h->prof_acc.push_ms += ms; h->prof_acc.push_count++; break;
        }
        h->ev_pool.push_back(pe.second.first);
        h->ev_pool.push_back(pe.second.second);
    }
    h->prof_ev.clear();
}

static int set_err(GeonHandle* h, int code, const std::string& msg) {
    if (h) h->err = msg; else g_err = msg;
    return code;
}

static int cuda_check(GeonHandle* h, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return GEON_OK;
    return set_err(h, GEON_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call) do { int _r = cuda_check(h, (call), #call); if (_r) return _r; } while (0)
#define CKL() do { int _r = cuda_check(h, cudaGetLastError(), "kernel launch"); if (_r) return _r; } while (0)

static int validate_params(GeonHandle* h, const GeonParams& p) {
    const uint32_t unsupported = GEON_BLACK_HOLE | GEON_HIGGS | GEON_AXION;
    if (p.toggles & unsupported) return set_err(h, GEON_ERR_UNSUPPORTED, "black-hole mode, Higgs and axion fields are not part of this library");
    if (!(p.domain_w > 0) || !(p.domain_h > 0)) return set_err(h, GEON_ERR_ARG, "domain_w and domain_h must be positive");
    if (p.boundary_mode < 0 || p.boundary_mode > 2) return set_err(h, GEON_ERR_ARG, "boundary_mode out of range");
    if (p.topology < 0 || p.topology > 2) return set_err(h, GEON_ERR_ARG, "topology out of range");
    if (!(p.theta >= 0)) return set_err(h, GEON_ERR_ARG, "theta must be >= 0");
    if (!(p.softening > 0)) return set_err(h, GEON_ERR_ARG, "softening must be > 0");
    if ((p.toggles & GEON_YUKAWA) && !(p.yukawa_mu > 0)) return set_err(h, GEON_ERR_ARG, "yukawa_mu must be > 0");
    if (p.collision_mode < GEON_COL_PASS || p.collision_mode > GEON_COL_BOUNCE) return set_err(h, GEON_ERR_ARG, "collision_mode out of range");
    if (p.collision_mode == GEON_COL_BOUNCE) return set_err(h, GEON_ERR_UNSUPPORTED, "the bounce collision mode (contact forces) is not part of this library");
    if (p.collision_mode == GEON_COL_MERGE && (p.flags & GEON_FLAG_LEARN))
        return set_err(h, GEON_ERR_UNSUPPORTED, "merge collisions and the learned correction cannot be combined");
    if ((p.flags & GEON_FLAG_LEARN) && p.boundary_mode == GEON_BOUND_LOOP)
        return set_err(h, GEON_ERR_UNSUPPORTED, "the learned correction covers open boxes (no periodic images)");
    return GEON_OK;
}

static void derive_params(GeonHandle* h) {
    const GeonParams& p = h->prm;
    DevParams& P = h->P;
    P = DevParams{};
    P.toggles = p.toggles; P.flags = p.flags;
    P.boundary = p.boundary_mode; P.topology = p.topology;
    P.periodic = p.boundary_mode == GEON_BOUND_LOOP;
    P.ghosts = P.periodic && !(p.flags & GEON_FLAG_NO_GHOSTS);
    P.rel = (p.toggles & GEON_RELATIVITY) ? 1 : 0;
    P.n_cap = h->slots;
    P.nsys = h->nsys;
    P.keyTop = h->nsys ? 10 : 2;
    P.keyLevels = h->nsys ? BATCH_KEY_LEVELS : KEY_LEVELS;
    P.Wd = p.domain_w; P.Hd = p.domain_h; P.offXd = p.off_x; P.offYd = p.off_y;
    P.W = (float)p.domain_w; P.H = (float)p.domain_h;
    P.W_lo = (float)(p.domain_w - (double)P.W); P.H_lo = (float)(p.domain_h - (double)P.H);
    P.halfW = (float)(p.domain_w * 0.5); P.halfH = (float)(p.domain_h * 0.5);
    P.rootX = p.off_x + p.domain_w / 2; P.rootY = p.off_y + p.domain_h / 2;     // integrator.js:727-730
    P.rootW = p.domain_w * 2; P.rootH = p.domain_h * 2;
    P.exact_grid = grid_exact(P.rootX, P.rootW) && grid_exact(P.rootY, P.rootH);
    P.soft = (float)p.softening;
    P.softSq = (float)(p.softening * p.softening);
    P.thetaD = p.theta;
    P.thetaSqD = p.theta * p.theta;
    P.thetaSq = (float)P.thetaSqD;
    P.yukOn = (p.toggles & GEON_YUKAWA) ? 1 : 0;
    P.yukMu = (float)p.yukawa_mu;
    if (P.yukOn) {
        const double c = 6.0 / p.yukawa_mu;                                    // forces.js:82-83
        P.yukCutSqD = c * c;
        P.yukCutSq = (float)P.yukCutSqD;
    }
    P.extGx = (float)(p.ext_gravity * std::cos(p.ext_gravity_angle));         // integrator.js:553-560
    P.extGy = (float)(p.ext_gravity * std::sin(p.ext_gravity_angle));
    P.extEx = (float)(p.ext_electric * std::cos(p.ext_electric_angle));
    P.extEy = (float)(p.ext_electric * std::sin(p.ext_electric_angle));
    P.extBz = (float)p.ext_bz;
    P.friction = (float)p.bounce_friction;
}

static void fill_state(DevArena& A, DevState& S, int cap) {
    S.pos = A.alloc<float4>(cap); S.pos_lo = A.alloc<float2>(cap); S.vel = A.alloc<float4>(cap);
    S.spin = A.alloc<float4>(cap); S.mom = A.alloc<float2>(cap); S.force = A.alloc<float4>(cap);
    S.grad = A.alloc<float4>(cap); S.torque = A.alloc<float4>(cap); S.f1pn = A.alloc<float2>(cap);
    S.f1pnOld = A.alloc<float2>(cap); S.brk = A.alloc<float>((size_t)12 * cap); S.ctime = A.alloc<double>(cap);
    S.id = A.alloc<int>(cap); S.hist_cnt = A.alloc<int>(cap); S.matter = A.alloc<float2>(cap);
    S.hist = nullptr; S.hist_angw = nullptr;
}

static bool merge_on(const GeonHandle* h) { return h->prm.collision_mode == GEON_COL_MERGE; }

// Particle slots needed: a merge spawns its particle into a new slot while the
// two it replaces stay in place until the end of the substep (each spawn
// removes at least one particle, so 2 n_cap slots always suffice).
static int slots_wanted(const GeonHandle* h) { return merge_on(h) ? 2 * h->n_cap : h->n_cap; }

// (Re)allocates S, S2 and the compaction buffers with `slots` slots, keeping
// the first n particles (every per-particle row; the history rings live in
// their own arena and are not moved).
static int alloc_state(GeonHandle* h, int slots) {
    DevArena A;
    DevState S{}, S2{};
    fill_state(A, S, slots);
    fill_state(A, S2, slots);
    int* keep = A.alloc<int>(slots);
    int* dst = A.alloc<int>(slots);
    int* tmp = A.alloc<int>(scan_temp_ints(slots) + 16);
    if (A.failed) { A.free_all(); return set_err(h, GEON_ERR_NOMEM, "state allocation failed"); }
    cudaMemsetAsync(S.hist_cnt, 0, (size_t)slots * sizeof(int), h->st);
    cudaMemsetAsync(S.brk, 0, (size_t)12 * slots * sizeof(float), h->st);
    const size_t n = (size_t)h->n;
    if (h->slots > 0 && n > 0) {
        const DevState& O = h->S;
        auto cp = [&](void* d, const void* s, size_t bytes) { return cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToDevice, h->st); };
        cudaError_t e = cudaSuccess;
        e = e ? e : cp(S.pos, O.pos, n * sizeof(float4));   e = e ? e : cp(S.pos_lo, O.pos_lo, n * sizeof(float2));
        e = e ? e : cp(S.vel, O.vel, n * sizeof(float4));   e = e ? e : cp(S.spin, O.spin, n * sizeof(float4));
        e = e ? e : cp(S.mom, O.mom, n * sizeof(float2));   e = e ? e : cp(S.force, O.force, n * sizeof(float4));
        e = e ? e : cp(S.grad, O.grad, n * sizeof(float4)); e = e ? e : cp(S.torque, O.torque, n * sizeof(float4));
        e = e ? e : cp(S.f1pn, O.f1pn, n * sizeof(float2)); e = e ? e : cp(S.f1pnOld, O.f1pnOld, n * sizeof(float2));
        e = e ? e : cp(S.ctime, O.ctime, n * sizeof(double)); e = e ? e : cp(S.id, O.id, n * sizeof(int));
        e = e ? e : cp(S.hist_cnt, O.hist_cnt, n * sizeof(int)); e = e ? e : cp(S.matter, O.matter, n * sizeof(float2));
        for (int r = 0; r < 12 && !e; r++) e = cp(S.brk + (size_t)r * slots, O.brk + (size_t)r * h->slots, n * sizeof(float));
        if (!e) e = cudaStreamSynchronize(h->st);
        if (e) { A.free_all(); return cuda_check(h, e, "state copy"); }
    }
    S.hist = h->S.hist; S.hist_angw = h->S.hist_angw; S.sys = h->S.sys;
    S2.hist = h->S2.hist; S2.hist_angw = h->S2.hist_angw; S2.sys = h->S2.sys;
    if (h->slots > 0) cudaStreamSynchronize(h->st);
    h->state_arena.free_all();
    h->state_arena.ptrs.swap(A.ptrs);
    h->S = S; h->S2 = S2;
    h->keep = keep; h->dst = dst; h->cscan_tmp = tmp;
    h->slots = slots;
    h->P.n_cap = slots;
    return GEON_OK;
}

static int ensure_history(GeonHandle* h) {
    if (h->hist_alloc || !h->P.rel) return GEON_OK;
    const size_t cnt = (size_t)h->n_cap * HIST_LEN;
    h->S.hist = h->hist_arena.alloc<float4>(cnt);
    h->S.hist_angw = h->hist_arena.alloc<float>(cnt);
    h->S2.hist = h->hist_arena.alloc<float4>(cnt);
    h->S2.hist_angw = h->hist_arena.alloc<float>(cnt);
    if (h->hist_arena.failed) { h->hist_arena.free_all(); return set_err(h, GEON_ERR_NOMEM, "history allocation failed"); }
    h->hist_alloc = true;
    return GEON_OK;
}

static int ensure_tree(GeonHandle* h) {
    const bool per = h->P.ghosts != 0;
    if (h->T.pt_ref && per == h->tree_periodic) return GEON_OK;
    CK(cudaStreamSynchronize(h->st));
    h->tree_arena.free_all();
    h->tree_arena.failed = false;
    TreeBufs& T = h->T;
    T = TreeBufs{};
    DevArena& A = h->tree_arena;
    const int cap = h->n_cap;
    const long long cp = (long long)cap * (per ? 1 + MAX_GHOSTS_PER_PARTICLE : 1);
    if (cp > (1ll << 30)) return set_err(h, GEON_ERR_ARG, "tree point capacity too large");
    T.cap_pts = (int)cp;
    T.cap_int = T.cap_pts + 1024;
    T.pt_ref = A.alloc<uint32_t>(T.cap_pts);
    T.ghost_cnt = A.alloc<int>(cap); T.ghost_off = A.alloc<int>(cap);
    T.key = A.alloc<uint64_t>(T.cap_pts); T.key_alt = A.alloc<uint64_t>(T.cap_pts);
    T.idx = A.alloc<uint32_t>(T.cap_pts); T.idx_alt = A.alloc<uint32_t>(T.cap_pts);
    T.sort_tmp = A.alloc<char>(radix_temp_bytes(T.cap_pts));
    T.scan_tmp = A.alloc<int>(scan_temp_ints(T.cap_pts) + 16);
    T.ps_a = A.alloc<float4>(T.cap_pts); T.ps_b = A.alloc<float4>(T.cap_pts); T.ps_c = A.alloc<float4>(T.cap_pts);
    T.lcp_a = A.alloc<int>(T.cap_pts); T.int_cnt = A.alloc<int>(T.cap_pts); T.int_base = A.alloc<int>(T.cap_pts);
    T.leaf_flag = A.alloc<int>(T.cap_pts); T.leaf_base = A.alloc<int>(T.cap_pts);
    T.real_flag = A.alloc<int>(T.cap_pts); T.tgt_base = A.alloc<int>(T.cap_pts);
    T.tgt = A.alloc<int>(cap);
    T.int_a = A.alloc<float4>(T.cap_int); T.int_b = A.alloc<float4>(T.cap_int); T.int_c = A.alloc<float4>(T.cap_int);
    T.int_child = A.alloc<int4>(T.cap_int); T.int_meta = A.alloc<int4>(T.cap_int); T.int_count = A.alloc<int>(T.cap_int);
    T.leaf_a = A.alloc<float4>(T.cap_pts); T.leaf_b = A.alloc<float4>(T.cap_pts); T.leaf_c = A.alloc<float4>(T.cap_pts);
    T.leaf_meta = A.alloc<int4>(T.cap_pts); T.leaf_of = A.alloc<int>(T.cap_pts);
    T.roots = h->batch ? h->batch->roots : nullptr;
    if (A.failed) { A.free_all(); T = TreeBufs{}; return set_err(h, GEON_ERR_NOMEM, "tree allocation failed"); }
    h->tree_moments = false;
    h->tree_periodic = per;
    return GEON_OK;
}

// ---- small kernels local to the driver --------------------------------------------------------
__global__ void set_n_kernel(FrameCtl* ctl, int n) { ctl->n = n; }

// rows: x, y, wx, wy, mass, charge, angw (and, with with_lo, the low parts of x, y)
__global__ void init_particles_kernel(DevParams P, DevState S, const float* __restrict__ rows, int cap, int first, int k,
                                      double ctime, int id0, int with_lo) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < k; t += gridDim.x * blockDim.x) {
        const float x = rows[t], y = rows[cap + t], wx = rows[2 * cap + t], wy = rows[3 * cap + t];
        const float m = rows[4 * cap + t], q = rows[5 * cap + t], angw = rows[6 * cap + t];
        const int i = first + t;
        const float r = cbrtf(m);
        float vx = wx, vy = wy, angVel = angw;
        if (P.rel) {
            const float invG = 1.f / sqrtf(1.f + wx * wx + wy * wy);
            vx = wx * invG; vy = wy * invG;
            angVel = angw / sqrtf(1.f + angw * angw * r * r);             // relativity.js:7-9
        }
        S.pos[i] = make_float4(x, y, m, q);
        S.pos_lo[i] = with_lo ? make_float2(rows[7 * cap + t], rows[8 * cap + t]) : make_float2(0.f, 0.f);
        S.vel[i] = make_float4(wx, wy, vx, vy);
        S.spin[i] = make_float4(angw, angVel, r, 1.f / m);
        S.mom[i] = make_float2(0.f, 0.f);                                   // particle.js:53-54
        S.force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        S.grad[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        S.torque[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        S.f1pn[i] = make_float2(0.f, 0.f);
        S.f1pnOld[i] = make_float2(0.f, 0.f);
        S.ctime[i] = ctime;
        S.id[i] = id0 + t;
        S.hist_cnt[i] = 0;
        S.matter[i] = make_float2(m, 0.f);                                  // baseMass = mass, matter
        for (int rr = 0; rr < 12; rr++) S.brk[(size_t)rr * P.n_cap + i] = 0.f;
    }
}

__global__ void bootstrap_angvel_kernel(DevParams P, DevState S, const FrameCtl* ctl) {   // integrator.js:751-753
    const int n = ctl->n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 s = S.spin[i];
        s.y = P.rel ? s.x / sqrtf(1.f + s.x * s.x * s.z * s.z) : s.x;
        S.spin[i] = s;
    }
}

template <class Tout>
__global__ void pack_state_kernel(DevState S, int n, int rows, int cap, Tout* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = S.pos[i];
        const float2 pl = S.pos_lo[i];
        const float4 v = S.vel[i];
        const float4 s = S.spin[i];
        double vals[GEON_ST_ROWS] = { (double)p.x + pl.x, (double)p.y + pl.y, v.x, v.y, p.z, p.w, s.x, v.z, v.w, s.y };
        for (int r = 0; r < rows; r++) out[(size_t)r * cap + i] = (Tout)vals[r];
    }
}

__global__ void pack_forces_kernel(DevState S, int n, int first, int rows, int cap, int n_cap, float* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int r = 0; r < rows; r++) {
            const int row = first + r;
            float v = 0.f;
            const float4 f = S.force[i], g = S.grad[i], t = S.torque[i];
            const float2 p1 = S.f1pn[i];
            switch (row) {
                case GEON_OUT_FX: v = f.x; break;
                case GEON_OUT_FY: v = f.y; break;
                case GEON_OUT_BZ: v = f.z; break;
                case GEON_OUT_BGZ: v = f.w; break;
                case GEON_OUT_DBZDX: v = g.x; break;
                case GEON_OUT_DBZDY: v = g.y; break;
                case GEON_OUT_DBGZDX: v = g.z; break;
                case GEON_OUT_DBGZDY: v = g.w; break;
                case GEON_OUT_TIDAL: v = t.x; break;
                case GEON_OUT_FRAMEDRAG: v = t.y; break;
                case GEON_OUT_F1PN_X: v = p1.x; break;
                case GEON_OUT_F1PN_Y: v = p1.y; break;
                case GEON_OUT_PE: v = t.w; break;
                default: v = S.brk[(size_t)(row - GEON_OUT_GRAV_X) * n_cap + i]; break;
            }
            out[(size_t)r * cap + i] = v;
        }
    }
}

__global__ void history_upload_kernel(DevState S, int n, int count, const float* __restrict__ samples) {
    const size_t plane = (size_t)n * count;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < plane; e += (size_t)gridDim.x * blockDim.x) {
        const size_t i = e / count, k = e % count;
        S.hist[i * HIST_LEN + k] = make_float4(samples[e], samples[plane + e], samples[2 * plane + e], samples[3 * plane + e]);
        S.hist_angw[i * HIST_LEN + k] = samples[4 * plane + e];
        if (k == 0) S.hist_cnt[i] = count;
    }
}

// FP32 FMA microbenchmark: 8 independent chains per thread.
__global__ void fma_peak_kernel(float* out, int iters, float a, float b) {
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 123456.789f) out[0] = s;
}

static inline int grid_for(int n, int threads) {
    int b = (n + threads - 1) / threads;
    return std::max(1, std::min(b, device_sms() * 16));
}

static inline double bits_to_double(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

static bool bh_on(const GeonHandle* h) { return (h->prm.toggles & GEON_BARNES_HUT) != 0; }

static ForceCtx make_ctx(GeonHandle* h) {
    ForceCtx C{};
    C.simTime = h->simTime;
    C.hist_t = h->hist_t;
    C.hist_age = h->hist_age;
    C.hist_segdt = h->hist_segdt;
    C.hist_head = (int)(h->histTotal & HIST_MASK);
    C.pe = (h->prm.flags & GEON_FLAG_PE) ? 1 : 0;
    C.brk = (h->prm.flags & GEON_FLAG_BREAKDOWN) ? 1 : 0;
    C.bounce = h->prm.boundary_mode == GEON_BOUND_BOUNCE;
    if (h->col_tgt_active) {            // force pass right after merge collisions
        C.tgt_list = h->col.tgt2;
        C.tgt_count = h->col_tgt_count;
    }
    return C;
}

static int read_ctl(GeonHandle* h) {
    CK(cudaMemcpyAsync(h->ctl_h, h->ctl, sizeof(FrameCtl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (h->ctl_h->err) {
        const int e = h->ctl_h->err;
        if (e & (ERR_MMA_TIMEOUT | ERR_AGG_TIMEOUT | ERR_FRAME_TIMEOUT))
            return set_err(h, GEON_ERR_TIMEOUT, std::string("device wait timed out, flag ") + std::to_string(e));
        return set_err(h, GEON_ERR_OVERFLOW, std::string("device overflow flag ") + std::to_string(e) +
                       ((e & ERR_NODE_OVERFLOW) ? " (node capacity)" : "") + ((e & ERR_STACK_OVERFLOW) ? " (walk stack)" : ""));
    }
    return GEON_OK;
}

// Cell moment arrays for the learned correction, allocated on first use.
static int ensure_moments(GeonHandle* h) {
    if (h->tree_moments) return GEON_OK;
    TreeBufs& T = h->T;
    DevArena& A = h->tree_arena;
    T.int_m1 = A.alloc<float4>(T.cap_int); T.int_m2 = A.alloc<float4>(T.cap_int); T.int_m3 = A.alloc<float4>(T.cap_int);
    T.leaf_m1 = A.alloc<float4>(T.cap_pts); T.leaf_m2 = A.alloc<float4>(T.cap_pts); T.leaf_m3 = A.alloc<float4>(T.cap_pts);
    if (A.failed) return set_err(h, GEON_ERR_NOMEM, "moment allocation failed");
    h->tree_moments = true;
    return GEON_OK;
}

static int build_tree(GeonHandle* h) {
    int r = ensure_tree(h);
    if (r) return r;
    h->T.mom_on = 0;
    if (h->prm.flags & GEON_FLAG_LEARN) {
        r = ensure_moments(h);
        if (r) return r;
        h->T.mom_on = 1;
    }
    const int ps = prof_begin(h, PH_TREE);
    tree_build(h->P, h->S, h->T, h->ctl, h->d_root, h->n_cap, h->st, h->lc);
    prof_end(h, ps);
    CKL();
    return GEON_OK;
}

// The force set the learned correction covers: gravity, Coulomb and Yukawa
// without relativity, dipoles, 1PN or per-type breakdown rows, in an open box.
static bool learn_supported(const GeonHandle* h) {
    return !h->P.rel && !(h->prm.toggles & (GEON_MAGNETIC | GEON_GRAVITOMAG | GEON_ONE_PN)) &&
           !(h->prm.flags & (GEON_FLAG_BREAKDOWN | GEON_FLAG_SIMPLE_WALK)) && !h->P.periodic && !h->batch;
}

static bool learn_active(const GeonHandle* h) {
    return h->learn_w && (h->prm.flags & GEON_FLAG_LEARN) && h->T.mom_on && h->n > 0 && learn_supported(h);
}

// Record buffers for `cap` records per group (contents discarded when they grow).
static int ensure_recs(GeonHandle* h, int cap) {
    const int groups = (h->n_cap + 31) / 32;
    if (!h->rec_max) {
        unsigned* m = h->learn_arena.alloc<unsigned>(1);
        unsigned long long* t = h->learn_arena.alloc<unsigned long long>(1);
        unsigned* q = h->learn_arena.alloc<unsigned>(1);
        if (h->learn_arena.failed) return set_err(h, GEON_ERR_NOMEM, "record counter allocation failed");
        h->rec_max = m;
        h->rec_total = t;
        h->apply_queue = q;
    }
    if (groups > h->rec_groups) {
        cudaStreamSynchronize(h->st);
        void** bufs[4] = { (void**)&h->rec_cnt, (void**)&h->gcen, (void**)&h->rec_off, &h->rec_scan };
        const size_t bytes[4] = { (size_t)groups * sizeof(int), (size_t)groups * sizeof(float4),
                                  (size_t)(groups + 1) * sizeof(int), learn_offsets_scratch_bytes(groups) };
        for (int b = 0; b < 4; b++) {
            if (*bufs[b]) { cudaFree(*bufs[b]); *bufs[b] = nullptr; }
            if (cudaMalloc(bufs[b], bytes[b]) != cudaSuccess) {
                cudaGetLastError();
                h->rec_groups = 0;
                return set_err(h, GEON_ERR_NOMEM, "record group buffer allocation failed");
            }
        }
        h->rec_groups = groups;
        h->rec_cap = 0;                       // the record buffer is sized per group: regrow it
    }
    if (cap <= h->rec_cap && h->recs) return GEON_OK;
    cap = std::max(cap, 256);
    if (h->recs) { cudaStreamSynchronize(h->st); cudaFree(h->recs); h->recs = nullptr; }
    if (cudaMalloc(&h->recs, (size_t)h->rec_groups * cap * sizeof(uint2)) != cudaSuccess) {
        cudaGetLastError();
        h->rec_cap = 0;
        return set_err(h, GEON_ERR_NOMEM, "learned-correction record buffer allocation failed");
    }
    h->rec_cap = cap;
    return GEON_OK;
}

// Barnes-Hut walk with record emission: the plain monopole forces of every
// particle, and the (cell, group) records.  A walk whose largest group
// overflowed the per-group capacity is redone with room for it.
static int learn_walk(GeonHandle* h) {
    int r = ensure_recs(h, std::max(h->rec_cap, 2048));
    if (r) return r;
    for (int attempt = 0; attempt < 3; attempt++) {
        CK(cudaMemsetAsync(h->rec_max, 0, sizeof(unsigned), h->st));
        CK(cudaMemsetAsync(h->rec_total, 0, sizeof(unsigned long long), h->st));
        ForceCtx C = make_ctx(h);
        C.recs = h->recs;
        C.rec_cap = h->rec_cap;
        C.rec_cnt = h->rec_cnt;
        C.rec_max = h->rec_max;
        C.rec_total = h->rec_total;
        C.gcen = h->gcen;
        const int ps = prof_begin(h, PH_FORCE);
        force_pass(h->P, h->S, h->T, h->d_root, h->ctl, C, true, h->n_cap, h->st, h->lc);
        prof_end(h, ps);
        CKL();
        unsigned mx = 0;
        unsigned long long tot = 0;
        CK(cudaMemcpyAsync(&mx, h->rec_max, sizeof(mx), cudaMemcpyDeviceToHost, h->st));
        CK(cudaMemcpyAsync(&tot, h->rec_total, sizeof(tot), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        if ((int)mx <= h->rec_cap) {
            h->rec_total_h = (long long)tot;
            if (h->prof) h->prof_acc.learn_pairs += (long long)tot;
            return GEON_OK;
        }
        r = ensure_recs(h, (int)std::min<unsigned>(mx + mx / 4 + 64, 1u << 24));
        if (r) return r;
    }
    return set_err(h, GEON_ERR_OVERFLOW, "learned-correction records of one group exceed the buffer");
}

// Scratch of the correction's phase A for `total` records.
static int ensure_rec_exp(GeonHandle* h, long long total) {
    if (total > INT_MAX) return set_err(h, GEON_ERR_OVERFLOW, "more than 2^31 learned-correction records");
    if (total <= h->rec_exp_cap) return GEON_OK;
    const long long cap = total + total / 8 + 1024;
    cudaStreamSynchronize(h->st);
    if (h->rec_exp) { cudaFree(h->rec_exp); h->rec_exp = nullptr; }
    if (h->rec_flags) { cudaFree(h->rec_flags); h->rec_flags = nullptr; }
    if (h->rec_net) { cudaFree(h->rec_net); h->rec_net = nullptr; }
    h->rec_exp_cap = 0;
    if (cudaMalloc(&h->rec_exp, (size_t)cap * 4 * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&h->rec_flags, (size_t)cap * sizeof(uint2)) != cudaSuccess ||
        cudaMalloc(&h->rec_net, (size_t)(cap + 1) * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return set_err(h, GEON_ERR_NOMEM, "learned-correction scratch allocation failed");
    }
    h->rec_exp_cap = cap;
    return GEON_OK;
}

// The correction of the last walk's records: network outputs from the
// weights, or from yext (device, records in group order) when given.
static int learn_correct_records(GeonHandle* h, const float* yext) {
    const int ngroups = (h->n + 31) / 32;
    int r = ensure_rec_exp(h, h->rec_total_h);
    if (r) return r;
    learn_record_offsets(h->rec_cnt, h->rec_cap, ngroups, 1, h->rec_off, h->rec_off + ngroups, h->rec_scan, h->st, h->lc);
    learn_correct(h->P, h->S, h->T, h->ctl, h->learn_w, h->recs, h->rec_cnt, h->gcen, h->rec_cap, ngroups, h->rec_off,
                  (int)h->rec_total_h, yext, h->rec_exp, h->rec_flags, h->rec_net, h->rec_net + h->rec_exp_cap,
                  h->apply_queue, &h->ctl->err, h->st, h->lc);
    return GEON_OK;
}

// Barnes-Hut force pass with the learned far-field correction: the walk's
// monopole forces, then the network and expansions of learn_correct; the
// planner reductions are redone from the corrected forces.
static int learned_force_pass(GeonHandle* h) {
    int r = learn_walk(h);
    if (r) return r;
    const int pl = prof_begin(h, PH_LEARN);
    r = learn_correct_records(h, nullptr);
    prof_end(h, pl);
    if (r) return r;
    CKL();
    launch_frame_scan(h->P, h->S, h->ctl, h->n_cap, h->st, h->lc);
    CKL();
    return GEON_OK;
}

static BosonTree boson_tree(GeonHandle* h) {
    BosonTree B{};
    B.T = h->bos->T;
    B.ctl = h->bos->ctl;
    B.d_root = h->bos->d_root;
    B.S = h->bos->S;
    B.kind = h->bkind;
    B.iq = h->biq;
    B.lq = h->blq;
    B.n = h->nb;
    return B;
}

static bool bosons_act(const GeonHandle* h) {
    return (h->prm.flags & GEON_FLAG_BOSONS) && h->nb > 0 && h->bos && (h->prm.toggles & GEON_GRAVITY);
}

// The pairwise sum over few targets runs split over source slices that fill
// the GPU; their partial sums need scratch, allocated on first use.  Without
// it the pass runs unsliced.
static void use_slices(GeonHandle* h, ForceCtx& C, const DirectPlan& pl) {
    if (pl.slices <= 1) return;
    if (h->dpart_floats < pl.floats) {
        cudaStreamSynchronize(h->st);
        if (h->dpart) cudaFree(h->dpart);
        h->dpart = nullptr;
        h->dpart_floats = 0;
        if (cudaMalloc(&h->dpart, pl.floats * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            h->dpart = nullptr;
            return;
        }
        h->dpart_floats = pl.floats;
    }
    C.dpart = h->dpart;
    C.dslices = pl.slices;
}

static void direct_slices(GeonHandle* h, ForceCtx& C) { use_slices(h, C, direct_plan(h->P, C.brk != 0, h->n_cap)); }

static ForceCtx onepn_ctx(GeonHandle* h, bool bh) {
    ForceCtx C = make_ctx(h);
    if (!bh) use_slices(h, C, direct1pn_plan(h->n_cap));
    return C;
}

static int run_force_pass(GeonHandle* h, bool rebuild) {
    const bool bh = bh_on(h);
    if (bh && rebuild) { int r = build_tree(h); if (r) return r; }
    if (h->P.rel) { launch_hist_tables(h->hist_t, h->simTime, h->hist_age, h->hist_segdt, h->st, h->lc); CKL(); }
    if (bh && learn_active(h)) {
        int r = learned_force_pass(h);
        if (r || !bosons_act(h)) return r;
    } else {
        ForceCtx C = make_ctx(h);
        if (!bh) direct_slices(h, C);
        const int ps = prof_begin(h, PH_FORCE);
        force_pass(h->P, h->S, h->T, h->d_root, h->ctl, C, bh, h->n_cap, h->st, h->lc);
        prof_end(h, ps);
        CKL();
    }
    if (bosons_act(h)) {                      // computeBosonGravity (integrator.js:773-777, 1508-1513)
        TreeBufs order = h->T;
        if (!bh) order.tgt = nullptr;         // pairwise sum: no tree of this state
        boson_gravity(h->P, h->S, order, h->ctl, boson_tree(h), h->col_tgt_active ? h->col.tgt2 : nullptr, h->col_tgt_count,
                      (h->prm.flags & GEON_FLAG_BREAKDOWN) != 0, h->n_cap, h->st, h->lc);
        CKL();
    }
    return GEON_OK;
}

static int compact(GeonHandle* h, int n_slots = -1) {
    const int n = n_slots < 0 ? h->n : n_slots;
    exclusive_scan(h->keep, h->dst, n, nullptr, nullptr, h->cscan_tmp, h->st, &h->lc);
    launch_compact(h->S, h->S2, h->keep, h->dst, n, h->slots, h->hist_alloc, true, h->st, h->lc);
    CKL();
    std::swap(h->S, h->S2);
    return GEON_OK;
}

// ---- merge collisions (collide.cu) ------------------------------------------------------------
// Buffers sized for the particle capacity and the tree's node capacity.
static int ensure_collide(GeonHandle* h) {
    if (h->col_alloc && h->col_cap_int == h->T.cap_int) return GEON_OK;
    CK(cudaStreamSynchronize(h->st));
    h->col_arena.free_all();
    h->col_arena.failed = false;
    h->col_alloc = false;
    DevArena& A = h->col_arena;
    CollBufs& B = h->col;
    B = CollBufs{};
    const int cap = h->n_cap;
    B.cc = A.alloc<CollCtl>(1);
    B.cnt = A.alloc<int>(cap);
    B.off = A.alloc<int>(cap);
    B.cap = (int)std::min<long long>((long long)cap * 4 + 4096, 1ll << 28);
    B.cand = A.alloc<int2>(B.cap);
    B.uf = A.alloc<int>(cap);
    B.skey = A.alloc<uint64_t>(B.cap); B.skey_alt = A.alloc<uint64_t>(B.cap);
    B.sval = A.alloc<uint32_t>(B.cap); B.sval_alt = A.alloc<uint32_t>(B.cap);
    B.sort_tmp = A.alloc<char>(radix_temp_bytes(B.cap));
    int bits = 1;
    while ((1ll << bits) < (long long)cap) bits++;
    B.sort_bits = 32 + bits;
    B.rec = A.alloc<PairRec>(B.cap);
    B.kind = A.alloc<int>(B.cap);
    B.sflag = A.alloc<int>(B.cap); B.spos = A.alloc<int>(B.cap);
    B.eflag = A.alloc<int>(B.cap); B.epos = A.alloc<int>(B.cap);
    B.inv = A.alloc<int>(cap);
    B.min5 = A.alloc<int>((size_t)h->T.cap_int * 5);
    B.ibox = A.alloc<float4>(h->T.cap_int);
    B.lbox = A.alloc<float4>(h->T.cap_pts);
    B.m5cnt = A.alloc<int>(h->T.cap_int);
    B.tflag = A.alloc<int>(cap);
    B.tpos = A.alloc<int>(cap);
    B.tk = A.alloc<int>(cap);
    B.acnt = A.alloc<int>(cap);
    B.abefore = A.alloc<int>(cap);
    B.amin = A.alloc<int>(cap);
    B.anch = A.alloc<int>(B.cap);
    B.tgt2 = A.alloc<int>((size_t)2 * cap);
    B.events = A.alloc<double>((size_t)COL_EVENT_CAP * 6);
    B.scan_tmp = A.alloc<int>(scan_temp_ints(std::max(cap, B.cap)) + 16);
    if (A.failed) { A.free_all(); B = CollBufs{}; return set_err(h, GEON_ERR_NOMEM, "collision buffer allocation failed"); }
    if (!h->col_h && cudaMallocHost(&h->col_h, sizeof(CollCtl)) != cudaSuccess) {
        h->col_h = nullptr;
        return set_err(h, GEON_ERR_NOMEM, "pinned allocation failed");
    }
    CK(cudaMemsetAsync(B.cc, 0, sizeof(CollCtl), h->st));
    h->col_cap_int = h->T.cap_int;
    h->col_alloc = true;
    return GEON_OK;
}

// handleCollisions for one substep, over the tree just built
// (integrator.js:1350-1381).  With Barnes-Hut the removed particles stay in
// their slots (they are still tree sources) and the spawns sit in slots n,
// n+1, ...: the force pass then walks the collision target list and
// collide_finish compacts after it.  The pairwise sum reads its sources from
// the particle slots, so there the compaction happens at once.  `spawned`
// stays -1 when no compaction is pending.
static int collide_step(GeonHandle* h, int& spawned, int& removed) {
    spawned = -1;
    removed = 0;
    int r = ensure_collide(h);
    if (r) return r;
    CollBufs& B = h->col;
    const int n = h->n;
    const int pc = prof_begin(h, PH_COLLIDE);
    collide_detect(h->P, h->S, h->T, h->d_root, h->ctl, B, h->n_cap, h->st, h->lc);
    CKL();
    CK(cudaMemcpyAsync(h->col_h, B.cc, sizeof(CollCtl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const int total = h->col_h->total;
    if (h->col_h->err & COL_ERR_QUERY) { prof_end(h, pc); return set_err(h, GEON_ERR_OVERFLOW, "merge collisions: tree query failed"); }
    if (total > B.cap) {
        prof_end(h, pc);
        return set_err(h, GEON_ERR_OVERFLOW, "merge collisions: " + std::to_string(total) +
                       " overlap candidates, more than the " + std::to_string(B.cap) + " the buffers hold");
    }
    if (total == 0) {                                     // nothing touches: no resolution, no compaction
        prof_end(h, pc);
        h->col_info.order_approx |= (h->col_h->err & COL_ERR_ORDER) ? 1 : 0;
        return GEON_OK;
    }
    collide_resolve(h->P, h->S, h->T, h->ctl, B, h->keep, n, total, h->slots, h->simTime, h->nextId, h->st, h->lc);
    CKL();
    prof_end(h, pc);
    CK(cudaMemcpyAsync(h->col_h, B.cc, sizeof(CollCtl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const CollCtl c = *h->col_h;
    if (c.err & (COL_ERR_SLOTS | COL_ERR_QUERY)) {
        std::string why = (c.err & COL_ERR_SLOTS) ? "no slot for a merged particle" : "pair components failed";
        return set_err(h, GEON_ERR_OVERFLOW, "merge collisions: " + why);
    }
    GeonCollisionInfo& I = h->col_info;
    I.merges += c.merges;
    I.annihilations += c.annihilations;
    I.spawned += c.spawned;
    I.removed += c.removed;
    I.candidates += c.total;
    I.events = c.events;
    I.events_dropped = c.events_dropped;
    I.order_approx |= (c.err & COL_ERR_ORDER) ? 1 : 0;
    if (c.spawned + c.annihilations == 0) return GEON_OK;
    h->nextId += c.spawned;
    if (bh_on(h)) {
        collide_targets(h->S, h->T, h->ctl, B, n, total, c.spawned, h->n_cap, h->st, h->lc);
        CKL();
        h->col_tgt_active = true;
        h->col_tgt_count = n - c.removed + c.spawned;
        set_n_kernel<<<1, 1, 0, h->st>>>(h->ctl, n + c.spawned);
        h->lc.add(1);
        spawned = c.spawned;
        removed = c.removed;
        return GEON_OK;
    }
    r = compact(h, n + c.spawned);
    if (r) return r;
    h->n = n - c.removed + c.spawned;
    set_n_kernel<<<1, 1, 0, h->st>>>(h->ctl, h->n);
    h->lc.add(1);
    return GEON_OK;
}

// Compaction after the force pass that followed the collisions (keep flags
// were written by the resolution): removed particles leave, spawns follow the
// survivors in spawn order (collisions.js:96-104, integrator.js:1363-1371).
static int collide_finish(GeonHandle* h, int spawned, int removed) {
    h->col_tgt_active = false;
    const int n = h->n;
    int r = compact(h, n + spawned);
    if (r) return r;
    h->n = n - removed + spawned;
    set_n_kernel<<<1, 1, 0, h->st>>>(h->ctl, h->n);
    h->lc.add(1);
    return GEON_OK;
}

// =============================================================================================
extern "C" {

const char* geon_version(void) { return GEON_VERSION_STRING; }

const char* geon_last_error(GeonHandle* h) { return h ? h->err.c_str() : g_err.c_str(); }

int geon_create(const GeonParams* params, int32_t max_particles, GeonHandle** out) {
    if (!params || !out) return set_err(nullptr, GEON_ERR_ARG, "null argument");
    if (max_particles <= 0 || max_particles > (int32_t)REF_INDEX_MASK) return set_err(nullptr, GEON_ERR_ARG, "max_particles out of range");
    *out = nullptr;
    GeonHandle* h = new GeonHandle();
    h->prm = *params;
    if (h->prm.max_substeps <= 0) h->prm.max_substeps = 32;
    int r = validate_params(h, h->prm);
    if (r) { g_err = h->err; delete h; return r; }
    h->n_cap = max_particles;
    derive_params(h);
    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
        g_err = "cudaStreamCreate failed"; delete h; return GEON_ERR_CUDA;
    }
    DevArena& A = h->arena;
    h->ctl = A.alloc<FrameCtl>(1);
    h->d_root = A.alloc<int>(1);
    h->hist_t = A.alloc<double>(HIST_LEN);
    h->hist_age = A.alloc<float>(HIST_LEN);
    h->hist_segdt = A.alloc<float>(HIST_LEN);
    h->staging = A.alloc<float>((size_t)GEON_ST_ROWS * h->n_cap);
    h->staging_d = A.alloc<double>((size_t)GEON_ST_ROWS * h->n_cap);
    h->stats_d = A.alloc<double>(16);
    h->frun = A.alloc<FrameRun>(1);
    if (A.failed || cudaMallocHost(&h->ctl_h, sizeof(FrameCtl)) != cudaSuccess ||
        cudaMallocHost(&h->stats_h, 16 * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&h->frun_h, sizeof(FrameRun)) != cudaSuccess) {
        A.free_all();
        if (h->ctl_h) cudaFreeHost(h->ctl_h);
        if (h->stats_h) cudaFreeHost(h->stats_h);
        if (h->frun_h) cudaFreeHost(h->frun_h);
        cudaStreamDestroy(h->st);
        g_err = "device allocation failed";
        delete h;
        return GEON_ERR_NOMEM;
    }
    cudaMemsetAsync(h->ctl, 0, sizeof(FrameCtl), h->st);
    cudaMemsetAsync(h->hist_t, 0, HIST_LEN * sizeof(double), h->st);
    cudaMemsetAsync(h->frun, 0, sizeof(FrameRun), h->st);
    memset(h->frun_h, 0, sizeof(FrameRun));
    r = alloc_state(h, slots_wanted(h));
    if (r) { g_err = h->err; geon_destroy(h); return r; }
    r = ensure_history(h);
    if (!r) r = ensure_tree(h);
    if (r) { g_err = h->err; geon_destroy(h); return r; }
    if (cudaStreamSynchronize(h->st) != cudaSuccess) { g_err = "initialisation failed"; geon_destroy(h); return GEON_ERR_CUDA; }
    *out = h;
    return GEON_OK;
}

int geon_destroy(GeonHandle* h) {
    if (!h) return GEON_ERR_ARG;
    if (h->st) cudaStreamSynchronize(h->st);
    h->tree_arena.free_all();
    h->hist_arena.free_all();
    h->learn_arena.free_all();
    h->state_arena.free_all();
    h->col_arena.free_all();
    h->boson_arena.free_all();
    if (h->bos) { geon_destroy(h->bos); h->bos = nullptr; }
    if (h->col_h) cudaFreeHost(h->col_h);
    if (h->recs) cudaFree(h->recs);
    if (h->learn_w_buf) cudaFree(h->learn_w_buf);
    if (h->gcen) cudaFree(h->gcen);
    if (h->rec_off) cudaFree(h->rec_off);
    if (h->rec_scan) cudaFree(h->rec_scan);
    if (h->rec_exp) cudaFree(h->rec_exp);
    if (h->rec_flags) cudaFree(h->rec_flags);
    if (h->rec_net) cudaFree(h->rec_net);
    if (h->rec_cnt) cudaFree(h->rec_cnt);
    if (h->dpart) cudaFree(h->dpart);
    if (h->batch) {
        Batch* B = h->batch;
        if (B->exec) cudaGraphExecDestroy(B->exec);
        if (B->graph) cudaGraphDestroy(B->graph);
        if (B->any_h) cudaFreeHost(B->any_h);
        if (B->dt_h) cudaFreeHost(B->dt_h);
        if (B->plan_h) cudaFreeHost(B->plan_h);
        B->A.free_all();
        delete B;
        h->batch = nullptr;
    }
    h->arena.free_all();
    prof_collect(h);
    for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
    if (h->ctl_h) cudaFreeHost(h->ctl_h);
    if (h->stats_h) cudaFreeHost(h->stats_h);
    if (h->frun_h) cudaFreeHost(h->frun_h);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
    return GEON_OK;
}

static int validate_batch_params(GeonHandle* h, const GeonParams& p);
static void batch_drop_graph(Batch& B);

int geon_set_params(GeonHandle* h, const GeonParams* params) {
    if (!h || !params) return GEON_ERR_ARG;
    GeonParams p = *params;
    if (p.max_substeps <= 0) p.max_substeps = 32;
    int r = validate_params(h, p);
    if (r) return r;
    if (h->batch) {
        r = validate_batch_params(h, p);
        if (r) return r;
        batch_drop_graph(*h->batch);
    }
    h->prm = p;
    derive_params(h);
    if (h->slots < slots_wanted(h)) {
        r = alloc_state(h, slots_wanted(h));
        if (r) return r;
    }
    r = ensure_history(h);
    if (r) return r;
    return ensure_tree(h);
}

int geon_get_params(GeonHandle* h, GeonParams* out) {
    if (!h || !out) return GEON_ERR_ARG;
    *out = h->prm;
    return GEON_OK;
}

int geon_add_particles(GeonHandle* h, int32_t n, const float* soa, double creation_time, int32_t* first_index) {
    if (!h || (!soa && n > 0) || n < 0) return GEON_ERR_ARG;
    if (h->batch && !(h->n == 0 && n == h->n_cap))
        return set_err(h, GEON_ERR_UNSUPPORTED, "a batched handle takes its whole batch at once (geon_upload_state)");
    if (n == 0) { if (first_index) *first_index = h->n; return GEON_OK; }
    if ((long long)h->n + n > h->n_cap) return set_err(h, GEON_ERR_FULL, "particle capacity exhausted");
    const int cap = h->n_cap;
    for (int r = 0; r < GEON_ST_ROWS_IN; r++)
        CK(cudaMemcpyAsync(h->staging + (size_t)r * cap, soa + (size_t)r * n, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
    init_particles_kernel<<<grid_for(n, 256), 256, 0, h->st>>>(h->P, h->S, h->staging, cap, h->n, n, creation_time, h->nextId, 0);
    CKL();
    h->lc.add(1);
    if (first_index) *first_index = h->n;
    h->n += n;
    h->nextId += n;
    set_n_kernel<<<1, 1, 0, h->st>>>(h->ctl, h->n);
    h->lc.add(1);
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_remove_particle(GeonHandle* h, int32_t index) {
    if (!h || index < 0 || index >= h->n) return GEON_ERR_ARG;
    if (h->batch) return set_err(h, GEON_ERR_UNSUPPORTED, "particles of a batched handle cannot be removed");
    std::vector<int> keep(h->n, 1);
    keep[index] = 0;
    CK(cudaMemcpyAsync(h->keep, keep.data(), h->n * sizeof(int), cudaMemcpyHostToDevice, h->st));
    int r = compact(h);
    if (r) return r;
    h->n -= 1;
    set_n_kernel<<<1, 1, 0, h->st>>>(h->ctl, h->n);
    h->lc.add(1);
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_reset(GeonHandle* h) {
    if (!h) return GEON_ERR_ARG;
    h->n = 0;
    h->simTime = 0;
    h->forcesInit = false;
    h->histStride = 0;
    h->histTotal = 0;
    h->lastSubsteps = 0;
    CK(cudaMemsetAsync(h->ctl, 0, sizeof(FrameCtl), h->st));
    CK(cudaMemsetAsync(h->hist_t, 0, HIST_LEN * sizeof(double), h->st));
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_upload_state(GeonHandle* h, int32_t n, const float* soa, double sim_time) {
    int r = geon_reset(h);
    if (r) return r;
    h->simTime = sim_time;
    // loaded particles are treated as always existing (save-load.js:231)
    return geon_add_particles(h, n, soa, -INFINITY, nullptr);
}

int geon_upload_state_f64(GeonHandle* h, int32_t n, const double* soa, double sim_time) {
    if (!h || n < 0 || (n > 0 && !soa)) return GEON_ERR_ARG;
    if (n > h->n_cap) return set_err(h, GEON_ERR_FULL, "particle capacity exhausted");
    if (h->batch && n != h->n_cap)
        return set_err(h, GEON_ERR_UNSUPPORTED, "a batched handle takes its whole batch at once (geon_upload_state)");
    int r = geon_reset(h);
    if (r) return r;
    h->simTime = sim_time;
    if (n == 0) return GEON_OK;
    const int cap = h->n_cap;
    std::vector<float> rows((size_t)9 * n);
    for (int i = 0; i < n; i++) {
        for (int c = 0; c < 2; c++) {                      // positions as hi + lo pairs
            const double v = soa[(size_t)c * n + i];
            const float hi = (float)v;
            rows[(size_t)c * n + i] = hi;
            rows[(size_t)(7 + c) * n + i] = (float)(v - (double)hi);
        }
        for (int c = 2; c < GEON_ST_ROWS_IN; c++) rows[(size_t)c * n + i] = (float)soa[(size_t)c * n + i];
    }
    for (int c = 0; c < 9; c++)
        CK(cudaMemcpyAsync(h->staging + (size_t)c * cap, rows.data() + (size_t)c * n, n * sizeof(float),
                           cudaMemcpyHostToDevice, h->st));
    init_particles_kernel<<<grid_for(n, 256), 256, 0, h->st>>>(h->P, h->S, h->staging, cap, 0, n, -INFINITY, h->nextId, 1);
    CKL();
    h->lc.add(1);
    h->n = n;
    h->nextId += n;
    set_n_kernel<<<1, 1, 0, h->st>>>(h->ctl, h->n);
    h->lc.add(1);
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_particle_count(GeonHandle* h, int32_t* n) {
    if (!h || !n) return GEON_ERR_ARG;
    *n = h->n;
    return GEON_OK;
}

int geon_download_state(GeonHandle* h, float* soa, int32_t rows, int32_t capacity, int32_t* n) {
    if (!h || !soa || rows <= 0 || rows > GEON_ST_ROWS || capacity < 0) return GEON_ERR_ARG;
    const int cnt = std::min(h->n, capacity);
    if (cnt > 0) {
        pack_state_kernel<float><<<grid_for(cnt, 256), 256, 0, h->st>>>(h->S, cnt, rows, h->n_cap, h->staging);
        CKL();
        h->lc.add(1);
        for (int r = 0; r < rows; r++)
            CK(cudaMemcpyAsync(soa + (size_t)r * capacity, h->staging + (size_t)r * h->n_cap, cnt * sizeof(float), cudaMemcpyDeviceToHost, h->st));
    }
    CK(cudaStreamSynchronize(h->st));
    if (n) *n = h->n;
    return GEON_OK;
}

int geon_download_state_f64(GeonHandle* h, double* soa, int32_t rows, int32_t capacity, int32_t* n) {
    if (!h || !soa || rows <= 0 || rows > GEON_ST_ROWS || capacity < 0) return GEON_ERR_ARG;
    const int cnt = std::min(h->n, capacity);
    if (cnt > 0) {
        pack_state_kernel<double><<<grid_for(cnt, 256), 256, 0, h->st>>>(h->S, cnt, rows, h->n_cap, h->staging_d);
        CKL();
        h->lc.add(1);
        for (int r = 0; r < rows; r++)
            CK(cudaMemcpyAsync(soa + (size_t)r * capacity, h->staging_d + (size_t)r * h->n_cap, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    }
    CK(cudaStreamSynchronize(h->st));
    if (n) *n = h->n;
    return GEON_OK;
}

int geon_download_ids(GeonHandle* h, int32_t* ids, int32_t capacity, int32_t* n) {
    if (!h || !ids || capacity < 0) return GEON_ERR_ARG;
    const int cnt = std::min(h->n, capacity);
    if (cnt > 0) CK(cudaMemcpyAsync(ids, h->S.id, cnt * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (n) *n = h->n;
    return GEON_OK;
}

static int batch_forces(GeonHandle* h, bool all);

int geon_compute_forces(GeonHandle* h) {
    if (!h) return GEON_ERR_ARG;
    if (h->n == 0) return GEON_OK;
    int r = h->batch ? batch_forces(h, true) : run_force_pass(h, true);
    if (r) return r;
    return read_ctl(h);
}

int geon_compute_1pn(GeonHandle* h) {
    if (!h) return GEON_ERR_ARG;
    if (h->batch) return set_err(h, GEON_ERR_UNSUPPORTED, "batched handles run without 1PN");
    if (h->n == 0) return GEON_OK;
    const bool bh = bh_on(h);
    if (bh) { int r = build_tree(h); if (r) return r; }
    launch_hist_tables(h->hist_t, h->simTime, h->hist_age, h->hist_segdt, h->st, h->lc);
    onepn_pass(h->P, h->S, h->T, h->d_root, h->ctl, onepn_ctx(h, bh), bh, h->n_cap, h->st, h->lc);
    CKL();
    return read_ctl(h);
}

int geon_direct_forces(GeonHandle* h, const int32_t* idx, int32_t k, float* fx, float* fy) {
    if (!h || k < 0 || (k > 0 && (!idx || !fx || !fy))) return GEON_ERR_ARG;
    if (h->batch) return set_err(h, GEON_ERR_UNSUPPORTED, "the pairwise subset sum would mix the systems of a batched handle");
    if (k == 0 || h->n == 0) return GEON_OK;
    for (int i = 0; i < k; i++)
        if (idx[i] < 0 || idx[i] >= h->n) return set_err(h, GEON_ERR_ARG, "index out of range");
    DevArena tmp;
    int* d_idx = tmp.alloc<int>(k);
    float* d_fx = tmp.alloc<float>(k);
    float* d_fy = tmp.alloc<float>(k);
    const DirectPlan pl = direct_subset_plan(h->P, k);           // source slices that fill the GPU
    float* d_part = pl.slices > 1 ? tmp.alloc<float>(pl.floats) : nullptr;
    if (tmp.failed) { tmp.free_all(); return set_err(h, GEON_ERR_NOMEM, "direct-forces allocation failed"); }
    ForceCtx C = make_ctx(h);
    C.dpart = d_part;
    C.dslices = pl.slices;
    cudaError_t e = cudaMemcpyAsync(d_idx, idx, k * sizeof(int), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess && h->P.rel) { launch_hist_tables(h->hist_t, h->simTime, h->hist_age, h->hist_segdt, h->st, h->lc); e = cudaGetLastError(); }
    if (e == cudaSuccess) {
        direct_subset(h->P, h->S, h->ctl, C, d_idx, k, d_fx, d_fy, h->st, h->lc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(fx, d_fx, k * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fy, d_fy, k * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    tmp.free_all();
    return cuda_check(h, e, "direct forces");
}

// Checks and tree of the learned-correction entry points: the force set the
// correction covers, a tree with cell moments at the handle's theta, and the
// Barnes-Hut walk with record emission (plain forces in S.force).
static int learn_prepare(GeonHandle* h) {
    if (!(h->prm.toggles & GEON_BARNES_HUT)) return set_err(h, GEON_ERR_ARG, "the learned correction needs Barnes-Hut");
    if (!learn_supported(h))
        return set_err(h, GEON_ERR_UNSUPPORTED, "the learned correction covers gravity, Coulomb and Yukawa without "
                                                "relativity, dipoles, 1PN or breakdown rows, in an open box, one system per handle");
    const uint32_t saved = h->prm.flags;
    h->prm.flags |= GEON_FLAG_LEARN;
    int r = build_tree(h);
    h->prm.flags = saved;
    if (r) return r;
    return learn_walk(h);
}

int geon_learn_dataset(GeonHandle* h, int32_t group_stride, int64_t cap, float gfloor, float* feat, float* target,
                       int32_t* rec_group, int64_t* count) {
    if (!h || group_stride < 1 || cap < 0 || (cap > 0 && (!feat || !target)) || !(gfloor >= 0.f)) return GEON_ERR_ARG;
    if (count) *count = 0;
    if (h->n == 0) return GEON_OK;
    int r = learn_prepare(h);
    if (r) return r;
    const int ngroups = (h->n + 31) / 32;
    const int nsel = (ngroups + group_stride - 1) / group_stride;
    DevArena tmp;
    int* d_off = tmp.alloc<int>(nsel + 1);
    int* d_total = tmp.alloc<int>(1);
    void* d_scan = tmp.alloc<char>(learn_offsets_scratch_bytes(nsel));
    if (tmp.failed) { tmp.free_all(); return set_err(h, GEON_ERR_NOMEM, "dataset allocation failed"); }
    learn_record_offsets(h->rec_cnt, h->rec_cap, ngroups, group_stride, d_off, d_total, d_scan, h->st, h->lc);
    int total = 0;
    cudaError_t e = cudaMemcpyAsync(&total, d_total, sizeof(int), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) { tmp.free_all(); return cuda_check(h, e, "dataset offsets"); }
    const long long m = std::min<long long>(total, cap);
    if (m > 0) {
        float* d_feat = tmp.alloc<float>((size_t)m * LF);
        float* d_tg = tmp.alloc<float>((size_t)m * LT);
        int* d_grp = rec_group ? tmp.alloc<int>((size_t)m) : nullptr;
        if (tmp.failed) { tmp.free_all(); return set_err(h, GEON_ERR_NOMEM, "dataset allocation failed"); }
        learn_records(h->P, h->S, h->T, h->recs, h->rec_cnt, h->gcen, h->rec_cap, ngroups, group_stride, d_off, (int)m,
                      gfloor, d_feat, d_tg, d_grp, h->ctl, h->st, h->lc);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(feat, d_feat, (size_t)m * LF * sizeof(float), cudaMemcpyDeviceToHost, h->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(target, d_tg, (size_t)m * LT * sizeof(float), cudaMemcpyDeviceToHost, h->st);
        if (e == cudaSuccess && d_grp) e = cudaMemcpyAsync(rec_group, d_grp, (size_t)m * sizeof(int), cudaMemcpyDeviceToHost, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    }
    tmp.free_all();
    if (count) *count = total;
    r = cuda_check(h, e, "learned-correction dataset");
    if (r) return r;
    return read_ctl(h);
}

int geon_learn_apply(GeonHandle* h, const float* y, int64_t n) {
    if (!h || n < 0 || (n > 0 && !y)) return GEON_ERR_ARG;
    if (h->n == 0) return n == 0 ? GEON_OK : set_err(h, GEON_ERR_ARG, "no particles");
    int r = learn_prepare(h);
    if (r) return r;
    if (h->rec_total_h != n) return set_err(h, GEON_ERR_ARG, "n differs from the record count");
    DevArena tmp;
    float* d_y = tmp.alloc<float>((size_t)std::max<int64_t>(n, 1) * LO);
    if (tmp.failed) { tmp.free_all(); return set_err(h, GEON_ERR_NOMEM, "allocation failed"); }
    cudaError_t e = n > 0 ? cudaMemcpyAsync(d_y, y, (size_t)n * LO * sizeof(float), cudaMemcpyHostToDevice, h->st) : cudaSuccess;
    if (e == cudaSuccess) {
        r = learn_correct_records(h, d_y);
        if (r) { cudaStreamSynchronize(h->st); tmp.free_all(); return r; }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    tmp.free_all();
    r = cuda_check(h, e, "learned-correction apply");
    return r ? r : read_ctl(h);
}

int geon_learn_set_weights(GeonHandle* h, const float* weights, int32_t n_param) {
    if (!h) return GEON_ERR_ARG;
    if (!weights) { h->learn_w = nullptr; return GEON_OK; }       // the buffer stays for reuse
    if (n_param != MLP_NPARAM) return set_err(h, GEON_ERR_ARG, "n_param must be GEON_MLP_NPARAM");
    static_assert(MLP_NPARAM == GEON_MLP_NPARAM, "weight count");
    static_assert(LF == GEON_LEARN_FEATURES && LO == GEON_LEARN_OUTPUTS && LT == GEON_LEARN_TARGETS, "record layout");
    if (!h->learn_w_buf) {
        float* w = nullptr;
        if (cudaMalloc(&w, MLP_NPARAM * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            return set_err(h, GEON_ERR_NOMEM, "weight allocation failed");
        }
        h->learn_w_buf = w;
    }
    CK(cudaMemcpyAsync(h->learn_w_buf, weights, MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->learn_w = h->learn_w_buf;
    return GEON_OK;
}

// Device copies of a training set for the network entry points.
struct MlpData {
    DevArena A;
    float* w = nullptr; float* x = nullptr; float* t = nullptr; float* wt = nullptr;
    float* grad = nullptr; double* loss = nullptr;
    float* part = nullptr; double* loss_part = nullptr;   // per-CTA gradient slots
};
static int mlp_upload(GeonHandle* h, MlpData& D, const float* weights, const float* x, const float* t, const float* wt,
                      int n, int nloss) {
    D.w = D.A.alloc<float>(MLP_NPARAM);
    D.x = D.A.alloc<float>((size_t)n * LF);
    if (t) D.t = D.A.alloc<float>((size_t)n * LT);
    if (wt) D.wt = D.A.alloc<float>(n);
    D.grad = D.A.alloc<float>(MLP_NPARAM);
    D.loss = D.A.alloc<double>(std::max(nloss, 1));
    D.part = D.A.alloc<float>(mlp_grad_scratch_floats());
    D.loss_part = D.A.alloc<double>(mlp_grad_scratch_ctas());
    if (D.A.failed) { D.A.free_all(); return set_err(h, GEON_ERR_NOMEM, "network buffer allocation failed"); }
    cudaError_t e = cudaMemcpyAsync(D.w, weights, MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(D.x, x, (size_t)n * LF * sizeof(float), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess && t) e = cudaMemcpyAsync(D.t, t, (size_t)n * LT * sizeof(float), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess && wt) e = cudaMemcpyAsync(D.wt, wt, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(D.grad, 0, MLP_NPARAM * sizeof(float), h->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(D.loss, 0, std::max(nloss, 1) * sizeof(double), h->st);
    if (e != cudaSuccess) { D.A.free_all(); return cuda_check(h, e, "network upload"); }
    return GEON_OK;
}

int geon_mlp_forward(GeonHandle* h, const float* weights, const float* x, int32_t n, float* y) {
    if (!h || !weights || n < 0 || (n > 0 && (!x || !y))) return GEON_ERR_ARG;
    if (n == 0) return GEON_OK;
    MlpData D;
    int r = mlp_upload(h, D, weights, x, nullptr, nullptr, n, 0);
    if (r) return r;
    float* dy = D.A.alloc<float>((size_t)n * LO);
    cudaError_t e = D.A.failed ? cudaErrorMemoryAllocation : cudaSuccess;
    if (e == cudaSuccess) {
        mlp_forward(D.w, D.x, n, dy, &h->ctl->err, h->st, h->lc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(y, dy, (size_t)n * LO * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    D.A.free_all();
    r = cuda_check(h, e, "network forward");
    return r ? r : read_ctl(h);
}

int geon_mlp_grad(GeonHandle* h, const float* weights, const float* x, const float* t, const float* wt, int32_t n,
                  float* grad, double* loss) {
    if (!h || !weights || !grad || n <= 0 || !x || !t) return GEON_ERR_ARG;
    MlpData D;
    int r = mlp_upload(h, D, weights, x, t, wt, n, 1);
    if (r) return r;
    mlp_grad(D.w, D.x, D.t, D.wt, n, n, 0ull, 0, D.grad, D.loss, D.part, D.loss_part, &h->ctl->err, h->st, h->lc);
    cudaError_t e = cudaGetLastError();
    double l = 0.0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad, D.grad, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&l, D.loss, sizeof(double), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    D.A.free_all();
    if (loss) *loss = l;
    r = cuda_check(h, e, "network gradient");
    return r ? r : read_ctl(h);
}

int geon_mlp_train(GeonHandle* h, float* weights, const float* x, const float* t, const float* wt, int32_t n,
                   int32_t steps, int32_t batch, float lr, uint64_t seed, double* loss_history) {
    if (!h || !weights || !x || !t || n <= 0 || steps < 0 || batch <= 0 || !(lr > 0.f)) return GEON_ERR_ARG;
    if (steps == 0) return GEON_OK;
    MlpData D;
    int r = mlp_upload(h, D, weights, x, t, wt, n, steps);
    if (r) return r;
    float* m = D.A.alloc<float>(MLP_NPARAM);
    float* v = D.A.alloc<float>(MLP_NPARAM);
    cudaError_t e = D.A.failed ? cudaErrorMemoryAllocation : cudaSuccess;
    if (e == cudaSuccess) e = cudaMemsetAsync(m, 0, MLP_NPARAM * sizeof(float), h->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(v, 0, MLP_NPARAM * sizeof(float), h->st);
    const uint64_t sd = seed ? seed : 0x5DEECE66Dull;
    for (int s = 0; s < steps && e == cudaSuccess; s++) {
        const double lr_s = 0.5 * (double)lr * (1.0 + std::cos(3.141592653589793 * (double)s / (double)steps));
        mlp_grad(D.w, D.x, D.t, D.wt, n, batch, sd, s, D.grad, D.loss + s, D.part, D.loss_part, &h->ctl->err, h->st,
                 h->lc);
        mlp_adam(D.w, D.grad, m, v, (float)lr_s, 0.9f, 0.999f, 1e-8f, s + 1, h->st, h->lc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(weights, D.w, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess && loss_history)
        e = cudaMemcpyAsync(loss_history, D.loss, (size_t)steps * sizeof(double), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    D.A.free_all();
    r = cuda_check(h, e, "network training");
    return r ? r : read_ctl(h);
}

__global__ void set_matter_kernel(DevState S, int first, int count, const float* __restrict__ rows, int has_anti,
                                  int has_base) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
        float2 m = S.matter[first + t];
        if (has_anti) m.y = rows[t] != 0.f ? 1.f : 0.f;
        if (has_base) m.x = rows[count + t];
        S.matter[first + t] = m;
    }
}

int geon_set_matter(GeonHandle* h, int32_t first, int32_t count, const int32_t* antimatter, const float* base_mass) {
    if (!h || first < 0 || count < 0 || (long long)first + count > h->n)
        return set_err(h, GEON_ERR_ARG, "matter range outside the particles");
    if (count == 0 || (!antimatter && !base_mass)) return GEON_OK;
    std::vector<float> rows((size_t)2 * count, 0.f);
    for (int t = 0; t < count; t++) {
        if (antimatter) rows[t] = antimatter[t] ? 1.f : 0.f;
        if (base_mass) rows[count + t] = base_mass[t];
    }
    // the staging area holds GEON_ST_ROWS x n_cap floats >= 2 * count
    CK(cudaMemcpyAsync(h->staging, rows.data(), rows.size() * sizeof(float), cudaMemcpyHostToDevice, h->st));
    set_matter_kernel<<<grid_for(count, 256), 256, 0, h->st>>>(h->S, first, count, h->staging, antimatter ? 1 : 0,
                                                               base_mass ? 1 : 0);
    CKL();
    h->lc.add(1);
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_get_matter(GeonHandle* h, int32_t* antimatter, float* base_mass, int32_t capacity, int32_t* n) {
    if (!h || capacity < 0 || !n) return GEON_ERR_ARG;
    const int cnt = std::min(capacity, h->n);
    *n = h->n;
    if (cnt == 0) return GEON_OK;
    std::vector<float2> m(cnt);
    CK(cudaMemcpyAsync(m.data(), h->S.matter, cnt * sizeof(float2), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (int i = 0; i < cnt; i++) {
        if (antimatter) antimatter[i] = m[i].y != 0.f ? 1 : 0;
        if (base_mass) base_mass[i] = m[i].x;
    }
    return GEON_OK;
}

int geon_collision_info(GeonHandle* h, GeonCollisionInfo* out) {
    if (!h || !out) return GEON_ERR_ARG;
    *out = h->col_info;
    return GEON_OK;
}

int geon_collision_events(GeonHandle* h, double* events, int32_t capacity, int32_t* n) {
    if (!h || !n || capacity < 0 || (capacity > 0 && !events)) return GEON_ERR_ARG;
    const int stored = h->col_info.events;
    *n = stored;
    const int cnt = std::min(capacity, stored);
    if (cnt > 0) {
        CK(cudaMemcpyAsync(events, h->col.events, (size_t)cnt * 6 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
    }
    return GEON_OK;
}

int geon_set_bosons(GeonHandle* h, int32_t n, const double* rows) {
    if (!h || n < 0 || (n > 0 && !rows)) return GEON_ERR_ARG;
    if (h->batch) return set_err(h, GEON_ERR_UNSUPPORTED, "batched handles have no boson pool");
    h->nb = 0;
    h->nb_massive = 0;
    if (n == 0) return GEON_OK;
    GeonParams bp = h->prm;                   // the pool's tree: same root box, no ghosts (integrator.js:263-277)
    bp.flags = GEON_FLAG_NO_GHOSTS;
    bp.collision_mode = GEON_COL_PASS;
    int r;
    if (!h->bos || h->bos->n_cap < n) {
        if (h->bos) { geon_destroy(h->bos); h->bos = nullptr; }
        h->boson_arena.free_all();
        h->boson_arena.failed = false;
        int cap = 1024;
        while (cap < n) cap *= 2;
        r = geon_create(&bp, cap, &h->bos);
        if (r) { h->bos = nullptr; return set_err(h, r, std::string("boson pool: ") + g_err); }
        h->bkind = h->boson_arena.alloc<float2>(cap);
        h->bkick = h->boson_arena.alloc<float2>(cap);
        h->biq = h->boson_arena.alloc<double>(h->bos->T.cap_int);
        h->blq = h->boson_arena.alloc<double>(h->bos->T.cap_pts);
        if (h->boson_arena.failed) return set_err(h, GEON_ERR_NOMEM, "boson pool allocation failed");
    } else {
        r = geon_set_params(h->bos, &bp);
        if (r) return set_err(h, r, std::string("boson pool: ") + h->bos->err);
    }
    std::vector<double> soa((size_t)GEON_ST_ROWS_IN * n, 0.0);
    std::vector<float2> kind(n);
    int massive = 0;
    for (int i = 0; i < n; i++) {
        const double* q = rows + (size_t)i * 6;
        soa[i] = q[0];                        // x, y, (w = 0), mass = _srcMass, charge = _srcCharge, (angw = 0)
        soa[(size_t)n + i] = q[1];
        soa[(size_t)4 * n + i] = q[2];
        soa[(size_t)5 * n + i] = q[3];
        kind[i] = make_float2(q[4] != 0 ? 1.f : 0.f, (float)q[5]);
        massive += q[4] != 0;
    }
    r = geon_upload_state_f64(h->bos, n, soa.data(), 0.0);
    if (r) return set_err(h, r, std::string("boson pool: ") + h->bos->err);
    r = build_tree(h->bos);
    if (r) return set_err(h, r, std::string("boson pool: ") + h->bos->err);
    r = read_ctl(h->bos);
    if (r) return set_err(h, r, std::string("boson pool: ") + h->bos->err);
    CK(cudaMemcpyAsync(h->bkind, kind.data(), n * sizeof(float2), cudaMemcpyHostToDevice, h->st));
    h->nb = n;
    boson_charges(boson_tree(h), h->biq, h->blq, h->st, h->lc);
    CKL();
    CK(cudaStreamSynchronize(h->st));
    h->nb_massive = massive;
    return GEON_OK;
}

int geon_boson_kicks(GeonHandle* h, double dt, uint32_t what, float* kicks) {
    if (!h || (h->nb > 0 && !kicks)) return GEON_ERR_ARG;
    if (h->nb == 0) return GEON_OK;
    boson_kicks(h->P, boson_tree(h), (float)dt, what, h->nb_massive, h->bkick, h->st, h->lc);
    CKL();
    CK(cudaMemcpyAsync(kicks, h->bkick, (size_t)h->nb * sizeof(float2), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_heatmap(GeonHandle* h, double left, double top, double cell_w, double cell_h, int32_t grid, uint32_t fields,
                 int32_t blur, float* grav, float* elec, float* yuk) {
    if (!h || grid < 1 || grid > 4096 || !grav || !elec || !yuk) return GEON_ERR_ARG;
    if (h->batch) return set_err(h, GEON_ERR_UNSUPPORTED, "the heat map covers one system");
    const uint32_t tg = h->prm.toggles;
    const bool doG = (fields & 1u) && (tg & GEON_GRAVITY);
    const bool doE = (fields & 2u) && (tg & GEON_COULOMB);
    const bool doY = (fields & 4u) && (tg & GEON_YUKAWA);
    const bool tree = bh_on(h) && h->n > 0;
    if (tree) { int r = build_tree(h); if (r) return r; }
    const size_t gg = (size_t)grid * grid;
    DevArena tmp;
    float* d_g = tmp.alloc<float>(gg);
    float* d_e = tmp.alloc<float>(gg);
    float* d_y = tmp.alloc<float>(gg);
    float* d_t = tmp.alloc<float>(gg);
    const int slices = heatmap_slices(h->P, grid, tree);
    float* d_part = slices > 1 ? tmp.alloc<float>((size_t)slices * 6 * gg) : nullptr;
    if (tmp.failed) { tmp.free_all(); return set_err(h, GEON_ERR_NOMEM, "heat map allocation failed"); }
    cudaError_t e = cudaSuccess;
    if (h->P.rel) { launch_hist_tables(h->hist_t, h->simTime, h->hist_age, h->hist_segdt, h->st, h->lc); e = cudaGetLastError(); }
    if (e == cudaSuccess) {
        heatmap_pass(h->P, h->S, h->T, h->d_root, h->ctl, make_ctx(h), left, top, cell_w, cell_h, grid, doG, doE, doY,
                     tree, blur != 0, d_g, d_e, d_y, d_t, d_part, slices, h->st, h->lc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(grav, d_g, gg * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(elec, d_e, gg * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(yuk, d_y, gg * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    tmp.free_all();
    int r = cuda_check(h, e, "heat map");
    return r ? r : read_ctl(h);
}

int geon_download_forces(GeonHandle* h, int32_t first_row, int32_t rows, float* out, int32_t capacity) {
    if (!h || !out || first_row < 0 || rows <= 0 || first_row + rows > GEON_OUT_ROWS || capacity < 0) return GEON_ERR_ARG;
    const int cnt = std::min(h->n, capacity);
    if (cnt > 0) {
        // staging holds GEON_ST_ROWS rows of n_cap floats: pack in chunks of that many rows
        for (int r0 = 0; r0 < rows; r0 += GEON_ST_ROWS) {
            const int rr = std::min(GEON_ST_ROWS, rows - r0);
            pack_forces_kernel<<<grid_for(cnt, 256), 256, 0, h->st>>>(h->S, cnt, first_row + r0, rr, h->n_cap, h->slots, h->staging);
            CKL();
            h->lc.add(1);
            for (int r = 0; r < rr; r++)
                CK(cudaMemcpyAsync(out + (size_t)(r0 + r) * capacity, h->staging + (size_t)r * h->n_cap, cnt * sizeof(float),
                                   cudaMemcpyDeviceToHost, h->st));
            CK(cudaStreamSynchronize(h->st));
        }
    }
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_build_tree(GeonHandle* h, GeonTreeInfo* info) {
    if (!h) return GEON_ERR_ARG;
    int r = build_tree(h);
    if (r) return r;
    r = read_ctl(h);
    if (r) return r;
    if (info) {
        const FrameCtl& c = *h->ctl_h;
        info->n_points = c.nPts;
        info->n_ghosts = c.nGhost;
        info->n_dropped = c.nPts - c.nValid;
        info->n_internal = c.nInternal;
        info->n_leaves = c.nLeaves;
        info->max_level = c.maxLevel;
        info->n_bucket = c.nBucket;
        info->reserved = 0;
    }
    return GEON_OK;
}

int geon_tree_leaves(GeonHandle* h, int32_t* leaf_of_point, int32_t n_points, double* leaf_bx, double* leaf_by,
                     double* leaf_bw, int32_t* leaf_level, int32_t n_leaves) {
    if (!h || !leaf_of_point || !leaf_bx || !leaf_by || !leaf_bw || !leaf_level) return GEON_ERR_ARG;
    int r = read_ctl(h);
    if (r) return r;
    const FrameCtl c = *h->ctl_h;
    if (n_points < c.nPts || n_leaves < c.nLeaves) return set_err(h, GEON_ERR_ARG, "output arrays too small");
    DevArena tmp;
    int* d_lop = tmp.alloc<int>(std::max(c.nPts, 1));
    double* d_bx = tmp.alloc<double>(std::max(c.nLeaves, 1));
    double* d_by = tmp.alloc<double>(std::max(c.nLeaves, 1));
    double* d_bw = tmp.alloc<double>(std::max(c.nLeaves, 1));
    int* d_lv = tmp.alloc<int>(std::max(c.nLeaves, 1));
    if (tmp.failed) { tmp.free_all(); return set_err(h, GEON_ERR_NOMEM, "leaf dump allocation failed"); }
    tree_leaf_dump(h->P, h->T, h->ctl, d_lop, d_bx, d_by, d_bw, d_lv, c.nPts, h->st, h->lc);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && c.nPts) e = cudaMemcpyAsync(leaf_of_point, d_lop, c.nPts * sizeof(int), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess && c.nLeaves) {
        cudaMemcpyAsync(leaf_bx, d_bx, c.nLeaves * sizeof(double), cudaMemcpyDeviceToHost, h->st);
        cudaMemcpyAsync(leaf_by, d_by, c.nLeaves * sizeof(double), cudaMemcpyDeviceToHost, h->st);
        cudaMemcpyAsync(leaf_bw, d_bw, c.nLeaves * sizeof(double), cudaMemcpyDeviceToHost, h->st);
        e = cudaMemcpyAsync(leaf_level, d_lv, c.nLeaves * sizeof(int), cudaMemcpyDeviceToHost, h->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    tmp.free_all();
    return cuda_check(h, e, "leaf dump");
}

int geon_interaction_count(GeonHandle* h, int64_t* count) {
    if (!h || !count) return GEON_ERR_ARG;
    int r = read_ctl(h);
    if (r) return r;
    *count = (int64_t)h->ctl_h->interactions;
    return GEON_OK;
}

static int batch_update(GeonHandle* h, double dt, int32_t* substeps);

// The whole frame in one launch (frame.cu): a single open system with forces
// already bootstrapped, Barnes-Hut without dipole / 1PN terms, breakdown
// rows, energy sums, merge collisions, learned correction, bosons or
// profiling, and at most FRAME_MAX_POINTS particles.
static bool frame_eligible(const GeonHandle* h) {
    const uint32_t tg = h->prm.toggles, fl = h->prm.flags;
    return !h->batch && h->forcesInit && frame_fits(h->n) && bh_on(h) && !h->P.periodic &&
           !(tg & (GEON_MAGNETIC | GEON_GRAVITOMAG | GEON_ONE_PN)) &&
           !(fl & (GEON_FLAG_PE | GEON_FLAG_BREAKDOWN | GEON_FLAG_SIMPLE_WALK | GEON_FLAG_LEARN | GEON_FLAG_BOSONS |
                   GEON_FLAG_SPLIT_FRAME)) &&
           !merge_on(h) && !h->prof;
}

// geon_update through the frame kernel: one launch, then one read of the
// control block and the frame's results.  FRAME_NOT_LAUNCHED (positive) when
// the device cannot hold the cooperative grid: the caller then runs the frame
// on the launch-per-phase path.
constexpr int FRAME_NOT_LAUNCHED = 1;
static int frame_update(GeonHandle* h, double dt, int32_t* substeps) {
    int r = ensure_tree(h);
    if (r) return r;
    const GeonParams& p = h->prm;
    const uint32_t tg = p.toggles;
    const bool rel = (tg & GEON_RELATIVITY) != 0;
    const bool hasMag = tg & GEON_MAGNETIC, hasGM = tg & GEON_GRAVITOMAG;
    const bool recordHist = rel && h->histStride + 1 >= HIST_STRIDE;    // integrator.js:1550-1565
    if (rel) { r = ensure_history(h); if (r) return r; }
    h->T.mom_on = 0;
    h->T.skey = h->T.key_alt;                 // where the frame kernel's sort leaves the tree order
    h->T.sidx = h->T.idx_alt;
    FrameArgs A{};
    A.dt = dt;
    A.simTime = h->simTime;
    A.softening = p.softening;
    A.maxSub = p.max_substeps;
    A.F.has1PN = 0;
    A.F.needBoris = hasMag || hasGM || p.ext_bz != 0;
    A.F.needSpinOrbit = (tg & GEON_SPIN_ORBIT) && (hasMag || hasGM);
    A.F.needTorques = (hasGM && rel) || (tg & GEON_GRAVITY);
    A.recordHist = recordHist ? 1 : 0;
    A.histSlot = (int)(h->histTotal & HIST_MASK);
    A.hist_t = h->hist_t;
    A.hist_age = h->hist_age;
    A.hist_segdt = h->hist_segdt;
    A.keep = h->keep;
    A.dst = h->dst;
    A.slots = h->slots;
    A.withHist = h->hist_alloc ? 1 : 0;
    A.waitNs = h->frame_wait_ns;
    A.extraArrivals = h->frame_extra;
    ForceCtx C = make_ctx(h);
    // the walk's four warps per group share the subtrees below level 8 (node
    // size 2 rootW / 256); config 1 (N = 2,048): levels 5 / 6 / 7 / 8..10 give
    // 112 / 112 / 101 / 100 us per walk, so 8 (and no deeper, where the
    // duplicated top of the walk grows)
    C.split_level = 8;
    const cudaError_t e = frame_launch(rel, h->P, h->S, h->S2, h->T, h->d_root, h->ctl, C, A, h->frun, h->n, h->st, h->lc);
    if (e == cudaErrorCooperativeLaunchTooLarge || e == cudaErrorNotSupported) {
        cudaGetLastError();                   // nothing was launched: this device takes the launch-per-phase path
        return FRAME_NOT_LAUNCHED;
    }
    if (e != cudaSuccess) return cuda_check(h, e, "frame kernel launch");
    CK(cudaMemcpyAsync(h->frun_h, h->frun, sizeof(FrameRun), cudaMemcpyDeviceToHost, h->st));
    r = read_ctl(h);
    if (r) {
        // a frame that gave up leaves the barrier mid-way: start the next one afresh
        cudaMemsetAsync(h->frun, 0, sizeof(FrameRun), h->st);
        cudaStreamSynchronize(h->st);
        return r;
    }
    const FrameRun& R = *h->frun_h;
    h->simTime = R.simTime;
    h->lastSubsteps = R.substeps;
    if (substeps) *substeps = R.substeps;
    if (rel && ++h->histStride >= HIST_STRIDE) {
        h->histStride -= HIST_STRIDE;
        h->histTotal++;
    }
    if (R.removed > 0) {                      // compacted into S2 by the kernel
        std::swap(h->S, h->S2);
        h->n -= R.removed;
    }
    return GEON_OK;
}

int geon_frame_phases(GeonHandle* h, double* us, int32_t n) {
    if (!h || n < 0 || (n > 0 && !us)) return GEON_ERR_ARG;
    const FrameRun& R = *h->frun_h;
    const int k = std::min(n, FRAME_STAMPS - 1);
    for (int i = 0; i < k; i++)
        us[i] = (R.stamp[i + 1] >= R.stamp[i] && R.stamp[i]) ? 1e-3 * (double)(R.stamp[i + 1] - R.stamp[i]) : 0.0;
    return FRAME_STAMPS - 1;
}

int geon_set_frame_wait(GeonHandle* h, int64_t wait_ns, int32_t extra_arrivals) {
    if (!h || wait_ns <= 0 || extra_arrivals < 0) return GEON_ERR_ARG;
    h->frame_wait_ns = wait_ns;
    h->frame_extra = extra_arrivals;
    return GEON_OK;
}

int geon_update(GeonHandle* h, double dt, int32_t* substeps) {
    if (!h) return GEON_ERR_ARG;
    if (h->batch) return batch_update(h, dt, substeps);
    if (!(dt >= 0)) return set_err(h, GEON_ERR_ARG, "dt must be >= 0");
    int r;
    const GeonParams& p = h->prm;
    const uint32_t tg = p.toggles;
    const bool rel = (tg & GEON_RELATIVITY) != 0;
    const bool hasGrav = tg & GEON_GRAVITY, hasMag = tg & GEON_MAGNETIC, hasGM = tg & GEON_GRAVITOMAG;
    const bool has1PN = tg & GEON_ONE_PN;
    const bool hasExtBz = p.ext_bz != 0;
    const bool bh = bh_on(h);
    const int maxSub = p.max_substeps;
    const double EPS = 1e-12;
    const bool merge = merge_on(h);
    h->col_tgt_active = false;
    h->col_info = GeonCollisionInfo{};
    if (merge) {
        r = ensure_tree(h);
        if (!r) r = ensure_collide(h);
        if (r) return r;
        CK(cudaMemsetAsync(h->col.cc, 0, sizeof(CollCtl), h->st));
    }
    if (!h->forcesInit && h->n > 0) {                                      // integrator.js:750-782
        bootstrap_angvel_kernel<<<grid_for(h->n, 256), 256, 0, h->st>>>(h->P, h->S, h->ctl);
        CKL();
        h->lc.add(1);
        r = run_force_pass(h, true);
        if (r) return r;
        h->forcesInit = true;
    }
    if (frame_eligible(h)) {
        r = frame_update(h, dt, substeps);
        if (r != FRAME_NOT_LAUNCHED) return r;
    }
    // frame-start planner scan (integrator.js:813-836)
    launch_frame_scan(h->P, h->S, h->ctl, h->n_cap, h->st, h->lc);
    CKL();
    r = read_ctl(h);
    if (r) return r;
    double curAccel = bits_to_double(h->ctl_h->maxAccelSqBits);
    double curCyc = bits_to_double(h->ctl_h->maxCycBits);
    double lastKick = 0.0;
    PushFlags F{};
    F.has1PN = has1PN;
    F.needBoris = hasMag || hasGM || hasExtBz;
    F.needSpinOrbit = (tg & GEON_SPIN_ORBIT) && (hasMag || hasGM);
    F.needTorques = (hasGM && rel) || hasGrav;
    double dtRemain = dt;
    int totalSteps = 0;
    while (dtRemain > EPS && totalSteps < maxSub) {                        // integrator.js:810
        const double useAccel = totalSteps == 0 ? curAccel : lastKick;
        double aMax = std::sqrt(useAccel);
        if (aMax != aMax) aMax = 0;
        double dtSafe = aMax > EPS ? std::sqrt(p.softening / aMax) : dtRemain;
        if (curCyc > 0) {
            const double dtCyc = 0.7853981633974483 / curCyc;
            if (dtCyc < dtSafe) dtSafe = dtCyc;
        }
        const double need = std::ceil(dtRemain / dtSafe);
        const double stepsNeeded = std::min(need, (double)(maxSub - totalSteps));
        const double dtSub = dtRemain / stepsNeeded;
        totalSteps++;
        dtRemain -= dtSub;
        lastKick = curAccel;
        if (h->n > 0) {
            const int ps = prof_begin(h, PH_PUSH);
            launch_push(h->P, h->S, h->ctl, (float)dtSub, F, h->n_cap, h->st, h->lc);
            prof_end(h, ps);
            CKL();
            if (h->prof) h->prof_acc.particle_substeps += h->n;
        }
        h->simTime += dtSub;
        if (h->n == 0) continue;
        bool haveTree = false;
        if (has1PN) {                                                      // integrator.js:1297-1318
            if (bh) { r = build_tree(h); if (r) return r; haveTree = true; }
            launch_hist_tables(h->hist_t, h->simTime, h->hist_age, h->hist_segdt, h->st, h->lc);
            const int ps = prof_begin(h, PH_ONEPN);
            onepn_pass(h->P, h->S, h->T, h->d_root, h->ctl, onepn_ctx(h, bh), bh, h->n_cap, h->st, h->lc);
            prof_end(h, ps);
            launch_vv_kick(h->P, h->S, h->ctl, (float)(dtSub * 0.5), h->n_cap, h->st, h->lc);
            CKL();
        }
        int colSpawned = -1, colRemoved = 0;
        if (merge) {                                                       // integrator.js:1340-1381
            if (!haveTree) { r = build_tree(h); if (r) return r; haveTree = true; }
            r = collide_step(h, colSpawned, colRemoved);
            if (r) { h->col_tgt_active = false; return r; }
        }
        r = run_force_pass(h, !haveTree);                                  // integrator.js:1336-1348, 1489-1493
        if (r) { h->col_tgt_active = false; return r; }
        // The planner maxima are read back only for a substep that follows;
        // after the last one the boundary step's read reports any device flag.
        const bool another = dtRemain > EPS && totalSteps < maxSub;
        if (!another && !merge && !h->prof) continue;
        r = read_ctl(h);
        if (r) { h->col_tgt_active = false; return r; }
        if (colSpawned >= 0) { r = collide_finish(h, colSpawned, colRemoved); if (r) return r; }
        if (h->prof) h->prof_acc.interactions += (int64_t)h->ctl_h->interactions;
        curAccel = bits_to_double(h->ctl_h->maxAccelSqBits);
        curCyc = bits_to_double(h->ctl_h->maxCycBits);
    }
    h->lastSubsteps = totalSteps;
    if (substeps) *substeps = totalSteps;
    if (rel && h->n > 0 && ++h->histStride >= HIST_STRIDE) {               // integrator.js:1550-1565
        h->histStride -= HIST_STRIDE;
        r = ensure_history(h);
        if (r) return r;
        const int slot = (int)(h->histTotal & HIST_MASK);
        launch_record_history(h->S, h->ctl, h->hist_t, slot, h->simTime, h->n_cap, h->st, h->lc);
        CKL();
        h->histTotal++;
    }
    if (h->n > 0) {                                                        // integrator.js:1798-1824
        CK(cudaMemsetAsync(&h->ctl->nRemoved, 0, sizeof(int), h->st));
        launch_boundary(h->P, h->S, h->ctl, h->keep, h->n_cap, h->st, h->lc);
        CKL();
        r = read_ctl(h);
        if (r) return r;
        const int removed = h->ctl_h->nRemoved;
        if (removed > 0) {
            r = compact(h);
            if (r) return r;
            h->n -= removed;
            set_n_kernel<<<1, 1, 0, h->st>>>(h->ctl, h->n);
            h->lc.add(1);
            CK(cudaStreamSynchronize(h->st));
        }
    }
    return GEON_OK;
}

int geon_synchronize(GeonHandle* h) {
    if (!h) return GEON_ERR_ARG;
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_stats(GeonHandle* h, GeonStats* out) {
    if (!h || !out) return GEON_ERR_ARG;
    launch_stats(h->P, h->S, h->ctl, h->stats_d, h->n_cap, h->st, h->lc);
    CKL();
    CK(cudaMemcpyAsync(h->stats_h, h->stats_d, 10 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const double* s = h->stats_h;
    out->linear_ke = s[0]; out->spin_ke = s[1]; out->px = s[2]; out->py = s[3];
    out->total_mass = s[4];
    out->com_x = s[4] > 0 ? s[5] / s[4] : 0; out->com_y = s[4] > 0 ? s[6] / s[4] : 0;
    out->pe = s[7] * 0.5;
    out->orbital_ang_mom = s[8]; out->spin_ang_mom = s[9];
    out->sim_time = h->simTime;
    out->alive_count = h->n;
    out->last_substeps = h->lastSubsteps;
    return GEON_OK;
}

int geon_upload_history(GeonHandle* h, int32_t n, int32_t count, const double* times, const float* samples) {
    if (!h || n != h->n || count < 0 || count > HIST_LEN || (count > 0 && (!times || !samples)))
        return set_err(h, GEON_ERR_ARG, "history upload: n must equal the particle count and count <= 256");
    if (!h->P.rel) return set_err(h, GEON_ERR_ARG, "history needs the relativity toggle");
    int r = ensure_history(h);
    if (r) return r;
    std::vector<double> t(HIST_LEN, 0.0);
    for (int k = 0; k < count; k++) t[k] = times[k];
    CK(cudaMemcpyAsync(h->hist_t, t.data(), HIST_LEN * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemsetAsync(h->S.hist_cnt, 0, h->n_cap * sizeof(int), h->st));
    if (count > 0 && n > 0) {
        const size_t elems = (size_t)5 * n * count;
        float* d = nullptr;
        CK(cudaMalloc(&d, elems * sizeof(float)));
        cudaError_t e = cudaMemcpyAsync(d, samples, elems * sizeof(float), cudaMemcpyHostToDevice, h->st);
        if (e == cudaSuccess) {
            history_upload_kernel<<<grid_for(n * count, 256), 256, 0, h->st>>>(h->S, n, count, d);
            e = cudaGetLastError();
            h->lc.add(1);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        cudaFree(d);
        if (e != cudaSuccess) return cuda_check(h, e, "history upload");
    }
    h->histTotal = count;
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

int geon_set_sim_time(GeonHandle* h, double sim_time) {
    if (!h) return GEON_ERR_ARG;
    h->simTime = sim_time;
    return GEON_OK;
}

int geon_get_sim_time(GeonHandle* h, double* sim_time) {
    if (!h || !sim_time) return GEON_ERR_ARG;
    *sim_time = h->simTime;
    return GEON_OK;
}

int geon_profile(GeonHandle* h, int32_t enable, GeonProfile* out) {
    if (!h) return GEON_ERR_ARG;
    prof_collect(h);
    if (out) *out = h->prof_acc;
    if (enable) { h->prof_acc = GeonProfile{}; h->prof = true; }
    else h->prof = false;
    return GEON_OK;
}

int geon_fp32_peak(GeonHandle* h, double* tflops) {
    if (!h || !tflops) return GEON_ERR_ARG;
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int threads = 256, blocks = sms * 8, iters = 2048;
    float* dummy = h->hist_age;
    cudaEvent_t a = get_event(h), b = get_event(h);
    fma_peak_kernel<<<blocks, threads, 0, h->st>>>(dummy, 64, 0.999999f, 1e-7f);   // warm-up
    double best = 0.0;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(a, h->st);
        fma_peak_kernel<<<blocks, threads, 0, h->st>>>(dummy, iters, 0.999999f, 1e-7f);
        cudaEventRecord(b, h->st);
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
        best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    h->ev_pool.push_back(a);
    h->ev_pool.push_back(b);
    h->lc.add(4);
    *tflops = best;
    return GEON_OK;
}

int geon_get_stream(GeonHandle* h, void** stream) {
    if (!h || !stream) return GEON_ERR_ARG;
    *stream = (void*)h->st;
    return GEON_OK;
}

int geon_launch_count(GeonHandle* h, int64_t* count) {
    if (!h || !count) return GEON_ERR_ARG;
    *count = h->lc.n;
    return GEON_OK;
}

}  // extern "C"

// =============================================================================================
// geon_direct_forces_noalloc: the pairwise subset sum of geon_direct_forces
// without any device allocation.
//
// geon_direct_forces allocates its index and output buffers with cudaMalloc
// and releases them with cudaFree on every call.  Some callers cannot do that:
// a host loop that samples the force error every frame while other streams
// of the device are busy (cudaFree waits for the whole device and would stall
// them), and embeddings that fix their device-memory footprint at start-up
// and must not meet an allocation failure in the middle of a run.  This
// variant stages the indices and the two output rows in one fixed array in
// device global memory, which the device holds from the time the library's
// device code is first loaded on it (its first upload or call) until the
// process exits, and allocates nothing.
//
// Limits and rules:
//   * at most GEON_DIRECT_NOALLOC_MAX_K targets per call (4.2 MiB of scratch:
//     k indices, then k x forces, then k y forces, each row sized for the
//     maximum, then the partial sums of up to 16 source slices, split as in
//     geon_direct_forces so that both give identical bits); larger k is
//     rejected with GEON_ERR_ARG;
//   * the first call on a device does the setup (it looks up the array's
//     device address with that device current and caches it per device), so
//     make that first call before any stream capture begins; a device reset
//     (cudaDeviceReset) while the library is loaded is not supported, as the
//     cached address would then be stale;
//   * the call makes the handle's device current for its duration and
//     restores the caller's device before it returns;
//   * nothing in the scratch has to start at zero: each call copies its k
//     indices in before the kernel reads them, and the kernel writes all k
//     outputs before they are copied out;
//   * the array is one per device, shared by every handle on it: calls that
//     overlap in time on the same device (from different host threads or
//     handles) race on it and must be serialised by the caller.  Calls made
//     one after another are safe, because each call waits for its stream
//     before it returns.
#include <mutex>

static constexpr int NOALLOC_MAX_K = GEON_DIRECT_NOALLOC_MAX_K;
static constexpr int NOALLOC_MAX_DEVICES = 64;
static constexpr size_t NOALLOC_PART_FLOATS = (size_t)16 * 4 * NOALLOC_MAX_K;   // slices x (fx, fy as hi, lo) x k
static_assert(NOALLOC_MAX_K % 256 == 0, "slice rows are whole CTAs of targets");
static __device__ __align__(256) unsigned char g_direct_scratch[(3 * NOALLOC_MAX_K + NOALLOC_PART_FLOATS) * sizeof(float)];
static void* g_direct_scratch_addr[NOALLOC_MAX_DEVICES] = {};
static std::mutex g_direct_scratch_mu;

// Device address of the scratch array on the device of h's stream.
static int direct_scratch(GeonHandle* h, void** out) {
    int dev = -1;
    cudaError_t e = cudaStreamGetDevice(h->st, &dev);
    if (e != cudaSuccess) return cuda_check(h, e, "cudaStreamGetDevice");
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return set_err(h, GEON_ERR_UNSUPPORTED, "device index beyond the scratch table");
    std::lock_guard<std::mutex> lock(g_direct_scratch_mu);
    if (!g_direct_scratch_addr[dev]) {
        int cur = -1;
        e = cudaGetDevice(&cur);
        if (e == cudaSuccess && cur != dev) e = cudaSetDevice(dev);
        void* p = nullptr;
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_direct_scratch);
        if (cur >= 0 && cur != dev) cudaSetDevice(cur);
        if (e != cudaSuccess) return cuda_check(h, e, "cudaGetSymbolAddress(direct-forces scratch)");
        if (!p) return set_err(h, GEON_ERR_CUDA, "direct-forces scratch has no device address");
        g_direct_scratch_addr[dev] = p;
    }
    *out = g_direct_scratch_addr[dev];
    return GEON_OK;
}

extern "C" int geon_direct_forces_noalloc(GeonHandle* h, const int32_t* idx, int32_t k, float* fx, float* fy) {
    if (!h || k < 0 || (k > 0 && (!idx || !fx || !fy))) return GEON_ERR_ARG;
    if (h->batch) return set_err(h, GEON_ERR_UNSUPPORTED, "the pairwise subset sum would mix the systems of a batched handle");
    if (k > NOALLOC_MAX_K)
        return set_err(h, GEON_ERR_ARG, "geon_direct_forces_noalloc: k = " + std::to_string(k) +
                       " exceeds GEON_DIRECT_NOALLOC_MAX_K = " + std::to_string(NOALLOC_MAX_K) +
                       " (use geon_direct_forces for larger subsets)");
    if (k == 0 || h->n == 0) return GEON_OK;
    for (int i = 0; i < k; i++)
        if (idx[i] < 0 || idx[i] >= h->n) return set_err(h, GEON_ERR_ARG, "index out of range");
    // the handle's device current for the whole call (the plan queries it)
    int dev = -1, cur = -1;
    cudaError_t de = cudaStreamGetDevice(h->st, &dev);
    if (de == cudaSuccess) de = cudaGetDevice(&cur);
    if (de == cudaSuccess && cur != dev) de = cudaSetDevice(dev);
    if (de != cudaSuccess) return cuda_check(h, de, "device of the handle");
    struct Restore { int d; ~Restore() { if (d >= 0) cudaSetDevice(d); } } restore{ cur != dev ? cur : -1 };
    void* base = nullptr;
    int r = direct_scratch(h, &base);
    if (r) return r;
    int* d_idx = static_cast<int*>(base);
    float* d_fx = reinterpret_cast<float*>(d_idx + NOALLOC_MAX_K);
    float* d_fy = d_fx + NOALLOC_MAX_K;
    ForceCtx C = make_ctx(h);
    const DirectPlan pl = direct_subset_plan(h->P, k);
    if (pl.slices > 1 && pl.floats <= NOALLOC_PART_FLOATS) {
        C.dpart = d_fy + NOALLOC_MAX_K;
        C.dslices = pl.slices;
    }
    cudaError_t e = cudaMemcpyAsync(d_idx, idx, k * sizeof(int), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess && h->P.rel) { launch_hist_tables(h->hist_t, h->simTime, h->hist_age, h->hist_segdt, h->st, h->lc); e = cudaGetLastError(); }
    if (e == cudaSuccess) {
        direct_subset(h->P, h->S, h->ctl, C, d_idx, k, d_fx, d_fy, h->st, h->lc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(fx, d_fx, k * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fy, d_fy, k * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    // wait for the stream on every path once work may be queued on the shared
    // array, so that the next call (from any handle) finds it free; report the
    // first error
    const cudaError_t ws = cudaStreamSynchronize(h->st);
    if (e == cudaSuccess) e = ws;
    return cuda_check(h, e, "direct forces (no allocation)");
}

// =============================================================================================
// Batched systems: many independent systems with one parameter set in one
// handle.  Particles are stored system by system; tree keys carry the system
// id above a 27-level Morton code, so one sort, one node emission and one
// walk serve every system, and no node mixes systems.  Each system keeps its
// own adaptive substep schedule (the planner runs on the device); the frame
// is captured once as a CUDA graph whose substep loop is a WHILE conditional
// node, so a frame costs one graph launch and one read of the per-system
// substep counts.
static int validate_batch_params(GeonHandle* h, const GeonParams& p) {
    if (!(p.toggles & GEON_BARNES_HUT))
        return set_err(h, GEON_ERR_UNSUPPORTED, "batched systems need Barnes-Hut (a pairwise sum would mix systems)");
    if (p.toggles & (GEON_RELATIVITY | GEON_ONE_PN))
        return set_err(h, GEON_ERR_UNSUPPORTED, "batched systems run without relativity and 1PN (one history ring per handle)");
    if (p.boundary_mode == GEON_BOUND_DESPAWN)
        return set_err(h, GEON_ERR_UNSUPPORTED, "batched systems need the loop or bounce boundary (despawning would reorder systems)");
    if (p.flags & GEON_FLAG_LEARN)
        return set_err(h, GEON_ERR_UNSUPPORTED, "batched systems run without the learned correction");
    if (p.collision_mode != GEON_COL_PASS)
        return set_err(h, GEON_ERR_UNSUPPORTED, "batched systems run without merge collisions (spawns would reorder systems)");
    if (p.flags & GEON_FLAG_BOSONS)
        return set_err(h, GEON_ERR_UNSUPPORTED, "batched systems run without a boson pool");
    return GEON_OK;
}

static void batch_drop_graph(Batch& B) {
    if (B.exec) { cudaGraphExecDestroy(B.exec); B.exec = nullptr; }
    if (B.graph) { cudaGraphDestroy(B.graph); B.graph = nullptr; }
}

static ForceCtx batch_ctx(GeonHandle* h, bool all) {
    ForceCtx C = make_ctx(h);
    Batch& B = *h->batch;
    C.tgt_list = B.dev.tgt_pad;
    C.tgt_count = B.slots;
    C.roots = B.roots;
    C.sys_dt = all ? nullptr : B.dev.sys_dt;
    C.sys_accel = B.dev.sys_accel;
    C.sys_cyc = B.dev.sys_cyc;
    C.walk_split = B.walk_split;
    C.split_level = B.split_level;
    C.walk_ctas = B.walk_ctas;
    C.walk_chunk = B.walk_chunk;
    C.walk_queue = B.walk_queue;
    return C;
}

static PushFlags batch_push_flags(const GeonParams& p) {
    const uint32_t tg = p.toggles;
    const bool hasMag = tg & GEON_MAGNETIC, hasGM = tg & GEON_GRAVITOMAG, hasGrav = tg & GEON_GRAVITY;
    PushFlags F{};
    F.has1PN = 0;
    F.needBoris = hasMag || hasGM || p.ext_bz != 0;
    F.needSpinOrbit = (tg & GEON_SPIN_ORBIT) && (hasMag || hasGM);
    F.needTorques = hasGrav;
    return F;
}

// Tree, walk order and force pass: every system (all) or those stepping now.
static int batch_forces(GeonHandle* h, bool all) {
    int r = build_tree(h);
    if (r) return r;
    batch_targets(h->S, h->T, h->ctl, h->batch->dev, h->n, h->st, h->lc);
    CKL();
    const int ps = prof_begin(h, PH_FORCE);
    force_pass(h->P, h->S, h->T, h->d_root, h->ctl, batch_ctx(h, all), true, h->n_cap, h->st, h->lc);
    prof_end(h, ps);
    CKL();
    return GEON_OK;
}

// One substep of the systems the planner gave a substep (integrator.js:884-1348).
static int batch_substep(GeonHandle* h) {
    const int ps = prof_begin(h, PH_PUSH);
    launch_push(h->P, h->S, h->ctl, 0.f, batch_push_flags(h->prm), h->n_cap, h->st, h->lc, h->batch->dev.sys_dt);
    prof_end(h, ps);
    CKL();
    return batch_forces(h, false);
}

// Captures the frame: frame start + first planning step, then WHILE(some
// system continues) { substep; planning step }, then the boundary.
static int batch_build_graph(GeonHandle* h) {
    Batch& B = *h->batch;
    batch_drop_graph(B);
    const GeonParams& p = h->prm;
    const bool prof = h->prof;
    h->prof = false;                       // no event nodes inside the graph
    const long long lc0 = h->lc.n;
    long long lc1 = lc0, lc2 = lc0, lc3 = lc0;
    int r = GEON_OK;
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle cond = 0;
    std::vector<cudaGraphNode_t> deps;
    cudaGraphNode_t cnode = nullptr;
    cudaGraph_t body = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(h->st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        batch_frame_start(h->P, h->S, B.dev, h->n, h->st, h->lc);
        batch_plan(h->P, B.dev, p.softening, p.max_substeps, (unsigned long long)cond, h->st, h->lc);
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* d = nullptr;
        size_t nd = 0;
        cudaError_t e2 = cudaStreamGetCaptureInfo(h->st, &cs, nullptr, nullptr, &d, nullptr, &nd);
        if (e2 == cudaSuccess && d) deps.assign(d, d + nd);
        cudaGraph_t out = nullptr;
        e = cudaStreamEndCapture(h->st, &out);
        if (e == cudaSuccess) e = e2;
    }
    lc1 = h->lc.n;
    if (e == cudaSuccess) {
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = cond;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        e = cudaGraphAddNode(&cnode, g, deps.data(), nullptr, deps.size(), &cp);
        if (e == cudaSuccess) body = cp.conditional.phGraph_out[0];
    }
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(h->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        r = batch_substep(h);
        batch_plan(h->P, B.dev, p.softening, p.max_substeps, (unsigned long long)cond, h->st, h->lc);
        cudaGraph_t out = nullptr;
        e = cudaStreamEndCapture(h->st, &out);
    }
    lc2 = h->lc.n;
    if (e == cudaSuccess && r == GEON_OK) e = cudaStreamBeginCaptureToGraph(h->st, g, &cnode, nullptr, 1, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess && r == GEON_OK) {
        launch_boundary(h->P, h->S, h->ctl, h->keep, h->n_cap, h->st, h->lc);
        cudaGraph_t out = nullptr;
        e = cudaStreamEndCapture(h->st, &out);
    }
    lc3 = h->lc.n;
    h->prof = prof;
    h->lc.n = lc0;                          // captured kernels are counted when the graph runs
    if (e == cudaSuccess && r == GEON_OK) e = cudaGraphInstantiate(&B.exec, g, 0);
    if (e != cudaSuccess || r != GEON_OK) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        B.exec = nullptr;
        if (r) return r;
        return set_err(h, GEON_ERR_CUDA, std::string("frame graph capture failed: ") + cudaGetErrorString(e));
    }
    B.graph = g;
    B.graph_head = lc1 - lc0;
    B.graph_body = lc2 - lc1;
    B.graph_tail = lc3 - lc2;
    B.graph_flags = h->P.flags;
    return GEON_OK;
}

static int batch_update(GeonHandle* h, double dt, int32_t* substeps) {
    if (!(dt >= 0)) return set_err(h, GEON_ERR_ARG, "dt must be >= 0");
    Batch& B = *h->batch;
    const GeonParams& p = h->prm;
    if (substeps) *substeps = 0;
    if (h->n == 0) return GEON_OK;
    int r;
    if (!h->forcesInit) {                                                  // integrator.js:750-782
        bootstrap_angvel_kernel<<<grid_for(h->n, 256), 256, 0, h->st>>>(h->P, h->S, h->ctl);
        CKL();
        h->lc.add(1);
        r = batch_forces(h, true);
        if (r) return r;
        h->forcesInit = true;
    }
    *B.dt_h = dt;
    CK(cudaMemcpyAsync(B.dev.frame_dt, B.dt_h, sizeof(double), cudaMemcpyHostToDevice, h->st));
    const bool graph = B.use_graph != 0;
    if (graph) {
        if (!B.exec || B.graph_flags != h->P.flags) {
            r = batch_build_graph(h);
            if (r) return r;
        }
        CK(cudaGraphLaunch(B.exec, h->st));
    } else {
        batch_frame_start(h->P, h->S, B.dev, h->n, h->st, h->lc);
        CKL();
        for (int it = 0; it <= p.max_substeps; it++) {
            batch_plan(h->P, B.dev, p.softening, p.max_substeps, 0ull, h->st, h->lc);
            CKL();
            CK(cudaMemcpyAsync(B.any_h, B.dev.any_active, sizeof(int), cudaMemcpyDeviceToHost, h->st));
            CK(cudaStreamSynchronize(h->st));
            if (!*B.any_h) break;
            r = batch_substep(h);
            if (r) return r;
        }
        launch_boundary(h->P, h->S, h->ctl, h->keep, h->n_cap, h->st, h->lc);
        CKL();
    }
    CK(cudaMemcpyAsync(B.plan_h, B.dev.plan, (size_t)B.dev.nsys * sizeof(SysPlan), cudaMemcpyDeviceToHost, h->st));
    r = read_ctl(h);                                                       // synchronises
    if (r) return r;
    int mx = 0;
    long long psub = 0;
    for (int s = 0; s < B.dev.nsys; s++) {
        mx = std::max(mx, B.plan_h[s].steps);
        psub += (long long)(B.off[s + 1] - B.off[s]) * B.plan_h[s].steps;
    }
    if (graph) h->lc.add((int)(B.graph_head + (long long)mx * B.graph_body + B.graph_tail));
    if (h->prof) h->prof_acc.particle_substeps += psub;
    B.last_max_steps = mx;
    h->lastSubsteps = mx;
    h->simTime += dt;
    if (substeps) *substeps = mx;
    return GEON_OK;
}

// State arrays a frame changes, saved to / restored from the scratch copy S2
// (the autotuner runs frames and then puts the state back).
static int batch_snapshot(GeonHandle* h, bool save) {
    const size_t n = (size_t)h->n_cap;
    const DevState& a = save ? h->S : h->S2;
    const DevState& b = save ? h->S2 : h->S;
    struct { void* dst; const void* src; size_t bytes; } cp[] = {
        { b.pos, a.pos, n * sizeof(float4) }, { b.pos_lo, a.pos_lo, n * sizeof(float2) },
        { b.vel, a.vel, n * sizeof(float4) }, { b.spin, a.spin, n * sizeof(float4) },
        { b.mom, a.mom, n * sizeof(float2) }, { b.force, a.force, n * sizeof(float4) },
        { b.grad, a.grad, n * sizeof(float4) }, { b.torque, a.torque, n * sizeof(float4) },
    };
    for (auto& c : cp) CK(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    return GEON_OK;
}

extern "C" {

int geon_create_batch(const GeonParams* params, int32_t n_systems, const int32_t* counts, GeonHandle** out) {
    if (!params || !counts || !out) return set_err(nullptr, GEON_ERR_ARG, "null argument");
    if (n_systems < 1 || n_systems > BATCH_MAX_SYSTEMS)
        return set_err(nullptr, GEON_ERR_ARG, "n_systems must be in [1, " + std::to_string(BATCH_MAX_SYSTEMS) + "]");
    long long total = 0;
    for (int s = 0; s < n_systems; s++) {
        if (counts[s] < 1) return set_err(nullptr, GEON_ERR_ARG, "every system needs at least one particle");
        total += counts[s];
    }
    if (total > (long long)REF_INDEX_MASK) return set_err(nullptr, GEON_ERR_ARG, "batch too large");
    GeonParams p = *params;
    if (p.max_substeps <= 0) p.max_substeps = 32;
    *out = nullptr;
    GeonHandle* h = nullptr;
    int r = geon_create(&p, (int32_t)total, &h);
    if (r) return r;
    r = validate_batch_params(h, h->prm);
    if (r) { g_err = h->err; geon_destroy(h); return r; }
    Batch* B = new Batch();
    h->batch = B;
    h->nsys = n_systems;
    B->off.assign(n_systems + 1, 0);
    B->pad.assign(n_systems, 0);
    int slots = 0;
    for (int s = 0; s < n_systems; s++) {
        B->off[s + 1] = B->off[s] + counts[s];
        B->pad[s] = slots;
        slots += (counts[s] + 31) / 32 * 32;
    }
    B->slots = slots;
    DevArena& A = B->A;
    B->sys = A.alloc<int>(total);
    B->roots = A.alloc<int>(n_systems);
    B->walk_queue = A.alloc<unsigned>(2);
    int* d_off = A.alloc<int>(n_systems + 1);
    int* d_pad = A.alloc<int>(n_systems);
    BatchDev& D = B->dev;
    D.nsys = n_systems;
    D.plan = A.alloc<SysPlan>(n_systems);
    D.sys_dt = A.alloc<double>(n_systems);
    D.sys_accel = A.alloc<unsigned long long>(n_systems);
    D.sys_cyc = A.alloc<unsigned long long>(n_systems);
    D.sys_off = d_off;
    D.pad_off = d_pad;
    D.tgt_pad = A.alloc<int>(slots);
    D.any_active = A.alloc<int>(1);
    D.frame_dt = A.alloc<double>(1);
    bool ok = !A.failed;
    ok = ok && cudaMallocHost(&B->any_h, sizeof(int)) == cudaSuccess;
    ok = ok && cudaMallocHost(&B->dt_h, sizeof(double)) == cudaSuccess;
    ok = ok && cudaMallocHost(&B->plan_h, (size_t)n_systems * sizeof(SysPlan)) == cudaSuccess;
    if (!ok) { g_err = "batch allocation failed"; geon_destroy(h); return GEON_ERR_NOMEM; }
    std::vector<int> sys(total);
    for (int s = 0; s < n_systems; s++)
        for (int i = B->off[s]; i < B->off[s + 1]; i++) sys[i] = s;
    cudaError_t e = cudaMemcpy(B->sys, sys.data(), total * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_off, B->off.data(), (n_systems + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_pad, B->pad.data(), n_systems * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(D.tgt_pad, 0xFF, (size_t)slots * sizeof(int));          // padding = -1
    if (e == cudaSuccess) e = cudaMemset(D.plan, 0, (size_t)n_systems * sizeof(SysPlan));
    if (e == cudaSuccess) e = cudaMemset(D.sys_dt, 0, (size_t)n_systems * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(B->roots, 0xFF, (size_t)n_systems * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(B->walk_queue, 0, 2 * sizeof(unsigned));
    if (e != cudaSuccess) { g_err = std::string("batch setup: ") + cudaGetErrorString(e); geon_destroy(h); return GEON_ERR_CUDA; }
    h->S.sys = B->sys;
    h->S2.sys = B->sys;
    h->T.roots = B->roots;
    derive_params(h);
    *out = h;
    return GEON_OK;
}

int geon_batch_substeps(GeonHandle* h, int32_t* steps, int32_t n_systems) {
    if (!h || !steps) return GEON_ERR_ARG;
    if (!h->batch) return set_err(h, GEON_ERR_ARG, "not a batched handle");
    if (n_systems < h->batch->dev.nsys) return set_err(h, GEON_ERR_ARG, "output array too small");
    for (int s = 0; s < h->batch->dev.nsys; s++) steps[s] = h->batch->plan_h[s].steps;
    return GEON_OK;
}

int geon_batch_set_mode(GeonHandle* h, int32_t use_graph, int32_t simple_walk) {
    if (!h) return GEON_ERR_ARG;
    if (!h->batch) return set_err(h, GEON_ERR_ARG, "not a batched handle");
    h->batch->use_graph = use_graph ? 1 : 0;
    if (simple_walk) h->prm.flags |= GEON_FLAG_SIMPLE_WALK;
    else h->prm.flags &= ~GEON_FLAG_SIMPLE_WALK;
    derive_params(h);
    batch_drop_graph(*h->batch);
    return GEON_OK;
}

int geon_batch_set_shape(GeonHandle* h, int32_t warps_per_group, int32_t split_level, int32_t ctas_per_sm,
                         int32_t queue_chunk) {
    if (!h) return GEON_ERR_ARG;
    if (!h->batch) return set_err(h, GEON_ERR_ARG, "not a batched handle");
    if ((warps_per_group != 1 && warps_per_group != 4) || split_level < 0 || split_level > KEY_LEVELS ||
        ctas_per_sm < 0 || ctas_per_sm > 32 || queue_chunk < 0 || queue_chunk > 4096)
        return set_err(h, GEON_ERR_ARG, "walk shape: warps_per_group 1 or 4, split_level 0..31, ctas_per_sm 0..32, "
                                        "queue_chunk 0..4096");
    Batch& B = *h->batch;
    B.walk_split = warps_per_group == 4 ? 1 : 0;
    B.split_level = split_level;
    B.walk_ctas = ctas_per_sm;
    B.walk_chunk = queue_chunk;
    if (queue_chunk > 0) {
        walk_queue_setup();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_check(h, e, "work-queue walk setup");
    }
    batch_drop_graph(B);
    return GEON_OK;
}

// The autotuner's candidates: use_graph, simple_walk, warps per group, split
// level, walk CTAs per SM, work-queue chunk.  0-3 are the graph / launch and
// grouped / simple modes; 4-6 cap the grouped walk's resident CTAs; 7-9 split
// each group's walk over four warps at three depths; 10-11 run the grouped
// walk as persistent CTAs taking 1 or 4 walk blocks at a time; 12 runs it
// with the short stack at seven CTAs per SM.
static const int32_t TUNE_MODES[GEON_BATCH_TUNE_MODES][6] = {
    { 0, 0, 1, 6, 0, 0 }, { 1, 0, 1, 6, 0, 0 }, { 0, 1, 1, 6, 0, 0 }, { 1, 1, 1, 6, 0, 0 },
    { 1, 0, 1, 6, 5, 0 }, { 1, 0, 1, 6, 4, 0 }, { 1, 0, 1, 6, 3, 0 },
    { 1, 0, 4, 4, 0, 0 }, { 1, 0, 4, 6, 0, 0 }, { 1, 0, 4, 8, 0, 0 },
    { 1, 0, 1, 6, 0, 1 }, { 1, 0, 1, 6, 0, 4 },
    { 1, 0, 1, 6, 7, 0 },
};

int geon_batch_tune_mode(int32_t mode, int32_t* desc) {
    if (mode < 0 || mode >= GEON_BATCH_TUNE_MODES || !desc) return GEON_ERR_ARG;
    for (int k = 0; k < 6; k++) desc[k] = TUNE_MODES[mode][k];
    return GEON_OK;
}

static int batch_apply_mode(GeonHandle* h, int c) {
    const int32_t* m = TUNE_MODES[c];
    int r = geon_batch_set_mode(h, m[0], m[1]);
    if (!r) r = geon_batch_set_shape(h, m[2], m[3], m[4], m[5]);
    return r;
}

int geon_batch_autotune(GeonHandle* h, double dt, int32_t frames, int32_t* choice, double* ms_per_frame) {
    if (!h || frames < 1 || !(dt >= 0)) return GEON_ERR_ARG;
    if (!h->batch) return set_err(h, GEON_ERR_ARG, "not a batched handle");
    if (h->n == 0) return set_err(h, GEON_ERR_ARG, "empty batch");
    Batch& B = *h->batch;
    int r = batch_snapshot(h, true);
    if (r) return r;
    const double t0 = h->simTime;
    const bool init0 = h->forcesInit;
    cudaEvent_t a = get_event(h), b = get_event(h);
    double best = 1e300;
    int bestc = 0;
    for (int c = 0; c < GEON_BATCH_TUNE_MODES; c++) {
        r = batch_apply_mode(h, c);
        if (r) break;
        r = batch_snapshot(h, false);
        if (r) break;
        h->simTime = t0;
        h->forcesInit = init0;
        r = batch_update(h, dt, nullptr);                 // warm-up (captures the graph)
        if (r) break;
        CK(cudaEventRecord(a, h->st));
        for (int f = 0; f < frames && !r; f++) r = batch_update(h, dt, nullptr);
        if (r) break;
        CK(cudaEventRecord(b, h->st));
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double per = ms / frames;
        if (ms_per_frame) ms_per_frame[c] = per;
        if (per < best) { best = per; bestc = c; }
    }
    h->ev_pool.push_back(a);
    h->ev_pool.push_back(b);
    const int r2 = batch_apply_mode(h, bestc);
    const int r3 = batch_snapshot(h, false);
    h->simTime = t0;
    h->forcesInit = init0;
    if (choice) *choice = bestc;
    (void)B;
    return r ? r : (r2 ? r2 : r3);
}

}  // extern "C"
