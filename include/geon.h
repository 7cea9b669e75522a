/*
 * geon.h — C ABI of the GB300 force-and-push library (libgeon_cuda.so).
 *
 * One handle owns one particle system resident in GPU memory: FP32 SoA
 * particle state, the signal-delay history ring, the quadtree built from
 * radix-sorted Morton keys, and the per-particle force/field accumulators.
 * Every entry point returns an int status (GEON_OK == 0, negative on error);
 * geon_last_error() returns a message for the last failure on that handle.
 *
 * Ownership: the library owns all device memory.  Host arrays passed in are
 * caller-owned and copied; host arrays passed out are caller-allocated.
 * Threading: one handle per host thread.  All work of a handle is ordered on
 * the handle's own CUDA stream (geon_get_stream); calls return when the
 * requested results are on the host.
 *
 * The reference (a9lim/physsim, "Geon") has no native interface; each entry
 * point below names the JavaScript method whose contract it carries.  The
 * JS side binds these entry points through a thin N-API addon.
 */
#ifndef GEON_H
#define GEON_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GEON_OK              0
#define GEON_ERR_ARG        -1   /* bad argument (null, out of range)          */
#define GEON_ERR_FULL       -2   /* capacity exhausted (src/gpu/gpu-physics.js:1864 returns -1) */
#define GEON_ERR_CUDA       -3   /* CUDA runtime error                           */
#define GEON_ERR_OVERFLOW   -4   /* device-side overflow flag (walk stack, node pool) */
#define GEON_ERR_TIMEOUT    -5   /* bounded device wait gave up                  */
#define GEON_ERR_NOMEM      -6   /* device allocation failed                     */
#define GEON_ERR_UNSUPPORTED -7  /* toggle combination outside this library     */

/* ---- toggle bits: same layout as the reference's toggles0 word
 *      (src/gpu/gpu-constants.js:265-280, packed by gpu-physics.js:1969-1985) */
#define GEON_GRAVITY      (1u << 0)
#define GEON_COULOMB      (1u << 1)
#define GEON_MAGNETIC     (1u << 2)
#define GEON_GRAVITOMAG   (1u << 3)
#define GEON_ONE_PN       (1u << 4)
#define GEON_RELATIVITY   (1u << 5)
#define GEON_SPIN_ORBIT   (1u << 6)
#define GEON_RADIATION    (1u << 7)   /* unsupported: radiation is off the path */
#define GEON_BLACK_HOLE   (1u << 8)   /* unsupported */
#define GEON_YUKAWA       (1u << 11)
#define GEON_HIGGS        (1u << 12)  /* unsupported: scalar fields off the path */
#define GEON_AXION        (1u << 13)  /* unsupported */
#define GEON_BARNES_HUT   (1u << 14)

/* boundary modes (src/config.js:16-18) and topologies (src/config.js:22-24) */
#define GEON_BOUND_DESPAWN 0
#define GEON_BOUND_BOUNCE  1
#define GEON_BOUND_LOOP    2
#define GEON_TORUS 0
#define GEON_KLEIN 1
#define GEON_RP2   2

/* option flags (GeonParams.flags) */
#define GEON_FLAG_PE          (1u << 0)  /* accumulate potential energy in force passes */
#define GEON_FLAG_BREAKDOWN   (1u << 1)  /* keep per-type force vectors (force breakdown) */
#define GEON_FLAG_NO_GHOSTS   (1u << 2)  /* periodic BH without image ghosts (min-image only) */
#define GEON_FLAG_SIMPLE_WALK (1u << 3)  /* one node per warp iteration (cross-check of the batched walk) */
#define GEON_FLAG_LEARN       (1u << 4)  /* cell moments + learned far-field correction (when weights are set) */
#define GEON_FLAG_BOSONS      (1u << 5)  /* Physics.bosonInterEnabled: boson gravity on particles in every force pass */
#define GEON_FLAG_SPLIT_FRAME (1u << 6)  /* geon_update launches every phase separately (cross-check of the one-launch frame) */

/* Physics parameters.  Mirrors the Physics fields that Physics.update reads
 * (src/integrator.js:65-107, :726-736) plus theta/softening, which the
 * reference hard-codes (src/config.js:44,57) and this library takes at run time. */
typedef struct GeonParams {
    uint32_t toggles;          /* GEON_* toggle bits                                  */
    uint32_t flags;            /* GEON_FLAG_* bits                                    */
    int32_t  boundary_mode;    /* GEON_BOUND_*                                        */
    int32_t  topology;         /* GEON_TORUS / GEON_KLEIN / GEON_RP2                  */
    double   domain_w;         /* width, height: Physics.update(width, height)        */
    double   domain_h;
    double   off_x;            /* offX, offY                                          */
    double   off_y;
    double   theta;            /* Barnes-Hut opening angle (BH_THETA = 0.5)           */
    double   softening;        /* SOFTENING (8): softeningSq = s^2, dtSafe = sqrt(s/a) */
    double   yukawa_mu;        /* Physics.yukawaMu (DEFAULT_PION_MASS = 0.15)         */
    double   bounce_friction;  /* Physics.bounceFriction (0.4)                        */
    double   ext_gravity;      /* Physics.extGravity / extGravityAngle               */
    double   ext_gravity_angle;
    double   ext_electric;     /* Physics.extElectric / extElectricAngle             */
    double   ext_electric_angle;
    double   ext_bz;           /* Physics.extBz                                       */
    int32_t  max_substeps;     /* MAX_SUBSTEPS (32)                                   */
    int32_t  collision_mode;   /* GEON_COL_*: the collisionMode argument of Physics.update */
} GeonParams;

/* collision modes (src/config.js:10-12).  GEON_COL_MERGE runs handleCollisions
 * (src/collisions.js:24-107) after the tree rebuild of every substep; the
 * bounce mode's contact forces are not part of this library. */
#define GEON_COL_PASS   0
#define GEON_COL_MERGE  1
#define GEON_COL_BOUNCE 2   /* unsupported */

/* Conserved quantities in FP64 (src/energy.js:11-62 passes 1-2, and the
 * potential energy of the last force pass, src/forces.js:26). */
typedef struct GeonStats {
    double linear_ke, spin_ke, pe;
    double px, py;
    double orbital_ang_mom, spin_ang_mom;
    double com_x, com_y, total_mass;
    double sim_time;
    int32_t alive_count;
    int32_t last_substeps;
} GeonStats;

/* Tree summary of the last build. */
typedef struct GeonTreeInfo {
    int32_t n_points;      /* tree points: particles + periodic ghosts            */
    int32_t n_ghosts;
    int32_t n_dropped;     /* points outside the closed root box (quadtree.js:186) */
    int32_t n_internal;    /* divided nodes                                        */
    int32_t n_leaves;      /* non-empty undivided nodes                            */
    int32_t max_level;     /* deepest leaf level                                   */
    int32_t n_bucket;      /* leaves at the depth cap holding > 4 points           */
    int32_t reserved;
} GeonTreeInfo;

/* Per-particle output rows of geon_download_forces (each row n floats). */
#define GEON_OUT_FX          0
#define GEON_OUT_FY          1
#define GEON_OUT_BZ          2
#define GEON_OUT_BGZ         3
#define GEON_OUT_DBZDX       4
#define GEON_OUT_DBZDY       5
#define GEON_OUT_DBGZDX      6
#define GEON_OUT_DBGZDY      7
#define GEON_OUT_TIDAL       8   /* _tidalTorque     */
#define GEON_OUT_FRAMEDRAG   9   /* _frameDragTorque */
#define GEON_OUT_F1PN_X     10
#define GEON_OUT_F1PN_Y     11
#define GEON_OUT_PE         12   /* per-particle PE sum (global PE = half the sum)  */
#define GEON_OUT_GRAV_X     13   /* per-type vectors (GEON_FLAG_BREAKDOWN)          */
#define GEON_OUT_GRAV_Y     14
#define GEON_OUT_COUL_X     15
#define GEON_OUT_COUL_Y     16
#define GEON_OUT_MAG_X      17
#define GEON_OUT_MAG_Y      18
#define GEON_OUT_GM_X       19
#define GEON_OUT_GM_Y       20
#define GEON_OUT_YUK_X      21
#define GEON_OUT_YUK_Y      22
#define GEON_OUT_EXT_X      23
#define GEON_OUT_EXT_Y      24
#define GEON_OUT_ROWS       25

/* Rows of the packed particle state (geon_upload_state / download_state). */
#define GEON_ST_X       0
#define GEON_ST_Y       1
#define GEON_ST_WX      2   /* proper velocity w = gamma v */
#define GEON_ST_WY      3
#define GEON_ST_MASS    4
#define GEON_ST_CHARGE  5
#define GEON_ST_ANGW    6   /* angular celerity */
#define GEON_ST_VX      7   /* coordinate velocity (download only; derived on upload) */
#define GEON_ST_VY      8
#define GEON_ST_ANGVEL  9   /* download only */
#define GEON_ST_ROWS_IN 7
#define GEON_ST_ROWS   10

typedef struct GeonHandle GeonHandle;

/* new GPUPhysics(device, domainW, domainH) + init()
 * (src/gpu/gpu-physics.js:155-160).  max_particles sizes every buffer once. */
int geon_create(const GeonParams* params, int32_t max_particles, GeonHandle** out);

/* GPUPhysics.destroy() (src/gpu/gpu-physics.js:4291). */
int geon_destroy(GeonHandle* h);

/* GPUPhysics.setToggles(physics) (src/gpu/gpu-physics.js:1969) together with
 * the domain/boundary fields main.js writes before update().  Takes effect at
 * the next call. */
int geon_set_params(GeonHandle* h, const GeonParams* params);
int geon_get_params(GeonHandle* h, GeonParams* out);

/* GPUPhysics.addParticle({x,y,vx,vy,mass,charge,angw}) (src/gpu/gpu-physics.js:1857),
 * batched.  `soa` holds GEON_ST_ROWS_IN rows of n floats (x, y, wx, wy, mass,
 * charge, angw) with the proper velocity already formed (the host layer turns
 * coordinate velocity into w as setVelocity does, src/relativity.js:15-25).
 * creation_time is the simTime stamp of the batch (Particle.creationTime).
 * Writes the first slot index; GEON_ERR_FULL when the batch does not fit. */
int geon_add_particles(GeonHandle* h, int32_t n, const float* soa,
                       double creation_time, int32_t* first_index);

/* GPUPhysics.removeParticle(idx) (src/gpu/gpu-physics.js:1936): the slot is
 * removed and later slots shift down by one, keeping the CPU path's array
 * order (integrator.js:1799-1824 compacts the same way). */
int geon_remove_particle(GeonHandle* h, int32_t index);

/* GPUPhysics.deserialize(state) (src/gpu/gpu-physics.js:3886): replaces the
 * whole state with n particles (soa as in geon_add_particles).  Resets forces,
 * moments and history; the next geon_update bootstraps forces. */
int geon_upload_state(GeonHandle* h, int32_t n, const float* soa, double sim_time);

/* GPUPhysics.serialize() (src/gpu/gpu-physics.js:3749): copies
 * min(n, capacity) particles out as `rows` (<= GEON_ST_ROWS) rows of
 * `capacity` floats each.  Writes the particle count. */
int geon_download_state(GeonHandle* h, float* soa, int32_t rows, int32_t capacity, int32_t* n);

/* Stable particle ids, in current slot order (ids are assigned by
 * geon_add_particles / geon_upload_state in order and travel with each
 * particle through compaction).  Lets a host keep GPUPhysics-style handles
 * (main.js stores p._gpuIdx) although slots shift on removal. */
int geon_download_ids(GeonHandle* h, int32_t* ids, int32_t capacity, int32_t* n);

/* Same as geon_download_state with FP64 rows; positions carry the low
 * parts of the compensated drift sums. */
int geon_download_state_f64(GeonHandle* h, double* soa, int32_t rows, int32_t capacity, int32_t* n);

/* GPUPhysics.reset() (src/gpu/gpu-physics.js:3973). */
int geon_reset(GeonHandle* h);

/* GPUPhysics.getParticleCount() (src/gpu/gpu-physics.js:4287). */
/* geon_upload_state from double precision (the reference's save files hold
 * doubles, save-load.js:94-98): positions are kept as compensated FP32
 * pairs (hi + lo), so a state written by geon_download_state_f64 comes back
 * exactly; the other rows are rounded to FP32.  `soa` holds GEON_ST_ROWS_IN
 * rows of n doubles. */
int geon_upload_state_f64(GeonHandle* h, int32_t n, const double* soa, double sim_time);

int geon_particle_count(GeonHandle* h, int32_t* n);

/* Physics.update(particles, dt, ...) (src/integrator.js:726-1825), the
 * in-scope part: force bootstrap on the first call, adaptive Boris substeps
 * (<= max_substeps) with tree rebuild and force recompute, 1PN velocity-Verlet,
 * history sampling every 64 calls, boundary handling.  `substeps` (may be
 * NULL) receives the number of substeps taken.
 *
 * A single system in an open box with at most 4,096 particles, Barnes-Hut on
 * and no dipole / 1PN terms, merge collisions, breakdown rows, energy sums,
 * learned correction or bosons runs the whole frame (planner, substeps, tree
 * builds, walks, history, boundary) as ONE kernel launch with a device-side
 * planner, then reads the results back once; GEON_FLAG_SPLIT_FRAME selects
 * the launch-per-phase path instead.  Same physics either way. */
int geon_update(GeonHandle* h, double dt, int32_t* substeps);

/* Waits of the one-launch frame: each grid-wide barrier gives up after
 * wait_ns nanoseconds (default 1e9); the frame then returns GEON_ERR_TIMEOUT
 * and the handle keeps the error.  extra_arrivals > 0 makes every barrier
 * wait for that many blocks that do not exist, so the wait runs out (a test
 * of the time-out path); 0 restores normal operation. */
int geon_set_frame_wait(GeonHandle* h, int64_t wait_ns, int32_t extra_arrivals);

/* Phase durations (microseconds, block 0's clock) of the last one-launch
 * frame: frame-start scan, then the first substep's push + keys, sort,
 * gather, scans, emit, link, aggregation and walk, then the rest of the
 * frame (later substeps, history, boundary).  Writes min(n, 10) values, 0
 * for phases the frame did not reach; returns 10. */
int geon_frame_phases(GeonHandle* h, double* us, int32_t n);

/* Waits for all work enqueued on the handle's stream. */
int geon_synchronize(GeonHandle* h);

/* One force pass at the current state without advancing it: resetForces +
 * tree build + computeAllForces (src/forces.js:31-154), i.e. the bootstrap of
 * Physics.update (src/integrator.js:750-758).  Uses Barnes-Hut when the
 * GEON_BARNES_HUT toggle is set, the O(N^2) pairwise sum otherwise. */
int geon_compute_forces(GeonHandle* h);

/* 1PN-only force pass (src/forces.js:578-610) at the current state; writes
 * the GEON_OUT_F1PN_* rows. */
int geon_compute_1pn(GeonHandle* h);

/* Pairwise forces on a subset of particles: the O(N^2) sum of
 * computeAllForces' pairwise branch (src/forces.js:94-125) for the k listed
 * particle indices, against all particles, written to fx[k], fy[k] (host
 * arrays).  The particle state and stored forces are not changed.  This is the
 * exact reference for measuring the Barnes-Hut force error on a subsample. */
int geon_direct_forces(GeonHandle* h, const int32_t* idx, int32_t k, float* fx, float* fy);

/* The same pairwise subset sum as geon_direct_forces, with no device
 * allocation (no reference counterpart: the reference's JS path has no
 * device memory to allocate).  For callers that must not call cudaMalloc /
 * cudaFree during a run: the indices and outputs are staged in a fixed
 * device array, one per device, which the device holds from the first load
 * of the library's device code on it (its first upload or call) until the
 * process exits, so
 *   - k is at most GEON_DIRECT_NOALLOC_MAX_K (larger k: GEON_ERR_ARG);
 *   - the first call on a device sets up the array's address; make it before
 *     any stream capture begins; a device reset while the library is loaded
 *     is not supported;
 *   - the call makes the handle's device current while it runs;
 *   - no part of the array needs to start at zero;
 *   - calls that overlap in time on one device race on the array: serialise
 *     them (consecutive calls are safe; each waits for its stream, on error
 *     paths too). */
#define GEON_DIRECT_NOALLOC_MAX_K 16384
int geon_direct_forces_noalloc(GeonHandle* h, const int32_t* idx, int32_t k, float* fx, float* fy);

/* ---- learned far-field correction (no reference counterpart) --------------
 * The reference's far field is the plain monopole of an accepted cell
 * (src/forces.js:680-685).  With GEON_FLAG_LEARN and weights set, a Barnes-Hut
 * force pass keeps that monopole for every target and adds, once per pair of
 * (accepted cell, group of 32 consecutive targets in walk order), a linear
 * expansion about the group's centre of
 *   - the cell's analytic second-order term (mass quadrupole through the
 *     softened gravity + Yukawa kernel, charge dipole through the Coulomb
 *     kernel), and
 *   - the network's residual of the mass-sourced field: 14 features of the
 *     cell seen from the group centre -> 64 -> 64 -> 6 (GELU; BF16 weights
 *     and activations, FP32 accumulation on the tensor cores), the value and
 *     gradient of the two field components in the frame of the cell's
 *     direction, scaled by M / re^2 and M / (re^2 s).
 * It applies to open boxes with gravity, Coulomb and Yukawa (no relativity,
 * dipoles or 1PN).  Weight vector (FP32, GEON_MLP_NPARAM floats, nn.Linear
 * layout W[out][in]):
 *     mu[14] isd[14] W1[64][14] b1[64] W2[64][64] b2[64] W3[6][64] b3[6]
 * where the features are first normalised in FP32, x' = (x - mu) * isd;
 * training (geon_mlp_grad / geon_mlp_train) leaves mu and isd unchanged. */
#define GEON_MLP_NPARAM 5538
#define GEON_LEARN_FEATURES 14
#define GEON_LEARN_OUTPUTS 6
#define GEON_LEARN_TARGETS 18   /* per training record: y*[6], then A[6] of each of the 2 components */

/* Training records.  Builds the tree with cell moments at the handle's
 * theta, runs the Barnes-Hut force pass recording the (cell, group) pairs,
 * and for the groups 0, stride, 2 stride, ... writes per record
 *   feat[14]      the network's inputs,
 *   target[18]    the least-squares outputs y*[6] that fit the exact residual
 *                 at the record's accepting targets (the cell's member sum,
 *                 src/forces.js:94-125 restricted to the cell, minus the
 *                 monopole and the analytic term), then for each of the two
 *                 components the quadratic form (A00 A11 A22 A01 A02 A12)
 *                 with which an output error adds to the sum over those
 *                 targets of the squared force error relative to |F|
 *                 (weights m^2 / max(|F|^2, (m gfloor)^2), |F| from this pass),
 *   rec_group     the group (may be NULL).
 * Arrays hold `cap` records; *count receives the records of the selected
 * groups (those beyond cap are dropped).  Forces are left as the plain pass
 * computed them. */
int geon_learn_dataset(GeonHandle* h, int32_t group_stride, int64_t cap, float gfloor, float* feat, float* target,
                       int32_t* rec_group, int64_t* count);

/* Test aid: the Barnes-Hut force pass at the handle's theta plus the
 * correction with the network outputs taken from y[n][6] instead of the
 * network, for the records of all groups in the order geon_learn_dataset
 * lists them with stride 1 (n must equal that count). */
int geon_learn_apply(GeonHandle* h, const float* y, int64_t n);

/* Sets the correction's weights (copied); NULL clears them.  The correction
 * runs in Barnes-Hut force passes while GEON_FLAG_LEARN is set and weights
 * are present.  n_param must be GEON_MLP_NPARAM. */
int geon_learn_set_weights(GeonHandle* h, const float* weights, int32_t n_param);

/* y[n][6] = net(x[n][14]) on the device (host arrays). */
int geon_mlp_forward(GeonHandle* h, const float* weights, const float* x, int32_t n, float* y);

/* Gradient of L = (1/n) sum_s wt_s sum_c (y_sc - y*_sc)^T A_sc (y_sc - y*_sc)
 * over all n samples, y_sc = outputs 3c..3c+2 of net(x_s), t_s[18] = y*_s[6]
 * then A_s0[6], A_s1[6] (A00 A11 A22 A01 A02 A12); wt may be NULL (all 1).
 * Computed by the tensor-core backward pass: grad[GEON_MLP_NPARAM], *loss = L. */
int geon_mlp_grad(GeonHandle* h, const float* weights, const float* x, const float* t, const float* wt, int32_t n,
                  float* grad, double* loss);

/* Trains the network in place with Adam (beta 0.9 / 0.999, eps 1e-8) on that
 * loss for `steps` steps of `batch` samples drawn uniformly (seeded counter
 * hash) from the n samples, with a cosine learning-rate schedule from lr to
 * 0.  loss_history[steps] (may be NULL) receives each step's batch loss. */
int geon_mlp_train(GeonHandle* h, float* weights, const float* x, const float* t, const float* wt, int32_t n,
                   int32_t steps, int32_t batch, float lr, uint64_t seed, double* loss_history);

/* ---- batched systems -----------------------------------------------------
 * One handle holding n_systems independent systems (up to 512) with the same
 * parameters and their own particle counts, stepped together: geon_update
 * advances every system by one frame, each with its own adaptive substeps
 * (src/integrator.js:810-875).  The reference runs one system per Physics
 * object; this is its per-system loop folded into one launch sequence.
 * Particles are given system by system (counts[0] particles of system 0,
 * then system 1, ...) through geon_upload_state with the total count.
 * Supported: Barnes-Hut, loop or bounce boundary, no relativity / 1PN,
 * no learned correction; geon_add_particles (other than the whole batch),
 * geon_remove_particle, geon_direct_forces and geon_compute_1pn return
 * GEON_ERR_UNSUPPORTED.  Trees use 27 Morton levels below the system id. */
#define GEON_BATCH_MAX_SYSTEMS 512
int geon_create_batch(const GeonParams* params, int32_t n_systems, const int32_t* counts, GeonHandle** out);

/* Substeps each system took in the last frame (n_systems entries). */
int geon_batch_substeps(GeonHandle* h, int32_t* steps, int32_t n_systems);

/* Frame execution mode: use_graph = 1 runs each frame as one CUDA graph
 * launch (the substep loop is a device-side WHILE node; default), 0 as
 * individual launches with one host read per substep; simple_walk selects
 * the one-node-per-step walk instead of the grouped walk. */
int geon_batch_set_mode(GeonHandle* h, int32_t use_graph, int32_t simple_walk);

/* Shape of the grouped walk: warps_per_group 1 (one warp walks a group of
 * 32 targets; default) or 4 (the four warps of a CTA share one group's
 * subtrees below split_level; plain forces in the lean form, otherwise the
 * one-warp walk runs); ctas_per_sm > 0 caps the resident walk CTAs per SM by
 * padding their shared memory (0: as many as fit; 7: the plain torus walk
 * with a 288-entry stack, which fits seven); queue_chunk > 0 runs the
 * one-warp walk of plain forces on the torus as persistent CTAs taking
 * queue_chunk walk blocks at a time from a counter (0: one CTA per block). */
int geon_batch_set_shape(GeonHandle* h, int32_t warps_per_group, int32_t split_level, int32_t ctas_per_sm,
                         int32_t queue_chunk);

/* Times `frames` frames of dt in each of the GEON_BATCH_TUNE_MODES candidate
 * modes (geon_batch_tune_mode), restores the state, and keeps the fastest;
 * `choice` receives its index, ms_per_frame[GEON_BATCH_TUNE_MODES] (may be
 * NULL) the time of each. */
#define GEON_BATCH_TUNE_MODES 13
int geon_batch_autotune(GeonHandle* h, double dt, int32_t frames, int32_t* choice, double* ms_per_frame);

/* Candidate `mode` of geon_batch_autotune as desc[6] = { use_graph,
 * simple_walk, warps_per_group, split_level, ctas_per_sm, queue_chunk }. */
int geon_batch_tune_mode(int32_t mode, int32_t* desc);

/* Potential heat map (Heatmap.update, src/heatmap.js:133-206, with the
 * tree walk treePotential of :38-101 and the box blur _blur of :278-302):
 * gravitational, electric and Yukawa potential at the centres of a grid x
 * grid lattice of cells of cell_w x cell_h whose corner is (left, top)
 * (the reference derives them from the camera, heatmap.js:136-142).  With
 * Barnes-Hut on the tree is rebuilt at the current state and walked;
 * otherwise the pairwise sum runs.  fields: bit 0 gravity, 1 electric,
 * 2 Yukawa (each only when its force is on); blur != 0 smooths each computed
 * field.  Outputs are host arrays of grid*grid floats, row-major (y, x); a
 * field not computed is zero.  The colour mapping and canvas are UI and
 * not part of the path; dead particles (not held by this path) are not
 * included. */
#define GEON_HEAT_GRAVITY  1u
#define GEON_HEAT_ELECTRIC 2u
#define GEON_HEAT_YUKAWA   4u
int geon_heatmap(GeonHandle* h, double left, double top, double cell_w, double cell_h, int32_t grid, uint32_t fields,
                 int32_t blur, float* grav, float* elec, float* yuk);

/* ---- merge collisions (GeonParams.collision_mode = GEON_COL_MERGE) ------
 * handleCollisions (src/collisions.js:24-158) runs after every substep's
 * tree rebuild, as Physics.update does (src/integrator.js:1350-1381):
 * overlapping particles merge (mass, proper momentum and charge add, orbital
 * plus spin angular momentum becomes spin) or, for matter against
 * antimatter, annihilate the smaller mass.  Merged particles are appended
 * after the survivors with new ids and creation time now, as
 * Simulation.addParticle makes them (main.js:504-523).  The annihilation
 * photons and field excitations the reference emits from these events are
 * not part of this library; the events are returned instead. */

/* Antimatter flags (0 / 1) and base masses (Particle.antimatter, .baseMass,
 * src/particle.js:48-50) of particles [first, first + count); either array
 * may be NULL to leave that field.  Particles start as matter with
 * base mass = mass (GPUPhysics.addParticle's antimatter field,
 * src/gpu/gpu-physics.js:1857-1870). */
int geon_set_matter(GeonHandle* h, int32_t first, int32_t count, const int32_t* antimatter, const float* base_mass);
int geon_get_matter(GeonHandle* h, int32_t* antimatter, float* base_mass, int32_t capacity, int32_t* n);

/* ---- boson pool (src/forces.js:697-901) ---------------------------------
 * The photons, pions and leptons of the Simulation, as the boson tree reads
 * them: n rows of 6 doubles (x, y, _srcMass, _srcCharge, kind, v^2), kind 0
 * for photons and 1 for pions and leptons (only alive ones).  The pool's
 * quadtree is built at once (Physics._buildBosonTree, integrator.js:263-277)
 * and kept until the next call; n = 0 clears the pool.  With the
 * GEON_FLAG_BOSONS flag and gravity on, every force pass of geon_update adds
 * computeBosonGravity (forces.js:788-804) for this pool, which stays where it
 * was uploaded for the whole frame (the reference moves bosons every
 * substep).  No reference counterpart as an entry point: the reference keeps
 * the pool in its Simulation object. */
int geon_set_bosons(GeonHandle* h, int32_t n, const double* rows);

/* The kicks the pool's bosons get from one another: what & 1 gravity
 * (applyBosonBosonGravity, forces.js:812-856: 2 dt for photons, (1 + v^2) dt
 * for pions and leptons, before the photons' speed renormalisation), what & 2
 * Coulomb between charged pions and leptons (applyPionPionCoulomb,
 * forces.js:878-901: -q dt).  kicks[2n] receives (dx, dy) per boson in
 * upload order: photons add it to their velocity, pions and leptons to w. */
int geon_boson_kicks(GeonHandle* h, double dt, uint32_t what, float* kicks);

/* Collision counts of the last geon_update. */
typedef struct GeonCollisionInfo {
    int32_t merges;          /* merged pairs (each appends one particle)                 */
    int32_t annihilations;   /* matter-antimatter contacts                               */
    int32_t spawned;         /* particles appended                                       */
    int32_t removed;         /* particles whose mass reached zero                        */
    int32_t candidates;      /* overlap candidates examined                              */
    int32_t events;          /* events stored for geon_collision_events (<= 65536)       */
    int32_t events_dropped;  /* events beyond that                                       */
    int32_t order_approx;    /* 1 if a leaf at the 31-level depth cap held > 4 points:
                                its candidates were taken in insertion-index order       */
} GeonCollisionInfo;
int geon_collision_info(GeonHandle* h, GeonCollisionInfo* out);

/* The last geon_update's events, the arrays handleCollisions returns
 * (collisions.js:9-14): rows of 6 doubles (type, x, y, energy, px, py),
 * type 1 = annihilation (energy 2 m + kinetic, the photon burst of
 * integrator.js:1387-1393) and 2 = merge (kinetic energy lost, the field
 * excitation of integrator.js:1394-1414; px = py = 0).  Copies
 * min(events, capacity) rows; `n` receives the number stored. */
int geon_collision_events(GeonHandle* h, double* events, int32_t capacity, int32_t* n);

/* Copies `rows` rows (GEON_OUT_*) of per-particle force data, each `capacity`
 * floats, starting at row `first_row`. */
int geon_download_forces(GeonHandle* h, int32_t first_row, int32_t rows,
                         float* out, int32_t capacity);

/* QuadTreePool.build (src/quadtree.js:412-419) at the current positions
 * (with periodic ghosts, src/integrator.js:247-260).  Fills `info`. */
int geon_build_tree(GeonHandle* h, GeonTreeInfo* info);

/* Leaf membership of the last build, for exact comparison with the
 * reference tree: leaf_of_point[i] is the leaf index of tree point i
 * (particles first, then ghosts in generation order) or -1 if the point was
 * dropped.  For each leaf: centre (bx, by), half-size bw (quadtree.js:52-59)
 * and level.  Arrays are sized by the caller from GeonTreeInfo. */
int geon_tree_leaves(GeonHandle* h, int32_t* leaf_of_point, int32_t n_points,
                     double* leaf_bx, double* leaf_by, double* leaf_bw,
                     int32_t* leaf_level, int32_t n_leaves);

/* Interaction count of the last Barnes-Hut force pass (pair evaluations
 * summed over particles), for the walk's work accounting. */
int geon_interaction_count(GeonHandle* h, int64_t* count);

/* FP64 conserved quantities (src/energy.js:11-62; PE from src/forces.js:26).
 * GPUPhysics.requestStats/readStats (src/gpu/gpu-physics.js:4146/4234). */
int geon_stats(GeonHandle* h, GeonStats* out);

/* Signal-delay history (Particle.histX.. ring, src/particle.js:77-85,124-134).
 * Uploads `count` (<= 256) samples per particle, oldest first: times[count]
 * (shared by all particles, as Physics records them together,
 * integrator.js:1549-1565) and five rows (x, y, vx, vy, angw) of
 * n*count floats, particle-major.  Used to start from a warmed history. */
int geon_upload_history(GeonHandle* h, int32_t n, int32_t count,
                        const double* times, const float* samples);

/* Simulation clock (Physics.simTime). */
int geon_set_sim_time(GeonHandle* h, double sim_time);
int geon_get_sim_time(GeonHandle* h, double* sim_time);

/* Per-phase device time, measured with CUDA events recorded on the handle's
 * stream around each phase while profiling is on. */
typedef struct GeonProfile {
    double tree_ms;          /* ghosts, keys, radix sort, node emission, aggregation */
    double force_ms;         /* force passes (BH walk or pairwise sum)               */
    double onepn_ms;         /* 1PN-only passes                                      */
    double push_ms;          /* Boris push, VV kick, boundary                        */
    int64_t tree_count, force_count, onepn_count, push_count;
    int64_t interactions;    /* pair evaluations summed over the profiled force passes */
    int64_t particle_substeps;
    double learn_ms;         /* learned correction: network and expansions            */
    int64_t learn_count;
    int64_t learn_pairs;     /* (cell, group) records corrected                       */
    double collide_ms;       /* merge collisions: detection, resolution, target list  */
    int64_t collide_count;
} GeonProfile;

/* enable = 1 clears the counters and starts recording; enable = 0 stops.
 * `out` (may be NULL) receives the totals recorded so far (synchronises). */
int geon_profile(GeonHandle* h, int32_t enable, GeonProfile* out);

/* Measured FP32 FMA throughput of this GPU in TFLOP/s (FMA = 2 FLOP), from a
 * short microbenchmark on the handle's stream: the roofline denominator for
 * the FP32-bound force kernels.  Diagnostic; no reference counterpart. */
int geon_fp32_peak(GeonHandle* h, double* tflops);

/* The handle's CUDA stream (a cudaStream_t), for timing with events. */
int geon_get_stream(GeonHandle* h, void** stream);

/* Number of kernels this handle has launched since creation. */
int geon_launch_count(GeonHandle* h, int64_t* count);

/* Message for the last error on h (or a global message if h is NULL). */
const char* geon_last_error(GeonHandle* h);

/* Library version string. */
const char* geon_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GEON_H */
