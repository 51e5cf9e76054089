// world_dev.cuh -- device-resident state of one GPU mechanical world and the
// kernel entry points of each phase of the step.
//
// Layout in HBM (all arrays sized by capacity at npgpu_create):
//  bodies     SoA by body slot (= generational-arena index of the host set)
//  colliders  SoA by collider slot
//  pairs      broad-phase pairs, double-buffered (current / previous step),
//             4 contact slots per pair; the previous buffer feeds the impulse
//             cache of the next narrow phase
//  solver     one record per solver manifold; per contact 64 bytes of
//             constant row data (normal, lever arms, r and rhs of the normal
//             and two friction rows, friction) and 16 bytes of impulses
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "npgpu.h"

#include "np_math.cuh"

namespace npgpu_dev {

// Body info word.
enum : uint32_t {
    BI_STATUS_MASK = 0x3u,           // NPGPU_BODY_*
    BI_KIND_SHIFT = 2,               // 3 bits
    BI_FLAGS_SHIFT = 8,              // NPGPU_BODY_* flag bits, 9 bits
    BI_ALIVE = 1u << 20,
    BI_CHANGED = 1u << 21,           // BodyUpdateStatus: inertia / colliders need update
    BI_ISLAND = 1u << 22,            // in an awake island this step
};
inline __host__ __device__ uint32_t bi_status(uint32_t i) { return i & BI_STATUS_MASK; }
inline __host__ __device__ uint32_t bi_flags(uint32_t i) { return (i >> BI_FLAGS_SHIFT) & 0x1ffu; }

// Error flag bits (device word, read by npgpu_synchronize).
enum : uint32_t {
    ERRF_PAIR_CAPACITY = 1u << 0,
    ERRF_TIMEOUT = 1u << 1,
    ERRF_NAN = 1u << 2,
    ERRF_COLOURS = 1u << 3,
    ERRF_UNION_FIND = 1u << 4,
    ERRF_WORLD_RANGE = 1u << 5,      // a batched world's body outside its slot range
    ERRF_TASKS = 1u << 6,            // more solver manifolds than a cooperative grid holds
    ERRF_CCD_CAPACITY = 1u << 7,     // a world's CCD lists or the island pool overflowed (its CCD stopped)
};

constexpr int kMaxContacts = 4;      // contacts per manifold
constexpr int kRowFloats = 28;       // J1[6] J2[6] WJ1[6] WJ2[6] r rhs impulse mu
constexpr int kColourBits = 56;      // colours in one colour word's mask
constexpr int kStepColours = 2 * kColourBits;   // colours a step may use: two words per body
constexpr int kMaxColours = 128;     // colour buckets of the per-world schedule (>= kStepColours)
constexpr unsigned long long kColourMask = (1ull << kColourBits) - 1ull;
constexpr int kLeafCap = 16;        // partners a broad-phase leaf keeps between its two passes
constexpr int kPosRec = 7 + 4;       // float4 of a manifold's position-solver record
// A contact's three rows as the iterations read them: per row 7 float4 =
// J1[6] J2[6] WJ1[6] WJ2[6] r rhs mu (one spare).
constexpr int kRowF4 = 7;
constexpr int kRowsF4 = 3 * kRowF4;

// Row field offsets.
enum { RF_J1 = 0, RF_J2 = 6, RF_WJ1 = 12, RF_WJ2 = 18, RF_R = 24, RF_RHS = 25, RF_IMP = 26, RF_MU = 27 };

struct Bodies {
    float4 *pos_t, *pos_q;           // Isometry3 (translation, quaternion i j k w)
    float4 *lin, *ang;               // velocity
    float4 *com, *local_com;
    float *mass;                     // inertia.linear
    float *local_I;                  // 9 per body, local angular inertia
    float *I;                        // 9 per body, world angular inertia
    float *inv_mass;                 // inv_augmented_mass.linear
    float *inv_I;                    // 9 per body, inv_augmented_mass.angular
    float4 *acc_lin, *acc_ang;       // generalized acceleration
    float4 *f_lin, *f_ang;           // external forces
    float *lin_damp, *ang_damp, *max_lin, *max_ang, *sleep_thr, *energy;
    uint32_t *info;
    uint32_t *world;
    unsigned long long *gen;         // generation of the body in each slot (handles are checked against it)
    uint32_t *fstamp;                // the last force batch that named the body
    float *dv;                       // mj_lambda, 6 per body
    float4 *sb;                      // 3 per body: inverse augmented mass as the solver reads it
    unsigned long long *dvf;         // 8 per body: Δv words flagged with the body's update count
    unsigned long long *posef;       // 12 per body: pose words flagged with the body's update count
    uint32_t *uf_parent;
    int *can_deact;
    unsigned long long *cw;          // 2 colour words per body: manifolds coloured so far << 56 | 56 mask bits
                                     // (colours 0-55 in the first word, 56-111 in the second)
    uint32_t *adj_count, *adj_start, *adj_fill;   // solver manifolds per body (CSR)
};

struct Colliders {
    uint32_t *body;
    uint32_t *local;                 // slot minus the smallest alive collider slot of its body's world: the
                                     // colouring priority hashes these, so that a world's colouring does not
                                     // depend on where its slots start
    uint32_t *info;                  // shape | friction_combine << 4 | restitution_combine << 8 | alive << 16
    float4 *params;                  // ball: radius in x; cuboid: half extents
    float4 *wrt_t, *wrt_q;           // position_wrt_body
    float *margin, *lin_pred, *friction, *restitution, *rank;
    float4 *pose_t, *pose_q;
    float4 *aabb_min, *aabb_max;     // fat AABB; aabb_min.w = 1 when set
    unsigned long long *keys, *keys_sorted;
    uint32_t *vals, *vals_sorted;
    // LBVH over the alive colliders (n - 1 internal nodes, n leaves).
    int *left, *right, *parent;
    float4 *node_min, *node_max;
    float4 *wide;                    // 5 per internal node: both children's boxes and references
    uint32_t *node_slot;             // per node: the largest slot among its colliders of the largest rank
    int *node_flag;
    uint32_t *leaf_count, *leaf_offset;
    uint32_t *leaf_tmp;              // up to kLeafCap partners per leaf from the counting traversal
};
enum : uint32_t { CI_ALIVE = 1u << 16, CI_CCD = 1u << 17, CI_SENSOR = 1u << 18 };
// Proximity of a pair with a sensor (ncollide3d query::Proximity).
enum : uint32_t { PROX_INTERSECTING = 0, PROX_WITHIN_MARGIN = 1, PROX_DISJOINT = 2 };

// Joint constraints by joint slot (= the generational-arena index of the
// host joint set). The host writes the description; the impulses and the
// state bits are the device's.
struct Joints {
    uint32_t *info;                  // kind | JI_ALIVE (host-written)
    uint32_t *state;                 // JS_BROKEN | JS_ACTIVE (device-written)
    uint32_t *body;                  // 2 per joint: body slots
    uint32_t *local;                 // slot minus the smallest alive joint slot of its world (colouring priority)
    float4 *anchor;                  // 2 per joint: the anchors in their bodies' frames (xyz)
    float4 *frame;                   // 2 per joint: the reference frames (quaternion i j k w)
    float4 *axis;                    // 3 per joint: axis1 (.w: angle), axis2 (.w: min offset), axis3 (.w: max offset)
    float4 *imp;                     // 2 per joint: the impulses (linear xyz, angular xyz)
    float2 *brk;                     // break force^2, break torque^2
};
enum : uint32_t {
    JI_KIND_MASK = 0xffu, JI_ALIVE = 1u << 8, JI_MIN_OFFSET = 1u << 9, JI_MAX_OFFSET = 1u << 10,
    JS_BROKEN = 1u << 0, JS_ACTIVE = 1u << 1
};
// A solver manifold list entry of a joint: kJointBit | joint slot.
constexpr uint32_t kJointBit = 0x80000000u;
// A joint's row group in the solver records: up to three rows of one kind
// (forces along, or torques about, the record's directions: the normal slot
// and the two friction-direction slots). The friction slot, non-negative for
// a contact, holds -(4 kind + rows): kind 1 linear, 2 angular.
// kind 3 is a linear row whose impulse stays in [0, max] (a prismatic offset
// limit, unit_constraint.rs:33-123).
enum : uint32_t { JR_LINEAR = 1u, JR_ANGULAR = 2u, JR_LIMIT = 3u };
__host__ __device__ inline float joint_code(uint32_t kind, uint32_t rows) { return -(float)(4u * kind + rows); }
__host__ __device__ inline uint32_t joint_rows_of(float code) { return (uint32_t)(-code) & 3u; }
__host__ __device__ inline bool joint_angular(float code) { return ((uint32_t)(-code) >> 2) == JR_ANGULAR; }
__host__ __device__ inline bool joint_limit(float code) { return ((uint32_t)(-code) >> 2) == JR_LIMIT; }
// Row groups (solver records) of a joint kind.
__host__ __device__ inline uint32_t joint_group_count(uint32_t kind) {
    if (kind == NPGPU_JOINT_BALL || kind == NPGPU_JOINT_CARTESIAN) return 1u;
    return kind == NPGPU_JOINT_PRISMATIC ? 3u : 2u;
}
// The impulse slot row r of group g of a joint kind starts from (store
// false) and is cached to (store true): 0-2 the joint's linear impulses, 3-5
// its angular ones, 6 the prismatic limit's. The cylindrical and pin-slot
// joints number their angular rows from DIM - 1 (cylindrical_constraint.rs,
// pin_slot_constraint.rs): they start from angular impulses 0 and 1 and are
// cached to linear impulse 2 and angular impulse 0.
__host__ __device__ inline uint32_t joint_slot(uint32_t kind, uint32_t g, uint32_t r, bool store) {
    switch (kind) {
    case NPGPU_JOINT_CYLINDRICAL:
    case NPGPU_JOINT_PIN_SLOT:
        if (g == 1u) return store ? (r == 0u ? 2u : 3u) : 3u + r;
        return r;
    case NPGPU_JOINT_PRISMATIC: return g == 0u ? r : (g == 1u ? 3u + r : 6u);
    case NPGPU_JOINT_CARTESIAN: return 3u + r;
    default: return g == 0u ? r : 3u + r;
    }
}

struct Pairs {
    uint2 *pair;                     // (collider1, collider2), collider1 < collider2
    uint32_t *owner_start, *owner_count;   // by collider slot: the pairs it owns
    uint8_t *ncont;                  // contacts in the manifold
    uint8_t *prox;                   // PROX_* of a pair with a sensor (PROX_DISJOINT otherwise)
    uint32_t *key;                   // 4 per pair: feature key (fid1 * 26 + fid2)
    float4 *w1;                      // world1 xyz, depth
    float4 *w2;                      // world2 xyz
    float4 *n;                       // normal xyz
    float4 *imp;                     // cached impulses (normal, tangent 1, tangent 2)
    float4 *nl;                      // normal in body 1's frame
};

struct Solver {
    uint32_t *sm_list;               // solver manifolds (pair indices), in no particular order
    uint32_t *sm_colour;             // colour of each solver manifold
    uint32_t *sm_prank;              // priority rank among the manifolds of body 1 | body 2 << 16
    uint32_t *sm_rk;                 // colour rank / manifold count on body 1 and body 2 (8 bits each)
    int *sm_b1, *sm_b2;              // dynamic body slots (-1 when the side has no dofs)
    uint32_t *sm_nc;
    float4 *con;                     // 4 contacts x 4 float4 per solver manifold (constant during the solve)
    float4 *lam;                     // 4 contacts per solver manifold: impulses (normal, tangent 1, tangent 2)
    float4 *lam_alt;                 // learned warm start: the start each prediction replaced (the cached
                                     // impulses, or zero for a contact without a cache entry)
    float4 *tan;                     // 4 contacts x 2 per solver manifold: the friction directions (xyz)
    float4 *rows;                    // 4 contacts x kRowsF4 per solver manifold: normal, friction 1, friction 2 rows
    uint32_t *sm_mask;               // unlocked dofs of body 1 (bits 0-5) and body 2 (bits 8-13); kJointBit: a joint's rows
    float4 *pos_rec;                 // kPosRec per solver manifold: what the position solver reads besides poses
    uint32_t *adj;                   // body -> its solver manifolds (CSR over adj_start)
    // Batched worlds: manifolds bucketed by (world, colour).
    uint32_t *world_start;           // body slot range of each world (n_worlds + 1)
    uint32_t *world_order;           // worlds by decreasing slot range: the order blocks take them in
    // bucket_count (n_worlds * kMaxColours + 1) and bucket_cursor follow each
    // other in one allocation, cleared by one memset each step.
    uint32_t *bucket_count, *bucket_start, *bucket_cursor;
    uint32_t *wm_order;              // solver manifolds ordered by (world, colour)
    // The per-world schedule renumbers the solver manifolds in that order
    // before assembly (through `perm`, 5 arrays of scratch), so each colour
    // of a world is one run of manifold indices.
    uint32_t *perm;
    // Learned warm start: per-contact features while recording (null otherwise)
    // and the sample buffer they are appended to after the solve.
    float *feat;
    float *samples;
    uint32_t sample_cap;
};

// Device counters and control words (one struct in device memory).
struct Control {
    uint32_t npairs;
    uint32_t nsolver;                // solver manifolds
    uint32_t ncolours;
    uint32_t err;
    uint32_t barrier_count;          // monotonic grid-barrier arrivals of the running cooperative kernel
    uint32_t pad1;
    uint32_t jp_remaining[2];
    uint32_t ncontacts;
    uint32_t nmanifolds;
    uint32_t nsolver_contacts;
    uint32_t nactive;
    uint32_t iterations;
    uint32_t pad0;
    double res_acc[2];               // FP64 residual accumulators (phi^2, lambda^2)
    double residual, residual_initial;
    double kinetic_energy;
    unsigned long long max_pen_bits; // order-preserving bits of the max penetration
    unsigned long long t_phase[16];  // %globaltimer stamps
    unsigned long long task_ns, wait_ns, tasks;   // velocity-task statistics (profile mode)
    double res_acc_init[2];          // batched worlds: residual sums after the warm start
    uint32_t world_next[4];          // batched worlds: block and warp work counters of the velocity / position kernels
    uint32_t mlp_samples;            // training samples recorded so far
    uint32_t learned_starts, learned_kept;   // learned warm start: predictions made / kept this step
    uint32_t force_flags;            // checks of the last force batch: 1 bad handle, 2 non-finite, 4 a body twice
    double mlp_loss;                 // loss of the last training step
    uint32_t nevents;                // contact events of this step so far (may exceed World::events_cap)
    uint32_t ccd_mcount;             // CCD island manifolds taken from the pool this step
    uint32_t ccd_substeps, ccd_impacts;
    uint32_t pad3;
    unsigned long long ccd_ns[4];    // profile mode: CCD time by part (toi, solver, broad, narrow), summed over worlds
    unsigned long long ccd_max_ns;   // ... and the longest world's
};

struct StepParams {
    float dt, inv_dt;
    float erp, warmstart_coeff, restitution_threshold;
    float allowed_linear_error, max_linear_correction;
    float activation_mix, broad_phase_margin;
    float gx, gy, gz;
    float residual_tolerance;
    uint32_t max_velocity_iterations, max_position_iterations;
    uint32_t solve_to_tolerance, max_iterations_to_tolerance;
    uint32_t warmstart_mode;
    uint32_t profile;
    uint32_t sweep_order;            // NPGPU_SWEEP_*
    float allowed_angular_error, max_angular_correction;
    uint32_t ccd;                    // 1: CCD runs after the solver (the update flags and the energy audit wait for it)
};

// Continuous collision detection (MechanicalWorld::solve_ccd), one block per
// world that has a CCD collider. Allocated when the first CCD collider
// appears. A world's lists live in its own region of each scratch array:
// region base kCcdRegion * order index of its first collider + kCcdSlack *
// world, length kCcdRegion * its colliders + kCcdSlack.
constexpr uint32_t kCcdRegion = 4, kCcdSlack = 64;
constexpr uint32_t kCcdStateWords = 16, kCcdColours = 256;
struct CcdToi {                      // a time of impact in a world's queue
    float toi;
    uint32_t c1, c2;
    uint32_t seq;                    // order of discovery; bit 31: superseded by a resweep
};
struct CcdContact {                  // a contact of a substep's island
    float4 n;                        // normal from collider 1 toward 2; depth in w
    float4 w1, w2;                   // world points (xyz); w1.w: feature key fid1 * 26 + fid2
    float4 nl;                       // normal in body 1's frame
    float4 pos1, pos2;               // lever arms from the centres of mass; r and rhs of the normal row in w
    float4 rr;                       // r, rhs of the two friction rows
    float4 lam;                      // impulses (normal, friction 1, friction 2)
    float4 t1, t2;                   // friction directions
};
struct CcdManifold {
    uint32_t c1, c2, nc, mask;       // mask: unlocked dofs (sm_mask's layout)
    int b1, b2;                      // dynamic body slots (-1: no dofs)
    float mu;
    uint32_t colour;                 // in the island's greedy colouring
    CcdContact k[kMaxContacts];
};
struct Ccd {
    uint32_t *order;                 // collider slots sorted by (world, slot)
    unsigned long long *keys, *keys_sorted;
    uint32_t *slots;                 // 0..n-1, the sort's values
    uint32_t *wstart;                // per world: first index into `order` (n_worlds + 1)
    uint32_t *wflag;                 // per world: 1 when it has a CCD collider
    float *wdts;                     // per world: the last substep's length (< 0: none this step)
    uint32_t *wstate;                // per world: kCcdStateWords words carried between the CCD kernels
    uint32_t *wcols;                 // per world: its substep island's colour starts (kCcdColours + 1)
    uint32_t *bc_start, *bc_list;    // colliders of each body, in slot order (host-built CSR)
    uint32_t *ccd_list, *ccd_wstart; // the CCD colliders by (world, slot), each world's range (host-built)
    uint32_t *adj_count, *adj_start, *adj_list;   // the step's broad-phase pairs by collider (CSR, partners in
                                                  // slot order), built on the device each step with CCD
    void* adj_scan;                  // exclusive-scan scratch of adj_count
    size_t adj_scan_bytes;
    uint32_t *bepoch;                // per body: the last neighbour sweep of the island search that saw it
    unsigned long long *bcol;        // per body: colours of the island manifolds on it
    float4 *sw_min, *sw_max;         // per collider: the box swept from the safe pose to the current one
    float4 *pos0_t, *pos0_q;         // per body: position0
    float *btime, *ftime;            // per body: SubstepState::body_times, frozen time
    uint32_t *bflag;                 // per body: 1 frozen, 2 prepared
    uint32_t *cflag;                 // per collider: 1 visited
    uint32_t *nbr, *nbr2, *stack, *island, *ccdb, *mlist, *mord;   // per-world regions
    uint2 *res;                      // per-world region: per neighbour, the prepared bits before a sweep and
                                     // the pool slot of the pair's contacts
    float2 *tres;                    // per-world region: TOI results aligned with nbr
    CcdToi *heap, *impacts;          // per-world regions
    CcdManifold *pool;               // island manifolds of all worlds, taken by an atomic counter
    uint32_t pool_cap;
    uint32_t n_worlds;               // world indices in use (max + 1)
    uint32_t substeps;               // max_ccd_substeps
    uint32_t on_penetration;         // ccd_on_penetration_enabled
    uint32_t max_position_iterations;   // max_ccd_position_iterations
};

struct MlpDev;

struct World {
    const MlpDev* mlp;               // the learned warm start's network (null when none is set)
    Bodies b;
    Colliders c;
    Pairs cur, prev;
    Solver s;
    Control* ctl;
    uint32_t nb_slots, nc_slots, cap_pairs, nc_alive;
    uint32_t world_bits;             // bits of the largest world index of any body so far
    uint2* events;                   // contact events (collider1, collider2 | stopped << 31), null when off
    uint32_t events_cap;
    Joints j;
    uint32_t nj_slots;               // joint slots in use (0: no joint kernels run)
    Ccd ccd;                         // allocated when a CCD collider exists (ccd.order non-null)
};

// ---- launchers (defined in the kernel translation units) ----
cudaError_t launch_body_start(const World& w, const StepParams& p, cudaStream_t st);
cudaError_t launch_sync_aabb(const World& w, const StepParams& p, cudaStream_t st);
cudaError_t launch_lbvh(const World& w, cudaStream_t st);
cudaError_t launch_pairs(const World& w, void* temp, size_t temp_bytes, cudaStream_t st);
cudaError_t launch_narrow(const World& w, cudaStream_t st);
cudaError_t launch_events(const World& w, cudaStream_t st);   // contact events of pairs no longer in the broad phase
// The solver half of a step (activation, colouring, assembly, SOR-Prox,
// integration, position correction, post-step updates). ev[0..6], when
// non-null, receive the phase boundaries for profiling.
struct SolverLaunch {
    int grid_colour, grid_velocity, grid_position;   // co-resident blocks of the cooperative kernels
    void* scan_temp;
    size_t scan_bytes;
    cudaEvent_t* ev;
    // Batched worlds (one block per world, Δv in shared memory).
    bool batched;
    uint32_t n_worlds;
    uint32_t max_world_bodies;       // largest body slot range of a world
    uint32_t n_big;                  // worlds wider than kWarpWorldBodies: one block each; the rest one warp each
    int grid_world;                  // blocks of the per-world kernels
    int world_threads;               // threads per world block of the velocity kernel: 64, 128 or 256
    int grid_world_position;         // blocks of the per-world position kernel (128 threads each)
    // Worlds wider than kMaxWorldBodies: one thread-block cluster each, first in the world order.
    uint32_t n_cluster;
    int cluster_ctas;                // blocks per cluster (16 where the part allows, else 8)
    uint32_t cluster_shift;          // 2^shift body rows per block
};
constexpr uint32_t kWarpWorldBodies = 256;    // widest world a single warp solves
constexpr uint32_t kMaxWorldBodies = 4096;    // per-world shared-memory Δv limit (96 KiB)
constexpr int kClusterThreads = 512;          // threads per block of the cluster kernels
constexpr uint32_t kClusterShiftMax = 13;     // at most 8192 body rows (192 KiB) per cluster block
// Blocks per cluster of the cluster kernels on this device (0: clusters unavailable).
int cluster_ctas(int device);
cudaError_t launch_solver(const World& w, const StepParams& p, const SolverLaunch& L, cudaStream_t st);
void solver_grid_sizes(int device, SolverLaunch& L);
// Blocks of the per-world kernels: resident blocks at this shared-memory size,
// at most one per world.
int world_grid(int device, uint32_t max_world_bodies, uint32_t n_worlds, int threads);
// Solver manifolds the one-grid schedule's cooperative kernels can hold.
uint64_t grid_task_capacity(const SolverLaunch& L);
size_t sort_temp_bytes(uint32_t n_items);
size_t scan_temp_bytes(uint32_t n_items);
cudaError_t launch_sort(const World& w, void* temp, size_t temp_bytes, cudaStream_t st);

// Learned warm start (k_mlp.cu).
cudaError_t mlp_upload(const float* prm_dev, MlpDev* net, cudaStream_t st);
cudaError_t mlp_normalise(const float* samples, uint32_t n, double* acc, float* prm, cudaStream_t st);
cudaError_t mlp_init(float* prm, uint32_t seed, cudaStream_t st);
cudaError_t mlp_grad(const MlpDev* net, const float* samples, uint32_t n, uint32_t batch, uint32_t seed, uint32_t step,
                     float* grad, double* loss, cudaStream_t st);
cudaError_t mlp_adam(float* prm, float* m1, float* m2, const float* grad, float lr, uint32_t t, MlpDev* net,
                     cudaStream_t st);

// Uploads / maintenance kernels.
struct BodyUpload {
    unsigned long long gen;
    uint32_t slot;
    uint32_t info;
    uint32_t world;
    uint32_t reset_energy;           // 1 for a new body: energy = 0.04 (or 0 for a ground)
    float pos[7], vel[6];
    float mass, local_I[9], local_com[3];
    float lin_damp, ang_damp, max_lin, max_ang, sleep_thr;
};
struct ColliderUpload {
    uint32_t slot, body, info;
    float params[4], wrt[7];
    float margin, lin_pred, friction, restitution, rank;
};
struct JointUpload {                 // one joint's description (info 0: removed)
    uint32_t slot, info, body1, body2;
    uint32_t reset;                  // 1: the impulses and the state start from zero
    float anchor1[3], anchor2[3], frame1[4], frame2[4];
    float brk_force2, brk_torque2;
    float axis1[3], axis2[3], angle;
    float axis3[3], min_offset, max_offset;
};
struct MassUpdate {                  // new local inertia / com of a body
    uint32_t slot;
    uint32_t activate;               // bit 0: inertia changed; bit 1: Body::activate (collider removal)
    float mass, local_I[9], local_com[3];
};
cudaError_t launch_upload_bodies(const World& w, const BodyUpload* d, uint32_t n, cudaStream_t st);
cudaError_t launch_upload_colliders(const World& w, const ColliderUpload* d, uint32_t n, cudaStream_t st);
cudaError_t launch_mass_updates(const World& w, const MassUpdate* d, uint32_t n, cudaStream_t st);
cudaError_t launch_upload_joints(const World& w, const JointUpload* d, uint32_t n, cudaStream_t st);
// CCD: position0 of every body at the step's start; the worlds' CCD after the solver.
cudaError_t launch_ccd_begin(const World& w, cudaStream_t st);
cudaError_t launch_ccd(const World& w, const StepParams& p, cudaStream_t st);
// Poses (7 floats) and velocities (6) of slots [first, first + n) into
// page-locked host arrays, given by their device-side addresses.
cudaError_t launch_pack_bodies_host(const World& w, uint32_t first, uint32_t n, float* pos7, float* vel6,
                                    cudaStream_t st);
// Checks a force batch on the device (handles against the slots' generations,
// finite forces, a body named twice) into ctl->force_flags, which the caller
// clears first, reading it from (handles, forces6) and keeping a copy in
// (hd, fd) when those differ. cap: body slots allocated.
cudaError_t launch_force_check(const World& w, const npgpu_handle* handles, const float* forces6, npgpu_handle* hd,
                               float* fd, uint32_t n, uint32_t batch, uint64_t cap, cudaStream_t st);
// Adds forces6[k] (linear, angular) to body handles[k].index; `serial`: in
// order on one thread, for batches that name a body twice.
cudaError_t launch_forces(const World& w, const npgpu_handle* handles, const float* forces6, uint32_t n, bool wake,
                          bool serial, cudaStream_t st);
cudaError_t launch_kill(const World& w, const uint32_t* slots, uint32_t n, int colliders, cudaStream_t st);
cudaError_t launch_forget_pairs(const World& w, const uint8_t* flags, cudaStream_t st);
cudaError_t launch_pack_bodies(const World& w, uint32_t first, uint32_t n, float* pos7, float* vel6, float* energy,
                               uint8_t* active, cudaStream_t st);

}  // namespace npgpu_dev
