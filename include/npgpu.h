/*
 * npgpu.h -- C ABI of the GB300 rigid-body step for nphysics3d.
 *
 * This is the drop-in boundary for `MechanicalWorld::step`
 * (src/world/mechanical_world.rs:182-396). A host binding (the Rust
 * `GpuMechanicalWorld` shim, the C++ `npgpu::GpuMechanicalWorld`, or the
 * Python ctypes mirror) owns the handle arenas (`DefaultBodySet`,
 * `DefaultColliderSet`, src/object/body_set.rs:178, collider_set.rs) and
 * forwards insertions, removals and the step through these entry points.
 * The device owns the body/collider state and the impulse cache
 * (src/solver/moreau_jean_solver.rs:14-23,
 * src/solver/signorini_coulomb_pyramid_model.rs:19-25).
 *
 * Conventions
 *  - Scalars are f32. Isometries are 7 floats: translation (x, y, z) then
 *    a unit quaternion (i, j, k, w) -- nalgebra's `Isometry3` storage order.
 *  - Velocities and forces are 6 floats: linear (x, y, z) then angular.
 *  - Body and collider slots are the generational-arena indices of the host
 *    sets; a handle is (index, generation). A slot whose generation does not
 *    match is INVALID_HANDLE.
 *  - No entry point aborts, traps or prints: every failure is a status code,
 *    and npgpu_last_error() holds a one-line description.
 *  - Calls on one world are not re-entrant and must come from one host
 *    thread. Each world owns one CUDA stream (npgpu_stream()).
 */
#ifndef NPGPU_H
#define NPGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NPGPU_ABI_VERSION 8u

/* generational_arena::Index (src/object/body_set.rs:178). */
typedef struct npgpu_handle {
    uint64_t index;
    uint64_t generation;
} npgpu_handle;

/* Errors: the reference panics or skips (src/solver/constraint.rs:89,234,
 * src/solver/moreau_jean_solver.rs:147, src/world/geometrical_world.rs:66-73);
 * the GPU world returns one of these instead. */
typedef enum npgpu_status {
    NPGPU_OK = 0,
    NPGPU_ERR_INVALID_HANDLE = 1,
    NPGPU_ERR_UNSUPPORTED_BODY = 2,   /* multibody, FEM, mass-spring, mass-constraint */
    NPGPU_ERR_UNSUPPORTED_SHAPE = 3,  /* anything but Ball, Cuboid and Capsule, or a sensor */
    NPGPU_ERR_NONEMPTY_JOINTS = 4,    /* the step's joint count differs from the joints uploaded */
    NPGPU_ERR_NONEMPTY_FORCES = 5,
    NPGPU_ERR_CAPACITY = 6,           /* a fixed-capacity device buffer overflowed */
    NPGPU_ERR_NAN = 7,                /* non-finite input or state */
    NPGPU_ERR_TIMEOUT = 8,            /* a bounded device wait gave up */
    NPGPU_ERR_CUDA = 9,
    NPGPU_ERR_INVALID_ARGUMENT = 10
} npgpu_status;

/* BodyStatus (src/object/body.rs:50-59). */
enum {
    NPGPU_BODY_DISABLED = 0,
    NPGPU_BODY_STATIC = 1,
    NPGPU_BODY_DYNAMIC = 2,
    NPGPU_BODY_KINEMATIC = 3
};

/* Body kinds. Only rigid bodies and grounds are accepted; the others exist
 * so that a binding can forward them and receive UNSUPPORTED_BODY. */
enum {
    NPGPU_KIND_RIGID_BODY = 0,   /* src/object/rigid_body.rs */
    NPGPU_KIND_GROUND = 1,       /* src/object/ground.rs: static, 0 dofs */
    NPGPU_KIND_MULTIBODY = 2,
    NPGPU_KIND_FEM_VOLUME = 3,
    NPGPU_KIND_FEM_SURFACE = 4,
    NPGPU_KIND_MASS_SPRING = 5,
    NPGPU_KIND_MASS_CONSTRAINT = 6
};

/* Body flags (RigidBodyDesc, src/object/rigid_body.rs:949-1086). */
enum {
    NPGPU_BODY_GRAVITY = 1u << 0,          /* gravity_enabled (default on) */
    NPGPU_BODY_LOCK_TX = 1u << 1,          /* kinematic_translations.x */
    NPGPU_BODY_LOCK_TY = 1u << 2,
    NPGPU_BODY_LOCK_TZ = 1u << 3,
    NPGPU_BODY_LOCK_RX = 1u << 4,          /* kinematic_rotations.x */
    NPGPU_BODY_LOCK_RY = 1u << 5,
    NPGPU_BODY_LOCK_RZ = 1u << 6,
    NPGPU_BODY_CAN_SLEEP = 1u << 7,        /* sleep_threshold is Some(..) */
    NPGPU_BODY_LINEAR_INTERP = 1u << 8     /* linear_motion_interpolation (CCD only) */
};

/* One body as built by RigidBodyDesc::build (rigid_body.rs:1064-1084). */
typedef struct npgpu_body_desc {
    float position[7];          /* Isometry3 */
    float velocity[6];          /* Velocity3 */
    float local_inertia[7];     /* mass, then the angular tensor (xx, xy, xz, yy, yz, zz) */
    float local_com[3];         /* local_center_of_mass */
    float linear_damping;
    float angular_damping;
    float max_linear_velocity;  /* FLT_MAX = unbounded (rigid_body.rs:72) */
    float max_angular_velocity;
    float sleep_threshold;      /* used when NPGPU_BODY_CAN_SLEEP; default 0.01 (body.rs:73) */
    uint32_t status;            /* NPGPU_BODY_* */
    uint32_t kind;              /* NPGPU_KIND_* */
    uint32_t flags;             /* NPGPU_BODY_* flag bits */
    uint32_t world;             /* index of the world in a batch (0 for one world) */
} npgpu_body_desc;

/* Shapes (ncollide3d::shape). */
enum {
    NPGPU_SHAPE_BALL = 0,        /* shape_params: radius */
    NPGPU_SHAPE_CUBOID = 1,      /* shape_params: half extents */
    NPGPU_SHAPE_OTHER = 2,       /* rejected with UNSUPPORTED_SHAPE */
    NPGPU_SHAPE_CAPSULE = 3      /* shape_params: radius, half height; the axis is the local y axis
                                    (ncollide3d::shape::Capsule::new(half_height, radius)) */
};

/* MaterialCombineMode (src/material/material.rs:49-64). */
enum {
    NPGPU_COMBINE_AVERAGE = 0,
    NPGPU_COMBINE_MIN = 1,
    NPGPU_COMBINE_MULTIPLY = 2,
    NPGPU_COMBINE_MAX = 3
};

/* One collider as built by ColliderDesc::build (src/object/collider.rs:538-572)
 * with a BasicMaterial (src/material/basic_material.rs). */
typedef struct npgpu_collider_desc {
    npgpu_handle body;          /* parent body (BodyPartHandle(body, 0)) */
    float position_wrt_body[7]; /* ColliderDesc::position */
    float shape_params[3];      /* ball: radius; cuboid: half extents; capsule: radius, half height */
    float margin;               /* default 0.01 (collider.rs:476-479) */
    float density;              /* default 0 (collider.rs:469) */
    float linear_prediction;    /* default 0.001 (collider.rs:457) */
    float angular_prediction;   /* default 5 degrees (collider.rs:458) */
    float friction;             /* BasicMaterial default 0.5 (basic_material.rs:59-63) */
    float restitution;          /* default 0 */
    uint32_t friction_combine;  /* NPGPU_COMBINE_* */
    uint32_t restitution_combine;
    uint32_t shape;             /* NPGPU_SHAPE_* */
    uint32_t is_sensor;         /* ColliderDesc::sensor: proximity events, no contacts; its query limit is
                                 * linear_prediction alone (collider.rs:542-543); CCD ignores its pairs */
    uint32_t ccd_enabled;       /* Collider::enable_ccd: time-of-impact substeps (MechanicalWorld::solve_ccd) */
} npgpu_collider_desc;

/* Joint constraints (src/joint/): BallConstraint (ball_constraint.rs) keeps anchor1 and anchor2
 * together; FixedConstraint (fixed_constraint.rs) also keeps the frames
 * (body rotation x reference frame) aligned; RevoluteConstraint
 * (revolute_constraint.rs) keeps the anchors together and axis1, axis2
 * aligned; CartesianConstraint (cartesian_constraint.rs) keeps only the
 * frames aligned; PlanarConstraint (planar_constraint.rs) keeps anchor2 in
 * the plane through anchor1 normal to axis1 and the axes aligned;
 * RectangularConstraint (rectangular_constraint.rs) keeps anchor2 in that
 * plane and the bodies' rotations equal; UniversalConstraint
 * (universal_constraint.rs) keeps the anchors together and the angle between
 * the axes; PrismaticConstraint (prismatic_constraint.rs) lets anchor2 slide
 * along axis1 only, within the optional offset limits, the rotations equal;
 * CylindricalConstraint (cylindrical_constraint.rs) lets it slide along and
 * turn about axis1; PinSlotConstraint (pin_slot_constraint.rs) lets it slide
 * along axis1 (axis_v1) and turn about axis3 (axis_w1, body 1) = axis2
 * (axis_w2, body 2). */
enum {
    NPGPU_JOINT_BALL = 0,
    NPGPU_JOINT_FIXED = 1,
    NPGPU_JOINT_REVOLUTE = 2,
    NPGPU_JOINT_CARTESIAN = 3,
    NPGPU_JOINT_PLANAR = 4,
    NPGPU_JOINT_RECTANGULAR = 5,
    NPGPU_JOINT_UNIVERSAL = 6,
    NPGPU_JOINT_PRISMATIC = 7,
    NPGPU_JOINT_CYLINDRICAL = 8,
    NPGPU_JOINT_PIN_SLOT = 9
};

/* Prismatic offset limits (enable_min_offset / enable_max_offset). */
enum {
    NPGPU_JOINT_MIN_OFFSET = 1u << 0,
    NPGPU_JOINT_MAX_OFFSET = 1u << 1
};

/* One joint constraint as its ::new builds it. Both bodies must belong to
 * the same world, and body1 != body2. */
typedef struct npgpu_joint_desc {
    uint32_t kind;              /* NPGPU_JOINT_* */
    uint32_t pad;
    npgpu_handle body1;         /* BodyPartHandle(body1, 0) */
    npgpu_handle body2;
    float anchor1[3];           /* in body 1's local frame */
    float anchor2[3];           /* in body 2's local frame */
    float frame1[4];            /* FIXED, CARTESIAN: ref_frame1, a unit quaternion (i, j, k, w) */
    float frame2[4];            /* FIXED, CARTESIAN: ref_frame2 */
    float break_force;          /* set_break_force; FLT_MAX (the default) never breaks */
    float break_torque;         /* set_break_torque */
    float axis1[3];             /* unit axis in body 1's frame (REVOLUTE, PLANAR, RECTANGULAR, UNIVERSAL,
                                   PRISMATIC, CYLINDRICAL; PIN_SLOT: axis_v1) */
    float axis2[3];             /* unit axis in body 2's frame (REVOLUTE, PLANAR, UNIVERSAL, CYLINDRICAL;
                                   PIN_SLOT: axis_w2) */
    float angle;                /* UNIVERSAL: the angle kept between the axes */
    uint32_t limit_flags;       /* PRISMATIC: NPGPU_JOINT_MIN_OFFSET | NPGPU_JOINT_MAX_OFFSET */
    float axis3[3];             /* PIN_SLOT: axis_w1, in body 1's frame */
    float min_offset;           /* PRISMATIC: the limits of the offset of anchor2 along axis1 */
    float max_offset;
    uint32_t pad2;
} npgpu_joint_desc;

/* A joint's state after the last step: the impulses JointConstraint::
 * cache_impulses keeps (its linear impulses, then its angular ones, in the
 * joint's own order), the prismatic limit's impulse, and is_broken(). */
typedef struct npgpu_joint_state {
    float impulses[6];
    float limit_impulse;
    uint32_t broken;
    uint32_t active;            /* solved in the last step (JointConstraint::is_active) */
    uint32_t pad;
} npgpu_joint_state;

/* IntegrationParameters (src/solver/integration_parameters.rs:5-190),
 * plus the GPU-only knobs at the end. */
/* Solver schedules. AUTO picks WORLDS when the step qualifies (at least two
 * worlds, each world's alive bodies in one contiguous run of slots with
 * world indices non-decreasing in slot order, no world wider than 4096 slots,
 * solve_to_tolerance off), else GRID. Both give identical results. */
enum {
    NPGPU_SCHEDULE_AUTO = 0,
    NPGPU_SCHEDULE_GRID = 1,      /* one cooperative grid, per-body dataflow between colours */
    NPGPU_SCHEDULE_WORLDS = 2     /* one block per world, world Δv in shared memory; falls back to GRID
                                     when the step does not qualify */
};

/* Row order within a velocity iteration. SEPARATE is SORProx::step's
 * structure (sor_prox.rs:48-80): every friction row, then every normal row,
 * each sweep over the manifolds in colour order. MANIFOLD solves a manifold's
 * friction rows and then its normal rows before the next manifold, one sweep
 * in colour order per iteration: another Gauss-Seidel order of the same rows,
 * with the same fixed point and half the chain of dependent updates. */
enum {
    NPGPU_SWEEP_SEPARATE = 0,
    NPGPU_SWEEP_MANIFOLD = 1
};

typedef struct npgpu_params {
    float dt;                              /* 1/60 */
    float erp;                             /* 0.2 */
    float warmstart_coeff;                 /* 1.0 */
    float restitution_velocity_threshold;  /* 1.0 */
    float allowed_linear_error;            /* 0.001 */
    float allowed_angular_error;           /* 0.001 */
    float max_linear_correction;           /* 0.2 */
    float max_angular_correction;          /* 0.2 */
    float max_stabilization_multiplier;    /* 0.2 */
    uint32_t max_velocity_iterations;      /* 8 */
    uint32_t max_position_iterations;      /* 3 */
    uint32_t max_ccd_position_iterations;  /* 10 */
    uint32_t max_ccd_substeps;             /* 1 (0: no CCD) */
    /* GPU-only. */
    uint32_t solve_to_tolerance;           /* 0: run max_velocity_iterations; 1: stop when residual <= tol */
    float residual_tolerance;              /* 1e-4 */
    uint32_t max_iterations_to_tolerance;  /* cap when solve_to_tolerance (e.g. 256) */
    uint32_t warmstart_mode;               /* 0: impulse cache (reference); 1: none; 2: impulse cache, and the
                                              learned network for contacts without a cache entry; 3: the
                                              network for every contact, each prediction kept only where
                                              it beats the start it replaces (cache or zero) */
    float broad_phase_margin;              /* DBVTBroadPhase::new(0.01), geometrical_world.rs:60 */
    float activation_mix;                  /* ActivationManager::new(0.01), mechanical_world.rs:80 */
    uint32_t profile;                      /* non-zero: time each phase with CUDA events */
    uint32_t solver_schedule;              /* NPGPU_SCHEDULE_*: how the velocity and position solvers run */
    uint32_t use_graph;                    /* 1: run each step from a CUDA graph, captured on first use and
                                              replayed while nothing the launches bake in changes (the
                                              world's shape, parameters, buffers); ignored when profiling */
    uint32_t world_threads;                /* threads per world block of NPGPU_SCHEDULE_WORLDS: 64, 128 or
                                              256 (0: 128); npgpu_autotune chooses it */
    uint32_t sweep_order;                  /* NPGPU_SWEEP_*: the order of the rows within an iteration */
    uint32_t ccd_on_penetration_enabled;   /* 0: a CCD pair already overlapping at the step's start has no
                                              time of impact (IntegrationParameters::ccd_on_penetration_enabled) */
} npgpu_params;

/* Per-step counters: the stage names of src/counters/mod.rs:18-209 plus
 * solver statistics. Times are milliseconds of the last step (0 unless
 * params.profile). */
typedef struct npgpu_counters {
    double step_time;
    double collision_detection_time;
    double broad_phase_time;
    double narrow_phase_time;
    double island_construction_time;
    double solver_time;
    double assembly_time;
    double velocity_resolution_time;
    double velocity_update_time;
    double position_resolution_time;
    double colouring_time;
    uint64_t steps;
    uint32_t num_pairs;              /* broad-phase pairs */
    uint32_t num_manifolds;          /* pairs with at least one contact */
    uint32_t num_contacts;           /* contacts in all manifolds */
    uint32_t num_solver_contacts;    /* contacts handed to the solver (awake islands) */
    uint32_t num_constraints;        /* velocity rows: 3 per solver contact */
    uint32_t num_colours;
    uint32_t num_active_bodies;      /* dynamic bodies in awake islands */
    uint32_t velocity_iterations;    /* iterations run in the last step */
    double residual;                 /* FP64 complementarity residual after the last iteration */
    double residual_initial;         /* ... after the warm start, before iteration 1 */
    double max_penetration;          /* FP64 audit: max(depth + margins) over contacts */
    double kinetic_energy;           /* FP64 audit: sum 1/2 (m v.v + w.I w) */
    /* Profile only (params.profile): velocity-solver task statistics. */
    double velocity_task_ms;         /* summed execution time of all velocity tasks */
    double velocity_wait_ms;         /* summed time threads spent waiting for their bodies */
    double velocity_kernel_ms;       /* duration of the velocity kernel on the device clock */
    uint64_t velocity_tasks;         /* tasks executed */
    /* Learned warm start (params.warmstart_mode == 2). */
    uint32_t learned_starts;         /* new contacts started from the network's prediction */
    uint32_t learned_kept;           /* ... of which the warm-start sweep kept the prediction */
    uint32_t graph_replay;           /* 1 if the last step ran from a CUDA graph */
    uint32_t ccd_substeps;           /* CCD substeps of the last step, over all worlds */
    uint32_t ccd_impacts;            /* time-of-impact events those substeps resolved */
    uint32_t reserved;
    /* Profile only: CCD time in ms summed over the worlds' CCD blocks
     * (CCDCounters, counters/ccd_counters.rs:6-17), and the longest world. */
    double ccd_toi_computation_time; /* times of impact and their queue */
    double ccd_solver_time;          /* island bodies, colouring, solves, integration */
    double ccd_broad_phase_time;     /* swept boxes and neighbour searches */
    double ccd_narrow_phase_time;    /* the island's contacts */
    double ccd_world_time_max;       /* the longest world's CCD */
} npgpu_counters;

/* Contact record returned for parity checks (a TrackedContact,
 * ncollide3d query::TrackedContact, plus the solver's impulses). */
typedef struct npgpu_contact {
    uint32_t collider1, collider2;   /* collider slots, collider1 < collider2 */
    uint32_t feature_key;            /* our ContactId within the pair */
    uint32_t kinematic;              /* approximation kinds (low byte: 1, next: 2) */
    float world1[3];
    float world2[3];
    float normal[3];                 /* from collider1 toward collider2 */
    float depth;                     /* > 0 means penetration */
    float impulse[3];                /* cached (normal, tangent1, tangent2) */
    uint32_t colour;                 /* solver colour of the manifold, or 0xffffffff */
} npgpu_contact;

typedef struct npgpu_world npgpu_world;

/* Library version (NPGPU_ABI_VERSION).
 * No counterpart in the reference (a crate version). */
uint32_t npgpu_abi_version(void);

/* Fills `out` with IntegrationParameters::default() (integration_parameters.rs:169-189). */
void npgpu_default_params(npgpu_params* out);

/* MechanicalWorld::new(gravity) (mechanical_world.rs:76-99) plus
 * GeometricalWorld::new() (geometrical_world.rs:57-63). Capacities bound the
 * slot indices and the pair/contact buffers; *status receives the outcome. */
npgpu_world* npgpu_create(const npgpu_params* params, const float gravity[3],
                          uint32_t capacity_bodies, uint32_t capacity_colliders,
                          uint32_t capacity_pairs, npgpu_status* status);
void npgpu_destroy(npgpu_world* w);

/* The world's CUDA stream (a cudaStream_t), for callers that time or order work.
 * No counterpart in the reference, whose step runs on the calling thread. */
void* npgpu_stream(npgpu_world* w);

/* Replace MechanicalWorld::integration_parameters and MechanicalWorld::gravity
 * (src/world/mechanical_world.rs:61, 65), read by the next step. */
npgpu_status npgpu_set_params(npgpu_world* w, const npgpu_params* params);
npgpu_status npgpu_set_gravity(npgpu_world* w, const float gravity[3]);

/* DefaultBodySet::insert + the mass bookkeeping of maintain (mechanical_world.rs:114-179).
 * Inserting or overwriting a body marks it changed (it is woken up on the
 * next step, rigid_body.rs:563-565). */
npgpu_status npgpu_upsert_bodies(npgpu_world* w, uint32_t n, const npgpu_handle* handles,
                                 const npgpu_body_desc* descs);

/* DefaultColliderSet::insert; the collider's mass properties are added to its
 * body at the next step (geometrical_world.rs:102-143). */
npgpu_status npgpu_upsert_colliders(npgpu_world* w, uint32_t n, const npgpu_handle* handles,
                                    const npgpu_collider_desc* descs);

/* DefaultBodySet::remove / DefaultColliderSet::remove. Removing a body removes
 * its colliders (mechanical_world.rs:130-139). */
npgpu_status npgpu_remove_bodies(npgpu_world* w, uint32_t n, const npgpu_handle* handles);
npgpu_status npgpu_remove_colliders(npgpu_world* w, uint32_t n, const npgpu_handle* handles);

/* RigidBody::apply_force(0, force, ForceType::Force, auto_wake_up)
 * (rigid_body.rs:783-820): accumulates into the external force, which the
 * next step uses and then clears. forces6[6n]: linear, then angular. The
 * batch is checked whole before any force is applied (an invalid handle or a
 * non-finite force applies nothing); a body named twice gets both forces in
 * order. Page-locked arrays are read by the copy engines directly; the call
 * returns once the arrays have been read. */
npgpu_status npgpu_apply_forces(npgpu_world* w, uint32_t n, const npgpu_handle* handles,
                                const float* forces6, int auto_wake_up);

/* DefaultJointConstraintSet::insert (joint_constraint.rs:54-72) of the joints
 * above (every joint constraint of the reference but the mouse constraint),
 * with the handles the host set gave them; inserting
 * wakes both bodies up at the next step (mechanical_world.rs:167-175). A
 * joint's impulses start at zero and persist across steps. The solver holds
 * the active joints beside the contact manifolds: capacity_pairs bounds the
 * manifolds plus the active joints of a step. */
npgpu_status npgpu_upsert_joints(npgpu_world* w, uint32_t n, const npgpu_handle* handles,
                                 const npgpu_joint_desc* descs);

/* DefaultJointConstraintSet::remove: wakes both bodies up at the next step
 * (mechanical_world.rs:156-165). Removing a body removes its joints
 * (mechanical_world.rs:141-154). */
npgpu_status npgpu_remove_joints(npgpu_world* w, uint32_t n, const npgpu_handle* handles);

/* The joints' impulses (what JointConstraint::cache_impulses keeps,
 * ball_constraint.rs:129-141, fixed_constraint.rs:174-199) and is_broken()
 * after the last completed step (synchronises the world's stream). */
npgpu_status npgpu_get_joints(npgpu_world* w, uint32_t n, const npgpu_handle* handles, npgpu_joint_state* out);

/* MechanicalWorld::step (mechanical_world.rs:182-396) run `nsteps` times,
 * asynchronously on the world's stream. `num_joints` / `num_force_generators`
 * are the sizes of the caller's sets: the joint count must equal the number
 * of joints mirrored into the world with npgpu_upsert_joints
 * (NONEMPTY_JOINTS otherwise), and a non-zero force-generator count is
 * rejected. */
npgpu_status npgpu_step(npgpu_world* w, uint32_t nsteps, uint32_t num_joints,
                        uint32_t num_force_generators);

/* Waits for the world's stream and reports any device-side error flag.
 * No counterpart in the reference: its step returns when done. */
npgpu_status npgpu_synchronize(npgpu_world* w);

/* Chooses the solver's launch shape for the current scene by timing real
 * steps: the one-grid schedule and, when the worlds qualify, the per-world
 * schedule with 64, 128 and 256 threads per world block (one candidate when
 * every world is solved by a thread-block cluster), each for 1 +
 * steps_per_candidate steps,
 * after one step with the automatic schedule that sizes the candidates.
 * Every candidate computes the same bits, so the world simply advances by
 * those steps. Sets params.solver_schedule and params.world_threads to the
 * fastest and reports them (any out pointer may be NULL). No counterpart in
 * the reference. */
npgpu_status npgpu_autotune(npgpu_world* w, uint32_t steps_per_candidate, uint32_t* schedule,
                            uint32_t* world_threads, float* ms_per_step);

/* Copies body state to host arrays indexed by slot (any pointer may be NULL):
 * position[7n], velocity[6n], energy[n] (activation energy), active[n]
 * (1 when awake), for slots [first, first + n). Waits for the world's
 * stream; page-locked arrays are written by the copy engines directly.
 * Replaces reading RigidBody::position / velocity
 * (src/object/rigid_body.rs:361-369) and Body::activation_status
 * (src/object/body.rs:181) after MechanicalWorld::step. */
npgpu_status npgpu_download_bodies(npgpu_world* w, uint32_t first, uint32_t n, float* position,
                                   float* velocity, float* energy, uint8_t* active);

/* The inertia the bodies carry after the colliders' mass was added:
 * local_inertia[7n] (mass, xx, xy, xz, yy, yz, zz) and local_com[3n].
 * Replaces Body::local_inertia / local_center_of_mass
 * (src/object/rigid_body.rs:913-930) once GeometricalWorld::maintain has
 * added the colliders' mass (src/world/geometrical_world.rs:102-227). */
npgpu_status npgpu_download_mass_properties(npgpu_world* w, uint32_t first, uint32_t n,
                                            float* local_inertia, float* local_com);

/* Broad-phase pairs as (collider1, collider2) with collider1 < collider2,
 * sorted ascending. *count receives the number of pairs; at most `max` are written.
 * Replaces the pair set of GeometricalWorld::perform_broad_phase
 * (src/world/geometrical_world.rs:285-312). */
npgpu_status npgpu_get_pairs(npgpu_world* w, uint32_t* pairs2, uint32_t max, uint32_t* count);

/* Fat AABBs (min xyz, max xyz) of colliders [first, first + n).
 * Replaces the broad-phase proxies' AABBs that
 * GeometricalWorld::sync_colliders updates
 * (src/world/geometrical_world.rs:230-265). */
npgpu_status npgpu_get_aabbs(npgpu_world* w, uint32_t first, uint32_t n, float* aabb6);

/* Contacts of every manifold, sorted by (collider1, collider2, feature_key).
 * Replaces GeometricalWorld::contact_pairs
 * (src/world/geometrical_world.rs:534-618) with each manifold's contacts and
 * the solver's impulses. */
npgpu_status npgpu_get_contacts(npgpu_world* w, npgpu_contact* out, uint32_t max,
                                uint32_t* count);

/* The last step's counters: replaces MechanicalWorld::counters
 * (src/world/mechanical_world.rs:57; src/counters/mod.rs:19). */
npgpu_status npgpu_get_counters(npgpu_world* w, npgpu_counters* out);

/* One-line description of the last failure on this world (or, when w is
 * NULL, of the calling thread's last failed npgpu_create /
 * npgpu_find_pairs_static; the string stays valid until that thread's next
 * such failure).
 * No counterpart in the reference, which panics or skips (try_ret! /
 * try_continue!, src/lib.rs:93-114). */
const char* npgpu_last_error(const npgpu_world* w);

/* ---- Geometric queries and contact events ----
 * The queries read the world as the last step left it: the broad phase's fat
 * AABBs and the colliders' poses of its final collision-detection pass, as
 * the reference's queries read its DBVT proxies and synced colliders.
 * `world` restricts a batch to one world of a batched world object
 * (0xffffffff: every world). Collision groups are not modelled: every
 * collider of the supported scenes has the default groups, which interact
 * with everything. Hits come sorted by (query, collider); *count receives the
 * number of hits and at most max_hits are written. */
typedef struct npgpu_ray_hit {
    uint32_t ray, collider;
    float toi;                       /* hit point = origin + toi * dir */
    float normal[3];                 /* outward surface normal; zero when the ray starts inside */
} npgpu_ray_hit;

/* GeometricalWorld::interferences_with_ray (src/world/geometrical_world.rs:327-341)
 * for n rays: rays6[6n] = origin, direction (not normalised), max_toi[n].
 * Shapes are solid: a ray starting inside a shape hits it at toi 0. */
npgpu_status npgpu_interferences_with_rays(npgpu_world* w, uint32_t n, const float* rays6, const float* max_toi,
                                           uint32_t world, npgpu_ray_hit* hits, uint32_t max_hits, uint32_t* count);
/* GeometricalWorld::interferences_with_point (geometrical_world.rs:343-355) for
 * n points: hits2[2k] = point index, hits2[2k + 1] = collider slot of each
 * collider whose shape contains the point (boundary included). */
npgpu_status npgpu_interferences_with_points(npgpu_world* w, uint32_t n, const float* points3, uint32_t world,
                                             uint32_t* hits2, uint32_t max_hits, uint32_t* count);
/* GeometricalWorld::interferences_with_aabb (geometrical_world.rs:357-370) for
 * n boxes (min xyz, max xyz): every collider whose broad-phase AABB
 * intersects the box; hits2 as above. */
npgpu_status npgpu_interferences_with_aabbs(npgpu_world* w, uint32_t n, const float* aabbs6, uint32_t world,
                                            uint32_t* hits2, uint32_t max_hits, uint32_t* count);

/* ContactEvent::Started / Stopped of the last step (stopped = 0 / 1). */
typedef struct npgpu_contact_event {
    uint32_t collider1, collider2;   /* collider1 < collider2 */
    uint32_t stopped;
} npgpu_contact_event;
/* Starts (capacity > 0) or stops (0) recording contact events: each step then
 * records, over its collision-detection passes, the pairs whose manifold
 * gains its first contact (started) or loses its last (stopped), as
 * GeometricalWorld::contact_events holds them after MechanicalWorld::step
 * (geometrical_world.rs:373-376, cleared at mechanical_world.rs:250). Pairs of
 * a removed or replaced collider give no event, as in the reference, whose
 * removal events are cleared before the step's first pass. */
npgpu_status npgpu_enable_contact_events(npgpu_world* w, uint32_t capacity);
/* The last step's contact events sorted by (collider1, collider2, stopped);
 * *count receives their number. NPGPU_ERR_CAPACITY if the step had more events
 * than the capacity (the first `capacity` recorded are returned).
 * Replaces GeometricalWorld::contact_events (geometrical_world.rs:373-376). */
npgpu_status npgpu_contact_events(npgpu_world* w, npgpu_contact_event* out, uint32_t max, uint32_t* count);

/* ncollide3d query::Proximity of a pair with a sensor. */
enum {
    NPGPU_PROXIMITY_INTERSECTING = 0,  /* the shapes touch or overlap */
    NPGPU_PROXIMITY_WITHIN_MARGIN = 1, /* apart by at most the pair's query limits */
    NPGPU_PROXIMITY_DISJOINT = 2
};
/* ProximityEvent: a pair with a sensor whose proximity changed in a
 * collision-detection pass of the last step. */
typedef struct npgpu_proximity_event {
    uint32_t collider1, collider2;   /* collider1 < collider2 */
    uint32_t prev_status, new_status;  /* NPGPU_PROXIMITY_* */
} npgpu_proximity_event;
/* The last step's proximity events (recorded with the contact events, into
 * the same capacity), by (collider1, collider2) and, for one pair, in the
 * order of the passes. A pair that leaves the broad phase goes to Disjoint.
 * Replaces GeometricalWorld::proximity_events (geometrical_world.rs:378-381). */
npgpu_status npgpu_proximity_events(npgpu_world* w, npgpu_proximity_event* out, uint32_t max, uint32_t* count);

/* Broad phase over caller-provided boxes that allocates nothing. This entry
 * point has no counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc (code running while a CUDA graph is captured,
 * real-time loops that must not block on the allocator, hosts whose device
 * memory belongs to another runtime's pool).
 *
 * Inputs (device memory): aabbs6[6n] = (min x, y, z, max x, y, z) per box;
 * groups[n] (or NULL): boxes pair only within the same group (< 65536).
 * Outputs (device memory): pairs2[2 * max_pairs] receives the pairs (i, j),
 * i < j, of boxes whose closed boxes intersect, in no particular order;
 * *count receives the number of pairs (only the first max_pairs are written),
 * or UINT32_MAX if a tree bound was hit. Work is queued on `stream` (a
 * cudaStream_t, NULL = default stream); results are ready when it completes.
 *
 * Limits: at most 32768 boxes per call (NPGPU_ERR_CAPACITY otherwise). The
 * scratch memory is one fixed 8 MiB __device__ array in the library, held on
 * every GPU that loads the library until the process exits. The first call on
 * a device (that device current) looks up the array's address; make it before
 * any stream capture. Calls share the array: calls whose work overlaps on the
 * GPU race. No call allocates or frees memory. */
npgpu_status npgpu_find_pairs_static(const float* aabbs6, const uint32_t* groups, uint32_t n, uint32_t* pairs2,
                                     uint32_t max_pairs, uint32_t* count, void* stream);

/* ---- Learned warm start (no counterpart in the reference) ----
 * A 24 -> 64 -> 64 -> 3 perceptron (ReLU, bf16 weights, fp32 accumulation)
 * predicts the starting impulses (normal, tangent 1, tangent 2) of contacts
 * that have no impulse-cache entry when params.warmstart_mode == 2, and of
 * every contact when it is 3. The warm-start sweep keeps a prediction only if
 * the contact's local residual is no larger than with the start it replaced
 * (the cached impulses, or zero), so the iteration count to a residual
 * tolerance stays the measure.
 *
 * Parameters (fp32, NPGPU_MLP_PARAMS floats): W1[64][24] b1[64] W2[64][64]
 * b2[64] W3[3][64] b3[3], then the normalisation x_mean[24] x_inv_std[24]
 * y_mean[3] y_std[3] (network input = (feature - mean) * inv_std; impulse =
 * output * y_std + y_mean). A training sample is NPGPU_MLP_SAMPLE_FLOATS
 * floats: the 24 features, the 3 converged impulses, and 1 if the contact had
 * no cache entry when it was assembled (else 0). */
#define NPGPU_MLP_PARAMS 6009u
#define NPGPU_MLP_TRAINABLE 5955u
#define NPGPU_MLP_SAMPLE_FLOATS 28u
#define NPGPU_MLP_INIT 1u      /* npgpu_mlp_train flag: new weights from the seed, normalisation from the samples */

/* Sets the network (n == NPGPU_MLP_PARAMS) and resets the optimiser state.
 * No counterpart in the reference (the learned warm start is this
 * library's). */
npgpu_status npgpu_mlp_set(npgpu_world* w, const float* params, uint32_t n);
/* Copies the network's fp32 parameters out (n >= NPGPU_MLP_PARAMS).
 * No counterpart in the reference. */
npgpu_status npgpu_mlp_get(npgpu_world* w, float* params, uint32_t n);
/* Records a training sample for every solver contact of the following steps
 * (features at assembly, impulses after the velocity solve) until `capacity`
 * samples are held; capacity 0 stops recording and keeps what was recorded. A
 * new capacity discards earlier samples.
 * No counterpart in the reference. */
npgpu_status npgpu_mlp_record(npgpu_world* w, uint32_t capacity);
/* Number of recorded samples, and up to max_samples of them when out != NULL.
 * No counterpart in the reference. */
npgpu_status npgpu_mlp_samples(npgpu_world* w, float* out, uint32_t max_samples, uint32_t* count);
/* Replaces the recorded samples with n host samples (NPGPU_MLP_SAMPLE_FLOATS
 * floats each, as npgpu_mlp_samples returns them) and stops recording: a
 * training set gathered from several worlds or runs trains one network.
 * No counterpart in the reference. */
npgpu_status npgpu_mlp_load_samples(npgpu_world* w, const float* samples, uint32_t n);
/* Trains on the recorded samples with Adam (lr, batch a multiple of 64):
 * `steps` batches drawn from the samples by a hash of (seed, step). With
 * NPGPU_MLP_INIT, or when no network is set yet, starts from He-uniform
 * weights drawn from `seed` and normalisation from the samples' statistics.
 * *final_loss (may be NULL) receives the last batch's loss.
 * No counterpart in the reference. */
npgpu_status npgpu_mlp_train(npgpu_world* w, uint32_t steps, uint32_t batch, float lr, uint32_t seed, uint32_t flags,
                             float* final_loss);
/* Loss and gradient (NPGPU_MLP_TRAINABLE floats, parameter layout above) of
 * the current network over n host samples, without updating it (n <= 65536).
 * No counterpart in the reference. */
npgpu_status npgpu_mlp_grad(npgpu_world* w, const float* samples, uint32_t n, float* grad, float* loss);

#ifdef __cplusplus
}
#endif

#endif /* NPGPU_H */
