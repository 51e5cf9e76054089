//! Raw bindings to include/npgpu.h (libnpgpu.so). Struct layouts mirror the
//! C declarations field for field; tests/test_abi.py checks that every
//! function the header declares has a declaration here.
#![allow(non_camel_case_types)]
use std::os::raw::{c_char, c_int, c_void};

pub const NPGPU_OK: c_int = 0;
pub const NPGPU_BODY_STATIC: u32 = 1;
pub const NPGPU_BODY_DYNAMIC: u32 = 2;
pub const NPGPU_BODY_KINEMATIC: u32 = 3;
pub const NPGPU_KIND_RIGID_BODY: u32 = 0;
pub const NPGPU_KIND_GROUND: u32 = 1;
pub const NPGPU_KIND_MULTIBODY: u32 = 2;
pub const NPGPU_BODY_GRAVITY: u32 = 1 << 0;
pub const NPGPU_BODY_LOCK_TX: u32 = 1 << 1;
pub const NPGPU_BODY_LOCK_RX: u32 = 1 << 4;
pub const NPGPU_BODY_CAN_SLEEP: u32 = 1 << 7;
pub const NPGPU_BODY_LINEAR_INTERP: u32 = 1 << 8;
pub const NPGPU_SHAPE_BALL: u32 = 0;
pub const NPGPU_SHAPE_CUBOID: u32 = 1;
pub const NPGPU_SHAPE_OTHER: u32 = 2;
pub const NPGPU_SHAPE_CAPSULE: u32 = 3;
pub const NPGPU_SWEEP_SEPARATE: u32 = 0;
pub const NPGPU_SWEEP_MANIFOLD: u32 = 1;

#[repr(C)]
#[derive(Copy, Clone, Default, Debug, PartialEq, Eq, Hash)]
pub struct npgpu_handle {
    pub index: u64,
    pub generation: u64,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_body_desc {
    pub position: [f32; 7],
    pub velocity: [f32; 6],
    pub local_inertia: [f32; 7],
    pub local_com: [f32; 3],
    pub linear_damping: f32,
    pub angular_damping: f32,
    pub max_linear_velocity: f32,
    pub max_angular_velocity: f32,
    pub sleep_threshold: f32,
    pub status: u32,
    pub kind: u32,
    pub flags: u32,
    pub world: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_collider_desc {
    pub body: npgpu_handle,
    pub position_wrt_body: [f32; 7],
    pub shape_params: [f32; 3],
    pub margin: f32,
    pub density: f32,
    pub linear_prediction: f32,
    pub angular_prediction: f32,
    pub friction: f32,
    pub restitution: f32,
    pub friction_combine: u32,
    pub restitution_combine: u32,
    pub shape: u32,
    pub is_sensor: u32,
    pub ccd_enabled: u32,
}

pub const NPGPU_JOINT_BALL: u32 = 0;
pub const NPGPU_JOINT_FIXED: u32 = 1;
pub const NPGPU_JOINT_REVOLUTE: u32 = 2;
pub const NPGPU_JOINT_CARTESIAN: u32 = 3;
pub const NPGPU_JOINT_PLANAR: u32 = 4;
pub const NPGPU_JOINT_RECTANGULAR: u32 = 5;
pub const NPGPU_JOINT_UNIVERSAL: u32 = 6;
pub const NPGPU_JOINT_PRISMATIC: u32 = 7;
pub const NPGPU_JOINT_CYLINDRICAL: u32 = 8;
pub const NPGPU_JOINT_PIN_SLOT: u32 = 9;
pub const NPGPU_JOINT_MIN_OFFSET: u32 = 1;
pub const NPGPU_JOINT_MAX_OFFSET: u32 = 2;

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_joint_desc {
    pub kind: u32,
    pub pad: u32,
    pub body1: npgpu_handle,
    pub body2: npgpu_handle,
    pub anchor1: [f32; 3],
    pub anchor2: [f32; 3],
    pub frame1: [f32; 4],
    pub frame2: [f32; 4],
    pub break_force: f32,
    pub break_torque: f32,
    pub axis1: [f32; 3],
    pub axis2: [f32; 3],
    pub angle: f32,
    pub limit_flags: u32,
    pub axis3: [f32; 3],
    pub min_offset: f32,
    pub max_offset: f32,
    pub pad2: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_joint_state {
    pub impulses: [f32; 6],
    pub limit_impulse: f32,
    pub broken: u32,
    pub active: u32,
    pub pad: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_params {
    pub dt: f32,
    pub erp: f32,
    pub warmstart_coeff: f32,
    pub restitution_velocity_threshold: f32,
    pub allowed_linear_error: f32,
    pub allowed_angular_error: f32,
    pub max_linear_correction: f32,
    pub max_angular_correction: f32,
    pub max_stabilization_multiplier: f32,
    pub max_velocity_iterations: u32,
    pub max_position_iterations: u32,
    pub max_ccd_position_iterations: u32,
    pub max_ccd_substeps: u32,
    pub solve_to_tolerance: u32,
    pub residual_tolerance: f32,
    pub max_iterations_to_tolerance: u32,
    pub warmstart_mode: u32,
    pub broad_phase_margin: f32,
    pub activation_mix: f32,
    pub profile: u32,
    pub solver_schedule: u32,
    pub use_graph: u32,
    pub world_threads: u32,
    pub sweep_order: u32,
    pub ccd_on_penetration_enabled: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_contact {
    pub collider1: u32,
    pub collider2: u32,
    pub feature_key: u32,
    pub kinematic: u32,
    pub world1: [f32; 3],
    pub world2: [f32; 3],
    pub normal: [f32; 3],
    pub depth: f32,
    pub impulse: [f32; 3],
    pub colour: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_counters {
    pub step_time: f64,
    pub collision_detection_time: f64,
    pub broad_phase_time: f64,
    pub narrow_phase_time: f64,
    pub island_construction_time: f64,
    pub solver_time: f64,
    pub assembly_time: f64,
    pub velocity_resolution_time: f64,
    pub velocity_update_time: f64,
    pub position_resolution_time: f64,
    pub colouring_time: f64,
    pub steps: u64,
    pub num_pairs: u32,
    pub num_manifolds: u32,
    pub num_contacts: u32,
    pub num_solver_contacts: u32,
    pub num_constraints: u32,
    pub num_colours: u32,
    pub num_active_bodies: u32,
    pub velocity_iterations: u32,
    pub residual: f64,
    pub residual_initial: f64,
    pub max_penetration: f64,
    pub kinetic_energy: f64,
    pub velocity_task_ms: f64,
    pub velocity_wait_ms: f64,
    pub velocity_kernel_ms: f64,
    pub velocity_tasks: u64,
    pub learned_starts: u32,
    pub learned_kept: u32,
    pub graph_replay: u32,
    pub ccd_substeps: u32,
    pub ccd_impacts: u32,
    pub reserved: u32,
    pub ccd_toi_computation_time: f64,
    pub ccd_solver_time: f64,
    pub ccd_broad_phase_time: f64,
    pub ccd_narrow_phase_time: f64,
    pub ccd_world_time_max: f64,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_ray_hit {
    pub ray: u32,
    pub collider: u32,
    pub toi: f32,
    pub normal: [f32; 3],
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_contact_event {
    pub collider1: u32,
    pub collider2: u32,
    pub stopped: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct npgpu_proximity_event {
    pub collider1: u32,
    pub collider2: u32,
    pub prev_status: u32,
    pub new_status: u32,
}

/// Opaque world handle (`npgpu_world*`).
pub enum npgpu_world {}

#[link(name = "npgpu")]
extern "C" {
    pub fn npgpu_abi_version() -> u32;
    pub fn npgpu_default_params(out: *mut npgpu_params);
    pub fn npgpu_create(p: *const npgpu_params, gravity: *const f32, cap_b: u32, cap_c: u32, cap_p: u32,
                        status: *mut c_int) -> *mut npgpu_world;
    pub fn npgpu_destroy(w: *mut npgpu_world);
    pub fn npgpu_stream(w: *mut npgpu_world) -> *mut c_void;
    pub fn npgpu_set_params(w: *mut npgpu_world, p: *const npgpu_params) -> c_int;
    pub fn npgpu_set_gravity(w: *mut npgpu_world, gravity: *const f32) -> c_int;
    pub fn npgpu_upsert_bodies(w: *mut npgpu_world, n: u32, h: *const npgpu_handle,
                               d: *const npgpu_body_desc) -> c_int;
    pub fn npgpu_upsert_colliders(w: *mut npgpu_world, n: u32, h: *const npgpu_handle,
                                  d: *const npgpu_collider_desc) -> c_int;
    pub fn npgpu_remove_bodies(w: *mut npgpu_world, n: u32, h: *const npgpu_handle) -> c_int;
    pub fn npgpu_remove_colliders(w: *mut npgpu_world, n: u32, h: *const npgpu_handle) -> c_int;
    pub fn npgpu_apply_forces(w: *mut npgpu_world, n: u32, h: *const npgpu_handle, f: *const f32,
                              wake: c_int) -> c_int;
    pub fn npgpu_upsert_joints(w: *mut npgpu_world, n: u32, h: *const npgpu_handle,
                               d: *const npgpu_joint_desc) -> c_int;
    pub fn npgpu_remove_joints(w: *mut npgpu_world, n: u32, h: *const npgpu_handle) -> c_int;
    pub fn npgpu_get_joints(w: *mut npgpu_world, n: u32, h: *const npgpu_handle,
                            out: *mut npgpu_joint_state) -> c_int;
    pub fn npgpu_step(w: *mut npgpu_world, nsteps: u32, num_joints: u32, num_forces: u32) -> c_int;
    pub fn npgpu_synchronize(w: *mut npgpu_world) -> c_int;
    pub fn npgpu_autotune(w: *mut npgpu_world, steps_per_candidate: u32, schedule: *mut u32,
                          world_threads: *mut u32, ms_per_step: *mut f32) -> c_int;
    pub fn npgpu_download_bodies(w: *mut npgpu_world, first: u32, n: u32, pos: *mut f32, vel: *mut f32,
                                 energy: *mut f32, active: *mut u8) -> c_int;
    pub fn npgpu_download_mass_properties(w: *mut npgpu_world, first: u32, n: u32, local_inertia: *mut f32,
                                          local_com: *mut f32) -> c_int;
    pub fn npgpu_get_pairs(w: *mut npgpu_world, pairs2: *mut u32, max: u32, count: *mut u32) -> c_int;
    pub fn npgpu_get_aabbs(w: *mut npgpu_world, first: u32, n: u32, aabb6: *mut f32) -> c_int;
    pub fn npgpu_get_contacts(w: *mut npgpu_world, out: *mut npgpu_contact, max: u32, count: *mut u32) -> c_int;
    pub fn npgpu_get_counters(w: *mut npgpu_world, out: *mut npgpu_counters) -> c_int;
    pub fn npgpu_last_error(w: *const npgpu_world) -> *const c_char;
    pub fn npgpu_find_pairs_static(aabbs6: *const f32, groups: *const u32, n: u32, pairs2: *mut u32,
                                   max_pairs: u32, count: *mut u32, stream: *mut c_void) -> c_int;
    pub fn npgpu_interferences_with_rays(w: *mut npgpu_world, n: u32, rays6: *const f32, max_toi: *const f32,
                                         world: u32, hits: *mut npgpu_ray_hit, max_hits: u32,
                                         count: *mut u32) -> c_int;
    pub fn npgpu_interferences_with_points(w: *mut npgpu_world, n: u32, points3: *const f32, world: u32,
                                           hits2: *mut u32, max_hits: u32, count: *mut u32) -> c_int;
    pub fn npgpu_interferences_with_aabbs(w: *mut npgpu_world, n: u32, aabbs6: *const f32, world: u32,
                                          hits2: *mut u32, max_hits: u32, count: *mut u32) -> c_int;
    pub fn npgpu_enable_contact_events(w: *mut npgpu_world, capacity: u32) -> c_int;
    pub fn npgpu_contact_events(w: *mut npgpu_world, out: *mut npgpu_contact_event, max: u32,
                                count: *mut u32) -> c_int;
    pub fn npgpu_proximity_events(w: *mut npgpu_world, out: *mut npgpu_proximity_event, max: u32,
                                  count: *mut u32) -> c_int;
    pub fn npgpu_mlp_set(w: *mut npgpu_world, params: *const f32, n: u32) -> c_int;
    pub fn npgpu_mlp_get(w: *mut npgpu_world, params: *mut f32, n: u32) -> c_int;
    pub fn npgpu_mlp_record(w: *mut npgpu_world, capacity: u32) -> c_int;
    pub fn npgpu_mlp_samples(w: *mut npgpu_world, out: *mut f32, max: u32, count: *mut u32) -> c_int;
    pub fn npgpu_mlp_load_samples(w: *mut npgpu_world, samples: *const f32, n: u32) -> c_int;
    pub fn npgpu_mlp_train(w: *mut npgpu_world, steps: u32, batch: u32, lr: f32, seed: u32, flags: u32,
                           final_loss: *mut f32) -> c_int;
    pub fn npgpu_mlp_grad(w: *mut npgpu_world, samples: *const f32, n: u32, grad: *mut f32,
                          loss: *mut f32) -> c_int;
}
