//! `GpuMechanicalWorld`: the rigid-body step of nphysics3d 0.23 run on the GPU
//! through libnpgpu.so, with `DefaultMechanicalWorld::step`'s signature
//! (src/world/mechanical_world.rs:182-196 of nphysics).
//!
//! The Rust sets stay authoritative for handles. Each step forwards what
//! changed on the host (removed and new bodies and colliders, bodies whose
//! position or velocity the caller set, applied forces), runs `npgpu_step`,
//! and writes the new poses, velocities and activation back into the set, as
//! `MechanicalWorld::step` leaves them. Scenes the GPU step does not support
//! (multibodies, FEM or mass-spring bodies, shapes other than balls,
//! cuboids and capsules, sensors, CCD colliders, mouse constraints, force
//! generators) make `step` panic with the library's message, where nphysics
//! would have run them. Balls, cuboids and capsules are supported; the ten
//! joint constraints (ball, fixed, revolute, cartesian, planar, rectangular,
//! universal, prismatic, cylindrical, pin-slot) go in as `GpuJoint`s.
pub mod ffi;

use std::collections::HashMap;
use std::ffi::CStr;

use generational_arena::Index;
use nalgebra::{DVector, Isometry3, Point3, Quaternion, Translation3, Unit, UnitQuaternion, Vector3};
use ncollide3d::shape::{Ball, Capsule, Cuboid};
use nphysics3d::algebra::{Force3, ForceType, Velocity3};
use nphysics3d::force_generator::ForceGeneratorSet;
use nphysics3d::joint::{BallConstraint, CartesianConstraint, CylindricalConstraint, DefaultJointConstraintHandle,
                        FixedConstraint, JointConstraint, JointConstraintSet, PinSlotConstraint, PlanarConstraint,
                        PrismaticConstraint, RectangularConstraint, RevoluteConstraint, UniversalConstraint};
use nphysics3d::material::{BasicMaterial, MaterialCombineMode};
use nphysics3d::object::{Body, BodyPartHandle, BodySet, BodyStatus, Collider, ColliderSet, DefaultBodyHandle,
                         DefaultColliderHandle, Ground, RigidBody};
use nphysics3d::solver::{GenericNonlinearConstraint, IntegrationParameters, LinearConstraints,
                         NonlinearConstraintGenerator};
use nphysics3d::world::GeometricalWorld;

fn handle(i: Index) -> ffi::npgpu_handle {
    let (index, generation) = i.into_raw_parts();
    ffi::npgpu_handle { index: index as u64, generation }
}

fn iso7(p: &Isometry3<f32>) -> [f32; 7] {
    let t = p.translation.vector;
    let q = p.rotation.quaternion().coords; // (i, j, k, w)
    [t.x, t.y, t.z, q.x, q.y, q.z, q.w]
}

fn combine(m: MaterialCombineMode) -> u32 {
    match m {
        MaterialCombineMode::Average => 0,
        MaterialCombineMode::Min => 1,
        MaterialCombineMode::Multiply => 2,
        MaterialCombineMode::Max => 3,
        _ => 0,
    }
}

/// Panics with the library's one-line message unless `st` is NPGPU_OK.
fn assert_ok(st: i32, w: *const ffi::npgpu_world) {
    if st != ffi::NPGPU_OK {
        let msg = unsafe { CStr::from_ptr(ffi::npgpu_last_error(w)) }.to_string_lossy().into_owned();
        panic!("GPU step failed (status {}): {}", st, msg);
    }
}

/// Body descriptor of a rigid body or a ground (RigidBodyDesc::build,
/// src/object/rigid_body.rs:1064-1084). Any other body kind is forwarded with
/// its kind, and the library rejects it.
fn body_desc(body: &dyn Body<f32>) -> ffi::npgpu_body_desc {
    let mut d = ffi::npgpu_body_desc::default();
    d.status = match body.status() {
        BodyStatus::Disabled => 0,
        BodyStatus::Static => ffi::NPGPU_BODY_STATIC,
        BodyStatus::Dynamic => ffi::NPGPU_BODY_DYNAMIC,
        BodyStatus::Kinematic => ffi::NPGPU_BODY_KINEMATIC,
    };
    if let Some(rb) = body.downcast_ref::<RigidBody<f32>>() {
        d.kind = ffi::NPGPU_KIND_RIGID_BODY;
        d.position = iso7(rb.position());
        let v = rb.velocity();
        d.velocity = [v.linear.x, v.linear.y, v.linear.z, v.angular.x, v.angular.y, v.angular.z];
        let inertia = rb.local_inertia();
        let a = inertia.angular;
        d.local_inertia = [inertia.linear, a[(0, 0)], a[(0, 1)], a[(0, 2)], a[(1, 1)], a[(1, 2)], a[(2, 2)]];
        let c = rb.local_center_of_mass();
        d.local_com = [c.x, c.y, c.z];
        d.linear_damping = rb.linear_damping();
        d.angular_damping = rb.angular_damping();
        d.max_linear_velocity = rb.max_linear_velocity();
        d.max_angular_velocity = rb.max_angular_velocity();
        if rb.gravity_enabled() {
            d.flags |= ffi::NPGPU_BODY_GRAVITY;
        }
        let (lt, lr) = (rb.kinematic_translations(), rb.kinematic_rotations());
        for k in 0..3 {
            if lt[k] {
                d.flags |= ffi::NPGPU_BODY_LOCK_TX << k;
            }
            if lr[k] {
                d.flags |= ffi::NPGPU_BODY_LOCK_RX << k;
            }
        }
        if let Some(thr) = rb.activation_status().deactivation_threshold() {
            d.flags |= ffi::NPGPU_BODY_CAN_SLEEP;
            d.sleep_threshold = thr;
        }
        if rb.linear_motion_interpolation_enabled() {
            d.flags |= ffi::NPGPU_BODY_LINEAR_INTERP;
        }
    } else if body.downcast_ref::<Ground<f32>>().is_some() {
        d.kind = ffi::NPGPU_KIND_GROUND;
        d.position = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0];
        d.max_linear_velocity = f32::MAX;
        d.max_angular_velocity = f32::MAX;
    } else {
        d.kind = ffi::NPGPU_KIND_MULTIBODY; // FEM, mass-spring and multibodies are all rejected
    }
    d
}

/// Collider descriptor (ColliderDesc::build, src/object/collider.rs:538-572).
fn collider_desc(c: &Collider<f32, DefaultBodyHandle>) -> ffi::npgpu_collider_desc {
    let mut d = ffi::npgpu_collider_desc::default();
    d.body = handle(c.body());
    d.position_wrt_body = iso7(&c.position_wrt_body());
    d.margin = c.margin();
    d.density = c.density();
    // ColliderDesc's defaults (collider.rs:457-458); the query type keeps them.
    d.linear_prediction = 0.001;
    d.angular_prediction = std::f32::consts::PI / 180.0 * 5.0;
    if let Some(m) = c.material().downcast_ref::<BasicMaterial<f32>>() {
        d.friction = m.friction;
        d.restitution = m.restitution;
        d.friction_combine = combine(m.friction_combine_mode);
        d.restitution_combine = combine(m.restitution_combine_mode);
    }
    let shape = c.shape();
    if let Some(b) = shape.as_shape::<Ball<f32>>() {
        d.shape = ffi::NPGPU_SHAPE_BALL;
        d.shape_params = [b.radius, 0.0, 0.0];
    } else if let Some(b) = shape.as_shape::<Cuboid<f32>>() {
        d.shape = ffi::NPGPU_SHAPE_CUBOID;
        d.shape_params = [b.half_extents.x, b.half_extents.y, b.half_extents.z];
    } else if let Some(c) = shape.as_shape::<Capsule<f32>>() {
        d.shape = ffi::NPGPU_SHAPE_CAPSULE;
        d.shape_params = [c.radius, c.half_height, 0.0];
    } else {
        d.shape = ffi::NPGPU_SHAPE_OTHER;
    }
    d.is_sensor = c.is_sensor() as u32;
    d.ccd_enabled = c.is_ccd_enabled() as u32;
    d
}

/// A joint the GPU world can forward: ball, fixed, revolute, cartesian,
/// planar, rectangular or universal. nphysics keeps its constraints' anchors,
/// axes and frames private, so this type builds the reference's constraint
/// and records its description beside it; it implements JointConstraint by
/// delegating to that constraint, so the same set still steps on the CPU.
/// Insert it into a DefaultJointConstraintSet as usual.
pub struct GpuJoint {
    inner: Box<dyn JointConstraint<f32, DefaultBodyHandle>>,
    desc: ffi::npgpu_joint_desc,
    gpu: ffi::npgpu_joint_state,
}

fn quat4(q: &UnitQuaternion<f32>) -> [f32; 4] {
    let c = q.quaternion().coords; // (i, j, k, w)
    [c.x, c.y, c.z, c.w]
}

fn v3a(v: &Vector3<f32>) -> [f32; 3] {
    [v.x, v.y, v.z]
}

type Part = BodyPartHandle<DefaultBodyHandle>;

/// set_break_force / set_break_torque on whichever constraint `inner` holds.
macro_rules! on_inner {
    ($inner:expr, $x:ident => $body:expr, $($t:ty),*) => {
        $(if let Some($x) = $inner.downcast_mut::<$t>() { $body; })*
    };
}

impl GpuJoint {
    fn with(kind: u32, b1: Part, b2: Part, anchor1: &Point3<f32>, anchor2: &Point3<f32>,
            inner: Box<dyn JointConstraint<f32, DefaultBodyHandle>>) -> Self {
        let mut desc = ffi::npgpu_joint_desc::default();
        desc.kind = kind;
        desc.body1 = handle(b1.0);
        desc.body2 = handle(b2.0);
        desc.anchor1 = [anchor1.x, anchor1.y, anchor1.z];
        desc.anchor2 = [anchor2.x, anchor2.y, anchor2.z];
        desc.frame1 = [0.0, 0.0, 0.0, 1.0];
        desc.frame2 = [0.0, 0.0, 0.0, 1.0];
        desc.axis1 = [1.0, 0.0, 0.0];
        desc.axis2 = [1.0, 0.0, 0.0];
        desc.break_force = f32::MAX;
        desc.break_torque = f32::MAX;
        GpuJoint { inner, desc, gpu: ffi::npgpu_joint_state::default() }
    }

    /// BallConstraint::new (src/joint/ball_constraint.rs:26-48).
    pub fn ball(b1: Part, b2: Part, anchor1: Point3<f32>, anchor2: Point3<f32>) -> Self {
        Self::with(ffi::NPGPU_JOINT_BALL, b1, b2, &anchor1, &anchor2,
                   Box::new(BallConstraint::new(b1, b2, anchor1, anchor2)))
    }

    /// FixedConstraint::new (src/joint/fixed_constraint.rs:35-58).
    pub fn fixed(b1: Part, b2: Part, anchor1: Point3<f32>, ref_frame1: UnitQuaternion<f32>, anchor2: Point3<f32>,
                 ref_frame2: UnitQuaternion<f32>) -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_FIXED, b1, b2, &anchor1, &anchor2,
                               Box::new(FixedConstraint::new(b1, b2, anchor1, ref_frame1, anchor2, ref_frame2)));
        j.desc.frame1 = quat4(&ref_frame1);
        j.desc.frame2 = quat4(&ref_frame2);
        j
    }

    /// RevoluteConstraint::new (src/joint/revolute_constraint.rs:52-80).
    pub fn revolute(b1: Part, b2: Part, anchor1: Point3<f32>, axis1: Unit<Vector3<f32>>, anchor2: Point3<f32>,
                    axis2: Unit<Vector3<f32>>) -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_REVOLUTE, b1, b2, &anchor1, &anchor2,
                               Box::new(RevoluteConstraint::new(b1, b2, anchor1, axis1, anchor2, axis2)));
        j.desc.axis1 = v3a(&axis1);
        j.desc.axis2 = v3a(&axis2);
        j
    }

    /// CartesianConstraint::new (src/joint/cartesian_constraint.rs).
    pub fn cartesian(b1: Part, b2: Part, anchor1: Point3<f32>, ref_frame1: UnitQuaternion<f32>, anchor2: Point3<f32>,
                     ref_frame2: UnitQuaternion<f32>) -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_CARTESIAN, b1, b2, &anchor1, &anchor2,
                               Box::new(CartesianConstraint::new(b1, b2, anchor1, ref_frame1, anchor2, ref_frame2)));
        j.desc.frame1 = quat4(&ref_frame1);
        j.desc.frame2 = quat4(&ref_frame2);
        j
    }

    /// PlanarConstraint::new (src/joint/planar_constraint.rs).
    pub fn planar(b1: Part, b2: Part, anchor1: Point3<f32>, axis1: Unit<Vector3<f32>>, anchor2: Point3<f32>,
                  axis2: Unit<Vector3<f32>>) -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_PLANAR, b1, b2, &anchor1, &anchor2,
                               Box::new(PlanarConstraint::new(b1, b2, anchor1, axis1, anchor2, axis2)));
        j.desc.axis1 = v3a(&axis1);
        j.desc.axis2 = v3a(&axis2);
        j
    }

    /// RectangularConstraint::new (src/joint/rectangular_constraint.rs).
    pub fn rectangular(b1: Part, b2: Part, anchor1: Point3<f32>, axis1: Unit<Vector3<f32>>, anchor2: Point3<f32>)
                       -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_RECTANGULAR, b1, b2, &anchor1, &anchor2,
                               Box::new(RectangularConstraint::new(b1, b2, anchor1, axis1, anchor2)));
        j.desc.axis1 = v3a(&axis1);
        j
    }

    /// UniversalConstraint::new (src/joint/universal_constraint.rs).
    pub fn universal(b1: Part, b2: Part, anchor1: Point3<f32>, axis1: Unit<Vector3<f32>>, anchor2: Point3<f32>,
                     axis2: Unit<Vector3<f32>>, angle: f32) -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_UNIVERSAL, b1, b2, &anchor1, &anchor2,
                               Box::new(UniversalConstraint::new(b1, b2, anchor1, axis1, anchor2, axis2, angle)));
        j.desc.axis1 = v3a(&axis1);
        j.desc.axis2 = v3a(&axis2);
        j.desc.angle = angle;
        j
    }

    /// PrismaticConstraint::new (src/joint/prismatic_constraint.rs:30-56);
    /// `enable_min_offset` / `enable_max_offset` set its limits.
    pub fn prismatic(b1: Part, b2: Part, anchor1: Point3<f32>, axis1: Unit<Vector3<f32>>, anchor2: Point3<f32>)
                     -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_PRISMATIC, b1, b2, &anchor1, &anchor2,
                               Box::new(PrismaticConstraint::new(b1, b2, anchor1, axis1, anchor2)));
        j.desc.axis1 = v3a(&axis1);
        j
    }

    /// PrismaticConstraint::enable_min_offset / enable_max_offset.
    pub fn enable_min_offset(&mut self, limit: f32) {
        self.desc.min_offset = limit;
        self.desc.limit_flags |= ffi::NPGPU_JOINT_MIN_OFFSET;
        on_inner!(self.inner, x => x.enable_min_offset(limit), PrismaticConstraint<f32, DefaultBodyHandle>);
    }
    pub fn enable_max_offset(&mut self, limit: f32) {
        self.desc.max_offset = limit;
        self.desc.limit_flags |= ffi::NPGPU_JOINT_MAX_OFFSET;
        on_inner!(self.inner, x => x.enable_max_offset(limit), PrismaticConstraint<f32, DefaultBodyHandle>);
    }

    /// CylindricalConstraint::new (src/joint/cylindrical_constraint.rs).
    pub fn cylindrical(b1: Part, b2: Part, anchor1: Point3<f32>, axis1: Unit<Vector3<f32>>, anchor2: Point3<f32>,
                       axis2: Unit<Vector3<f32>>) -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_CYLINDRICAL, b1, b2, &anchor1, &anchor2,
                               Box::new(CylindricalConstraint::new(b1, b2, anchor1, axis1, anchor2, axis2)));
        j.desc.axis1 = v3a(&axis1);
        j.desc.axis2 = v3a(&axis2);
        j
    }

    /// PinSlotConstraint::new (src/joint/pin_slot_constraint.rs).
    pub fn pin_slot(b1: Part, b2: Part, anchor1: Point3<f32>, axis_v1: Unit<Vector3<f32>>,
                    axis_w1: Unit<Vector3<f32>>, anchor2: Point3<f32>, axis_w2: Unit<Vector3<f32>>) -> Self {
        let mut j = Self::with(ffi::NPGPU_JOINT_PIN_SLOT, b1, b2, &anchor1, &anchor2,
                               Box::new(PinSlotConstraint::new(b1, b2, anchor1, axis_v1, axis_w1, anchor2, axis_w2)));
        j.desc.axis1 = v3a(&axis_v1);
        j.desc.axis3 = v3a(&axis_w1);
        j.desc.axis2 = v3a(&axis_w2);
        j
    }

    /// set_break_force of the constraint.
    pub fn set_break_force(&mut self, f: f32) {
        self.desc.break_force = f;
        on_inner!(self.inner, x => x.set_break_force(f), BallConstraint<f32, DefaultBodyHandle>,
                  FixedConstraint<f32, DefaultBodyHandle>, RevoluteConstraint<f32, DefaultBodyHandle>,
                  PlanarConstraint<f32, DefaultBodyHandle>, RectangularConstraint<f32, DefaultBodyHandle>,
                  UniversalConstraint<f32, DefaultBodyHandle>, PrismaticConstraint<f32, DefaultBodyHandle>,
                  CylindricalConstraint<f32, DefaultBodyHandle>, PinSlotConstraint<f32, DefaultBodyHandle>);
    }

    /// set_break_torque of the constraint (every kind but the ball joint).
    pub fn set_break_torque(&mut self, t: f32) {
        self.desc.break_torque = t;
        on_inner!(self.inner, x => x.set_break_torque(t), FixedConstraint<f32, DefaultBodyHandle>,
                  RevoluteConstraint<f32, DefaultBodyHandle>, CartesianConstraint<f32, DefaultBodyHandle>,
                  PlanarConstraint<f32, DefaultBodyHandle>, RectangularConstraint<f32, DefaultBodyHandle>,
                  UniversalConstraint<f32, DefaultBodyHandle>, PrismaticConstraint<f32, DefaultBodyHandle>,
                  CylindricalConstraint<f32, DefaultBodyHandle>, PinSlotConstraint<f32, DefaultBodyHandle>);
    }

    /// The impulses the GPU step cached for this joint (linear, then angular).
    pub fn impulses(&self) -> [f32; 6] {
        self.gpu.impulses
    }

    /// The prismatic limit's impulse of the last GPU step.
    pub fn limit_impulse(&self) -> f32 {
        self.gpu.limit_impulse
    }
}

impl NonlinearConstraintGenerator<f32, DefaultBodyHandle> for GpuJoint {
    fn num_position_constraints(&self, bodies: &dyn BodySet<f32, Handle = DefaultBodyHandle>) -> usize {
        self.inner.num_position_constraints(bodies)
    }
    fn position_constraint(&self, parameters: &IntegrationParameters<f32>, i: usize,
                           bodies: &mut dyn BodySet<f32, Handle = DefaultBodyHandle>, jacobians: &mut [f32])
                           -> Option<GenericNonlinearConstraint<f32, DefaultBodyHandle>> {
        self.inner.position_constraint(parameters, i, bodies, jacobians)
    }
}

impl JointConstraint<f32, DefaultBodyHandle> for GpuJoint {
    fn num_velocity_constraints(&self) -> usize {
        self.inner.num_velocity_constraints()
    }
    fn anchors(&self) -> (BodyPartHandle<DefaultBodyHandle>, BodyPartHandle<DefaultBodyHandle>) {
        self.inner.anchors()
    }
    fn velocity_constraints(&mut self, parameters: &IntegrationParameters<f32>,
                            bodies: &dyn BodySet<f32, Handle = DefaultBodyHandle>, ext_vels: &DVector<f32>,
                            ground_j_id: &mut usize, j_id: &mut usize, jacobians: &mut [f32],
                            velocity_constraints: &mut LinearConstraints<f32, usize>) {
        self.inner.velocity_constraints(parameters, bodies, ext_vels, ground_j_id, j_id, jacobians,
                                        velocity_constraints)
    }
    fn cache_impulses(&mut self, constraints: &LinearConstraints<f32, usize>, inv_dt: f32) {
        self.inner.cache_impulses(constraints, inv_dt)
    }
    fn is_broken(&self) -> bool {
        self.gpu.broken != 0 || self.inner.is_broken()
    }
}

/// Number of elements of a joint or force-generator set (they have no `len`).
fn count_joints<C: JointConstraintSet<f32, DefaultBodyHandle, Handle = DefaultJointConstraintHandle>>(set: &C) -> u32 {
    let mut n = 0u32;
    set.foreach(|_, _| n += 1);
    n
}

fn count_forces<F: ForceGeneratorSet<f32, DefaultBodyHandle>>(set: &F) -> u32 {
    let mut n = 0u32;
    set.foreach(|_, _| n += 1);
    n
}

pub struct GpuMechanicalWorld {
    raw: *mut ffi::npgpu_world,
    /// IntegrationParameters (npgpu_default_params = IntegrationParameters::default()).
    pub integration_parameters: ffi::npgpu_params,
    /// Body, collider and joint slots the device holds, with their generation.
    bodies_on_device: HashMap<u64, u64>,
    colliders_on_device: HashMap<u64, u64>,
    joints_on_device: HashMap<u64, u64>,
    /// Scratch arrays of the per-step exchange, reused across steps.
    upserts: (Vec<ffi::npgpu_handle>, Vec<ffi::npgpu_body_desc>),
    forces: (Vec<ffi::npgpu_handle>, Vec<f32>),
    poses: Vec<f32>,
    vels: Vec<f32>,
    active: Vec<u8>,
}

impl GpuMechanicalWorld {
    /// MechanicalWorld::new(gravity) (mechanical_world.rs:76-99) with room for
    /// `capacity_bodies` bodies and `capacity_colliders` colliders.
    pub fn new(gravity: Vector3<f32>, capacity_bodies: u32, capacity_colliders: u32) -> Self {
        let mut p = ffi::npgpu_params::default();
        unsafe { ffi::npgpu_default_params(&mut p) };
        let g = [gravity.x, gravity.y, gravity.z];
        let mut st = 0;
        let raw = unsafe {
            ffi::npgpu_create(&p, g.as_ptr(), capacity_bodies, capacity_colliders, 16 * capacity_colliders, &mut st)
        };
        assert_ok(st, std::ptr::null());
        GpuMechanicalWorld {
            raw,
            integration_parameters: p,
            bodies_on_device: HashMap::new(),
            colliders_on_device: HashMap::new(),
            joints_on_device: HashMap::new(),
            upserts: (Vec::new(), Vec::new()),
            forces: (Vec::new(), Vec::new()),
            poses: Vec::new(),
            vels: Vec::new(),
            active: Vec::new(),
        }
    }

    /// MechanicalWorld::step: same generic signature.
    pub fn step<Bodies, Colliders, Constraints, Forces>(
        &mut self,
        _gworld: &mut GeometricalWorld<f32, DefaultBodyHandle, DefaultColliderHandle>,
        bodies: &mut Bodies,
        colliders: &mut Colliders,
        constraints: &mut Constraints,
        forces: &mut Forces,
    ) where
        Bodies: BodySet<f32, Handle = DefaultBodyHandle>,
        Colliders: ColliderSet<f32, DefaultBodyHandle, Handle = DefaultColliderHandle>,
        Constraints: JointConstraintSet<f32, DefaultBodyHandle, Handle = DefaultJointConstraintHandle>,
        Forces: ForceGeneratorSet<f32, DefaultBodyHandle>,
    {
        assert_ok(unsafe { ffi::npgpu_set_params(self.raw, &self.integration_parameters) }, self.raw);
        self.forward_events(bodies, colliders);
        self.forward_joints(constraints);
        let (nj, nf) = (count_joints(constraints), count_forces(forces));
        assert_ok(unsafe { ffi::npgpu_step(self.raw, 1, nj, nf) }, self.raw);
        assert_ok(unsafe { ffi::npgpu_synchronize(self.raw) }, self.raw);
        self.write_back_poses(bodies);
        self.write_back_joints(constraints);
    }

    /// The joint set's removals and insertions (mechanical_world.rs:156-175).
    /// A joint that is not a GpuJoint goes in as an unknown kind, which the
    /// library rejects.
    fn forward_joints<Constraints>(&mut self, constraints: &mut Constraints)
    where
        Constraints: JointConstraintSet<f32, DefaultBodyHandle, Handle = DefaultJointConstraintHandle>,
    {
        let mut removed = Vec::new();
        while let Some((h, _, _)) = constraints.pop_removal_event() {
            if self.joints_on_device.remove(&(h.into_raw_parts().0 as u64)).is_some() {
                removed.push(handle(h));
            }
        }
        if !removed.is_empty() {
            let st = unsafe { ffi::npgpu_remove_joints(self.raw, removed.len() as u32, removed.as_ptr()) };
            assert_ok(st, self.raw);
        }
        let (mut jh, mut jd) = (Vec::new(), Vec::new());
        while let Some((h, _, _)) = constraints.pop_insertion_event() {
            if let Some(j) = constraints.get(h) {
                let desc = match j.downcast_ref::<GpuJoint>() {
                    Some(g) => g.desc,
                    None => ffi::npgpu_joint_desc { kind: u32::MAX, ..Default::default() },
                };
                jh.push(handle(h));
                jd.push(desc);
                let (index, generation) = h.into_raw_parts();
                self.joints_on_device.insert(index as u64, generation);
            }
        }
        if !jh.is_empty() {
            let st = unsafe { ffi::npgpu_upsert_joints(self.raw, jh.len() as u32, jh.as_ptr(), jd.as_ptr()) };
            assert_ok(st, self.raw);
        }
    }

    /// JointConstraint::cache_impulses / is_broken as the step left them.
    fn write_back_joints<Constraints>(&mut self, constraints: &mut Constraints)
    where
        Constraints: JointConstraintSet<f32, DefaultBodyHandle, Handle = DefaultJointConstraintHandle>,
    {
        let mut hs = Vec::new();
        constraints.foreach(|h, _| hs.push(h));
        if hs.is_empty() {
            return;
        }
        let raw: Vec<ffi::npgpu_handle> = hs.iter().map(|h| handle(*h)).collect();
        let mut st = vec![ffi::npgpu_joint_state::default(); raw.len()];
        assert_ok(unsafe { ffi::npgpu_get_joints(self.raw, raw.len() as u32, raw.as_ptr(), st.as_mut_ptr()) },
                  self.raw);
        for (h, s) in hs.iter().zip(st.iter()) {
            if let Some(g) = constraints.get_mut(*h).and_then(|j| j.downcast_mut::<GpuJoint>()) {
                g.gpu = *s;
            }
        }
    }

    /// MechanicalWorld::maintain (mechanical_world.rs:114-179) as the device
    /// sees it: removals first (a removed body takes its colliders with it),
    /// then new or edited bodies, new colliders, and the bodies' accumulated
    /// external forces.
    fn forward_events<Bodies, Colliders>(&mut self, bodies: &mut Bodies, colliders: &mut Colliders)
    where
        Bodies: BodySet<f32, Handle = DefaultBodyHandle>,
        Colliders: ColliderSet<f32, DefaultBodyHandle, Handle = DefaultColliderHandle>,
    {
        let mut removed = Vec::new();
        while let Some(h) = bodies.pop_removal_event() {
            if self.bodies_on_device.remove(&(h.into_raw_parts().0 as u64)).is_some() {
                removed.push(handle(h));
            }
        }
        if !removed.is_empty() {
            let st = unsafe { ffi::npgpu_remove_bodies(self.raw, removed.len() as u32, removed.as_ptr()) };
            assert_ok(st, self.raw);
        }
        let mut removed = Vec::new();
        while let Some((h, _)) = colliders.pop_removal_event() {
            if self.colliders_on_device.remove(&(h.into_raw_parts().0 as u64)).is_some() {
                removed.push(handle(h));
            }
        }
        if !removed.is_empty() {
            let st = unsafe { ffi::npgpu_remove_colliders(self.raw, removed.len() as u32, removed.as_ptr()) };
            assert_ok(st, self.raw);
        }

        // Bodies the device does not hold yet, or whose state the caller set
        // since the last step (BodyUpdateStatus, src/object/body.rs:11-47).
        let (hs, ds) = (&mut self.upserts.0, &mut self.upserts.1);
        hs.clear();
        ds.clear();
        let (fh, fv) = (&mut self.forces.0, &mut self.forces.1);
        fh.clear();
        fv.clear();
        let known = &mut self.bodies_on_device;
        bodies.foreach(&mut |h: DefaultBodyHandle, b: &dyn Body<f32>| {
            let (index, generation) = h.into_raw_parts();
            let fresh = known.get(&(index as u64)) != Some(&generation);
            let st = b.update_status();
            if fresh || st.position_changed() || st.velocity_changed() || st.status_changed() {
                hs.push(handle(h));
                ds.push(body_desc(b));
                known.insert(index as u64, generation);
            }
            if let Some(rb) = b.downcast_ref::<RigidBody<f32>>() {
                let f = rb.external_forces();
                if f.linear != Vector3::zeros() || f.angular != Vector3::zeros() {
                    fh.push(handle(h));
                    fv.extend_from_slice(&[f.linear.x, f.linear.y, f.linear.z, f.angular.x, f.angular.y,
                                           f.angular.z]);
                }
            }
        });
        if !hs.is_empty() {
            let st = unsafe { ffi::npgpu_upsert_bodies(self.raw, hs.len() as u32, hs.as_ptr(), ds.as_ptr()) };
            assert_ok(st, self.raw);
        }

        let mut ch = Vec::new();
        let mut cd = Vec::new();
        while let Some(h) = colliders.pop_insertion_event() {
            if let Some(c) = colliders.get(h) {
                ch.push(handle(h));
                cd.push(collider_desc(c));
                let (index, generation) = h.into_raw_parts();
                self.colliders_on_device.insert(index as u64, generation);
            }
        }
        if !ch.is_empty() {
            let st = unsafe { ffi::npgpu_upsert_colliders(self.raw, ch.len() as u32, ch.as_ptr(), cd.as_ptr()) };
            assert_ok(st, self.raw);
        }
        if !fh.is_empty() {
            // The forces were accumulated with apply_force(.., auto_wake_up) on
            // the host, which already woke the body: no second wake-up here.
            let st = unsafe { ffi::npgpu_apply_forces(self.raw, fh.len() as u32, fh.as_ptr(), fv.as_ptr(), 0) };
            assert_ok(st, self.raw);
        }
    }

    /// Poses, velocities and activation back into the set after the step, as
    /// RigidBody::integrate and ActivationManager leave them
    /// (src/object/rigid_body.rs:467-505, src/detection/activation_manager.rs:61-201).
    fn write_back_poses<Bodies>(&mut self, bodies: &mut Bodies)
    where
        Bodies: BodySet<f32, Handle = DefaultBodyHandle>,
    {
        let slots = self.bodies_on_device.keys().copied().max().map_or(0, |m| m + 1) as usize;
        self.poses.resize(7 * slots, 0.0);
        self.vels.resize(6 * slots, 0.0);
        self.active.resize(slots, 0);
        let st = unsafe {
            ffi::npgpu_download_bodies(self.raw, 0, slots as u32, self.poses.as_mut_ptr(), self.vels.as_mut_ptr(),
                                       std::ptr::null_mut(), self.active.as_mut_ptr())
        };
        assert_ok(st, self.raw);
        let (poses, vels, active) = (&self.poses, &self.vels, &self.active);
        bodies.foreach_mut(&mut |h: DefaultBodyHandle, b: &mut dyn Body<f32>| {
            let i = h.into_raw_parts().0;
            if i >= active.len() {
                return;
            }
            if let Some(rb) = b.downcast_mut::<RigidBody<f32>>() {
                if rb.status() != BodyStatus::Dynamic && rb.status() != BodyStatus::Kinematic {
                    return;
                }
                let p = &poses[7 * i..7 * i + 7];
                let q = UnitQuaternion::new_unchecked(Quaternion::new(p[6], p[3], p[4], p[5]));
                rb.set_position(Isometry3::from_parts(Translation3::new(p[0], p[1], p[2]), q));
                let v = &vels[6 * i..6 * i + 6];
                rb.set_velocity(Velocity3::new(Vector3::new(v[0], v[1], v[2]), Vector3::new(v[3], v[4], v[5])));
                if active[i] == 0 {
                    rb.deactivate();
                }
                rb.clear_forces();
                rb.clear_update_flags();
            }
        });
    }

    /// Applies a force the way RigidBody::apply_force does, for callers that
    /// keep forces off the host bodies (src/object/rigid_body.rs:771-820).
    pub fn apply_force(&mut self, body: DefaultBodyHandle, force: &Force3<f32>, _kind: ForceType, wake: bool) {
        let h = [handle(body)];
        let f = [force.linear.x, force.linear.y, force.linear.z, force.angular.x, force.angular.y, force.angular.z];
        assert_ok(unsafe { ffi::npgpu_apply_forces(self.raw, 1, h.as_ptr(), f.as_ptr(), wake as i32) }, self.raw);
    }

    /// GeometricalWorld::interferences_with_ray (geometrical_world.rs:327-341)
    /// for one ray: (collider slot, time of impact, normal) of every hit.
    pub fn interferences_with_ray(&mut self, origin: &Vector3<f32>, dir: &Vector3<f32>, max_toi: f32)
                                  -> Vec<(u32, f32, Vector3<f32>)> {
        let ray = [origin.x, origin.y, origin.z, dir.x, dir.y, dir.z];
        let mut n = 0u32;
        assert_ok(unsafe {
            ffi::npgpu_interferences_with_rays(self.raw, 1, ray.as_ptr(), &max_toi, u32::MAX,
                                               std::ptr::null_mut(), 0, &mut n)
        }, self.raw);
        let mut hits = vec![ffi::npgpu_ray_hit::default(); n as usize];
        assert_ok(unsafe {
            ffi::npgpu_interferences_with_rays(self.raw, 1, ray.as_ptr(), &max_toi, u32::MAX, hits.as_mut_ptr(),
                                               n, &mut n)
        }, self.raw);
        hits.iter().map(|h| (h.collider, h.toi, Vector3::new(h.normal[0], h.normal[1], h.normal[2]))).collect()
    }

    /// GeometricalWorld::contact_events (geometrical_world.rs:373-376) of the
    /// last step as (collider1, collider2, stopped); `enable_contact_events`
    /// first.
    pub fn enable_contact_events(&mut self, capacity: u32) {
        assert_ok(unsafe { ffi::npgpu_enable_contact_events(self.raw, capacity) }, self.raw);
    }
    pub fn contact_events(&mut self) -> Vec<(u32, u32, bool)> {
        let mut n = 0u32;
        assert_ok(unsafe { ffi::npgpu_contact_events(self.raw, std::ptr::null_mut(), 0, &mut n) }, self.raw);
        let mut ev = vec![ffi::npgpu_contact_event::default(); n as usize];
        assert_ok(unsafe { ffi::npgpu_contact_events(self.raw, ev.as_mut_ptr(), n, &mut n) }, self.raw);
        ev.iter().map(|e| (e.collider1, e.collider2, e.stopped != 0)).collect()
    }

    /// MechanicalWorld::counters (mechanical_world.rs:57).
    pub fn counters(&self) -> ffi::npgpu_counters {
        let mut c = ffi::npgpu_counters::default();
        assert_ok(unsafe { ffi::npgpu_get_counters(self.raw, &mut c) }, self.raw);
        c
    }
}

impl Drop for GpuMechanicalWorld {
    fn drop(&mut self) {
        unsafe { ffi::npgpu_destroy(self.raw) };
    }
}
