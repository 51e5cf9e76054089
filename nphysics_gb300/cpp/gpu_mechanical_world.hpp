// gpu_mechanical_world.hpp -- C++ host mirror of nphysics3d's world API over
// the GPU step (include/npgpu.h).
//
// A drop-in for code written against DefaultMechanicalWorld
// (src/world/mechanical_world.rs:24, 182-396): the same set types, handle
// semantics and `step(gworld, bodies, colliders, joints, forces)` call, with
// the step running on the GPU. Sets are generational arenas
// (generational_arena::Index, src/object/body_set.rs:178) whose slot indices
// are the device slots. Insertions, removals and user edits are forwarded to
// the device on the next step (the reference's `maintain`,
// mechanical_world.rs:114-179); after the step the bodies' poses and
// velocities are copied back into the set.
//
// Header-only; link against libnpgpu.so. Errors throw nphysics_gpu::Error
// carrying the npgpu_status (the reference panics or silently skips).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <variant>
#include <vector>

#include "../../include/npgpu.h"

namespace nphysics_gpu {

struct Error : std::runtime_error {
    npgpu_status status;
    Error(npgpu_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

struct Vector3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
};

// Isometry3: translation + unit quaternion (i, j, k, w).
struct Isometry3 {
    Vector3 translation;
    float rotation[4] = {0.0f, 0.0f, 0.0f, 1.0f};
    static Isometry3 identity() { return Isometry3(); }
    static Isometry3 from_translation(float x, float y, float z) {
        Isometry3 r;
        r.translation = {x, y, z};
        return r;
    }
    // UnitQuaternion::from_scaled_axis.
    static Isometry3 new_(Vector3 t, Vector3 axisangle) {
        Isometry3 r;
        r.translation = t;
        double n = std::sqrt(double(axisangle.x) * axisangle.x + double(axisangle.y) * axisangle.y +
                             double(axisangle.z) * axisangle.z);
        if (n > 0.0) {
            double s = std::sin(0.5 * n) / n;
            r.rotation[0] = float(axisangle.x * s);
            r.rotation[1] = float(axisangle.y * s);
            r.rotation[2] = float(axisangle.z * s);
            r.rotation[3] = float(std::cos(0.5 * n));
        }
        return r;
    }
};

struct Velocity3 {
    Vector3 linear, angular;
};

enum class BodyStatus : uint32_t {
    Disabled = NPGPU_BODY_DISABLED,
    Static = NPGPU_BODY_STATIC,
    Dynamic = NPGPU_BODY_DYNAMIC,
    Kinematic = NPGPU_BODY_KINEMATIC
};

// generational_arena::Index.
struct Index {
    uint64_t index = 0, generation = 0;
    bool operator==(const Index& o) const { return index == o.index && generation == o.generation; }
    npgpu_handle raw() const { return npgpu_handle{index, generation}; }
};
using DefaultBodyHandle = Index;
using DefaultColliderHandle = Index;
struct BodyPartHandle {
    DefaultBodyHandle body;
    size_t part = 0;
};

// Arena with generation bumps on removal and LIFO slot reuse (generational_arena 0.2).
template <class T> class Arena {
public:
    Index insert(T value) {
        Index h;
        if (!free_.empty()) {
            h.index = free_.back();
            free_.pop_back();
            slots_[h.index].emplace(std::move(value));
        } else {
            h.index = slots_.size();
            slots_.emplace_back(std::move(value));
            gens_.push_back(0);
        }
        h.generation = generation_;
        gens_[h.index] = generation_;
        return h;
    }
    std::optional<T> remove(Index h) {
        if (!contains(h)) return std::nullopt;
        std::optional<T> out = std::move(slots_[h.index]);
        slots_[h.index].reset();
        free_.push_back(h.index);
        ++generation_;
        return out;
    }
    bool contains(Index h) const {
        return h.index < slots_.size() && slots_[h.index].has_value() && gens_[h.index] == h.generation;
    }
    T* get(Index h) { return contains(h) ? &*slots_[h.index] : nullptr; }
    const T* get(Index h) const { return contains(h) ? &*slots_[h.index] : nullptr; }
    Index handle_at(size_t i) const { return Index{i, gens_[i]}; }
    bool occupied(size_t i) const { return i < slots_.size() && slots_[i].has_value(); }
    size_t capacity_used() const { return slots_.size(); }

private:
    std::vector<std::optional<T>> slots_;
    std::vector<uint64_t> gens_;
    std::vector<uint64_t> free_;
    uint64_t generation_ = 0;
};

// A rigid body as built by RigidBodyDesc::build (src/object/rigid_body.rs:1064-1084).
class RigidBody {
public:
    npgpu_body_desc desc;

    RigidBody() {
        std::memset(&desc, 0, sizeof(desc));
        desc.position[6] = 1.0f;
        desc.max_linear_velocity = std::numeric_limits<float>::max();
        desc.max_angular_velocity = std::numeric_limits<float>::max();
        desc.sleep_threshold = 0.01f;
        desc.status = NPGPU_BODY_DYNAMIC;
        desc.kind = NPGPU_KIND_RIGID_BODY;
        desc.flags = NPGPU_BODY_GRAVITY | NPGPU_BODY_CAN_SLEEP;
    }
    Isometry3 position() const {
        Isometry3 r;
        r.translation = {desc.position[0], desc.position[1], desc.position[2]};
        for (int k = 0; k < 4; ++k) r.rotation[k] = desc.position[3 + k];
        return r;
    }
    Velocity3 velocity() const {
        return Velocity3{{desc.velocity[0], desc.velocity[1], desc.velocity[2]},
                         {desc.velocity[3], desc.velocity[4], desc.velocity[5]}};
    }
    BodyStatus status() const { return BodyStatus(desc.status); }
    bool is_active() const { return active_; }
    // Setters mark the body changed: it is re-uploaded (and woken) on the next step.
    void set_position(const Isometry3& p) {
        desc.position[0] = p.translation.x;
        desc.position[1] = p.translation.y;
        desc.position[2] = p.translation.z;
        for (int k = 0; k < 4; ++k) desc.position[3 + k] = p.rotation[k];
        dirty_ = true;
    }
    void set_velocity(const Velocity3& v) {
        float a[6] = {v.linear.x, v.linear.y, v.linear.z, v.angular.x, v.angular.y, v.angular.z};
        std::memcpy(desc.velocity, a, sizeof(a));
        dirty_ = true;
    }
    void set_status(BodyStatus s) {
        desc.status = uint32_t(s);
        dirty_ = true;
    }
    // RigidBody::apply_force(0, force, ForceType::Force, auto_wake_up).
    void apply_force(const Velocity3& f, bool auto_wake_up) {
        float a[6] = {f.linear.x, f.linear.y, f.linear.z, f.angular.x, f.angular.y, f.angular.z};
        for (int k = 0; k < 6; ++k) force_.v[k] += a[k];
        force_.wake = force_.wake || auto_wake_up;
        force_.any = true;
    }

    struct Force {
        float v[6] = {0, 0, 0, 0, 0, 0};
        bool wake = false, any = false;
    };

private:
    friend class GpuMechanicalWorld;
    Force force_;
    bool dirty_ = true;
    bool active_ = true;
};

// RigidBodyDesc builder (src/object/rigid_body.rs:949-1086).
class RigidBodyDesc {
public:
    RigidBodyDesc& translation(Vector3 t) {
        b_.desc.position[0] = t.x;
        b_.desc.position[1] = t.y;
        b_.desc.position[2] = t.z;
        return *this;
    }
    RigidBodyDesc& rotation(Vector3 axisangle) {
        Isometry3 r = Isometry3::new_({}, axisangle);
        for (int k = 0; k < 4; ++k) b_.desc.position[3 + k] = r.rotation[k];
        return *this;
    }
    RigidBodyDesc& position(const Isometry3& p) {
        b_.set_position(p);
        return *this;
    }
    RigidBodyDesc& velocity(const Velocity3& v) {
        b_.set_velocity(v);
        return *this;
    }
    RigidBodyDesc& status(BodyStatus s) {
        b_.desc.status = uint32_t(s);
        return *this;
    }
    RigidBodyDesc& mass(float m) {
        b_.desc.local_inertia[0] = m;
        return *this;
    }
    RigidBodyDesc& gravity_enabled(bool on) {
        b_.desc.flags = on ? (b_.desc.flags | NPGPU_BODY_GRAVITY) : (b_.desc.flags & ~NPGPU_BODY_GRAVITY);
        return *this;
    }
    RigidBodyDesc& linear_damping(float d) {
        b_.desc.linear_damping = d;
        return *this;
    }
    RigidBodyDesc& angular_damping(float d) {
        b_.desc.angular_damping = d;
        return *this;
    }
    RigidBodyDesc& max_linear_velocity(float v) {
        b_.desc.max_linear_velocity = v;
        return *this;
    }
    RigidBodyDesc& max_angular_velocity(float v) {
        b_.desc.max_angular_velocity = v;
        return *this;
    }
    // None disables sleeping.
    RigidBodyDesc& sleep_threshold(std::optional<float> t) {
        if (t) {
            b_.desc.sleep_threshold = *t;
            b_.desc.flags |= NPGPU_BODY_CAN_SLEEP;
        } else {
            b_.desc.flags &= ~NPGPU_BODY_CAN_SLEEP;
        }
        return *this;
    }
    RigidBodyDesc& kinematic_translations(bool x, bool y, bool z) {
        set_flag(NPGPU_BODY_LOCK_TX, x);
        set_flag(NPGPU_BODY_LOCK_TY, y);
        set_flag(NPGPU_BODY_LOCK_TZ, z);
        return *this;
    }
    RigidBodyDesc& kinematic_rotations(bool x, bool y, bool z) {
        set_flag(NPGPU_BODY_LOCK_RX, x);
        set_flag(NPGPU_BODY_LOCK_RY, y);
        set_flag(NPGPU_BODY_LOCK_RZ, z);
        return *this;
    }
    RigidBody build() const { return b_; }

private:
    void set_flag(uint32_t f, bool on) { b_.desc.flags = on ? (b_.desc.flags | f) : (b_.desc.flags & ~f); }
    RigidBody b_;
};

// Ground::new() (src/object/ground.rs): a static body with no dofs.
struct Ground {};

// A body of a kind the GPU world rejects (multibody, FEM, mass-spring...): it
// can sit in the set, and the step reports NPGPU_ERR_UNSUPPORTED_BODY.
struct UnsupportedBody {
    uint32_t kind;
};

using BodyVariant = std::variant<RigidBody, Ground, UnsupportedBody>;

class DefaultBodySet {
public:
    DefaultBodyHandle insert(BodyVariant b) {
        DefaultBodyHandle h = arena_.insert(std::move(b));
        inserted_.push_back(h);
        return h;
    }
    std::optional<BodyVariant> remove(DefaultBodyHandle h) {
        auto r = arena_.remove(h);
        if (r) removed_.push_back(h);
        return r;
    }
    RigidBody* rigid_body(DefaultBodyHandle h) {
        BodyVariant* v = arena_.get(h);
        return v ? std::get_if<RigidBody>(v) : nullptr;
    }
    const RigidBody* rigid_body(DefaultBodyHandle h) const {
        const BodyVariant* v = arena_.get(h);
        return v ? std::get_if<RigidBody>(v) : nullptr;
    }
    bool contains(DefaultBodyHandle h) const { return arena_.contains(h); }

private:
    friend class GpuMechanicalWorld;
    Arena<BodyVariant> arena_;
    std::vector<DefaultBodyHandle> inserted_, removed_;
};

enum class Shape { Ball, Cuboid };

struct BasicMaterial {
    float restitution = 0.0f, friction = 0.5f;   // basic_material.rs:59-63
    uint32_t restitution_combine = NPGPU_COMBINE_AVERAGE, friction_combine = NPGPU_COMBINE_AVERAGE;
};

class Collider {
public:
    npgpu_collider_desc desc;
    DefaultBodyHandle body() const { return DefaultBodyHandle{desc.body.index, desc.body.generation}; }
};

// ColliderDesc builder (src/object/collider.rs:441-573).
class ColliderDesc {
public:
    static ColliderDesc ball(float radius) { return ColliderDesc(NPGPU_SHAPE_BALL, radius, 0.0f, 0.0f); }
    static ColliderDesc cuboid(Vector3 half) { return ColliderDesc(NPGPU_SHAPE_CUBOID, half.x, half.y, half.z); }
    // ColliderDesc::new(ShapeHandle::new(Capsule::new(half_height, radius))): axis along local y.
    static ColliderDesc capsule(float half_height, float radius) {
        return ColliderDesc(NPGPU_SHAPE_CAPSULE, radius, half_height, 0.0f);
    }
    static ColliderDesc other_shape() { return ColliderDesc(NPGPU_SHAPE_OTHER, 0.0f, 0.0f, 0.0f); }
    ColliderDesc& translation(Vector3 t) {
        d_.position_wrt_body[0] = t.x;
        d_.position_wrt_body[1] = t.y;
        d_.position_wrt_body[2] = t.z;
        return *this;
    }
    ColliderDesc& rotation(Vector3 axisangle) {
        Isometry3 r = Isometry3::new_({}, axisangle);
        for (int k = 0; k < 4; ++k) d_.position_wrt_body[3 + k] = r.rotation[k];
        return *this;
    }
    ColliderDesc& density(float v) {
        d_.density = v;
        return *this;
    }
    ColliderDesc& margin(float v) {
        d_.margin = v;
        return *this;
    }
    ColliderDesc& linear_prediction(float v) {
        d_.linear_prediction = v;
        return *this;
    }
    ColliderDesc& material(const BasicMaterial& m) {
        d_.friction = m.friction;
        d_.restitution = m.restitution;
        d_.friction_combine = m.friction_combine;
        d_.restitution_combine = m.restitution_combine;
        return *this;
    }
    ColliderDesc& sensor(bool s) {
        d_.is_sensor = s;
        return *this;
    }
    ColliderDesc& ccd_enabled(bool s) {
        d_.ccd_enabled = s;
        return *this;
    }
    Collider build(BodyPartHandle parent) const {
        Collider c;
        c.desc = d_;
        c.desc.body = parent.body.raw();
        return c;
    }

private:
    ColliderDesc(uint32_t shape, float a, float b, float c) {
        std::memset(&d_, 0, sizeof(d_));
        d_.position_wrt_body[6] = 1.0f;
        d_.shape = shape;
        d_.shape_params[0] = a;
        d_.shape_params[1] = b;
        d_.shape_params[2] = c;
        d_.margin = 0.01f;
        d_.linear_prediction = 0.001f;
        d_.angular_prediction = 3.14159265358979323846f / 180.0f * 5.0f;
        d_.friction = 0.5f;
    }
    npgpu_collider_desc d_;
};

class DefaultColliderSet {
public:
    DefaultColliderHandle insert(Collider c) {
        DefaultColliderHandle h = arena_.insert(std::move(c));
        inserted_.push_back(h);
        return h;
    }
    std::optional<Collider> remove(DefaultColliderHandle h) {
        auto r = arena_.remove(h);
        if (r) removed_.push_back(h);
        return r;
    }
    const Collider* get(DefaultColliderHandle h) const { return arena_.get(h); }

private:
    friend class GpuMechanicalWorld;
    Arena<Collider> arena_;
    std::vector<DefaultColliderHandle> inserted_, removed_;
};

// The collision state lives on the device; this type exists for the signature.
class DefaultGeometricalWorld {};

// What every joint constraint below keeps: its description, and the state
// the GPU step leaves (JointConstraint::is_broken, the cached impulses).
class JointConstraintBase {
public:
    void set_break_force(float f) { desc.break_force = f; }
    void set_break_torque(float t) { desc.break_torque = t; }
    bool is_broken() const { return broken_; }
    // The impulses cache_impulses kept in the last step: linear, then angular,
    // then a prismatic limit's.
    const float* impulses() const { return impulses_; }
    npgpu_joint_desc desc;

protected:
    JointConstraintBase(uint32_t kind, BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 anchor2) {
        std::memset(&desc, 0, sizeof(desc));
        desc.kind = kind;
        desc.body1 = b1.body.raw();
        desc.body2 = b2.body.raw();
        set3(desc.anchor1, anchor1);
        set3(desc.anchor2, anchor2);
        desc.frame1[3] = desc.frame2[3] = 1.0f;
        desc.axis1[0] = desc.axis2[0] = desc.axis3[0] = 1.0f;
        desc.break_force = desc.break_torque = std::numeric_limits<float>::max();
    }
    static void set3(float* o, Vector3 v) {
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
    }
    // UnitQuaternion::from_scaled_axis.
    static void set_frame(float* o, Vector3 scaled_axis) {
        Isometry3 f = Isometry3::new_({}, scaled_axis);
        std::memcpy(o, f.rotation, 4 * sizeof(float));
    }

private:
    friend class GpuMechanicalWorld;
    bool broken_ = false;
    float impulses_[7] = {0, 0, 0, 0, 0, 0, 0};
};

// BallConstraint::new(b1, b2, anchor1, anchor2) (src/joint/ball_constraint.rs:26-48):
// keeps the two anchors (in their bodies' frames) together.
class BallConstraint : public JointConstraintBase {
public:
    BallConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 anchor2)
        : JointConstraintBase(NPGPU_JOINT_BALL, b1, b2, anchor1, anchor2) {}
};

// FixedConstraint::new(b1, b2, anchor1, ref_frame1, anchor2, ref_frame2)
// (src/joint/fixed_constraint.rs:35-58): also keeps the frames (body rotation
// times reference frame) aligned. Reference frames are scaled axes.
class FixedConstraint : public JointConstraintBase {
public:
    FixedConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 ref_frame1, Vector3 anchor2,
                    Vector3 ref_frame2)
        : JointConstraintBase(NPGPU_JOINT_FIXED, b1, b2, anchor1, anchor2) {
        set_frame(desc.frame1, ref_frame1);
        set_frame(desc.frame2, ref_frame2);
    }
};

// RevoluteConstraint::new(b1, b2, anchor1, axis1, anchor2, axis2)
// (src/joint/revolute_constraint.rs:52-80): a hinge about axis1 = axis2.
class RevoluteConstraint : public JointConstraintBase {
public:
    RevoluteConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 axis1, Vector3 anchor2,
                       Vector3 axis2)
        : JointConstraintBase(NPGPU_JOINT_REVOLUTE, b1, b2, anchor1, anchor2) {
        set3(desc.axis1, axis1);
        set3(desc.axis2, axis2);
    }
};

// CartesianConstraint::new(b1, b2, anchor1, ref_frame1, anchor2, ref_frame2):
// keeps the frames aligned, the translation free.
class CartesianConstraint : public JointConstraintBase {
public:
    CartesianConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 ref_frame1, Vector3 anchor2,
                        Vector3 ref_frame2)
        : JointConstraintBase(NPGPU_JOINT_CARTESIAN, b1, b2, anchor1, anchor2) {
        set_frame(desc.frame1, ref_frame1);
        set_frame(desc.frame2, ref_frame2);
    }
};

// PlanarConstraint::new(b1, b2, anchor1, axis1, anchor2, axis2): anchor2 in
// the plane through anchor1 normal to axis1, the axes aligned.
class PlanarConstraint : public JointConstraintBase {
public:
    PlanarConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 axis1, Vector3 anchor2,
                     Vector3 axis2)
        : JointConstraintBase(NPGPU_JOINT_PLANAR, b1, b2, anchor1, anchor2) {
        set3(desc.axis1, axis1);
        set3(desc.axis2, axis2);
    }
};

// RectangularConstraint::new(b1, b2, anchor1, axis1, anchor2): anchor2 in
// that plane, the rotations equal.
class RectangularConstraint : public JointConstraintBase {
public:
    RectangularConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 axis1, Vector3 anchor2)
        : JointConstraintBase(NPGPU_JOINT_RECTANGULAR, b1, b2, anchor1, anchor2) {
        set3(desc.axis1, axis1);
    }
};

// UniversalConstraint::new(b1, b2, anchor1, axis1, anchor2, axis2, angle):
// the anchors together, the angle between the axes kept.
class UniversalConstraint : public JointConstraintBase {
public:
    UniversalConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 axis1, Vector3 anchor2,
                        Vector3 axis2, float angle)
        : JointConstraintBase(NPGPU_JOINT_UNIVERSAL, b1, b2, anchor1, anchor2) {
        set3(desc.axis1, axis1);
        set3(desc.axis2, axis2);
        desc.angle = angle;
    }
};

// PrismaticConstraint::new(b1, b2, anchor1, axis1, anchor2)
// (src/joint/prismatic_constraint.rs:30-56): anchor2 slides along axis1, the
// rotations equal, within the optional offset limits.
class PrismaticConstraint : public JointConstraintBase {
public:
    PrismaticConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 axis1, Vector3 anchor2)
        : JointConstraintBase(NPGPU_JOINT_PRISMATIC, b1, b2, anchor1, anchor2) {
        set3(desc.axis1, axis1);
    }
    void enable_min_offset(float limit) {
        desc.min_offset = limit;
        desc.limit_flags |= NPGPU_JOINT_MIN_OFFSET;
    }
    void enable_max_offset(float limit) {
        desc.max_offset = limit;
        desc.limit_flags |= NPGPU_JOINT_MAX_OFFSET;
    }
    void disable_min_offset() { desc.limit_flags &= ~uint32_t(NPGPU_JOINT_MIN_OFFSET); }
    void disable_max_offset() { desc.limit_flags &= ~uint32_t(NPGPU_JOINT_MAX_OFFSET); }
};

// CylindricalConstraint::new(b1, b2, anchor1, axis1, anchor2, axis2): slides
// along and turns about axis1 = axis2.
class CylindricalConstraint : public JointConstraintBase {
public:
    CylindricalConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 axis1, Vector3 anchor2,
                          Vector3 axis2)
        : JointConstraintBase(NPGPU_JOINT_CYLINDRICAL, b1, b2, anchor1, anchor2) {
        set3(desc.axis1, axis1);
        set3(desc.axis2, axis2);
    }
};

// PinSlotConstraint::new(b1, b2, anchor1, axis_v1, axis_w1, anchor2, axis_w2):
// slides along axis_v1, turns about axis_w1 = axis_w2.
class PinSlotConstraint : public JointConstraintBase {
public:
    PinSlotConstraint(BodyPartHandle b1, BodyPartHandle b2, Vector3 anchor1, Vector3 axis_v1, Vector3 axis_w1,
                      Vector3 anchor2, Vector3 axis_w2)
        : JointConstraintBase(NPGPU_JOINT_PIN_SLOT, b1, b2, anchor1, anchor2) {
        set3(desc.axis1, axis_v1);
        set3(desc.axis3, axis_w1);
        set3(desc.axis2, axis_w2);
    }
};

using JointConstraint = std::variant<BallConstraint, FixedConstraint, RevoluteConstraint, CartesianConstraint,
                                     PlanarConstraint, RectangularConstraint, UniversalConstraint,
                                     PrismaticConstraint, CylindricalConstraint, PinSlotConstraint>;
using DefaultJointConstraintHandle = Index;

// DefaultJointConstraintSet (src/joint/joint_constraint.rs:31-130): the
// joints live on the host with their handles; the step forwards insertions
// and removals and reads the impulses and broken flags back.
class DefaultJointConstraintSet {
public:
    DefaultJointConstraintHandle insert(JointConstraint j) {
        DefaultJointConstraintHandle h = arena_.insert(std::move(j));
        inserted_.push_back(h);
        ++n_;
        return h;
    }
    std::optional<JointConstraint> remove(DefaultJointConstraintHandle h) {
        auto r = arena_.remove(h);
        if (r) {
            removed_.push_back(h);
            --n_;
        }
        return r;
    }
    JointConstraint* get(DefaultJointConstraintHandle h) { return arena_.get(h); }
    bool contains(DefaultJointConstraintHandle h) const { return arena_.contains(h); }
    size_t len() const { return n_; }

private:
    friend class GpuMechanicalWorld;
    Arena<JointConstraint> arena_;
    std::vector<DefaultJointConstraintHandle> inserted_, removed_;
    size_t n_ = 0;
};

// Force generators are not run on the GPU: a non-empty set makes the step
// fail with NPGPU_ERR_NONEMPTY_FORCES.
class DefaultForceGeneratorSet {
public:
    size_t len() const { return n_; }
    void insert_placeholder() { ++n_; }

private:
    size_t n_ = 0;
};

class GpuMechanicalWorld {
public:
    npgpu_params integration_parameters;
    // Copy poses and velocities back into the body set after each step.
    bool write_back = true;

    explicit GpuMechanicalWorld(Vector3 gravity, uint32_t capacity_bodies = 1u << 16,
                                uint32_t capacity_colliders = 1u << 16, uint32_t capacity_pairs = 0)
        : gravity_(gravity) {
        npgpu_default_params(&integration_parameters);
        float g[3] = {gravity.x, gravity.y, gravity.z};
        npgpu_status st = NPGPU_OK;
        if (capacity_pairs == 0) capacity_pairs = 16u * capacity_colliders;
        w_ = npgpu_create(&integration_parameters, g, capacity_bodies, capacity_colliders, capacity_pairs, &st);
        if (!w_) throw Error(st, npgpu_last_error(nullptr));
    }
    ~GpuMechanicalWorld() { npgpu_destroy(w_); }
    GpuMechanicalWorld(const GpuMechanicalWorld&) = delete;
    GpuMechanicalWorld& operator=(const GpuMechanicalWorld&) = delete;

    float timestep() const { return integration_parameters.dt; }
    void set_timestep(float dt) { integration_parameters.dt = dt; }
    npgpu_world* raw() { return w_; }

    // MechanicalWorld::step (mechanical_world.rs:182-196).
    void step(DefaultGeometricalWorld&, DefaultBodySet& bodies, DefaultColliderSet& colliders,
              DefaultJointConstraintSet& joints, DefaultForceGeneratorSet& forces) {
        check(npgpu_set_params(w_, &integration_parameters));
        maintain(bodies, colliders);
        maintain_joints(joints);
        check(npgpu_step(w_, 1, uint32_t(joints.len()), uint32_t(forces.len())));
        check(npgpu_synchronize(w_));
        if (write_back) {
            download(bodies);
            download_joints(joints);
        }
    }

    // Times the solver's launch shapes on real steps and keeps the fastest in
    // integration_parameters (npgpu_autotune). Every shape computes the same
    // bits, so this is the same as stepping the world that many times.
    void autotune(DefaultBodySet& bodies, DefaultColliderSet& colliders, uint32_t steps_per_candidate = 5) {
        check(npgpu_set_params(w_, &integration_parameters));
        maintain(bodies, colliders);
        uint32_t schedule = 0, threads = 0;
        check(npgpu_autotune(w_, steps_per_candidate, &schedule, &threads, nullptr));
        integration_parameters.solver_schedule = schedule;
        integration_parameters.world_threads = threads;
        if (write_back) download(bodies);
    }

    // The learned warm start (npgpu_mlp_set): NPGPU_MLP_PARAMS floats, used
    // for contacts without a cache entry once warmstart_mode is 2.
    void set_warmstart_network(const std::vector<float>& params) {
        check(npgpu_mlp_set(w_, params.data(), uint32_t(params.size())));
        integration_parameters.warmstart_mode = 2;
    }

    // GeometricalWorld::interferences_with_ray (geometrical_world.rs:327-341)
    // for one ray: every collider the ray hits within max_toi, with its time
    // of impact and normal, sorted by collider.
    std::vector<npgpu_ray_hit> interferences_with_ray(Vector3 origin, Vector3 dir, float max_toi) {
        const float ray[6] = {origin.x, origin.y, origin.z, dir.x, dir.y, dir.z};
        uint32_t n = 0;
        check(npgpu_interferences_with_rays(w_, 1, ray, &max_toi, 0xffffffffu, nullptr, 0, &n));
        std::vector<npgpu_ray_hit> hits(n);
        if (n) check(npgpu_interferences_with_rays(w_, 1, ray, &max_toi, 0xffffffffu, hits.data(), n, &n));
        return hits;
    }

    // GeometricalWorld::contact_events (geometrical_world.rs:373-376): the
    // last step's events, once enable_contact_events was called.
    void enable_contact_events(uint32_t capacity = 1u << 20) { check(npgpu_enable_contact_events(w_, capacity)); }
    std::vector<npgpu_contact_event> contact_events() {
        uint32_t n = 0;
        check(npgpu_contact_events(w_, nullptr, 0, &n));
        std::vector<npgpu_contact_event> ev(n);
        if (n) check(npgpu_contact_events(w_, ev.data(), n, &n));
        return ev;
    }

private:
    void check(npgpu_status s) {
        if (s != NPGPU_OK) throw Error(s, npgpu_last_error(w_));
    }

    // The joint set's removals, then its insertions (mechanical_world.rs:156-175).
    void maintain_joints(DefaultJointConstraintSet& joints) {
        std::vector<npgpu_handle> h;
        for (auto& j : joints.removed_) h.push_back(j.raw());
        joints.removed_.clear();
        if (!h.empty()) check(npgpu_remove_joints(w_, uint32_t(h.size()), h.data()));
        h.clear();
        std::vector<npgpu_joint_desc> d;
        for (auto& j : joints.inserted_) {
            const JointConstraint* c = joints.arena_.get(j);
            if (!c) continue;
            h.push_back(j.raw());
            d.push_back(std::visit([](const auto& x) { return x.desc; }, *c));
        }
        joints.inserted_.clear();
        if (!h.empty()) check(npgpu_upsert_joints(w_, uint32_t(h.size()), h.data(), d.data()));
    }

    // JointConstraint::cache_impulses / is_broken as the step left them.
    void download_joints(DefaultJointConstraintSet& joints) {
        std::vector<npgpu_handle> h;
        for (size_t i = 0; i < joints.arena_.capacity_used(); ++i)
            if (joints.arena_.occupied(i)) h.push_back(joints.arena_.handle_at(i).raw());
        if (h.empty()) return;
        std::vector<npgpu_joint_state> st(h.size());
        check(npgpu_get_joints(w_, uint32_t(h.size()), h.data(), st.data()));
        for (size_t k = 0; k < h.size(); ++k) {
            JointConstraint* c = joints.arena_.get(Index{h[k].index, h[k].generation});
            std::visit([&](auto& x) {
                JointConstraintBase& jb = x;
                jb.broken_ = st[k].broken != 0;
                std::memcpy(jb.impulses_, st[k].impulses, sizeof(st[k].impulses));
                jb.impulses_[6] = st[k].limit_impulse;
            }, *c);
        }
    }

    // MechanicalWorld::maintain: removals first, then insertions and edits.
    void maintain(DefaultBodySet& bodies, DefaultColliderSet& colliders) {
        std::vector<npgpu_handle> h;
        for (auto& c : colliders.removed_) h.push_back(c.raw());
        colliders.removed_.clear();
        if (!h.empty()) check(npgpu_remove_colliders(w_, uint32_t(h.size()), h.data()));
        h.clear();
        for (auto& b : bodies.removed_) h.push_back(b.raw());
        bodies.removed_.clear();
        if (!h.empty()) check(npgpu_remove_bodies(w_, uint32_t(h.size()), h.data()));

        std::vector<npgpu_handle> bh;
        std::vector<npgpu_body_desc> bd;
        std::vector<npgpu_handle> fh;
        std::vector<float> fv;
        std::vector<int> fw;
        for (size_t i = 0; i < bodies.arena_.capacity_used(); ++i) {
            if (!bodies.arena_.occupied(i)) continue;
            Index hi = bodies.arena_.handle_at(i);
            BodyVariant* v = bodies.arena_.get(hi);
            if (auto* rb = std::get_if<RigidBody>(v)) {
                if (rb->dirty_) {
                    bh.push_back(hi.raw());
                    bd.push_back(rb->desc);
                    rb->dirty_ = false;
                }
                if (rb->force_.any) {
                    fh.push_back(hi.raw());
                    fv.insert(fv.end(), rb->force_.v, rb->force_.v + 6);
                    fw.push_back(rb->force_.wake);
                    rb->force_ = RigidBody::Force();
                }
            } else if (std::holds_alternative<Ground>(*v) || std::holds_alternative<UnsupportedBody>(*v)) {
                bool known = known_static_.size() > i && known_static_[i] == hi.generation + 1;
                if (!known) {
                    npgpu_body_desc d = RigidBody().desc;
                    d.kind = std::holds_alternative<Ground>(*v) ? uint32_t(NPGPU_KIND_GROUND)
                                                                : std::get<UnsupportedBody>(*v).kind;
                    d.status = NPGPU_BODY_STATIC;
                    bh.push_back(hi.raw());
                    bd.push_back(d);
                    if (known_static_.size() <= i) known_static_.resize(i + 1, 0);
                    known_static_[i] = hi.generation + 1;
                }
            }
        }
        if (!bh.empty()) check(npgpu_upsert_bodies(w_, uint32_t(bh.size()), bh.data(), bd.data()));
        // Forces are applied per wake flag.
        for (int wake = 0; wake < 2; ++wake) {
            std::vector<npgpu_handle> hh;
            std::vector<float> ff;
            for (size_t k = 0; k < fh.size(); ++k)
                if (fw[k] == wake) {
                    hh.push_back(fh[k]);
                    ff.insert(ff.end(), fv.begin() + 6 * k, fv.begin() + 6 * k + 6);
                }
            if (!hh.empty()) check(npgpu_apply_forces(w_, uint32_t(hh.size()), hh.data(), ff.data(), wake));
        }
        std::vector<npgpu_handle> ch;
        std::vector<npgpu_collider_desc> cd;
        for (auto& c : colliders.inserted_) {
            const Collider* col = colliders.get(c);
            if (!col) continue;
            ch.push_back(c.raw());
            cd.push_back(col->desc);
        }
        colliders.inserted_.clear();
        bodies.inserted_.clear();
        if (!ch.empty()) check(npgpu_upsert_colliders(w_, uint32_t(ch.size()), ch.data(), cd.data()));
    }

    void download(DefaultBodySet& bodies) {
        uint32_t n = uint32_t(bodies.arena_.capacity_used());
        if (n == 0) return;
        pos_.resize(7 * size_t(n));
        vel_.resize(6 * size_t(n));
        act_.resize(n);
        check(npgpu_download_bodies(w_, 0, n, pos_.data(), vel_.data(), nullptr, act_.data()));
        for (uint32_t i = 0; i < n; ++i) {
            if (!bodies.arena_.occupied(i)) continue;
            BodyVariant* v = bodies.arena_.get(bodies.arena_.handle_at(i));
            if (auto* rb = std::get_if<RigidBody>(v)) {
                std::memcpy(rb->desc.position, &pos_[7 * size_t(i)], 7 * sizeof(float));
                std::memcpy(rb->desc.velocity, &vel_[6 * size_t(i)], 6 * sizeof(float));
                rb->active_ = act_[i] != 0;
            }
        }
    }

    npgpu_world* w_ = nullptr;
    Vector3 gravity_;
    std::vector<float> pos_, vel_;
    std::vector<uint8_t> act_;
    std::vector<uint64_t> known_static_;
};

}  // namespace nphysics_gpu
