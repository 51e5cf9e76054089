// ref_world.hpp -- CPU oracle of the nphysics3d 0.23 rigid-body step.
//
// TEST INFRASTRUCTURE ONLY. This restates MechanicalWorld::step
// (src/world/mechanical_world.rs:182-396) for scenes of static, dynamic and
// kinematic rigid bodies with ball and cuboid colliders, single-threaded, in
// R = float or double. It is the checker of the GPU step: tests, the smoke
// check and the CPU-baseline leg of the benchmark load it; the product never
// links it.
//
// Parity status. The reference (Rust) cannot be built here. The solver,
// dynamics, activation and material code below restate the reference files
// cited at each function. The collision arithmetic lives in ncollide3d 0.31,
// which is not vendored; it is restated from published methods (loosened
// AABBs with DBVT fat-AABB hysteresis, SAT + Sutherland-Hodgman clipping,
// Ericson's segment-segment closest points) and is pinned only by analytic
// known-answer tests, not by the reference's own outputs.
//
// Two Gauss-Seidel orders are provided:
//  - ORDER_REFERENCE: the reference's row order (non-ground rows, then ground
//    rows; manifolds in ascending collider-pair order);
//  - ORDER_COLOUR: the order of the GPU solver (manifolds grouped by their
//    Jones-Plassmann colour). It is a permutation of the same rows.
#pragma once
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <limits>
#include <array>
#include <limits>
#include <map>
#include <type_traits>
#include <string>
#include <vector>
#include <algorithm>
#include "ref_math.hpp"
#include "ref_ccd.hpp"
#include "../include/npgpu.h"

namespace oracle {

enum { ORDER_REFERENCE = 0, ORDER_COLOUR = 1 };
enum { AP_POINT = 1, AP_SEGMENT = 2, AP_PLANE = 3 };

// Feature ids of a cuboid: vertices 0-7 (bit k set = +h along axis k),
// edges 8-19 (8 + 4*axis + sign bits of the two other axes in increasing order),
// faces 20-25 (20 + 2*axis + positive). A ball has the single feature 0.
inline int box_vertex_id(int sx, int sy, int sz) { return sx | (sy << 1) | (sz << 2); }
inline void edge_other_axes(int a, int& o1, int& o2) {
    o1 = (a == 0) ? 1 : 0;
    o2 = (a == 2) ? 1 : 2;
}
inline int box_edge_id(int axis, int s_o1, int s_o2) { return 8 + 4 * axis + (s_o1 | (s_o2 << 1)); }
inline int box_face_id(int axis, int positive) { return 20 + 2 * axis + positive; }

inline uint32_t pair_hash22(uint32_t c1, uint32_t c2) {
    uint32_t h = c1 * 0x9E3779B1u ^ (c2 + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h >> 10;
}
// Jones-Plassmann priority of a manifold: unique per collider pair. The hash
// takes the colliders' world-local slots (slot minus the smallest alive
// collider slot of the world), so a world's colouring does not depend on
// where its slots start; ties are broken by the slots themselves.
inline uint64_t pair_priority(uint32_t l1, uint32_t l2, uint32_t c1, uint32_t c2) {
    return (uint64_t(pair_hash22(l1, l2)) << 42) | (uint64_t(c1) << 21) | uint64_t(c2);
}

template <class R> struct Approx {
    int kind;
    V3<R> a, b;  // point: a; segment: a..b; plane: point a, normal b
};

template <class R> inline Approx<R> box_feature(V3<R> h, int fid) {
    Approx<R> ap;
    if (fid < 8) {
        ap.kind = AP_POINT;
        ap.a = v3<R>((fid & 1) ? h.x : -h.x, (fid & 2) ? h.y : -h.y, (fid & 4) ? h.z : -h.z);
        ap.b = v3<R>(R(0), R(0), R(0));
    } else if (fid < 20) {
        int e = fid - 8, axis = e / 4, bits = e % 4, o1, o2;
        edge_other_axes(axis, o1, o2);
        V3<R> p = v3<R>(R(0), R(0), R(0));
        setc(p, o1, (bits & 1) ? comp(h, o1) : -comp(h, o1));
        setc(p, o2, (bits & 2) ? comp(h, o2) : -comp(h, o2));
        ap.kind = AP_SEGMENT;
        ap.a = p;
        ap.b = p;
        setc(ap.a, axis, -comp(h, axis));
        setc(ap.b, axis, comp(h, axis));
    } else {
        int f = fid - 20, axis = f / 2, pos = f % 2;
        ap.kind = AP_PLANE;
        ap.a = v3<R>(R(0), R(0), R(0));
        ap.b = v3<R>(R(0), R(0), R(0));
        setc(ap.a, axis, pos ? comp(h, axis) : -comp(h, axis));
        setc(ap.b, axis, pos ? R(1) : R(-1));
    }
    return ap;
}

// Closest points of two segments (Ericson, Real-Time Collision Detection, 5.1.9).
template <class R>
inline void closest_segment_segment(V3<R> p1, V3<R> q1, V3<R> p2, V3<R> q2, V3<R>& c1, V3<R>& c2,
                                    R* so = nullptr, R* to = nullptr) {
    const R eps = std::numeric_limits<R>::epsilon();
    V3<R> d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
    R a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    R s, t;
    if (a <= eps && e <= eps) {
        s = R(0); t = R(0);
    } else if (a <= eps) {
        s = R(0);
        t = std::min(std::max(f / e, R(0)), R(1));
    } else {
        R c = dot(d1, r);
        if (e <= eps) {
            t = R(0);
            s = std::min(std::max(-c / a, R(0)), R(1));
        } else {
            R b = dot(d1, d2);
            R denom = a * e - b * b;
            s = (denom != R(0)) ? std::min(std::max((b * f - c * e) / denom, R(0)), R(1)) : R(0);
            t = (b * s + f) / e;
            if (t < R(0)) {
                t = R(0);
                s = std::min(std::max(-c / a, R(0)), R(1));
            } else if (t > R(1)) {
                t = R(1);
                s = std::min(std::max((b - c) / a, R(0)), R(1));
            }
        }
    }
    c1 = p1 + d1 * s;
    c2 = p2 + d2 * t;
    if (so) *so = s;
    if (to) *to = t;
}

template <class R> struct ContactGeom {
    V3<R> world1, world2, normal;
    R depth;
};

// ContactKinematic::contact restated for the Point / Segment / Plane
// approximations (ncollide3d query::ContactKinematic, called at
// src/solver/nonlinear_sor_prox.rs:221-229). `n0` is the world default
// normal (from collider 1 toward collider 2), used when the feature
// points coincide and to orient point/segment normals.
template <class R>
inline ContactGeom<R> kinematic_contact(const Approx<R>& a1, const Iso<R>& m1, R dil1, const Approx<R>& a2,
                                        const Iso<R>& m2, R dil2, V3<R> n0) {
    V3<R> q1, q2, n;
    R s;
    if (a1.kind == AP_PLANE && a2.kind == AP_POINT) {
        n = qrot(m1.q, a1.b);
        V3<R> p1 = iso_pt(m1, a1.a);
        V3<R> p2 = iso_pt(m2, a2.a);
        s = dot(p2 - p1, n);
        q1 = p2 - n * s;
        q2 = p2;
    } else if (a1.kind == AP_POINT && a2.kind == AP_PLANE) {
        V3<R> n2 = qrot(m2.q, a2.b);
        V3<R> p1 = iso_pt(m1, a1.a);
        V3<R> p2 = iso_pt(m2, a2.a);
        s = dot(p1 - p2, n2);
        q1 = p1;
        q2 = p1 - n2 * s;
        n = -n2;
    } else {
        V3<R> s1a = iso_pt(m1, a1.a);
        V3<R> s1b = (a1.kind == AP_SEGMENT) ? iso_pt(m1, a1.b) : s1a;
        V3<R> s2a = iso_pt(m2, a2.a);
        V3<R> s2b = (a2.kind == AP_SEGMENT) ? iso_pt(m2, a2.b) : s2a;
        closest_segment_segment(s1a, s1b, s2a, s2b, q1, q2);
        V3<R> v = q2 - q1;
        R l2 = dot(v, v);
        const R eps = std::numeric_limits<R>::epsilon();
        if (l2 > eps * eps) {
            R l = std::sqrt(l2);
            n = vdiv(v, l);
            s = l;
            if (dot(n, n0) < R(0)) {
                n = -n;
                s = -l;
            }
        } else {
            n = n0;
            s = R(0);
        }
    }
    ContactGeom<R> g;
    g.world1 = q1 + n * dil1;
    g.world2 = q2 - n * dil2;
    g.normal = n;
    g.depth = (dil1 + dil2) - s;
    return g;
}

template <class R> struct Body {
    bool alive = false;
    uint64_t generation = 0;
    uint32_t status = NPGPU_BODY_DYNAMIC, kind = NPGPU_KIND_RIGID_BODY, flags = 0, world = 0;
    Iso<R> pos;
    Iso<R> pos0;                    // position0: the pose at the step's start, or where CCD advanced it
    V3<R> lin, ang;                 // velocity
    Inertia<R> local_inertia, inertia, aug, inv_aug;
    V3<R> local_com, com;
    V3<R> acc_lin, acc_ang;         // generalized acceleration
    V3<R> f_lin, f_ang;             // external forces
    R lin_damp, ang_damp, max_lin, max_ang;
    R sleep_threshold;
    bool can_sleep = true;
    R energy;
    R mask[6];
    bool changed = true;            // BodyUpdateStatus::inertia_needs_update / colliders_need_update
    bool in_island = false;
    bool linear_interp() const { return (flags & NPGPU_BODY_LINEAR_INTERP) != 0; }
    bool dynamic() const { return status == NPGPU_BODY_DYNAMIC; }
    bool kinematic() const { return status == NPGPU_BODY_KINEMATIC; }
    int ndofs() const { return dynamic() ? 6 : 0; }
    bool is_active() const {   // Body::is_active (src/object/body.rs:296-304)
        if (status == NPGPU_BODY_DYNAMIC) return energy != R(0);
        return status == NPGPU_BODY_KINEMATIC;
    }
};

template <class R> struct Collider {
    bool alive = false;
    bool registered = false;   // mass added to the body (maintain ran)
    uint64_t generation = 0;
    uint32_t body = 0;
    Iso<R> pos_wrt_body, pose;
    uint32_t shape = NPGPU_SHAPE_BALL;
    V3<R> half;                 // cuboid half extents
    R radius = R(0);
    R margin, density, linear_prediction, friction, restitution;
    uint32_t friction_combine = 0, restitution_combine = 0;
    R aabb_min[3], aabb_max[3];   // fat AABB
    bool has_fat = false;
    bool ccd = false;             // Collider::is_ccd_enabled
    bool sensor = false;          // Collider::is_sensor: a proximity query (margin taken as 0)
    R sw_min[3], sw_max[3];       // CCD: the box swept from the safe pose to the current one
    R query_limit() const { return margin + linear_prediction; }
    R dilation() const { return (shape == NPGPU_SHAPE_BALL || shape == NPGPU_SHAPE_CAPSULE) ? radius : R(0); }
};

template <class R> struct MContact {
    ContactGeom<R> g;
    int fid1, fid2;
    V3<R> normal1_local;   // contact normal in body 1's frame (signorini_model.rs:174)
    R impulse[3];          // ImpulseCache entry (normal, tangent1, tangent2)
    bool cached = false;   // the entry came from the cache (false: a new contact)
    uint32_t key() const { return uint32_t(fid1 * 26 + fid2); }
};

template <class R> struct Manifold {
    uint32_t c1, c2;
    std::vector<MContact<R>> contacts;
    uint32_t colour = 0xffffffffu;
    bool in_solver = false;
    uint32_t prox = NPGPU_PROXIMITY_DISJOINT;   // a pair with a sensor: its ncollide3d Proximity
};

template <class R> struct Row {
    R impulse, r, rhs;
    int b1, b2;            // dynamic body slots, -1 when the side has no dofs
    R J1[6], J2[6], WJ1[6], WJ2[6];
    int dep;               // friction: index of its normal row
    R mu;
    bool friction;
    bool bilateral;        // a joint row: Independent limits of +-max (helper.rs:186-189)
    bool limit;            // ... or of [0, max] (a prismatic offset limit, unit_constraint.rs:94-103)
    int joint, joint_slot; // its joint and impulse slot (0-2 linear, 3-5 angular)
    void* cache;           // MContact the impulse is cached to
    int cache_slot;
    bool predicted;        // normal row of a contact started from the learned network
    R alt[3];              // ... and the start the prediction replaced (cached impulses, or zero)
};

// A joint constraint (BallConstraint / FixedConstraint, src/joint/).
template <class R> struct Joint {
    bool alive = false;
    uint64_t generation = 0;
    uint32_t kind = NPGPU_JOINT_BALL, b1 = 0, b2 = 0;
    V3<R> anchor1, anchor2;     // in the bodies' frames
    Quat<R> frame1, frame2;     // the reference frames (fixed, cartesian)
    V3<R> axis1, axis2, axis3;  // the axes in the bodies' frames (axis3: the pin-slot's axis_w1)
    R angle = R(0);             // universal: the angle kept between the axes
    bool has_min = false, has_max = false;   // prismatic offset limits
    R min_offset = R(0), max_offset = R(0);
    R brk_force2, brk_torque2;  // set_break_force / set_break_torque keep the squares
    R imp[7] = {R(0), R(0), R(0), R(0), R(0), R(0), R(0)};   // linear 0-2, angular 3-5, the limit's 6
    bool broken = false, active = false;
};

template <class R> struct PosConstraint {
    uint32_t c1, c2;
    int fid1, fid2;
    V3<R> normal1_local;
    int joint = -1;           // >= 0: the position constraints of that joint
};

template <class R> class World {
public:
    using Real = R;
    npgpu_params params;
    V3<R> gravity;
    std::vector<Body<R>> bodies;
    std::vector<Collider<R>> colliders;
    std::map<uint64_t, Manifold<R>> manifolds;   // every broad-phase pair, keyed (c1 << 32) | c2
    std::vector<uint64_t> pairs;                  // sorted broad-phase pair set
    int order = ORDER_REFERENCE;
    npgpu_counters counters;
    std::string last_error;
    bool cd_dirty = true;
    uint32_t num_colours = 0;
    uint32_t num_solver_contacts = 0;   // contacts the last solve took, counted when they were collected
    std::vector<Joint<R>> joints;        // by joint slot (the host set's arena index)
    R cur_dt = R(0);                     // the step length of the body and row arithmetic: dt, or a CCD substep's

    World(const npgpu_params& p, const float g[3]) : params(p) {
        gravity = v3<R>(R(g[0]), R(g[1]), R(g[2]));
        cur_dt = R(p.dt);
        std::memset(&counters, 0, sizeof(counters));
    }

    // ---------------------------------------------------------------- host API
    npgpu_status fail(npgpu_status s, const std::string& m) {
        last_error = m;
        return s;
    }

    npgpu_status upsert_body(const npgpu_handle& h, const npgpu_body_desc& d) {
        if (d.kind != NPGPU_KIND_RIGID_BODY && d.kind != NPGPU_KIND_GROUND)
            return fail(NPGPU_ERR_UNSUPPORTED_BODY, "only rigid bodies and grounds are supported");
        if (h.index >= (1u << 21)) return fail(NPGPU_ERR_CAPACITY, "body index too large");
        if (h.index >= bodies.size()) bodies.resize(h.index + 1);
        Body<R>& b = bodies[h.index];
        bool existed = b.alive;
        b.alive = true;
        b.generation = h.generation;
        b.kind = d.kind;
        b.status = (d.kind == NPGPU_KIND_GROUND) ? NPGPU_BODY_STATIC : d.status;
        b.flags = d.flags;
        b.world = d.world;
        b.pos.t = v3<R>(R(d.position[0]), R(d.position[1]), R(d.position[2]));
        b.pos.q = Quat<R>{R(d.position[3]), R(d.position[4]), R(d.position[5]), R(d.position[6])};
        b.lin = v3<R>(R(d.velocity[0]), R(d.velocity[1]), R(d.velocity[2]));
        b.ang = v3<R>(R(d.velocity[3]), R(d.velocity[4]), R(d.velocity[5]));
        if (d.kind == NPGPU_KIND_GROUND) {
            b.pos = iso_identity<R>();
            b.lin = b.ang = v3<R>(R(0), R(0), R(0));
        }
        if (!existed) {
            // RigidBody::new + RigidBodyDesc::build (rigid_body.rs:54-83, 1064-1084).
            b.local_inertia.linear = R(d.local_inertia[0]);
            M3<R> a = mzero<R>();
            a.m[0][0] = R(d.local_inertia[1]); a.m[0][1] = a.m[1][0] = R(d.local_inertia[2]);
            a.m[0][2] = a.m[2][0] = R(d.local_inertia[3]); a.m[1][1] = R(d.local_inertia[4]);
            a.m[1][2] = a.m[2][1] = R(d.local_inertia[5]); a.m[2][2] = R(d.local_inertia[6]);
            b.local_inertia.angular = a;
            b.local_com = v3<R>(R(d.local_com[0]), R(d.local_com[1]), R(d.local_com[2]));
            b.acc_lin = b.acc_ang = v3<R>(R(0), R(0), R(0));
            b.f_lin = b.f_ang = v3<R>(R(0), R(0), R(0));
            // ActivationStatus::new_active (body.rs:79-84) uses the default threshold 0.01
            // whatever threshold is set afterwards; a ground starts inactive (ground.rs:24).
            b.energy = (d.kind == NPGPU_KIND_GROUND) ? R(0) : R(0.01) * R(4);
        }
        b.com = iso_pt(b.pos, b.local_com);
        b.pos0 = b.pos;
        update_inertia_from_local_inertia(b);
        b.lin_damp = R(d.linear_damping);
        b.ang_damp = R(d.angular_damping);
        b.max_lin = R(d.max_linear_velocity);
        b.max_ang = R(d.max_angular_velocity);
        b.sleep_threshold = R(d.sleep_threshold);
        b.can_sleep = (d.flags & NPGPU_BODY_CAN_SLEEP) != 0;
        for (int k = 0; k < 6; ++k) b.mask[k] = (d.flags & (NPGPU_BODY_LOCK_TX << k)) ? R(0) : R(1);
        b.changed = true;
        cd_dirty = true;
        return NPGPU_OK;
    }

    npgpu_status upsert_collider(const npgpu_handle& h, const npgpu_collider_desc& d) {
        if (d.shape != NPGPU_SHAPE_BALL && d.shape != NPGPU_SHAPE_CUBOID && d.shape != NPGPU_SHAPE_CAPSULE)
            return fail(NPGPU_ERR_UNSUPPORTED_SHAPE, "only balls, cuboids and capsules are supported");
        if (d.body.index >= bodies.size() || !bodies[d.body.index].alive ||
            bodies[d.body.index].generation != d.body.generation)
            return fail(NPGPU_ERR_INVALID_HANDLE, "collider parent body handle is invalid");
        if (h.index >= (1u << 21)) return fail(NPGPU_ERR_CAPACITY, "collider index too large");
        if (h.index >= colliders.size()) colliders.resize(h.index + 1);
        Collider<R>& c = colliders[h.index];
        if (c.alive && c.registered) remove_collider_mass(c);
        c = Collider<R>();
        c.alive = true;
        c.generation = h.generation;
        c.body = uint32_t(d.body.index);
        c.pos_wrt_body.t = v3<R>(R(d.position_wrt_body[0]), R(d.position_wrt_body[1]), R(d.position_wrt_body[2]));
        c.pos_wrt_body.q = Quat<R>{R(d.position_wrt_body[3]), R(d.position_wrt_body[4]), R(d.position_wrt_body[5]),
                                   R(d.position_wrt_body[6])};
        c.shape = d.shape;
        c.radius = R(d.shape_params[0]);
        c.half = v3<R>(R(d.shape_params[0]), R(d.shape_params[1]), R(d.shape_params[2]));
        // A sensor's query limit is its linear prediction alone
        // (GeometricQueryType::Proximity, collider.rs:542-543).
        c.sensor = d.is_sensor != 0;
        c.margin = c.sensor ? R(0) : R(d.margin);
        c.density = R(d.density);
        c.linear_prediction = R(d.linear_prediction);
        c.friction = R(d.friction);
        c.restitution = R(d.restitution);
        c.friction_combine = d.friction_combine;
        c.restitution_combine = d.restitution_combine;
        c.ccd = d.ccd_enabled != 0;
        // Drop manifolds involving the replaced collider.
        drop_manifolds_of(uint32_t(h.index));
        cd_dirty = true;
        return NPGPU_OK;
    }

    npgpu_status remove_body(const npgpu_handle& h) {
        if (h.index >= bodies.size() || !bodies[h.index].alive || bodies[h.index].generation != h.generation)
            return fail(NPGPU_ERR_INVALID_HANDLE, "invalid body handle");
        // Removing a body removes its colliders (mechanical_world.rs:130-139).
        for (size_t i = 0; i < colliders.size(); ++i)
            if (colliders[i].alive && colliders[i].body == h.index) remove_collider_slot(uint32_t(i), false);
        bodies[h.index].alive = false;
        // Joints with a removed body go too (mechanical_world.rs:141-154).
        for (uint32_t j = 0; j < joints.size(); ++j)
            if (joints[j].alive && (joints[j].b1 == h.index || joints[j].b2 == h.index)) drop_joint(j);
        cd_dirty = true;
        return NPGPU_OK;
    }

    npgpu_status remove_collider(const npgpu_handle& h) {
        if (h.index >= colliders.size() || !colliders[h.index].alive || colliders[h.index].generation != h.generation)
            return fail(NPGPU_ERR_INVALID_HANDLE, "invalid collider handle");
        remove_collider_slot(uint32_t(h.index), true);
        cd_dirty = true;
        return NPGPU_OK;
    }

    npgpu_status apply_force(const npgpu_handle& h, const float* f, bool wake) {
        if (h.index >= bodies.size() || !bodies[h.index].alive || bodies[h.index].generation != h.generation)
            return fail(NPGPU_ERR_INVALID_HANDLE, "invalid body handle");
        Body<R>& b = bodies[h.index];
        // RigidBody::apply_force, ForceType::Force (rigid_body.rs:771-792).
        if (b.status != NPGPU_BODY_DYNAMIC) return NPGPU_OK;
        if (wake) activate(b);
        b.f_lin = b.f_lin + v3<R>(R(f[0]) * b.mask[0], R(f[1]) * b.mask[1], R(f[2]) * b.mask[2]);
        b.f_ang = b.f_ang + v3<R>(R(f[3]) * b.mask[3], R(f[4]) * b.mask[4], R(f[5]) * b.mask[5]);
        return NPGPU_OK;
    }

    // DefaultJointConstraintSet::insert / remove, waking both bodies
    // (mechanical_world.rs:156-175).
    npgpu_status upsert_joint(const npgpu_handle& h, const npgpu_joint_desc& d) {
        auto body_ok = [&](const npgpu_handle& b) {
            return b.index < bodies.size() && bodies[b.index].alive && bodies[b.index].generation == b.generation;
        };
        if (d.kind > NPGPU_JOINT_PIN_SLOT) return fail(NPGPU_ERR_INVALID_ARGUMENT, "unknown joint kind");
        if ((d.limit_flags & NPGPU_JOINT_MIN_OFFSET) && (d.limit_flags & NPGPU_JOINT_MAX_OFFSET) &&
            !(d.min_offset <= d.max_offset))
            return fail(NPGPU_ERR_INVALID_ARGUMENT, "min offset above max offset");
        if (!body_ok(d.body1) || !body_ok(d.body2)) return fail(NPGPU_ERR_INVALID_HANDLE, "joint body handle is invalid");
        if (d.body1.index == d.body2.index) return fail(NPGPU_ERR_INVALID_ARGUMENT, "a joint needs two different bodies");
        if (bodies[d.body1.index].world != bodies[d.body2.index].world)
            return fail(NPGPU_ERR_INVALID_ARGUMENT, "a joint's bodies must belong to the same world");
        if (h.index >= (1u << 21) - 1u) return fail(NPGPU_ERR_CAPACITY, "joint index too large");
        if (h.index >= joints.size()) joints.resize(h.index + 1);
        Joint<R>& j = joints[h.index];
        if (j.alive) {
            activate_alive(j.b1);
            activate_alive(j.b2);
        }
        j = Joint<R>();
        j.alive = true;
        j.generation = h.generation;
        j.kind = d.kind;
        j.b1 = uint32_t(d.body1.index);
        j.b2 = uint32_t(d.body2.index);
        j.anchor1 = v3<R>(R(d.anchor1[0]), R(d.anchor1[1]), R(d.anchor1[2]));
        j.anchor2 = v3<R>(R(d.anchor2[0]), R(d.anchor2[1]), R(d.anchor2[2]));
        j.frame1 = Quat<R>{R(d.frame1[0]), R(d.frame1[1]), R(d.frame1[2]), R(d.frame1[3])};
        j.frame2 = Quat<R>{R(d.frame2[0]), R(d.frame2[1]), R(d.frame2[2]), R(d.frame2[3])};
        j.axis1 = v3<R>(R(d.axis1[0]), R(d.axis1[1]), R(d.axis1[2]));
        j.axis2 = v3<R>(R(d.axis2[0]), R(d.axis2[1]), R(d.axis2[2]));
        j.axis3 = v3<R>(R(d.axis3[0]), R(d.axis3[1]), R(d.axis3[2]));
        j.angle = R(d.angle);
        j.has_min = d.kind == NPGPU_JOINT_PRISMATIC && (d.limit_flags & NPGPU_JOINT_MIN_OFFSET) != 0;
        j.has_max = d.kind == NPGPU_JOINT_PRISMATIC && (d.limit_flags & NPGPU_JOINT_MAX_OFFSET) != 0;
        j.min_offset = R(d.min_offset);
        j.max_offset = R(d.max_offset);
        const R f = R(d.break_force), t = R(d.break_torque);
        j.brk_force2 = f * f;
        j.brk_torque2 = t * t;
        activate_alive(j.b1);
        activate_alive(j.b2);
        return NPGPU_OK;
    }
    npgpu_status remove_joint(const npgpu_handle& h) {
        if (h.index >= joints.size() || !joints[h.index].alive || joints[h.index].generation != h.generation)
            return fail(NPGPU_ERR_INVALID_HANDLE, "invalid joint handle");
        drop_joint(uint32_t(h.index));
        return NPGPU_OK;
    }
    void drop_joint(uint32_t j) {
        joints[j].alive = false;
        activate_alive(joints[j].b1);
        activate_alive(joints[j].b2);
    }
    void activate_alive(uint32_t b) {
        if (b < bodies.size() && bodies[b].alive) activate(bodies[b]);
    }

    // ------------------------------------------------------- body dynamics
    static void activate(Body<R>& b) {   // Body::activate (body.rs:335-340)
        if (b.can_sleep) b.energy = b.sleep_threshold * R(2);
    }
    static void deactivate(Body<R>& b) {   // RigidBody::deactivate (rigid_body.rs:396-400)
        b.changed = false;
        b.energy = R(0);
        b.lin = b.ang = v3<R>(R(0), R(0), R(0));
    }
    // Inertia3::transformed (inertia3.rs:68-71): R I R^-1.
    static Inertia<R> transformed(const Inertia<R>& in, const Quat<R>& q) {
        M3<R> rot = qmat(q);
        Inertia<R> r;
        r.linear = in.linear;
        r.angular = mm(mm(rot, in.angular), mtr(rot));
        return r;
    }
    static Inertia<R> inverse(const Inertia<R>& in) {   // inertia3.rs:75-86
        Inertia<R> r;
        r.linear = (in.linear == R(0)) ? R(0) : R(1) / in.linear;
        r.angular = minv_or_zero(in.angular);
        return r;
    }
    static void update_inertia_from_local_inertia(Body<R>& b) {   // rigid_body.rs:266-271
        b.inertia = transformed(b.local_inertia, b.pos.q);
        b.aug = b.inertia;
        b.inv_aug = inverse(b.inertia);
    }
    // RigidBody::add_local_inertia_and_com (rigid_body.rs:747-766).
    static void add_local_inertia_and_com(Body<R>& b, V3<R> com, const Inertia<R>& in) {
        R mass_sum = b.inertia.linear + in.linear;
        if (mass_sum != R(0)) {
            b.local_com = vdiv(b.local_com * b.inertia.linear + com * in.linear, mass_sum);
            b.com = iso_pt(b.pos, b.local_com);
        } else {
            b.local_com = v3<R>(R(0), R(0), R(0));
            b.com = b.pos.t;
        }
        b.local_inertia.linear = b.local_inertia.linear + in.linear;
        b.local_inertia.angular = madd(b.local_inertia.angular, in.angular);
        update_inertia_from_local_inertia(b);
        b.changed = true;
    }
    // Volumetric::transformed_mass_properties (volumetric.rs:55-59) for Ball
    // (volumetric_ball.rs:8-47) and Cuboid (volumetric_cuboid.rs:9-78).
    static void mass_properties(const Collider<R>& c, V3<R>& com, Inertia<R>& in) {
        const R pi = R(3.14159265358979323846);
        R mass;
        M3<R> unit = mzero<R>();
        if (c.shape == NPGPU_SHAPE_BALL) {
            R r = c.radius;
            R vol = pi * r * r * r * R(4.0 / 3.0);
            mass = vol * c.density;
            R diag = r * r * R(2.0 / 5.0);
            unit.m[0][0] = unit.m[1][1] = unit.m[2][2] = diag;
        } else if (c.shape == NPGPU_SHAPE_CAPSULE) {
            // volumetric_capsule.rs:7-37: cylinder + ball volume; the
            // cylinder's and the ball's unit inertia plus the hemispheres'
            // parallel-axis term on x and z.
            R r = c.radius, hh = c.half.y;
            R vol = hh * r * r * pi * R(2) + pi * r * r * r * R(4.0 / 3.0);
            mass = vol * c.density;
            R sq_radius = r * r;
            R sq_height = hh * hh * R(4);
            R off = (sq_radius * R(3) + sq_height) / R(12);
            R diag = r * r * R(2.0 / 5.0);
            R h = hh * R(2);
            R extra = h * h * R(0.5) + h * r * R(3.0 / 8.0);
            unit.m[0][0] = (off + diag) + extra;
            unit.m[1][1] = sq_radius / R(2) + diag;
            unit.m[2][2] = (off + diag) + extra;
        } else {
            R vol = R(1);
            vol = vol * c.half.x * R(2);
            vol = vol * c.half.y * R(2);
            vol = vol * c.half.z * R(2);
            mass = vol * c.density;
            R w = R(1.0 / 12.0) * R(2) * R(2);
            R ix = w * c.half.x * c.half.x, iy = w * c.half.y * c.half.y, iz = w * c.half.z * c.half.z;
            unit.m[0][0] = iy + iz;
            unit.m[1][1] = ix + iz;
            unit.m[2][2] = ix + iy;
        }
        Inertia<R> local;
        local.linear = mass;
        local.angular = mscale(unit, mass);
        com = iso_pt(c.pos_wrt_body, v3<R>(R(0), R(0), R(0)));
        in = transformed(local, c.pos_wrt_body.q);
    }
    void remove_collider_mass(Collider<R>& c) {
        Body<R>& b = bodies[c.body];
        if (!b.alive) return;
        if (c.density != R(0) && b.kind == NPGPU_KIND_RIGID_BODY) {
            V3<R> com;
            Inertia<R> in;
            mass_properties(c, com, in);
            Inertia<R> neg;
            neg.linear = -in.linear;
            neg.angular = mscale(in.angular, R(-1));
            add_local_inertia_and_com(b, -com, neg);
        }
        activate(b);
    }
    void drop_manifolds_of(uint32_t ci) {
        for (auto it = manifolds.begin(); it != manifolds.end();) {
            if (it->second.c1 == ci || it->second.c2 == ci) it = manifolds.erase(it);
            else ++it;
        }
    }
    // GeometricalWorld::handle_removals (geometrical_world.rs:145-227).
    void remove_collider_slot(uint32_t ci, bool body_remains) {
        Collider<R>& c = colliders[ci];
        for (auto& kv : manifolds) {
            Manifold<R>& m = kv.second;
            if (m.contacts.empty()) continue;
            uint32_t other = (m.c1 == ci) ? m.c2 : ((m.c2 == ci) ? m.c1 : 0xffffffffu);
            if (other != 0xffffffffu) activate(bodies[colliders[other].body]);
        }
        if (body_remains && c.registered) remove_collider_mass(c);
        drop_manifolds_of(ci);
        c.alive = false;
    }

    // RigidBody::update_dynamics (rigid_body.rs:558-588).
    void update_dynamics(Body<R>& b, R dt) {
        if (!b.changed || b.status != NPGPU_BODY_DYNAMIC) return;
        if (!b.is_active()) activate(b);
        b.inertia = transformed(b.local_inertia, b.pos.q);
        b.aug = b.inertia;
        const M3<R>& i = b.inertia.angular;
        V3<R> w = b.ang;
        V3<R> iw = mv(i, w);
        V3<R> w_dt = w * dt;
        M3<R> w_dt_cross = cross_matrix(w_dt);
        M3<R> iw_dt_cross = cross_matrix(iw * dt);
        b.aug.angular = madd(b.aug.angular, msub(mm(w_dt_cross, i), iw_dt_cross));
        b.inv_aug = inverse(b.aug);
    }
    // RigidBody::update_acceleration (rigid_body.rs:590-619).
    void update_acceleration(Body<R>& b) { update_acceleration(b, gravity); }
    void update_acceleration(Body<R>& b, V3<R> g) {
        b.acc_lin = b.acc_ang = v3<R>(R(0), R(0), R(0));
        if (b.status != NPGPU_BODY_DYNAMIC) return;
        V3<R> iw = mv(b.inertia.angular, b.ang);
        V3<R> gyro = -cross(b.ang, iw);
        b.acc_ang = mv(b.inv_aug.angular, gyro);
        if (b.inv_aug.linear != R(0) && (b.flags & NPGPU_BODY_GRAVITY)) b.acc_lin = g;
        b.acc_lin = b.acc_lin + b.f_lin * b.inv_aug.linear;
        b.acc_ang = b.acc_ang + mv(b.inv_aug.angular, b.f_ang);
        b.acc_lin = v3<R>(b.acc_lin.x * b.mask[0], b.acc_lin.y * b.mask[1], b.acc_lin.z * b.mask[2]);
        b.acc_ang = v3<R>(b.acc_ang.x * b.mask[3], b.acc_ang.y * b.mask[4], b.acc_ang.z * b.mask[5]);
    }
    // RigidBody::apply_displacement (rigid_body.rs:371-381) and set_position (:297-307).
    static void apply_displacement(Body<R>& b, V3<R> dlin, V3<R> dang) {
        Quat<R> qd = qexp_scaled_axis(dang);
        // shift * disp * shift^-1 with shift = Translation(com).
        V3<R> t = (b.com + dlin) + qrot(qd, -b.com);
        Iso<R> np;
        np.t = t + qrot(qd, b.pos.t);
        np.q = qmul(qd, b.pos.q);
        b.pos = np;
        b.com = iso_pt(b.pos, b.local_com);
        b.changed = true;
    }
    // RigidBody::integrate (rigid_body.rs:467-505).
    void integrate(Body<R>& b) {
        R dt = cur_dt;
        b.lin = b.lin * (R(1) / (R(1) + dt * b.lin_damp));
        b.ang = b.ang * (R(1) / (R(1) + dt * b.ang_damp));
        R ln = norm(b.lin);
        if (ln > b.max_lin) {
            if (b.max_lin == R(0)) b.lin = v3<R>(R(0), R(0), R(0));
            else b.lin = b.lin * (b.max_lin / ln);
        }
        R an = norm(b.ang);
        if (an > b.max_ang) {
            if (b.max_ang == R(0)) b.ang = v3<R>(R(0), R(0), R(0));
            else b.ang = b.ang * (b.max_ang / an);
        }
        apply_displacement(b, b.lin * dt, b.ang * dt);
    }

    // ------------------------------------------------------- collision detection
    void collider_aabb(const Collider<R>& c, R mn[3], R mx[3]) const { aabb_at(c, c.pose, mn, mx); }
    void aabb_at(const Collider<R>& c, const Iso<R>& pose, R mn[3], R mx[3]) const {
        // Shape AABB at the collider pose (ncollide3d bounding_volume), loosened by
        // the query limit margin + linear prediction (collider.rs:542-549).
        V3<R> ctr = pose.t;
        V3<R> half;
        if (c.shape == NPGPU_SHAPE_BALL) {
            half = v3<R>(c.radius, c.radius, c.radius);
        } else if (c.shape == NPGPU_SHAPE_CAPSULE) {
            M3<R> rot = qmat(pose.q);
            for (int a = 0; a < 3; ++a) setc(half, a, std::fabs(rot.m[a][1]) * c.half.y + c.radius);
        } else {
            M3<R> rot = qmat(pose.q);
            for (int a = 0; a < 3; ++a) {
                R s = std::fabs(rot.m[a][0]) * c.half.x + std::fabs(rot.m[a][1]) * c.half.y +
                      std::fabs(rot.m[a][2]) * c.half.z;
                setc(half, a, s);
            }
        }
        R ql = c.query_limit();
        for (int a = 0; a < 3; ++a) {
            mn[a] = (comp(ctr, a) - comp(half, a)) - ql;
            mx[a] = (comp(ctr, a) + comp(half, a)) + ql;
        }
    }
    // sync_colliders (geometrical_world.rs:230-265) + the DBVT proxy update:
    // the fat AABB is the tight one loosened by the broad-phase margin, and is
    // replaced only when the tight AABB leaves it.
    void sync_colliders() {
        R margin = R(params.broad_phase_margin);
        for (auto& c : colliders) {
            if (!c.alive) continue;
            const Body<R>& b = bodies[c.body];
            c.pose = iso_mul(b.pos, c.pos_wrt_body);
            R mn[3], mx[3];
            collider_aabb(c, mn, mx);
            bool inside = c.has_fat;
            for (int a = 0; a < 3 && inside; ++a)
                if (!(c.aabb_min[a] <= mn[a] && mx[a] <= c.aabb_max[a])) inside = false;
            if (!inside) {
                for (int a = 0; a < 3; ++a) {
                    c.aabb_min[a] = mn[a] - margin;
                    c.aabb_max[a] = mx[a] + margin;
                }
                c.has_fat = true;
            }
        }
    }
    static bool aabb_overlap(const Collider<R>& a, const Collider<R>& b) {
        for (int k = 0; k < 3; ++k)
            if (!(a.aabb_min[k] <= b.aabb_max[k] && b.aabb_min[k] <= a.aabb_max[k])) return false;
        return true;
    }
    // DefaultCollisionFilter (geometrical_world.rs:926-970) + one world per batch entry.
    bool pair_allowed(uint32_t i, uint32_t j) const {
        const Collider<R>& a = colliders[i];
        const Collider<R>& b = colliders[j];
        if (a.body == b.body) return false;
        const Body<R>& ba = bodies[a.body];
        const Body<R>& bb = bodies[b.body];
        if (ba.world != bb.world) return false;
        return ba.ndofs() != 0 || bb.ndofs() != 0;
    }
    // Broad phase: the set of allowed pairs whose fat AABBs intersect, found by
    // sweep-and-prune along x (the set equals the brute-force one).
    void broad_phase() {
        std::vector<uint32_t> idx;
        for (uint32_t i = 0; i < colliders.size(); ++i)
            if (colliders[i].alive) idx.push_back(i);
        std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
            if (colliders[a].aabb_min[0] != colliders[b].aabb_min[0])
                return colliders[a].aabb_min[0] < colliders[b].aabb_min[0];
            return a < b;
        });
        pairs.clear();
        for (size_t s = 0; s < idx.size(); ++s) {
            const Collider<R>& a = colliders[idx[s]];
            for (size_t t = s + 1; t < idx.size(); ++t) {
                const Collider<R>& b = colliders[idx[t]];
                if (b.aabb_min[0] > a.aabb_max[0]) break;
                if (!aabb_overlap(a, b)) continue;
                uint32_t i = std::min(idx[s], idx[t]), j = std::max(idx[s], idx[t]);
                if (!pair_allowed(i, j)) continue;
                pairs.push_back((uint64_t(i) << 32) | j);
            }
        }
        std::sort(pairs.begin(), pairs.end());
    }
    std::vector<uint64_t> broad_phase_brute_force() const {
        std::vector<uint64_t> out;
        for (uint32_t i = 0; i < colliders.size(); ++i) {
            if (!colliders[i].alive) continue;
            for (uint32_t j = i + 1; j < colliders.size(); ++j) {
                if (!colliders[j].alive) continue;
                if (aabb_overlap(colliders[i], colliders[j]) && pair_allowed(i, j)) out.push_back((uint64_t(i) << 32) | j);
            }
        }
        return out;
    }

    Approx<R> feature(const Collider<R>& c, int fid) const {
        if (c.shape == NPGPU_SHAPE_BALL) {
            Approx<R> ap;
            ap.kind = AP_POINT;
            ap.a = ap.b = v3<R>(R(0), R(0), R(0));
            return ap;
        }
        if (c.shape == NPGPU_SHAPE_CAPSULE) {
            // A capsule's axis (fid 0) or its ends (1 at -half height, 2 at +).
            Approx<R> ap;
            const V3<R> lo = v3<R>(R(0), -c.half.y, R(0)), hi = v3<R>(R(0), c.half.y, R(0));
            if (fid == 0) {
                ap.kind = AP_SEGMENT;
                ap.a = lo;
                ap.b = hi;
            } else {
                ap.kind = AP_POINT;
                ap.a = ap.b = fid == 1 ? lo : hi;
            }
            return ap;
        }
        return box_feature(c.half, fid);
    }

    // Candidate contact: features + default normal; evaluated by kinematic_contact.
    struct Cand {
        int fid1, fid2;
        ContactGeom<R> g;
    };

    void push_eval(std::vector<Cand>& out, const Collider<R>& c1, const Collider<R>& c2, int f1, int f2, V3<R> n0,
                   R prediction) const {
        ContactGeom<R> g = kinematic_contact(feature(c1, f1), c1.pose, c1.dilation(), feature(c2, f2), c2.pose,
                                             c2.dilation(), n0);
        if (g.depth >= -prediction) out.push_back(Cand{f1, f2, g});
    }

    // A sphere around `centre` (feature sfid of cb: a ball, or a capsule's
    // end) against cuboid cx: the closest point of the cuboid to the centre.
    void sphere_box(const Collider<R>& cb, int sfid, V3<R> centre, const Collider<R>& cx, bool box_first, R prediction,
                    std::vector<Cand>& out) const {
        V3<R> c = iso_inv_pt(cx.pose, centre);
        V3<R> h = cx.half;
        int sign[3], nclamped = 0;
        V3<R> p = c;
        for (int k = 0; k < 3; ++k) {
            R ck = comp(c, k), hk = comp(h, k);
            if (ck > hk) { sign[k] = 1; setc(p, k, hk); ++nclamped; }
            else if (ck < -hk) { sign[k] = -1; setc(p, k, -hk); ++nclamped; }
            else sign[k] = 0;
        }
        int fid;
        V3<R> nl;
        if (nclamped == 0) {
            int best = 0;
            R bd = comp(h, 0) - std::fabs(comp(c, 0));
            for (int k = 1; k < 3; ++k) {
                R dk = comp(h, k) - std::fabs(comp(c, k));
                if (dk < bd) { bd = dk; best = k; }
            }
            int pos = comp(c, best) >= R(0) ? 1 : 0;
            fid = box_face_id(best, pos);
            nl = v3<R>(R(0), R(0), R(0));
            setc(nl, best, pos ? R(1) : R(-1));
        } else {
            if (nclamped == 1) {
                int k = sign[0] ? 0 : (sign[1] ? 1 : 2);
                fid = box_face_id(k, sign[k] > 0 ? 1 : 0);
            } else if (nclamped == 2) {
                int a = !sign[0] ? 0 : (!sign[1] ? 1 : 2), o1, o2;
                edge_other_axes(a, o1, o2);
                fid = box_edge_id(a, sign[o1] > 0 ? 1 : 0, sign[o2] > 0 ? 1 : 0);
            } else {
                fid = box_vertex_id(sign[0] > 0, sign[1] > 0, sign[2] > 0);
            }
            V3<R> v = c - p;
            nl = vdiv(v, norm(v));
        }
        V3<R> n = qrot(cx.pose.q, nl);   // from the cuboid toward the ball
        if (box_first) push_eval(out, cx, cb, fid, sfid, n, prediction);
        else push_eval(out, cb, cx, sfid, fid, -n, prediction);
    }

    // Ball-cuboid: closest point of the cuboid to the ball center.
    void ball_box(const Collider<R>& cb, const Collider<R>& cx, bool box_first, R prediction, std::vector<Cand>& out) const {
        sphere_box(cb, 0, cb.pose.t, cx, box_first, prediction, out);
    }

    // ---- capsules: a segment along the local y axis dilated by the radius ----
    void capsule_axis(const Collider<R>& c, V3<R>& p0, V3<R>& p1) const {
        p0 = iso_pt(c.pose, v3<R>(R(0), -c.half.y, R(0)));
        p1 = iso_pt(c.pose, v3<R>(R(0), c.half.y, R(0)));
    }
    static V3<R> unit_or(V3<R> v, V3<R> fallback) {
        const R eps = std::numeric_limits<R>::epsilon();
        const R l2 = dot(v, v);
        return l2 > eps * eps ? vdiv(v, std::sqrt(l2)) : fallback;
    }
    // Ball against capsule: the closest point of the capsule's axis.
    void ball_capsule(const Collider<R>& cb, const Collider<R>& cc, bool capsule_first, R prediction,
                      std::vector<Cand>& out) const {
        V3<R> p0, p1, qa, qb;
        capsule_axis(cc, p0, p1);
        closest_segment_segment(p0, p1, cb.pose.t, cb.pose.t, qa, qb);
        const V3<R> n0 = unit_or(qb - qa, v3<R>(R(1), R(0), R(0)));
        if (capsule_first) push_eval(out, cc, cb, 0, 0, n0, prediction);
        else push_eval(out, cb, cc, 0, 0, -n0, prediction);
    }
    // Capsule-capsule: the closest points of the axes; for parallel axes
    // (sine below 1e-3), the two ends of their overlap.
    void capsule_capsule(const Collider<R>& A, const Collider<R>& B, R prediction, std::vector<Cand>& out) const {
        V3<R> a0, a1, b0, b1, qa, qb;
        capsule_axis(A, a0, a1);
        capsule_axis(B, b0, b1);
        closest_segment_segment(a0, a1, b0, b1, qa, qb);
        const V3<R> da = a1 - a0, db = b1 - b0;
        const V3<R> cr = cross(da, db);
        const V3<R> n0 = unit_or(qb - qa, unit_or(cr, v3<R>(R(1), R(0), R(0))));
        const R la2 = dot(da, da), lb2 = dot(db, db);
        if (dot(cr, cr) > R(1e-6f) * la2 * lb2 || la2 <= std::numeric_limits<R>::epsilon()) {
            push_eval(out, A, B, 0, 0, n0, prediction);
            return;
        }
        const R tb0 = dot(b0 - a0, da) / la2, tb1 = dot(b1 - a0, da) / la2;
        const int flo = tb0 <= tb1 ? 1 : 2, fhi = tb0 <= tb1 ? 2 : 1;
        const R blo = tb0 <= tb1 ? tb0 : tb1, bhi = tb0 <= tb1 ? tb1 : tb0;
        if (bhi < R(0) || blo > R(1)) {
            push_eval(out, A, B, 0, 0, n0, prediction);
            return;
        }
        if (blo > R(0)) push_eval(out, A, B, 0, flo, n0, prediction);
        else push_eval(out, A, B, 1, 0, n0, prediction);
        if (bhi < R(1)) push_eval(out, A, B, 0, fhi, n0, prediction);
        else push_eval(out, A, B, 2, 0, n0, prediction);
    }
    void push_eval_unique(std::vector<Cand>& out, const Collider<R>& c1, const Collider<R>& c2, int f1, int f2,
                          V3<R> n0, R prediction) const {
        for (const Cand& c : out)
            if (c.fid1 == f1 && c.fid2 == f2) return;
        push_eval(out, c1, c2, f1, f2, n0, prediction);
    }
    // The cuboid edge where face (k, sk) meets the side plane (o, so).
    static int face_side_edge(int k, int sk, int o, int so) {
        const int a = 3 - k - o;
        int o1, o2;
        edge_other_axes(a, o1, o2);
        const int s1 = (o1 == k ? sk : so) > 0 ? 1 : 0, s2 = (o2 == k ? sk : so) > 0 ? 1 : 0;
        return box_edge_id(a, s1, s2);
    }
    static int vertex_at(V3<R> p) { return box_vertex_id(p.x > R(0), p.y > R(0), p.z > R(0)); }
    // Capsule-cuboid: the reference face is the cuboid face farthest from the
    // capsule's axis (the largest of the six face separations of the axis's
    // nearer end); the axis is clipped to that face's rectangle and each end of
    // the clipped axis gives a candidate (a capsule end against the face, or
    // the axis against the clipping edge). When the axis misses the rectangle:
    // each capsule end as a sphere against the cuboid, and the axis against the
    // nearest edge (edge-edge when both closest points are inside their
    // segments; for a parallel axis, the two ends of the overlap).
    void capsule_box(const Collider<R>& cc, const Collider<R>& cx, bool box_first, R prediction,
                     std::vector<Cand>& out) const {
        V3<R> p0, p1;
        capsule_axis(cc, p0, p1);
        const V3<R> l0 = iso_inv_pt(cx.pose, p0), l1 = iso_inv_pt(cx.pose, p1);
        const V3<R> h = cx.half;
        auto cand = [&](int fb, int fc, V3<R> nl) {
            const V3<R> n = qrot(cx.pose.q, nl);
            if (box_first) push_eval_unique(out, cx, cc, fb, fc, n, prediction);
            else push_eval_unique(out, cc, cx, fc, fb, -n, prediction);
        };
        int k = 0, sk = 1;
        R best = -std::numeric_limits<R>::max();
        for (int a = 0; a < 3; ++a) {
            for (int sg = 1; sg >= -1; sg -= 2) {
                const R e0 = R(sg) * comp(l0, a), e1 = R(sg) * comp(l1, a);
                const R sep = (e0 < e1 ? e0 : e1) - comp(h, a);
                if (sep > best) {
                    best = sep;
                    k = a;
                    sk = sg;
                }
            }
        }
        V3<R> nf = v3<R>(R(0), R(0), R(0));
        setc(nf, k, R(sk));
        const int face = box_face_id(k, sk > 0 ? 1 : 0);
        R tlo = R(0), thi = R(1);
        int elo = -1, ehi = -1;
        bool empty = false;
        for (int o = 0; o < 3 && !empty; ++o) {
            if (o == k) continue;
            for (int so = 1; so >= -1 && !empty; so -= 2) {
                const R f0 = R(so) * comp(l0, o) - comp(h, o);
                const R f1 = R(so) * comp(l1, o) - comp(h, o);
                if (f0 > R(0) && f1 > R(0)) {
                    empty = true;
                } else if (f0 > R(0)) {
                    const R t = f0 / (f0 - f1);
                    if (t > tlo) {
                        tlo = t;
                        elo = face_side_edge(k, sk, o, so);
                    }
                } else if (f1 > R(0)) {
                    const R t = f0 / (f0 - f1);
                    if (t < thi) {
                        thi = t;
                        ehi = face_side_edge(k, sk, o, so);
                    }
                }
            }
        }
        if (!empty && tlo <= thi) {
            if (elo < 0) cand(face, 1, nf);
            else cand(elo, 0, nf);
            if (ehi < 0) cand(face, 2, nf);
            else cand(ehi, 0, nf);
            return;
        }
        sphere_box(cc, 1, p0, cx, box_first, prediction, out);
        sphere_box(cc, 2, p1, cx, box_first, prediction, out);
        int be = -1;
        R bd = std::numeric_limits<R>::max(), bp = R(-1), bs = R(0), bt = R(0);
        V3<R> bq = v3<R>(R(0), R(0), R(0)), bqe = bq;
        const V3<R> dl0 = l1 - l0;
        for (int e = 0; e < 12; ++e) {
            const Approx<R> ed = box_feature(h, 8 + e);
            V3<R> qa, qe;
            R sa, te;
            closest_segment_segment(l0, l1, ed.a, ed.b, qa, qe, &sa, &te);
            const V3<R> v = qa - qe;
            const R d2 = dot(v, v);
            const V3<R> de0 = ed.b - ed.a;
            const R c = dot(dl0, de0), par = c * c / (dot(dl0, dl0) * dot(de0, de0) + std::numeric_limits<R>::min());
            if (d2 < bd || (d2 == bd && par > bp)) {
                bp = par;
                bd = d2;
                be = e;
                bs = sa;
                bt = te;
                bq = qa;
                bqe = qe;
            }
        }
        const Approx<R> ed = box_feature(h, 8 + be);
        const V3<R> nl = unit_or(bq - bqe, unit_or(bq, v3<R>(R(0), R(1), R(0))));
        const V3<R> dl = l1 - l0, de = ed.b - ed.a;
        const V3<R> cr = cross(dl, de);
        const R ll2 = dot(dl, dl);
        if (dot(cr, cr) > R(1e-6f) * ll2 * dot(de, de) || ll2 <= std::numeric_limits<R>::epsilon()) {
            if (bs > R(0) && bs < R(1) && bt > R(0) && bt < R(1)) cand(8 + be, 0, nl);
            return;
        }
        const R ta = dot(ed.a - l0, dl) / ll2, tb = dot(ed.b - l0, dl) / ll2;
        const V3<R> vlo = ta <= tb ? ed.a : ed.b, vhi = ta <= tb ? ed.b : ed.a;
        const R lo = ta <= tb ? ta : tb, hi = ta <= tb ? tb : ta;
        if (hi < R(0) || lo > R(1)) return;
        if (lo > R(0)) cand(vertex_at(vlo), 0, nl);
        else cand(8 + be, 1, nl);
        if (hi < R(1)) cand(vertex_at(vhi), 0, nl);
        else cand(8 + be, 2, nl);
    }

    // Cuboid-cuboid: SAT over the 15 axes, then clipping of the incident face
    // against the reference face (Sutherland-Hodgman) with feature tracking.
    void box_box(const Collider<R>& A, const Collider<R>& B, R prediction, std::vector<Cand>& out) const {
        M3<R> RA = qmat(A.pose.q), RB = qmat(B.pose.q);
        V3<R> axA[3] = {mcol(RA, 0), mcol(RA, 1), mcol(RA, 2)};
        V3<R> axB[3] = {mcol(RB, 0), mcol(RB, 1), mcol(RB, 2)};
        V3<R> d = B.pose.t - A.pose.t;
        R sepA = -std::numeric_limits<R>::max(), sepB = sepA, sepE = sepA;
        int ia = 0, ib = 0, ea = -1, eb = -1;
        V3<R> LE = v3<R>(R(0), R(0), R(0));
        for (int i = 0; i < 3; ++i) {
            V3<R> L = axA[i];
            R rb = comp(B.half, 0) * std::fabs(dot(axB[0], L)) + comp(B.half, 1) * std::fabs(dot(axB[1], L)) +
                   comp(B.half, 2) * std::fabs(dot(axB[2], L));
            R sep = std::fabs(dot(d, L)) - (comp(A.half, i) + rb);
            if (sep > prediction) return;
            if (sep > sepA) { sepA = sep; ia = i; }
        }
        for (int j = 0; j < 3; ++j) {
            V3<R> L = axB[j];
            R ra = comp(A.half, 0) * std::fabs(dot(axA[0], L)) + comp(A.half, 1) * std::fabs(dot(axA[1], L)) +
                   comp(A.half, 2) * std::fabs(dot(axA[2], L));
            R sep = std::fabs(dot(d, L)) - (ra + comp(B.half, j));
            if (sep > prediction) return;
            if (sep > sepB) { sepB = sep; ib = j; }
        }
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) {
                V3<R> L = cross(axA[i], axB[j]);
                R len = norm(L);
                if (len < R(1e-5)) continue;
                L = vdiv(L, len);
                R ra = comp(A.half, 0) * std::fabs(dot(axA[0], L)) + comp(A.half, 1) * std::fabs(dot(axA[1], L)) +
                       comp(A.half, 2) * std::fabs(dot(axA[2], L));
                R rb = comp(B.half, 0) * std::fabs(dot(axB[0], L)) + comp(B.half, 1) * std::fabs(dot(axB[1], L)) +
                       comp(B.half, 2) * std::fabs(dot(axB[2], L));
                R sep = std::fabs(dot(d, L)) - (ra + rb);
                if (sep > prediction) return;
                if (sep > sepE) { sepE = sep; ea = i; eb = j; LE = L; }
            }
        }
        bool refA = !(sepB > sepA + R(1e-4));
        R sepF = refA ? sepA : sepB;
        if (ea >= 0 && sepE > sepF + R(5e-3)) {
            // Edge-edge: supporting edges along L (oriented from A to B).
            V3<R> L = LE;
            if (dot(d, L) < R(0)) L = -L;
            int o1, o2;
            edge_other_axes(ea, o1, o2);
            int fa = box_edge_id(ea, dot(axA[o1], L) > R(0) ? 1 : 0, dot(axA[o2], L) > R(0) ? 1 : 0);
            edge_other_axes(eb, o1, o2);
            int fb = box_edge_id(eb, dot(axB[o1], L) < R(0) ? 1 : 0, dot(axB[o2], L) < R(0) ? 1 : 0);
            push_eval(out, A, B, fa, fb, L, prediction);
            return;
        }
        const Collider<R>& Rf = refA ? A : B;
        const Collider<R>& In = refA ? B : A;
        V3<R>* axR = refA ? axA : axB;
        V3<R>* axI = refA ? axB : axA;
        int ri = refA ? ia : ib;
        V3<R> dRI = refA ? d : -d;
        int rpos = dot(dRI, axR[ri]) >= R(0) ? 1 : 0;
        V3<R> nref = rpos ? axR[ri] : -axR[ri];
        int ik = 0;
        R best = std::fabs(dot(axI[0], nref));
        for (int k = 1; k < 3; ++k) {
            R v = std::fabs(dot(axI[k], nref));
            if (v > best) { best = v; ik = k; }
        }
        int ipos = dot(axI[ik], nref) < R(0) ? 1 : 0;
        int ref_face = box_face_id(ri, rpos), inc_face = box_face_id(ik, ipos);
        // Incident face polygon (vertex ids), in the reference box's local frame.
        int u = (ik + 1) % 3, v = (ik + 2) % 3;
        int vids[4];
        int su[4] = {0, 1, 1, 0}, sv[4] = {0, 0, 1, 1};
        struct PV { V3<R> p; int tag, a, b; int esrc; };   // tag 0: inc vertex a; 1: edge-edge (ref a, inc b); 2: ref vertex a
        // esrc >= 0: incident edge id; esrc < 0: -(1 + reference side plane)
        std::vector<PV> poly, next;
        for (int k = 0; k < 4; ++k) {
            int s[3];
            s[ik] = ipos;
            s[u] = su[k];
            s[v] = sv[k];
            vids[k] = box_vertex_id(s[0], s[1], s[2]);
        }
        for (int k = 0; k < 4; ++k) {
            int a = vids[k], b = vids[(k + 1) % 4];
            int diff = a ^ b, axis = diff == 1 ? 0 : (diff == 2 ? 1 : 2), o1, o2;
            edge_other_axes(axis, o1, o2);
            int eid = box_edge_id(axis, (a >> o1) & 1, (a >> o2) & 1);
            Approx<R> ap = box_feature(In.half, a);
            V3<R> w = iso_pt(In.pose, ap.a);
            PV pv;
            pv.p = iso_inv_pt(Rf.pose, w);
            pv.tag = 0; pv.a = a; pv.b = -1; pv.esrc = eid;
            poly.push_back(pv);
        }
        int ru = (ri + 1) % 3, rv = (ri + 2) % 3;
        int planes_axis[4] = {ru, ru, rv, rv};
        int planes_pos[4] = {1, 0, 1, 0};
        for (int pl = 0; pl < 4 && !poly.empty(); ++pl) {
            int ax = planes_axis[pl], pp = planes_pos[pl];
            R hc = comp(Rf.half, ax);
            next.clear();
            size_t n = poly.size();
            for (size_t k = 0; k < n; ++k) {
                const PV& P = poly[k];
                const PV& Q = poly[(k + 1) % n];
                R dp = (pp ? comp(P.p, ax) : -comp(P.p, ax)) - hc;
                R dq = (pp ? comp(Q.p, ax) : -comp(Q.p, ax)) - hc;
                bool pin = dp <= R(0), qin = dq <= R(0);
                if (pin) next.push_back(P);
                if (pin != qin) {
                    R t = dp / (dp - dq);
                    PV X;
                    X.p = P.p + (Q.p - P.p) * t;
                    // Reference edge lying on this side plane of the reference face.
                    int third = 3 - ri - ax;
                    int s[3];
                    s[ri] = rpos;
                    s[ax] = pp;
                    if (P.esrc >= 0) {
                        int o1, o2;
                        edge_other_axes(third, o1, o2);
                        X.tag = 1;
                        X.a = box_edge_id(third, s[o1], s[o2]);
                        X.b = P.esrc;
                    } else {
                        int other_plane = -P.esrc - 1;
                        s[planes_axis[other_plane]] = planes_pos[other_plane];
                        X.tag = 2;
                        X.a = box_vertex_id(s[0], s[1], s[2]);
                        X.b = -1;
                    }
                    if (pin) {
                        // Exit point: the edge that follows runs along this side plane.
                        if (!next.empty()) next.back().esrc = P.esrc;
                        X.esrc = -(1 + pl);
                    } else {
                        X.esrc = P.esrc;
                    }
                    next.push_back(X);
                }
            }
            poly.swap(next);
        }
        V3<R> n0 = refA ? nref : -nref;
        std::vector<Cand> cands;
        for (const PV& P : poly) {
            int fr, fi;
            if (P.tag == 0) { fr = ref_face; fi = P.a; }
            else if (P.tag == 1) { fr = P.a; fi = P.b; }
            else { fr = P.a; fi = inc_face; }
            if (refA) push_eval(cands, A, B, fr, fi, n0, prediction);
            else push_eval(cands, A, B, fi, fr, n0, prediction);
        }
        reduce4(cands, out);
    }

    // Keeps at most 4 contacts: the deepest, the farthest from it, the one
    // spanning the largest triangle with both, and the one that grows that
    // triangle most; the kept contacts stay in clipping order.
    static void reduce4(std::vector<Cand>& c, std::vector<Cand>& out) {
        size_t n = c.size();
        if (n <= 4) {
            for (auto& x : c) out.push_back(x);
            return;
        }
        int i0 = 0;
        for (size_t k = 1; k < n; ++k)
            if (c[k].g.depth > c[i0].g.depth) i0 = int(k);
        int i1 = -1;
        R bd = R(-1);
        for (size_t k = 0; k < n; ++k) {
            if (int(k) == i0) continue;
            R dd = norm2(c[k].g.world1 - c[i0].g.world1);
            if (dd > bd) { bd = dd; i1 = int(k); }
        }
        int i2 = -1;
        R ba = R(-1);
        V3<R> e01 = c[i1].g.world1 - c[i0].g.world1;
        for (size_t k = 0; k < n; ++k) {
            if (int(k) == i0 || int(k) == i1) continue;
            R aa = norm2(cross(e01, c[k].g.world1 - c[i0].g.world1));
            if (aa > ba) { ba = aa; i2 = int(k); }
        }
        int i3 = -1;
        R bs = R(-1);
        V3<R> a = c[i0].g.world1, b = c[i1].g.world1, cc = c[i2].g.world1;
        for (size_t k = 0; k < n; ++k) {
            if (int(k) == i0 || int(k) == i1 || int(k) == i2) continue;
            V3<R> x = c[k].g.world1;
            R s = norm(cross(x - a, x - b)) + norm(cross(x - b, x - cc)) + norm(cross(x - cc, x - a));
            if (s > bs) { bs = s; i3 = int(k); }
        }
        for (size_t k = 0; k < n; ++k)
            if (int(k) == i0 || int(k) == i1 || int(k) == i2 || int(k) == i3) out.push_back(c[k]);
    }

    // One-shot manifold of a pair (c1 < c2). Contacts keep the impulses cached
    // under the same feature key in the pair's previous manifold.
    void narrow_pair(Manifold<R>& m) const {
        const Collider<R>& a = colliders[m.c1];
        const Collider<R>& b = colliders[m.c2];
        R prediction = a.query_limit() + b.query_limit();
        std::vector<Cand> cands;
        if (a.shape == NPGPU_SHAPE_BALL && b.shape == NPGPU_SHAPE_BALL) {
            V3<R> v = b.pose.t - a.pose.t;
            R l2 = dot(v, v);
            V3<R> n0 = l2 > R(0) ? vdiv(v, std::sqrt(l2)) : v3<R>(R(1), R(0), R(0));
            push_eval(cands, a, b, 0, 0, n0, prediction);
        } else if (a.shape == NPGPU_SHAPE_CUBOID && b.shape == NPGPU_SHAPE_BALL) {
            ball_box(b, a, true, prediction, cands);
        } else if (a.shape == NPGPU_SHAPE_BALL && b.shape == NPGPU_SHAPE_CUBOID) {
            ball_box(a, b, false, prediction, cands);
        } else if (a.shape == NPGPU_SHAPE_CAPSULE || b.shape == NPGPU_SHAPE_CAPSULE) {
            if (a.shape == NPGPU_SHAPE_CAPSULE && b.shape == NPGPU_SHAPE_CAPSULE) capsule_capsule(a, b, prediction, cands);
            else if (a.shape == NPGPU_SHAPE_BALL) ball_capsule(a, b, false, prediction, cands);
            else if (b.shape == NPGPU_SHAPE_BALL) ball_capsule(b, a, true, prediction, cands);
            else if (a.shape == NPGPU_SHAPE_CUBOID) capsule_box(b, a, true, prediction, cands);
            else capsule_box(a, b, false, prediction, cands);
        } else {
            box_box(a, b, prediction, cands);
        }
        if (a.sensor || b.sensor) {
            // A proximity pair (ProximityDetector): Intersecting when the
            // shapes touch or overlap, WithinMargin when the contact
            // generator finds them within the query limits, Disjoint
            // otherwise; no contacts.
            uint32_t st = NPGPU_PROXIMITY_DISJOINT;
            for (const Cand& cd : cands) {
                if (cd.g.depth >= R(0)) st = NPGPU_PROXIMITY_INTERSECTING;
                else if (st == NPGPU_PROXIMITY_DISJOINT) st = NPGPU_PROXIMITY_WITHIN_MARGIN;
            }
            m.prox = st;
            m.contacts.clear();
            return;
        }
        std::vector<MContact<R>> nc;
        const Body<R>& b1 = bodies[a.body];
        for (const Cand& cd : cands) {
            MContact<R> k;
            k.g = cd.g;
            k.fid1 = cd.fid1;
            k.fid2 = cd.fid2;
            k.normal1_local = qrot_inv(b1.pos.q, cd.g.normal);
            k.impulse[0] = k.impulse[1] = k.impulse[2] = R(0);
            for (const MContact<R>& old : m.contacts)
                if (old.key() == k.key()) {
                    k.impulse[0] = old.impulse[0];
                    k.impulse[1] = old.impulse[1];
                    k.impulse[2] = old.impulse[2];
                    k.cached = true;
                    break;
                }
            nc.push_back(k);
        }
        m.contacts.swap(nc);
    }

    void collision_detection() {
        sync_colliders();
        broad_phase();
        std::map<uint64_t, Manifold<R>> next;
        for (uint64_t key : pairs) {
            Manifold<R> m;
            auto it = manifolds.find(key);
            const bool had = it != manifolds.end() && !it->second.contacts.empty();
            const uint32_t was = it != manifolds.end() ? it->second.prox : uint32_t(NPGPU_PROXIMITY_DISJOINT);
            if (it != manifolds.end()) m = it->second;
            m.c1 = uint32_t(key >> 32);
            m.c2 = uint32_t(key & 0xffffffffu);
            narrow_pair(m);
            // ContactEvent::Started / Stopped and ProximityEvent of this pass.
            if (record_events && had != !m.contacts.empty()) events.push_back({m.c1, m.c2, had ? 1u : 0u});
            if (record_events && was != m.prox) prox_events.push_back({m.c1, m.c2, was, m.prox});
            next[key] = m;
        }
        if (record_events)
            for (auto& kv : manifolds)
                if (next.find(kv.first) == next.end()) {
                    if (!kv.second.contacts.empty()) events.push_back({kv.second.c1, kv.second.c2, 1u});
                    if (kv.second.prox != NPGPU_PROXIMITY_DISJOINT)
                        prox_events.push_back({kv.second.c1, kv.second.c2, kv.second.prox,
                                               uint32_t(NPGPU_PROXIMITY_DISJOINT)});
                }
        manifolds.swap(next);
        cd_dirty = false;
    }

    // ---- contact events and geometric queries ----
    // GeometricalWorld::contact_events (geometrical_world.rs:373-376): the
    // started / stopped pairs of the step's collision-detection passes,
    // cleared when the step begins (mechanical_world.rs:250).
    bool record_events = false;
    std::vector<std::array<uint32_t, 3>> events;
    // GeometricalWorld::proximity_events (geometrical_world.rs:378-381):
    // (collider1, collider2, previous, new) in the order the passes made them.
    std::vector<std::array<uint32_t, 4>> prox_events;

    // interferences_with_ray (geometrical_world.rs:327-341) for one ray on
    // solid shapes: the sphere's quadratic, or the cuboid's three slabs in its
    // frame (the face of the last slab entered gives the normal).
    // First entry of a ray into a sphere from outside it (-1 when it misses).
    static R ray_sphere_entry(V3<R> o, V3<R> d, V3<R> c, R r) {
        const V3<R> m = o - c;
        const R a = dot(d, d), b = dot(m, d), cc = dot(m, m) - r * r;
        if ((cc > R(0) && b > R(0)) || a == R(0)) return R(-1);
        const R disc = b * b - a * cc;
        if (disc < R(0)) return R(-1);
        return (-b - std::sqrt(disc)) / a;
    }
    bool ray_shape(const Collider<R>& c, V3<R> o, V3<R> d, R max_toi, R& toi, V3<R>& n) const {
        const V3<R> zero = v3<R>(R(0), R(0), R(0));
        if (c.shape == NPGPU_SHAPE_CAPSULE) {
            // The union of the cylinder (clipped to the axis) and the end spheres.
            const V3<R> lo = qrot_inv(c.pose.q, o - c.pose.t), ld = qrot_inv(c.pose.q, d);
            const R r = c.half.x, hh = c.half.y;
            {
                V3<R> qa, qb;
                closest_segment_segment(v3<R>(R(0), -hh, R(0)), v3<R>(R(0), hh, R(0)), lo, lo, qa, qb);
                const V3<R> v = qb - qa;
                if (dot(v, v) <= r * r) {
                    toi = R(0);
                    n = zero;
                    return true;
                }
            }
            R best = std::numeric_limits<R>::infinity();
            V3<R> bn = zero;
            const R a = ld.x * ld.x + ld.z * ld.z;
            if (a > R(0)) {
                const R b = lo.x * ld.x + lo.z * ld.z, cc = lo.x * lo.x + lo.z * lo.z - r * r;
                const R disc = b * b - a * cc;
                if (disc >= R(0)) {
                    const R t = (-b - std::sqrt(disc)) / a;
                    const R y = lo.y + t * ld.y;
                    if (t >= R(0) && std::fabs(y) <= hh) {
                        best = t;
                        bn = vdiv(v3<R>(lo.x + t * ld.x, R(0), lo.z + t * ld.z), r);
                    }
                }
            }
            for (int e = 0; e < 2; ++e) {
                const V3<R> cen = v3<R>(R(0), e ? hh : -hh, R(0));
                const R t = ray_sphere_entry(lo, ld, cen, r);
                if (t >= R(0) && t < best) {
                    best = t;
                    bn = vdiv((lo + ld * t) - cen, r);
                }
            }
            if (!(best <= max_toi)) return false;
            toi = best;
            n = qrot(c.pose.q, bn);
            return true;
        }
        if (c.shape == NPGPU_SHAPE_BALL) {
            const V3<R> m = o - c.pose.t;
            const R a = dot(d, d), b = dot(m, d), cc = dot(m, m) - c.radius * c.radius;
            if (cc > R(0) && b > R(0)) return false;
            const R disc = b * b - a * cc;
            if (disc < R(0) || a == R(0)) {
                if (cc <= R(0)) {
                    toi = R(0);
                    n = zero;
                    return true;
                }
                return false;
            }
            const R t = (-b - std::sqrt(disc)) / a;
            if (t <= R(0)) {
                toi = R(0);
                n = zero;
                return true;
            }
            if (t > max_toi) return false;
            toi = t;
            const V3<R> hit = m + d * t;
            const R l = std::sqrt(dot(hit, hit));
            n = l > R(0) ? vdiv(hit, l) : zero;
            return true;
        }
        const V3<R> lo = qrot_inv(c.pose.q, o - c.pose.t), ld = qrot_inv(c.pose.q, d);
        const R os[3] = {lo.x, lo.y, lo.z}, ds[3] = {ld.x, ld.y, ld.z}, hs[3] = {c.half.x, c.half.y, c.half.z};
        R tmin = -std::numeric_limits<R>::infinity(), tmax = std::numeric_limits<R>::infinity();
        int axis = -1;
        R sign = R(0);
        for (int i = 0; i < 3; ++i) {
            if (ds[i] == R(0)) {
                if (os[i] < -hs[i] || os[i] > hs[i]) return false;
                continue;
            }
            R t1 = (-hs[i] - os[i]) / ds[i], t2 = (hs[i] - os[i]) / ds[i];
            R sg = R(-1);
            if (t1 > t2) {
                std::swap(t1, t2);
                sg = R(1);
            }
            if (t1 > tmin) {
                tmin = t1;
                axis = i;
                sign = sg;
            }
            if (t2 < tmax) tmax = t2;
            if (tmin > tmax) return false;
        }
        if (tmax < R(0)) return false;
        if (tmin <= R(0) || axis < 0) {
            toi = R(0);
            n = zero;
            return true;
        }
        if (tmin > max_toi) return false;
        toi = tmin;
        n = qrot(c.pose.q, v3<R>(axis == 0 ? sign : R(0), axis == 1 ? sign : R(0), axis == 2 ? sign : R(0)));
        return true;
    }
    bool point_in_shape(const Collider<R>& c, V3<R> p) const {
        if (c.shape == NPGPU_SHAPE_BALL) {
            const V3<R> m = p - c.pose.t;
            return dot(m, m) <= c.radius * c.radius;
        }
        if (c.shape == NPGPU_SHAPE_CAPSULE) {
            const V3<R> l = qrot_inv(c.pose.q, p - c.pose.t);
            V3<R> qa, qb;
            closest_segment_segment(v3<R>(R(0), -c.half.y, R(0)), v3<R>(R(0), c.half.y, R(0)), l, l, qa, qb);
            const V3<R> v = qb - qa;
            return dot(v, v) <= c.half.x * c.half.x;
        }
        const V3<R> l = qrot_inv(c.pose.q, p - c.pose.t);
        return std::fabs(l.x) <= c.half.x && std::fabs(l.y) <= c.half.y && std::fabs(l.z) <= c.half.z;
    }
    bool in_world(const Collider<R>& c, uint32_t world) const {
        return world == 0xffffffffu || bodies[c.body].world == world;
    }

    // ------------------------------------------------------- activation
    // ActivationManager::update (src/detection/activation_manager.rs:61-201)
    // with the union-find of src/utils/union_find.rs.
    std::vector<uint32_t> uf_parent, uf_rank;
    uint32_t uf_find(uint32_t x) {
        if (uf_parent[x] != x) uf_parent[x] = uf_find(uf_parent[x]);
        return uf_parent[x];
    }
    void uf_union(uint32_t x, uint32_t y) {
        uint32_t xr = uf_find(x), yr = uf_find(y);
        if (xr == yr) return;
        if (uf_rank[xr] < uf_rank[yr]) uf_parent[xr] = yr;
        else if (uf_rank[xr] > uf_rank[yr]) uf_parent[yr] = xr;
        else { uf_parent[yr] = xr; uf_rank[xr] += 1; }
    }
    void activation_update() {
        R mix = R(params.activation_mix);
        std::vector<int> comp_id(bodies.size(), -1);
        std::vector<uint32_t> id_to_body;
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            Body<R>& b = bodies[i];
            if (!b.alive) continue;
            if (b.ndofs() != 0) {
                if (b.is_active() && b.can_sleep) {
                    R v2 = b.lin.x * b.lin.x + b.lin.y * b.lin.y + b.lin.z * b.lin.z + b.ang.x * b.ang.x +
                         b.ang.y * b.ang.y + b.ang.z * b.ang.z;
                    R e = (R(1) - mix) * b.energy + mix * v2;
                    b.energy = std::min(e, b.sleep_threshold * R(4));
                }
                comp_id[i] = int(id_to_body.size());
                id_to_body.push_back(i);
            }
            if (b.kinematic()) {
                comp_id[i] = int(id_to_body.size());
                id_to_body.push_back(i);
            }
        }
        uf_parent.resize(id_to_body.size());
        uf_rank.assign(id_to_body.size(), 0);
        for (uint32_t i = 0; i < id_to_body.size(); ++i) uf_parent[i] = i;
        for (auto& kv : manifolds) {
            const Manifold<R>& m = kv.second;
            if (m.contacts.empty()) continue;
            int a = comp_id[colliders[m.c1].body], b = comp_id[colliders[m.c2].body];
            if (a >= 0 && b >= 0) uf_union(uint32_t(a), uint32_t(b));
        }
        for (const Joint<R>& j : joints) {   // activation_manager.rs:154-159
            if (!j.alive || j.broken) continue;
            int a = comp_id[j.b1], b = comp_id[j.b2];
            if (a >= 0 && b >= 0) uf_union(uint32_t(a), uint32_t(b));
        }
        std::vector<char> can_deactivate(id_to_body.size(), 1);
        for (uint32_t i = 0; i < id_to_body.size(); ++i) {
            uint32_t root = uf_find(i);
            const Body<R>& b = bodies[id_to_body[i]];
            can_deactivate[root] = b.can_sleep ? (can_deactivate[root] && b.energy < b.sleep_threshold) : 0;
        }
        for (auto& b : bodies) b.in_island = false;
        for (uint32_t i = 0; i < id_to_body.size(); ++i) {
            uint32_t root = uf_find(i);
            Body<R>& b = bodies[id_to_body[i]];
            if (can_deactivate[root]) {
                if (b.is_active()) deactivate(b);
            } else if (!b.kinematic()) {
                b.in_island = true;
                if (!(b.energy != R(0)) && b.can_sleep) activate(b);
            }
        }
    }

    // ------------------------------------------------------- solver
    static R combine(R a, uint32_t ma, R b, uint32_t mb) {   // MaterialCombineMode::combine (material.rs:71-86)
        if (ma == NPGPU_COMBINE_MAX || mb == NPGPU_COMBINE_MAX) return std::max(a, b);
        if (ma == NPGPU_COMBINE_MULTIPLY || mb == NPGPU_COMBINE_MULTIPLY) return a * b;
        if (ma == NPGPU_COMBINE_MIN || mb == NPGPU_COMBINE_MIN) return std::min(a, b);
        return (a + b) * R(0.5);
    }

    // RigidBody::fill_constraint_geometry (rigid_body.rs:672-722).
    // The side's unit force f: ForceDirection::at_point (helper.rs:24-33).
    void fill(const Body<R>& b, V3<R> point, V3<R> dir, R* J, R* WJ, R& inv_r, R& rhs, bool with_ext) const {
        V3<R> pos = point - b.com;
        V3<R> fl = dir, fa = cross(pos, dir);
        const R f[6] = {fl.x, fl.y, fl.z, fa.x, fa.y, fa.z};
        fill_force(b, f, J, WJ, inv_r, rhs, with_ext);
    }
    void fill_torque(const Body<R>& b, V3<R> axis, R* J, R* WJ, R& inv_r, R& rhs, bool with_ext) const {
        const R f[6] = {R(0), R(0), R(0), axis.x, axis.y, axis.z};
        fill_force(b, f, J, WJ, inv_r, rhs, with_ext);
    }
    void fill_force(const Body<R>& b, const R* f, R* J, R* WJ, R& inv_r, R& rhs, bool with_ext) const {
        R mf[6];
        for (int k = 0; k < 6; ++k) mf[k] = f[k] * b.mask[k];
        R vel[6] = {b.lin.x, b.lin.y, b.lin.z, b.ang.x, b.ang.y, b.ang.z};
        if (b.status == NPGPU_BODY_KINEMATIC) {
            R s = R(0);
            for (int k = 0; k < 6; ++k) s = s + f[k] * vel[k];
            rhs = rhs + s;
        } else if (b.status == NPGPU_BODY_DYNAMIC) {
            for (int k = 0; k < 6; ++k) J[k] = mf[k];
            V3<R> ml = v3<R>(mf[0], mf[1], mf[2]), ma = v3<R>(mf[3], mf[4], mf[5]);
            V3<R> wl = ml * b.inv_aug.linear;
            V3<R> wa = mv(b.inv_aug.angular, ma);
            WJ[0] = wl.x; WJ[1] = wl.y; WJ[2] = wl.z; WJ[3] = wa.x; WJ[4] = wa.y; WJ[5] = wa.z;
            inv_r = inv_r + (b.inv_aug.linear + dot(ma, wa));
            R s = R(0);
            for (int k = 0; k < 6; ++k) s = s + f[k] * vel[k];
            rhs = rhs + s;
            if (with_ext) {
                R dt = cur_dt;
                R ext[6] = {b.acc_lin.x * dt, b.acc_lin.y * dt, b.acc_lin.z * dt,
                            b.acc_ang.x * dt, b.acc_ang.y * dt, b.acc_ang.z * dt};
                R e = R(0);
                for (int k = 0; k < 6; ++k) e = e + mf[k] * ext[k];
                rhs = rhs + e;
            }
        }
    }

    // helper::constraint_pair_geometry (solver/helper.rs:53-135) for one row.
    Row<R> make_row(const Body<R>& b1, uint32_t s1, const Body<R>& b2, uint32_t s2, V3<R> center1, V3<R> center2,
                    V3<R> dir, R rhs0) const {
        Row<R> r;
        std::memset(&r, 0, sizeof(r));
        r.b1 = b1.dynamic() ? int(s1) : -1;
        r.b2 = b2.dynamic() ? int(s2) : -1;
        R inv_r = R(0), rhs = rhs0;
        fill(b1, center1, dir, r.J1, r.WJ1, inv_r, rhs, true);
        fill(b2, center2, -dir, r.J2, r.WJ2, inv_r, rhs, true);
        r.r = (inv_r != R(0)) ? R(1) / inv_r : R(1);
        r.rhs = rhs;
        return r;
    }

    // constraint_pair_geometry for ForceDirection::Angular(axis).
    Row<R> make_row_angular(const Body<R>& b1, uint32_t s1, const Body<R>& b2, uint32_t s2, V3<R> axis) const {
        Row<R> r;
        std::memset(&r, 0, sizeof(r));
        r.b1 = b1.dynamic() ? int(s1) : -1;
        r.b2 = b2.dynamic() ? int(s2) : -1;
        R inv_r = R(0), rhs = R(0);
        fill_torque(b1, axis, r.J1, r.WJ1, inv_r, rhs, true);
        fill_torque(b2, -axis, r.J2, r.WJ2, inv_r, rhs, true);
        r.r = (inv_r != R(0)) ? R(1) / inv_r : R(1);
        r.rhs = rhs;
        return r;
    }

    // nalgebra Vector3::orthonormal_subspace_basis for one vector.
    static void tangent_basis(V3<R> n, V3<R>& t1, V3<R>& t2) {
        V3<R> a;
        if (std::fabs(n.x) > std::fabs(n.y)) a = v3<R>(n.z, R(0), -n.x);
        else a = v3<R>(R(0), -n.z, n.y);
        t1 = vdiv(a, norm(a));
        V3<R> b = cross(n, a);
        t2 = vdiv(b, norm(b));
    }

    // ---- learned warm start (the network of the GPU's npgpu_mlp_*) ----
    // Parameters in the fp32 layout W1[64][24] b1[64] W2[64][64] b2[64]
    // W3[3][64] b3[3] x_mean[24] x_inv_std[24] y_mean[3] y_std[3]; the
    // weights as the forward pass reads them are rounded to bf16.
    std::vector<float> mlp;
    static float bf16_round(float v) {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        if ((u & 0x7f800000u) != 0x7f800000u) {   // finite: round to nearest, ties to even
            u += 0x7fffu + ((u >> 16) & 1u);
        }
        u &= 0xffff0000u;
        float r;
        std::memcpy(&r, &u, 4);
        return r;
    }
    void set_mlp(const float* p, size_t n) {
        mlp.assign(p, p + n);
        for (size_t i = 0; i < n; ++i) {
            bool weight = i < 1536 || (i >= 1600 && i < 1600 + 4096) || (i >= 5760 && i < 5760 + 192);
            if (weight) mlp[i] = bf16_round(mlp[i]);
        }
    }
    // Forward pass in fp32 with sums in index order (no fused multiply-add).
    void mlp_forward(const float* feat, float* out) const {
        const float* W1 = mlp.data();
        const float* b1 = W1 + 1536;
        const float* W2 = b1 + 64;
        const float* b2 = W2 + 4096;
        const float* W3 = b2 + 64;
        const float* b3 = W3 + 192;
        const float* xm = b3 + 3;
        const float* xs = xm + 24;
        const float* ym = xs + 24;
        const float* ys = ym + 3;
        float x[24], h1[64], y[3];
        for (int i = 0; i < 24; ++i) x[i] = (feat[i] - xm[i]) * xs[i];
        for (int j = 0; j < 64; ++j) {
            float a = b1[j];
            for (int i = 0; i < 24; ++i) a = a + W1[j * 24 + i] * x[i];
            h1[j] = a > 0.0f ? a : 0.0f;
        }
        for (int o = 0; o < 3; ++o) y[o] = b3[o];
        for (int j = 0; j < 64; ++j) {
            float a = b2[j];
            for (int i = 0; i < 64; ++i) a = a + W2[j * 64 + i] * h1[i];
            float h = a > 0.0f ? a : 0.0f;
            for (int o = 0; o < 3; ++o) y[o] = y[o] + W3[o * 64 + j] * h;
        }
        for (int o = 0; o < 3; ++o) out[o] = y[o] * ys[o] + ym[o];
    }
    // The 24 contact features (see the GPU's mlp_features for the list).
    static void mlp_features(const Row<R>* rows3, R depth, R im1, R im2, R mu, R gn_dt, R nc, R k1, R k2, R* f) {
        for (int r = 0; r < 3; ++r) {
            f[r] = rows3[r].rhs;
            f[3 + r] = rows3[r].r;
        }
        f[6] = depth;
        f[7] = im1;
        f[8] = im2;
        for (int r = 0; r < 3; ++r) {
            R a1 = R(0), a2 = R(0);
            for (int k = 3; k < 6; ++k) {
                a1 = a1 + rows3[r].J1[k] * rows3[r].WJ1[k];
                a2 = a2 + rows3[r].J2[k] * rows3[r].WJ2[k];
            }
            f[9 + r] = a1;
            f[12 + r] = a2;
        }
        f[15] = mu;
        f[16] = gn_dt;
        f[17] = nc;
        f[18] = k1;
        f[19] = k2;
        R iso = -(f[3] * f[0]);
        f[20] = iso > R(0) ? iso : R(0);
        f[21] = -(f[4] * f[1]);
        f[22] = -(f[5] * f[2]);
        f[23] = f[3] * gn_dt;
    }
    // Squared residual of one contact's rows (normal, tangent 1, tangent 2)
    // at the current Δv for impulses lam.
    R local_residual(const Row<R>* r3, const R* lam) const {
        R s = R(0);
        {
            R d = jdot(r3[0]) + r3[0].rhs;
            R x = lam[0] - r3[0].r * d;
            R pr = x > R(0) ? x : R(0);
            R phi = lam[0] - pr;
            s = s + phi * phi;
        }
        R lim = r3[1].mu * lam[0];
        for (int k = 1; k < 3; ++k) {
            R d = jdot(r3[k]) + r3[k].rhs;
            R x = lam[k] - r3[k].r * d;
            R pr = x < -lim ? -lim : (x > lim ? lim : x);
            R phi = lam[k] - pr;
            s = s + phi * phi;
        }
        return s;
    }

    std::vector<Row<R>> rows;
    std::vector<PosConstraint<R>> pos_constraints;
    std::vector<int> seq_warm, seq_friction, seq_normal, seq_pos;
    // NPGPU_SWEEP_MANIFOLD: per manifold (in the order of `seq`), its friction
    // rows, then its normal rows.
    std::vector<int> seq_merged;
    std::vector<Manifold<R>*> solver_manifolds;

    // A solver item: a contact manifold or an active joint, with its two
    // bodies and its Jones-Plassmann priority.
    struct Item {
        Manifold<R>* m = nullptr;
        int joint = -1;
        uint32_t b1 = 0, b2 = 0;
        uint64_t prio = 0;
        uint32_t colour = 0xffffffffu;
    };

    // JP colouring with first-fit colours (the GPU solver's schedule), at
    // most kOracleColours colours (the GPU keeps a body's colour mask in two
    // 56-bit words). Priorities: a manifold hashes its colliders' world-local
    // slots; a joint hashes its world-local joint slot with a second input no
    // collider pair has (the GPU's joint_priority).
    static constexpr uint32_t kOracleColours = 112;
    uint32_t colour_items(std::vector<Item>& items) {
        std::vector<uint32_t> base, local(colliders.size());
        for (uint32_t c = 0; c < colliders.size(); ++c) {
            if (!colliders[c].alive) continue;
            uint32_t wd = bodies[colliders[c].body].world;
            if (wd >= base.size()) base.resize(wd + 1, 0xffffffffu);
            base[wd] = std::min(base[wd], c);
        }
        for (uint32_t c = 0; c < colliders.size(); ++c) {
            uint32_t wd = colliders[c].alive ? bodies[colliders[c].body].world : 0xffffffffu;
            local[c] = (wd < base.size() && base[wd] <= c) ? c - base[wd] : c;
        }
        std::vector<uint32_t> jbase, jlocal(joints.size());
        for (uint32_t j = 0; j < joints.size(); ++j) {
            if (!joints[j].alive) continue;
            uint32_t wd = bodies[joints[j].b1].world;
            if (wd >= jbase.size()) jbase.resize(wd + 1, 0xffffffffu);
            jbase[wd] = std::min(jbase[wd], j);
        }
        for (uint32_t j = 0; j < joints.size(); ++j) {
            uint32_t wd = joints[j].alive ? bodies[joints[j].b1].world : 0xffffffffu;
            jlocal[j] = (wd < jbase.size() && jbase[wd] <= j) ? j - jbase[wd] : j;
        }
        for (Item& it : items) {
            if (it.joint >= 0)
                it.prio = (uint64_t(pair_hash22(jlocal[it.joint], 0x3fffffu)) << 42) | (uint64_t(0x1fffff) << 21) |
                          uint64_t(it.joint);
            else
                it.prio = pair_priority(local[it.m->c1], local[it.m->c2], it.m->c1, it.m->c2);
        }
        std::vector<uint64_t> best(bodies.size(), 0);
        std::vector<uint64_t> used(2 * bodies.size(), 0);   // colours 0-63 and 64-127 of each body
        std::vector<Item*> todo;
        for (Item& it : items) todo.push_back(&it);
        uint32_t ncol = 0;
        while (!todo.empty()) {
            for (Item* m : todo) {
                if (bodies[m->b1].dynamic()) best[m->b1] = std::max(best[m->b1], m->prio);
                if (bodies[m->b2].dynamic()) best[m->b2] = std::max(best[m->b2], m->prio);
            }
            std::vector<Item*> rest, won;
            for (Item* m : todo) {
                bool w = (!bodies[m->b1].dynamic() || best[m->b1] == m->prio) &&
                         (!bodies[m->b2].dynamic() || best[m->b2] == m->prio);
                (w ? won : rest).push_back(m);
            }
            for (Item* m : won) {
                uint64_t mask[2] = {0, 0};
                for (int h = 0; h < 2; ++h) {
                    if (bodies[m->b1].dynamic()) mask[h] |= used[2 * m->b1 + h];
                    if (bodies[m->b2].dynamic()) mask[h] |= used[2 * m->b2 + h];
                }
                uint32_t c = 0;
                while (c < kOracleColours && (mask[c >> 6] >> (c & 63u)) & 1u) ++c;
                m->colour = c;
                if (m->m) m->m->colour = c;
                if (c >= kOracleColours) continue;
                if (bodies[m->b1].dynamic()) used[2 * m->b1 + (c >> 6)] |= (uint64_t(1) << (c & 63u));
                if (bodies[m->b2].dynamic()) used[2 * m->b2 + (c >> 6)] |= (uint64_t(1) << (c & 63u));
                ncol = std::max(ncol, c + 1);
            }
            for (Item* m : todo) {
                best[m->b1] = 0;
                best[m->b2] = 0;
            }
            todo.swap(rest);
        }
        return ncol;
    }

    // Unit::try_new_and_get(v, eps): v / |v| when |v|^2 > eps^2.
    static bool unit_try(V3<R> v, R eps, V3<R>& u, R& n) {
        const R sq = dot(v, v);
        if (!(sq > eps * eps)) return false;
        n = std::sqrt(sq);
        u = vdiv(v, n);
        return true;
    }
    static V3<R> basis(int r) { return v3<R>(r == 0 ? R(1) : R(0), r == 1 ? R(1) : R(0), r == 2 ? R(1) : R(0)); }

    // A joint's row group: `rows` forces along (linear) or torques about the
    // directions d; a limit group's impulse stays in [0, max].
    struct JointGroup {
        bool angular;
        int rows;
        bool limit;
        V3<R> d[3];
    };
    // The impulse slot row r of group g starts from (store false) and is
    // cached to (store true): 0-2 linear, 3-5 angular, 6 the prismatic
    // limit's. The cylindrical and pin-slot joints number their angular rows
    // from DIM - 1 (cylindrical_constraint.rs, pin_slot_constraint.rs): they
    // start from angular impulses 0 and 1 and are cached to linear impulse 2
    // and angular impulse 0.
    static int joint_slot(uint32_t kind, int g, int r, bool store) {
        switch (kind) {
        case NPGPU_JOINT_CYLINDRICAL:
        case NPGPU_JOINT_PIN_SLOT:
            if (g == 1) return store ? (r == 0 ? 2 : 3) : 3 + r;
            return r;
        case NPGPU_JOINT_PRISMATIC: return g == 0 ? r : (g == 1 ? 3 + r : 6);
        case NPGPU_JOINT_CARTESIAN: return 3 + r;
        default: return g == 0 ? r : 3 + r;
        }
    }
    // relative_eq! with approx's default epsilon and max relative difference.
    static bool relative_eq(R a, R b) {
        const R eps = std::numeric_limits<R>::epsilon();
        const R d = std::fabs(a - b);
        if (d <= eps) return true;
        return d <= std::max(std::fabs(a), std::fabs(b)) * eps;
    }
    // The row groups of a joint kind as each constraint's velocity_constraints
    // builds them (ball_constraint.rs:80-127, fixed_constraint.rs:107-172,
    // revolute_constraint.rs:181-266, cartesian_constraint.rs,
    // planar_constraint.rs, rectangular_constraint.rs, universal_constraint.rs,
    // prismatic_constraint.rs, cylindrical_constraint.rs,
    // pin_slot_constraint.rs) from helper.rs:167-296, 422-551, 614-857 and the
    // prismatic offset limit (unit_constraint.rs:33-123); the subspace basis
    // of an axis is the contact model's tangent basis.
    int joint_groups(const Joint<R>& jt, Quat<R> q1, Quat<R> q2, V3<R> a1, V3<R> a2, JointGroup* g) const {
        const V3<R> ex = basis(0), ey = basis(1), ez = basis(2), zero = v3<R>(R(0), R(0), R(0));
        const JointGroup lin3{false, 3, false, {ex, ey, ez}}, ang3{true, 3, false, {ex, ey, ez}};
        switch (jt.kind) {
        case NPGPU_JOINT_BALL: g[0] = lin3; return 1;
        case NPGPU_JOINT_FIXED: g[0] = lin3; g[1] = ang3; return 2;
        case NPGPU_JOINT_CARTESIAN: g[0] = ang3; return 1;
        case NPGPU_JOINT_REVOLUTE: {
            V3<R> t1, t2;
            tangent_basis(qrot(q1, jt.axis1), t1, t2);
            g[0] = lin3;
            g[1] = JointGroup{true, 2, false, {t1, t2, zero}};
            return 2;
        }
        case NPGPU_JOINT_PLANAR: {
            const V3<R> a = qrot(q1, jt.axis1);
            V3<R> t1, t2;
            tangent_basis(a, t1, t2);
            g[0] = JointGroup{false, 1, false, {a, zero, zero}};
            g[1] = JointGroup{true, 2, false, {t1, t2, zero}};
            return 2;
        }
        case NPGPU_JOINT_RECTANGULAR:
            g[0] = JointGroup{false, 1, false, {qrot(q1, jt.axis1), zero, zero}};
            g[1] = ang3;
            return 2;
        case NPGPU_JOINT_UNIVERSAL: {
            V3<R> o;
            R n;
            const bool has = unit_try(cross(qrot(q1, jt.axis1), qrot(q2, jt.axis2)),
                                      std::numeric_limits<R>::epsilon(), o, n);
            g[0] = lin3;
            g[1] = JointGroup{true, has ? 1 : 0, false, {has ? o : zero, zero, zero}};
            return 2;
        }
        case NPGPU_JOINT_PRISMATIC: {
            const V3<R> a = qrot(q1, jt.axis1);
            V3<R> t1, t2;
            tangent_basis(a, t1, t2);
            g[0] = JointGroup{false, 2, false, {t1, t2, zero}};
            g[1] = ang3;
            const R offset = dot(a, a2 - a1);
            g[2] = JointGroup{false, 0, true, {zero, zero, zero}};
            if (jt.has_min && jt.has_max && relative_eq(jt.min_offset, jt.max_offset)) {
                g[2] = JointGroup{false, 1, false, {a, zero, zero}};
            } else if (jt.has_min && offset <= jt.min_offset) {
                g[2] = JointGroup{false, 1, true, {-a, zero, zero}};
            } else if (jt.has_max && offset >= jt.max_offset) {
                g[2] = JointGroup{false, 1, true, {a, zero, zero}};
            }
            return 3;
        }
        default: {   // cylindrical, pin-slot
            const V3<R> al = qrot(q1, jt.axis1), aa = qrot(q1, jt.kind == NPGPU_JOINT_PIN_SLOT ? jt.axis3 : jt.axis1);
            V3<R> t1, t2, u1, u2;
            tangent_basis(al, t1, t2);
            tangent_basis(aa, u1, u2);
            g[0] = JointGroup{false, 2, false, {t1, t2, zero}};
            g[1] = JointGroup{true, 2, false, {u1, u2, zero}};
            return 2;
        }
        }
    }

    // The rows of active joint j: one bilateral row per direction, started
    // from the joint's impulse.
    void joint_rows(uint32_t j, std::vector<int>& out) {
        const Joint<R>& jt = joints[j];
        const Body<R>& b1 = bodies[jt.b1];
        const Body<R>& b2 = bodies[jt.b2];
        const V3<R> a1 = iso_pt(b1.pos, jt.anchor1), a2 = iso_pt(b2.pos, jt.anchor2);
        JointGroup g[3];
        const int ng = joint_groups(jt, b1.pos.q, b2.pos.q, a1, a2, g);
        for (int t = 0; t < ng; ++t)
            for (int r = 0; r < g[t].rows; ++r) {
                Row<R> row = g[t].angular ? make_row_angular(b1, jt.b1, b2, jt.b2, g[t].d[r])
                                          : make_row(b1, jt.b1, b2, jt.b2, a1, a2, g[t].d[r], R(0));
                row.impulse = jt.imp[joint_slot(jt.kind, t, r, false)];
                row.bilateral = true;
                row.limit = g[t].limit;
                row.joint = int(j);
                row.joint_slot = joint_slot(jt.kind, t, r, true);
                row.cache = nullptr;
                out.push_back(int(rows.size()));
                rows.push_back(row);
            }
    }

    // MoreauJeanSolver::assemble_system + SignoriniCoulombPyramidModel::constraints
    // (moreau_jean_solver.rs:129-260, signorini_coulomb_pyramid_model.rs:56-224,
    // signorini_model.rs:37-197).
    bool assemble() {
        rows.clear();
        pos_constraints.clear();
        seq_warm.clear(); seq_friction.clear(); seq_normal.clear(); seq_pos.clear(); seq_merged.clear();
        solver_manifolds.clear();
        // Manifold collection (mechanical_world.rs:287-300).
        for (auto& kv : manifolds) {
            Manifold<R>& m = kv.second;
            m.colour = 0xffffffffu;
            m.in_solver = false;
            if (m.contacts.empty()) continue;
            const Body<R>& b1 = bodies[colliders[m.c1].body];
            const Body<R>& b2 = bodies[colliders[m.c2].body];
            if (b1.status == NPGPU_BODY_DISABLED || b2.status == NPGPU_BODY_DISABLED) continue;
            if ((b1.ndofs() != 0 && b1.is_active()) || (b2.ndofs() != 0 && b2.is_active())) {
                m.in_solver = true;
                solver_manifolds.push_back(&m);
            }
        }
        num_solver_contacts = 0;
        for (const Manifold<R>* m : solver_manifolds) num_solver_contacts += uint32_t(m->contacts.size());
        // Active joints (mechanical_world.rs:274-279, joint_constraint.rs:218-227),
        // in slot order (the arena's iteration order).
        std::vector<Item> items;
        for (Manifold<R>* m : solver_manifolds) {
            Item it;
            it.m = m;
            it.b1 = colliders[m->c1].body;
            it.b2 = colliders[m->c2].body;
            items.push_back(it);
        }
        for (uint32_t j = 0; j < joints.size(); ++j) {
            Joint<R>& jt = joints[j];
            jt.active = false;
            if (!jt.alive || jt.broken) continue;
            const Body<R>& b1 = bodies[jt.b1];
            const Body<R>& b2 = bodies[jt.b2];
            if ((b1.ndofs() != 0 && b1.is_active()) || (b2.ndofs() != 0 && b2.is_active())) {
                jt.active = true;
                Item it;
                it.joint = int(j);
                it.b1 = jt.b1;
                it.b2 = jt.b2;
                items.push_back(it);
            }
        }
        num_colours = 0;
        if (order == ORDER_COLOUR) {
            num_colours = colour_items(items);
            if (std::any_of(items.begin(), items.end(), [](const Item& m) { return m.colour >= kOracleColours; })) {
                last_error = "colour overflow";
                return false;
            }
            std::stable_sort(items.begin(), items.end(),
                             [](const Item& a, const Item& b) { return a.colour < b.colour; });
        }
        std::vector<Manifold<R>*> seq;
        for (const Item& it : items)
            if (it.m) seq.push_back(it.m);
        R inv_dt = (params.dt == 0.0f) ? R(0) : R(1) / R(params.dt);
        // Learned starts: mode 2 for contacts without a cache entry, mode 3
        // for every contact.
        const bool learned = params.warmstart_mode == 2 || params.warmstart_mode == 3;
        if (learned && (mlp.size() != 6009 || order != ORDER_COLOUR)) {
            last_error = "learned warm start needs a network and the colour order";
            return false;
        }
        std::vector<uint32_t> kb(bodies.size(), 0);   // solver manifolds (and joints) per dynamic body
        for (const Item& it : items) {
            if (bodies[it.b1].dynamic()) ++kb[it.b1];
            if (bodies[it.b2].dynamic()) ++kb[it.b2];
        }
        std::vector<int> ug, un, bg, bn;   // unilateral ground / non-ground, bilateral ...
        std::vector<int> jn, jg;           // joint rows, non-ground / ground
        std::vector<int> jpos;             // joints' position constraints (reference order)
        for (const Item& item : items) {
            if (item.joint >= 0) {
                // A joint: its rows run with the friction rows (colour order),
                // or before them (SORProx::step, sor_prox.rs:159-179).
                std::vector<int> jr;
                joint_rows(uint32_t(item.joint), jr);
                PosConstraint<R> pc{};
                pc.joint = item.joint;
                pos_constraints.push_back(pc);
                const int pi = int(pos_constraints.size()) - 1;
                if (order == ORDER_COLOUR) {
                    for (int i : jr) {
                        seq_warm.push_back(i);
                        seq_friction.push_back(i);
                    }
                    seq_pos.push_back(pi);
                } else {
                    const bool ground = bodies[item.b1].ndofs() == 0 || bodies[item.b2].ndofs() == 0;
                    for (int i : jr) (ground ? jg : jn).push_back(i);
                    jpos.push_back(pi);
                }
                seq_merged.insert(seq_merged.end(), jr.begin(), jr.end());
                continue;
            }
            Manifold<R>* m = item.m;
            const Collider<R>& c1 = colliders[m->c1];
            const Collider<R>& c2 = colliders[m->c2];
            const Body<R>& b1 = bodies[c1.body];
            const Body<R>& b2 = bodies[c2.body];
            R mu = combine(c1.friction, c1.friction_combine, c2.friction, c2.friction_combine);
            R e = combine(c1.restitution, c1.restitution_combine, c2.restitution, c2.restitution_combine);
            bool ground = b1.ndofs() == 0 || b2.ndofs() == 0;
            std::vector<int> m_friction, m_normal;
            for (MContact<R>& k : m->contacts) {
                V3<R> n = k.g.normal;
                V3<R> center1 = k.g.world1 + n * c1.margin;
                V3<R> center2 = k.g.world2 - n * c2.margin;
                // Normal row (SignoriniModel::build_velocity_constraint).
                Row<R> rn = make_row(b1, c1.body, b2, c2.body, center1, center2, -n, R(0));
                if (rn.rhs <= -R(params.restitution_velocity_threshold)) rn.rhs = rn.rhs + e * rn.rhs;
                R depth = k.g.depth + c1.margin + c2.margin;
                if (depth < R(0)) rn.rhs = rn.rhs + (-depth) * inv_dt;
                rn.impulse = k.impulse[0] * R(params.warmstart_coeff);
                if (params.warmstart_mode == 1) rn.impulse = R(0);
                rn.friction = false;
                rn.cache = &k;
                rn.cache_slot = 0;
                int in = int(rows.size());
                rows.push_back(rn);
                pos_constraints.push_back(PosConstraint<R>{m->c1, m->c2, k.fid1, k.fid2, k.normal1_local});
                V3<R> t[2];
                tangent_basis(n, t[0], t[1]);
                int it[2];
                for (int s = 0; s < 2; ++s) {
                    Row<R> rt = make_row(b1, c1.body, b2, c2.body, center1, center2, t[s], R(0));
                    rt.impulse = k.impulse[1 + s] * R(params.warmstart_coeff);
                    if (params.warmstart_mode == 1) rt.impulse = R(0);
                    rt.friction = true;
                    rt.dep = in;
                    rt.mu = mu;
                    rt.cache = &k;
                    rt.cache_slot = 1 + s;
                    it[s] = int(rows.size());
                    rows.push_back(rt);
                }
                if (learned && (!k.cached || params.warmstart_mode == 3)) {
                    Row<R> r3[3] = {rows[in], rows[it[0]], rows[it[1]]};
                    R f[24];
                    R gn_dt = (gravity.x * n.x + gravity.y * n.y + gravity.z * n.z) * R(params.dt);
                    R im1 = b1.dynamic() ? b1.inv_aug.linear : R(0), im2 = b2.dynamic() ? b2.inv_aug.linear : R(0);
                    mlp_features(r3, depth, im1, im2, mu, gn_dt, R(m->contacts.size()),
                                 b1.dynamic() ? R(kb[c1.body]) : R(0), b2.dynamic() ? R(kb[c2.body]) : R(0), f);
                    float ff[24], pl[3];
                    for (int i = 0; i < 24; ++i) ff[i] = float(f[i]);
                    mlp_forward(ff, pl);
                    float ln = pl[0] > 0.0f ? pl[0] : 0.0f;
                    float mx = float(mu) * ln;
                    pl[0] = ln;
                    for (int q = 1; q < 3; ++q) pl[q] = pl[q] < -mx ? -mx : (pl[q] > mx ? mx : pl[q]);
                    const bool fresh = !k.cached;
                    rows[in].alt[0] = fresh ? R(0) : rows[in].impulse;
                    rows[in].alt[1] = fresh ? R(0) : rows[it[0]].impulse;
                    rows[in].alt[2] = fresh ? R(0) : rows[it[1]].impulse;
                    rows[in].impulse = R(pl[0]);
                    rows[it[0]].impulse = R(pl[1]);
                    rows[it[1]].impulse = R(pl[2]);
                    rows[in].predicted = true;
                }
                if (order == ORDER_COLOUR) {
                    seq_warm.push_back(in);
                    seq_warm.push_back(it[0]);
                    seq_warm.push_back(it[1]);
                    seq_friction.push_back(it[0]);
                    seq_friction.push_back(it[1]);
                    seq_normal.push_back(in);
                } else {
                    (ground ? ug : un).push_back(in);
                    (ground ? bg : bn).push_back(it[0]);
                    (ground ? bg : bn).push_back(it[1]);
                }
                m_friction.push_back(it[0]);
                m_friction.push_back(it[1]);
                m_normal.push_back(in);
                seq_pos.push_back(int(pos_constraints.size()) - 1);
            }
            seq_merged.insert(seq_merged.end(), m_friction.begin(), m_friction.end());
            seq_merged.insert(seq_merged.end(), m_normal.begin(), m_normal.end());
        }
        if (order == ORDER_REFERENCE) {
            // SORProx::warmstart_set / step (sor_prox.rs:19-45, 159-179):
            // the contacts' warm start, then the joints'; each iteration the
            // joints' bilateral rows, the contacts' friction rows, then the
            // contacts' normal rows. NonlinearSORProx::solve takes the joints
            // before the contacts (nonlinear_sor_prox.rs:33-54).
            for (int i : un) seq_warm.push_back(i);
            for (int i : ug) seq_warm.push_back(i);
            for (int i : bn) seq_warm.push_back(i);
            for (int i : bg) seq_warm.push_back(i);
            for (int i : jn) seq_warm.push_back(i);
            for (int i : jg) seq_warm.push_back(i);
            for (int i : jn) seq_friction.push_back(i);
            for (int i : jg) seq_friction.push_back(i);
            for (int i : bn) seq_friction.push_back(i);
            for (int i : bg) seq_friction.push_back(i);
            for (int i : un) seq_normal.push_back(i);
            for (int i : ug) seq_normal.push_back(i);
            seq_pos.insert(seq_pos.begin(), jpos.begin(), jpos.end());
        }
        return true;
    }

    std::vector<R> dv;   // mj_lambda, 6 per body slot

    R jdot(const Row<R>& r) const {
        R d = R(0);
        if (r.b1 >= 0 && r.b2 >= 0) {
            R s1 = R(0), s2 = R(0);
            for (int k = 0; k < 6; ++k) s1 = s1 + r.J1[k] * dv[6 * r.b1 + k];
            for (int k = 0; k < 6; ++k) s2 = s2 + r.J2[k] * dv[6 * r.b2 + k];
            d = s1 + s2;
        } else if (r.b1 >= 0) {
            for (int k = 0; k < 6; ++k) d = d + r.J1[k] * dv[6 * r.b1 + k];
        } else if (r.b2 >= 0) {
            for (int k = 0; k < 6; ++k) d = d + r.J2[k] * dv[6 * r.b2 + k];
        }
        return d;
    }
    void axpy(const Row<R>& r, R a) {
        if (r.b1 >= 0)
            for (int k = 0; k < 6; ++k) dv[6 * r.b1 + k] = a * r.WJ1[k] + dv[6 * r.b1 + k];
        if (r.b2 >= 0)
            for (int k = 0; k < 6; ++k) dv[6 * r.b2 + k] = a * r.WJ2[k] + dv[6 * r.b2 + k];
    }
    // SORProx::solve_unilateral[_ground] (sor_prox.rs:181-230).
    void solve_normal(Row<R>& r) {
        R dimpulse = jdot(r) + r.rhs;
        R ni = r.impulse - r.r * dimpulse;
        ni = ni > R(0) ? ni : R(0);
        R dl = ni - r.impulse;
        r.impulse = ni;
        axpy(r, dl);
    }
    // SORProx::solve_bilateral[_ground] with ImpulseLimits::Dependent (sor_prox.rs:232-343).
    void solve_friction(Row<R>& r) {
        R li = rows[r.dep].impulse;
        if (li == R(0)) {
            if (r.impulse != R(0)) {
                axpy(r, -r.impulse);
                r.impulse = R(0);
            }
            return;
        }
        R mx = r.mu * li, mn = -mx;
        R dimpulse = jdot(r) + r.rhs;
        R ni = r.impulse - r.r * dimpulse;
        if (ni < mn) ni = mn;
        else if (ni > mx) ni = mx;
        R dl = ni - r.impulse;
        r.impulse = ni;
        axpy(r, dl);
    }
    // SORProx::solve_bilateral[_ground] with ImpulseLimits::Independent of
    // +-max (a joint row, helper.rs:186-189).
    void solve_bilateral(Row<R>& r) {
        const R mx = std::numeric_limits<R>::max();
        const R lo = r.limit ? R(0) : -mx;
        R dimpulse = jdot(r) + r.rhs;
        R ni = r.impulse - r.r * dimpulse;
        ni = ni < lo ? lo : (ni > mx ? mx : ni);
        R dl = ni - r.impulse;
        r.impulse = ni;
        axpy(r, dl);
    }
    // J dv + rhs of a row, for the residual. f32: the compensated dot product
    // Dot2 of Ogita, Rump and Oishi (SIAM J. Sci. Comput. 26(6), 2005) as the
    // unevaluated float sum s + c (TwoProduct by a fused multiply-add, TwoSum,
    // error terms summed on the side), as accurate as a sum in twice the f32
    // precision; f64: plain sums.
    double residual_dot(const Row<R>& r) const {
        if constexpr (std::is_same<R, float>::value) {
            float s = 0.0f, c = 0.0f;
            auto sum = [&](float h, float e) {
                float t = s + h;
                float z = t - s;
                float q = (s - (t - z)) + (h - z);
                s = t;
                c = c + (q + e);
            };
            auto prod = [&](float x, float y) {
                float h = x * y;
                sum(h, std::fma(x, y, -h));
            };
            if (r.b1 >= 0)
                for (int k = 0; k < 6; ++k) prod(r.J1[k], dv[6 * r.b1 + k]);
            if (r.b2 >= 0)
                for (int k = 0; k < 6; ++k) prod(r.J2[k], dv[6 * r.b2 + k]);
            sum(r.rhs, 0.0f);
            return double(s) + double(c);
        } else {
            double d = 0;
            if (r.b1 >= 0)
                for (int k = 0; k < 6; ++k) d += double(r.J1[k]) * double(dv[6 * r.b1 + k]);
            if (r.b2 >= 0)
                for (int k = 0; k < 6; ++k) d += double(r.J2[k]) * double(dv[6 * r.b2 + k]);
            return d + double(r.rhs);
        }
    }
    // FP64 complementarity residual: ||lambda - proj(lambda - r (J dv + rhs))|| / max(1, ||lambda||).
    double residual() const {
        double s2 = 0, l2 = 0;
        for (const Row<R>& r : rows) {
            const double d = residual_dot(r);
            double lam = double(r.impulse);
            double x = lam - double(r.r) * d;
            double p;
            if (r.bilateral) p = r.limit ? (x > 0 ? x : 0) : x;
            else if (!r.friction) p = x > 0 ? x : 0;
            else {
                double mx = double(r.mu) * double(rows[r.dep].impulse);
                p = std::min(std::max(x, -mx), mx);
            }
            double phi = lam - p;
            s2 += phi * phi;
            l2 += lam * lam;
        }
        return std::sqrt(s2) / std::max(1.0, std::sqrt(l2));
    }
    void sor_prox() {
        // SORProx::solve (sor_prox.rs:48-80).
        std::fill(dv.begin(), dv.end(), R(0));
        for (size_t q = 0; q < seq_warm.size(); ++q) {
            Row<R>& r = rows[seq_warm[q]];
            if (!r.predicted) {
                if (r.impulse != R(0)) axpy(r, r.impulse);
                continue;
            }
            // A learned start (colour order: the contact's three rows follow
            // each other) stays only if its local residual is no larger than
            // that of the start it replaced (the cached impulses, or zero),
            // which is otherwise applied instead.
            Row<R>* r3[3] = {&rows[seq_warm[q]], &rows[seq_warm[q + 1]], &rows[seq_warm[q + 2]]};
            Row<R> c3[3] = {*r3[0], *r3[1], *r3[2]};
            std::vector<R> before = dv;
            R lam[3] = {c3[0].impulse, c3[1].impulse, c3[2].impulse};
            for (int k = 0; k < 3; ++k)
                if (lam[k] != R(0)) axpy(c3[k], lam[k]);
            const R alt[3] = {c3[0].alt[0], c3[0].alt[1], c3[0].alt[2]};
            R with = local_residual(c3, lam);
            std::vector<R> after = dv;
            dv = before;
            for (int k = 0; k < 3; ++k)
                if (alt[k] != R(0)) axpy(c3[k], alt[k]);
            R without = local_residual(c3, alt);
            if (with > without) {
                for (int k = 0; k < 3; ++k) r3[k]->impulse = alt[k];
            } else {
                dv = after;
            }
            q += 2;
        }
        counters.residual_initial = residual();
        uint32_t iters = 0;
        uint32_t maxit = params.solve_to_tolerance ? params.max_iterations_to_tolerance : params.max_velocity_iterations;
        double res = counters.residual_initial;
        for (uint32_t it = 0; it < maxit; ++it) {
            if (params.solve_to_tolerance && res <= double(params.residual_tolerance)) break;
            if (params.sweep_order == NPGPU_SWEEP_MANIFOLD) {
                for (int i : seq_merged) {
                    if (rows[i].bilateral) solve_bilateral(rows[i]);
                    else if (rows[i].friction) solve_friction(rows[i]);
                    else solve_normal(rows[i]);
                }
            } else {
                for (int i : seq_friction) {
                    if (rows[i].bilateral) solve_bilateral(rows[i]);
                    else solve_friction(rows[i]);
                }
                for (int i : seq_normal) solve_normal(rows[i]);
            }
            ++iters;
            if (params.solve_to_tolerance) res = residual();
        }
        if (!params.solve_to_tolerance) res = residual();
        counters.residual = res;
        counters.velocity_iterations = iters;
    }
    // SignoriniCoulombPyramidModel::cache_impulses (signorini_coulomb_pyramid_model.rs:226-261).
    // JointConstraint::cache_impulses (ball_constraint.rs:129-141,
    // fixed_constraint.rs:174-199): the joint keeps its rows' impulses and
    // breaks when |impulse|^2 / dt^2 exceeds the squared break force / torque.
    void cache_impulses() {
        for (const Row<R>& r : rows) {
            if (r.bilateral) joints[r.joint].imp[r.joint_slot] = r.impulse;
            else static_cast<MContact<R>*>(r.cache)->impulse[r.cache_slot] = r.impulse;
        }
        const R inv_dt = (params.dt == 0.0f) ? R(0) : R(1) / R(params.dt);
        for (Joint<R>& j : joints)
            if (j.alive && j.active && joint_breaks(j, inv_dt)) j.broken = true;
    }
    // Each kind's break test in its own arithmetic (ball_constraint.rs:129-141,
    // fixed_constraint.rs:174-199, revolute_constraint.rs:268-292, ...).
    static bool joint_breaks(const Joint<R>& j, R inv_dt) {
        const R* l = j.imp;
        const R* a = j.imp + 3;
        const R l2 = R(0) + l[0] * l[0] + l[1] * l[1] + l[2] * l[2];
        const R a2 = R(0) + a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        const R inv_dt2 = inv_dt * inv_dt;
        switch (j.kind) {
        case NPGPU_JOINT_BALL: return l2 * inv_dt * inv_dt > j.brk_force2;
        case NPGPU_JOINT_CARTESIAN: return a2 * inv_dt * inv_dt > j.brk_torque2;
        case NPGPU_JOINT_PLANAR:
            return l[0] * l[0] * inv_dt2 > j.brk_force2 || a[0] * a[0] * inv_dt2 + a[1] * a[1] * inv_dt2 > j.brk_torque2;
        case NPGPU_JOINT_RECTANGULAR: return l[0] * l[0] * inv_dt2 > j.brk_force2 || a2 * inv_dt2 > j.brk_torque2;
        case NPGPU_JOINT_UNIVERSAL: return l2 * inv_dt2 > j.brk_force2 || a[0] * a[0] * inv_dt2 > j.brk_torque2;
        default: return l2 * inv_dt2 > j.brk_force2 || a2 * inv_dt2 > j.brk_torque2;
        }
    }

    // NonlinearSORProx::solve_generic (nonlinear_sor_prox.rs:78-117) of one
    // position row: clamp_rhs (nonlinear_sor_prox.rs:297-309), then each side
    // with dofs moves by its W times -rhs r.
    void generic_position_row(R depth, bool angular, R inv_r, Body<R>& b1, Body<R>& b2, R* W1, R* W2) {
        R rhs = -depth;
        if (angular) {
            rhs = (rhs + R(params.allowed_angular_error)) * R(params.erp);
            rhs = rhs < -R(params.max_angular_correction) ? -R(params.max_angular_correction) : rhs;
        } else {
            rhs = (rhs + R(params.allowed_linear_error)) * R(params.erp);
            rhs = rhs < -R(params.max_linear_correction) ? -R(params.max_linear_correction) : rhs;
        }
        if (!(rhs < R(0))) return;
        const R r = inv_r != R(0) ? R(1) / inv_r : R(1);
        const R impulse = -rhs * r;
        if (b1.ndofs() != 0) {
            for (int k = 0; k < 6; ++k) W1[k] = W1[k] * impulse;
            apply_displacement(b1, v3<R>(W1[0], W1[1], W1[2]), v3<R>(W1[3], W1[4], W1[5]));
        }
        if (b2.ndofs() != 0) {
            for (int k = 0; k < 6; ++k) W2[k] = W2[k] * impulse;
            apply_displacement(b2, v3<R>(W2[0], W2[1], W2[2]), v3<R>(W2[3], W2[4], W2[5]));
        }
    }

    // UnitQuaternion::rotation_between_axis + scaled_axis (helper.rs:701-769):
    // the unit axis of a x b times acos(a . b); false for opposite axes. The
    // angle is the axis-angle form's directly (acos in double, rounded as the
    // GPU rounds it in f32).
    static bool rotation_between_scaled(V3<R> a, V3<R> b, V3<R>& out) {
        V3<R> ax;
        R n;
        const V3<R> zero = v3<R>(R(0), R(0), R(0));
        if (unit_try(cross(a, b), std::numeric_limits<R>::epsilon(), ax, n)) {
            const R c = dot(a, b);
            if (c <= -R(1)) return false;
            if (c >= R(1)) {
                out = zero;
                return true;
            }
            out = ax * R(std::acos(double(c)));
            return true;
        }
        if (dot(a, b) < R(0)) return false;
        out = zero;
        return true;
    }
    static V3<R> axis_separation(V3<R> a1, V3<R> a2) {
        V3<R> e;
        if (rotation_between_scaled(a1, a2, e)) return e;
        const R c[3] = {std::fabs(a1.x), std::fabs(a1.y), std::fabs(a1.z)};
        int imin = 0;
        if (c[1] < c[imin]) imin = 1;
        if (c[2] < c[imin]) imin = 2;
        const V3<R> o = cross(basis(imin), a1);
        return vdiv(o, norm(o)) * R(3.14159265358979);
    }

    // The position constraints of joint j, in each kind's order
    // (NonlinearSORProx::solve_generator, nonlinear_sor_prox.rs:57-76; each
    // constraint's position_constraint(i) with the poses its predecessors
    // left): the anchors' separation (cancel_relative_translation), the
    // separation along body 1's axis (cancel_relative_translation_wrt_axis),
    // the frames' or bodies' relative rotation (cancel_relative_rotation), the
    // axes' alignment (align_axis) or the angle between them
    // (restore_angle_between_axis), helper.rs:298-418, 553-611, 701-769,
    // 921-998. An error below the allowed one is skipped.
    // PA the anchor's distance from the axis line (project_anchor_to_axis,
    // helper.rs:858-919), AL3 the alignment of axis3 with axis2, LIM the
    // prismatic offset limits (unit_constraint.rs:125-198).
    enum { JP_T = 1, JP_TA = 2, JP_R_FRAMES = 3, JP_R_BODIES = 4, JP_AL = 5, JP_RA = 6, JP_PA = 7, JP_AL3 = 8,
           JP_LIM = 9 };
    void joint_position(uint32_t j) {
        Joint<R>& jt = joints[j];
        Body<R>& b1 = bodies[jt.b1];
        Body<R>& b2 = bodies[jt.b2];
        int ops[3] = {0, 0, 0};
        switch (jt.kind) {
        case NPGPU_JOINT_BALL: ops[0] = JP_T; break;
        case NPGPU_JOINT_FIXED: ops[0] = JP_R_FRAMES; ops[1] = JP_T; break;
        case NPGPU_JOINT_REVOLUTE: ops[0] = JP_T; ops[1] = JP_AL; break;
        case NPGPU_JOINT_CARTESIAN: ops[0] = JP_R_FRAMES; break;
        case NPGPU_JOINT_PLANAR: ops[0] = JP_TA; ops[1] = JP_AL; break;
        case NPGPU_JOINT_RECTANGULAR: ops[0] = JP_TA; ops[1] = JP_R_BODIES; break;
        case NPGPU_JOINT_UNIVERSAL: ops[0] = JP_T; ops[1] = JP_RA; break;
        case NPGPU_JOINT_PRISMATIC:
            ops[0] = JP_PA;
            ops[1] = JP_R_BODIES;
            if (jt.has_min || jt.has_max) ops[2] = JP_LIM;
            break;
        case NPGPU_JOINT_CYLINDRICAL: ops[0] = JP_AL; ops[1] = JP_PA; break;
        default: ops[0] = JP_AL3; ops[1] = JP_PA; break;
        }
        R J1[6], J2[6], W1[6], W2[6];
        for (int o = 0; o < 3 && ops[o] != 0; ++o) {
            const int op = ops[o];
            const V3<R> a1 = iso_pt(b1.pos, jt.anchor1), a2 = iso_pt(b2.pos, jt.anchor2);
            bool angular = false, have = false;
            V3<R> dir;
            R depth = R(0);
            if (op == JP_T) {
                have = unit_try(a2 - a1, R(params.allowed_linear_error), dir, depth);
            } else if (op == JP_TA) {
                const V3<R> ax = qrot(b1.pos.q, jt.axis1);
                depth = dot(ax, a2 - a1);
                dir = ax;
                if (depth < R(0)) {
                    depth = -depth;
                    dir = -ax;
                }
                have = depth > R(params.allowed_linear_error);
            } else if (op == JP_R_FRAMES || op == JP_R_BODIES) {
                Quat<R> r1 = b1.pos.q, r2 = b2.pos.q;
                if (op == JP_R_FRAMES) {
                    r1 = qmul(b1.pos.q, jt.frame1);
                    r2 = qmul(b2.pos.q, jt.frame2);
                }
                angular = true;
                have = unit_try(qscaled_axis(qmul(r2, qconj(r1))), R(params.allowed_angular_error), dir, depth);
            } else if (op == JP_AL || op == JP_AL3) {
                angular = true;
                have = unit_try(axis_separation(qrot(b1.pos.q, op == JP_AL ? jt.axis1 : jt.axis3),
                                                qrot(b2.pos.q, jt.axis2)),
                                R(params.allowed_angular_error), dir, depth);
            } else if (op == JP_PA) {
                const V3<R> ax = qrot(b1.pos.q, jt.axis1);
                const V3<R> proj = a1 + ax * dot(ax, a2 - a1);
                have = unit_try(a2 - proj, R(params.allowed_linear_error), dir, depth);
            } else if (op == JP_LIM) {
                const V3<R> ax = qrot(b1.pos.q, jt.axis1);
                const R offset = dot(ax, a2 - a1);
                depth = R(0);
                dir = ax;
                if (jt.has_min) {
                    depth = jt.min_offset - offset;
                    dir = -ax;
                }
                if (depth < R(0) && jt.has_max) {
                    depth = offset - jt.max_offset;
                    dir = ax;
                }
                have = depth > R(params.allowed_linear_error);
            } else {
                angular = true;
                R cur;
                if (unit_try(axis_separation(qrot(b1.pos.q, jt.axis1), qrot(b2.pos.q, jt.axis2)),
                             std::numeric_limits<R>::epsilon(), dir, cur)) {
                    depth = cur - jt.angle;
                    if (depth < R(0)) {
                        depth = -depth;
                        dir = -dir;
                    }
                    have = !(depth < R(params.allowed_angular_error));
                }
            }
            if (!have) continue;
            R inv_r = R(0), dummy = R(0);
            if (angular) {
                if (b1.ndofs() != 0) fill_torque(b1, dir, J1, W1, inv_r, dummy, false);
                if (b2.ndofs() != 0) fill_torque(b2, -dir, J2, W2, inv_r, dummy, false);
            } else {
                if (b1.ndofs() != 0) fill(b1, a1, dir, J1, W1, inv_r, dummy, false);
                if (b2.ndofs() != 0) fill(b2, a2, -dir, J2, W2, inv_r, dummy, false);
            }
            generic_position_row(depth, angular, inv_r, b1, b2, W1, W2);
        }
    }

    void solve_position(const PosConstraint<R>& pc) {
        if (pc.joint >= 0) {
            joint_position(uint32_t(pc.joint));
            return;
        }
        const Collider<R>& c1 = colliders[pc.c1];
        const Collider<R>& c2 = colliders[pc.c2];
        Body<R>& b1 = bodies[c1.body];
        Body<R>& b2 = bodies[c2.body];
        Iso<R> m1 = iso_mul(b1.pos, c1.pos_wrt_body);
        Iso<R> m2 = iso_mul(b2.pos, c2.pos_wrt_body);
        V3<R> n0 = qrot(m1.q, pc.normal1_local);
        ContactGeom<R> g = kinematic_contact(feature(c1, pc.fid1), m1, c1.dilation() + c1.margin, feature(c2, pc.fid2),
                                             m2, c2.dilation() + c2.margin, n0);
        // clamp_rhs (nonlinear_sor_prox.rs:296-309).
        R rhs = (-g.depth + R(params.allowed_linear_error)) * R(params.erp);
        rhs = std::max(rhs, -R(params.max_linear_correction));
        if (rhs >= R(0)) return;
        R inv_r = R(0), dummy = R(0);
        R J1[6], J2[6], W1[6], W2[6];
        if (b1.ndofs() != 0) fill(b1, g.world1, -g.normal, J1, W1, inv_r, dummy, false);
        if (b2.ndofs() != 0) fill(b2, g.world2, g.normal, J2, W2, inv_r, dummy, false);
        if (inv_r == R(0)) return;
        R r = R(1) / inv_r;
        R impulse = -rhs * r;
        if (b1.ndofs() != 0) {
            for (int k = 0; k < 6; ++k) W1[k] = W1[k] * impulse;
            apply_displacement(b1, v3<R>(W1[0], W1[1], W1[2]), v3<R>(W1[3], W1[4], W1[5]));
        }
        if (b2.ndofs() != 0) {
            for (int k = 0; k < 6; ++k) W2[k] = W2[k] * impulse;
            apply_displacement(b2, v3<R>(W2[0], W2[1], W2[2]), v3<R>(W2[3], W2[4], W2[5]));
        }
    }

    // ------------------------------------------------------- CCD
    // MechanicalWorld::solve_ccd (mechanical_world.rs:561-908) with
    // predict_next_impacts (:400-559) and TOIEntry::try_from_colliders
    // (:942-1031), for one world (every world of a batch is stepped as its
    // own MechanicalWorld). The interactions a collider has during CCD are its
    // broad-phase pairs (fat AABBs overlapping) and, where either collider has
    // CCD enabled, the pairs whose boxes swept from the safe pose to the
    // current one overlap. Pairs are taken in collider-slot order and TOIs of
    // equal time in the order they were found.
    std::vector<R> ccd_time;                       // SubstepState::body_times, per body slot
    std::vector<std::vector<uint32_t>> body_colliders;
    struct TOIEntry {
        R toi;
        uint32_t c1, c2, b1, b2;
        uint32_t ts;
        uint64_t seq;
    };
    enum { PRED_NONE = 0, PRED_IMPACTS = 1, PRED_AFTER = 2 };

    // RigidBody::safe_position (rigid_body.rs:904-910).
    Iso<R> safe_pose(const Body<R>& b) const { return b.linear_interp() ? Iso<R>{b.pos0.t, b.pos.q} : b.pos0; }

    void ccd_sweep_boxes() {
        for (auto& c : colliders) {
            if (!c.alive) continue;
            const Body<R>& b = bodies[c.body];
            R a0[3], b0[3], a1[3], b1[3];
            aabb_at(c, iso_mul(safe_pose(b), c.pos_wrt_body), a0, b0);
            aabb_at(c, iso_mul(b.pos, c.pos_wrt_body), a1, b1);
            for (int k = 0; k < 3; ++k) {
                c.sw_min[k] = std::min(a0[k], a1[k]);
                c.sw_max[k] = std::max(b0[k], b1[k]);
            }
        }
    }
    bool interacts(uint32_t i, uint32_t j) const {
        const Collider<R>& a = colliders[i];
        const Collider<R>& b = colliders[j];
        if (a.sensor || b.sensor) return false;   // proximity pairs take no part in CCD
        if (!pair_allowed(i, j)) return false;
        if (aabb_overlap(a, b)) return true;
        if (!a.ccd && !b.ccd) return false;
        for (int k = 0; k < 3; ++k)
            if (!(a.sw_min[k] <= b.sw_max[k] && b.sw_min[k] <= a.sw_max[k])) return false;
        return true;
    }
    void interactions(uint32_t c, std::vector<uint32_t>& out) const {
        out.clear();
        for (uint32_t d = 0; d < colliders.size(); ++d)
            if (d != c && colliders[d].alive && interacts(c, d)) out.push_back(d);
    }

    CcdShape<R> ccd_shape(const Collider<R>& c) const {
        CcdShape<R> s;
        const V3<R> zero = v3<R>(R(0), R(0), R(0));
        s.local.a = s.local.b = s.local.h = zero;
        s.local.q = Quat<R>{R(0), R(0), R(0), R(1)};
        s.wrt = c.pos_wrt_body;
        R extent;
        if (c.shape == NPGPU_SHAPE_BALL) {
            s.local.kind = CORE_POINT;
            s.local.radius = c.radius;
            extent = c.radius;
        } else if (c.shape == NPGPU_SHAPE_CAPSULE) {
            s.local.kind = CORE_SEGMENT;
            s.local.a = v3<R>(R(0), -c.half.y, R(0));
            s.local.b = v3<R>(R(0), c.half.y, R(0));
            s.local.radius = c.radius;
            extent = c.half.y + c.radius;
        } else {
            s.local.kind = CORE_BOX;
            s.local.h = c.half;
            s.local.radius = R(0);
            extent = norm(c.half);
        }
        s.reach = norm(c.pos_wrt_body.t - bodies[c.body].local_com) + extent;
        return s;
    }
    // BodyPart::part_motion (rigid_body.rs:539-553) shifted by tau, or the
    // still pose a frozen body holds (displaced by `frozen_by` from position0).
    CcdMotion<R> ccd_motion(uint32_t bi, bool frozen, R by) const {
        const Body<R>& b = bodies[bi];
        CcdMotion<R> m;
        m.start = safe_pose(b);
        m.local_com = b.local_com;
        m.lin = b.lin;
        m.ang = b.ang;
        m.linear_only = b.linear_interp();
        const bool still = b.lin.x == R(0) && b.lin.y == R(0) && b.lin.z == R(0) &&
                           (m.linear_only || (b.ang.x == R(0) && b.ang.y == R(0) && b.ang.z == R(0)));
        m.tau = frozen ? R(0) : by;
        m.moving = !still;
        if (frozen) {
            if (m.moving) m.start = ccd_displace(m.start, m.local_com, m.lin * by, m.ang * by, m.linear_only);
            m.moving = false;
        }
        return m;
    }
    // TOIEntry::try_from_colliders: the first time in [start, end_time] the
    // colliders come within allowed_linear_error; f1 / f2 are the frozen times.
    bool try_toi(uint32_t c1, uint32_t c2, const R* f1, const R* f2, R end_time, TOIEntry& e) const {
        const Collider<R>& A = colliders[c1];
        const Collider<R>& B = colliders[c2];
        const uint32_t b1 = A.body, b2 = B.body;
        const R bt1 = ccd_time[b1], bt2 = ccd_time[b2];
        const R t1 = f1 ? *f1 : bt1, t2 = f2 ? *f2 : bt2;
        const R start = std::max(t1, t2);
        const CcdMotion<R> m1 = f1 ? ccd_motion(b1, true, *f1 - bt1) : ccd_motion(b1, false, start - bt1);
        const CcdMotion<R> m2 = f2 ? ccd_motion(b2, true, *f2 - bt2) : ccd_motion(b2, false, start - bt2);
        R t;
        const CaResult r = conservative_advancement(ccd_shape(A), m1, ccd_shape(B), m2, end_time - start,
                                                    R(params.allowed_linear_error), t);
        if (!r.some) return false;
        if (r.penetrating && !params.ccd_on_penetration_enabled) return false;
        e = TOIEntry{start + t, c1, c2, b1, b2, 0u, 0u};
        return true;
    }

    // predict_next_impacts: the impacts up to end_time in time order, the
    // bodies frozen at their first impact, the smallest TOI beyond end_time.
    int predict(uint32_t world, R end_time, std::vector<TOIEntry>& impacts, std::vector<R>& frozen,
                std::vector<char>& is_frozen, R& min_overstep) {
        impacts.clear();
        frozen.assign(bodies.size(), R(0));
        is_frozen.assign(bodies.size(), 0);
        std::map<uint64_t, uint32_t> ts;
        std::vector<TOIEntry> heap;
        uint64_t seq = 0;
        std::map<uint64_t, char> seen;
        const R dt0 = R(params.dt);
        min_overstep = dt0;
        std::vector<uint32_t> nbr;
        for (uint32_t c = 0; c < colliders.size(); ++c) {
            if (!colliders[c].alive || !colliders[c].ccd || bodies[colliders[c].body].world != world) continue;
            interactions(c, nbr);
            for (uint32_t d : nbr) {
                const uint32_t i = std::min(c, d), j = std::max(c, d);
                const uint64_t key = (uint64_t(i) << 32) | j;
                if (!seen.emplace(key, 1).second) continue;
                TOIEntry e;
                if (!try_toi(i, j, nullptr, nullptr, min_overstep, e)) continue;
                if (e.toi > end_time) {
                    min_overstep = std::min(min_overstep, e.toi);
                } else {
                    min_overstep = end_time;
                    e.seq = seq++;
                    heap.push_back(e);
                    ts[key] = 0;
                }
            }
        }
        if (min_overstep == dt0 && heap.empty()) return PRED_NONE;
        if (min_overstep > end_time) return PRED_AFTER;
        while (!heap.empty()) {
            size_t best = 0;
            for (size_t k = 1; k < heap.size(); ++k)
                if (heap[k].toi < heap[best].toi || (heap[k].toi == heap[best].toi && heap[k].seq < heap[best].seq)) best = k;
            const TOIEntry e = heap[best];
            heap.erase(heap.begin() + long(best));
            if (e.ts != ts[(uint64_t(e.c1) << 32) | e.c2]) continue;   // superseded by a resweep
            if (is_frozen[e.b1] && is_frozen[e.b2]) {
                if (e.toi == std::max(frozen[e.b1], frozen[e.b2])) impacts.push_back(e);
                continue;
            }
            if (!is_frozen[e.b1]) {
                is_frozen[e.b1] = 1;
                frozen[e.b1] = e.toi;
            }
            if (!is_frozen[e.b2]) {
                is_frozen[e.b2] = 1;
                frozen[e.b2] = e.toi;
            }
            // Resweep every pair of the frozen bodies' colliders.
            for (uint32_t fb : {e.b1, e.b2}) {
                if (!bodies[fb].dynamic()) continue;
                for (uint32_t cc : body_colliders[fb]) {
                    interactions(cc, nbr);
                    for (uint32_t d : nbr) {
                        const uint32_t ch1 = std::min(cc, d), ch2 = std::max(cc, d);
                        if (!colliders[ch1].ccd && !colliders[ch2].ccd) continue;
                        const uint32_t x1 = colliders[ch1].body, x2 = colliders[ch2].body;
                        const bool s1 = !bodies[x1].dynamic(), s2 = !bodies[x2].dynamic();
                        if ((is_frozen[x1] || s1) && (is_frozen[x2] || s2)) continue;
                        const uint64_t key = (uint64_t(ch1) << 32) | ch2;
                        const uint32_t stamp = ++ts[key];
                        TOIEntry ne;
                        if (try_toi(ch1, ch2, is_frozen[x1] ? &frozen[x1] : nullptr, is_frozen[x2] ? &frozen[x2] : nullptr,
                                    end_time, ne)) {
                            ne.ts = stamp;
                            ne.seq = seq++;
                            heap.push_back(ne);
                        }
                    }
                }
            }
            impacts.push_back(e);
        }
        return PRED_IMPACTS;
    }

    // RigidBody::advance then clamp_advancement (rigid_body.rs:521-537).
    void advance_clamp(Body<R>& b, R by) {
        b.pos0 = ccd_displace(safe_pose(b), b.local_com, b.lin * by, b.ang * by, b.linear_interp());
        clamp_advancement(b);
    }
    void clamp_advancement(Body<R>& b) {
        b.pos = b.linear_interp() ? Iso<R>{b.pos0.t, b.pos.q} : b.pos0;
        b.com = iso_pt(b.pos, b.local_com);
        b.changed = true;
    }

    // One CCD substep (mechanical_world.rs:624-889): the impacting bodies and
    // those in contact with them, moved back to the latest TOI, solved
    // (MoreauJeanSolver::step_ccd, moreau_jean_solver.rs:94-127) and
    // integrated over the rest of the step.
    void ccd_substep(uint32_t world, const std::vector<TOIEntry>& impacts, const std::vector<R>& frozen,
                     const std::vector<char>& is_frozen) {
        const R dt0 = R(params.dt);
        const R last = impacts.back().toi;
        const R dts = dt0 - last;
        cur_dt = dts;
        std::vector<char> prepared(bodies.size(), 0), visited(colliders.size(), 0);
        std::vector<uint32_t> stack, island, ccd_bodies, nbr;
        for (const TOIEntry& e : impacts) {
            stack.insert(stack.end(), body_colliders[e.b1].begin(), body_colliders[e.b1].end());
            stack.insert(stack.end(), body_colliders[e.b2].begin(), body_colliders[e.b2].end());
            ccd_bodies.push_back(e.b1);
            ccd_bodies.push_back(e.b2);
        }
        const V3<R> zero = v3<R>(R(0), R(0), R(0));
        auto prepare = [&](uint32_t h) {
            Body<R>& b = bodies[h];
            b.f_lin = b.f_ang = zero;
            update_dynamics(b, dts);
            update_acceleration(b, zero);
            const R target = is_frozen[h] ? frozen[h] : last;
            advance_clamp(b, target - ccd_time[h]);
            ccd_time[h] = last;
            prepared[h] = 1;
            island.push_back(h);
        };
        std::vector<Manifold<R>> mlist;
        if (order == ORDER_COLOUR) {
            // The GPU's island: the closure through contacts, level by level
            // (a level's pairs: those of its colliders with colliders not
            // explored before it, each once; its bodies prepared first; a
            // pair with contacts explores the colliders of its other body,
            // when dynamic), the manifolds in collider-pair order.
            std::vector<char> explored_body(bodies.size(), 0), explored(colliders.size(), 0), front(colliders.size(), 0);
            std::vector<uint32_t> frontier;
            for (const TOIEntry& e : impacts)
                for (uint32_t b : {e.b1, e.b2})
                    if (!explored_body[b]) {
                        explored_body[b] = 1;
                        for (uint32_t c : body_colliders[b]) frontier.push_back(c);
                    }
            for (uint32_t c : frontier) explored[c] = front[c] = 1;
            std::map<uint64_t, Manifold<R>> found;
            while (!frontier.empty()) {
                std::vector<std::pair<uint32_t, uint32_t>> pairs;
                for (uint32_t c : frontier) {
                    interactions(c, nbr);
                    for (uint32_t d : nbr) {
                        if (explored[d] && !front[d]) continue;   // its pairs were a former level's
                        if (front[d] && d < c) continue;          // taken from d
                        pairs.push_back({std::min(c, d), std::max(c, d)});
                    }
                }
                for (auto& pr : pairs)
                    for (uint32_t x : {colliders[pr.first].body, colliders[pr.second].body})
                        if (!prepared[x] && bodies[x].dynamic()) prepare(x);
                std::vector<uint32_t> next;
                for (auto& pr : pairs) {
                    const uint32_t x1 = colliders[pr.first].body, x2 = colliders[pr.second].body;
                    colliders[pr.first].pose = iso_mul(bodies[x1].pos, colliders[pr.first].pos_wrt_body);
                    colliders[pr.second].pose = iso_mul(bodies[x2].pos, colliders[pr.second].pos_wrt_body);
                    Manifold<R> m;
                    m.c1 = pr.first;
                    m.c2 = pr.second;
                    narrow_pair(m);
                    if (m.contacts.empty()) continue;
                    found[(uint64_t(m.c1) << 32) | m.c2] = m;
                    const uint32_t other = front[pr.first] ? pr.second : pr.first;
                    const uint32_t xo = colliders[other].body;
                    if (!front[other] && bodies[xo].dynamic() && !explored_body[xo]) {
                        explored_body[xo] = 1;
                        next.push_back(xo);
                    }
                }
                for (uint32_t c : frontier) front[c] = 0;
                frontier.clear();
                for (uint32_t b : next)
                    for (uint32_t c : body_colliders[b]) {
                        explored[c] = front[c] = 1;
                        frontier.push_back(c);
                    }
            }
            for (auto& kv : found) mlist.push_back(kv.second);
        }
        while (order != ORDER_COLOUR && !stack.empty()) {
            const uint32_t c = stack.back();
            stack.pop_back();
            if (visited[c]) continue;
            interactions(c, nbr);
            for (uint32_t d : nbr) {
                if (visited[d]) continue;
                const uint32_t ch1 = std::min(c, d), ch2 = std::max(c, d);
                const uint32_t x1 = colliders[ch1].body, x2 = colliders[ch2].body;
                const bool p1 = !prepared[x1] && bodies[x1].dynamic();
                if (p1) prepare(x1);
                const bool p2 = !prepared[x2] && bodies[x2].dynamic();
                if (p2) prepare(x2);
                colliders[ch1].pose = iso_mul(bodies[x1].pos, colliders[ch1].pos_wrt_body);
                colliders[ch2].pose = iso_mul(bodies[x2].pos, colliders[ch2].pos_wrt_body);
                Manifold<R> m;
                m.c1 = ch1;
                m.c2 = ch2;
                narrow_pair(m);
                if (m.contacts.empty()) continue;
                mlist.push_back(m);
                if (ch1 != c && p1) stack.insert(stack.end(), body_colliders[x1].begin(), body_colliders[x1].end());
                if (ch2 != c && p2) stack.insert(stack.end(), body_colliders[x2].begin(), body_colliders[x2].end());
            }
            visited[c] = 1;
        }
        // step_ccd: assembly, position solve, validate_advancement of the
        // impacting bodies, velocity solve, integration of the island.
        if (!assemble_ccd(mlist)) {
            last_error = "a CCD island needs more than 256 colours";
            cur_dt = dt0;
            return;
        }
        for (uint32_t it = 0; it < params.max_ccd_position_iterations; ++it)
            for (int i : seq_pos) solve_position(pos_constraints[i]);
        for (uint32_t h : ccd_bodies) bodies[h].pos0 = bodies[h].pos;
        dv.assign(6 * bodies.size(), R(0));
        for (uint32_t it = 0; it < params.max_velocity_iterations; ++it) {
            for (int i : seq_friction) solve_friction(rows[i]);
            for (int i : seq_normal) solve_normal(rows[i]);
        }
        for (uint32_t h : island) {
            Body<R>& b = bodies[h];
            V3<R> el = b.acc_lin * dts, ea = b.acc_ang * dts;
            b.lin = (b.lin + el) + v3<R>(dv[6 * h + 0], dv[6 * h + 1], dv[6 * h + 2]);
            b.ang = (b.ang + ea) + v3<R>(dv[6 * h + 3], dv[6 * h + 4], dv[6 * h + 5]);
            b.changed = true;
            integrate(b);
        }
        for (auto& b : bodies) {
            if (!b.alive || b.world != world) continue;
            b.f_lin = b.f_ang = zero;
            update_dynamics(b, dts);
        }
        cur_dt = dt0;
        counters.ccd_substeps += 1;
        counters.ccd_impacts += uint32_t(impacts.size());
    }

    // The island's contact rows, all started from zero (warmstart_coeff 0),
    // and their position constraints. ORDER_REFERENCE: the reference's order
    // (SORProx::step, sor_prox.rs:159-179; manifolds in the order the island
    // found them). ORDER_COLOUR: the GPU's order, manifolds by their
    // Jones-Plassmann colour, ties in collider-pair order; each iteration the
    // friction rows, then the normal rows, in that order. Returns false when
    // kCcdColours colours do not suffice.
    static constexpr uint32_t kCcdColours = 256;
    static uint32_t ccd_pair_hash(uint32_t c1, uint32_t c2) {
        uint32_t h = c1 * 0x9E3779B1u ^ (c2 + 0x7F4A7C15u) * 0x85EBCA77u;
        h ^= h >> 15;
        h *= 0x2C1B3C6Du;
        h ^= h >> 12;
        h *= 0x297A2D39u;
        h ^= h >> 15;
        return h >> 10;
    }
    bool assemble_ccd(std::vector<Manifold<R>>& ms) {
        rows.clear();
        pos_constraints.clear();
        seq_warm.clear(); seq_friction.clear(); seq_normal.clear(); seq_pos.clear(); seq_merged.clear();
        const R inv_dt = cur_dt == R(0) ? R(0) : R(1) / cur_dt;
        std::vector<int> ug, un, bg, bn;
        std::vector<size_t> morder(ms.size());
        for (size_t q = 0; q < ms.size(); ++q) morder[q] = q;
        std::vector<uint32_t> mcol(ms.size(), 0u);
        if (order == ORDER_COLOUR) {
            // Jones-Plassmann rounds: a manifold takes the round's colour when
            // its priority (a hash of its colliders' world-local slots, ties
            // by the slots) is above every uncoloured manifold's sharing a
            // dynamic body with it.
            const uint32_t world = bodies[colliders[ms.empty() ? 0 : ms[0].c1].body].world;
            uint32_t base = 0xffffffffu;
            for (uint32_t c = 0; c < colliders.size(); ++c)
                if (colliders[c].alive && bodies[colliders[c].body].world == world) {
                    base = c;
                    break;
                }
            std::vector<uint64_t> prio(ms.size());
            std::map<uint32_t, std::vector<size_t>> on_body;
            for (size_t q = 0; q < ms.size(); ++q) {
                const uint32_t l1 = ms[q].c1 - base, l2 = ms[q].c2 - base;
                prio[q] = (uint64_t(ccd_pair_hash(l1, l2)) << 42) | (uint64_t(l1) << 21) | uint64_t(l2);
                for (uint32_t x : {colliders[ms[q].c1].body, colliders[ms[q].c2].body})
                    if (bodies[x].dynamic()) on_body[x].push_back(q);
            }
            std::vector<int> colour(ms.size(), -1);
            size_t left = ms.size();
            for (int round = 0; left > 0; ++round) {
                if (round >= int(kCcdColours)) return false;
                std::vector<size_t> take;
                for (size_t q = 0; q < ms.size(); ++q) {
                    if (colour[q] >= 0) continue;
                    bool top = true;
                    for (uint32_t x : {colliders[ms[q].c1].body, colliders[ms[q].c2].body}) {
                        if (!bodies[x].dynamic()) continue;
                        for (size_t o : on_body[x])
                            if (o != q && colour[o] < 0 && prio[o] > prio[q]) top = false;
                    }
                    if (top) take.push_back(q);
                }
                for (size_t q : take) colour[q] = round;
                left -= take.size();
            }
            for (size_t q = 0; q < ms.size(); ++q) mcol[q] = uint32_t(colour[q]);
            std::stable_sort(morder.begin(), morder.end(), [&](size_t a, size_t b) { return mcol[a] < mcol[b]; });
        }
        for (size_t qi : morder) {
            Manifold<R>& m = ms[qi];
            const Collider<R>& c1 = colliders[m.c1];
            const Collider<R>& c2 = colliders[m.c2];
            const Body<R>& b1 = bodies[c1.body];
            const Body<R>& b2 = bodies[c2.body];
            const R mu = combine(c1.friction, c1.friction_combine, c2.friction, c2.friction_combine);
            const R e = combine(c1.restitution, c1.restitution_combine, c2.restitution, c2.restitution_combine);
            const bool ground = b1.ndofs() == 0 || b2.ndofs() == 0;
            for (MContact<R>& k : m.contacts) {
                const V3<R> n = k.g.normal;
                const V3<R> center1 = k.g.world1 + n * c1.margin;
                const V3<R> center2 = k.g.world2 - n * c2.margin;
                Row<R> rn = make_row(b1, c1.body, b2, c2.body, center1, center2, -n, R(0));
                if (rn.rhs <= -R(params.restitution_velocity_threshold)) rn.rhs = rn.rhs + e * rn.rhs;
                const R depth = k.g.depth + c1.margin + c2.margin;
                if (depth < R(0)) rn.rhs = rn.rhs + (-depth) * inv_dt;
                rn.impulse = R(0);
                rn.friction = false;
                rn.cache = nullptr;
                const int in = int(rows.size());
                rows.push_back(rn);
                pos_constraints.push_back(PosConstraint<R>{m.c1, m.c2, k.fid1, k.fid2, k.normal1_local});
                seq_pos.push_back(int(pos_constraints.size()) - 1);
                V3<R> t[2];
                tangent_basis(n, t[0], t[1]);
                if (order == ORDER_COLOUR) seq_normal.push_back(in);
                else (ground ? ug : un).push_back(in);
                for (int s = 0; s < 2; ++s) {
                    Row<R> rt = make_row(b1, c1.body, b2, c2.body, center1, center2, t[s], R(0));
                    rt.impulse = R(0);
                    rt.friction = true;
                    rt.dep = in;
                    rt.mu = mu;
                    rt.cache = nullptr;
                    if (order == ORDER_COLOUR) seq_friction.push_back(int(rows.size()));
                    else (ground ? bg : bn).push_back(int(rows.size()));
                    rows.push_back(rt);
                }
            }
        }
        for (int i : bn) seq_friction.push_back(i);
        for (int i : bg) seq_friction.push_back(i);
        for (int i : un) seq_normal.push_back(i);
        for (int i : ug) seq_normal.push_back(i);
        return true;
    }

    // Test hooks: the distance of two colliders' shapes at the current poses
    // (direction from c1 toward c2), and the TOI of the pair over [0, horizon]
    // from the current poses (returns -1: none, 0: an impact, 1: penetrating).
    R collider_distance(uint32_t c1, uint32_t c2, V3<R>& dir) const {
        const Collider<R>& A = colliders[c1];
        const Collider<R>& B = colliders[c2];
        const CcdShape<R> s1 = ccd_shape(A), s2 = ccd_shape(B);
        const Iso<R> p1 = bodies[A.body].pos, p2 = bodies[B.body].pos;
        const V3<R> origin = iso_pt(p1, s1.wrt.t);
        const Core<R> k1 = place_core(s1, p1, origin), k2 = place_core(s2, p2, origin);
        return (core_distance(k1, k2, dir) - k1.radius) - k2.radius;
    }
    int pair_toi(uint32_t c1, uint32_t c2, R horizon, R& toi) const {
        const Collider<R>& A = colliders[c1];
        const Collider<R>& B = colliders[c2];
        auto motion = [&](const Body<R>& b) {
            CcdMotion<R> m;
            m.start = b.pos;
            m.local_com = b.local_com;
            m.lin = b.lin;
            m.ang = b.ang;
            m.tau = R(0);
            m.linear_only = b.linear_interp();
            m.moving = true;
            return m;
        };
        const CaResult r = conservative_advancement(ccd_shape(A), motion(bodies[A.body]), ccd_shape(B),
                                                    motion(bodies[B.body]), horizon, R(params.allowed_linear_error), toi);
        return !r.some ? -1 : (r.penetrating ? 1 : 0);
    }

    // Every world of a batch runs its own CCD loop (its own impacts, latest
    // TOI and substep length), in world order.
    void solve_ccd() {
        const R dt0 = R(params.dt);
        if (dt0 == R(0) || params.max_ccd_substeps == 0) return;
        std::vector<uint32_t> worlds;
        for (const auto& c : colliders)
            if (c.alive && c.ccd) worlds.push_back(bodies[c.body].world);
        if (worlds.empty()) return;
        std::sort(worlds.begin(), worlds.end());
        worlds.erase(std::unique(worlds.begin(), worlds.end()), worlds.end());
        body_colliders.assign(bodies.size(), {});
        for (uint32_t c = 0; c < colliders.size(); ++c)
            if (colliders[c].alive) body_colliders[colliders[c].body].push_back(c);
        for (uint32_t wd : worlds) solve_ccd_world(wd);
    }
    void solve_ccd_world(uint32_t world) {
        const R dt0 = R(params.dt);
        const R sub = dt0 / R(params.max_ccd_substeps);
        ccd_time.assign(bodies.size(), R(0));
        R end_time = R(0);
        bool last_iter = false;
        std::vector<TOIEntry> impacts;
        std::vector<R> frozen;
        std::vector<char> is_frozen;
        for (;;) {
            if (end_time < dt0) end_time = std::min(end_time + sub, dt0);
            else last_iter = true;
            ccd_sweep_boxes();
            R mo;
            int pr = predict(world, end_time, impacts, frozen, is_frozen, mo);
            if (pr == PRED_AFTER) {
                end_time = std::floor(mo / sub) * sub;
                end_time = std::min(end_time + sub, dt0);
                pr = predict(world, end_time, impacts, frozen, is_frozen, mo);
                if (pr != PRED_IMPACTS) impacts.clear();
            }
            if (!last_iter && !impacts.empty()) {
                ccd_substep(world, impacts, frozen, is_frozen);
                continue;
            }
            for (uint32_t h = 0; h < bodies.size(); ++h)
                if (is_frozen.size() > h && is_frozen[h] && bodies[h].alive && bodies[h].status != NPGPU_BODY_STATIC)
                    clamp_advancement(bodies[h]);
            break;
        }
        ccd_time.assign(bodies.size(), R(0));
    }

    // ------------------------------------------------------- the step
    // MechanicalWorld::step_with_filter (mechanical_world.rs:199-396).
    npgpu_status step() {
        cur_dt = R(params.dt);
        R dt = cur_dt;
        events.clear();
        prox_events.clear();
        // maintain: register new colliders (geometrical_world.rs:102-143).
        for (auto& c : colliders) {
            if (!c.alive || c.registered) continue;
            c.registered = true;
            Body<R>& b = bodies[c.body];
            if (c.density != R(0) && b.kind == NPGPU_KIND_RIGID_BODY) {
                V3<R> com;
                Inertia<R> in;
                mass_properties(c, com, in);
                add_local_inertia_and_com(b, com, in);
            }
            cd_dirty = true;
        }
        for (auto& b : bodies) {
            if (!b.alive) continue;
            b.pos0 = b.pos;   // RigidBody::step_started (rigid_body.rs:517-519)
            update_dynamics(b, dt);
        }
        for (auto& b : bodies)
            if (b.alive) update_acceleration(b);
        if (cd_dirty) collision_detection();
        activation_update();
        if (!assemble()) return NPGPU_ERR_CAPACITY;
        dv.assign(6 * bodies.size(), R(0));
        sor_prox();
        cache_impulses();
        // update_velocities_and_integrate (moreau_jean_solver.rs:328-347).
        for (uint32_t i = 0; i < bodies.size(); ++i) {
            Body<R>& b = bodies[i];
            if (!b.alive || !b.in_island) continue;
            V3<R> el = b.acc_lin * dt, ea = b.acc_ang * dt;
            b.lin = (b.lin + el) + v3<R>(dv[6 * i + 0], dv[6 * i + 1], dv[6 * i + 2]);
            b.ang = (b.ang + ea) + v3<R>(dv[6 * i + 3], dv[6 * i + 4], dv[6 * i + 5]);
            b.changed = true;
            integrate(b);
        }
        // NonlinearSORProx::solve (nonlinear_sor_prox.rs:17-55).
        for (uint32_t it = 0; it < params.max_position_iterations; ++it)
            for (int i : seq_pos) solve_position(pos_constraints[i]);
        for (auto& b : bodies)
            if (b.alive && b.kinematic()) integrate(b);
        for (auto& b : bodies)
            if (b.alive) update_dynamics(b, dt);
        counters.ccd_substeps = counters.ccd_impacts = 0;
        solve_ccd();
        for (auto& b : bodies)
            if (b.alive) b.f_lin = b.f_ang = v3<R>(R(0), R(0), R(0));
        collision_detection();
        for (auto& b : bodies) b.changed = false;
        counters.steps += 1;
        fill_counters();
        return NPGPU_OK;
    }

    void fill_counters() {
        uint32_t nm = 0, nc = 0, na = 0;
        double maxpen = -1e30, ke = 0;
        for (auto& kv : manifolds) {
            const Manifold<R>& m = kv.second;
            if (!m.contacts.empty()) ++nm;
            nc += uint32_t(m.contacts.size());
            for (auto& k : m.contacts)
                maxpen = std::max(maxpen, double(k.g.depth) + double(colliders[m.c1].margin) + double(colliders[m.c2].margin));
        }
        for (auto& b : bodies) {
            if (!b.alive || !b.dynamic()) continue;
            if (b.in_island) ++na;
            double m = double(b.inertia.linear);
            double v2 = double(b.lin.x) * b.lin.x + double(b.lin.y) * b.lin.y + double(b.lin.z) * b.lin.z;
            V3<R> iw = mv(b.inertia.angular, b.ang);
            double wiw = double(b.ang.x) * iw.x + double(b.ang.y) * iw.y + double(b.ang.z) * iw.z;
            ke += 0.5 * (m * v2 + wiw);
        }
        counters.num_pairs = uint32_t(pairs.size());
        counters.num_manifolds = nm;
        counters.num_contacts = nc;
        counters.num_solver_contacts = num_solver_contacts;
        counters.num_constraints = 3 * num_solver_contacts;
        counters.num_colours = num_colours;
        counters.num_active_bodies = na;
        counters.max_penetration = nc ? maxpen : 0.0;
        counters.kinetic_energy = ke;
    }
};

}  // namespace oracle
