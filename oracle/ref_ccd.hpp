// ref_ccd.hpp -- time of impact for the oracle's CCD (test infrastructure only).
//
// The oracle is the checker for the GPU step: only tests, the smoke check and
// the CPU-baseline leg of the benchmark load it. Nothing in the product links it.
//
// MechanicalWorld::predict_next_impacts and TOIEntry::try_from_colliders
// (src/world/mechanical_world.rs:400-559, 942-1031) take the time of impact
// from ncollide3d 0.31's query::time_of_impact / nonlinear_time_of_impact,
// which is not vendored here. This file restates the published methods
// instead, and the GPU (csrc/ccd.cuh) performs the same operations in the same
// order:
//  - the body motion is ConstantVelocityRigidMotion: the pose a time s after
//    position0 is position0 displaced by (v s, w s) about the centre of mass
//    (the displacement of RigidBody::apply_displacement, rigid_body.rs:371-381);
//    a body with linear motion interpolation keeps its current rotation and
//    only translates (ConstantLinearVelocityRigidMotion, rigid_body.rs:539-553);
//  - the distance of two shapes is that of their cores (a ball's centre, a
//    capsule's axis segment, a cuboid) less the radii, by the
//    Gilbert-Johnson-Keerthi algorithm with the closest-point-on-simplex
//    regions of Ericson, Real-Time Collision Detection (2005) 5.1.2-5.1.6;
//  - the time of impact is found by conservative advancement (Mirtich, 1996):
//    each step advances by the distance left over the largest closing speed
//    along the current normal (the relative velocity plus |w| times the
//    shape's reach from its centre of mass), until the distance is at most the
//    target (allowed_linear_error), aiming at half the target. A pair already
//    overlapping at the start is Penetrating.
#pragma once
#include <cmath>
#include "ref_math.hpp"

namespace oracle {

enum { CORE_POINT = 0, CORE_SEGMENT = 1, CORE_BOX = 2 };

// A shape's core in a local frame: a point, a segment or a box (with its
// rotation and half extents), and the radius added around it.
template <class R> struct Core {
    int kind;
    V3<R> a, b;      // point: a; segment: a, b
    Quat<R> q;       // box: rotation, centre a, half extents h
    V3<R> h;
    R radius;
};

template <class R> inline V3<R> core_support(const Core<R>& c, V3<R> d) {
    if (c.kind == CORE_POINT) return c.a;
    if (c.kind == CORE_SEGMENT) return dot(c.b - c.a, d) > R(0) ? c.b : c.a;
    const V3<R> l = qrot_inv(c.q, d);
    const V3<R> p = v3<R>(l.x > R(0) ? c.h.x : -c.h.x, l.y > R(0) ? c.h.y : -c.h.y, l.z > R(0) ? c.h.z : -c.h.z);
    return qrot(c.q, p) + c.a;
}

// The simplex of GJK and its reduction to the feature closest to the origin.
template <class R> struct Simplex {
    V3<R> p[4] = {};
    int n = 0;
};

// Ericson 5.1.2 (segment), 5.1.5 (triangle): the closest point to the origin
// of the simplex, which keeps only the vertices of the closest feature.
template <class R> inline V3<R> closest_segment(Simplex<R>& s) {
    const V3<R> a = s.p[0], b = s.p[1];
    const V3<R> ab = b - a;
    const R t = -dot(a, ab);
    if (t <= R(0)) {
        s.n = 1;
        return a;
    }
    const R den = dot(ab, ab);
    if (t >= den) {
        s.p[0] = b;
        s.n = 1;
        return b;
    }
    return a + ab * (t / den);
}

template <class R> inline V3<R> closest_triangle(Simplex<R>& s) {
    const V3<R> a = s.p[0], b = s.p[1], c = s.p[2];
    const V3<R> ab = b - a, ac = c - a;
    const V3<R> ap = -a;
    const R d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= R(0) && d2 <= R(0)) {
        s.n = 1;
        return a;
    }
    const V3<R> bp = -b;
    const R d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= R(0) && d4 <= d3) {
        s.p[0] = b;
        s.n = 1;
        return b;
    }
    const R vc = d1 * d4 - d3 * d2;
    if (vc <= R(0) && d1 >= R(0) && d3 <= R(0)) {
        const R v = d1 / (d1 - d3);
        s.n = 2;
        return a + ab * v;
    }
    const V3<R> cp = -c;
    const R d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= R(0) && d5 <= d6) {
        s.p[0] = c;
        s.n = 1;
        return c;
    }
    const R vb = d5 * d2 - d1 * d6;
    if (vb <= R(0) && d2 >= R(0) && d6 <= R(0)) {
        const R w = d2 / (d2 - d6);
        s.p[1] = c;
        s.n = 2;
        return a + ac * w;
    }
    const R va = d3 * d6 - d5 * d4;
    if (va <= R(0) && (d4 - d3) >= R(0) && (d5 - d6) >= R(0)) {
        const R w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        s.p[0] = b;
        s.p[1] = c;
        s.n = 2;
        return b + (c - b) * w;
    }
    const R sum = (va + vb) + vc;
    if (!(sum > R(0))) {
        // A degenerate (flat) triangle: its longest edge holds the closest point.
        const V3<R> bc = c - b;
        const R lab = dot(ab, ab), lac = dot(ac, ac), lbc = dot(bc, bc);
        if (lbc > lab && lbc > lac) {
            s.p[0] = b;
            s.p[1] = c;
        } else if (lac > lab) {
            s.p[1] = c;
        }
        s.n = 2;
        return closest_segment(s);
    }
    const R den = R(1) / sum;
    const R v = vb * den, w = vc * den;
    return (a + ab * v) + ac * w;
}

// Ericson 5.1.6: the origin outside the face (a, b, c) on the side away from d.
template <class R> inline bool outside_face(V3<R> a, V3<R> b, V3<R> c, V3<R> d) {
    const V3<R> n = cross(b - a, c - a);
    const R sp = -dot(a, n), sd = dot(d - a, n);
    return sp * sd < R(0);
}

// A flat tetrahedron (volume below 1e-4 times the product of its edge
// lengths from a) holds no interior: its faces are all candidates.
template <class R> inline V3<R> closest_tetrahedron(Simplex<R>& s, bool& inside) {
    const V3<R> a = s.p[0], b = s.p[1], c = s.p[2], d = s.p[3];
    const V3<R> ab = b - a, ac = c - a, ad = d - a;
    const R vol = dot(ad, cross(ab, ac));
    const R scale = (norm(ab) * norm(ac)) * norm(ad);
    const bool flat = !(std::fabs(vol) > R(1e-4) * scale);
    inside = true;
    R best = R(0);
    V3<R> out = v3<R>(R(0), R(0), R(0));
    Simplex<R> keep;
    const V3<R> f[4][4] = {{a, b, c, d}, {a, c, d, b}, {a, d, b, c}, {b, d, c, a}};
    for (int k = 0; k < 4; ++k) {
        if (!flat && !outside_face(f[k][0], f[k][1], f[k][2], f[k][3])) continue;
        Simplex<R> t;
        t.p[0] = f[k][0];
        t.p[1] = f[k][1];
        t.p[2] = f[k][2];
        t.n = 3;
        const V3<R> q = closest_triangle(t);
        const R dd = dot(q, q);
        if (inside || dd < best) {
            inside = false;
            best = dd;
            out = q;
            keep = t;
        }
    }
    if (!inside) s = keep;
    return out;
}

// Distance between the cores A and B (both given relative to a common origin)
// and the unit direction from A toward B; 0 and (1, 0, 0) when they overlap.
template <class R> inline R core_distance(const Core<R>& A, const Core<R>& B, V3<R>& dir) {
    dir = v3<R>(R(1), R(0), R(0));
    if (A.kind == CORE_POINT && B.kind == CORE_POINT) {
        const V3<R> d = B.a - A.a;
        const R l2 = dot(d, d);
        if (!(l2 > R(0))) return R(0);
        const R l = std::sqrt(l2);
        dir = vdiv(d, l);
        return l;
    }
    Simplex<R> s;
    // A point of the Minkowski difference A - B: the difference of the cores' first points.
    V3<R> v = A.a - B.a;
    const R kRel = R(1e-6), kAbs = R(1e-14);
    for (int it = 0; it < 32; ++it) {
        const R vv = dot(v, v);
        if (vv <= kAbs) return R(0);
        const V3<R> w = core_support(A, -v) - core_support(B, v);
        if (vv - dot(v, w) <= kRel * vv) break;   // no progress along -v: v is the closest point
        bool dup = false;
        for (int k = 0; k < s.n; ++k) dup = dup || (s.p[k].x == w.x && s.p[k].y == w.y && s.p[k].z == w.z);
        if (dup) break;
        s.p[s.n++] = w;
        if (s.n == 1) v = w;
        else if (s.n == 2) v = closest_segment(s);
        else if (s.n == 3) v = closest_triangle(s);
        else {
            bool inside;
            v = closest_tetrahedron(s, inside);
            if (inside) return R(0);
        }
    }
    const R vv = dot(v, v);
    if (!(vv > kAbs)) return R(0);
    const R l = std::sqrt(vv);
    dir = vdiv(-v, l);
    return l;
}

// A body's motion over one search: pose(s) = start displaced by (s + tau)
// times the velocities; frozen or still bodies stay at `start`.
template <class R> struct CcdMotion {
    Iso<R> start;
    V3<R> local_com, lin, ang;
    R tau;
    bool moving, linear_only;
};

// The pose `p` displaced by (dl, da) about its centre of mass
// (apply_displacement, rigid_body.rs:371-381), or only translated.
template <class R> inline Iso<R> ccd_displace(const Iso<R>& p, V3<R> local_com, V3<R> dl, V3<R> da, bool linear_only) {
    if (linear_only) return Iso<R>{p.t + dl, p.q};
    const Quat<R> qd = qexp_scaled_axis(da);
    const V3<R> com = iso_pt(p, local_com);
    const V3<R> t = (com + dl) + qrot(qd, -com);
    return Iso<R>{t + qrot(qd, p.t), qmul(qd, p.q)};
}

template <class R> inline Iso<R> motion_pose(const CcdMotion<R>& m, R s) {
    if (!m.moving) return m.start;
    const R u = s + m.tau;
    return ccd_displace(m.start, m.local_com, m.lin * u, m.ang * u, m.linear_only);
}

// One collider of a TOI query: the core in the collider's frame, its pose on
// the body, and its reach from the body's centre of mass.
template <class R> struct CcdShape {
    Core<R> local;       // core in the collider frame (box centre at 0, identity rotation)
    Iso<R> wrt;          // collider pose on its body
    R reach;
};

template <class R> inline Core<R> place_core(const CcdShape<R>& s, const Iso<R>& body, V3<R> origin) {
    const Iso<R> m = iso_mul(body, s.wrt);
    Core<R> c = s.local;
    if (c.kind == CORE_BOX) {
        c.q = m.q;
        c.a = m.t - origin;
    } else {
        c.a = iso_pt(m, s.local.a) - origin;
        c.b = iso_pt(m, s.local.b) - origin;
    }
    return c;
}

struct CaResult {
    bool some;          // an impact within the horizon
    bool penetrating;   // the shapes overlap at the start
};

// Conservative advancement over [0, horizon]; t is the time of impact.
template <class R> inline CaResult conservative_advancement(const CcdShape<R>& s1, const CcdMotion<R>& m1,
                                                             const CcdShape<R>& s2, const CcdMotion<R>& m2,
                                                             R horizon, R target, R& t) {
    t = R(0);
    const R w1 = m1.moving && !m1.linear_only ? norm(m1.ang) : R(0);
    const R w2 = m2.moving && !m2.linear_only ? norm(m2.ang) : R(0);
    const V3<R> zero = v3<R>(R(0), R(0), R(0));
    const V3<R> v1 = m1.moving ? m1.lin : zero, v2 = m2.moving ? m2.lin : zero;
    const V3<R> dv = v1 - v2;
    const R spin = w1 * s1.reach + w2 * s2.reach;
    for (int it = 0; it < 64; ++it) {
        if (t > horizon) return CaResult{false, false};
        const Iso<R> p1 = motion_pose(m1, t), p2 = motion_pose(m2, t);
        const V3<R> origin = iso_pt(p1, s1.wrt.t);
        const Core<R> c1 = place_core(s1, p1, origin), c2 = place_core(s2, p2, origin);
        V3<R> n;
        const R dist = (core_distance(c1, c2, n) - c1.radius) - c2.radius;
        if (dist <= target) return CaResult{true, it == 0 && dist < R(0)};
        const R bound = dot(dv, n) + spin;
        if (!(bound > R(0))) return CaResult{false, false};
        t = t + (dist - target * R(0.5)) / bound;
    }
    return CaResult{!(t > horizon), false};
}

}  // namespace oracle
