// ccd.cuh -- time of impact for continuous collision detection.
//
// MechanicalWorld::predict_next_impacts and TOIEntry::try_from_colliders
// (src/world/mechanical_world.rs:400-559, 942-1031) take the time of impact
// from ncollide3d's query::time_of_impact / nonlinear_time_of_impact, which
// is not part of the reference sources. This file restates the published
// methods, operation for operation with the CPU oracle (bit-identical in
// f32 under --fmad=false):
//  - the body motion is ConstantVelocityRigidMotion: the pose a time s after
//    position0 is position0 displaced by (v s, w s) about the centre of mass,
//    as RigidBody::apply_displacement displaces it (rigid_body.rs:371-381); a
//    body with linear motion interpolation keeps its current rotation and only
//    translates (rigid_body.rs:539-553);
//  - the distance of two shapes is that of their cores (a ball's centre, a
//    capsule's axis segment, a cuboid) less the radii, by the
//    Gilbert-Johnson-Keerthi algorithm with the closest-point-on-simplex
//    regions of Ericson, Real-Time Collision Detection (2005) 5.1.2-5.1.6;
//  - the time of impact is found by conservative advancement (Mirtich, 1996):
//    each step advances by the distance left over the largest closing speed
//    along the current normal (relative velocity plus |w| times the shape's
//    reach from its centre of mass) aiming at half the target distance
//    (allowed_linear_error), until the distance is at most the target. A pair
//    already overlapping at the start is Penetrating.
#pragma once
#include "np_math.cuh"

namespace npgpu_dev {
namespace ccd {

enum { CORE_POINT = 0, CORE_SEGMENT = 1, CORE_BOX = 2 };

struct Core {
    int kind;
    np::V a, b;      // point: a; segment: a, b; box: centre a
    np::Q q;         // box rotation
    np::V h;         // box half extents
    float radius;
};

NP_HD np::V core_support(const Core& c, np::V d) {
    if (c.kind == CORE_POINT) return c.a;
    if (c.kind == CORE_SEGMENT) return np::dot(np::sub(c.b, c.a), d) > 0.0f ? c.b : c.a;
    const np::V l = np::qrot_inv(c.q, d);
    const np::V p = np::mk(l.x > 0.0f ? c.h.x : -c.h.x, l.y > 0.0f ? c.h.y : -c.h.y, l.z > 0.0f ? c.h.z : -c.h.z);
    return np::add(np::qrot(c.q, p), c.a);
}

struct Simplex {
    np::V p[4];
    int n;
};

NP_HD np::V closest_segment(Simplex& s) {
    const np::V a = s.p[0], b = s.p[1];
    const np::V ab = np::sub(b, a);
    const float t = -np::dot(a, ab);
    if (t <= 0.0f) {
        s.n = 1;
        return a;
    }
    const float den = np::dot(ab, ab);
    if (t >= den) {
        s.p[0] = b;
        s.n = 1;
        return b;
    }
    return np::add(a, np::mul(ab, t / den));
}

NP_HD np::V closest_triangle(Simplex& s) {
    const np::V a = s.p[0], b = s.p[1], c = s.p[2];
    const np::V ab = np::sub(b, a), ac = np::sub(c, a);
    const np::V ap = np::neg(a);
    const float d1 = np::dot(ab, ap), d2 = np::dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) {
        s.n = 1;
        return a;
    }
    const np::V bp = np::neg(b);
    const float d3 = np::dot(ab, bp), d4 = np::dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) {
        s.p[0] = b;
        s.n = 1;
        return b;
    }
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        const float v = d1 / (d1 - d3);
        s.n = 2;
        return np::add(a, np::mul(ab, v));
    }
    const np::V cp = np::neg(c);
    const float d5 = np::dot(ab, cp), d6 = np::dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) {
        s.p[0] = c;
        s.n = 1;
        return c;
    }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        const float w = d2 / (d2 - d6);
        s.p[1] = c;
        s.n = 2;
        return np::add(a, np::mul(ac, w));
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        s.p[0] = b;
        s.p[1] = c;
        s.n = 2;
        return np::add(b, np::mul(np::sub(c, b), w));
    }
    const float sum = (va + vb) + vc;
    if (!(sum > 0.0f)) {
        // A degenerate (flat) triangle: its longest edge holds the closest point.
        const np::V bc = np::sub(c, b);
        const float lab = np::dot(ab, ab), lac = np::dot(ac, ac), lbc = np::dot(bc, bc);
        if (lbc > lab && lbc > lac) {
            s.p[0] = b;
            s.p[1] = c;
        } else if (lac > lab) {
            s.p[1] = c;
        }
        s.n = 2;
        return closest_segment(s);
    }
    const float den = 1.0f / sum;
    const float v = vb * den, w = vc * den;
    return np::add(np::add(a, np::mul(ab, v)), np::mul(ac, w));
}

NP_HD bool outside_face(np::V a, np::V b, np::V c, np::V d) {
    const np::V n = np::cross(np::sub(b, a), np::sub(c, a));
    const float sp = -np::dot(a, n), sd = np::dot(np::sub(d, a), n);
    return sp * sd < 0.0f;
}

// A flat tetrahedron (volume below 1e-4 times the product of its edge
// lengths from a) holds no interior: its faces are all candidates.
NP_HD np::V closest_tetrahedron(Simplex& s, bool& inside) {
    const np::V a = s.p[0], b = s.p[1], c = s.p[2], d = s.p[3];
    const np::V ab = np::sub(b, a), ac = np::sub(c, a), ad = np::sub(d, a);
    const float vol = np::dot(ad, np::cross(ab, ac));
    const float scale = (np::norm(ab) * np::norm(ac)) * np::norm(ad);
    const bool flat = !(fabsf(vol) > 1e-4f * scale);
    inside = true;
    float best = 0.0f;
    np::V out = np::mk(0.0f, 0.0f, 0.0f);
    Simplex keep = s;
    const np::V f[4][4] = {{a, b, c, d}, {a, c, d, b}, {a, d, b, c}, {b, d, c, a}};
    for (int k = 0; k < 4; ++k) {
        if (!flat && !outside_face(f[k][0], f[k][1], f[k][2], f[k][3])) continue;
        Simplex t;
        t.p[0] = f[k][0];
        t.p[1] = f[k][1];
        t.p[2] = f[k][2];
        t.p[3] = np::mk(0.0f, 0.0f, 0.0f);
        t.n = 3;
        const np::V q = closest_triangle(t);
        const float dd = np::dot(q, q);
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

// Distance between the cores A and B (relative to a common origin) and the
// unit direction from A toward B; 0 and (1, 0, 0) when they overlap.
NP_HD float core_distance(const Core& A, const Core& B, np::V& dir) {
    dir = np::mk(1.0f, 0.0f, 0.0f);
    if (A.kind == CORE_POINT && B.kind == CORE_POINT) {
        const np::V d = np::sub(B.a, A.a);
        const float l2 = np::dot(d, d);
        if (!(l2 > 0.0f)) return 0.0f;
        const float l = sqrtf(l2);
        dir = np::divs(d, l);
        return l;
    }
    Simplex s;
    s.n = 0;
    for (int k = 0; k < 4; ++k) s.p[k] = np::mk(0.0f, 0.0f, 0.0f);
    np::V v = np::sub(A.a, B.a);
    const float kRel = 1e-6f, kAbs = 1e-14f;
    for (int it = 0; it < 32; ++it) {
        const float vv = np::dot(v, v);
        if (vv <= kAbs) return 0.0f;
        const np::V w = np::sub(core_support(A, np::neg(v)), core_support(B, v));
        if (vv - np::dot(v, w) <= kRel * vv) break;
        bool dup = false;
        for (int k = 0; k < s.n; ++k) dup = dup || (s.p[k].x == w.x && s.p[k].y == w.y && s.p[k].z == w.z);
        if (dup) break;
        s.p[s.n++] = w;
        if (s.n == 1) {
            v = w;
        } else if (s.n == 2) {
            v = closest_segment(s);
        } else if (s.n == 3) {
            v = closest_triangle(s);
        } else {
            bool inside;
            v = closest_tetrahedron(s, inside);
            if (inside) return 0.0f;
        }
    }
    const float vv = np::dot(v, v);
    if (!(vv > kAbs)) return 0.0f;
    const float l = sqrtf(vv);
    dir = np::divs(np::neg(v), l);
    return l;
}

// A body's motion over one search: pose(s) = start displaced by (s + tau)
// times the velocities; frozen or still bodies stay at `start`.
struct Motion {
    np::Iso start;
    np::V local_com, lin, ang;
    float tau;
    bool moving, linear_only;
};

NP_HD np::Iso displace(const np::Iso& p, np::V local_com, np::V dl, np::V da, bool linear_only) {
    if (linear_only) return np::Iso{np::add(p.t, dl), p.q};
    const np::Q qd = np::qexp(da);
    const np::V com = np::iso_pt(p, local_com);
    const np::V t = np::add(np::add(com, dl), np::qrot(qd, np::neg(com)));
    return np::Iso{np::add(t, np::qrot(qd, p.t)), np::qmul(qd, p.q)};
}

NP_HD np::Iso motion_pose(const Motion& m, float s) {
    if (!m.moving) return m.start;
    const float u = s + m.tau;
    return displace(m.start, m.local_com, np::mul(m.lin, u), np::mul(m.ang, u), m.linear_only);
}

// One collider of a query: its core in the collider frame, its pose on the
// body, and its reach from the body's centre of mass.
struct Shape {
    Core local;
    np::Iso wrt;
    float reach;
};

NP_HD Core place_core(const Shape& s, const np::Iso& body, np::V origin) {
    const np::Iso m = np::iso_mul(body, s.wrt);
    Core c = s.local;
    if (c.kind == CORE_BOX) {
        c.q = m.q;
        c.a = np::sub(m.t, origin);
    } else {
        c.a = np::sub(np::iso_pt(m, s.local.a), origin);
        c.b = np::sub(np::iso_pt(m, s.local.b), origin);
    }
    return c;
}

struct CaResult {
    bool some, penetrating;
};

// Conservative advancement over [0, horizon]; t is the time of impact.
NP_HD CaResult conservative_advancement(const Shape& s1, const Motion& m1, const Shape& s2, const Motion& m2,
                                        float horizon, float target, float& t) {
    t = 0.0f;
    const float w1 = m1.moving && !m1.linear_only ? np::norm(m1.ang) : 0.0f;
    const float w2 = m2.moving && !m2.linear_only ? np::norm(m2.ang) : 0.0f;
    const np::V zero = np::mk(0.0f, 0.0f, 0.0f);
    const np::V v1 = m1.moving ? m1.lin : zero, v2 = m2.moving ? m2.lin : zero;
    const np::V dv = np::sub(v1, v2);
    const float spin = w1 * s1.reach + w2 * s2.reach;
    for (int it = 0; it < 64; ++it) {
        if (t > horizon) return CaResult{false, false};
        const np::Iso p1 = motion_pose(m1, t), p2 = motion_pose(m2, t);
        const np::V origin = np::iso_pt(p1, s1.wrt.t);
        const Core c1 = place_core(s1, p1, origin), c2 = place_core(s2, p2, origin);
        np::V n;
        const float dist = (core_distance(c1, c2, n) - c1.radius) - c2.radius;
        if (dist <= target) return CaResult{true, it == 0 && dist < 0.0f};
        const float bound = np::dot(dv, n) + spin;
        if (!(bound > 0.0f)) return CaResult{false, false};
        t = t + (dist - target * 0.5f) / bound;
    }
    return CaResult{!(t > horizon), false};
}

}  // namespace ccd
}  // namespace npgpu_dev
