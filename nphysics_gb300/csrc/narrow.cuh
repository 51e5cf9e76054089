// narrow.cuh -- contact geometry on the device: cuboid features, the contact
// kinematic re-evaluation (ncollide3d query::ContactKinematic::contact, used by
// NonlinearSORProx at src/solver/nonlinear_sor_prox.rs:221-229) and one-shot
// manifolds for ball-ball, ball-cuboid and cuboid-cuboid pairs (ncollide3d's
// NarrowPhase, driven by src/world/geometrical_world.rs:315-320), and for
// capsules (a segment along the local y axis dilated by a radius) against
// balls, capsules and cuboids.
//
// Methods: SAT over the 15 box axes with a bias toward face axes, then
// Sutherland-Hodgman clipping of the incident face against the reference
// face with per-point feature tracking, and a 4-point reduction; Ericson's
// segment-segment closest points. Feature ids of a cuboid: vertices 0-7,
// edges 8-19, faces 20-25; a ball has the single feature 0; a capsule has its
// axis (0, a segment) and its two ends (1 at -half_height, 2 at +half_height,
// points), each dilated by the radius.
#pragma once
#include <cfloat>
#include "dyn.cuh"

namespace npgpu_dev {

enum { AP_POINT = 1, AP_SEGMENT = 2, AP_PLANE = 3 };
enum { SHAPE_BALL = 0, SHAPE_CUBOID = 1, SHAPE_CAPSULE = 3 };

struct Approx {
    int kind;
    np::V a, b;
};

__device__ __forceinline__ int box_vertex_id(int sx, int sy, int sz) { return sx | (sy << 1) | (sz << 2); }
__device__ __forceinline__ void edge_other_axes(int a, int& o1, int& o2) {
    o1 = (a == 0) ? 1 : 0;
    o2 = (a == 2) ? 1 : 2;
}
__device__ __forceinline__ int box_edge_id(int axis, int s1, int s2) { return 8 + 4 * axis + (s1 | (s2 << 1)); }
__device__ __forceinline__ int box_face_id(int axis, int pos) { return 20 + 2 * axis + pos; }

__device__ __forceinline__ Approx box_feature(np::V h, int fid) {
    Approx ap;
    np::V z = np::mk(0.0f, 0.0f, 0.0f);
    if (fid < 8) {
        ap.kind = AP_POINT;
        ap.a = np::mk((fid & 1) ? h.x : -h.x, (fid & 2) ? h.y : -h.y, (fid & 4) ? h.z : -h.z);
        ap.b = z;
    } else if (fid < 20) {
        int e = fid - 8, axis = e / 4, bits = e % 4, o1, o2;
        edge_other_axes(axis, o1, o2);
        np::V p = z;
        np::setc(p, o1, (bits & 1) ? np::comp(h, o1) : -np::comp(h, o1));
        np::setc(p, o2, (bits & 2) ? np::comp(h, o2) : -np::comp(h, o2));
        ap.kind = AP_SEGMENT;
        ap.a = p;
        ap.b = p;
        np::setc(ap.a, axis, -np::comp(h, axis));
        np::setc(ap.b, axis, np::comp(h, axis));
    } else {
        int f = fid - 20, axis = f / 2, pos = f % 2;
        ap.kind = AP_PLANE;
        ap.a = z;
        ap.b = z;
        np::setc(ap.a, axis, pos ? np::comp(h, axis) : -np::comp(h, axis));
        np::setc(ap.b, axis, pos ? 1.0f : -1.0f);
    }
    return ap;
}

// A capsule's feature: its axis (fid 0) or one of its ends (1, 2); h = (radius, half_height, 0).
__device__ __forceinline__ Approx capsule_feature(np::V h, int fid) {
    Approx ap;
    const np::V lo = np::mk(0.0f, -h.y, 0.0f), hi = np::mk(0.0f, h.y, 0.0f);
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

__device__ __forceinline__ Approx feature_of(uint32_t shape, np::V h, int fid) {
    if (shape == SHAPE_BALL) {
        Approx ap;
        ap.kind = AP_POINT;
        ap.a = ap.b = np::mk(0.0f, 0.0f, 0.0f);
        return ap;
    }
    if (shape == SHAPE_CAPSULE) return capsule_feature(h, fid);
    return box_feature(h, fid);
}

__device__ __forceinline__ float clamp01(float x) { return np_min(np_max(x, 0.0f), 1.0f); }

// Ericson, Real-Time Collision Detection 5.1.9. The segments' parameters of
// the closest points go to *so and *to when given.
__device__ __forceinline__ void closest_segment_segment(np::V p1, np::V q1, np::V p2, np::V q2, np::V& c1, np::V& c2,
                                                        float* so = nullptr, float* to = nullptr) {
    const float eps = FLT_EPSILON;
    np::V d1 = np::sub(q1, p1), d2 = np::sub(q2, p2), r = np::sub(p1, p2);
    float a = np::dot(d1, d1), e = np::dot(d2, d2), f = np::dot(d2, r);
    float s, t;
    if (a <= eps && e <= eps) {
        s = 0.0f;
        t = 0.0f;
    } else if (a <= eps) {
        s = 0.0f;
        t = clamp01(f / e);
    } else {
        float c = np::dot(d1, r);
        if (e <= eps) {
            t = 0.0f;
            s = clamp01(-c / a);
        } else {
            float b = np::dot(d1, d2);
            float denom = a * e - b * b;
            s = (denom != 0.0f) ? clamp01((b * f - c * e) / denom) : 0.0f;
            t = (b * s + f) / e;
            if (t < 0.0f) {
                t = 0.0f;
                s = clamp01(-c / a);
            } else if (t > 1.0f) {
                t = 1.0f;
                s = clamp01((b - c) / a);
            }
        }
    }
    c1 = np::add(p1, np::mul(d1, s));
    c2 = np::add(p2, np::mul(d2, t));
    if (so) *so = s;
    if (to) *to = t;
}

struct Geom {
    np::V w1, w2, n;
    float depth;
};

// ContactKinematic::contact for Point / Segment / Plane approximations.
__device__ __forceinline__ Geom kinematic_contact(const Approx& a1, const np::Iso& m1, float dil1, const Approx& a2,
                                                  const np::Iso& m2, float dil2, np::V n0) {
    np::V q1, q2, n;
    float s;
    if (a1.kind == AP_PLANE && a2.kind == AP_POINT) {
        n = np::qrot(m1.q, a1.b);
        np::V p1 = np::iso_pt(m1, a1.a);
        np::V p2 = np::iso_pt(m2, a2.a);
        s = np::dot(np::sub(p2, p1), n);
        q1 = np::sub(p2, np::mul(n, s));
        q2 = p2;
    } else if (a1.kind == AP_POINT && a2.kind == AP_PLANE) {
        np::V n2 = np::qrot(m2.q, a2.b);
        np::V p1 = np::iso_pt(m1, a1.a);
        np::V p2 = np::iso_pt(m2, a2.a);
        s = np::dot(np::sub(p1, p2), n2);
        q1 = p1;
        q2 = np::sub(p1, np::mul(n2, s));
        n = np::neg(n2);
    } else {
        np::V s1a = np::iso_pt(m1, a1.a);
        np::V s1b = (a1.kind == AP_SEGMENT) ? np::iso_pt(m1, a1.b) : s1a;
        np::V s2a = np::iso_pt(m2, a2.a);
        np::V s2b = (a2.kind == AP_SEGMENT) ? np::iso_pt(m2, a2.b) : s2a;
        closest_segment_segment(s1a, s1b, s2a, s2b, q1, q2);
        np::V v = np::sub(q2, q1);
        float l2 = np::dot(v, v);
        const float eps = FLT_EPSILON;
        if (l2 > eps * eps) {
            float l = sqrtf(l2);
            n = np::divs(v, l);
            s = l;
            if (np::dot(n, n0) < 0.0f) {
                n = np::neg(n);
                s = -l;
            }
        } else {
            n = n0;
            s = 0.0f;
        }
    }
    Geom g;
    g.w1 = np::add(q1, np::mul(n, dil1));
    g.w2 = np::sub(q2, np::mul(n, dil2));
    g.n = n;
    g.depth = (dil1 + dil2) - s;
    return g;
}

// A collider as seen by the narrow phase.
struct Shape {
    uint32_t shape;
    np::V h;         // half extents (cuboid) or (radius, 0, 0)
    float radius;
    np::Iso pose;
    __device__ float dil() const { return (shape == SHAPE_BALL || shape == SHAPE_CAPSULE) ? radius : 0.0f; }
};

struct Cand {
    int f1, f2;
    Geom g;
};

// Candidate contacts: up to 8 from a clipped polygon, of which a manifold
// keeps at most 4.
template <int N>
struct CandListN {
    Cand c[N];
    int n;
};
using CandList = CandListN<8>;

template <int N>
__device__ __forceinline__ void push_eval(CandListN<N>& out, const Shape& s1, const Shape& s2, int f1, int f2, np::V n0,
                                          float prediction) {
    Geom g = kinematic_contact(feature_of(s1.shape, s1.h, f1), s1.pose, s1.dil(), feature_of(s2.shape, s2.h, f2),
                               s2.pose, s2.dil(), n0);
    if (g.depth >= -prediction && out.n < N) {
        out.c[out.n].f1 = f1;
        out.c[out.n].f2 = f2;
        out.c[out.n].g = g;
        out.n++;
    }
}

// A sphere around `centre` (feature sfid of shape sb: a ball, or a capsule's
// end) against cuboid sx: the closest point of the cuboid to the centre.
__device__ __forceinline__ void sphere_box(const Shape& sb, int sfid, np::V centre, const Shape& sx, bool box_first,
                                           float prediction, CandList& out) {
    np::V c = np::iso_inv_pt(sx.pose, centre);
    np::V h = sx.h;
    int sign[3], nclamped = 0;
    np::V p = c;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float ck = np::comp(c, k), hk = np::comp(h, k);
        if (ck > hk) {
            sign[k] = 1;
            np::setc(p, k, hk);
            ++nclamped;
        } else if (ck < -hk) {
            sign[k] = -1;
            np::setc(p, k, -hk);
            ++nclamped;
        } else {
            sign[k] = 0;
        }
    }
    int fid;
    np::V nl;
    if (nclamped == 0) {
        int best = 0;
        float bd = np::comp(h, 0) - fabsf(np::comp(c, 0));
        for (int k = 1; k < 3; ++k) {
            float dk = np::comp(h, k) - fabsf(np::comp(c, k));
            if (dk < bd) {
                bd = dk;
                best = k;
            }
        }
        int pos = np::comp(c, best) >= 0.0f ? 1 : 0;
        fid = box_face_id(best, pos);
        nl = np::mk(0.0f, 0.0f, 0.0f);
        np::setc(nl, best, pos ? 1.0f : -1.0f);
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
        np::V v = np::sub(c, p);
        nl = np::divs(v, np::norm(v));
    }
    np::V n = np::qrot(sx.pose.q, nl);
    if (box_first) push_eval(out, sx, sb, fid, sfid, n, prediction);
    else push_eval(out, sb, sx, sfid, fid, np::neg(n), prediction);
}

// Ball (sb) against cuboid (sx): closest point of the cuboid to the center.
__device__ __forceinline__ void ball_box(const Shape& sb, const Shape& sx, bool box_first, float prediction,
                                         CandList& out) {
    sphere_box(sb, 0, sb.pose.t, sx, box_first, prediction, out);
}

// A capsule's axis in world coordinates.
__device__ __forceinline__ void capsule_axis(const Shape& s, np::V& p0, np::V& p1) {
    p0 = np::iso_pt(s.pose, np::mk(0.0f, -s.h.y, 0.0f));
    p1 = np::iso_pt(s.pose, np::mk(0.0f, s.h.y, 0.0f));
}

// Unit vector along v, or `fallback` for a null v.
__device__ __forceinline__ np::V unit_or(np::V v, np::V fallback) {
    const float l2 = np::dot(v, v);
    return l2 > FLT_EPSILON * FLT_EPSILON ? np::divs(v, sqrtf(l2)) : fallback;
}

// Ball (sb) against capsule (sc): the closest point of the capsule's axis.
__device__ __forceinline__ void ball_capsule(const Shape& sb, const Shape& sc, bool capsule_first, float prediction,
                                             CandList& out) {
    np::V p0, p1, qa, qb;
    capsule_axis(sc, p0, p1);
    closest_segment_segment(p0, p1, sb.pose.t, sb.pose.t, qa, qb);
    const np::V n0 = unit_or(np::sub(qb, qa), np::mk(1.0f, 0.0f, 0.0f));   // from the capsule toward the ball
    if (capsule_first) push_eval(out, sc, sb, 0, 0, n0, prediction);
    else push_eval(out, sb, sc, 0, 0, np::neg(n0), prediction);
}

// Capsule A (collider 1) against capsule B: the closest points of the axes;
// for parallel axes (sine below 1e-3), the two ends of their overlap.
__device__ __forceinline__ void capsule_capsule(const Shape& A, const Shape& B, float prediction, CandList& out) {
    np::V a0, a1, b0, b1, qa, qb;
    capsule_axis(A, a0, a1);
    capsule_axis(B, b0, b1);
    closest_segment_segment(a0, a1, b0, b1, qa, qb);
    const np::V da = np::sub(a1, a0), db = np::sub(b1, b0);
    const np::V cr = np::cross(da, db);
    const np::V n0 = unit_or(np::sub(qb, qa), unit_or(cr, np::mk(1.0f, 0.0f, 0.0f)));
    const float la2 = np::dot(da, da), lb2 = np::dot(db, db);
    if (np::dot(cr, cr) > 1e-6f * la2 * lb2 || la2 <= FLT_EPSILON) {
        push_eval(out, A, B, 0, 0, n0, prediction);
        return;
    }
    // Parallel: B's ends projected on A's axis (parameters in A's length).
    const float tb0 = np::dot(np::sub(b0, a0), da) / la2, tb1 = np::dot(np::sub(b1, a0), da) / la2;
    const int flo = tb0 <= tb1 ? 1 : 2, fhi = tb0 <= tb1 ? 2 : 1;
    const float blo = tb0 <= tb1 ? tb0 : tb1, bhi = tb0 <= tb1 ? tb1 : tb0;
    if (bhi < 0.0f || blo > 1.0f) {
        push_eval(out, A, B, 0, 0, n0, prediction);
        return;
    }
    if (blo > 0.0f) push_eval(out, A, B, 0, flo, n0, prediction);
    else push_eval(out, A, B, 1, 0, n0, prediction);
    if (bhi < 1.0f) push_eval(out, A, B, 0, fhi, n0, prediction);
    else push_eval(out, A, B, 2, 0, n0, prediction);
}

// push_eval for a candidate whose feature pair is not already in `out`.
template <int N>
__device__ __forceinline__ void push_eval_unique(CandListN<N>& out, const Shape& s1, const Shape& s2, int f1, int f2,
                                                 np::V n0, float prediction) {
    for (int k = 0; k < out.n; ++k)
        if (out.c[k].f1 == f1 && out.c[k].f2 == f2) return;
    push_eval(out, s1, s2, f1, f2, n0, prediction);
}

// The cuboid edge where face (k, sk) meets the side plane (o, so); sk, so = +-1.
__device__ __forceinline__ int face_side_edge(int k, int sk, int o, int so) {
    const int a = 3 - k - o;
    int o1, o2;
    edge_other_axes(a, o1, o2);
    const int s1 = (o1 == k ? sk : so) > 0 ? 1 : 0, s2 = (o2 == k ? sk : so) > 0 ? 1 : 0;
    return box_edge_id(a, s1, s2);
}

__device__ __forceinline__ int vertex_at(np::V p) { return box_vertex_id(p.x > 0.0f, p.y > 0.0f, p.z > 0.0f); }

// Capsule (sc) against cuboid (sx). The reference face is the cuboid face
// farthest from the capsule's axis (the largest of the six face separations
// of the axis's nearer end); the axis is clipped to that face's rectangle and
// each end of the clipped axis gives a candidate: an end of the capsule
// against the face (point-plane), or the axis against the face edge that
// clipped it (segment-segment). When the axis does not overlap the face's
// rectangle, the candidates are each end of the capsule as a sphere against
// the cuboid, and the axis against the nearest cuboid edge: an edge-edge
// contact when both closest points lie inside their segments, or, for an
// axis parallel to the edge (sine below 1e-3), the two ends of their overlap.
__device__ __forceinline__ void capsule_box(const Shape& sc, const Shape& sx, bool box_first, float prediction,
                                            CandList& out) {
    np::V p0, p1;
    capsule_axis(sc, p0, p1);
    const np::V l0 = np::iso_inv_pt(sx.pose, p0), l1 = np::iso_inv_pt(sx.pose, p1);
    const np::V h = sx.h;
    // A candidate (cuboid feature fb, capsule feature fc) with the default
    // normal nl (cuboid frame, from the cuboid toward the capsule).
    auto cand = [&](int fb, int fc, np::V nl) {
        const np::V n = np::qrot(sx.pose.q, nl);
        if (box_first) push_eval_unique(out, sx, sc, fb, fc, n, prediction);
        else push_eval_unique(out, sc, sx, fc, fb, np::neg(n), prediction);
    };
    int k = 0, sk = 1;
    float best = -FLT_MAX;
    for (int a = 0; a < 3; ++a) {
        for (int sg = 1; sg >= -1; sg -= 2) {
            const float e0 = (float)sg * np::comp(l0, a), e1 = (float)sg * np::comp(l1, a);
            const float sep = (e0 < e1 ? e0 : e1) - np::comp(h, a);
            if (sep > best) {
                best = sep;
                k = a;
                sk = sg;
            }
        }
    }
    np::V nf = np::mk(0.0f, 0.0f, 0.0f);
    np::setc(nf, k, (float)sk);
    const int face = box_face_id(k, sk > 0 ? 1 : 0);
    float tlo = 0.0f, thi = 1.0f;
    int elo = -1, ehi = -1;
    bool empty = false;
    for (int o = 0; o < 3 && !empty; ++o) {
        if (o == k) continue;
        for (int so = 1; so >= -1 && !empty; so -= 2) {
            const float f0 = (float)so * np::comp(l0, o) - np::comp(h, o);
            const float f1 = (float)so * np::comp(l1, o) - np::comp(h, o);
            if (f0 > 0.0f && f1 > 0.0f) {
                empty = true;
            } else if (f0 > 0.0f) {
                const float t = f0 / (f0 - f1);
                if (t > tlo) {
                    tlo = t;
                    elo = face_side_edge(k, sk, o, so);
                }
            } else if (f1 > 0.0f) {
                const float t = f0 / (f0 - f1);
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
    sphere_box(sc, 1, p0, sx, box_first, prediction, out);
    sphere_box(sc, 2, p1, sx, box_first, prediction, out);
    // The nearest edge; at equal distances (a shared vertex) the edge most
    // parallel to the axis.
    int be = -1;
    float bd = FLT_MAX, bp = -1.0f, bs = 0.0f, bt = 0.0f;
    np::V bq = np::mk(0.0f, 0.0f, 0.0f), bqe = bq;
    const np::V dl0 = np::sub(l1, l0);
    for (int e = 0; e < 12; ++e) {
        const Approx ed = box_feature(h, 8 + e);
        np::V qa, qe;
        float sa, te;
        closest_segment_segment(l0, l1, ed.a, ed.b, qa, qe, &sa, &te);
        const np::V v = np::sub(qa, qe);
        const float d2 = np::dot(v, v);
        const np::V de0 = np::sub(ed.b, ed.a);
        const float c = np::dot(dl0, de0), par = c * c / (np::dot(dl0, dl0) * np::dot(de0, de0) + FLT_MIN);
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
    const Approx ed = box_feature(h, 8 + be);
    const np::V nl = unit_or(np::sub(bq, bqe), unit_or(bq, np::mk(0.0f, 1.0f, 0.0f)));
    const np::V dl = np::sub(l1, l0), de = np::sub(ed.b, ed.a);
    const np::V cr = np::cross(dl, de);
    const float ll2 = np::dot(dl, dl);
    if (np::dot(cr, cr) > 1e-6f * ll2 * np::dot(de, de) || ll2 <= FLT_EPSILON) {
        if (bs > 0.0f && bs < 1.0f && bt > 0.0f && bt < 1.0f) cand(8 + be, 0, nl);
        return;
    }
    // Parallel: the edge's ends projected on the axis (parameters in its length).
    const float ta = np::dot(np::sub(ed.a, l0), dl) / ll2, tb = np::dot(np::sub(ed.b, l0), dl) / ll2;
    const np::V vlo = ta <= tb ? ed.a : ed.b, vhi = ta <= tb ? ed.b : ed.a;
    const float lo = ta <= tb ? ta : tb, hi = ta <= tb ? tb : ta;
    if (hi < 0.0f || lo > 1.0f) return;
    if (lo > 0.0f) cand(vertex_at(vlo), 0, nl);
    else cand(8 + be, 1, nl);
    if (hi < 1.0f) cand(vertex_at(vhi), 0, nl);
    else cand(8 + be, 2, nl);
}

// A vertex of the clipped polygon and where it comes from, packed in one
// word: tag (2 bits: incident vertex, edge crossing, reference corner), a and
// b (feature ids, -1 allowed) and esrc (the incident edge it lies on, or
// -(1 + clipping plane)).
struct PV {
    np::V p;
    uint32_t bits;
    __device__ __forceinline__ int tag() const { return (int)(bits & 3u); }
    __device__ __forceinline__ int a() const { return (int)((bits >> 2) & 63u) - 1; }
    __device__ __forceinline__ int b() const { return (int)((bits >> 8) & 63u) - 1; }
    __device__ __forceinline__ int esrc() const { return (int)((bits >> 14) & 63u) - 8; }
    __device__ __forceinline__ void set(int tag, int a, int b, int esrc) {
        bits = (uint32_t)tag | ((uint32_t)(a + 1) << 2) | ((uint32_t)(b + 1) << 8) | ((uint32_t)(esrc + 8) << 14);
    }
};

// Keeps at most 4 candidates (deepest, farthest, largest triangle, largest
// growth), in their original order. Writes the kept indices to keep[].
__device__ __forceinline__ int reduce4(const CandListN<8>& c, int keep[4]) {
    int n = c.n;
    if (n <= 4) {
        for (int k = 0; k < n; ++k) keep[k] = k;
        return n;
    }
    int i0 = 0;
    for (int k = 1; k < n; ++k)
        if (c.c[k].g.depth > c.c[i0].g.depth) i0 = k;
    int i1 = -1;
    float bd = -1.0f;
    for (int k = 0; k < n; ++k) {
        if (k == i0) continue;
        np::V d = np::sub(c.c[k].g.w1, c.c[i0].g.w1);
        float dd = np::dot(d, d);
        if (dd > bd) {
            bd = dd;
            i1 = k;
        }
    }
    int i2 = -1;
    float ba = -1.0f;
    np::V e01 = np::sub(c.c[i1].g.w1, c.c[i0].g.w1);
    for (int k = 0; k < n; ++k) {
        if (k == i0 || k == i1) continue;
        np::V cr = np::cross(e01, np::sub(c.c[k].g.w1, c.c[i0].g.w1));
        float aa = np::dot(cr, cr);
        if (aa > ba) {
            ba = aa;
            i2 = k;
        }
    }
    int i3 = -1;
    float bs = -1.0f;
    np::V a = c.c[i0].g.w1, b = c.c[i1].g.w1, cc = c.c[i2].g.w1;
    for (int k = 0; k < n; ++k) {
        if (k == i0 || k == i1 || k == i2) continue;
        np::V x = c.c[k].g.w1;
        float s = np::norm(np::cross(np::sub(x, a), np::sub(x, b))) + np::norm(np::cross(np::sub(x, b), np::sub(x, cc))) +
                  np::norm(np::cross(np::sub(x, cc), np::sub(x, a)));
        if (s > bs) {
            bs = s;
            i3 = k;
        }
    }
    int m = 0;
    for (int k = 0; k < n; ++k)
        if (k == i0 || k == i1 || k == i2 || k == i3) keep[m++] = k;
    return m;
}

// ax[k] for a k known only at run time, by selects (keeps ax in registers).
__device__ __forceinline__ np::V pick3(const np::V ax[3], int k) { return k == 0 ? ax[0] : (k == 1 ? ax[1] : ax[2]); }

__device__ __forceinline__ float box_radius_along(const np::V ax[3], np::V h, np::V L) {
    return h.x * fabsf(np::dot(ax[0], L)) + h.y * fabsf(np::dot(ax[1], L)) + h.z * fabsf(np::dot(ax[2], L));
}

// Cuboid A (collider 1) against cuboid B (collider 2).
// The candidates go to `out`; keep[0..return) are the indices the manifold
// keeps, in increasing order.
static __device__ __noinline__ int box_box(const Shape& A, const Shape& B, float prediction, CandList& out,
                                           int keep[kMaxContacts]) {
    np::M RA = np::qmat(A.pose.q), RB = np::qmat(B.pose.q);
    np::V axA[3] = {np::mcol(RA, 0), np::mcol(RA, 1), np::mcol(RA, 2)};
    np::V axB[3] = {np::mcol(RB, 0), np::mcol(RB, 1), np::mcol(RB, 2)};
    np::V d = np::sub(B.pose.t, A.pose.t);
    float sepA = -FLT_MAX, sepB = -FLT_MAX, sepE = -FLT_MAX;
    int ia = 0, ib = 0, ea = -1, eb = -1;
    np::V LE = np::mk(0.0f, 0.0f, 0.0f);
    for (int i = 0; i < 3; ++i) {
        np::V L = axA[i];
        float rb = box_radius_along(axB, B.h, L);
        float sep = fabsf(np::dot(d, L)) - (np::comp(A.h, i) + rb);
        if (sep > prediction) return 0;
        if (sep > sepA) {
            sepA = sep;
            ia = i;
        }
    }
    for (int j = 0; j < 3; ++j) {
        np::V L = axB[j];
        float ra = box_radius_along(axA, A.h, L);
        float sep = fabsf(np::dot(d, L)) - (ra + np::comp(B.h, j));
        if (sep > prediction) return 0;
        if (sep > sepB) {
            sepB = sep;
            ib = j;
        }
    }
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            np::V L = np::cross(axA[i], axB[j]);
            float len = np::norm(L);
            if (len < 1e-5f) continue;
            L = np::divs(L, len);
            float ra = box_radius_along(axA, A.h, L);
            float rb = box_radius_along(axB, B.h, L);
            float sep = fabsf(np::dot(d, L)) - (ra + rb);
            if (sep > prediction) return 0;
            if (sep > sepE) {
                sepE = sep;
                ea = i;
                eb = j;
                LE = L;
            }
        }
    }
    bool refA = !(sepB > sepA + 1e-4f);
    float sepF = refA ? sepA : sepB;
    if (ea >= 0 && sepE > sepF + 5e-3f) {
        np::V L = LE;
        if (np::dot(d, L) < 0.0f) L = np::neg(L);
        int o1, o2;
        edge_other_axes(ea, o1, o2);
        int fa = box_edge_id(ea, np::dot(pick3(axA, o1), L) > 0.0f ? 1 : 0, np::dot(pick3(axA, o2), L) > 0.0f ? 1 : 0);
        edge_other_axes(eb, o1, o2);
        int fb = box_edge_id(eb, np::dot(pick3(axB, o1), L) < 0.0f ? 1 : 0, np::dot(pick3(axB, o2), L) < 0.0f ? 1 : 0);
        push_eval(out, A, B, fa, fb, L, prediction);
        keep[0] = 0;
        return out.n;
    }
    const Shape& Rf = refA ? A : B;
    const Shape& In = refA ? B : A;
    const np::V axR[3] = {refA ? axA[0] : axB[0], refA ? axA[1] : axB[1], refA ? axA[2] : axB[2]};
    const np::V axI[3] = {refA ? axB[0] : axA[0], refA ? axB[1] : axA[1], refA ? axB[2] : axA[2]};
    int ri = refA ? ia : ib;
    np::V dRI = refA ? d : np::neg(d);
    const np::V axr = pick3(axR, ri);
    int rpos = np::dot(dRI, axr) >= 0.0f ? 1 : 0;
    np::V nref = rpos ? axr : np::neg(axr);
    int ik = 0;
    float best = fabsf(np::dot(axI[0], nref));
    for (int k = 1; k < 3; ++k) {
        float v = fabsf(np::dot(axI[k], nref));
        if (v > best) {
            best = v;
            ik = k;
        }
    }
    int ipos = np::dot(pick3(axI, ik), nref) < 0.0f ? 1 : 0;
    int ref_face = box_face_id(ri, rpos), inc_face = box_face_id(ik, ipos);
    int u = (ik + 1) % 3, v = (ik + 2) % 3;
    const int su[4] = {0, 1, 1, 0}, sv[4] = {0, 0, 1, 1};
    PV poly[8], next[8];
    int np_ = 0, nn = 0;
    int vids[4];
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
        Approx ap = box_feature(In.h, a);
        np::V w = np::iso_pt(In.pose, ap.a);
        poly[np_].p = np::iso_inv_pt(Rf.pose, w);
        poly[np_].set(0, a, -1, eid);
        ++np_;
    }
    int ru = (ri + 1) % 3, rv = (ri + 2) % 3;
    const int planes_axis[4] = {ru, ru, rv, rv};
    const int planes_pos[4] = {1, 0, 1, 0};
    for (int pl = 0; pl < 4 && np_ > 0; ++pl) {
        int ax = planes_axis[pl], pp = planes_pos[pl];
        float hc = np::comp(Rf.h, ax);
        nn = 0;
        for (int k = 0; k < np_; ++k) {
            const PV P = poly[k];
            const PV Q = poly[(k + 1) % np_];
            float dp = (pp ? np::comp(P.p, ax) : -np::comp(P.p, ax)) - hc;
            float dq = (pp ? np::comp(Q.p, ax) : -np::comp(Q.p, ax)) - hc;
            bool pin = dp <= 0.0f, qin = dq <= 0.0f;
            if (pin && nn < 8) next[nn++] = P;
            if (pin != qin) {
                float t = dp / (dp - dq);
                PV X;
                X.p = np::add(P.p, np::mul(np::sub(Q.p, P.p), t));
                int third = 3 - ri - ax;
                int s[3];
                s[ri] = rpos;
                s[ax] = pp;
                const int pe = P.esrc();
                const int xe = pin ? -(1 + pl) : pe;
                if (pe >= 0) {
                    int o1, o2;
                    edge_other_axes(third, o1, o2);
                    X.set(1, box_edge_id(third, s[o1], s[o2]), pe, xe);
                } else {
                    int other_plane = -pe - 1;
                    s[planes_axis[other_plane]] = planes_pos[other_plane];
                    X.set(2, box_vertex_id(s[0], s[1], s[2]), -1, xe);
                }
                if (nn < 8) next[nn++] = X;
            }
        }
        for (int k = 0; k < nn; ++k) poly[k] = next[k];
        np_ = nn;
    }
    np::V n0 = refA ? nref : np::neg(nref);
    CandList& cands = out;
    for (int k = 0; k < np_; ++k) {
        const PV& P = poly[k];
        int fr, fi;
        if (P.tag() == 0) {
            fr = ref_face;
            fi = P.a();
        } else if (P.tag() == 1) {
            fr = P.a();
            fi = P.b();
        } else {
            fr = P.a();
            fi = inc_face;
        }
        if (refA) push_eval(cands, A, B, fr, fi, n0, prediction);
        else push_eval(cands, A, B, fi, fr, n0, prediction);
    }
    return reduce4(cands, keep);
}

// The contacts of two posed shapes within `prediction`: the candidates in
// `out` and the ones the manifold keeps, keep[0 .. returned count).
__device__ __forceinline__ int shape_pair_contacts(const Shape& a, const Shape& b, float prediction, CandList& out,
                                                   int keep[kMaxContacts]) {
    out.n = 0;
    for (int k = 0; k < kMaxContacts; ++k) keep[k] = k;
    if (a.shape == SHAPE_BALL && b.shape == SHAPE_BALL) {
        np::V v = np::sub(b.pose.t, a.pose.t);
        float l2 = np::dot(v, v);
        np::V n0 = l2 > 0.0f ? np::divs(v, sqrtf(l2)) : np::mk(1.0f, 0.0f, 0.0f);
        push_eval(out, a, b, 0, 0, n0, prediction);
        return out.n;
    }
    if (a.shape == SHAPE_CUBOID && b.shape == SHAPE_BALL) {
        ball_box(b, a, true, prediction, out);
        return out.n;
    }
    if (a.shape == SHAPE_BALL && b.shape == SHAPE_CUBOID) {
        ball_box(a, b, false, prediction, out);
        return out.n;
    }
    if (a.shape == SHAPE_CAPSULE || b.shape == SHAPE_CAPSULE) {
        if (a.shape == SHAPE_CAPSULE && b.shape == SHAPE_CAPSULE) capsule_capsule(a, b, prediction, out);
        else if (a.shape == SHAPE_BALL) ball_capsule(a, b, false, prediction, out);
        else if (b.shape == SHAPE_BALL) ball_capsule(b, a, true, prediction, out);
        else if (a.shape == SHAPE_CUBOID) capsule_box(b, a, true, prediction, out);
        else capsule_box(a, b, false, prediction, out);
        return out.n;
    }
    return box_box(a, b, prediction, out, keep);
}

}  // namespace npgpu_dev
