// k_query.cu -- geometric queries against the world's colliders on the device.
//
// GeometricalWorld::interferences_with_ray / _with_point / _with_aabb
// (src/world/geometrical_world.rs:327-370) for batches of queries. They read
// the linear BVH of the last collision-detection pass (the broad phase's fat
// AABBs) and the colliders' poses of that pass, as the reference's queries
// read its DBVT proxies and the colliders' positions synced by the step:
//  - ray: every collider whose shape the ray (origin + t dir, t in
//    [0, max_toi], dir not normalised) hits; shapes are solid, so a ray that
//    starts inside hits at t = 0 with a zero normal. The ball test solves the
//    sphere's quadratic, the cuboid test clips the ray against the three slabs
//    in the cuboid's frame (Kay and Kajiya), the normal being the face of the
//    last slab entered; a capsule is the union of its cylinder (clipped to the
//    axis's extent) and its two end spheres, the first hit the earliest.
//  - point: every collider whose shape contains the point (boundary included).
//  - aabb: every collider whose fat AABB intersects the box (closed boxes),
//    the broad-phase test the reference's query makes.
// Each query kind runs twice: a counting pass, then (after an exclusive scan
// of the counts) a writing pass that stores each query's hits at its offset.
#include "narrow.cuh"
#include "sortscan.cuh"

namespace npgpu_dev {
namespace {

constexpr int kQThreads = 128;

struct QHit {
    uint32_t q, collider;
    float toi, nx, ny, nz;
};

enum { Q_RAY = 0, Q_POINT = 1, Q_AABB = 2 };

__device__ __forceinline__ Shape query_shape(const Colliders& c, uint32_t i) {
    Shape s;
    s.shape = c.info[i] & 0xfu;
    float4 p = c.params[i];
    s.h = np::mk(p.x, p.y, p.z);
    s.radius = p.x;
    s.pose.t = np::mk(c.pose_t[i].x, c.pose_t[i].y, c.pose_t[i].z);
    const float4 q = c.pose_q[i];
    s.pose.q = np::Q{q.x, q.y, q.z, q.w};
    return s;
}

// First entry of a ray into the sphere of centre c and radius r, from a
// start outside it (t = -1 when it misses).
__device__ __forceinline__ float ray_sphere_entry(np::V o, np::V d, np::V c, float r) {
    const np::V m = np::sub(o, c);
    const float a = np::dot(d, d), b = np::dot(m, d), cc = np::dot(m, m) - r * r;
    if ((cc > 0.0f && b > 0.0f) || a == 0.0f) return -1.0f;
    const float disc = b * b - a * cc;
    if (disc < 0.0f) return -1.0f;
    return (-b - sqrtf(disc)) / a;
}

// Ray against a solid capsule (axis along its local y, half height h.y, radius h.x).
__device__ __forceinline__ bool ray_capsule(np::V o, np::V d, const Shape& s, float max_toi, float& toi, np::V& n) {
    const np::V lo = np::qrot_inv(s.pose.q, np::sub(o, s.pose.t));
    const np::V ld = np::qrot_inv(s.pose.q, d);
    const float r = s.h.x, hh = s.h.y;
    {
        np::V qa, qb;
        closest_segment_segment(np::mk(0.0f, -hh, 0.0f), np::mk(0.0f, hh, 0.0f), lo, lo, qa, qb);
        const np::V v = np::sub(qb, qa);
        if (np::dot(v, v) <= r * r) {
            toi = 0.0f;
            n = np::mk(0.0f, 0.0f, 0.0f);
            return true;
        }
    }
    float best = INFINITY;
    np::V bn = np::mk(0.0f, 0.0f, 0.0f);
    const float a = ld.x * ld.x + ld.z * ld.z;
    if (a > 0.0f) {
        const float b = lo.x * ld.x + lo.z * ld.z, c = lo.x * lo.x + lo.z * lo.z - r * r;
        const float disc = b * b - a * c;
        if (disc >= 0.0f) {
            const float t = (-b - sqrtf(disc)) / a;
            const float y = lo.y + t * ld.y;
            if (t >= 0.0f && fabsf(y) <= hh) {
                best = t;
                bn = np::divs(np::mk(lo.x + t * ld.x, 0.0f, lo.z + t * ld.z), r);
            }
        }
    }
    for (int e = 0; e < 2; ++e) {
        const np::V c = np::mk(0.0f, e ? hh : -hh, 0.0f);
        const float t = ray_sphere_entry(lo, ld, c, r);
        if (t >= 0.0f && t < best) {
            best = t;
            bn = np::divs(np::sub(np::add(lo, np::mul(ld, t)), c), r);
        }
    }
    if (!(best <= max_toi)) return false;
    toi = best;
    n = np::qrot(s.pose.q, bn);
    return true;
}

// Ray against a solid ball: the smaller root of |o + t d - c|^2 = r^2.
__device__ __forceinline__ bool ray_ball(np::V o, np::V d, const Shape& s, float max_toi, float& toi, np::V& n) {
    const np::V m = np::sub(o, s.pose.t);
    const float a = np::dot(d, d);
    const float b = np::dot(m, d);
    const float cc = np::dot(m, m) - s.radius * s.radius;
    if (cc > 0.0f && b > 0.0f) return false;   // outside and moving away
    const float disc = b * b - a * cc;
    if (disc < 0.0f || a == 0.0f) {
        if (cc <= 0.0f) {                     // a still point inside
            toi = 0.0f;
            n = np::mk(0.0f, 0.0f, 0.0f);
            return true;
        }
        return false;
    }
    float t = (-b - sqrtf(disc)) / a;
    if (t <= 0.0f) {
        toi = 0.0f;
        n = np::mk(0.0f, 0.0f, 0.0f);
        return true;
    }
    if (t > max_toi) return false;
    toi = t;
    const np::V hit = np::add(m, np::mul(d, t));
    const float l = sqrtf(np::dot(hit, hit));
    n = l > 0.0f ? np::divs(hit, l) : np::mk(0.0f, 0.0f, 0.0f);
    return true;
}

// Ray against a solid cuboid: the three slabs in the cuboid's frame.
__device__ __forceinline__ bool ray_cuboid(np::V o, np::V d, const Shape& s, float max_toi, float& toi, np::V& n) {
    const np::V lo = np::qrot_inv(s.pose.q, np::sub(o, s.pose.t));
    const np::V ld = np::qrot_inv(s.pose.q, d);
    const float os[3] = {lo.x, lo.y, lo.z}, ds[3] = {ld.x, ld.y, ld.z}, hs[3] = {s.h.x, s.h.y, s.h.z};
    float tmin = -INFINITY, tmax = INFINITY;
    int axis = -1;
    float sign = 0.0f;
    for (int i = 0; i < 3; ++i) {
        if (ds[i] == 0.0f) {
            if (os[i] < -hs[i] || os[i] > hs[i]) return false;
            continue;
        }
        float t1 = (-hs[i] - os[i]) / ds[i], t2 = (hs[i] - os[i]) / ds[i];
        float sg = -1.0f;                      // entering through the -h face
        if (t1 > t2) {
            const float x = t1;
            t1 = t2;
            t2 = x;
            sg = 1.0f;
        }
        if (t1 > tmin) {
            tmin = t1;
            axis = i;
            sign = sg;
        }
        if (t2 < tmax) tmax = t2;
        if (tmin > tmax) return false;
    }
    if (tmax < 0.0f) return false;
    if (tmin <= 0.0f || axis < 0) {
        toi = 0.0f;
        n = np::mk(0.0f, 0.0f, 0.0f);
        return true;
    }
    if (tmin > max_toi) return false;
    toi = tmin;
    np::V ln = np::mk(axis == 0 ? sign : 0.0f, axis == 1 ? sign : 0.0f, axis == 2 ? sign : 0.0f);
    n = np::qrot(s.pose.q, ln);
    return true;
}

__device__ __forceinline__ bool point_in(np::V p, const Shape& s) {
    if (s.shape == SHAPE_BALL) {
        const np::V m = np::sub(p, s.pose.t);
        return np::dot(m, m) <= s.radius * s.radius;
    }
    if (s.shape == SHAPE_CAPSULE) {
        const np::V l = np::qrot_inv(s.pose.q, np::sub(p, s.pose.t));
        np::V qa, qb;
        closest_segment_segment(np::mk(0.0f, -s.h.y, 0.0f), np::mk(0.0f, s.h.y, 0.0f), l, l, qa, qb);
        const np::V v = np::sub(qb, qa);
        return np::dot(v, v) <= s.h.x * s.h.x;
    }
    const np::V l = np::qrot_inv(s.pose.q, np::sub(p, s.pose.t));
    return fabsf(l.x) <= s.h.x && fabsf(l.y) <= s.h.y && fabsf(l.z) <= s.h.z;
}

// Slab test of a ray against a node's box for t in [0, max_toi].
__device__ __forceinline__ bool ray_box(np::V o, np::V d, float max_toi, float4 mn, float4 mx) {
    const float os[3] = {o.x, o.y, o.z}, ds[3] = {d.x, d.y, d.z};
    const float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    float t0 = 0.0f, t1 = max_toi;
    for (int i = 0; i < 3; ++i) {
        if (ds[i] == 0.0f) {
            if (os[i] < lo[i] || os[i] > hi[i]) return false;
            continue;
        }
        float a = (lo[i] - os[i]) / ds[i], b = (hi[i] - os[i]) / ds[i];
        if (a > b) {
            const float x = a;
            a = b;
            b = x;
        }
        t0 = a > t0 ? a : t0;
        t1 = b < t1 ? b : t1;
        if (t0 > t1) return false;
    }
    return true;
}

struct Query {
    int kind;
    np::V o, d;          // ray origin and direction, or the point (o)
    float max_toi;
    float4 bmin, bmax;   // the query box
};

__device__ __forceinline__ bool node_hit(const Query& q, float4 mn, float4 mx, uint32_t world) {
    if (world != 0xffffffffu && world < 0x10000u) {
        const uint32_t wr = __float_as_uint(mn.w);
        if (world < (wr >> 16) || world > (wr & 0xffffu)) return false;
    }
    if (q.kind == Q_RAY) return ray_box(q.o, q.d, q.max_toi, mn, mx);
    if (q.kind == Q_POINT)
        return q.o.x >= mn.x && q.o.x <= mx.x && q.o.y >= mn.y && q.o.y <= mx.y && q.o.z >= mn.z && q.o.z <= mx.z;
    return q.bmin.x <= mx.x && mn.x <= q.bmax.x && q.bmin.y <= mx.y && mn.y <= q.bmax.y && q.bmin.z <= mx.z &&
           mn.z <= q.bmax.z;
}

// The exact test of collider ci (its fat AABB already passed).
__device__ __forceinline__ bool leaf_hit(const World& w, const Query& q, uint32_t ci, uint32_t world, QHit& h) {
    if (world != 0xffffffffu && w.b.world[w.c.body[ci]] != world) return false;
    if (q.kind == Q_AABB) return true;
    const Shape s = query_shape(w.c, ci);
    if (q.kind == Q_POINT) return point_in(q.o, s);
    float toi = 0.0f;
    np::V n;
    const bool hit = s.shape == SHAPE_BALL      ? ray_ball(q.o, q.d, s, q.max_toi, toi, n)
                     : s.shape == SHAPE_CAPSULE ? ray_capsule(q.o, q.d, s, q.max_toi, toi, n)
                                                : ray_cuboid(q.o, q.d, s, q.max_toi, toi, n);
    if (hit) {
        h.toi = toi;
        h.nx = n.x;
        h.ny = n.y;
        h.nz = n.z;
    }
    return hit;
}

template <bool WRITE>
__global__ void k_query(World w, int kind, const float* qd, const float* max_toi, uint32_t nq, uint32_t world,
                        uint32_t* counts, const uint32_t* offsets, QHit* out, uint32_t cap_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    Query q;
    q.kind = kind;
    if (kind == Q_RAY) {
        q.o = np::mk(qd[6 * i], qd[6 * i + 1], qd[6 * i + 2]);
        q.d = np::mk(qd[6 * i + 3], qd[6 * i + 4], qd[6 * i + 5]);
        q.max_toi = max_toi[i];
    } else if (kind == Q_POINT) {
        q.o = np::mk(qd[3 * i], qd[3 * i + 1], qd[3 * i + 2]);
    } else {
        q.bmin = make_float4(qd[6 * i], qd[6 * i + 1], qd[6 * i + 2], 0.0f);
        q.bmax = make_float4(qd[6 * i + 3], qd[6 * i + 4], qd[6 * i + 5], 0.0f);
    }
    const int n = (int)w.nc_alive;
    uint32_t count = 0, base = WRITE ? offsets[i] : 0u;
    auto take = [&](uint32_t ci) {
        QHit h{i, ci, 0.0f, 0.0f, 0.0f, 0.0f};
        if (!leaf_hit(w, q, ci, world, h)) return;
        if (WRITE && base + count < cap_out) out[base + count] = h;
        ++count;
    };
    if (n == 1) {
        if (node_hit(q, w.c.node_min[0], w.c.node_max[0], world)) take(w.c.vals_sorted[0]);
    } else if (n >= 2 && node_hit(q, w.c.node_min[0], w.c.node_max[0], world)) {
        int stack[64];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const float4* wd = w.c.wide + 5 * (size_t)stack[--sp];
            const float4 lmin = wd[0], lmax = wd[1], rmin = wd[2], rmax = wd[3], refs = wd[4];
            const uint32_t lref = __float_as_uint(refs.x), rref = __float_as_uint(refs.y);
            const bool el = node_hit(q, lmin, lmax, world), er = node_hit(q, rmin, rmax, world);
            if (el && (lref & 0x80000000u)) take(lref & 0x7fffffffu);
            if (er && (rref & 0x80000000u)) take(rref & 0x7fffffffu);
            const bool pl = el && !(lref & 0x80000000u), pr = er && !(rref & 0x80000000u);
            if (sp + (int)pl + (int)pr > 64) {
                atomicOr(&w.ctl->err, ERRF_PAIR_CAPACITY);
                break;
            }
            if (pr) stack[sp++] = (int)rref;
            if (pl) stack[sp++] = (int)lref;
        }
    }
    if (!WRITE) counts[i] = count;
}

}  // namespace

size_t query_hit_bytes() { return sizeof(QHit); }

// Pass 1 (out == nullptr): counts[i] = hits of query i, offsets = their
// exclusive prefix sum. Pass 2: the hits, query i's at offsets[i].
cudaError_t launch_query(const World& w, int kind, const float* qd, const float* max_toi, uint32_t nq, uint32_t world,
                         uint32_t* counts, uint32_t* offsets, void* scan_temp, size_t scan_bytes, void* out,
                         uint32_t cap_out, cudaStream_t st) {
    if (nq == 0) return cudaSuccess;
    const unsigned blocks = (nq + kQThreads - 1) / kQThreads;
    if (out == nullptr) {
        k_query<false><<<blocks, kQThreads, 0, st>>>(w, kind, qd, max_toi, nq, world, counts, nullptr, nullptr, 0u);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        return exclusive_scan(scan_temp, scan_bytes, counts, offsets, nq, st);
    }
    k_query<true><<<blocks, kQThreads, 0, st>>>(w, kind, qd, max_toi, nq, world, counts, offsets, (QHit*)out,
                                                cap_out);
    return cudaGetLastError();
}

}  // namespace npgpu_dev
