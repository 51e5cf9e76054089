// k_cd.cu -- collision detection on the device.
//
// GeometricalWorld::sync_colliders + perform_broad_phase + perform_narrow_phase
// (src/world/geometrical_world.rs:230-265, 285-320) for ball and cuboid
// colliders. The broad phase keeps ncollide's DBVTBroadPhase semantics
// (geometrical_world.rs:60): every collider carries a fat AABB (its tight AABB
// loosened by the query limit, then by the 0.01 margin) that is refreshed only
// when the tight box leaves it, and the pair set is every allowed pair whose
// fat AABBs intersect. It is found with a linear BVH (Karras 2012) over
// 64-bit keys (world index | 48-bit Morton code), rebuilt every pass:
//   sync_aabb -> radix sort -> build -> refit -> count -> scan -> write -> narrow.
// Each pair is written by its owner (the collider with the smaller bounding
// radius, ties by slot) so the list is deterministic and the previous step's
// pairs of a collider are found without hashing.
#include "narrow.cuh"
#include "sortscan.cuh"

namespace npgpu_dev {

constexpr int kThreads = 256;
static inline unsigned nblocks(uint32_t n) { return (n + kThreads - 1) / kThreads; }

// Sort keys: dead bit | world index | static bit | 30-bit Morton code of the
// fat-AABB centre on a 1 m grid (10 bits per axis, +-512 m; farther centres
// clamp to the edge cells, which only affects the tree's shape, never the
// pairs). The static bit puts a world's colliders of static bodies after its
// moving ones, so the tree splits each world into a moving and a static
// subtree at its top: a query reaches a large static collider (a ground)
// through one node instead of down the long path its box spans in a mixed
// tree. The dead bit sits just above the highest world bit in use, so that
// the radix sort only looks at 32 + world-bit bits.
constexpr int kMortonBits = 30;
constexpr int kWorldShift = kMortonBits + 1;
__device__ __forceinline__ uint64_t expand10(uint32_t v) {
    uint64_t x = v & 0x3ffu;
    x = (x | (x << 16)) & 0x30000ffull;
    x = (x | (x << 8)) & 0x300f00full;
    x = (x | (x << 4)) & 0x30c30c3ull;
    x = (x | (x << 2)) & 0x9249249ull;
    return x;
}
__device__ __forceinline__ uint32_t quantize(float c) {
    float q = floorf(c) + 512.0f;
    q = q < 0.0f ? 0.0f : (q > 1023.0f ? 1023.0f : q);
    return (uint32_t)q;
}
__device__ __forceinline__ uint32_t key_world(unsigned long long k) { return (uint32_t)(k >> kWorldShift) & 0xffffu; }

__device__ __forceinline__ Shape load_shape(const Colliders& c, uint32_t i) {
    Shape s;
    uint32_t info = c.info[i];
    s.shape = info & 0xfu;
    float4 p = c.params[i];
    s.h = np::mk(p.x, p.y, p.z);
    s.radius = p.x;
    s.pose.t = v3(c.pose_t[i]);
    s.pose.q = q4(c.pose_q[i]);
    return s;
}

// Collider pose, tight AABB (loosened by margin + linear prediction,
// src/object/collider.rs:542-549), fat AABB update and sort key.
__global__ void k_sync_aabb(World w, float bp_margin, int world_bits) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nc_slots) return;
    const Colliders& c = w.c;
    if (!(c.info[i] & CI_ALIVE)) {
        c.keys[i] = 1ull << (kWorldShift + world_bits);
        c.vals[i] = i;
        return;
    }
    uint32_t bi = c.body[i];
    np::Iso bp{v3(w.b.pos_t[bi]), q4(w.b.pos_q[bi])};
    np::Iso wrt{v3(c.wrt_t[i]), q4(c.wrt_q[i])};
    np::Iso pose = np::iso_mul(bp, wrt);
    c.pose_t[i] = f4(pose.t);
    c.pose_q[i] = f4q(pose.q);
    uint32_t shape = c.info[i] & 0xfu;
    float4 prm = c.params[i];
    np::V half;
    if (shape == SHAPE_BALL) {
        half = np::mk(prm.x, prm.x, prm.x);
    } else if (shape == SHAPE_CAPSULE) {
        // The axis's extent along each world axis, loosened by the radius.
        np::M rot = np::qmat(pose.q);
        for (int a = 0; a < 3; ++a) np::setc(half, a, fabsf(rot.m[a][1]) * prm.y + prm.x);
    } else {
        np::M rot = np::qmat(pose.q);
        for (int a = 0; a < 3; ++a) {
            float s = fabsf(rot.m[a][0]) * prm.x + fabsf(rot.m[a][1]) * prm.y + fabsf(rot.m[a][2]) * prm.z;
            np::setc(half, a, s);
        }
    }
    float ql = c.margin[i] + c.lin_pred[i];
    float mn[3], mx[3];
    for (int a = 0; a < 3; ++a) {
        mn[a] = (np::comp(pose.t, a) - np::comp(half, a)) - ql;
        mx[a] = (np::comp(pose.t, a) + np::comp(half, a)) + ql;
    }
    float4 fmn = c.aabb_min[i], fmx = c.aabb_max[i];
    bool inside = fmn.w != 0.0f && fmn.x <= mn[0] && mx[0] <= fmx.x && fmn.y <= mn[1] && mx[1] <= fmx.y &&
                  fmn.z <= mn[2] && mx[2] <= fmx.z;
    if (!inside) {
        fmn = make_float4(mn[0] - bp_margin, mn[1] - bp_margin, mn[2] - bp_margin, 1.0f);
        fmx = make_float4(mx[0] + bp_margin, mx[1] + bp_margin, mx[2] + bp_margin, 0.0f);
        c.aabb_min[i] = fmn;
        c.aabb_max[i] = fmx;
    }
    float cx = 0.5f * (fmn.x + fmx.x), cy = 0.5f * (fmn.y + fmx.y), cz = 0.5f * (fmn.z + fmx.z);
    uint64_t morton = expand10(quantize(cx)) | (expand10(quantize(cy)) << 1) | (expand10(quantize(cz)) << 2);
    uint64_t world = w.b.world[bi] & 0xffffu;
    uint64_t stat = bi_status(w.b.info[bi]) == 1u ? 1ull : 0ull;   // NPGPU_BODY_STATIC
    c.keys[i] = (world << kWorldShift) | (stat << kMortonBits) | morton;
    c.vals[i] = i;
}

__device__ __forceinline__ int lbvh_delta(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll((long long)(a ^ b));
}

// Karras 2012: internal node i of n - 1; leaves are nodes n - 1 .. 2n - 2.
__global__ void k_lbvh_build(World w, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const unsigned long long* k = w.c.keys_sorted;
    int d = (lbvh_delta(k, n, i, i + 1) - lbvh_delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = lbvh_delta(k, n, i, i - d);
    int lmax = 2;
    while (lbvh_delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (lbvh_delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = lbvh_delta(k, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (lbvh_delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + (d < 0 ? d : 0);
    int lo = i < j ? i : j, hi = i < j ? j : i;
    int left = (lo == gamma) ? (n - 1 + gamma) : gamma;
    int right = (hi == gamma + 1) ? (n - 1 + gamma + 1) : (gamma + 1);
    w.c.left[i] = left;
    w.c.right[i] = right;
    w.c.parent[left] = i;
    w.c.parent[right] = i;
    if (i == 0) w.c.parent[0] = -1;
}

__device__ __forceinline__ float4 ld_cg(const float4* p) { return __ldcg(p); }

// Arrival count of a node: release orders this thread's writes of the child
// before the count, acquire orders the second arrival's reads of the sibling
// after it (one ordered atomic instead of a full fence and a plain atomic).
__device__ __forceinline__ int arrive_acq_rel(int* p) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// Bottom-up refit: the second child to arrive computes the parent.
__global__ void k_lbvh_refit(World w, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t ci = w.c.vals_sorted[k];
    int node = n - 1 + k;
    // node_min.w carries the worlds under the node (first << 16 | last; the
    // leaves sort by world first), node_max.w the largest owner rank
    // (bounding radius) of the subtree.
    float4 mn = w.c.aabb_min[ci], mx = w.c.aabb_max[ci];
    uint32_t wk = key_world(w.c.keys_sorted[k]);
    float4 c0 = make_float4(mn.x, mn.y, mn.z, __uint_as_float(wk << 16 | wk));
    float4 c1 = make_float4(mx.x, mx.y, mx.z, w.c.rank[ci]);
    uint32_t cs = ci;   // node_slot: with the largest rank in node_max.w, the owner test's (rank, slot) maximum
    w.c.node_min[node] = c0;
    w.c.node_max[node] = c1;
    w.c.node_slot[node] = cs;
    if (n == 1) return;
    int p = w.c.parent[node];
    for (int guard = 0; p >= 0; ++guard) {
        if (guard > 256) {   // deeper than any tree over 64-bit keys plus 32-bit tie-breaks
            atomicOr(&w.ctl->err, ERRF_PAIR_CAPACITY);
            return;
        }
        if (arrive_acq_rel(&w.c.node_flag[p]) == 0) return;
        // This thread holds its own child's box; only the sibling's is read.
        int l = w.c.left[p], r = w.c.right[p];
        const bool from_left = l == node;
        const int sib = from_left ? r : l;
        const float4 s0 = ld_cg(&w.c.node_min[sib]), s1 = ld_cg(&w.c.node_max[sib]);
        const uint32_t ss = __ldcg(&w.c.node_slot[sib]);
        const float4 a0 = from_left ? c0 : s0, a1 = from_left ? c1 : s1;
        const float4 b0 = from_left ? s0 : c0, b1 = from_left ? s1 : c1;
        const uint32_t as = from_left ? cs : ss, bs = from_left ? ss : cs;
        cs = a1.w > b1.w ? as : (b1.w > a1.w ? bs : (as > bs ? as : bs));
        uint32_t wr = (__float_as_uint(a0.w) & 0xffff0000u) | (__float_as_uint(b0.w) & 0xffffu);
        c0 = make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), __uint_as_float(wr));
        c1 = make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), fmaxf(a1.w, b1.w));
        w.c.node_min[p] = c0;
        w.c.node_max[p] = c1;
        w.c.node_slot[p] = cs;
        // The traversal's copy: both children's boxes and references in one
        // 80-byte record, a leaf child referenced by its collider (top bit set).
        float4* wd = w.c.wide + 5 * (size_t)p;
        wd[0] = a0;
        wd[1] = a1;
        wd[2] = b0;
        wd[3] = b1;
        uint32_t lref = l >= n - 1 ? (0x80000000u | w.c.vals_sorted[l - (n - 1)]) : (uint32_t)l;
        uint32_t rref = r >= n - 1 ? (0x80000000u | w.c.vals_sorted[r - (n - 1)]) : (uint32_t)r;
        wd[4] = make_float4(__uint_as_float(lref), __uint_as_float(rref), __uint_as_float(as), __uint_as_float(bs));
        node = p;
        p = w.c.parent[p];
    }
}

// The owner of a pair is the collider with the smaller bounding radius (ties: smaller slot).
__device__ __forceinline__ bool owns(const Colliders& c, uint32_t a, uint32_t b) {
    float ra = c.rank[a], rb = c.rank[b];
    return ra < rb || (ra == rb && a < b);
}

// DefaultCollisionFilter (geometrical_world.rs:926-970): not on the same body,
// at least one body with dofs; plus: both in the same world of a batch.
__device__ __forceinline__ bool pair_allowed(const World& w, uint32_t a, uint32_t b) {
    uint32_t ba = w.c.body[a], bb = w.c.body[b];
    if (ba == bb) return false;
    if (w.b.world[ba] != w.b.world[bb]) return false;
    return bi_status(w.b.info[ba]) == 2u || bi_status(w.b.info[bb]) == 2u;
}

__device__ __forceinline__ bool overlap(float4 amin, float4 amax, float4 bmin, float4 bmax) {
    return amin.x <= bmax.x && bmin.x <= amax.x && amin.y <= bmax.y && bmin.y <= amax.y && amin.z <= bmax.z &&
           bmin.z <= amax.z;
}

// Traverses the tree with leaf k's fat AABB. WRITE = false counts the pairs
// leaf k owns and keeps up to kLeafCap partners in leaf_tmp; WRITE = true
// stores the pairs at the leaf's offset, from leaf_tmp when they fit there,
// by traversing again otherwise.
template <bool WRITE>
__global__ void k_bp_traverse(World w, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const Colliders& c = w.c;
    uint32_t a = c.vals_sorted[k];
    uint32_t count = 0, base = 0;
    if (WRITE) {
        base = c.leaf_offset[k];
        uint32_t kept = c.leaf_count[k];
        if (kept <= (uint32_t)kLeafCap) {
            for (uint32_t i = 0; i < kept; ++i) {
                uint32_t b = c.leaf_tmp[(size_t)k * kLeafCap + i];
                uint32_t slot = base + i;
                if (slot < w.cap_pairs) w.cur.pair[slot] = make_uint2(a < b ? a : b, a < b ? b : a);
            }
            uint32_t stored = base >= w.cap_pairs ? 0u : (kept < w.cap_pairs - base ? kept : w.cap_pairs - base);
            w.cur.owner_start[a] = base;
            w.cur.owner_count[a] = stored;
            return;
        }
    }
    float4 amin = c.aabb_min[a], amax = c.aabb_max[a];
    float ra = c.rank[a];
    const uint32_t qw = key_world(c.keys_sorted[k]);
    // A subtree is entered when it holds the query's world (batched worlds
    // share space), a collider the query may own (a larger bounding radius
    // somewhere below) and an AABB overlapping the query's. An internal node's
    // record carries both children's boxes, so a visited node costs one
    // memory round trip, and leaf children are tested without visiting them.
    // The query owns a collider of the subtree only if the subtree's largest
    // (rank, slot) pair is above its own: a larger rank, or the same rank
    // and a larger slot (owns()).
    auto enter = [&](float4 nmin, float4 nmax, uint32_t nslot) {
        uint32_t nw = __float_as_uint(nmin.w);
        const bool may_own = ra < nmax.w || (ra == nmax.w && a < nslot);
        return qw >= (nw >> 16) && qw <= (nw & 0xffffu) && may_own && overlap(amin, amax, nmin, nmax);
    };
    auto emit = [&](uint32_t b, float rb) {
        // owns(): the smaller bounding radius owns the pair, ties by slot.
        const bool own = ra < rb || (ra == rb && a < b);
        if (b != a && own && pair_allowed(w, a, b)) {
            if (WRITE) {
                uint32_t slot = base + count;
                if (slot < w.cap_pairs) w.cur.pair[slot] = make_uint2(a < b ? a : b, a < b ? b : a);
            } else if (count < (uint32_t)kLeafCap) {
                c.leaf_tmp[(size_t)k * kLeafCap + count] = b;
            }
            ++count;
        }
    };
    if (n >= 2 && enter(c.node_min[0], c.node_max[0], c.node_slot[0])) {
        int stack[64];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const float4* wd = c.wide + 5 * (size_t)stack[--sp];
            const float4 lmin = wd[0], lmax = wd[1], rmin = wd[2], rmax = wd[3], refs = wd[4];
            const uint32_t lref = __float_as_uint(refs.x), rref = __float_as_uint(refs.y);
            const bool el = enter(lmin, lmax, __float_as_uint(refs.z)), er = enter(rmin, rmax, __float_as_uint(refs.w));
            if (el && (lref & 0x80000000u)) emit(lref & 0x7fffffffu, lmax.w);
            if (er && (rref & 0x80000000u)) emit(rref & 0x7fffffffu, rmax.w);
            const bool pl = el && !(lref & 0x80000000u), pr = er && !(rref & 0x80000000u);
            if (sp + (int)pl + (int)pr > 64) {
                atomicOr(&w.ctl->err, ERRF_PAIR_CAPACITY);
                break;
            }
            if (pr) stack[sp++] = (int)rref;
            if (pl) stack[sp++] = (int)lref;
        }
    }
    if (!WRITE) {
        c.leaf_count[k] = count;
    } else {
        // Only the pairs that fit in the buffer are visible to the next pass.
        uint32_t stored = base >= w.cap_pairs ? 0u : (count < w.cap_pairs - base ? count : w.cap_pairs - base);
        w.cur.owner_start[a] = base;
        w.cur.owner_count[a] = stored;
    }
}

__global__ void k_bp_total(World w, int n) {
    uint32_t total = 0;
    if (n > 0) total = w.c.leaf_offset[n - 1] + w.c.leaf_count[n - 1];
    if (total > w.cap_pairs) {
        atomicOr(&w.ctl->err, ERRF_PAIR_CAPACITY);
        total = w.cap_pairs;
    }
    w.ctl->npairs = total;
    w.ctl->ncontacts = 0;
    w.ctl->nmanifolds = 0;
    w.ctl->max_pen_bits = 0;
}

__device__ __forceinline__ unsigned long long order_bits(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

// Per-thread totals of the narrow phase, folded into the step's counters once
// per block: same-address atomics from every pair serialise in L2.
struct NarrowTotals {
    uint32_t contacts = 0, manifolds = 0;
    unsigned long long pen_bits = 0;   // order_bits of the deepest penetration
};

// ContactEvent::Started / Stopped (ncollide3d's narrow phase, read through
// GeometricalWorld::contact_events, src/world/geometrical_world.rs:373-376):
// a pair whose manifold gains its first contact, or loses its last, in a
// collision-detection pass. Events accumulate over the step's passes (the
// body-start kernel clears the count, as MechanicalWorld::step clears them
// before its first pass, mechanical_world.rs:250).
__device__ __forceinline__ void emit_event(const World& w, uint32_t c1, uint32_t c2, bool stopped) {
    const uint32_t at = atomicAdd(&w.ctl->nevents, 1u);
    if (at < w.events_cap) w.events[at] = make_uint2(c1, c2 | (stopped ? 0x80000000u : 0u));
}
// ProximityEvent (ncollide3d, read through GeometricalWorld::proximity_events,
// geometrical_world.rs:378-381): a pair with a sensor whose proximity changed.
// Shares the event buffer: bit 30 marks it, bits 26-27 and 28-29 hold the
// previous and new PROX_* (collider slots stay below 2^26).
__device__ __forceinline__ void emit_proximity(const World& w, uint32_t c1, uint32_t c2, uint32_t prev, uint32_t now) {
    const uint32_t at = atomicAdd(&w.ctl->nevents, 1u);
    if (at < w.events_cap) w.events[at] = make_uint2(c1, c2 | 0x40000000u | (prev << 26) | (now << 28));
}

// One-shot manifold of pair p, keeping the impulses cached under the same
// feature key in the pair's previous manifold.
__device__ __noinline__ void narrow_pair(const World& w, uint32_t p, NarrowTotals& tot) {
    uint2 pr = w.cur.pair[p];
    uint32_t c1 = pr.x, c2 = pr.y;
    const Colliders& c = w.c;
    Shape a = load_shape(c, c1), b = load_shape(c, c2);
    float m1 = c.margin[c1], m2 = c.margin[c2];
    float prediction = (m1 + c.lin_pred[c1]) + (m2 + c.lin_pred[c2]);
    CandList out;
    int keep[kMaxContacts];
    const int nk = shape_pair_contacts(a, b, prediction, out, keep);
    // Previous manifold of this pair: among the pairs its owner wrote last pass.
    uint32_t owner = owns(c, c1, c2) ? c1 : c2;
    uint32_t qs = w.prev.owner_start[owner], qn = w.prev.owner_count[owner];
    int prev = -1;
    for (uint32_t q = 0; q < qn; ++q) {
        uint2 o = w.prev.pair[qs + q];
        if (o.x == c1 && o.y == c2) {
            prev = int(qs + q);
            break;
        }
    }
    if ((c.info[c1] | c.info[c2]) & CI_SENSOR) {
        // A proximity pair (ProximityDetector): Intersecting when the shapes
        // touch or overlap, WithinMargin when the contact generator finds
        // them within the query limits, Disjoint otherwise. It makes no
        // contacts.
        uint32_t st = PROX_DISJOINT;
        for (int k = 0; k < nk && k < kMaxContacts; ++k) {
            const float d = out.c[keep[k]].g.depth;
            if (d >= 0.0f) st = PROX_INTERSECTING;
            else if (st == PROX_DISJOINT) st = PROX_WITHIN_MARGIN;
        }
        const uint32_t was = prev >= 0 ? (uint32_t)w.prev.prox[prev] : PROX_DISJOINT;
        w.cur.ncont[p] = 0;
        w.cur.prox[p] = (uint8_t)st;
        if (w.events != nullptr && st != was) emit_proximity(w, c1, c2, was, st);
        return;
    }
    w.cur.prox[p] = (uint8_t)PROX_DISJOINT;
    uint32_t pkeys[kMaxContacts];
    int pn = 0;
    if (prev >= 0) {
        pn = w.prev.ncont[prev];
        for (int k = 0; k < pn; ++k) pkeys[k] = w.prev.key[prev * kMaxContacts + k];
    }
    np::Q bq = q4(w.b.pos_q[c.body[c1]]);
    int nc = nk > kMaxContacts ? kMaxContacts : nk;
    // The deepest contact, in f32: the penetration depth + m1 + m2 (in FP64)
    // rises with the depth, and the margins are the manifold's.
    float maxdepth = -INFINITY;
    for (int k = 0; k < nc; ++k) {
        const Cand& cd = out.c[keep[k]];
        uint32_t key = uint32_t(cd.f1 * 26 + cd.f2);
        float4 imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int j = 0; j < pn; ++j)
            if (pkeys[j] == key) {
                imp = w.prev.imp[prev * kMaxContacts + j];
                imp.w = 1.0f;   // found in the impulse cache
                break;
            }
        uint32_t slot = p * kMaxContacts + k;
        w.cur.key[slot] = key;
        w.cur.w1[slot] = f4(cd.g.w1, cd.g.depth);
        w.cur.w2[slot] = f4(cd.g.w2);
        w.cur.n[slot] = f4(cd.g.n);
        w.cur.imp[slot] = imp;
        w.cur.nl[slot] = f4(np::qrot_inv(bq, cd.g.n));
        maxdepth = cd.g.depth > maxdepth ? cd.g.depth : maxdepth;
    }
    w.cur.ncont[p] = (uint8_t)nc;
    if (w.events != nullptr && (nc > 0) != (pn > 0)) emit_event(w, c1, c2, nc == 0);
    if (nc > 0) {
        tot.contacts += (uint32_t)nc;
        tot.manifolds += 1u;
        const double maxpen = maxdepth == -INFINITY ? -1e300 : (double)maxdepth + (double)m1 + (double)m2;
        const unsigned long long pb = order_bits(maxpen);
        tot.pen_bits = pb > tot.pen_bits ? pb : tot.pen_bits;
    }
}

__global__ void k_narrow(World w) {
    uint32_t npairs = w.ctl->npairs;
    NarrowTotals tot;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x)
        narrow_pair(w, p, tot);
    // Block totals: warp shuffles, then one warp over the per-warp partials.
    __shared__ NarrowTotals part[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        tot.contacts += __shfl_xor_sync(0xffffffffu, tot.contacts, o);
        tot.manifolds += __shfl_xor_sync(0xffffffffu, tot.manifolds, o);
        const unsigned long long pb = __shfl_xor_sync(0xffffffffu, tot.pen_bits, o);
        tot.pen_bits = pb > tot.pen_bits ? pb : tot.pen_bits;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) part[warp] = tot;
    __syncthreads();
    if (warp == 0) {
        tot = lane < (int)(blockDim.x >> 5) ? part[lane] : NarrowTotals{};
        for (int o = 16; o > 0; o >>= 1) {
            tot.contacts += __shfl_xor_sync(0xffffffffu, tot.contacts, o);
            tot.manifolds += __shfl_xor_sync(0xffffffffu, tot.manifolds, o);
            const unsigned long long pb = __shfl_xor_sync(0xffffffffu, tot.pen_bits, o);
            tot.pen_bits = pb > tot.pen_bits ? pb : tot.pen_bits;
        }
        if (lane == 0 && tot.manifolds > 0) {
            atomicAdd(&w.ctl->ncontacts, tot.contacts);
            atomicAdd(&w.ctl->nmanifolds, tot.manifolds);
            atomicMax(&w.ctl->max_pen_bits, tot.pen_bits);
        }
    }
}

size_t sort_temp_bytes(uint32_t n) { return radix_sort_temp_bytes(n); }
size_t scan_temp_bytes(uint32_t n) { return exclusive_scan_temp_bytes(n); }

cudaError_t launch_sync_aabb(const World& w, const StepParams& p, cudaStream_t st) {
    if (w.nc_slots == 0) return cudaSuccess;
    k_sync_aabb<<<nblocks(w.nc_slots), kThreads, 0, st>>>(w, p.broad_phase_margin, (int)w.world_bits);
    return cudaGetLastError();
}

cudaError_t launch_sort(const World& w, void* temp, size_t temp_bytes, cudaStream_t st) {
    if (w.nc_slots == 0) return cudaSuccess;
    return radix_sort_pairs(temp, temp_bytes, w.c.keys, w.c.keys_sorted, w.c.vals, w.c.vals_sorted, w.nc_slots,
                            kWorldShift + (int)w.world_bits + 1, st);
}

cudaError_t launch_lbvh(const World& w, cudaStream_t st) {
    int n = (int)w.nc_alive;
    if (n >= 2) {
        cudaMemsetAsync(w.c.node_flag, 0, sizeof(int) * (size_t)(n - 1), st);
        k_lbvh_build<<<nblocks(n - 1), kThreads, 0, st>>>(w, n);
    }
    if (n >= 1) k_lbvh_refit<<<nblocks(n), kThreads, 0, st>>>(w, n);
    return cudaGetLastError();
}

cudaError_t launch_pairs(const World& w, void* temp, size_t temp_bytes, cudaStream_t st) {
    int n = (int)w.nc_alive;
    cudaMemsetAsync(w.cur.owner_count, 0, sizeof(uint32_t) * w.nc_slots, st);
    if (n >= 1) {
        k_bp_traverse<false><<<nblocks(n), kThreads, 0, st>>>(w, n);
        cudaError_t e = exclusive_scan(temp, temp_bytes, w.c.leaf_count, w.c.leaf_offset, (uint32_t)n, st);
        if (e != cudaSuccess) return e;
        k_bp_traverse<true><<<nblocks(n), kThreads, 0, st>>>(w, n);
    }
    k_bp_total<<<1, 1, 0, st>>>(w, n);
    return cudaGetLastError();
}

// Stopped events of the pairs that had contacts in the previous pass and are
// no longer broad-phase pairs, and proximity events to Disjoint of the
// sensor pairs that were not Disjoint (the pairs present in both passes are handled
// by the narrow phase). A pair's owner is the same collider in both passes,
// so it is looked up among its owner's pairs of this pass.
__global__ void k_events_vanished(World w) {
    for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < w.nc_slots; a += gridDim.x * blockDim.x) {
        const uint32_t qs = w.prev.owner_start[a], qn = w.prev.owner_count[a];
        if (qn == 0) continue;
        const uint32_t cs = w.cur.owner_start[a], cn = w.cur.owner_count[a];
        for (uint32_t q = 0; q < qn; ++q) {
            const uint2 o = w.prev.pair[qs + q];
            const uint32_t was = w.prev.prox[qs + q];
            if (o.x == 0xffffffffu || (w.prev.ncont[qs + q] == 0 && was == PROX_DISJOINT)) continue;
            bool found = false;
            for (uint32_t r = 0; r < cn && !found; ++r) {
                const uint2 x = w.cur.pair[cs + r];
                found = x.x == o.x && x.y == o.y;
            }
            if (found) continue;
            if (was != PROX_DISJOINT) emit_proximity(w, o.x, o.y, was, PROX_DISJOINT);
            else emit_event(w, o.x, o.y, true);
        }
    }
}

cudaError_t launch_events(const World& w, cudaStream_t st) {
    if (w.events == nullptr || w.nc_slots == 0) return cudaSuccess;
    unsigned blocks = nblocks(w.nc_slots);
    if (blocks > 152u * 16u) blocks = 152u * 16u;
    k_events_vanished<<<blocks, kThreads, 0, st>>>(w);
    return cudaGetLastError();
}

cudaError_t launch_narrow(const World& w, cudaStream_t st) {
    // The pair count lives on the device: a grid-stride launch sized for the
    // capacity, capped at 16 blocks per SM of a 152-SM part.
    uint32_t blocks = nblocks(w.cap_pairs);
    if (blocks == 0) return cudaSuccess;
    if (blocks > 152u * 16u) blocks = 152u * 16u;
    k_narrow<<<blocks, kThreads, 0, st>>>(w);
    return cudaGetLastError();
}

}  // namespace npgpu_dev
