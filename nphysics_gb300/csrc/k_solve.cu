// k_solve.cu -- the solver half of MechanicalWorld::step on the device.
//
//   activation   ActivationManager::update (src/detection/activation_manager.rs:61-201):
//                RWA energies, islands by lock-free union-find, sleep / wake
//   collection   manifolds handed to the solver (src/world/mechanical_world.rs:287-300)
//   colouring    greedy first-fit colouring of the manifolds in decreasing hash
//                priority (the Jones-Plassmann first-fit colouring); manifolds of
//                one colour share no dynamic body
//   assembly     SignoriniCoulombPyramidModel::constraints
//                (src/solver/signorini_coulomb_pyramid_model.rs:56-224,
//                signorini_model.rs:37-138, helper.rs:53-135, rigid_body.rs:672-722)
//   SOR-Prox     SORProx::solve (src/solver/sor_prox.rs:48-179): warm start, then per
//                iteration every friction row, then every normal row
//   residual     FP64 complementarity residual
//   cache        cache_impulses (signorini_coulomb_pyramid_model.rs:226-261)
//   integrate    update_velocities_and_integrate (moreau_jean_solver.rs:328-347)
//   position     NonlinearSORProx::solve (src/solver/nonlinear_sor_prox.rs:17-309)
//   post         kinematic integration, update_dynamics, clear_forces (mechanical_world.rs:328-367)
//
// Gauss-Seidel order. The sequential order the GPU reproduces is: manifolds
// sorted by colour, each manifold's contacts in order. Instead of a grid
// barrier between colours, every dynamic body carries a version counter: the
// task (sweep s, manifold m) may touch body b once b's counter equals
// s * k_b + r, where k_b is the number of b's solver manifolds and r the
// number of them with a smaller colour; it then publishes b's new state and
// the counter r + 1 with release semantics. Each body therefore sees its
// updates in exactly the sequential order, and the critical path is a chain of
// dependent manifolds rather than a barrier per colour. The colouring uses the
// same scheme over priorities. Threads poll their tasks without blocking, so
// any assignment of manifolds to resident threads makes progress.
#include <cfloat>

#include <cooperative_groups.h>

#include "ccd.cuh"
#include "mlp.cuh"
#include "narrow.cuh"
#include "sortscan.cuh"

namespace npgpu_dev {

namespace cg = cooperative_groups;

// This file is compiled twice. With NPGPU_EXCHANGE_TU=1 (and -dlcm=cg: global
// loads bypass L1, so none is served stale) it holds the kernels whose blocks
// exchange data through global memory within one launch: the islands'
// union-find, the dataflow colouring, the one-grid velocity and position
// solvers and the thread-block-cluster solvers. With NPGPU_EXCHANGE_TU=0 it
// holds the other kernels, whose global reads may be cached in L1, and the
// launchers, which reach the first group through exchange_kernel().
#ifndef NPGPU_EXCHANGE_TU
#define NPGPU_EXCHANGE_TU 0
#endif
// The solver kernels come in two instantiations: with joint rows (JOINTS,
// launched when the world has joint slots) and without, so that contact-only
// worlds run code with no joint branch or call in it.
enum ExchangeKernel { XK_COLOUR, XK_VELOCITY, XK_POSITION, XK_CLUSTER_VELOCITY, XK_CLUSTER_POSITION };
const void* exchange_kernel(ExchangeKernel k, bool joints = false);
cudaError_t launch_activation(const World& w, const StepParams& p, unsigned nbb, unsigned npb, cudaStream_t st);

constexpr int kItemThreads = 256;
constexpr int kCoopThreads = 256;
constexpr int kMaxPerThread = 16;
constexpr unsigned long long kWaitLimitNs = 1000000000ull;   // a bounded wait gives up after one second

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_release_add(uint32_t* p, uint32_t v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Flagged Δv of the dataflow velocity solver: per body 8 words of 64 bits
// (6 used), each = update count << 32 | float bits. A 64-bit aligned word is
// written and read as a whole, so a reader that finds the expected count in
// all six words holds the Δv of exactly that update, with no fence on either
// side: the count is the flag.
__device__ __forceinline__ bool poll_dvf(const unsigned long long* dvf, int b, uint32_t t, float* out) {
    if (b < 0) return true;
    const unsigned long long* p = dvf + 8 * (size_t)b;
    unsigned long long w0, w1, w2, w3, w4, w5;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(w0), "=l"(w1) : "l"(p) : "memory");
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(w2), "=l"(w3) : "l"(p + 2) : "memory");
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(w4), "=l"(w5) : "l"(p + 4) : "memory");
    const unsigned long long w[6] = {w0, w1, w2, w3, w4, w5};
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        ok = ok && (uint32_t)(w[k] >> 32) == t;
        out[k] = __uint_as_float((uint32_t)w[k]);
    }
    return ok;
}
// The Δv part of a body's flagged words (after a grid-wide sync).
__device__ __forceinline__ void load_dvf(const unsigned long long* dvf, int b, float* out) {
    if (b < 0) return;
#pragma unroll
    for (int k = 0; k < 6; ++k) out[k] = __uint_as_float((uint32_t)__ldcg(dvf + 8 * (size_t)b + k));
}
__device__ __forceinline__ void publish_dvf(unsigned long long* dvf, int b, uint32_t t, const float* v) {
    if (b < 0) return;
    unsigned long long* p = dvf + 8 * (size_t)b;
    const unsigned long long hi = (unsigned long long)t << 32;
    unsigned long long w[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = hi | __float_as_uint(v[k]);
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(w[0]), "l"(w[1]) : "memory");
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p + 2), "l"(w[2]), "l"(w[3]) : "memory");
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p + 4), "l"(w[4]), "l"(w[5]) : "memory");
}

__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void ld_relaxed_v2(const unsigned long long* p, unsigned long long& a,
                                              unsigned long long& b) {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}
__device__ __forceinline__ void st_relaxed_v2(unsigned long long* p, unsigned long long a, unsigned long long b) {
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}
__device__ __forceinline__ bool err_set(const Control* ctl, uint32_t bits) {
    return (ld_acquire(&ctl->err) & bits) != 0;
}

// Grid-wide barrier over a monotonic arrival counter (zeroed before the launch).
// Returns false when the wait gave up (ERRF_TIMEOUT); the caller then leaves.
__device__ __forceinline__ bool grid_sync(Control* ctl, uint32_t& epoch) {
    __syncthreads();
    ++epoch;
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        uint32_t target = epoch * gridDim.x;
        red_release_add(&ctl->barrier_count, 1u);
        if (ld_acquire(&ctl->barrier_count) < target) {
            unsigned long long t0 = global_ns();
            unsigned spins = 0;
            while (ld_acquire(&ctl->barrier_count) < target) {
                if ((++spins & 63u) == 0u) {
                    if (err_set(ctl, ERRF_TIMEOUT) || global_ns() - t0 > kWaitLimitNs) {
                        atomicOr(&ctl->err, ERRF_TIMEOUT);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Backs off while a whole warp waits: 32 ns doubling up to 256 ns, so that
// waiting warps do not crowd the L2 that the running ones need. Called by all
// 32 lanes together; the decision is warp-uniform. The time limit and the
// error word are looked at every 64th wait. Returns false on timeout.
__device__ __forceinline__ bool warp_wait_backoff(const Control* ctl, unsigned long long& t0, unsigned& backoff) {
    if (t0 == 0) t0 = global_ns();
    __nanosleep(backoff & 0xffffu);
    unsigned waits = (backoff >> 16) + 1u;
    unsigned ns = backoff & 0xffffu;
    backoff = ((waits & 0xffffu) << 16) | (ns < 256u ? ns * 2u : 256u);
    if ((waits & 63u) != 0u) return true;
    bool give_up = err_set(ctl, ERRF_TIMEOUT) || global_ns() - t0 > kWaitLimitNs;
    if (__any_sync(0xffffffffu, give_up)) {
        if ((threadIdx.x & 31u) == 0u) atomicOr((uint32_t*)&ctl->err, ERRF_TIMEOUT);
        return false;
    }
    return true;
}

#define GRID_FOR(i, n) for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

__device__ __forceinline__ uint32_t pair_hash22(uint32_t c1, uint32_t c2) {
    uint32_t h = c1 * 0x9E3779B1u ^ (c2 + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h >> 10;
}
// Jones-Plassmann priority of a manifold, unique per collider pair: a hash of
// the colliders' world-local slots (l1, l2), ties broken by the slots. Two
// manifolds are compared only when they share a body, hence a world, so a
// world's colouring does not change when its slots are shifted together.
__device__ __forceinline__ unsigned long long pair_priority(uint32_t l1, uint32_t l2, uint32_t c1, uint32_t c2) {
    return ((unsigned long long)pair_hash22(l1, l2) << 42) | ((unsigned long long)c1 << 21) | (unsigned long long)c2;
}

// Lock-free union-find over body slots (the larger root is linked under the smaller).
__device__ __forceinline__ uint32_t uf_find(uint32_t* parent, uint32_t x) {
    uint32_t p = ((volatile uint32_t*)parent)[x];
    int guard = 0;
    while (p != x && guard++ < 4096) {
        uint32_t gp = ((volatile uint32_t*)parent)[p];
        if (gp != p) parent[x] = gp;   // path halving; parents only decrease
        x = p;
        p = gp;
    }
    return x;
}
__device__ __forceinline__ void uf_union(uint32_t* parent, uint32_t a, uint32_t b, uint32_t* err) {
    for (int guard = 0; guard < 4096; ++guard) {
        uint32_t ra = uf_find(parent, a), rb = uf_find(parent, b);
        if (ra == rb) return;
        uint32_t lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
        if (atomicCAS(&parent[hi], hi, lo) == hi) return;
    }
    atomicOr(err, ERRF_UNION_FIND);
}

__device__ __forceinline__ float combine(float a, uint32_t ma, float b, uint32_t mb) {
    // MaterialCombineMode::combine (src/material/material.rs:71-86).
    if (ma == 3u || mb == 3u) return (a < b) ? b : a;
    if (ma == 2u || mb == 2u) return a * b;
    if (ma == 1u || mb == 1u) return (b < a) ? b : a;
    return (a + b) * 0.5f;
}

struct BodyView {
    np::V com, lin, ang, acc_lin, acc_ang;
    float inv_mass;
    np::M inv_I;
    uint32_t info;
};

__device__ __forceinline__ BodyView load_view(const Bodies& b, uint32_t i) {
    BodyView v;
    v.com = v3(b.com[i]);
    v.lin = v3(b.lin[i]);
    v.ang = v3(b.ang[i]);
    v.acc_lin = v3(b.acc_lin[i]);
    v.acc_ang = v3(b.acc_ang[i]);
    v.inv_mass = b.inv_mass[i];
    v.inv_I = load_m9(b.inv_I + 9 * i);
    v.info = b.info[i];
    return v;
}

// RigidBody::fill_constraint_geometry for one side of one row, given the
// side's unit force f (ForceDirection::at_point, helper.rs:24-33).
__device__ __forceinline__ void fill_force_side(const BodyView& b, const float* f, float* J, float* WJ, float& inv_r,
                                                float& rhs, bool with_ext, float dt) {
    uint32_t st = bi_status(b.info);
    float mf[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) mf[k] = f[k] * body_mask(b.info, k);
    float vel[6] = {b.lin.x, b.lin.y, b.lin.z, b.ang.x, b.ang.y, b.ang.z};
    if (st == 3u) {
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < 6; ++k) s = s + f[k] * vel[k];
        rhs = rhs + s;
    } else if (st == 2u) {
#pragma unroll
        for (int k = 0; k < 6; ++k) J[k] = mf[k];
        np::V ml = np::mk(mf[0], mf[1], mf[2]), ma = np::mk(mf[3], mf[4], mf[5]);
        np::V wl = np::mul(ml, b.inv_mass);
        np::V wa = np::mv(b.inv_I, ma);
        WJ[0] = wl.x; WJ[1] = wl.y; WJ[2] = wl.z; WJ[3] = wa.x; WJ[4] = wa.y; WJ[5] = wa.z;
        inv_r = inv_r + (b.inv_mass + np::dot(ma, wa));
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < 6; ++k) s = s + f[k] * vel[k];
        rhs = rhs + s;
        if (with_ext) {
            float ext[6] = {b.acc_lin.x * dt, b.acc_lin.y * dt, b.acc_lin.z * dt,
                            b.acc_ang.x * dt, b.acc_ang.y * dt, b.acc_ang.z * dt};
            float e = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; ++k) e = e + mf[k] * ext[k];
            rhs = rhs + e;
        }
    }
}

// A linear force along dir at point: Force::linear_at_point.
__device__ __forceinline__ void fill_row_side(const BodyView& b, np::V point, np::V dir, float* J, float* WJ, float& inv_r,
                                              float& rhs, bool with_ext, float dt) {
    np::V pos = np::sub(point, b.com);
    np::V fa = np::cross(pos, dir);
    const float f[6] = {dir.x, dir.y, dir.z, fa.x, fa.y, fa.z};
    fill_force_side(b, f, J, WJ, inv_r, rhs, with_ext, dt);
}

// A torque about axis: Force::torque_from_vector.
__device__ __forceinline__ void fill_torque_side(const BodyView& b, np::V axis, float* J, float* WJ, float& inv_r,
                                                 float& rhs, bool with_ext, float dt) {
    const float f[6] = {0.0f, 0.0f, 0.0f, axis.x, axis.y, axis.z};
    fill_force_side(b, f, J, WJ, inv_r, rhs, with_ext, dt);
}

// helper::constraint_pair_geometry for one row; writes J1 J2 WJ1 WJ2 r rhs.
__device__ __forceinline__ void make_row(float* row, const BodyView& b1, const BodyView& b2, np::V c1, np::V c2, np::V dir,
                                         float dt) {
#pragma unroll
    for (int k = 0; k < kRowFloats; ++k) row[k] = 0.0f;
    float inv_r = 0.0f, rhs = 0.0f;
    fill_row_side(b1, c1, dir, row + RF_J1, row + RF_WJ1, inv_r, rhs, true, dt);
    fill_row_side(b2, c2, np::neg(dir), row + RF_J2, row + RF_WJ2, inv_r, rhs, true, dt);
    row[RF_R] = (inv_r != 0.0f) ? 1.0f / inv_r : 1.0f;
    row[RF_RHS] = rhs;
}

// helper::constraint_pair_geometry for a torque row (ForceDirection::Angular
// about axis on body 1, about -axis on body 2).
__device__ __forceinline__ void make_row_angular(float* row, const BodyView& b1, const BodyView& b2, np::V axis, float dt) {
#pragma unroll
    for (int k = 0; k < kRowFloats; ++k) row[k] = 0.0f;
    float inv_r = 0.0f, rhs = 0.0f;
    fill_torque_side(b1, axis, row + RF_J1, row + RF_WJ1, inv_r, rhs, true, dt);
    fill_torque_side(b2, np::neg(axis), row + RF_J2, row + RF_WJ2, inv_r, rhs, true, dt);
    row[RF_R] = (inv_r != 0.0f) ? 1.0f / inv_r : 1.0f;
    row[RF_RHS] = rhs;
}

// The canonical basis vector e_r (helper.rs:247-296, 502-551).
__device__ __forceinline__ np::V basis_axis(int r) {
    return np::mk(r == 0 ? 1.0f : 0.0f, r == 1 ? 1.0f : 0.0f, r == 2 ? 1.0f : 0.0f);
}

// Unit::try_new_and_get(v, eps): v / |v| when |v|^2 > eps^2.
__device__ __forceinline__ bool unit_try(np::V v, float eps, np::V& u, float& n) {
    const float sq = np::dot(v, v);
    if (!(sq > eps * eps)) return false;
    n = sqrtf(sq);
    u = np::divs(v, n);
    return true;
}

// nalgebra Vector3::orthonormal_subspace_basis of one vector.
__device__ __forceinline__ void tangent_basis(np::V n, np::V& t1, np::V& t2) {
    np::V a;
    if (fabsf(n.x) > fabsf(n.y)) a = np::mk(n.z, 0.0f, -n.x);
    else a = np::mk(0.0f, -n.z, n.y);
    t1 = np::divs(a, np::norm(a));
    np::V b = np::cross(n, a);
    t2 = np::divs(b, np::norm(b));
}

struct DV {
    float a[6], b[6];
};

// Inverse augmented mass of a dynamic body as the solver reads it: three
// float4 per body, (inv_I row k, inv_mass in the first .w).
struct SB {
    np::M I;
    float im;
};
__device__ __forceinline__ SB load_sb(const float4* sb, int i) {
    SB s;
    float4 a = sb[3 * i], b = sb[3 * i + 1], c = sb[3 * i + 2];
    s.I.m[0][0] = a.x; s.I.m[0][1] = a.y; s.I.m[0][2] = a.z;
    s.I.m[1][0] = b.x; s.I.m[1][1] = b.y; s.I.m[1][2] = b.z;
    s.I.m[2][0] = c.x; s.I.m[2][1] = c.y; s.I.m[2][2] = c.z;
    s.im = a.w;
    return s;
}

// The Jacobians of one row, J_b = mask_b . [d_b, pos_b x d_b] and
// WJ_b = (inv_mass_b J_b.lin, inv_I_b J_b.ang) with d_1 = dir, d_2 = -dir
// (helper.rs:53-135, rigid_body.rs:672-722). The solver rebuilds them from the
// row direction and the lever arms with the same operations as assembly, so
// they carry the same bits as rows stored in full; they are formed where they
// are used rather than kept in registers.
__device__ __forceinline__ void side_j(np::V pos, np::V dir, uint32_t m6, float* J) {
    np::V fa = np::cross(pos, dir);
    float f[6] = {dir.x, dir.y, dir.z, fa.x, fa.y, fa.z};
#pragma unroll
    for (int k = 0; k < 6; ++k) J[k] = f[k] * (((m6 >> k) & 1u) ? 1.0f : 0.0f);
}

__device__ __forceinline__ float side_dot_j(const float* J, const float* dv) {
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; ++k) s = s + J[k] * dv[k];
    return s;
}

__device__ __forceinline__ void side_axpy_j(const float* J, const SB& sb, float a, float* dv) {
    np::V wl = np::mul(np::mk(J[0], J[1], J[2]), sb.im);
    np::V wa = np::mv(sb.I, np::mk(J[3], J[4], J[5]));
    float W[6] = {wl.x, wl.y, wl.z, wa.x, wa.y, wa.z};
#pragma unroll
    for (int k = 0; k < 6; ++k) dv[k] = a * W[k] + dv[k];
}

__device__ __forceinline__ float side_dot(np::V pos, np::V dir, uint32_t m6, const float* dv) {
    float J[6];
    side_j(pos, dir, m6, J);
    return side_dot_j(J, dv);
}

__device__ __forceinline__ void side_axpy(np::V pos, np::V dir, uint32_t m6, const SB& sb, float a, float* dv) {
    float J[6];
    side_j(pos, dir, m6, J);
    side_axpy_j(J, sb, a, dv);
}

// The Jacobian of one side of a joint row: a force along +-e at the anchor
// (lever arm pos) or a torque about +-e; side 2 takes the negated direction.
__device__ __forceinline__ void joint_side_j(bool angular, np::V e, np::V pos, bool side2, uint32_t m6, float* J) {
    if (side2) e = np::neg(e);
    if (angular) {
        const float f[6] = {0.0f, 0.0f, 0.0f, e.x, e.y, e.z};
#pragma unroll
        for (int k = 0; k < 6; ++k) J[k] = f[k] * (((m6 >> k) & 1u) ? 1.0f : 0.0f);
    } else {
        side_j(pos, e, m6, J);
    }
}

// J . dv over both sides: side sums, then their sum, when both sides have dofs.
__device__ __forceinline__ float jdot(np::V dir, np::V pos1, np::V pos2, uint32_t mask, const DV& dv, bool has1,
                                      bool has2) {
    if (has1 && has2) {
        float s1 = side_dot(pos1, dir, mask & 0x3fu, dv.a);
        float s2 = side_dot(pos2, np::neg(dir), (mask >> 8) & 0x3fu, dv.b);
        return s1 + s2;
    }
    if (has1) return side_dot(pos1, dir, mask & 0x3fu, dv.a);
    if (has2) return side_dot(pos2, np::neg(dir), (mask >> 8) & 0x3fu, dv.b);
    return 0.0f;
}

// Inverse masses of a task's two bodies, held in registers.
struct BodyMasses {
    SB s[2];
    __device__ __forceinline__ SB get(int side) const { return s[side]; }
};

template <class BM>
__device__ __forceinline__ void axpy(np::V dir, np::V pos1, np::V pos2, uint32_t mask, const BM& bm, DV& dv, float a,
                                     bool has1, bool has2) {
    if (has1) side_axpy(pos1, dir, mask & 0x3fu, bm.get(0), a, dv.a);
    if (has2) side_axpy(pos2, np::neg(dir), (mask >> 8) & 0x3fu, bm.get(1), a, dv.b);
}

// One contact of a solver manifold: 4 float4 (64 bytes), constant during the
// velocity solve, read through the non-coherent path.
//   c0 = (n, mu)   c1 = (pos1, r_n)   c2 = (pos2, rhs_n)   c3 = (r_t1, rhs_t1, r_t2, rhs_t2)
// pos1 / pos2 are the contact points minus the body centres of mass; n points
// from body 1 to body 2. The impulses (normal, tangent 1, tangent 2) live in a
// separate float4 per contact.
struct ContactRec {
    np::V n, pos1, pos2;
    float mu, r[3], rhs[3];
};
__device__ __forceinline__ ContactRec load_con(const float4* con, size_t i) {
    float4 c0 = __ldg(con + 4 * i), c1 = __ldg(con + 4 * i + 1), c2 = __ldg(con + 4 * i + 2), c3 = __ldg(con + 4 * i + 3);
    ContactRec c;
    c.n = np::mk(c0.x, c0.y, c0.z);
    c.mu = c0.w;
    c.pos1 = np::mk(c1.x, c1.y, c1.z);
    c.r[0] = c1.w;
    c.pos2 = np::mk(c2.x, c2.y, c2.z);
    c.rhs[0] = c2.w;
    c.r[1] = c3.x; c.rhs[1] = c3.y; c.r[2] = c3.z; c.rhs[2] = c3.w;
    return c;
}

__device__ __forceinline__ void load_dv(const float* dvg, int i, float* o) {
    if (i < 0) return;
#pragma unroll
    for (int k = 0; k < 6; ++k) o[k] = dvg[6 * i + k];
}
__device__ __forceinline__ void store_dv(float* dvg, int i, const float* o) {
    if (i < 0) return;
#pragma unroll
    for (int k = 0; k < 6; ++k) dvg[6 * i + k] = o[k];
}

// The FP64 residual's rows in float-float arithmetic: a value is the
// unevaluated sum hi + lo of two floats, built from the error-free
// transformations TwoSum (Knuth), FastTwoSum and TwoProduct by a fused
// multiply-add (Dekker), which carry about twice the f32 precision. J dv + rhs
// is the compensated dot product Dot2 of Ogita, Rump and Oishi ("Accurate sum
// and dot product", SIAM J. Sci. Comput. 26(6), 2005). A thread sums its rows'
// phi^2 and lambda^2 the same way and widens them to double once; the
// reduction across threads is FP64. The rows' arithmetic so stays on the f32
// pipes (GB300 issues FP64 at a small fraction of the f32 rate).
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float z = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z))};
}
__device__ __forceinline__ FF fast_two_sum(float a, float b) {   // |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ FF ff_norm(FF a) {
    return two_sum(a.hi, a.lo);
}
__device__ __forceinline__ bool ff_less(FF a, FF b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
// a + b for normalised a, b.
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    FF s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
// a^2 for normalised a.
__device__ __forceinline__ FF ff_sq(FF a) {
    FF p = two_prod(a.hi, a.hi);
    return fast_two_sum(p.hi, __fadd_rn(p.lo, __fmul_rn(2.0f, __fmul_rn(a.hi, a.lo))));
}
// Per-thread sums of phi^2 and lambda^2.
struct ResidualSums {
    FF s2{0.0f, 0.0f}, l2{0.0f, 0.0f};
    __device__ __forceinline__ double phi2() const { return (double)s2.hi + (double)s2.lo; }
    __device__ __forceinline__ double lam2() const { return (double)l2.hi + (double)l2.lo; }
};
struct Dot2 {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void sum(float h, float e) {
        const FF t = two_sum(s, h);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, e));
    }
    __device__ __forceinline__ void prod(float x, float y) {
        const FF p = two_prod(x, y);
        sum(p.hi, p.lo);
    }
};

// phi = lambda - proj(lambda - r (J dv + rhs)) of one row, squared and summed
// with lambda^2 into `acc`; proj = max(., 0) for a normal row (and a
// prismatic limit row), the clamp to +-mu lambda_n for a friction row, and
// the identity for a joint's bilateral row (Independent limits of +-FLT_MAX,
// helper.rs:186-189). jac(side, J) forms the row's Jacobian on side 0 or 1.
enum { RES_NORMAL = 0, RES_FRICTION = 1, RES_BILATERAL = 2 };
template <class Jac>
__device__ __forceinline__ void residual_row_f(const Jac& jac, float r, float rhs, float lam, const DV& dv, bool has1,
                                               bool has2, int kind, float normal_impulse, float mu, ResidualSums& acc) {
    Dot2 dot;
    float J[6];
    if (has1) {
        jac(0, J);
        for (int k = 0; k < 6; ++k) dot.prod(J[k], dv.a[k]);
    }
    if (has2) {
        jac(1, J);
        for (int k = 0; k < 6; ++k) dot.prod(J[k], dv.b[k]);
    }
    dot.sum(rhs, 0.0f);
    const FF d = two_sum(dot.s, dot.c);
    // rd = r d; x = lambda - rd; lambda - x = rd when the projection keeps x.
    FF rd = two_prod(r, d.hi);
    rd = fast_two_sum(rd.hi, __fadd_rn(rd.lo, __fmul_rn(r, d.lo)));
    FF x = two_sum(lam, -rd.hi);
    x = ff_norm(FF{x.hi, __fsub_rn(x.lo, rd.lo)});
    FF phi = rd;
    if (kind == RES_BILATERAL) {
        // x stays: phi = rd.
    } else if (kind == RES_NORMAL) {
        if (!(x.hi > 0.0f || (x.hi == 0.0f && x.lo > 0.0f))) phi = FF{lam, 0.0f};
    } else {
        const FF mx = two_prod(mu, normal_impulse);
        if (ff_less(x, FF{-mx.hi, -mx.lo})) {
            FF t = two_sum(lam, mx.hi);
            phi = ff_norm(FF{t.hi, __fadd_rn(t.lo, mx.lo)});
        } else if (ff_less(mx, x)) {
            FF t = two_sum(lam, -mx.hi);
            phi = ff_norm(FF{t.hi, __fsub_rn(t.lo, mx.lo)});
        }
    }
    acc.s2 = ff_add(acc.s2, ff_sq(phi));
    acc.l2 = ff_add(acc.l2, two_prod(lam, lam));
}

// A contact row: a force along dir at the lever arms pos1, pos2.
__device__ __forceinline__ void residual_row(np::V dir, np::V pos1, np::V pos2, uint32_t mask, float r, float rhs,
                                             float lam, const DV& dv, bool has1, bool has2, bool friction,
                                             float normal_impulse, float mu, ResidualSums& acc) {
    const auto jac = [&](int side, float* J) {
        if (side == 0) side_j(pos1, dir, mask & 0x3fu, J);
        else side_j(pos2, np::neg(dir), (mask >> 8) & 0x3fu, J);
    };
    residual_row_f(jac, r, rhs, lam, dv, has1, has2, friction ? RES_FRICTION : RES_NORMAL, normal_impulse, mu, acc);
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    __syncthreads();
    return t;
}

// ================================================================ activation
#if NPGPU_EXCHANGE_TU
__global__ void k_act_init(World w, StepParams p) {
    const Bodies& b = w.b;
    GRID_FOR(i, w.nb_slots) {
        uint32_t info = b.info[i];
        b.uf_parent[i] = i;
        b.can_deact[i] = 1;
        b.cw[2 * i] = 0ull;
        b.cw[2 * i + 1] = 0ull;
        b.adj_count[i] = 0;
        b.adj_fill[i] = 0;
#pragma unroll
        for (int k = 0; k < 6; ++k) b.dv[6 * i + k] = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) b.dvf[8 * i + k] = 0ull;   // Δv 0 at update count 0
        if ((info & BI_ALIVE) && bi_status(info) == 2u) {
            const float* iI = b.inv_I + 9 * i;
            float im = b.inv_mass[i];
            b.sb[3 * i] = make_float4(iI[0], iI[1], iI[2], im);
            b.sb[3 * i + 1] = make_float4(iI[3], iI[4], iI[5], 0.0f);
            b.sb[3 * i + 2] = make_float4(iI[6], iI[7], iI[8], 0.0f);
        }
        info &= ~BI_ISLAND;
        b.info[i] = info;
        if (!(info & BI_ALIVE)) continue;
        if (bi_status(info) == 2u && body_is_active(info, b.energy[i]) && body_can_sleep(info)) {
            // ActivationManager::update_energy (activation_manager.rs:47-58).
            float4 l = b.lin[i], a = b.ang[i];
            float v2 = l.x * l.x + l.y * l.y + l.z * l.z + a.x * a.x + a.y * a.y + a.z * a.z;
            float e = (1.0f - p.activation_mix) * b.energy[i] + p.activation_mix * v2;
            float cap = b.sleep_thr[i] * 4.0f;
            b.energy[i] = (cap < e) ? cap : e;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Control* c = w.ctl;
        c->nsolver = 0;
        c->ncolours = 0;
        c->nsolver_contacts = 0;
        c->nactive = 0;
        c->iterations = 0;
        c->res_acc[0] = 0.0;
        c->res_acc[1] = 0.0;
        c->residual = 0.0;
        c->residual_initial = 0.0;
        c->kinetic_energy = 0.0;
        c->task_ns = 0ull;
        c->wait_ns = 0ull;
        c->tasks = 0ull;
        c->res_acc_init[0] = 0.0;
        c->res_acc_init[1] = 0.0;
        for (int k = 0; k < 4; ++k) c->world_next[k] = 0u;
        c->learned_starts = 0u;
        c->learned_kept = 0u;
    }
}
#endif

// A body is sleepy when it may sleep and its energy is below its threshold
// (the per-body condition of activation_manager.rs:172-175).
__device__ __forceinline__ bool body_sleepy(const Bodies& b, uint32_t i, uint32_t info) {
    return body_can_sleep(info) && b.energy[i] < b.sleep_thr[i];
}

// Islands: an island sleeps only if every body in it is sleepy, so only the
// contact edges with a sleepy end matter (a path from a sleepy body to the
// nearest non-sleepy one uses only such edges); edges between two non-sleepy
// bodies are skipped. The resulting sleep decisions equal the union-find over
// all edges (activation_manager.rs:148-200).
#if NPGPU_EXCHANGE_TU
__global__ void k_act_union(World w) {
    const uint32_t npairs = w.ctl->npairs;
    const Bodies& b = w.b;
    GRID_FOR(q, npairs) {
        if (w.cur.ncont[q] == 0) continue;
        uint2 pr = w.cur.pair[q];
        uint32_t b1 = w.c.body[pr.x], b2 = w.c.body[pr.y];
        uint32_t i1 = b.info[b1], i2 = b.info[b2];
        uint32_t s1 = bi_status(i1), s2 = bi_status(i2);
        if (!((s1 == 2u || s1 == 3u) && (s2 == 2u || s2 == 3u))) continue;
        if (!body_sleepy(b, b1, i1) && !body_sleepy(b, b2, i2)) continue;
        uf_union(b.uf_parent, b1, b2, &w.ctl->err);
    }
    // Unbroken joints join their bodies' islands (activation_manager.rs:154-159).
    GRID_FOR(jj, w.nj_slots) {
        if (!(w.j.info[jj] & JI_ALIVE) || (w.j.state[jj] & JS_BROKEN)) continue;
        uint32_t b1 = w.j.body[2 * jj], b2 = w.j.body[2 * jj + 1];
        uint32_t i1 = b.info[b1], i2 = b.info[b2];
        uint32_t s1 = bi_status(i1), s2 = bi_status(i2);
        if (!((s1 == 2u || s1 == 3u) && (s2 == 2u || s2 == 3u))) continue;
        if (!body_sleepy(b, b1, i1) && !body_sleepy(b, b2, i2)) continue;
        uf_union(b.uf_parent, b1, b2, &w.ctl->err);
    }
}
#endif

#if NPGPU_EXCHANGE_TU
__global__ void k_act_root(World w) {
    const Bodies& b = w.b;
    GRID_FOR(i, w.nb_slots) {
        uint32_t info = b.info[i];
        uint32_t st = bi_status(info);
        if (!(info & BI_ALIVE) || !(st == 2u || st == 3u)) continue;
        if (!body_sleepy(b, i, info)) atomicAnd(&b.can_deact[uf_find(b.uf_parent, i)], 0);
    }
}
#endif

#if NPGPU_EXCHANGE_TU
__global__ void k_act_apply(World w) {
    const Bodies& b = w.b;
    uint32_t active = 0;   // folded per warp below
    GRID_FOR(i, w.nb_slots) {
        uint32_t info = b.info[i];
        uint32_t st = bi_status(info);
        if (!(info & BI_ALIVE) || !(st == 2u || st == 3u)) continue;
        uint32_t r = uf_find(b.uf_parent, i);
        float en = b.energy[i];
        if (b.can_deact[r]) {
            if (body_is_active(info, en)) {
                // RigidBody::deactivate (rigid_body.rs:396-400).
                b.info[i] = info & ~BI_CHANGED;
                b.energy[i] = 0.0f;
                b.lin[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                b.ang[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        } else if (st != 3u) {
            b.info[i] = info | BI_ISLAND;
            ++active;
            if (!(en != 0.0f) && body_can_sleep(info)) body_activate(b, i);
        }
    }
    active = __reduce_add_sync(0xffffffffu, active);
    if ((threadIdx.x & 31u) == 0u && active > 0u) atomicAdd(&w.ctl->nactive, active);
}
#endif

// ================================================================ collection + colouring
// Whole warps walk the pairs together, so a warp takes the solver slots of
// its manifolds with one atomic (same-address atomics serialise in L2). The
// slot order is free: everything downstream orders manifolds by priority.
#if !NPGPU_EXCHANGE_TU
__global__ void k_collect(World w) {
    const uint32_t npairs = w.ctl->npairs;
    const Bodies& b = w.b;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t q0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); q0 < npairs; q0 += gridDim.x * blockDim.x) {
        const uint32_t q = q0 + lane;
        uint32_t nc = 0, b1 = 0, b2 = 0, s1 = 0, s2 = 0;
        bool take = false;
        if (q < npairs) nc = w.cur.ncont[q];
        if (nc != 0) {
            uint2 pr = w.cur.pair[q];
            b1 = w.c.body[pr.x];
            b2 = w.c.body[pr.y];
            s1 = bi_status(b.info[b1]);
            s2 = bi_status(b.info[b2]);
            if (s1 != 0u && s2 != 0u) {
                bool a1 = s1 == 2u && b.energy[b1] != 0.0f;
                bool a2 = s2 == 2u && b.energy[b2] != 0.0f;
                take = a1 || a2;
            }
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, take);
        if (bal == 0u) continue;
        const uint32_t contacts = __reduce_add_sync(0xffffffffu, take ? nc : 0u);
        uint32_t base = 0;
        if (lane == 0) {
            base = atomicAdd(&w.ctl->nsolver, (uint32_t)__popc(bal));
            atomicAdd(&w.ctl->nsolver_contacts, contacts);
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        if (!take) continue;
        const uint32_t m = base + (uint32_t)__popc(bal & ((1u << lane) - 1u));
        w.s.sm_list[m] = q;
        w.s.sm_b1[m] = s1 == 2u ? (int)b1 : -1;
        w.s.sm_b2[m] = s2 == 2u ? (int)b2 : -1;
        w.s.sm_nc[m] = nc;
        if (s1 == 2u) atomicAdd(&b.adj_count[b1], 1u);
        if (s2 == 2u) atomicAdd(&b.adj_count[b2], 1u);
    }
}
#endif

// The active joints (JointConstraint::is_active, joint_constraint.rs:218-227:
// a dynamic body of the joint is awake, mechanical_world.rs:274-279) join
// the solver manifolds after the contact manifolds; their state records
// whether they were solved this step.
#if !NPGPU_EXCHANGE_TU
__global__ void k_collect_joints(World w) {
    const Bodies& b = w.b;
    GRID_FOR(jj, w.nj_slots) {
        const uint32_t ji = w.j.info[jj];
        if (!(ji & JI_ALIVE)) continue;
        uint32_t st = w.j.state[jj] & ~JS_ACTIVE;
        if (!(st & JS_BROKEN)) {
            const uint32_t b1 = w.j.body[2 * jj], b2 = w.j.body[2 * jj + 1];
            const uint32_t s1 = bi_status(b.info[b1]), s2 = bi_status(b.info[b2]);
            const bool a1 = s1 == 2u && b.energy[b1] != 0.0f;
            const bool a2 = s2 == 2u && b.energy[b2] != 0.0f;
            if (a1 || a2) {
                const uint32_t m = atomicAdd(&w.ctl->nsolver, 1u);
                if (m >= w.cap_pairs) {
                    atomicOr(&w.ctl->err, ERRF_PAIR_CAPACITY);
                } else {
                    w.s.sm_list[m] = kJointBit | jj;
                    w.s.sm_b1[m] = s1 == 2u ? (int)b1 : -1;
                    w.s.sm_b2[m] = s2 == 2u ? (int)b2 : -1;
                    w.s.sm_nc[m] = joint_group_count(ji & JI_KIND_MASK);
                    if (s1 == 2u) atomicAdd(&b.adj_count[b1], 1u);
                    if (s2 == 2u) atomicAdd(&b.adj_count[b2], 1u);
                    st |= JS_ACTIVE;
                }
            }
        }
        w.j.state[jj] = st;
    }
}

// The solver manifold count stays within the solver arrays after an overflow
// (reported as a capacity error).
__global__ void k_clamp_solver(World w) {
    if (w.ctl->nsolver > w.cap_pairs) w.ctl->nsolver = w.cap_pairs;
}
#endif

#if !NPGPU_EXCHANGE_TU
__global__ void k_adj_fill(World w) {
    const uint32_t ms = w.ctl->nsolver;
    GRID_FOR(m, ms) {
        int b1 = w.s.sm_b1[m], b2 = w.s.sm_b2[m];
        if (b1 >= 0) w.s.adj[w.b.adj_start[b1] + atomicAdd(&w.b.adj_fill[b1], 1u)] = m;
        if (b2 >= 0) w.s.adj[w.b.adj_start[b2] + atomicAdd(&w.b.adj_fill[b2], 1u)] = m;
    }
}
#endif

// A joint's priority hashes its world-local slot with a second input no
// collider pair has, and keeps the joint slot under a collider field no
// collider slot reaches, so that it never equals a pair's.
__device__ __forceinline__ unsigned long long joint_priority(uint32_t local, uint32_t j) {
    return ((unsigned long long)pair_hash22(local, 0x3fffffu) << 42) | (0x1fffffull << 21) | (unsigned long long)j;
}

__device__ __forceinline__ unsigned long long sm_priority(const World& w, uint32_t m) {
    const uint32_t q = w.s.sm_list[m];
    if (q & kJointBit) return joint_priority(w.j.local[q & ~kJointBit], q & ~kJointBit);
    uint2 pr = w.cur.pair[q];
    return pair_priority(w.c.local[pr.x], w.c.local[pr.y], pr.x, pr.y);
}

// Rank of each manifold among the solver manifolds of each of its dynamic
// bodies, by decreasing priority.
#if !NPGPU_EXCHANGE_TU
__global__ void k_prank(World w) {
    const uint32_t ms = w.ctl->nsolver;
    GRID_FOR(m, ms) {
        unsigned long long pm = sm_priority(w, m);
        uint32_t r[2] = {0u, 0u};
        int bs[2] = {w.s.sm_b1[m], w.s.sm_b2[m]};
        for (int side = 0; side < 2; ++side) {
            int b = bs[side];
            if (b < 0) continue;
            uint32_t s0 = w.b.adj_start[b], n = w.b.adj_count[b], cnt = 0;
            for (uint32_t e = 0; e < n; ++e) {
                uint32_t o = w.s.adj[s0 + e];
                if (o != m && sm_priority(w, o) > pm) ++cnt;
            }
            r[side] = cnt;
        }
        w.s.sm_prank[m] = r[0] | (r[1] << 16);
    }
}
#endif

// Greedy first-fit colouring in decreasing priority: a manifold takes the
// smallest colour unused by the higher-priority manifolds of its dynamic
// bodies, as soon as those are coloured.
#if NPGPU_EXCHANGE_TU
__global__ void __launch_bounds__(kCoopThreads) k_colour(World w) {
    const uint32_t ms = w.ctl->nsolver;
    const uint32_t T = gridDim.x * blockDim.x;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nmine = t < ms ? (ms - t + T - 1) / T : 0u;
    if ((ms + T - 1) / T > (uint32_t)kMaxPerThread) {
        if (t == 0) atomicOr(&w.ctl->err, ERRF_TASKS);
        return;
    }
    const Bodies& b = w.b;
    uint32_t done = 0, todo = (nmine >= 32u) ? 0xffffffffu : ((1u << nmine) - 1u);
    int mb1[kMaxPerThread], mb2[kMaxPerThread];
    uint32_t mpr[kMaxPerThread];
    for (uint32_t k = 0; k < nmine; ++k) {
        uint32_t m = t + k * T;
        mb1[k] = w.s.sm_b1[m];
        mb2[k] = w.s.sm_b2[m];
        mpr[k] = w.s.sm_prank[m];
    }
    unsigned long long t0 = 0;
    unsigned backoff = 32;
    uint32_t ncol = 0;   // colours this thread used, folded per warp below
    while (__any_sync(0xffffffffu, done != todo)) {
        bool progress = false;
        for (uint32_t k = 0; k < nmine; ++k) {
            if (done & (1u << k)) continue;
            uint32_t m = t + k * T;
            int b1 = mb1[k], b2 = mb2[k];
            uint32_t pr = mpr[k];
            uint32_t r1 = pr & 0xffffu, r2 = pr >> 16;
            // Each body's two colour words hold its colour mask (colours
            // 0-55, then 56-111) and, in both, how many of its manifolds have
            // been coloured: the count is the flag.
            unsigned long long u1a = (unsigned long long)r1 << 56, u1b = u1a;
            unsigned long long u2a = (unsigned long long)r2 << 56, u2b = u2a;
            if (b1 >= 0) ld_relaxed_v2(b.cw + 2 * (size_t)b1, u1a, u1b);
            if (b2 >= 0) ld_relaxed_v2(b.cw + 2 * (size_t)b2, u2a, u2b);
            if ((u1a >> 56) != r1 || (u1b >> 56) != r1 || (u2a >> 56) != r2 || (u2b >> 56) != r2) continue;
            const unsigned long long ma = (u1a | u2a) & kColourMask, mb = (u1b | u2b) & kColourMask;
            uint32_t col;
            if (ma != kColourMask) {
                col = (uint32_t)(__ffsll((long long)~ma) - 1);
            } else if (mb != kColourMask) {
                col = (uint32_t)kColourBits + (uint32_t)(__ffsll((long long)~mb) - 1);
            } else {
                atomicOr(&w.ctl->err, ERRF_COLOURS);
                col = kStepColours - 1;
            }
            w.s.sm_colour[m] = col;
            const unsigned long long bita = col < (uint32_t)kColourBits ? 1ull << col : 0ull;
            const unsigned long long bitb = col < (uint32_t)kColourBits ? 0ull : 1ull << (col - kColourBits);
            if (b1 >= 0) {
                const unsigned long long hi = (unsigned long long)(r1 + 1u) << 56;
                st_relaxed_v2(b.cw + 2 * (size_t)b1, hi | (u1a & kColourMask) | bita, hi | (u1b & kColourMask) | bitb);
            }
            if (b2 >= 0) {
                const unsigned long long hi = (unsigned long long)(r2 + 1u) << 56;
                st_relaxed_v2(b.cw + 2 * (size_t)b2, hi | (u2a & kColourMask) | bita, hi | (u2b & kColourMask) | bitb);
            }
            ncol = col + 1u > ncol ? col + 1u : ncol;
            done |= 1u << k;
            progress = true;
        }
        if (__any_sync(0xffffffffu, progress)) {
            t0 = 0;
            backoff = 32;
        } else if (!warp_wait_backoff(w.ctl, t0, backoff)) {
            return;
        }
    }
    ncol = __reduce_max_sync(0xffffffffu, ncol);
    if ((threadIdx.x & 31u) == 0u && ncol > 0u) atomicMax(&w.ctl->ncolours, ncol);
}
#endif

// ================================================================ assembly
// A point given in a body's frame, in world space: Isometry * Point
// (world_point_at_material_point, rigid_body.rs:641-643).
__device__ __forceinline__ np::V body_point(np::V t, np::Q q, np::V local) {
    return np::add(np::qrot(q, local), t);
}

// `rows`: also store each contact's three rows in full, for the one-grid
// schedule's iterations.
#if !NPGPU_EXCHANGE_TU

// A joint's row group: `rows` forces along (JR_LINEAR) or torques about
// (JR_ANGULAR) the directions d, their impulses in the joint's slots
// slot..slot + rows - 1 (0-2 linear, 3-5 angular).
struct JointGroup {
    uint32_t kind, rows, slot;
    np::V d[3];
};

// The row groups of joint kind `kind` (at most two) with body rotations q1, q2
// and local axes ax1, ax2, as each constraint's velocity_constraints builds
// them (ball_constraint.rs:80-127, fixed_constraint.rs:107-172,
// revolute_constraint.rs:181-266, cartesian_constraint.rs,
// planar_constraint.rs, rectangular_constraint.rs, universal_constraint.rs)
// from helper::cancel_relative_linear_velocity[_wrt_axis],
// cancel_relative_angular_velocity[_wrt_axis] and
// restrict_relative_angular_velocity_to_axis (helper.rs:167-296, 422-551,
// 614-699); the subspace basis of an axis is the contact model's tangent basis.
// relative_eq!(a, b) of two f32 (approx's defaults: epsilon and max
// relative difference f32::EPSILON).
__device__ __forceinline__ bool relative_eq_f(float a, float b) {
    const float d = fabsf(a - b);
    if (d <= FLT_EPSILON) return true;
    const float m = fabsf(a) > fabsf(b) ? fabsf(a) : fabsf(b);
    return d <= m * FLT_EPSILON;
}

// The offset-limit row of a prismatic joint (unit_constraint.rs:33-123): none
// while the offset of anchor2 along the axis is within the limits; else a
// force along -axis (below the minimum) or +axis (above the maximum) whose
// impulse stays in [0, max], or an unlimited one when the limits are equal.
__device__ __forceinline__ JointGroup limit_group(np::V axis, float offset, uint32_t info, float mn, float mx) {
    const np::V zero = np::mk(0.0f, 0.0f, 0.0f);
    JointGroup g{JR_LIMIT, 0u, 6u, {zero, zero, zero}};
    const bool has_min = (info & JI_MIN_OFFSET) != 0u, has_max = (info & JI_MAX_OFFSET) != 0u;
    if (has_min && has_max && relative_eq_f(mn, mx)) {
        g.kind = JR_LINEAR;
        g.rows = 1u;
        g.d[0] = axis;
    } else if (has_min && offset <= mn) {
        g.rows = 1u;
        g.d[0] = np::neg(axis);
    } else if (has_max && offset >= mx) {
        g.rows = 1u;
        g.d[0] = axis;
    }
    return g;
}

__device__ __forceinline__ uint32_t joint_groups(uint32_t kind, np::Q q1, np::Q q2, np::V a1, np::V a2,
                                                 const float4* ax, uint32_t info, JointGroup* g) {
    const np::V ex = basis_axis(0), ey = basis_axis(1), ez = basis_axis(2), zero = np::mk(0.0f, 0.0f, 0.0f);
    const JointGroup lin3{JR_LINEAR, 3u, 0u, {ex, ey, ez}}, ang3{JR_ANGULAR, 3u, 3u, {ex, ey, ez}};
    const np::V ax1 = v3(ax[0]), ax2 = v3(ax[1]), ax3 = v3(ax[2]);
    switch (kind) {
    case NPGPU_JOINT_BALL: g[0] = lin3; return 1;
    case NPGPU_JOINT_FIXED: g[0] = lin3; g[1] = ang3; return 2;
    case NPGPU_JOINT_CARTESIAN: g[0] = ang3; return 1;
    case NPGPU_JOINT_REVOLUTE: {
        np::V t1, t2;
        tangent_basis(np::qrot(q1, ax1), t1, t2);
        g[0] = lin3;
        g[1] = JointGroup{JR_ANGULAR, 2u, 3u, {t1, t2, zero}};
        return 2;
    }
    case NPGPU_JOINT_PLANAR: {
        const np::V a = np::qrot(q1, ax1);
        np::V t1, t2;
        tangent_basis(a, t1, t2);
        g[0] = JointGroup{JR_LINEAR, 1u, 0u, {a, zero, zero}};
        g[1] = JointGroup{JR_ANGULAR, 2u, 3u, {t1, t2, zero}};
        return 2;
    }
    case NPGPU_JOINT_RECTANGULAR:
        g[0] = JointGroup{JR_LINEAR, 1u, 0u, {np::qrot(q1, ax1), zero, zero}};
        g[1] = ang3;
        return 2;
    case NPGPU_JOINT_UNIVERSAL: {
        np::V o;
        float n;
        const bool has = unit_try(np::cross(np::qrot(q1, ax1), np::qrot(q2, ax2)), FLT_EPSILON, o, n);
        g[0] = lin3;
        g[1] = JointGroup{JR_ANGULAR, has ? 1u : 0u, 3u, {has ? o : zero, zero, zero}};
        return 2;
    }
    case NPGPU_JOINT_PRISMATIC: {
        // restrict_relative_linear_velocity_to_axis, cancel_relative_angular_velocity,
        // then the offset limit (prismatic_constraint.rs).
        const np::V a = np::qrot(q1, ax1);
        np::V t1, t2;
        tangent_basis(a, t1, t2);
        g[0] = JointGroup{JR_LINEAR, 2u, 0u, {t1, t2, zero}};
        g[1] = ang3;
        g[2] = limit_group(a, np::dot(a, np::sub(a2, a1)), info, ax[1].w, ax[2].w);
        return 3;
    }
    default: {
        // Cylindrical: both restricted to axis1; pin-slot: the linear rows to
        // axis1 (axis_v1), the angular rows to axis3 (axis_w1).
        const np::V al = np::qrot(q1, ax1), aa = np::qrot(q1, kind == NPGPU_JOINT_PIN_SLOT ? ax3 : ax1);
        np::V t1, t2, u1, u2;
        tangent_basis(al, t1, t2);
        tangent_basis(aa, u1, u2);
        g[0] = JointGroup{JR_LINEAR, 2u, 0u, {t1, t2, zero}};
        g[1] = JointGroup{JR_ANGULAR, 2u, 3u, {u1, u2, zero}};
        return 2;
    }
    }
}

// The rows of active joint j as solver manifold m: one record per row group,
// the rows' directions in the normal and friction-direction slots, each row
// started from the joint's cached impulse (no warm-start coefficient).
static __device__ void assemble_joint(const World& w, const StepParams& p, uint32_t m, uint32_t j, int b1, int b2,
                                      bool rows) {
    const Bodies& b = w.b;
    const uint32_t bb1 = w.j.body[2 * j], bb2 = w.j.body[2 * j + 1];
    const BodyView v1 = load_view(b, bb1), v2 = load_view(b, bb2);
    uint32_t mask = 0;
    if (b1 >= 0) mask |= ~(bi_flags(v1.info) >> 1) & 0x3fu;
    if (b2 >= 0) mask |= (~(bi_flags(v2.info) >> 1) & 0x3fu) << 8;
    w.s.sm_mask[m] = mask | kJointBit;   // the solver tasks take a joint's records apart from contacts'
    const np::Q q1 = q4(b.pos_q[bb1]), q2 = q4(b.pos_q[bb2]);
    const np::V a1 = body_point(v3(b.pos_t[bb1]), q1, v3(w.j.anchor[2 * j]));
    const np::V a2 = body_point(v3(b.pos_t[bb2]), q2, v3(w.j.anchor[2 * j + 1]));
    JointGroup grp[3];
    const uint32_t info = w.j.info[j], kind = info & JI_KIND_MASK;
    const float4 axes[3] = {w.j.axis[3 * j], w.j.axis[3 * j + 1], w.j.axis[3 * j + 2]};
    const uint32_t ng = joint_groups(kind, q1, q2, a1, a2, axes, info, grp);
    float4* pr4 = w.s.pos_rec + (size_t)m * kPosRec;
    pr4[4] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(kJointBit | j));
    pr4[6] = make_float4(__uint_as_float(bb1), __uint_as_float(bb2), __uint_as_float(v1.info), __uint_as_float(v2.info));
    float4* con = w.s.con + (size_t)m * kMaxContacts * 4;
    float4* lam = w.s.lam + (size_t)m * kMaxContacts;
    float4* tan = w.s.tan + (size_t)m * kMaxContacts * 2;
    const float4 imp[2] = {w.j.imp[2 * j], w.j.imp[2 * j + 1]};
    for (uint32_t k = 0; k < ng; ++k) {
        const JointGroup& G = grp[k];
        const bool ang = G.kind == JR_ANGULAR;   // limit rows are linear
        float R[3][kRowFloats];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            if ((uint32_t)r >= G.rows) {
#pragma unroll
                for (int e = 0; e < kRowFloats; ++e) R[r][e] = 0.0f;
            } else if (ang) {
                make_row_angular(R[r], v1, v2, G.d[r], p.dt);
            } else {
                make_row(R[r], v1, v2, a1, a2, G.d[r], p.dt);
            }
        }
        const np::V zero = np::mk(0.0f, 0.0f, 0.0f);
        const np::V pos1 = ang ? zero : np::sub(a1, v1.com), pos2 = ang ? zero : np::sub(a2, v2.com);
        const float code = joint_code(G.kind, G.rows);
        con[4 * k] = make_float4(G.d[0].x, G.d[0].y, G.d[0].z, code);
        con[4 * k + 1] = make_float4(pos1.x, pos1.y, pos1.z, R[0][RF_R]);
        con[4 * k + 2] = make_float4(pos2.x, pos2.y, pos2.z, R[0][RF_RHS]);
        con[4 * k + 3] = make_float4(R[1][RF_R], R[1][RF_RHS], R[2][RF_R], R[2][RF_RHS]);
        tan[2 * k] = make_float4(G.d[1].x, G.d[1].y, G.d[1].z, 0.0f);
        tan[2 * k + 1] = make_float4(G.d[2].x, G.d[2].y, G.d[2].z, 0.0f);
        if (rows) {
            float4* ro = w.s.rows + ((size_t)m * kMaxContacts + k) * kRowsF4;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
#pragma unroll
                for (int e = 0; e < 6; ++e)
                    ro[kRowF4 * r + e] = make_float4(R[r][4 * e], R[r][4 * e + 1], R[r][4 * e + 2], R[r][4 * e + 3]);
                ro[kRowF4 * r + 6] = make_float4(R[r][RF_R], R[r][RF_RHS], code, 0.0f);
            }
        }
        const float iv[7] = {imp[0].x, imp[0].y, imp[0].z, imp[1].x, imp[1].y, imp[1].z, imp[0].w};
        float l[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t r = 0; r < G.rows; ++r) l[r] = iv[joint_slot(kind, k, r, false)];
        lam[k] = make_float4(l[0], l[1], l[2], -(float)(1u + G.rows));   // a joint record: w = -(1 + rows)
    }
}

// JOINTS: the world has joint slots (their manifolds are assembled too).
template <bool JOINTS>
__global__ void k_assemble(World w, StepParams p, bool rows) {
    const uint32_t ms = w.ctl->nsolver;
    const Bodies& b = w.b;
    const Colliders& c = w.c;
    const float dt = p.dt;
    GRID_FOR(m, ms) {
        uint32_t q = w.s.sm_list[m];
        int b1 = w.s.sm_b1[m], b2 = w.s.sm_b2[m];
        // Colour rank and manifold count on each dynamic body.
        uint32_t col = w.s.sm_colour[m];
        // The colours below col in each of the two words.
        const unsigned long long below_a =
            col >= (uint32_t)kColourBits ? kColourMask : ((col == 0u) ? 0ull : ((1ull << col) - 1ull));
        const unsigned long long below_b =
            col <= (uint32_t)kColourBits ? 0ull : ((1ull << (col - kColourBits)) - 1ull);
        uint32_t rk = 0;
        if (b1 >= 0) {
            const unsigned long long ua = b.cw[2 * (size_t)b1] & kColourMask, ub = b.cw[2 * (size_t)b1 + 1] & kColourMask;
            rk |= (uint32_t)(__popcll(ua & below_a) + __popcll(ub & below_b)) |
                  ((uint32_t)(__popcll(ua) + __popcll(ub)) << 8);
        }
        if (b2 >= 0) {
            const unsigned long long ua = b.cw[2 * (size_t)b2] & kColourMask, ub = b.cw[2 * (size_t)b2 + 1] & kColourMask;
            rk |= ((uint32_t)(__popcll(ua & below_a) + __popcll(ub & below_b)) << 16) |
                  ((uint32_t)(__popcll(ua) + __popcll(ub)) << 24);
        }
        w.s.sm_rk[m] = rk;
        if (JOINTS && (q & kJointBit)) {
            assemble_joint(w, p, m, q & ~kJointBit, b1, b2, rows);
            continue;
        }
        uint2 pr = w.cur.pair[q];
        uint32_t c1 = pr.x, c2 = pr.y;
        uint32_t bb1 = c.body[c1], bb2 = c.body[c2];
        BodyView v1 = load_view(b, bb1), v2 = load_view(b, bb2);
        uint32_t nc = w.s.sm_nc[m];
        uint32_t ci1 = c.info[c1], ci2 = c.info[c2];
        float mu = combine(c.friction[c1], (ci1 >> 4) & 0xfu, c.friction[c2], (ci2 >> 4) & 0xfu);
        float e = combine(c.restitution[c1], (ci1 >> 8) & 0xfu, c.restitution[c2], (ci2 >> 8) & 0xfu);
        float m1 = c.margin[c1], m2 = c.margin[c2];
        // Unlocked dofs of each dynamic side (jacobian_mask, rigid_body.rs:708).
        uint32_t mask = 0;
        if (b1 >= 0) mask |= ~(bi_flags(v1.info) >> 1) & 0x3fu;
        if (b2 >= 0) mask |= (~(bi_flags(v2.info) >> 1) & 0x3fu) << 8;
        w.s.sm_mask[m] = mask;
        {
            // The position solver's record of this manifold (position_core).
            float4* pr4 = w.s.pos_rec + (size_t)m * kPosRec;
            const uint32_t sh1 = ci1 & 0xfu, sh2 = ci2 & 0xfu;
            const float4 pp1 = c.params[c1], pp2 = c.params[c2];
            const float4 wt1 = c.wrt_t[c1], wt2 = c.wrt_t[c2];
            pr4[0] = make_float4(wt1.x, wt1.y, wt1.z, (sh1 == SHAPE_BALL || sh1 == SHAPE_CAPSULE ? pp1.x : 0.0f) + m1);
            pr4[1] = c.wrt_q[c1];
            pr4[2] = make_float4(wt2.x, wt2.y, wt2.z, (sh2 == SHAPE_BALL || sh2 == SHAPE_CAPSULE ? pp2.x : 0.0f) + m2);
            pr4[3] = c.wrt_q[c2];
            pr4[4] = make_float4(pp1.x, pp1.y, pp1.z, __uint_as_float(sh1 | (nc << 8)));
            pr4[5] = make_float4(pp2.x, pp2.y, pp2.z, __uint_as_float(sh2));
            pr4[6] = make_float4(__uint_as_float(bb1), __uint_as_float(bb2), __uint_as_float(v1.info),
                                 __uint_as_float(v2.info));
            for (uint32_t k = 0; k < nc; ++k) {
                const float4 nl = w.cur.nl[q * kMaxContacts + k];
                pr4[7 + k] = make_float4(nl.x, nl.y, nl.z, __uint_as_float(w.cur.key[q * kMaxContacts + k]));
            }
        }
        float4* con = w.s.con + (size_t)m * kMaxContacts * 4;
        float4* lam = w.s.lam + (size_t)m * kMaxContacts;
        // Learned starts: mode 2 for contacts without a cache entry, mode 3
        // for every contact.
        const bool learned = (p.warmstart_mode == 2u || p.warmstart_mode == 3u) && w.mlp != nullptr;
        const bool record = w.s.feat != nullptr;
        const float k1 = (float)((rk >> 8) & 0xffu), k2 = (float)(rk >> 24);
        for (uint32_t k = 0; k < nc; ++k) {
            uint32_t slot = q * kMaxContacts + k;
            float4 w1 = w.cur.w1[slot], w2 = w.cur.w2[slot], nn = w.cur.n[slot], imp = w.cur.imp[slot];
            np::V n = v3(nn);
            np::V center1 = np::add(v3(w1), np::mul(n, m1));
            np::V center2 = np::sub(v3(w2), np::mul(n, m2));
            float rn[kRowFloats], rt[2][kRowFloats];
            make_row(rn, v1, v2, center1, center2, np::neg(n), dt);
            float rhs = rn[RF_RHS];
            if (rhs <= -p.restitution_threshold) rhs = rhs + e * rhs;
            float depth = w1.w + m1 + m2;
            if (depth < 0.0f) rhs = rhs + (-depth) * p.inv_dt;
            np::V t[2];
            tangent_basis(n, t[0], t[1]);
            w.s.tan[((size_t)m * kMaxContacts + k) * 2] = make_float4(t[0].x, t[0].y, t[0].z, 0.0f);
            w.s.tan[((size_t)m * kMaxContacts + k) * 2 + 1] = make_float4(t[1].x, t[1].y, t[1].z, 0.0f);
            for (int sdir = 0; sdir < 2; ++sdir) make_row(rt[sdir], v1, v2, center1, center2, t[sdir], dt);
            np::V pos1 = np::sub(center1, v1.com), pos2 = np::sub(center2, v2.com);
            con[4 * k] = make_float4(n.x, n.y, n.z, mu);
            con[4 * k + 1] = make_float4(pos1.x, pos1.y, pos1.z, rn[RF_R]);
            con[4 * k + 2] = make_float4(pos2.x, pos2.y, pos2.z, rhs);
            con[4 * k + 3] = make_float4(rt[0][RF_R], rt[0][RF_RHS], rt[1][RF_R], rt[1][RF_RHS]);
            if (rows) {
                // The three rows in full for the iterations (J and WJ as
                // fill_constraint_geometry forms them, r, rhs, friction).
                float4* ro = w.s.rows + ((size_t)m * kMaxContacts + k) * kRowsF4;
                const float* src[3] = {rn, rt[0], rt[1]};
                const float rhs3[3] = {rhs, rt[0][RF_RHS], rt[1][RF_RHS]};
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float* R = src[r];
#pragma unroll
                    for (int q = 0; q < 6; ++q) ro[kRowF4 * r + q] = make_float4(R[4 * q], R[4 * q + 1], R[4 * q + 2], R[4 * q + 3]);
                    ro[kRowF4 * r + 6] = make_float4(R[RF_R], rhs3[r], mu, 0.0f);
                }
            }
            const bool cold = p.warmstart_mode == 1u;
            const float4 start = make_float4(cold ? 0.0f : imp.x * p.warmstart_coeff,
                                             cold ? 0.0f : imp.y * p.warmstart_coeff,
                                             cold ? 0.0f : imp.z * p.warmstart_coeff, 0.0f);
            lam[k] = start;
            const bool fresh = imp.w == 0.0f;   // no impulse-cache entry
            const bool predict = learned && (fresh || p.warmstart_mode == 3u);
            if (record || predict) {
                rn[RF_RHS] = rhs;
                float feat[kMlpIn];
                float gn_dt = (p.gx * n.x + p.gy * n.y + p.gz * n.z) * dt;
                mlp_features(rn, rt[0], rt[1], depth, b1 >= 0 ? v1.inv_mass : 0.0f, b2 >= 0 ? v2.inv_mass : 0.0f, mu,
                             gn_dt, (float)nc, k1, k2, feat);
                if (record) {
                    float* fo = w.s.feat + ((size_t)m * kMaxContacts + k) * kMlpIn;
#pragma unroll
                    for (int i = 0; i < kMlpIn; ++i) fo[i] = feat[i];
                }
                if (predict) {
                    float pl[kMlpOut];
                    mlp_forward(w.mlp, feat, pl);
                    mlp_project(mu, pl);
                    // .w = 1: a predicted start, checked in the warm-start
                    // sweep against the start it replaces (kept beside it).
                    w.s.lam_alt[(size_t)m * kMaxContacts + k] = fresh ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : start;
                    lam[k] = make_float4(pl[0], pl[1], pl[2], 1.0f);
                    atomicAdd(&w.ctl->learned_starts, 1u);
                }
            }
        }
    }
}
#endif

// ================================================================ SOR-Prox
// Row directions of a contact: -n for the normal row (body 1 side), and the
// orthonormal basis of n for the friction rows.
__device__ __forceinline__ np::V row_dir(const ContactRec& c, int row, const np::V* t) {
    return row == 0 ? np::neg(c.n) : t[row - 1];
}

// Squared projected-gradient residual of one contact's three rows at Δv for
// impulses lam (fp32; the friction limit follows lam's normal impulse).
__device__ __forceinline__ float local_residual(const ContactRec& c, const np::V* t, uint32_t mask, const DV& dv,
                                                const float* lam, bool h1, bool h2) {
    float s = 0.0f;
    {
        float d = jdot(np::neg(c.n), c.pos1, c.pos2, mask, dv, h1, h2) + c.rhs[0];
        float x = lam[0] - c.r[0] * d;
        float pr = x > 0.0f ? x : 0.0f;
        float phi = lam[0] - pr;
        s = s + phi * phi;
    }
    const float lim = c.mu * lam[0];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        float d = jdot(t[r], c.pos1, c.pos2, mask, dv, h1, h2) + c.rhs[1 + r];
        float x = lam[1 + r] - c.r[1 + r] * d;
        float pr = x < -lim ? -lim : (x > lim ? lim : x);
        float phi = lam[1 + r] - pr;
        s = s + phi * phi;
    }
    return s;
}

// Where a velocity task reads its contacts: global memory, or the running
// thread's slice of a shared-memory cache (element e at base[e * blockDim.x],
// so that the lanes of a warp read consecutive float4).
struct GlobalContacts {
    const float4* con;
    float4* lam;
    const float4* tan;               // the friction directions assembly stored
    const float4* alt;               // learned starts: the start each prediction replaced
    __device__ __forceinline__ ContactRec rec(uint32_t k) const { return load_con(con, k); }
    __device__ __forceinline__ void tangents(const ContactRec&, uint32_t k, np::V* t) const {
        const float4 a = __ldg(tan + 2 * k), b = __ldg(tan + 2 * k + 1);
        t[0] = np::mk(a.x, a.y, a.z);
        t[1] = np::mk(b.x, b.y, b.z);
    }
    __device__ __forceinline__ float4 get_lam(uint32_t k) const { return lam[k]; }
    __device__ __forceinline__ void set_lam(uint32_t k, float4 v) const { lam[k] = v; }
    __device__ __forceinline__ float4 get_alt(uint32_t k) const { return alt[k]; }
};

// A contact row as the iterations read it (stored in full at assembly).
struct RowRec {
    float J1[6], J2[6], W1[6], W2[6];
    float r, rhs, mu;
};
__device__ __forceinline__ RowRec unpack_row(const float4* q) {
    RowRec R;
    const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3], q4 = q[4], q5 = q[5], q6 = q[6];
    const float f[24] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x, q2.y, q2.z, q2.w,
                         q3.x, q3.y, q3.z, q3.w, q4.x, q4.y, q4.z, q4.w, q5.x, q5.y, q5.z, q5.w};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        R.J1[k] = f[RF_J1 + k];
        R.J2[k] = f[RF_J2 + k];
        R.W1[k] = f[RF_WJ1 + k];
        R.W2[k] = f[RF_WJ2 + k];
    }
    R.r = q6.x;
    R.rhs = q6.y;
    R.mu = q6.z;
    return R;
}

// J . dv and dv += a WJ of one row, in the order jdot / axpy use (side sums,
// then their sum; side 1, then side 2), so stored and rebuilt rows give the
// same bits.
__device__ __forceinline__ float row_dot(const RowRec& R, const DV& dv, bool h1, bool h2) {
    float s1 = 0.0f, s2 = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; ++k) s1 = s1 + R.J1[k] * dv.a[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) s2 = s2 + R.J2[k] * dv.b[k];
    if (h1 && h2) return s1 + s2;
    if (h1) return s1;
    if (h2) return s2;
    return 0.0f;
}
__device__ __forceinline__ void row_axpy(const RowRec& R, DV& dv, float a, bool h1, bool h2) {
    if (h1) {
#pragma unroll
        for (int k = 0; k < 6; ++k) dv.a[k] = a * R.W1[k] + dv.a[k];
    }
    if (h2) {
#pragma unroll
        for (int k = 0; k < 6; ++k) dv.b[k] = a * R.W2[k] + dv.b[k];
    }
}

// Where the iterations read a task's rows and impulses: global memory, or
// the running thread's slice of a shared-memory cache (element e at
// base[e * blockDim.x], so that the lanes of a warp read consecutive float4):
// the impulses, then the rows, of one contact.
struct GlobalRows {
    const float4* rows;
    float4* lam;
    __device__ __forceinline__ RowRec row(uint32_t k, int r) const {
        const float4* q = rows + (size_t)k * kRowsF4 + r * kRowF4;
        float4 v[kRowF4];
#pragma unroll
        for (int e = 0; e < kRowF4; ++e) v[e] = __ldg(q + e);
        return unpack_row(v);
    }
    __device__ __forceinline__ float4 get_lam(uint32_t k) const { return lam[k]; }
    __device__ __forceinline__ void set_lam(uint32_t k, float4 v) const { lam[k] = v; }
};
constexpr int kCacheContacts = 1;
constexpr int kCacheF4 = kCacheContacts * (1 + kRowsF4);
// The first kCacheContacts contacts of a manifold from the cache, the rest
// from global memory.
struct CachedRows {
    float4* base;
    GlobalRows g;
    __device__ __forceinline__ float4& at(int e) const { return base[e * (int)blockDim.x]; }
    __device__ __forceinline__ RowRec row(uint32_t k, int r) const {
        if (k >= (uint32_t)kCacheContacts) return g.row(k, r);
        float4 v[kRowF4];
#pragma unroll
        for (int e = 0; e < kRowF4; ++e) v[e] = at((int)k * (1 + kRowsF4) + 1 + r * kRowF4 + e);
        return unpack_row(v);
    }
    __device__ __forceinline__ float4 get_lam(uint32_t k) const {
        return k < (uint32_t)kCacheContacts ? at((int)k * (1 + kRowsF4)) : g.get_lam(k);
    }
    __device__ __forceinline__ void set_lam(uint32_t k, float4 v) const {
        if (k < (uint32_t)kCacheContacts) at((int)k * (1 + kRowsF4)) = v;
        else g.set_lam(k, v);
    }
};

// The warm start (sor_prox.rs:19-45) of a task without learned starts: the
// cached impulses applied along the stored rows.
template <class RS>
__device__ __forceinline__ void warm_rows(const RS& src, uint32_t nc, bool h1, bool h2, DV& dv) {
    for (uint32_t k = 0; k < nc; ++k) {
        const float4 l = src.get_lam(k);
        const float li[3] = {l.x, l.y, l.z};
#pragma unroll 1
        for (int r = 0; r < 3; ++r) {
            if (li[r] == 0.0f) continue;
            row_axpy(src.row(k, r), dv, li[r], h1, h2);
        }
    }
}

// The friction rows (sor_prox.rs:232-343) and the normal rows
// (sor_prox.rs:181-230) of one task's contacts, from stored rows.
template <class RS>
__device__ __forceinline__ void friction_rows(const RS& src, uint32_t nc, bool h1, bool h2, DV& dv) {
    for (uint32_t k = 0; k < nc; ++k) {
        const float4 l = src.get_lam(k);
        const float li = l.x;
        float imps[2] = {l.y, l.z};
#pragma unroll
        for (int sdir = 0; sdir < 2; ++sdir) {
            const float imp = imps[sdir];
            if (li == 0.0f) {
                if (imp != 0.0f) {
                    row_axpy(src.row(k, 1 + sdir), dv, -imp, h1, h2);
                    imps[sdir] = 0.0f;
                }
                continue;
            }
            const RowRec R = src.row(k, 1 + sdir);
            float mx = R.mu * li, mn = -mx;
            float dimp = row_dot(R, dv, h1, h2) + R.rhs;
            float ni = imp - R.r * dimp;
            if (ni < mn) ni = mn;
            else if (ni > mx) ni = mx;
            float dl = ni - imp;
            imps[sdir] = ni;
            row_axpy(R, dv, dl, h1, h2);
        }
        src.set_lam(k, make_float4(li, imps[0], imps[1], 0.0f));
    }
}
template <class RS>
__device__ __forceinline__ void normal_rows(const RS& src, uint32_t nc, bool h1, bool h2, DV& dv) {
    for (uint32_t k = 0; k < nc; ++k) {
        const float4 l = src.get_lam(k);
        const RowRec R = src.row(k, 0);
        float imp = l.x;
        float dimp = row_dot(R, dv, h1, h2) + R.rhs;
        float ni = imp - R.r * dimp;
        ni = ni > 0.0f ? ni : 0.0f;
        float dl = ni - imp;
        src.set_lam(k, make_float4(ni, l.y, l.z, 0.0f));
        row_axpy(R, dv, dl, h1, h2);
    }
}

// One pass over a joint's rows (its row groups' records) from stored rows:
// the bilateral rows of sor_prox.rs:232-293 with Independent limits of
// +-FLT_MAX (helper.rs:186-189), a prismatic limit row's within [0, max]. A
// record's impulses carry w = -(1 + rows). The solver tasks dispatch a joint's
// manifold here (sm_mask's kJointBit) and the call is out of line, Δv passed
// and returned by value, so that the contact sweeps keep their registers.
static __device__ __noinline__ DV joint_rows(const GlobalRows src, uint32_t nc, bool h1, bool h2, DV dv) {
#pragma unroll 1
    for (uint32_t k = 0; k < nc; ++k) {
        const float4 l = src.get_lam(k);
        const uint32_t rows = (uint32_t)(-l.w) - 1u;
        float li[3] = {l.x, l.y, l.z};
#pragma unroll 1
        for (uint32_t r = 0; r < rows; ++r) {
            const RowRec R = src.row(k, (int)r);
            float ni = li[r] - R.r * (row_dot(R, dv, h1, h2) + R.rhs);
            const float lo = joint_limit(R.mu) ? 0.0f : -FLT_MAX;
            ni = ni < lo ? lo : (ni > FLT_MAX ? FLT_MAX : ni);
            const float dl = ni - li[r];
            li[r] = ni;
            row_axpy(R, dv, dl, h1, h2);
        }
        src.set_lam(k, make_float4(li[0], li[1], li[2], l.w));
    }
    return dv;
}

// One velocity task from the compact records, rows rebuilt from the normal,
// the friction directions and the lever arms: KIND 0 is the warm start
// (sor_prox.rs:19-45), 1 the friction rows of an iteration
// (sor_prox.rs:232-343), 2 its normal rows (sor_prox.rs:181-230).
enum { SWEEP_WARM = 0, SWEEP_FRICTION = 1, SWEEP_NORMAL = 2, SWEEP_MANIFOLD = 3 };
// A joint's rows from its compact records, rows rebuilt from the stored
// directions and lever arms: the warm start (warm true) or one pass of the
// bilateral rows (sor_prox.rs:232-293 with Independent limits: +-FLT_MAX, or
// [0, max] for a prismatic limit). Dispatched per manifold and out of line,
// Δv by value, so that the contact tasks keep their registers.
static __device__ __noinline__ DV joint_task(const float4* con, float4* lam, const float4* tan, uint32_t nc,
                                             uint32_t mask, const float4* sb, int g1, int g2, bool warm, DV dv) {
    const bool h1 = g1 >= 0, h2 = g2 >= 0;
    SB s1, s2;
    if (h1) s1 = load_sb(sb, g1);
    if (h2) s2 = load_sb(sb, g2);
#pragma unroll 1
    for (uint32_t k = 0; k < nc; ++k) {
        const ContactRec c = load_con(con, k);
        const float4 l = lam[k];
        const float4 ta = __ldg(tan + 2 * k), tb = __ldg(tan + 2 * k + 1);
        const np::V d[3] = {c.n, np::mk(ta.x, ta.y, ta.z), np::mk(tb.x, tb.y, tb.z)};
        const bool ang = joint_angular(c.mu), lim = joint_limit(c.mu);
        const uint32_t rows = joint_rows_of(c.mu);
        float li[3] = {l.x, l.y, l.z};
#pragma unroll 1
        for (uint32_t r = 0; r < rows; ++r) {
            float J1[6], J2[6];
            if (h1) joint_side_j(ang, d[r], c.pos1, false, mask & 0x3fu, J1);
            if (h2) joint_side_j(ang, d[r], c.pos2, true, (mask >> 8) & 0x3fu, J2);
            float dl = li[r];
            if (warm) {
                if (li[r] == 0.0f) continue;
            } else {
                float dd = 0.0f;
                if (h1 && h2) dd = side_dot_j(J1, dv.a) + side_dot_j(J2, dv.b);
                else if (h1) dd = side_dot_j(J1, dv.a);
                else if (h2) dd = side_dot_j(J2, dv.b);
                float ni = li[r] - c.r[r] * (dd + c.rhs[r]);
                const float lo = lim ? 0.0f : -FLT_MAX;
                ni = ni < lo ? lo : (ni > FLT_MAX ? FLT_MAX : ni);
                dl = ni - li[r];
                li[r] = ni;
            }
            if (h1) side_axpy_j(J1, s1, dl, dv.a);
            if (h2) side_axpy_j(J2, s2, dl, dv.b);
        }
        if (!warm) lam[k] = make_float4(li[0], li[1], li[2], l.w);
    }
    return dv;
}

template <int KIND, class Src, class BM>
__device__ __forceinline__ void velocity_task_src(const Src& src, uint32_t nc, uint32_t mask, uint32_t sweep,
                                                  const BM& bm, bool h1, bool h2, DV& dv, Control* ctl) {
    if (KIND == SWEEP_MANIFOLD) {
        // The manifold's friction rows, then its normal rows.
        velocity_task_src<SWEEP_FRICTION>(src, nc, mask, sweep, bm, h1, h2, dv, ctl);
        velocity_task_src<SWEEP_NORMAL>(src, nc, mask, sweep, bm, h1, h2, dv, ctl);
        return;
    }
    const int kind = KIND;
    for (uint32_t k = 0; k < nc; ++k) {
        const ContactRec c = src.rec(k);
        float4 l = src.get_lam(k);
        if (kind == SWEEP_WARM) {
            np::V t[2];
            src.tangents(c, k, t);
            float li[3] = {l.x, l.y, l.z};
            const bool predicted = l.w != 0.0f;
            DV before;
            if (predicted) before = dv;
#pragma unroll 1
            for (int row = 0; row < 3; ++row) {
                if (li[row] == 0.0f) continue;
                axpy(row_dir(c, row, t), c.pos1, c.pos2, mask, bm, dv, li[row], h1, h2);
            }
            if (predicted) {
                // A learned start stays only if its local residual is no larger
                // than that of the start it replaced (the cached impulses, or
                // zero), which is otherwise applied instead.
                const float4 a4 = src.get_alt(k);
                const float alt[3] = {a4.x, a4.y, a4.z};
                float with = local_residual(c, t, mask, dv, li, h1, h2);
                DV dv_alt = before;
#pragma unroll 1
                for (int row = 0; row < 3; ++row) {
                    if (alt[row] == 0.0f) continue;
                    axpy(row_dir(c, row, t), c.pos1, c.pos2, mask, bm, dv_alt, alt[row], h1, h2);
                }
                float without = local_residual(c, t, mask, dv_alt, alt, h1, h2);
                if (with > without) {
                    dv = dv_alt;
                    src.set_lam(k, make_float4(alt[0], alt[1], alt[2], 0.0f));
                } else {
                    src.set_lam(k, make_float4(li[0], li[1], li[2], 0.0f));
                    atomicAdd(&ctl->learned_kept, 1u);
                }
            }
        } else if (kind == SWEEP_FRICTION) {
            np::V t[2];
            src.tangents(c, k, t);
            float li = l.x;
            float imps[2] = {l.y, l.z};
#pragma unroll
            for (int sdir = 0; sdir < 2; ++sdir) {
                float imp = imps[sdir];
                if (li == 0.0f) {
                    if (imp != 0.0f) {
                        axpy(t[sdir], c.pos1, c.pos2, mask, bm, dv, -imp, h1, h2);
                        imps[sdir] = 0.0f;
                    }
                    continue;
                }
                float mx = c.mu * li, mn = -mx;
                float dimp = jdot(t[sdir], c.pos1, c.pos2, mask, dv, h1, h2) + c.rhs[1 + sdir];
                float ni = imp - c.r[1 + sdir] * dimp;
                if (ni < mn) ni = mn;
                else if (ni > mx) ni = mx;
                float dl = ni - imp;
                imps[sdir] = ni;
                axpy(t[sdir], c.pos1, c.pos2, mask, bm, dv, dl, h1, h2);
            }
            src.set_lam(k, make_float4(li, imps[0], imps[1], 0.0f));
        } else {
            const np::V dn = np::neg(c.n);
            float imp = l.x;
            float dimp = jdot(dn, c.pos1, c.pos2, mask, dv, h1, h2) + c.rhs[0];
            float ni = imp - c.r[0] * dimp;
            ni = ni > 0.0f ? ni : 0.0f;
            float dl = ni - imp;
            src.set_lam(k, make_float4(ni, l.y, l.z, 0.0f));
            axpy(dn, c.pos1, c.pos2, mask, bm, dv, dl, h1, h2);
        }
    }
}

// Where a world's Δv rows live during its velocity solve: one array in the
// block's shared memory (6 floats per body), or spread over the shared
// memories of a thread-block cluster, 2^shift bodies per block, reached
// through distributed shared memory.
struct SharedDv {
    float* base;   // 8-byte aligned: a row is three float2
    __device__ __forceinline__ void load(int l, float* o) const {
        if (l < 0) return;
        const float2* r = (const float2*)(base + 6 * l);
        const float2 a = r[0], b = r[1], c = r[2];
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y; o[4] = c.x; o[5] = c.y;
    }
    __device__ __forceinline__ void store(int l, const float* o) const {
        if (l < 0) return;
        float2* r = (float2*)(base + 6 * l);
        r[0] = make_float2(o[0], o[1]);
        r[1] = make_float2(o[2], o[3]);
        r[2] = make_float2(o[4], o[5]);
    }
};
struct ClusterDv {
    float* base;
    uint32_t shift;
    __device__ __forceinline__ float2* row(int l) const {
        float* r = cg::this_cluster().map_shared_rank(base, (unsigned)((uint32_t)l >> shift));
        return (float2*)(r + 6 * ((uint32_t)l & ((1u << shift) - 1u)));
    }
    __device__ __forceinline__ void load(int l, float* o) const {
        if (l < 0) return;
        const float2* r = row(l);
        float2 a = r[0], b = r[1], c = r[2];
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y; o[4] = c.x; o[5] = c.y;
    }
    __device__ __forceinline__ void store(int l, const float* o) const {
        if (l < 0) return;
        float2* r = row(l);
        r[0] = make_float2(o[0], o[1]);
        r[1] = make_float2(o[2], o[3]);
        r[2] = make_float2(o[4], o[5]);
    }
};

// Velocity task of manifold m read from global memory; g1, g2 are the dynamic
// bodies' slots (-1: no dofs), l1, l2 their Δv rows in `dva`.
// The warm start of manifold m (sweep 0), from the compact records, the
// stored friction directions and the bodies' inverse masses.
__device__ __forceinline__ void warm_task(const World& w, uint32_t m, int g1, int g2, DV& dv) {
    BodyMasses bm;
    if (g1 >= 0) bm.s[0] = load_sb(w.b.sb, g1);
    if (g2 >= 0) bm.s[1] = load_sb(w.b.sb, g2);
    GlobalContacts src{w.s.con + (size_t)m * kMaxContacts * 4, w.s.lam + (size_t)m * kMaxContacts,
                       w.s.tan + (size_t)m * kMaxContacts * 2,
                       w.s.lam_alt ? w.s.lam_alt + (size_t)m * kMaxContacts : nullptr};
    velocity_task_src<SWEEP_WARM>(src, w.s.sm_nc[m], w.s.sm_mask[m], 0u, bm, g1 >= 0, g2 >= 0, dv, w.ctl);
}

__device__ __forceinline__ GlobalRows global_rows(const World& w, uint32_t m) {
    return GlobalRows{w.s.rows + (size_t)m * kMaxContacts * kRowsF4, w.s.lam + (size_t)m * kMaxContacts};
}

// Velocity task of manifold m read from global memory; g1, g2 are the dynamic
// bodies' slots (-1: no dofs), l1, l2 their Δv rows in `dva`.
// The per-world kernels rebuild the rows from the compact records (their
// batches are large enough for the stored rows' bytes to cost more than the
// arithmetic they save).
template <int KIND, bool JOINTS, class DvA>
__device__ __forceinline__ void velocity_task(const World& w, uint32_t m, uint32_t sweep, int g1, int g2, int l1, int l2,
                                              const DvA& dva) {
    BodyMasses bm;
    if (g1 >= 0) bm.s[0] = load_sb(w.b.sb, g1);
    if (g2 >= 0) bm.s[1] = load_sb(w.b.sb, g2);
    GlobalContacts src{w.s.con + (size_t)m * kMaxContacts * 4, w.s.lam + (size_t)m * kMaxContacts,
                       w.s.tan + (size_t)m * kMaxContacts * 2,
                       w.s.lam_alt ? w.s.lam_alt + (size_t)m * kMaxContacts : nullptr};
    DV dv;
    dva.load(g1 >= 0 ? l1 : -1, dv.a);
    dva.load(g2 >= 0 ? l2 : -1, dv.b);
    const uint32_t mask = w.s.sm_mask[m];
    if (JOINTS && (mask & kJointBit)) {
        // A joint's rows: warm-started, then solved once per iteration with
        // the friction rows.
        if (KIND == SWEEP_NORMAL) return;
        dv = joint_task(src.con, src.lam, src.tan, w.s.sm_nc[m], mask, w.b.sb, g1, g2, KIND == SWEEP_WARM, dv);
    } else {
        velocity_task_src<KIND>(src, w.s.sm_nc[m], mask, sweep, bm, g1 >= 0, g2 >= 0, dv, w.ctl);
    }
    dva.store(g1 >= 0 ? l1 : -1, dv.a);
    dva.store(g2 >= 0 ? l2 : -1, dv.b);
}

// Fills the running thread's cache with manifold m's impulses and rows (nc <= kCacheContacts).
__device__ __forceinline__ void cache_task(const World& w, uint32_t m, uint32_t nc, const CachedRows& cc) {
    const float4* rows = w.s.rows + (size_t)m * kMaxContacts * kRowsF4;
    for (uint32_t k = 0; k < nc && k < (uint32_t)kCacheContacts; ++k) {
        cc.at((int)k * (1 + kRowsF4)) = w.s.lam[(size_t)m * kMaxContacts + k];
        for (int e = 0; e < kRowsF4; ++e) cc.at((int)k * (1 + kRowsF4) + 1 + e) = rows[(size_t)k * kRowsF4 + e];
    }
}

// The residual terms of a joint's rows (its row groups' records).
__device__ __forceinline__ void joint_residual(const float4* con, const float4* lam, const float4* tan, uint32_t nc,
                                               uint32_t mask, const DV& dv, bool h1, bool h2, ResidualSums& acc) {
#pragma unroll 1
    for (uint32_t k = 0; k < nc; ++k) {
        const ContactRec c = load_con(con, k);
        const float4 l = lam[k];
        const bool ang = joint_angular(c.mu);
        const uint32_t rows = joint_rows_of(c.mu);
#pragma unroll 1
        for (uint32_t r = 0; r < rows; ++r) {
            np::V d = c.n;
            if (r > 0) {
                const float4 t = tan[2 * k + r - 1];
                d = np::mk(t.x, t.y, t.z);
            }
            const auto jac = [&](int side, float* J) {
                joint_side_j(ang, d, side ? c.pos2 : c.pos1, side != 0, side ? (mask >> 8) & 0x3fu : mask & 0x3fu, J);
            };
            const float li = r == 0 ? l.x : (r == 1 ? l.y : l.z);
            const float rr = r == 0 ? c.r[0] : (r == 1 ? c.r[1] : c.r[2]);
            const float rhs = r == 0 ? c.rhs[0] : (r == 1 ? c.rhs[1] : c.rhs[2]);
            residual_row_f(jac, rr, rhs, li, dv, h1, h2, joint_limit(c.mu) ? RES_NORMAL : RES_BILATERAL, 0.0f, 0.0f,
                           acc);
        }
    }
}

// FP64 residual terms of one manifold (normal rows, then friction rows with
// the normal impulse as the limit).
template <bool JOINTS>
__device__ __forceinline__ void manifold_residual(const World& w, uint32_t m, int g1, int g2, const DV& dv,
                                                  ResidualSums& acc) {
    const bool h1 = g1 >= 0, h2 = g2 >= 0;
    const uint32_t nc = w.s.sm_nc[m], mask = w.s.sm_mask[m];
    const float4* lam = w.s.lam + (size_t)m * kMaxContacts;
    const float4* con = w.s.con + (size_t)m * kMaxContacts * 4;
    if (JOINTS && (mask & kJointBit)) {
        joint_residual(con, lam, w.s.tan + (size_t)m * kMaxContacts * 2, nc, mask, dv, h1, h2, acc);
        return;
    }
    for (uint32_t k = 0; k < nc; ++k) {
        const ContactRec c = load_con(con, k);
        float4 l = lam[k];
        const float4 ta = w.s.tan[((size_t)m * kMaxContacts + k) * 2], tb = w.s.tan[((size_t)m * kMaxContacts + k) * 2 + 1];
        const np::V t[2] = {np::mk(ta.x, ta.y, ta.z), np::mk(tb.x, tb.y, tb.z)};
        residual_row(np::neg(c.n), c.pos1, c.pos2, mask, c.r[0], c.rhs[0], l.x, dv, h1, h2, false, 0.0f, c.mu, acc);
        residual_row(t[0], c.pos1, c.pos2, mask, c.r[1], c.rhs[1], l.y, dv, h1, h2, true, l.x, c.mu, acc);
        residual_row(t[1], c.pos1, c.pos2, mask, c.r[2], c.rhs[2], l.z, dv, h1, h2, true, l.x, c.mu, acc);
    }
}

// The dataflow tasks of one thread: its manifolds m = t + k T, with their
// dynamic bodies and colour ranks read once.
struct MyTasks {
    uint32_t n;
    int b1[kMaxPerThread], b2[kMaxPerThread];
    uint32_t rk[kMaxPerThread];
    uint16_t next[kMaxPerThread];
};

__device__ __forceinline__ void load_tasks(const World& w, uint32_t ms, MyTasks& mt, uint32_t s_begin) {
    const uint32_t T = gridDim.x * blockDim.x;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    mt.n = t < ms ? (ms - t + T - 1) / T : 0u;
    for (uint32_t k = 0; k < mt.n; ++k) {
        uint32_t m = t + k * T;
        mt.b1[k] = w.s.sm_b1[m];
        mt.b2[k] = w.s.sm_b2[m];
        mt.rk[k] = w.s.sm_rk[m];
        mt.next[k] = (uint16_t)s_begin;
    }
}

// Runs sweeps [s_begin, s_end) of this thread's manifolds as their bodies'
// versions allow. Returns false on timeout.
struct TaskStats {
    unsigned long long exec_ns, wait_ns, tasks;
};

template <bool JOINTS>
static __device__ bool velocity_sweeps(const World& w, uint32_t s_begin, uint32_t s_end, uint32_t ms, bool prof,
                                bool learned, bool merged, TaskStats& ts, float4* cache) {
    const uint32_t T = gridDim.x * blockDim.x;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    MyTasks mt;
    load_tasks(w, ms, mt, s_begin);
    // For the iterations (not the warm start), the rows and impulses of the
    // first task's first contact stay in shared memory for the whole call
    // (the impulses are written back at the end); its other contacts are
    // read from global memory.
    const CachedRows cc{cache + threadIdx.x, global_rows(w, t)};
    uint32_t nc0 = 0;
    bool cached = false;
    // Joints' manifolds (sm_mask's kJointBit) take their own pass, from
    // global memory.
    const bool joints = JOINTS;
    if (mt.n > 0 && cache != nullptr && s_begin > 0 && !(joints && (w.s.sm_mask[t] & kJointBit))) {
        nc0 = w.s.sm_nc[t];
        cached = true;
        cache_task(w, t, nc0, cc);
    }
    uint32_t left = mt.n * (s_end - s_begin);
    unsigned long long t0 = 0, tw = prof ? global_ns() : 0ull;
    unsigned backoff = 32;
    bool ok = true;
    // Warp-uniform loop: each pass, the lanes whose next task is ready run it
    // together; the warp sleeps only when no lane could run anything.
    while (__any_sync(0xffffffffu, left > 0)) {
        bool progress = false;
        for (uint32_t k = 0; k < mt.n; ++k) {
            uint32_t sw = mt.next[k];
            if (sw >= s_end) continue;
            int b1 = mt.b1[k], b2 = mt.b2[k];
            uint32_t rk = mt.rk[k];
            uint32_t t1 = sw * ((rk >> 8) & 0xffu) + (rk & 0xffu);
            uint32_t t2 = sw * (rk >> 24) + ((rk >> 16) & 0xffu);
            DV dv;
            bool r1 = poll_dvf(w.b.dvf, b1, t1, dv.a);
            bool r2 = poll_dvf(w.b.dvf, b2, t2, dv.b);
            if (!(r1 && r2)) continue;
            unsigned long long te = prof ? global_ns() : 0ull;
            if (prof) ts.wait_ns += te - tw;
            const uint32_t m = t + k * T;
            const bool h1 = b1 >= 0, h2 = b2 >= 0;
            const bool jt = joints && (w.s.sm_mask[m] & kJointBit);
            if (sw == 0) {
                // Learned starts need the check on the compact records; a
                // joint's records start from their cached impulses.
                if (learned && !jt) warm_task(w, m, b1, b2, dv);
                else warm_rows(global_rows(w, m), w.s.sm_nc[m], h1, h2, dv);
            } else if (jt) {
                // A joint's rows run once per iteration, with the friction rows.
                if (merged || (sw & 1u)) dv = joint_rows(global_rows(w, m), w.s.sm_nc[m], h1, h2, dv);
            } else if (k == 0 && cached) {
                // Merged order: every sweep is the manifold's friction rows
                // and then its normal rows; else odd sweeps are friction rows,
                // even sweeps normal rows.
                if (merged || (sw & 1u)) friction_rows(cc, nc0, h1, h2, dv);
                if (merged || !(sw & 1u)) normal_rows(cc, nc0, h1, h2, dv);
            } else {
                const uint32_t nc = w.s.sm_nc[m];
                if (merged || (sw & 1u)) friction_rows(global_rows(w, m), nc, h1, h2, dv);
                if (merged || !(sw & 1u)) normal_rows(global_rows(w, m), nc, h1, h2, dv);
            }
            publish_dvf(w.b.dvf, b1, t1 + 1u, dv.a);
            publish_dvf(w.b.dvf, b2, t2 + 1u, dv.b);
            if (prof) {
                tw = global_ns();
                ts.exec_ns += tw - te;
                ts.tasks += 1;
            }
            mt.next[k] = (uint16_t)(sw + 1u);
            --left;
            progress = true;
        }
        if (__any_sync(0xffffffffu, progress)) {
            t0 = 0;
            backoff = 32;
        } else if (!warp_wait_backoff(w.ctl, t0, backoff)) {
            ok = false;
            break;
        }
    }
    if (cached)
        for (uint32_t k = 0; k < nc0 && k < (uint32_t)kCacheContacts; ++k)
            w.s.lam[(size_t)t * kMaxContacts + k] = cc.get_lam(k);
    return ok;
}

// FP64 residual over all rows; the result lands in ctl->residual.
template <bool JOINTS>
static __device__ bool eval_residual(const World& w, uint32_t ms, double* sh, uint32_t& epoch, bool initial) {
    ResidualSums acc;
    GRID_FOR(m, ms) {
        int b1 = w.s.sm_b1[m], b2 = w.s.sm_b2[m];
        DV dv;
        load_dvf(w.b.dvf, b1, dv.a);
        load_dvf(w.b.dvf, b2, dv.b);
        manifold_residual<JOINTS>(w, m, b1, b2, dv, acc);
    }
    double ts = block_sum(acc.phi2(), sh);
    double tl = block_sum(acc.lam2(), sh);
    if (threadIdx.x == 0) {
        atomicAdd(&w.ctl->res_acc[0], ts);
        atomicAdd(&w.ctl->res_acc[1], tl);
    }
    if (!grid_sync(w.ctl, epoch)) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double a = w.ctl->res_acc[0], bsum = w.ctl->res_acc[1];
        double r = sqrt(a) / fmax(1.0, sqrt(bsum));
        w.ctl->residual = r;
        if (initial) w.ctl->residual_initial = r;
        w.ctl->res_acc[0] = 0.0;
        w.ctl->res_acc[1] = 0.0;
    }
    return grid_sync(w.ctl, epoch);
}

#if NPGPU_EXCHANGE_TU
template <bool JOINTS>
__global__ void __launch_bounds__(kCoopThreads, 2) k_velocity(World w, StepParams p) {
    __shared__ double sh[32];
    extern __shared__ float4 s_cache[];   // kCacheF4 per thread
    const uint32_t ms = w.ctl->nsolver;
    const uint32_t T = gridDim.x * blockDim.x;
    if ((ms + T - 1) / T > (uint32_t)kMaxPerThread) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&w.ctl->err, ERRF_TASKS);
        return;
    }
    // A failed colouring leaves no consistent order to wait on: the step
    // reports it instead of solving.
    if (w.ctl->err & ERRF_COLOURS) return;
    const bool prof = p.profile != 0;
    const bool learned = p.warmstart_mode == 2u || p.warmstart_mode == 3u;
    TaskStats ts{0ull, 0ull, 0ull};
    unsigned long long k0 = 0;
    if (prof && blockIdx.x == 0 && threadIdx.x == 0) k0 = global_ns();
    uint32_t epoch = 0;
    const bool merged = p.sweep_order == NPGPU_SWEEP_MANIFOLD;
    const uint32_t spi = merged ? 1u : 2u;   // sweeps per iteration
    if (!velocity_sweeps<JOINTS>(w, 0, 1, ms, prof, learned, merged, ts, s_cache)) return;
    if (!grid_sync(w.ctl, epoch)) return;
    if (!eval_residual<JOINTS>(w, ms, sh, epoch, true)) return;
    uint32_t iters = 0;
    if (!p.solve_to_tolerance) {
        iters = p.max_velocity_iterations;
        if (!velocity_sweeps<JOINTS>(w, 1, 1 + spi * iters, ms, prof, learned, merged, ts, s_cache)) return;
        if (!grid_sync(w.ctl, epoch)) return;
        if (!eval_residual<JOINTS>(w, ms, sh, epoch, false)) return;
    } else {
        for (uint32_t it = 0; it < p.max_iterations_to_tolerance; ++it) {
            if (((volatile double*)&w.ctl->residual)[0] <= (double)p.residual_tolerance) break;
            if (!velocity_sweeps<JOINTS>(w, 1 + spi * it, 1 + spi * (it + 1), ms, prof, learned, merged, ts, s_cache)) return;
            ++iters;
            if (!grid_sync(w.ctl, epoch)) return;
            if (!eval_residual<JOINTS>(w, ms, sh, epoch, false)) return;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) w.ctl->iterations = iters;
    // The solved Δv of every body, for the integration that follows.
    GRID_FOR(i, w.nb_slots) load_dvf(w.b.dvf, (int)i, w.b.dv + 6 * i);
    if (prof) {
        if (ts.tasks) {
            atomicAdd(&w.ctl->task_ns, ts.exec_ns);
            atomicAdd(&w.ctl->wait_ns, ts.wait_ns);
            atomicAdd(&w.ctl->tasks, ts.tasks);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) w.ctl->t_phase[0] = global_ns() - k0;
    }
}
#endif

// ================================================================ batched worlds
// Thousands of independent worlds: one block per world, the world's Δv in
// shared memory, colours swept with __syncthreads. A world's manifolds are
// bucketed by colour; two manifolds of one colour share no dynamic body, so
// every body sees its updates in the same colour order as in the dataflow
// kernels (and in the oracle's colour order), and the results are identical.

__device__ __forceinline__ uint32_t manifold_world(const World& w, uint32_t m) {
    int b = w.s.sm_b1[m];
    if (b < 0) b = w.s.sm_b2[m];
    return b < 0 ? 0xffffffffu : w.b.world[b];
}

// Bucket of manifold m, or UINT32_MAX (with the error flag set) when its world
// or colour is out of range.
__device__ __forceinline__ uint32_t world_bucket(const World& w, uint32_t m, uint32_t n_worlds) {
    uint32_t wd = manifold_world(w, m), col = w.s.sm_colour[m];
    if (wd >= n_worlds || col >= (uint32_t)kMaxColours) {
        atomicOr(&w.ctl->err, ERRF_WORLD_RANGE);
        return 0xffffffffu;
    }
    return wd * kMaxColours + col;
}

#if !NPGPU_EXCHANGE_TU
__global__ void k_world_count(World w, uint32_t n_worlds) {
    const uint32_t ms = w.ctl->nsolver;
    GRID_FOR(m, ms) {
        uint32_t bucket = world_bucket(w, m, n_worlds);
        if (bucket != 0xffffffffu) atomicAdd(&w.s.bucket_count[bucket], 1u);
    }
}
#endif

#if !NPGPU_EXCHANGE_TU
__global__ void k_world_scatter(World w, uint32_t n_worlds) {
    const uint32_t ms = w.ctl->nsolver;
    GRID_FOR(m, ms) {
        uint32_t bucket = world_bucket(w, m, n_worlds);
        if (bucket == 0xffffffffu) continue;
        w.s.wm_order[w.s.bucket_start[bucket] + atomicAdd(&w.s.bucket_cursor[bucket], 1u)] = m;
    }
}
#endif

// Renumbers the solver manifolds in (world, colour) order: manifold i of the
// new numbering is wm_order[i] of the old. Gathered into the scratch arrays
// first, then copied back; assembly and everything after it use the new
// numbering, so a colour of a world is one run of indices.
#if !NPGPU_EXCHANGE_TU
__global__ void k_world_permute(World w, uint32_t n_worlds) {
    const uint32_t ms = w.ctl->nsolver, total = w.s.bucket_start[n_worlds * kMaxColours];
    const size_t P = w.cap_pairs;
    uint32_t* t = w.s.perm;
    GRID_FOR(i, ms) {
        const uint32_t m = i < total ? w.s.wm_order[i] : i;
        t[i] = w.s.sm_list[m];
        t[P + i] = (uint32_t)w.s.sm_b1[m];
        t[2 * P + i] = (uint32_t)w.s.sm_b2[m];
        t[3 * P + i] = w.s.sm_nc[m];
        t[4 * P + i] = w.s.sm_colour[m];
    }
}
#endif

#if !NPGPU_EXCHANGE_TU
__global__ void k_world_permute_back(World w) {
    const uint32_t ms = w.ctl->nsolver;
    const size_t P = w.cap_pairs;
    const uint32_t* t = w.s.perm;
    GRID_FOR(i, ms) {
        w.s.sm_list[i] = t[i];
        w.s.sm_b1[i] = (int)t[P + i];
        w.s.sm_b2[i] = (int)t[2 * P + i];
        w.s.sm_nc[i] = t[3 * P + i];
        w.s.sm_colour[i] = t[4 * P + i];
    }
}
#endif

// World-local index of body slot b (-1 stays -1). A body outside the world's
// slot range flags an error and the task is skipped.
__device__ __forceinline__ bool world_locals(const World& w, uint32_t m, uint32_t base, uint32_t nbw, int& l1, int& l2) {
    int b1 = w.s.sm_b1[m], b2 = w.s.sm_b2[m];
    l1 = b1 < 0 ? -1 : b1 - (int)base;
    l2 = b2 < 0 ? -1 : b2 - (int)base;
    if ((b1 >= 0 && (uint32_t)l1 >= nbw) || (b2 >= 0 && (uint32_t)l2 >= nbw)) {
        atomicOr(&w.ctl->err, ERRF_WORLD_RANGE);
        return false;
    }
    return true;
}

// A world is processed by a group of threads: a thread-block cluster (the
// widest worlds), a whole block (large worlds) or one warp (small worlds,
// several per block). `lane` and `width` place the thread in its group; the
// group's barrier orders the colours.
enum : uint32_t { GROUP_BLOCK = 0, GROUP_WARP = 1, GROUP_CLUSTER = 2 };
struct WorldGroup {
    uint32_t lane, width;
    uint32_t kind;
    __device__ __forceinline__ bool warp() const { return kind == GROUP_WARP; }
    __device__ __forceinline__ void sync() const {
        if (kind == GROUP_WARP) __syncwarp();
        else if (kind == GROUP_CLUSTER) cg::this_cluster().sync();
        else __syncthreads();
    }
    // The thread that adds this block's (or warp's) partial sums.
    __device__ __forceinline__ bool leader() const { return kind == GROUP_WARP ? lane == 0 : threadIdx.x == 0; }
};

// One sweep (warm start, friction or normal rows) over a world's manifolds,
// colour by colour.
template <int KIND, bool JOINTS, class DvA>
__device__ __forceinline__ void world_sweep(const World& w, uint32_t wd, uint32_t base, uint32_t nbw, uint32_t ncol,
                                            uint32_t sweep, const DvA& dva, const WorldGroup& g) {
    const uint32_t* bs = w.s.bucket_start + wd * kMaxColours;
    for (uint32_t c = 0; c < ncol; ++c) {
        uint32_t lo = bs[c], hi = bs[c + 1];
        if (lo == hi) continue;
        for (uint32_t m = lo + g.lane; m < hi; m += g.width) {
            int l1, l2;
            if (world_locals(w, m, base, nbw, l1, l2))
                velocity_task<KIND, JOINTS>(w, m, sweep, w.s.sm_b1[m], w.s.sm_b2[m], l1, l2, dva);
        }
        g.sync();
    }
}

// FP64 residual partial sums of one world, added to acc[0..1].
template <bool JOINTS, class DvA>
__device__ __forceinline__ void world_residual(const World& w, uint32_t wd, uint32_t base, uint32_t nbw,
                                               const DvA& dva, double* sh, double* acc, const WorldGroup& g) {
    uint32_t lo = w.s.bucket_start[wd * kMaxColours], hi = w.s.bucket_start[wd * kMaxColours + kMaxColours];
    ResidualSums rs;
    for (uint32_t m = lo + g.lane; m < hi; m += g.width) {
        int b1, b2;
        if (!world_locals(w, m, base, nbw, b1, b2)) continue;
        DV dv;
        dva.load(b1, dv.a);
        dva.load(b2, dv.b);
        manifold_residual<JOINTS>(w, m, w.s.sm_b1[m], w.s.sm_b2[m], dv, rs);
    }
    double s2 = rs.phi2(), l2 = rs.lam2();
    double ts, tl;
    if (g.warp()) {
        for (int o = 16; o > 0; o >>= 1) {
            s2 += __shfl_down_sync(0xffffffffu, s2, o);
            l2 += __shfl_down_sync(0xffffffffu, l2, o);
        }
        ts = s2;
        tl = l2;
    } else {
        ts = block_sum(s2, sh);
        tl = block_sum(l2, sh);
    }
    if (g.leader() && (ts != 0.0 || tl != 0.0)) {
        atomicAdd(&acc[0], ts);
        atomicAdd(&acc[1], tl);
    }
}

// The sweeps and residuals of one world's velocity solve by one group.
template <bool JOINTS, class DvA>
__device__ __forceinline__ void world_solve(const World& w, const StepParams& p, uint32_t wd, uint32_t base,
                                            uint32_t nbw, uint32_t ncol, const DvA& dva, double* sh,
                                            const WorldGroup& g) {
    world_sweep<SWEEP_WARM, JOINTS>(w, wd, base, nbw, ncol, 0, dva, g);
    world_residual<JOINTS>(w, wd, base, nbw, dva, sh, w.ctl->res_acc_init, g);
    for (uint32_t it = 0; it < p.max_velocity_iterations; ++it) {
        if (p.sweep_order == NPGPU_SWEEP_MANIFOLD) {
            world_sweep<SWEEP_MANIFOLD, JOINTS>(w, wd, base, nbw, ncol, 1 + it, dva, g);
        } else {
            world_sweep<SWEEP_FRICTION, JOINTS>(w, wd, base, nbw, ncol, 1 + 2 * it, dva, g);
            world_sweep<SWEEP_NORMAL, JOINTS>(w, wd, base, nbw, ncol, 2 + 2 * it, dva, g);
        }
    }
    world_residual<JOINTS>(w, wd, base, nbw, dva, sh, w.ctl->res_acc, g);
}

// The whole velocity solve of one world by one group, its Δv in s_dv.
template <bool JOINTS>
__device__ __forceinline__ void world_velocity(const World& w, const StepParams& p, uint32_t wd, uint32_t max_bodies,
                                               float* s_dv, double* sh, const WorldGroup& g) {
    const uint32_t base = w.s.world_start[wd];
    uint32_t nbw = w.s.world_start[wd + 1] - base;
    if (nbw > max_bodies) {
        if (g.lane == 0) atomicOr(&w.ctl->err, ERRF_WORLD_RANGE);
        nbw = 0;
    }
    const uint32_t ncol = w.ctl->ncolours;
    for (uint32_t i = g.lane; i < 6 * nbw; i += g.width) s_dv[i] = 0.0f;
    g.sync();
    world_solve<JOINTS>(w, p, wd, base, nbw, ncol, SharedDv{s_dv}, sh, g);
    for (uint32_t i = g.lane; i < 6 * nbw; i += g.width) w.b.dv[6 * base + i] = s_dv[i];
    g.sync();
}

// Persistent. Blocks first take the n_big large worlds from a counter,
// largest first, one world per block; when none is left each warp takes
// small worlds (at most kWarpWorldBodies body slots) from a second counter.
// The first n_cluster worlds of the order are the cluster kernel's.
// Dynamic shared memory: the larger of 6 floats per body slot of the largest
// world and 6 floats per slot of a small world for each warp.
#if !NPGPU_EXCHANGE_TU
template <int THREADS, bool JOINTS>
__global__ void __launch_bounds__(THREADS, 384 / THREADS) k_world_velocity(World w, StepParams p, uint32_t n_worlds,
                                                                  uint32_t max_world_bodies, uint32_t n_big,
                                                                  uint32_t n_cluster) {
    extern __shared__ float s_dv[];
    __shared__ double sh[32];
    __shared__ uint32_t s_world;
    if (w.ctl->err & ERRF_COLOURS) return;   // no consistent colour order to sweep
    const WorldGroup block{threadIdx.x, blockDim.x, GROUP_BLOCK};
    const uint32_t* order = w.s.world_order + n_cluster;
    for (;;) {
        if (threadIdx.x == 0) {
            uint32_t k = atomicAdd(&w.ctl->world_next[0], 1u);
            s_world = k < n_big ? order[k] : 0xffffffffu;
        }
        __syncthreads();
        const uint32_t wd = s_world;
        __syncthreads();
        if (wd >= n_worlds) break;
        world_velocity<JOINTS>(w, p, wd, max_world_bodies, s_dv, sh, block);
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const WorldGroup wg{lane, 32u, GROUP_WARP};
    float* my_dv = s_dv + (size_t)warp * 6 * kWarpWorldBodies;
    for (;;) {
        uint32_t k = 0;
        if (lane == 0) k = atomicAdd(&w.ctl->world_next[2], 1u);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (n_cluster + n_big + k >= n_worlds) break;
        world_velocity<JOINTS>(w, p, order[n_big + k], kWarpWorldBodies, my_dv, nullptr, wg);
    }
}
#endif

// The widest worlds, one thread-block cluster each (cluster c takes world
// order[c]): the world's Δv rows are spread over the cluster's shared
// memories, 2^shift bodies per block, and the cluster barrier orders the
// colours. Each block writes its own rows back to global memory.
#if NPGPU_EXCHANGE_TU
template <int THREADS, bool JOINTS>
__global__ void __launch_bounds__(THREADS, 1) k_cluster_velocity(World w, StepParams p, uint32_t shift) {
    extern __shared__ float s_dv[];
    __shared__ double sh[32];
    if (w.ctl->err & ERRF_COLOURS) return;   // every block of every cluster leaves together
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t nct = cl.num_blocks(), rank = cl.block_rank();
    const uint32_t wd = w.s.world_order[blockIdx.x / nct];
    const uint32_t base = w.s.world_start[wd];
    uint32_t nbw = w.s.world_start[wd + 1] - base;
    if (nbw > (nct << shift)) {
        if (threadIdx.x == 0) atomicOr(&w.ctl->err, ERRF_WORLD_RANGE);
        nbw = 0;
    }
    for (uint32_t i = threadIdx.x; i < (6u << shift); i += blockDim.x) s_dv[i] = 0.0f;
    cl.sync();
    const WorldGroup g{rank * blockDim.x + threadIdx.x, nct * blockDim.x, GROUP_CLUSTER};
    world_solve<JOINTS>(w, p, wd, base, nbw, w.ctl->ncolours, ClusterDv{s_dv, shift}, sh, g);
    const uint32_t lo = rank << shift, hi = nbw < lo + (1u << shift) ? nbw : lo + (1u << shift);
    for (uint32_t i = threadIdx.x; lo + i / 6u < hi && i < (6u << shift); i += blockDim.x)
        w.b.dv[6 * (size_t)(base + lo) + i] = s_dv[i];
    // No block leaves while another may still read its shared memory.
    cl.sync();
}
#endif

#if !NPGPU_EXCHANGE_TU
__global__ void k_world_finish(World w, StepParams p) {
    Control* c = w.ctl;
    c->residual_initial = sqrt(c->res_acc_init[0]) / fmax(1.0, sqrt(c->res_acc_init[1]));
    c->residual = sqrt(c->res_acc[0]) / fmax(1.0, sqrt(c->res_acc[1]));
    c->res_acc[0] = c->res_acc[1] = 0.0;
    c->iterations = p.max_velocity_iterations;
}
#endif

// A body pose as the position solver moves it.
struct Pose {
    np::V t, com;
    np::Q q;
};

__device__ __forceinline__ Pose load_pose(const Bodies& b, uint32_t i) {
    return Pose{v3(b.pos_t[i]), v3(b.com[i]), q4(b.pos_q[i])};
}
__device__ __forceinline__ void store_pose(const Bodies& b, uint32_t i, const Pose& P) {
    b.pos_t[i] = f4(P.t);
    b.pos_q[i] = f4q(P.q);
    b.com[i] = f4(P.com);
    atomicOr(&b.info[i], BI_CHANGED);
}

// Flagged poses of the dataflow position solver: per body 12 words of 64 bits
// (10 used: translation, centre of mass, rotation), each = update count << 32
// | float bits, the same protocol as the flagged Δv; word 10 holds the moved
// flag in its float bits.
__device__ __forceinline__ bool poll_posef(const unsigned long long* pf, int b, uint32_t t, Pose& P, bool& moved) {
    const unsigned long long* p = pf + 12 * (size_t)b;
    unsigned long long w[12];
#pragma unroll
    for (int k = 0; k < 6; ++k)
        asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(w[2 * k]), "=l"(w[2 * k + 1]) : "l"(p + 2 * k)
                     : "memory");
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 11; ++k) ok = ok && (uint32_t)(w[k] >> 32) == t;
    float f[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) f[k] = __uint_as_float((uint32_t)w[k]);
    P.t = np::mk(f[0], f[1], f[2]);
    P.com = np::mk(f[3], f[4], f[5]);
    P.q = np::Q{f[6], f[7], f[8], f[9]};
    moved = (uint32_t)w[10] != 0u;
    return ok;
}
__device__ __forceinline__ void publish_posef(unsigned long long* pf, int b, uint32_t t, const Pose& P, bool moved) {
    unsigned long long* p = pf + 12 * (size_t)b;
    const unsigned long long hi = (unsigned long long)t << 32;
    const float f[10] = {P.t.x, P.t.y, P.t.z, P.com.x, P.com.y, P.com.z, P.q.i, P.q.j, P.q.k, P.q.w};
    unsigned long long w[12];
#pragma unroll
    for (int k = 0; k < 10; ++k) w[k] = hi | __float_as_uint(f[k]);
    w[10] = hi | (moved ? 1u : 0u);
    w[11] = 0ull;
#pragma unroll
    for (int k = 0; k < 6; ++k)
        asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p + 2 * k), "l"(w[2 * k]), "l"(w[2 * k + 1])
                     : "memory");
}

// JointConstraint::cache_impulses' break test of each kind, in its own
// arithmetic: |linear|^2 / dt^2 against the squared break force, |angular|^2
// / dt^2 against the squared break torque (ball_constraint.rs:129-141,
// fixed_constraint.rs:174-199, revolute_constraint.rs:268-292,
// cartesian_constraint.rs, planar_constraint.rs, rectangular_constraint.rs,
// universal_constraint.rs).
__device__ __forceinline__ bool joint_breaks(uint32_t kind, float4 l, float4 a, float2 brk, float inv_dt) {
    const float l2 = 0.0f + l.x * l.x + l.y * l.y + l.z * l.z;
    const float a2 = 0.0f + a.x * a.x + a.y * a.y + a.z * a.z;
    const float inv_dt2 = inv_dt * inv_dt;
    switch (kind) {
    case NPGPU_JOINT_BALL: return l2 * inv_dt * inv_dt > brk.x;
    case NPGPU_JOINT_CARTESIAN: return a2 * inv_dt * inv_dt > brk.y;
    case NPGPU_JOINT_PLANAR:
        return l.x * l.x * inv_dt2 > brk.x || a.x * a.x * inv_dt2 + a.y * a.y * inv_dt2 > brk.y;
    case NPGPU_JOINT_RECTANGULAR: return l.x * l.x * inv_dt2 > brk.x || a2 * inv_dt2 > brk.y;
    case NPGPU_JOINT_UNIVERSAL: return l2 * inv_dt2 > brk.x || a.x * a.x * inv_dt2 > brk.y;
    default: return l2 * inv_dt2 > brk.x || a2 * inv_dt2 > brk.y;   // fixed, revolute
    }
}

// ================================================================ integrate
#if !NPGPU_EXCHANGE_TU
__global__ void k_cache_integrate(World w, StepParams p, bool posef) {
    const uint32_t ms = w.ctl->nsolver;
    const Bodies& b = w.b;
    GRID_FOR(m, ms) {
        uint32_t q = w.s.sm_list[m];
        uint32_t nc = w.s.sm_nc[m];
        if (q & kJointBit) {
            // JointConstraint::cache_impulses (ball_constraint.rs:129-141,
            // fixed_constraint.rs:174-199): the impulses, and the joint breaks
            // when |impulse|^2 / dt^2 exceeds the squared break force / torque.
            const uint32_t j = q & ~kJointBit;
            const float4 i0 = w.j.imp[2 * j], i1 = w.j.imp[2 * j + 1];
            float iv[7] = {i0.x, i0.y, i0.z, i1.x, i1.y, i1.z, i0.w};
            const uint32_t kind = w.j.info[j] & JI_KIND_MASK;
            for (uint32_t k = 0; k < nc; ++k) {
                const uint32_t rows = joint_rows_of(w.s.con[((size_t)m * kMaxContacts + k) * 4].w);
                const float4 l4 = w.s.lam[(size_t)m * kMaxContacts + k];
                const float l[3] = {l4.x, l4.y, l4.z};
                for (uint32_t r = 0; r < rows; ++r) iv[joint_slot(kind, k, r, true)] = l[r];
            }
            const float4 imp[2] = {make_float4(iv[0], iv[1], iv[2], iv[6]), make_float4(iv[3], iv[4], iv[5], 0.0f)};
            w.j.imp[2 * j] = imp[0];
            w.j.imp[2 * j + 1] = imp[1];
            if (joint_breaks(kind, imp[0], imp[1], w.j.brk[j], p.inv_dt))
                w.j.state[j] |= JS_BROKEN;
            continue;
        }
        for (uint32_t k = 0; k < nc; ++k) {
            float4 l = w.s.lam[(size_t)m * kMaxContacts + k];
            if (w.s.feat != nullptr) {
                // Training sample: the contact's features and converged impulses.
                uint32_t at = atomicAdd(&w.ctl->mlp_samples, 1u);
                if (at < w.s.sample_cap) {
                    float* so = w.s.samples + (size_t)at * kMlpSampleFloats;
                    const float* fi = w.s.feat + ((size_t)m * kMaxContacts + k) * kMlpIn;
                    for (int i = 0; i < kMlpIn; ++i) so[i] = fi[i];
                    so[kMlpIn] = l.x;
                    so[kMlpIn + 1] = l.y;
                    so[kMlpIn + 2] = l.z;
                    so[kMlpIn + 3] = w.cur.imp[q * kMaxContacts + k].w == 0.0f ? 1.0f : 0.0f;
                }
            }
            w.cur.imp[q * kMaxContacts + k] = l;
        }
    }
    const float dt = p.dt;
    GRID_FOR(i, w.nb_slots) {
        uint32_t info = b.info[i];
        if (!(info & BI_ISLAND)) continue;
        np::V el = np::mul(v3(b.acc_lin[i]), dt), ea = np::mul(v3(b.acc_ang[i]), dt);
        const float* d = b.dv + 6 * i;
        np::V lin = np::add(np::add(v3(b.lin[i]), el), np::mk(d[0], d[1], d[2]));
        np::V ang = np::add(np::add(v3(b.ang[i]), ea), np::mk(d[3], d[4], d[5]));
        b.lin[i] = f4(lin);
        b.ang[i] = f4(ang);
        b.info[i] = info | BI_CHANGED;
        body_integrate(b, i, dt);
        if (posef) publish_posef(b.posef, (int)i, 0u, load_pose(b, i), false);
    }
}
#endif

// ================================================================ NonlinearSORProx
// NonlinearSORProx::solve_unilateral for the contacts of manifold m
// (nonlinear_sor_prox.rs:121-154), on the two bodies' poses P1, P2 (the
// poses of sides without dofs are not changed). moved1 / moved2 report a
// displacement.
// What a position task of manifold m reads besides the poses, gathered by
// assembly into one record (kPosRec float4) so that a task waits for memory
// once rather than through the pair -> collider -> body chain:
//   0 (wrt1.t, dil1)  1 wrt1.q  2 (wrt2.t, dil2)  3 wrt2.q
//   4 (half extents 1, shape1 | nc << 8)  5 (half extents 2, shape2)
//   6 (body1, body2, info1, info2)  7..10 per contact (normal in body 1's frame, feature key)
// NonlinearSORProx::solve_generic (nonlinear_sor_prox.rs:78-117) of one
// position row whose sides J1/W1, J2/W2 and 1/r were formed by
// constraint_pair_geometry: clamp_rhs (nonlinear_sor_prox.rs:297-309), then
// each side with dofs moves by its W times -rhs r.
__device__ __forceinline__ void generic_position_row(const StepParams& p, float depth, bool angular, float inv_r, bool d1,
                                                     bool d2, float* W1, float* W2, np::V& t1, np::Q& q1, np::V& com1,
                                                     np::V lc1, np::V& t2, np::Q& q2, np::V& com2, np::V lc2,
                                                     bool& moved1, bool& moved2) {
    float rhs = -depth;
    if (angular) {
        rhs = (rhs + p.allowed_angular_error) * p.erp;
        rhs = rhs < -p.max_angular_correction ? -p.max_angular_correction : rhs;
    } else {
        rhs = (rhs + p.allowed_linear_error) * p.erp;
        rhs = rhs < -p.max_linear_correction ? -p.max_linear_correction : rhs;
    }
    if (!(rhs < 0.0f)) return;
    const float r = inv_r != 0.0f ? 1.0f / inv_r : 1.0f;
    const float impulse = -rhs * r;
    if (d1) {
        for (int k = 0; k < 6; ++k) W1[k] = W1[k] * impulse;
        apply_displacement(t1, q1, com1, lc1, np::mk(W1[0], W1[1], W1[2]), np::mk(W1[3], W1[4], W1[5]));
        moved1 = true;
    }
    if (d2) {
        for (int k = 0; k < 6; ++k) W2[k] = W2[k] * impulse;
        apply_displacement(t2, q2, com2, lc2, np::mk(W2[0], W2[1], W2[2]), np::mk(W2[3], W2[4], W2[5]));
        moved2 = true;
    }
}

// UnitQuaternion::rotation_between_axis(a, b) followed by scaled_axis
// (helper.rs:701-769): the unit axis of a x b times acos(a . b), zero when
// the axes coincide; false when they are opposite (the callers then take a
// rotation by pi). The angle is the axis-angle form's directly, without the
// quaternion in between.
__device__ __forceinline__ bool rotation_between_scaled(np::V a, np::V b, np::V& out) {
    np::V ax;
    float n;
    const np::V zero = np::mk(0.0f, 0.0f, 0.0f);
    if (unit_try(np::cross(a, b), FLT_EPSILON, ax, n)) {
        const float c = np::dot(a, b);
        if (c <= -1.0f) return false;
        if (c >= 1.0f) {
            out = zero;
            return true;
        }
        out = np::mul(ax, (float)acos((double)c));
        return true;
    }
    if (np::dot(a, b) < 0.0f) return false;
    out = zero;
    return true;
}

// The separation of two axes as a scaled axis; for opposite axes, a rotation
// by pi about the cross product of axis1 with the canonical axis of its
// smallest component (helper.rs:717-724).
__device__ __forceinline__ np::V axis_separation(np::V a1, np::V a2) {
    np::V e;
    if (rotation_between_scaled(a1, a2, e)) return e;
    const float c[3] = {fabsf(a1.x), fabsf(a1.y), fabsf(a1.z)};
    int imin = 0;
    if (c[1] < c[imin]) imin = 1;
    if (c[2] < c[imin]) imin = 2;
    const np::V o = np::cross(basis_axis(imin), a1);
    return np::mul(np::divs(o, np::norm(o)), 3.14159265358979f);
}

// Which position constraints a joint kind generates, in order (each
// constraint's position_constraint(i), with the poses its predecessors left):
// T the anchors' separation (cancel_relative_translation), TA the separation
// along body 1's axis (cancel_relative_translation_wrt_axis), R the frames'
// relative rotation (cancel_relative_rotation), AL the axes' alignment
// (align_axis), RA the angle between the axes (restore_angle_between_axis).
// PA the anchor's distance from the axis line (project_anchor_to_axis), AL3
// the alignment of axis3 with axis2, LIM the prismatic offset limits
// (unit_constraint.rs:125-198).
enum { JP_T = 1, JP_TA = 2, JP_R_FRAMES = 3, JP_R_BODIES = 4, JP_AL = 5, JP_RA = 6, JP_PA = 7, JP_AL3 = 8, JP_LIM = 9 };
__device__ __forceinline__ void joint_position_ops(uint32_t kind, uint32_t info, int* op) {
    op[0] = op[1] = op[2] = 0;
    switch (kind) {
    case NPGPU_JOINT_BALL: op[0] = JP_T; break;
    case NPGPU_JOINT_FIXED: op[0] = JP_R_FRAMES; op[1] = JP_T; break;
    case NPGPU_JOINT_REVOLUTE: op[0] = JP_T; op[1] = JP_AL; break;
    case NPGPU_JOINT_CARTESIAN: op[0] = JP_R_FRAMES; break;
    case NPGPU_JOINT_PLANAR: op[0] = JP_TA; op[1] = JP_AL; break;
    case NPGPU_JOINT_RECTANGULAR: op[0] = JP_TA; op[1] = JP_R_BODIES; break;
    case NPGPU_JOINT_UNIVERSAL: op[0] = JP_T; op[1] = JP_RA; break;
    case NPGPU_JOINT_PRISMATIC:
        op[0] = JP_PA;
        op[1] = JP_R_BODIES;
        if (info & (JI_MIN_OFFSET | JI_MAX_OFFSET)) op[2] = JP_LIM;
        break;
    case NPGPU_JOINT_CYLINDRICAL: op[0] = JP_AL; op[1] = JP_PA; break;
    default: op[0] = JP_AL3; op[1] = JP_PA; break;   // pin-slot
    }
}

// The position constraints of joint j on the poses P1, P2
// (NonlinearSORProx::solve_generator, nonlinear_sor_prox.rs:57-76), each
// through helper.rs's position helpers (helper.rs:298-418, 553-611, 701-769,
// 921-998) and solve_generic. An error below the allowed one is skipped
// (Unit::try_new_and_get). Out of line, everything passed and returned by
// value, so that the contact tasks keep their registers.
struct JointPoses {
    Pose P1, P2;
    bool moved1, moved2;
};
static __device__ __noinline__ JointPoses joint_position(const Joints J, const float4* local_com, const float4* sb,
                                                         const StepParams p, uint32_t j, uint32_t bb1, uint32_t bb2,
                                                         uint32_t i1, uint32_t i2, Pose P1, Pose P2) {
    bool moved1 = false, moved2 = false;
    const bool d1 = bi_status(i1) == 2u, d2 = bi_status(i2) == 2u;
    np::V t1 = P1.t, t2 = P2.t;
    np::Q q1 = P1.q, q2 = P2.q;
    np::V com1 = P1.com, com2 = P2.com;
    np::V lc1 = np::mk(0.0f, 0.0f, 0.0f), lc2 = lc1;
    BodyView v1, v2;
    v1.lin = v1.ang = v1.acc_lin = v1.acc_ang = lc1;
    v2.lin = v2.ang = v2.acc_lin = v2.acc_ang = lc1;
    v1.inv_mass = v2.inv_mass = 0.0f;
    v1.info = i1;
    v2.info = i2;
    if (d1) {
        lc1 = v3(__ldg(local_com + bb1));
        const SB s = load_sb(sb, (int)bb1);
        v1.inv_mass = s.im;
        v1.inv_I = s.I;
    }
    if (d2) {
        lc2 = v3(__ldg(local_com + bb2));
        const SB s = load_sb(sb, (int)bb2);
        v2.inv_mass = s.im;
        v2.inv_I = s.I;
    }
    const uint32_t info = J.info[j], kind = info & JI_KIND_MASK;
    const np::V la1 = v3(J.anchor[2 * j]), la2 = v3(J.anchor[2 * j + 1]);
    const float4 ax1 = J.axis[3 * j], ax2 = J.axis[3 * j + 1], ax3 = J.axis[3 * j + 2];
    int ops[3];
    joint_position_ops(kind, info, ops);
    float J1[6], J2[6], W1[6], W2[6];
    for (int o = 0; o < 3 && ops[o] != 0; ++o) {
        const int op = ops[o];
        const np::V a1 = body_point(t1, q1, la1), a2 = body_point(t2, q2, la2);
        bool angular = false, have = false;
        np::V dir;
        float depth = 0.0f;
        if (op == JP_T) {
            have = unit_try(np::sub(a2, a1), p.allowed_linear_error, dir, depth);
        } else if (op == JP_TA) {
            const np::V ax = np::qrot(q1, v3(ax1));
            depth = np::dot(ax, np::sub(a2, a1));
            dir = ax;
            if (depth < 0.0f) {
                depth = -depth;
                dir = np::neg(ax);
            }
            have = depth > p.allowed_linear_error;
        } else if (op == JP_R_FRAMES || op == JP_R_BODIES) {
            np::Q r1 = q1, r2 = q2;
            if (op == JP_R_FRAMES) {
                r1 = np::qmul(q1, q4(J.frame[2 * j]));
                r2 = np::qmul(q2, q4(J.frame[2 * j + 1]));
            }
            angular = true;
            have = unit_try(np::qscaled_axis(np::qmul(r2, np::qconj(r1))), p.allowed_angular_error, dir, depth);
        } else if (op == JP_AL || op == JP_AL3) {
            angular = true;
            const np::V e = axis_separation(np::qrot(q1, v3(op == JP_AL ? ax1 : ax3)), np::qrot(q2, v3(ax2)));
            have = unit_try(e, p.allowed_angular_error, dir, depth);
        } else if (op == JP_PA) {
            const np::V ax = np::qrot(q1, v3(ax1));
            const np::V proj = np::add(a1, np::mul(ax, np::dot(ax, np::sub(a2, a1))));
            have = unit_try(np::sub(a2, proj), p.allowed_linear_error, dir, depth);
        } else if (op == JP_LIM) {
            const np::V ax = np::qrot(q1, v3(ax1));
            const float offset = np::dot(ax, np::sub(a2, a1));
            depth = 0.0f;
            dir = ax;
            if (info & JI_MIN_OFFSET) {
                depth = ax2.w - offset;
                dir = np::neg(ax);
            }
            if (depth < 0.0f && (info & JI_MAX_OFFSET)) {
                depth = offset - ax3.w;
                dir = ax;
            }
            have = depth > p.allowed_linear_error;
        } else {   // JP_RA
            angular = true;
            float cur;
            const np::V e = axis_separation(np::qrot(q1, v3(ax1)), np::qrot(q2, v3(ax2)));
            if (unit_try(e, FLT_EPSILON, dir, cur)) {
                depth = cur - ax1.w;
                if (depth < 0.0f) {
                    depth = -depth;
                    dir = np::neg(dir);
                }
                have = !(depth < p.allowed_angular_error);
            }
        }
        if (!have) continue;
        float inv_r = 0.0f, dummy = 0.0f;
        v1.com = com1;
        v2.com = com2;
        if (angular) {
            if (d1) fill_torque_side(v1, dir, J1, W1, inv_r, dummy, false, p.dt);
            if (d2) fill_torque_side(v2, np::neg(dir), J2, W2, inv_r, dummy, false, p.dt);
        } else {
            if (d1) fill_row_side(v1, a1, dir, J1, W1, inv_r, dummy, false, p.dt);
            if (d2) fill_row_side(v2, a2, np::neg(dir), J2, W2, inv_r, dummy, false, p.dt);
        }
        generic_position_row(p, depth, angular, inv_r, d1, d2, W1, W2, t1, q1, com1, lc1, t2, q2, com2, lc2, moved1,
                             moved2);
    }
    P1.t = t1; P1.q = q1; P1.com = com1;
    P2.t = t2; P2.q = q2; P2.com = com2;
    return JointPoses{P1, P2, moved1, moved2};
}

template <bool JOINTS>
__device__ __forceinline__ void position_core(const World& w, const StepParams& p, uint32_t m, Pose& P1, Pose& P2,
                                              bool& moved1, bool& moved2) {
    const Bodies& b = w.b;
    const float4* rec = w.s.pos_rec + (size_t)m * kPosRec;
    const float4 r0 = __ldg(rec), r1 = __ldg(rec + 1), r2 = __ldg(rec + 2), r3 = __ldg(rec + 3);
    const float4 r4 = __ldg(rec + 4), r5 = __ldg(rec + 5), r6 = __ldg(rec + 6);
    const uint32_t bb1 = __float_as_uint(r6.x), bb2 = __float_as_uint(r6.y);
    const uint32_t i1 = __float_as_uint(r6.z), i2 = __float_as_uint(r6.w);
    if (JOINTS && (__float_as_uint(r4.w) & kJointBit)) {
        const JointPoses o =
            joint_position(w.j, b.local_com, b.sb, p, __float_as_uint(r4.w) & ~kJointBit, bb1, bb2, i1, i2, P1, P2);
        P1 = o.P1;
        P2 = o.P2;
        moved1 = o.moved1;
        moved2 = o.moved2;
        return;
    }
    bool d1 = bi_status(i1) == 2u, d2 = bi_status(i2) == 2u;
    np::V t1 = P1.t, t2 = P2.t;
    np::Q q1 = P1.q, q2 = P2.q;
    np::V com1 = P1.com, com2 = P2.com;
    np::V lc1 = np::mk(0.0f, 0.0f, 0.0f), lc2 = lc1;
    SB s1, s2;
    s1.im = s2.im = 0.0f;
    if (d1) {
        lc1 = v3(__ldg(b.local_com + bb1));
        s1 = load_sb(b.sb, (int)bb1);
    }
    if (d2) {
        lc2 = v3(__ldg(b.local_com + bb2));
        s2 = load_sb(b.sb, (int)bb2);
    }
    const float im1 = s1.im, im2 = s2.im;
    const np::M iI1 = s1.I, iI2 = s2.I;
    np::Iso wrt1{v3(r0), q4(r1)}, wrt2{v3(r2), q4(r3)};
    const uint32_t sh1 = __float_as_uint(r4.w) & 0xfu, sh2 = __float_as_uint(r5.w) & 0xfu;
    np::V hh1 = v3(r4), hh2 = v3(r5);
    const float dil1 = r0.w, dil2 = r2.w;
    const uint32_t nc = __float_as_uint(r4.w) >> 8;
    moved1 = moved2 = false;
    for (uint32_t k = 0; k < nc; ++k) {
        const float4 ck = __ldg(rec + 7 + k);
        uint32_t key = __float_as_uint(ck.w);
        int f1 = (int)(key / 26u), f2 = (int)(key % 26u);
        np::Iso m1 = np::iso_mul(np::Iso{t1, q1}, wrt1);
        np::Iso m2 = np::iso_mul(np::Iso{t2, q2}, wrt2);
        np::V n0 = np::qrot(m1.q, v3(ck));
        Geom g = kinematic_contact(feature_of(sh1, hh1, f1), m1, dil1, feature_of(sh2, hh2, f2), m2, dil2, n0);
        // NonlinearSORProx::clamp_rhs.
        float rhs = (-g.depth + p.allowed_linear_error) * p.erp;
        float lim = -p.max_linear_correction;
        rhs = (rhs < lim) ? lim : rhs;
        if (rhs >= 0.0f) continue;
        float inv_r = 0.0f, dummy = 0.0f;
        float J1[6], J2[6], W1[6], W2[6];
        if (d1) {
            BodyView v;
            v.com = com1; v.inv_mass = im1; v.inv_I = iI1; v.info = i1;
            v.lin = v.ang = v.acc_lin = v.acc_ang = np::mk(0.0f, 0.0f, 0.0f);
            fill_row_side(v, g.w1, np::neg(g.n), J1, W1, inv_r, dummy, false, p.dt);
        }
        if (d2) {
            BodyView v;
            v.com = com2; v.inv_mass = im2; v.inv_I = iI2; v.info = i2;
            v.lin = v.ang = v.acc_lin = v.acc_ang = np::mk(0.0f, 0.0f, 0.0f);
            fill_row_side(v, g.w2, g.n, J2, W2, inv_r, dummy, false, p.dt);
        }
        if (inv_r == 0.0f) continue;
        float r = 1.0f / inv_r;
        float impulse = -rhs * r;
        if (d1) {
            for (int kk = 0; kk < 6; ++kk) W1[kk] = W1[kk] * impulse;
            apply_displacement(t1, q1, com1, lc1, np::mk(W1[0], W1[1], W1[2]), np::mk(W1[3], W1[4], W1[5]));
            moved1 = true;
        }
        if (d2) {
            for (int kk = 0; kk < 6; ++kk) W2[kk] = W2[kk] * impulse;
            apply_displacement(t2, q2, com2, lc2, np::mk(W2[0], W2[1], W2[2]), np::mk(W2[3], W2[4], W2[5]));
            moved2 = true;
        }
    }
    P1.t = t1; P1.q = q1; P1.com = com1;
    P2.t = t2; P2.q = q2; P2.com = com2;
}

// Position task on poses in global memory (one block per world, where
// __syncthreads orders the tasks of successive colours).
template <bool JOINTS>
__device__ __forceinline__ void position_task(const World& w, const StepParams& p, uint32_t m) {
    const float4 r6 = __ldg(w.s.pos_rec + (size_t)m * kPosRec + 6);
    const uint32_t bb1 = __float_as_uint(r6.x), bb2 = __float_as_uint(r6.y);
    Pose P1 = load_pose(w.b, bb1), P2 = load_pose(w.b, bb2);
    bool moved1, moved2;
    position_core<JOINTS>(w, p, m, P1, P2, moved1, moved2);
    if (moved1) store_pose(w.b, bb1, P1);
    if (moved2) store_pose(w.b, bb2, P2);
}

#if NPGPU_EXCHANGE_TU
template <bool JOINTS>
__global__ void __launch_bounds__(kCoopThreads, 2) k_position(World w, StepParams p) {
    const uint32_t ms = w.ctl->nsolver;
    const uint32_t T = gridDim.x * blockDim.x;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if ((ms + T - 1) / T > (uint32_t)kMaxPerThread) {
        if (t == 0) atomicOr(&w.ctl->err, ERRF_TASKS);
        return;
    }
    if (w.ctl->err & ERRF_COLOURS) return;
    const uint32_t nsw = p.max_position_iterations;
    MyTasks mt;
    load_tasks(w, ms, mt, 0);
    uint32_t left = mt.n * nsw;
    unsigned long long t0 = 0;
    unsigned backoff = 32;
    while (__any_sync(0xffffffffu, left > 0)) {
        bool progress = false;
        for (uint32_t k = 0; k < mt.n; ++k) {
            uint32_t sw = mt.next[k];
            if (sw >= nsw) continue;
            int b1 = mt.b1[k], b2 = mt.b2[k];
            uint32_t rk = mt.rk[k];
            uint32_t t1 = sw * ((rk >> 8) & 0xffu) + (rk & 0xffu);
            uint32_t t2 = sw * (rk >> 24) + ((rk >> 16) & 0xffu);
            const uint32_t m = t + k * T;
            Pose P1, P2;
            bool mv1 = false, mv2 = false;
            bool r1 = true, r2 = true;
            if (b1 >= 0) r1 = poll_posef(w.b.posef, b1, t1, P1, mv1);
            if (b2 >= 0) r2 = poll_posef(w.b.posef, b2, t2, P2, mv2);
            if (!(r1 && r2)) continue;
            if (b1 < 0 || b2 < 0) {
                const float4 r6 = __ldg(w.s.pos_rec + (size_t)m * kPosRec + 6);
                if (b1 < 0) P1 = load_pose(w.b, __float_as_uint(r6.x));
                if (b2 < 0) P2 = load_pose(w.b, __float_as_uint(r6.y));
            }
            bool n1, n2;
            position_core<JOINTS>(w, p, m, P1, P2, n1, n2);
            if (b1 >= 0) publish_posef(w.b.posef, b1, t1 + 1u, P1, mv1 || n1);
            if (b2 >= 0) publish_posef(w.b.posef, b2, t2 + 1u, P2, mv2 || n2);
            mt.next[k] = (uint16_t)(sw + 1u);
            --left;
            progress = true;
        }
        if (__any_sync(0xffffffffu, progress)) {
            t0 = 0;
            backoff = 32;
        } else if (!warp_wait_backoff(w.ctl, t0, backoff)) {
            return;
        }
    }
}
#endif

// Batched worlds: block per world, colour by colour, poses in global memory.
// NonlinearSORProx sweeps of one world by one group, poses in global memory.
template <bool JOINTS>
__device__ __forceinline__ void world_position(const World& w, const StepParams& p, uint32_t wd, const WorldGroup& g) {
    const uint32_t ncol = w.ctl->ncolours;
    const uint32_t* bs = w.s.bucket_start + wd * kMaxColours;
    for (uint32_t it = 0; it < p.max_position_iterations; ++it) {
        for (uint32_t c = 0; c < ncol; ++c) {
            uint32_t lo = bs[c], hi = bs[c + 1];
            if (lo == hi) continue;
            for (uint32_t m = lo + g.lane; m < hi; m += g.width) position_task<JOINTS>(w, p, m);
            g.sync();
        }
    }
    g.sync();
}

// Batched worlds: large worlds one per block, then small worlds one per warp,
// as in the velocity kernel. Three blocks of 128 threads stay resident per SM
// (at most 170 registers a thread; the contacts' tasks need about 164).
#if !NPGPU_EXCHANGE_TU
template <int THREADS, bool JOINTS>
__global__ void __launch_bounds__(THREADS, 384 / THREADS) k_world_position(World w, StepParams p, uint32_t n_worlds, uint32_t n_big,
                                                            uint32_t n_cluster) {
    __shared__ uint32_t s_world;
    if (w.ctl->err & ERRF_COLOURS) return;
    const WorldGroup block{threadIdx.x, blockDim.x, GROUP_BLOCK};
    const uint32_t* order = w.s.world_order + n_cluster;
    for (;;) {
        if (threadIdx.x == 0) {
            uint32_t k = atomicAdd(&w.ctl->world_next[1], 1u);
            s_world = k < n_big ? order[k] : 0xffffffffu;
        }
        __syncthreads();
        const uint32_t wd = s_world;
        __syncthreads();
        if (wd >= n_worlds) break;
        world_position<JOINTS>(w, p, wd, block);
    }
    const uint32_t lane = threadIdx.x & 31u;
    const WorldGroup wg{lane, 32u, GROUP_WARP};
    for (;;) {
        uint32_t k = 0;
        if (lane == 0) k = atomicAdd(&w.ctl->world_next[3], 1u);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (n_cluster + n_big + k >= n_worlds) break;
        world_position<JOINTS>(w, p, order[n_big + k], wg);
    }
}
#endif

// The cluster worlds' position sweeps: cluster c takes world order[c], the
// cluster barrier between colours (poses stay in global memory).
#if NPGPU_EXCHANGE_TU
template <bool JOINTS>
__global__ void __launch_bounds__(kClusterThreads, 1) k_cluster_position(World w, StepParams p) {
    if (w.ctl->err & ERRF_COLOURS) return;
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t nct = cl.num_blocks();
    const WorldGroup g{cl.block_rank() * blockDim.x + threadIdx.x, nct * blockDim.x, GROUP_CLUSTER};
    world_position<JOINTS>(w, p, w.s.world_order[blockIdx.x / nct], g);
}
#endif

#if !NPGPU_EXCHANGE_TU
#include "k_ccd.cuh"
#endif

// ================================================================ post
#if !NPGPU_EXCHANGE_TU
__global__ void k_post(World w, StepParams p, bool posef) {
    __shared__ double sh[32];
    const Bodies& b = w.b;
    double ke = 0.0;
    GRID_FOR(i, w.nb_slots) {
        uint32_t info = b.info[i];
        if (!(info & BI_ALIVE)) continue;
        uint32_t st = bi_status(info);
        if (posef && st == 2u && (info & BI_ISLAND)) {
            // The dataflow position solver's result.
            Pose P;
            bool moved;
            poll_posef(b.posef, (int)i, 0u, P, moved);
            if (moved) {
                b.pos_t[i] = f4(P.t);
                b.pos_q[i] = f4q(P.q);
                b.com[i] = f4(P.com);
            }
        }
        if (st == 3u) {
            body_integrate(b, i, p.dt);
            info = b.info[i];
        }
        if ((info & BI_CHANGED) && st == 2u) body_update_dynamics(b, i, p.dt);
        b.f_lin[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        b.f_ang[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        // With CCD the update flags stay until its substeps have run, and the
        // energy audit is taken after them (k_ccd_finish).
        if (!p.ccd) b.info[i] = b.info[i] & ~BI_CHANGED;
        if (st == 2u) {
            float4 l = b.lin[i], a = b.ang[i], tt = b.pos_t[i];
            if (!(isfinite(l.x) && isfinite(l.y) && isfinite(l.z) && isfinite(a.x) && isfinite(a.y) && isfinite(a.z) &&
                  isfinite(tt.x) && isfinite(tt.y) && isfinite(tt.z)))
                atomicOr(&w.ctl->err, ERRF_NAN);
            if (p.ccd) continue;
            np::M I = load_m9(b.I + 9 * i);
            np::V av = v3(a);
            np::V iw = np::mv(I, av);
            double m = (double)b.mass[i];
            double v2 = (double)l.x * l.x + (double)l.y * l.y + (double)l.z * l.z;
            double wiw = (double)av.x * iw.x + (double)av.y * iw.y + (double)av.z * iw.z;
            ke += 0.5 * (m * v2 + wiw);
        }
    }
    double tke = block_sum(ke, sh);
    if (threadIdx.x == 0 && tke != 0.0) atomicAdd(&w.ctl->kinetic_energy, tke);
}
#endif

#if NPGPU_EXCHANGE_TU
const void* exchange_kernel(ExchangeKernel k, bool joints) {
    switch (k) {
    case XK_COLOUR: return (const void*)k_colour;
    case XK_VELOCITY: return joints ? (const void*)k_velocity<true> : (const void*)k_velocity<false>;
    case XK_POSITION: return joints ? (const void*)k_position<true> : (const void*)k_position<false>;
    case XK_CLUSTER_VELOCITY:
        return joints ? (const void*)k_cluster_velocity<kClusterThreads, true>
                      : (const void*)k_cluster_velocity<kClusterThreads, false>;
    case XK_CLUSTER_POSITION: return joints ? (const void*)k_cluster_position<true> : (const void*)k_cluster_position<false>;
    }
    return nullptr;
}

// ActivationManager::update on the device: energies, the islands' union-find
// over the contact pairs, and the islands' sleep decision.
cudaError_t launch_activation(const World& w, const StepParams& p, unsigned nbb, unsigned npb, cudaStream_t st) {
    k_act_init<<<nbb, kItemThreads, 0, st>>>(w, p);
    k_act_union<<<npb, kItemThreads, 0, st>>>(w);
    k_act_root<<<nbb, kItemThreads, 0, st>>>(w);
    k_act_apply<<<nbb, kItemThreads, 0, st>>>(w);
    return cudaGetLastError();
}
#else
// ================================================================ launchers
static unsigned item_blocks(uint32_t n) {
    unsigned b = (n + kItemThreads - 1) / kItemThreads;
    if (b < 1) b = 1;
    if (b > 152u * 16u) b = 152u * 16u;
    return b;
}

static const size_t kVelocitySmem = (size_t)kCoopThreads * kCacheF4 * sizeof(float4);

// Dynamic shared memory of the per-world velocity kernel: Δv (6 floats) per
// body slot of the largest world, or per slot of a small world for each warp.
// The per-world velocity kernel for a block size (64, 128 or 256).
static const void* world_velocity_fn(int threads, bool joints) {
    switch (threads) {
    case 64: return joints ? (const void*)k_world_velocity<64, true> : (const void*)k_world_velocity<64, false>;
    case 256: return joints ? (const void*)k_world_velocity<256, true> : (const void*)k_world_velocity<256, false>;
    default: return joints ? (const void*)k_world_velocity<128, true> : (const void*)k_world_velocity<128, false>;
    }
}
static const void* world_position_fn(bool joints) {
    return joints ? (const void*)k_world_position<128, true> : (const void*)k_world_position<128, false>;
}

// Blocks of fn resident per SM, the smaller over both instantiations (a
// kernel's grid fits either).
static int resident(const void* (*pick)(bool), int threads, size_t smem) {
    int lo = 0;
    for (bool j : {false, true}) {
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pick(j), threads, smem);
        if (!j || per < lo) lo = per;
    }
    return lo < 1 ? 1 : lo;
}

static size_t world_smem(uint32_t max_world_bodies, int threads) {
    size_t big = 6 * (size_t)max_world_bodies, warps = (size_t)(threads / 32) * 6 * kWarpWorldBodies;
    return (big > warps ? big : warps) * sizeof(float);
}

void solver_grid_sizes(int device, SolverLaunch& L) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, exchange_kernel(XK_COLOUR), kCoopThreads, 0);
    L.grid_colour = sms * (per < 1 ? 1 : per);
    for (bool j : {false, true})
        cudaFuncSetAttribute(exchange_kernel(XK_VELOCITY, j), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kVelocitySmem);
    L.grid_velocity = sms * resident([](bool j) { return exchange_kernel(XK_VELOCITY, j); }, kCoopThreads, kVelocitySmem);
    L.grid_position = sms * resident([](bool j) { return exchange_kernel(XK_POSITION, j); }, kCoopThreads, 0);
    L.grid_world_position = sms * resident(world_position_fn, 128, 0);
    for (int t : {64, 128, 256})
        for (bool j : {false, true})
            cudaFuncSetAttribute(world_velocity_fn(t, j), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)world_smem(kMaxWorldBodies, t));
    L.cluster_ctas = cluster_ctas(device);
}

uint64_t grid_task_capacity(const SolverLaunch& L) {
    int g = L.grid_velocity < L.grid_position ? L.grid_velocity : L.grid_position;
    return (uint64_t)g * kCoopThreads * kMaxPerThread;
}

int world_grid(int device, uint32_t max_world_bodies, uint32_t n_worlds, int threads) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    for (bool j : {false, true}) {
        int pj = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pj, world_velocity_fn(threads, j), threads,
                                                      world_smem(max_world_bodies, threads));
        if (!j || pj < per) per = pj;
    }
    long g = (long)sms * (per < 1 ? 1 : per);
    if (g > (long)n_worlds) g = n_worlds;
    return g < 1 ? 1 : (int)g;
}

static cudaError_t coop(const void* fn, int grid, void** args, cudaStream_t st, size_t smem = 0) {
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kCoopThreads), args, smem, st);
}

static size_t cluster_smem(uint32_t shift) { return (6u * sizeof(float)) << shift; }

int cluster_ctas(int device) {
    int ok = 0;
    cudaDeviceGetAttribute(&ok, cudaDevAttrClusterLaunch, device);
    if (!ok) return 0;
    for (bool j : {false, true}) {
        const void* fn = exchange_kernel(XK_CLUSTER_VELOCITY, j);
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cluster_smem(kClusterShiftMax));
        cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(exchange_kernel(XK_CLUSTER_POSITION, j), cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    }
    // The cluster size both instantiations hold resident.
    for (int c : {16, 8}) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)c;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)c);
        cfg.blockDim = dim3(kClusterThreads);
        cfg.dynamicSmemBytes = cluster_smem(kClusterShiftMax);
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0, nj = 0;
        if (cudaOccupancyMaxActiveClusters(&n, exchange_kernel(XK_CLUSTER_VELOCITY, false), &cfg) == cudaSuccess &&
            cudaOccupancyMaxActiveClusters(&nj, exchange_kernel(XK_CLUSTER_VELOCITY, true), &cfg) == cudaSuccess &&
            n > 0 && nj > 0)
            return c;
        cudaGetLastError();
    }
    return 0;
}

static cudaError_t launch_cluster(const void* fn, const SolverLaunch& L, size_t smem, void** args, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)L.cluster_ctas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)L.cluster_ctas * L.n_cluster);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

cudaError_t launch_solver(const World& w, const StepParams& p, const SolverLaunch& L, cudaStream_t st) {
    World wc = w;
    StepParams pc = p;
    void* args1[] = {&wc};
    void* args2[] = {&wc, &pc};
    const unsigned nbb = item_blocks(w.nb_slots), npb = item_blocks(w.cap_pairs);
    auto rec = [&](int k) {
        if (L.ev) cudaEventRecord(L.ev[k], st);
    };
    rec(0);
    cudaError_t e = launch_activation(wc, pc, nbb, npb, st);
    if (e != cudaSuccess) return e;
    rec(1);
    k_collect<<<npb, kItemThreads, 0, st>>>(wc);
    if (w.nj_slots) {
        k_collect_joints<<<item_blocks(w.nj_slots), kItemThreads, 0, st>>>(wc);
        k_clamp_solver<<<1, 1, 0, st>>>(wc);
    }
    size_t scan_bytes = L.scan_bytes;
    e = exclusive_scan(L.scan_temp, scan_bytes, w.b.adj_count, w.b.adj_start,
                                   w.nb_slots ? w.nb_slots : 1u, st);
    if (e != cudaSuccess) return e;
    k_adj_fill<<<npb, kItemThreads, 0, st>>>(wc);
    k_prank<<<npb, kItemThreads, 0, st>>>(wc);
    e = coop(exchange_kernel(XK_COLOUR), L.grid_colour, args1, st);
    if (e != cudaSuccess) return e;
    if (L.batched) {
        // Bucket the manifolds by (world, colour) and renumber them in that order.
        const uint32_t nbk = L.n_worlds * kMaxColours;
        e = cudaMemsetAsync(w.s.bucket_count, 0, (2 * (size_t)nbk + 1) * sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
        k_world_count<<<npb, kItemThreads, 0, st>>>(wc, L.n_worlds);
        scan_bytes = L.scan_bytes;
        e = exclusive_scan(L.scan_temp, scan_bytes, w.s.bucket_count, w.s.bucket_start, nbk + 1u, st);
        if (e != cudaSuccess) return e;
        k_world_scatter<<<npb, kItemThreads, 0, st>>>(wc, L.n_worlds);
        k_world_permute<<<npb, kItemThreads, 0, st>>>(wc, L.n_worlds);
        k_world_permute_back<<<npb, kItemThreads, 0, st>>>(wc);
    }
    rec(2);
    const bool joints = w.nj_slots != 0u;
    if (joints) k_assemble<true><<<npb, kItemThreads, 0, st>>>(wc, pc, !L.batched);
    else k_assemble<false><<<npb, kItemThreads, 0, st>>>(wc, pc, !L.batched);
    rec(3);
    if (L.batched) {
        if (L.n_cluster > 0) {
            uint32_t shift = L.cluster_shift;
            void* cargs[] = {&wc, &pc, &shift};
            e = launch_cluster(exchange_kernel(XK_CLUSTER_VELOCITY, joints), L, cluster_smem(shift), cargs, st);
            if (e != cudaSuccess) return e;
        }
        if (L.n_worlds > L.n_cluster) {
            const size_t smem = world_smem(L.max_world_bodies, L.world_threads);
            uint32_t nw = L.n_worlds, mwb = L.max_world_bodies, nbig = L.n_big, ncl = L.n_cluster;
            void* wargs[] = {&wc, &pc, &nw, &mwb, &nbig, &ncl};
            e = cudaLaunchKernel(world_velocity_fn(L.world_threads, joints), dim3(L.grid_world), dim3(L.world_threads),
                                 wargs, smem, st);
            if (e != cudaSuccess) return e;
        }
        k_world_finish<<<1, 1, 0, st>>>(wc, pc);
    } else {
        e = cudaMemsetAsync(&w.ctl->barrier_count, 0, sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
        e = coop(exchange_kernel(XK_VELOCITY, joints), L.grid_velocity, args2, st, kVelocitySmem);
        if (e != cudaSuccess) return e;
    }
    rec(4);
    const bool posef = !L.batched;
    k_cache_integrate<<<nbb > npb ? nbb : npb, kItemThreads, 0, st>>>(wc, pc, posef);
    rec(5);
    if (L.batched) {
        // The position sweeps run 128 threads a block whatever the velocity
        // kernel's block size: large worlds a block each, small ones a warp.
        if (L.n_cluster > 0) {
            void* cargs[] = {&wc, &pc};
            e = launch_cluster(exchange_kernel(XK_CLUSTER_POSITION, joints), L, 0, cargs, st);
            if (e != cudaSuccess) return e;
        }
        if (L.n_worlds > L.n_cluster) {
            uint32_t nw = L.n_worlds, nbig = L.n_big, ncl = L.n_cluster;
            void* pargs[] = {&wc, &pc, &nw, &nbig, &ncl};
            e = cudaLaunchKernel(world_position_fn(joints), dim3(L.grid_world_position), dim3(128), pargs, 0, st);
            if (e != cudaSuccess) return e;
        }
    } else {
        e = coop(exchange_kernel(XK_POSITION, joints), L.grid_position, args2, st);
        if (e != cudaSuccess) return e;
    }
    rec(6);
    k_post<<<nbb, kItemThreads, 0, st>>>(wc, pc, posef);
    return cudaGetLastError();
}

cudaError_t launch_ccd_begin(const World& w, cudaStream_t st) {
    k_ccd_begin<<<item_blocks(w.nb_slots), kItemThreads, 0, st>>>(w);
    return cudaGetLastError();
}

cudaError_t launch_ccd(const World& w, const StepParams& p, cudaStream_t st) {
    if (!p.ccd || w.ccd.n_worlds == 0) return cudaSuccess;
    const uint32_t nc = w.nc_slots;
    cudaError_t e = cudaMemsetAsync(w.ccd.adj_count, 0, sizeof(uint32_t) * (nc + 1), st);
    if (e != cudaSuccess) return e;
    k_ccd_adj_count<<<item_blocks(w.cap_pairs), kItemThreads, 0, st>>>(w);
    size_t bytes = w.ccd.adj_scan_bytes;
    e = exclusive_scan(w.ccd.adj_scan, bytes, w.ccd.adj_count, w.ccd.adj_start, nc + 1, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(w.ccd.adj_count, 0, sizeof(uint32_t) * (nc + 1), st);
    if (e != cudaSuccess) return e;
    k_ccd_adj_fill<<<item_blocks(w.cap_pairs), kItemThreads, 0, st>>>(w);
    k_ccd_adj_sort<<<item_blocks(nc), kItemThreads, 0, st>>>(w);
    // 256 threads a world when every world gets an SM of its own (the
    // kernel's registers allow one such block an SM), else 128 (two an SM):
    // the same results either way.
    int dev = 0, sms = 1;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 1;
    const int threads = w.ccd.n_worlds <= (uint32_t)sms ? kCcdThreads : kCcdThreads / 2;
    // solve_ccd's loop: a pass kernel, then the solve of the islands the
    // pass prepared, at most max_ccd_substeps + 2 times.
    for (uint32_t pass = 0; pass <= w.ccd.substeps + 1u; ++pass) {
        k_ccd_world<<<w.ccd.n_worlds, threads, 0, st>>>(w, p, pass);
        k_ccd_solve<<<w.ccd.n_worlds, kCcdSolveThreads, 0, st>>>(w, p);
    }
    k_ccd_finish<<<item_blocks(w.nb_slots), kItemThreads, 0, st>>>(w);
    return cudaGetLastError();
}

#endif  // NPGPU_EXCHANGE_TU

}  // namespace npgpu_dev
