// k_solve.cu -- the solver half of MechanicalWorld::step as one persistent,
// cooperatively launched kernel (grid = co-resident blocks, phases separated
// by a bounded software grid barrier):
//
//   activation   ActivationManager::update (src/detection/activation_manager.rs:61-201):
//                RWA energies, islands by lock-free union-find, sleep / wake
//   collection   manifolds handed to the solver (src/world/mechanical_world.rs:287-300)
//   colouring    Jones-Plassmann rounds with first-fit colours over dynamic-body
//                conflicts; manifolds of one colour share no dynamic body
//   assembly     SignoriniCoulombPyramidModel::constraints
//                (src/solver/signorini_coulomb_pyramid_model.rs:56-224,
//                signorini_model.rs:37-138, helper.rs:53-135, rigid_body.rs:672-722)
//   SOR-Prox     SORProx::solve (src/solver/sor_prox.rs:48-179): warm start, then per
//                iteration every friction row, then every normal row, colour by colour
//   residual     FP64 complementarity residual
//   cache        cache_impulses (signorini_coulomb_pyramid_model.rs:226-261)
//   integrate    update_velocities_and_integrate (moreau_jean_solver.rs:328-347)
//   position     NonlinearSORProx::solve (src/solver/nonlinear_sor_prox.rs:17-309), colour by colour
//   post         kinematic integration, update_dynamics, clear_forces (mechanical_world.rs:328-367)
//
// Within one colour every manifold is handled by one thread, which walks its
// contacts in order; the result equals a sequential Gauss-Seidel sweep over
// the manifolds sorted by colour.
#include "narrow.cuh"

namespace npgpu_dev {

constexpr int kSolveThreads = 256;
constexpr unsigned long long kWaitLimitNs = 1000000000ull;   // a bounded wait gives up after one second

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier. Returns false when the wait gave up (ERRF_TIMEOUT set);
// the caller then leaves the kernel.
__device__ __forceinline__ bool grid_sync(Control* ctl) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile uint32_t* genp = &ctl->barrier_gen;
        uint32_t gen = *genp;
        __threadfence();
        uint32_t arrived = atomicAdd(&ctl->barrier_count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&ctl->barrier_count, 0u);
            __threadfence();
            atomicAdd(&ctl->barrier_gen, 1u);
        } else {
            unsigned long long t0 = global_ns();
            unsigned spins = 0;
            while (*genp == gen) {
                if ((++spins & 255u) == 0u) {
                    if (((volatile uint32_t*)&ctl->err)[0] & ERRF_TIMEOUT) break;
                    if (global_ns() - t0 > kWaitLimitNs) {
                        atomicOr(&ctl->err, ERRF_TIMEOUT);
                        break;
                    }
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return !(((volatile uint32_t*)&ctl->err)[0] & ERRF_TIMEOUT);
}

#define GRID_FOR(i, n) for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)
#define SYNC_OR_RETURN() \
    do {                 \
        if (!grid_sync(w.ctl)) return; \
    } while (0)

__device__ __forceinline__ uint32_t pair_hash22(uint32_t c1, uint32_t c2) {
    uint32_t h = c1 * 0x9E3779B1u ^ (c2 + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h >> 10;
}
__device__ __forceinline__ unsigned long long pair_priority(uint32_t c1, uint32_t c2) {
    return ((unsigned long long)pair_hash22(c1, c2) << 42) | ((unsigned long long)c1 << 21) | (unsigned long long)c2;
}

// Lock-free union-find over body slots (link the larger root under the smaller).
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

// RigidBody::fill_constraint_geometry for one side of one row.
__device__ __forceinline__ void fill_row_side(const BodyView& b, np::V point, np::V dir, float* J, float* WJ, float& inv_r,
                                              float& rhs, bool with_ext, float dt) {
    uint32_t st = bi_status(b.info);
    np::V pos = np::sub(point, b.com);
    np::V fa = np::cross(pos, dir);
    float f[6] = {dir.x, dir.y, dir.z, fa.x, fa.y, fa.z};
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

// nalgebra Vector3::orthonormal_subspace_basis of one vector.
__device__ __forceinline__ void tangent_basis(np::V n, np::V& t1, np::V& t2) {
    np::V a;
    if (fabsf(n.x) > fabsf(n.y)) a = np::mk(n.z, 0.0f, -n.x);
    else a = np::mk(0.0f, -n.z, n.y);
    t1 = np::divs(a, np::norm(a));
    np::V b = np::cross(n, a);
    t2 = np::divs(b, np::norm(b));
}

// Velocity-solver state of one manifold: the dv of its dynamic bodies.
struct DV {
    float a[6], b[6];
};

__device__ __forceinline__ float jdot(const float* row, const DV& dv, bool has1, bool has2) {
    float d = 0.0f;
    if (has1 && has2) {
        float s1 = 0.0f, s2 = 0.0f;
#pragma unroll
        for (int k = 0; k < 6; ++k) s1 = s1 + row[RF_J1 + k] * dv.a[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) s2 = s2 + row[RF_J2 + k] * dv.b[k];
        d = s1 + s2;
    } else if (has1) {
#pragma unroll
        for (int k = 0; k < 6; ++k) d = d + row[RF_J1 + k] * dv.a[k];
    } else if (has2) {
#pragma unroll
        for (int k = 0; k < 6; ++k) d = d + row[RF_J2 + k] * dv.b[k];
    }
    return d;
}
__device__ __forceinline__ void axpy(const float* row, DV& dv, float a, bool has1, bool has2) {
    if (has1) {
#pragma unroll
        for (int k = 0; k < 6; ++k) dv.a[k] = a * row[RF_WJ1 + k] + dv.a[k];
    }
    if (has2) {
#pragma unroll
        for (int k = 0; k < 6; ++k) dv.b[k] = a * row[RF_WJ2 + k] + dv.b[k];
    }
}
// A row is 7 float4 (112 bytes, 16-byte aligned): loaded into registers at once.
__device__ __forceinline__ void load_row(const float* p, float* r) {
    const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        float4 x = q[k];
        r[4 * k] = x.x;
        r[4 * k + 1] = x.y;
        r[4 * k + 2] = x.z;
        r[4 * k + 3] = x.w;
    }
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

// FP64 residual terms of one row.
__device__ __forceinline__ void residual_row(const float* row, const DV& dv, bool has1, bool has2, bool friction,
                                             double normal_impulse, double& s2, double& l2) {
    double d = 0.0;
    if (has1)
        for (int k = 0; k < 6; ++k) d += (double)row[RF_J1 + k] * (double)dv.a[k];
    if (has2)
        for (int k = 0; k < 6; ++k) d += (double)row[RF_J2 + k] * (double)dv.b[k];
    d += (double)row[RF_RHS];
    double lam = (double)row[RF_IMP];
    double x = lam - (double)row[RF_R] * d;
    double p;
    if (!friction) {
        p = x > 0.0 ? x : 0.0;
    } else {
        double mx = (double)row[RF_MU] * normal_impulse;
        p = x < -mx ? -mx : (x > mx ? mx : x);
    }
    double phi = lam - p;
    s2 += phi * phi;
    l2 += lam * lam;
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
    return t;
}

// Evaluates the FP64 residual over all solver rows; the result lands in ctl->residual.
__device__ bool eval_residual(const World& w, uint32_t ms, double* sh, bool initial) {
    double s2 = 0.0, l2 = 0.0;
    GRID_FOR(s, ms) {
        int b1 = w.s.sm_b1[s], b2 = w.s.sm_b2[s];
        uint32_t nc = w.s.sm_nc[s];
        DV dv;
        load_dv(w.b.dv, b1, dv.a);
        load_dv(w.b.dv, b2, dv.b);
        const float* rows = w.s.rows + (size_t)s * 12 * kRowFloats;
        for (uint32_t k = 0; k < nc; ++k) {
            const float* rn = rows + (3 * k) * kRowFloats;
            residual_row(rn, dv, b1 >= 0, b2 >= 0, false, 0.0, s2, l2);
            residual_row(rn + kRowFloats, dv, b1 >= 0, b2 >= 0, true, (double)rn[RF_IMP], s2, l2);
            residual_row(rn + 2 * kRowFloats, dv, b1 >= 0, b2 >= 0, true, (double)rn[RF_IMP], s2, l2);
        }
    }
    double ts = block_sum(s2, sh);
    double tl = block_sum(l2, sh);
    if (threadIdx.x == 0) {
        atomicAdd(&w.ctl->res_acc[0], ts);
        atomicAdd(&w.ctl->res_acc[1], tl);
    }
    if (!grid_sync(w.ctl)) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double a = w.ctl->res_acc[0], b = w.ctl->res_acc[1];
        double r = sqrt(a) / fmax(1.0, sqrt(b));
        w.ctl->residual = r;
        if (initial) w.ctl->residual_initial = r;
        w.ctl->res_acc[0] = 0.0;
        w.ctl->res_acc[1] = 0.0;
    }
    return grid_sync(w.ctl);
}

__device__ __forceinline__ void stamp(const World& w, const StepParams& p, int k) {
    if (p.profile && blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        w.ctl->t_phase[k] = t;
    }
}

__global__ void __launch_bounds__(kSolveThreads) k_solve(World w, StepParams p) {
    __shared__ double sh[32];
    __shared__ uint32_t sh_scan[kMaxColours + 1];
    const Bodies& b = w.b;
    const Colliders& c = w.c;
    const uint32_t nb = w.nb_slots;
    stamp(w, p, 0);

    // ---- activation: energies, union-find init -------------------------------------------
    GRID_FOR(i, nb) {
        uint32_t info = b.info[i];
        b.uf_parent[i] = i;
        b.can_deact[i] = 1;
        b.jp_used[i] = 0ull;
#pragma unroll
        for (int k = 0; k < 6; ++k) b.dv[6 * i + k] = 0.0f;
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
    if (blockIdx.x == 0 && threadIdx.x < kMaxColours) {
        w.s.colour_count[threadIdx.x] = 0;
        if (threadIdx.x == 0) {
            w.ctl->nsolver = 0;
            w.ctl->ncolours = 0;
            w.ctl->jp_remaining[0] = 0;
            w.ctl->jp_remaining[1] = 0;
            w.ctl->nsolver_contacts = 0;
            w.ctl->nactive = 0;
            w.ctl->res_acc[0] = 0.0;
            w.ctl->res_acc[1] = 0.0;
            w.ctl->kinetic_energy = 0.0;
        }
    }
    SYNC_OR_RETURN();
    const uint32_t npairs = w.ctl->npairs;
    GRID_FOR(q, npairs) {
        if (w.cur.ncont[q] == 0) continue;
        uint2 pr = w.cur.pair[q];
        uint32_t b1 = c.body[pr.x], b2 = c.body[pr.y];
        uint32_t s1 = bi_status(b.info[b1]), s2 = bi_status(b.info[b2]);
        if ((s1 == 2u || s1 == 3u) && (s2 == 2u || s2 == 3u)) uf_union(b.uf_parent, b1, b2, &w.ctl->err);
    }
    SYNC_OR_RETURN();
    GRID_FOR(i, nb) {
        uint32_t info = b.info[i];
        uint32_t st = bi_status(info);
        if (!(info & BI_ALIVE) || !(st == 2u || st == 3u)) continue;
        uint32_t r = uf_find(b.uf_parent, i);
        bool ok = body_can_sleep(info) && b.energy[i] < b.sleep_thr[i];
        if (!ok) atomicAnd(&b.can_deact[r], 0);
    }
    SYNC_OR_RETURN();
    GRID_FOR(i, nb) {
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
            atomicAdd(&w.ctl->nactive, 1u);
            if (!(en != 0.0f) && body_can_sleep(info)) body_activate(b, i);
        }
    }
    SYNC_OR_RETURN();
    stamp(w, p, 1);

    // ---- manifold collection ----------------------------------------------------------------
    GRID_FOR(q, npairs) {
        uint32_t nc = w.cur.ncont[q];
        if (nc == 0) continue;
        uint2 pr = w.cur.pair[q];
        uint32_t b1 = c.body[pr.x], b2 = c.body[pr.y];
        uint32_t i1 = b.info[b1], i2 = b.info[b2];
        uint32_t s1 = bi_status(i1), s2 = bi_status(i2);
        if (s1 == 0u || s2 == 0u) continue;
        bool a1 = s1 == 2u && b.energy[b1] != 0.0f;
        bool a2 = s2 == 2u && b.energy[b2] != 0.0f;
        if (!(a1 || a2)) continue;
        uint32_t idx = atomicAdd(&w.ctl->nsolver, 1u);
        w.s.sm_list[idx] = q;
        w.s.sm_state[idx] = 0;
        atomicAdd(&w.ctl->nsolver_contacts, nc);
    }
    SYNC_OR_RETURN();
    const uint32_t ms = w.ctl->nsolver;

    // ---- colouring: Jones-Plassmann rounds, first-fit colours -------------------------------
    for (uint32_t round = 0;; ++round) {
        GRID_FOR(m, ms) {
            if (w.s.sm_state[m] != 0) continue;
            uint2 pr = w.cur.pair[w.s.sm_list[m]];
            unsigned long long pri = pair_priority(pr.x, pr.y);
            uint32_t b1 = c.body[pr.x], b2 = c.body[pr.y];
            if (bi_status(b.info[b1]) == 2u) atomicMax(&b.jp_best[b1], pri);
            if (bi_status(b.info[b2]) == 2u) atomicMax(&b.jp_best[b2], pri);
        }
        SYNC_OR_RETURN();
        GRID_FOR(m, ms) {
            if (w.s.sm_state[m] != 0) continue;
            uint2 pr = w.cur.pair[w.s.sm_list[m]];
            unsigned long long pri = pair_priority(pr.x, pr.y);
            uint32_t b1 = c.body[pr.x], b2 = c.body[pr.y];
            bool d1 = bi_status(b.info[b1]) == 2u, d2 = bi_status(b.info[b2]) == 2u;
            bool won = (!d1 || b.jp_best[b1] == pri) && (!d2 || b.jp_best[b2] == pri);
            if (!won) {
                atomicAdd(&w.ctl->jp_remaining[round & 1u], 1u);
                continue;
            }
            unsigned long long mask = 0ull;
            if (d1) mask |= b.jp_used[b1];
            if (d2) mask |= b.jp_used[b2];
            uint32_t col = (uint32_t)(__ffsll((long long)~mask) - 1);
            if (mask == ~0ull) {
                atomicOr(&w.ctl->err, ERRF_COLOURS);
                col = kMaxColours - 1;
            }
            w.s.sm_colour[m] = col;
            w.s.sm_state[m] = 1;
            if (d1) b.jp_used[b1] |= (1ull << col);
            if (d2) b.jp_used[b2] |= (1ull << col);
            atomicMax(&w.ctl->ncolours, col + 1);
            atomicAdd(&w.s.colour_count[col], 1u);
        }
        SYNC_OR_RETURN();
        GRID_FOR(m, ms) {
            uint8_t stt = w.s.sm_state[m];
            if (stt == 2) continue;
            uint2 pr = w.cur.pair[w.s.sm_list[m]];
            b.jp_best[c.body[pr.x]] = 0ull;
            b.jp_best[c.body[pr.y]] = 0ull;
            if (stt == 1) w.s.sm_state[m] = 2;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) w.ctl->jp_remaining[(round + 1) & 1u] = 0;
        SYNC_OR_RETURN();
        if (((volatile uint32_t*)w.ctl->jp_remaining)[round & 1u] == 0) break;
        if (round > 4096) {
            if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&w.ctl->err, ERRF_COLOURS);
            return;
        }
    }
    // Bucket the manifolds by colour.
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int k = 0; k < kMaxColours; ++k) {
            w.s.colour_start[k] = acc;
            w.s.colour_cursor[k] = acc;
            acc += w.s.colour_count[k];
        }
        w.s.colour_start[kMaxColours] = acc;
    }
    SYNC_OR_RETURN();
    GRID_FOR(m, ms) {
        uint32_t col = w.s.sm_colour[m];
        uint32_t pos = atomicAdd(&w.s.colour_cursor[col], 1u);
        w.s.sm_sorted[pos] = w.s.sm_list[m];
    }
    SYNC_OR_RETURN();
    const uint32_t ncol = w.ctl->ncolours;
    if (threadIdx.x <= kMaxColours) sh_scan[threadIdx.x] = w.s.colour_start[threadIdx.x];
    __syncthreads();
    stamp(w, p, 2);

    // ---- assembly -----------------------------------------------------------------------
    const float dt = p.dt;
    GRID_FOR(s, ms) {
        uint32_t q = w.s.sm_sorted[s];
        uint2 pr = w.cur.pair[q];
        uint32_t c1 = pr.x, c2 = pr.y;
        uint32_t bb1 = c.body[c1], bb2 = c.body[c2];
        BodyView v1 = load_view(b, bb1), v2 = load_view(b, bb2);
        bool d1 = bi_status(v1.info) == 2u, d2 = bi_status(v2.info) == 2u;
        w.s.sm_b1[s] = d1 ? (int)bb1 : -1;
        w.s.sm_b2[s] = d2 ? (int)bb2 : -1;
        uint32_t nc = w.cur.ncont[q];
        w.s.sm_nc[s] = nc;
        uint32_t ci1 = c.info[c1], ci2 = c.info[c2];
        float mu = combine(c.friction[c1], (ci1 >> 4) & 0xfu, c.friction[c2], (ci2 >> 4) & 0xfu);
        float e = combine(c.restitution[c1], (ci1 >> 8) & 0xfu, c.restitution[c2], (ci2 >> 8) & 0xfu);
        float m1 = c.margin[c1], m2 = c.margin[c2];
        float* rows = w.s.rows + (size_t)s * 12 * kRowFloats;
        for (uint32_t k = 0; k < nc; ++k) {
            uint32_t slot = q * kMaxContacts + k;
            float4 w1 = w.cur.w1[slot], w2 = w.cur.w2[slot], nn = w.cur.n[slot], imp = w.cur.imp[slot];
            np::V n = v3(nn);
            np::V center1 = np::add(v3(w1), np::mul(n, m1));
            np::V center2 = np::sub(v3(w2), np::mul(n, m2));
            float* rn = rows + (3 * k) * kRowFloats;
            make_row(rn, v1, v2, center1, center2, np::neg(n), dt);
            float rhs = rn[RF_RHS];
            if (rhs <= -p.restitution_threshold) rhs = rhs + e * rhs;
            float depth = w1.w + m1 + m2;
            if (depth < 0.0f) rhs = rhs + (-depth) * p.inv_dt;
            rn[RF_RHS] = rhs;
            rn[RF_IMP] = p.warmstart_mode == 1u ? 0.0f : imp.x * p.warmstart_coeff;
            np::V t[2];
            tangent_basis(n, t[0], t[1]);
            for (int sdir = 0; sdir < 2; ++sdir) {
                float* rt = rn + (1 + sdir) * kRowFloats;
                make_row(rt, v1, v2, center1, center2, t[sdir], dt);
                float ci = sdir == 0 ? imp.y : imp.z;
                rt[RF_IMP] = p.warmstart_mode == 1u ? 0.0f : ci * p.warmstart_coeff;
                rt[RF_MU] = mu;
            }
        }
    }
    SYNC_OR_RETURN();
    stamp(w, p, 3);

    // ---- warm start (sor_prox.rs:19-45), colour by colour -----------------------------------
    for (uint32_t col = 0; col < ncol; ++col) {
        uint32_t lo = sh_scan[col], hi = sh_scan[col + 1];
        for (uint32_t s = lo + blockIdx.x * blockDim.x + threadIdx.x; s < hi; s += gridDim.x * blockDim.x) {
            int b1 = w.s.sm_b1[s], b2 = w.s.sm_b2[s];
            DV dv;
            load_dv(b.dv, b1, dv.a);
            load_dv(b.dv, b2, dv.b);
            const float* rows = w.s.rows + (size_t)s * 12 * kRowFloats;
            uint32_t nc = w.s.sm_nc[s];
            for (uint32_t k = 0; k < 3 * nc; ++k) {
                const float* r = rows + k * kRowFloats;
                float imp = r[RF_IMP];
                if (imp != 0.0f) axpy(r, dv, imp, b1 >= 0, b2 >= 0);
            }
            store_dv(b.dv, b1, dv.a);
            store_dv(b.dv, b2, dv.b);
        }
        SYNC_OR_RETURN();
    }
    if (!eval_residual(w, ms, sh, true)) return;

    // ---- SOR-Prox iterations ---------------------------------------------------------------
    uint32_t maxit = p.solve_to_tolerance ? p.max_iterations_to_tolerance : p.max_velocity_iterations;
    uint32_t iters = 0;
    for (uint32_t it = 0; it < maxit; ++it) {
        if (p.solve_to_tolerance && ((volatile double*)&w.ctl->residual)[0] <= (double)p.residual_tolerance) break;
        // Friction rows (bilateral, ImpulseLimits::Dependent), sor_prox.rs:232-343.
        for (uint32_t col = 0; col < ncol; ++col) {
            uint32_t lo = sh_scan[col], hi = sh_scan[col + 1];
            for (uint32_t s = lo + blockIdx.x * blockDim.x + threadIdx.x; s < hi; s += gridDim.x * blockDim.x) {
                int b1 = w.s.sm_b1[s], b2 = w.s.sm_b2[s];
                bool h1 = b1 >= 0, h2 = b2 >= 0;
                DV dv;
                load_dv(b.dv, b1, dv.a);
                load_dv(b.dv, b2, dv.b);
                float* rows = w.s.rows + (size_t)s * 12 * kRowFloats;
                uint32_t nc = w.s.sm_nc[s];
                for (uint32_t k = 0; k < nc; ++k) {
                    float li = rows[(3 * k) * kRowFloats + RF_IMP];
                    float rr[2][kRowFloats];
                    load_row(rows + (3 * k + 1) * kRowFloats, rr[0]);
                    load_row(rows + (3 * k + 2) * kRowFloats, rr[1]);
#pragma unroll
                    for (int sdir = 0; sdir < 2; ++sdir) {
                        const float* r = rr[sdir];
                        float* rg = rows + (3 * k + 1 + sdir) * kRowFloats;
                        float imp = r[RF_IMP];
                        if (li == 0.0f) {
                            if (imp != 0.0f) {
                                axpy(r, dv, -imp, h1, h2);
                                rg[RF_IMP] = 0.0f;
                            }
                            continue;
                        }
                        float mx = r[RF_MU] * li, mn = -mx;
                        float dimp = jdot(r, dv, h1, h2) + r[RF_RHS];
                        float ni = imp - r[RF_R] * dimp;
                        if (ni < mn) ni = mn;
                        else if (ni > mx) ni = mx;
                        float dl = ni - imp;
                        rg[RF_IMP] = ni;
                        axpy(r, dv, dl, h1, h2);
                    }
                }
                store_dv(b.dv, b1, dv.a);
                store_dv(b.dv, b2, dv.b);
            }
            SYNC_OR_RETURN();
        }
        // Normal rows (unilateral), sor_prox.rs:181-230.
        for (uint32_t col = 0; col < ncol; ++col) {
            uint32_t lo = sh_scan[col], hi = sh_scan[col + 1];
            for (uint32_t s = lo + blockIdx.x * blockDim.x + threadIdx.x; s < hi; s += gridDim.x * blockDim.x) {
                int b1 = w.s.sm_b1[s], b2 = w.s.sm_b2[s];
                bool h1 = b1 >= 0, h2 = b2 >= 0;
                DV dv;
                load_dv(b.dv, b1, dv.a);
                load_dv(b.dv, b2, dv.b);
                float* rows = w.s.rows + (size_t)s * 12 * kRowFloats;
                uint32_t nc = w.s.sm_nc[s];
                for (uint32_t k = 0; k < nc; ++k) {
                    float r[kRowFloats];
                    float* rg = rows + (3 * k) * kRowFloats;
                    load_row(rg, r);
                    float imp = r[RF_IMP];
                    float dimp = jdot(r, dv, h1, h2) + r[RF_RHS];
                    float ni = imp - r[RF_R] * dimp;
                    ni = ni > 0.0f ? ni : 0.0f;
                    float dl = ni - imp;
                    rg[RF_IMP] = ni;
                    axpy(r, dv, dl, h1, h2);
                }
                store_dv(b.dv, b1, dv.a);
                store_dv(b.dv, b2, dv.b);
            }
            SYNC_OR_RETURN();
        }
        ++iters;
        if (p.solve_to_tolerance)
            if (!eval_residual(w, ms, sh, false)) return;
    }
    if (!p.solve_to_tolerance)
        if (!eval_residual(w, ms, sh, false)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) w.ctl->iterations = iters;
    stamp(w, p, 4);

    // ---- cache impulses + integrate ------------------------------------------------------
    GRID_FOR(s, ms) {
        uint32_t q = w.s.sm_sorted[s];
        const float* rows = w.s.rows + (size_t)s * 12 * kRowFloats;
        uint32_t nc = w.s.sm_nc[s];
        for (uint32_t k = 0; k < nc; ++k) {
            float4 imp = make_float4(rows[(3 * k) * kRowFloats + RF_IMP], rows[(3 * k + 1) * kRowFloats + RF_IMP],
                                     rows[(3 * k + 2) * kRowFloats + RF_IMP], 0.0f);
            w.cur.imp[q * kMaxContacts + k] = imp;
        }
    }
    GRID_FOR(i, nb) {
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
    }
    SYNC_OR_RETURN();
    stamp(w, p, 5);

    // ---- NonlinearSORProx, colour by colour -------------------------------------------------
    for (uint32_t it = 0; it < p.max_position_iterations; ++it) {
        for (uint32_t col = 0; col < ncol; ++col) {
            uint32_t lo = sh_scan[col], hi = sh_scan[col + 1];
            for (uint32_t s = lo + blockIdx.x * blockDim.x + threadIdx.x; s < hi; s += gridDim.x * blockDim.x) {
                uint32_t q = w.s.sm_sorted[s];
                uint2 pr = w.cur.pair[q];
                uint32_t c1 = pr.x, c2 = pr.y;
                uint32_t bb1 = c.body[c1], bb2 = c.body[c2];
                uint32_t i1 = b.info[bb1], i2 = b.info[bb2];
                bool d1 = bi_status(i1) == 2u, d2 = bi_status(i2) == 2u;
                // Poses of both bodies (static and kinematic ones are read only).
                np::V t1 = v3(b.pos_t[bb1]), t2 = v3(b.pos_t[bb2]);
                np::Q q1 = q4(b.pos_q[bb1]), q2 = q4(b.pos_q[bb2]);
                np::V com1 = v3(b.com[bb1]), com2 = v3(b.com[bb2]);
                np::V lc1 = v3(b.local_com[bb1]), lc2 = v3(b.local_com[bb2]);
                float im1 = b.inv_mass[bb1], im2 = b.inv_mass[bb2];
                np::M iI1 = load_m9(b.inv_I + 9 * bb1), iI2 = load_m9(b.inv_I + 9 * bb2);
                np::Iso wrt1{v3(c.wrt_t[c1]), q4(c.wrt_q[c1])}, wrt2{v3(c.wrt_t[c2]), q4(c.wrt_q[c2])};
                uint32_t sh1 = c.info[c1] & 0xfu, sh2 = c.info[c2] & 0xfu;
                float4 pp1 = c.params[c1], pp2 = c.params[c2];
                np::V hh1 = v3(pp1), hh2 = v3(pp2);
                float dil1 = (sh1 == SHAPE_BALL ? pp1.x : 0.0f) + c.margin[c1];
                float dil2 = (sh2 == SHAPE_BALL ? pp2.x : 0.0f) + c.margin[c2];
                uint32_t nc = w.cur.ncont[q];
                bool moved1 = false, moved2 = false;
                for (uint32_t k = 0; k < nc; ++k) {
                    uint32_t slot = q * kMaxContacts + k;
                    uint32_t key = w.cur.key[slot];
                    int f1 = (int)(key / 26u), f2 = (int)(key % 26u);
                    np::Iso m1 = np::iso_mul(np::Iso{t1, q1}, wrt1);
                    np::Iso m2 = np::iso_mul(np::Iso{t2, q2}, wrt2);
                    np::V n0 = np::qrot(m1.q, v3(w.cur.nl[slot]));
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
                        fill_row_side(v, g.w1, np::neg(g.n), J1, W1, inv_r, dummy, false, dt);
                    }
                    if (d2) {
                        BodyView v;
                        v.com = com2; v.inv_mass = im2; v.inv_I = iI2; v.info = i2;
                        v.lin = v.ang = v.acc_lin = v.acc_ang = np::mk(0.0f, 0.0f, 0.0f);
                        fill_row_side(v, g.w2, g.n, J2, W2, inv_r, dummy, false, dt);
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
                if (moved1) {
                    b.pos_t[bb1] = f4(t1);
                    b.pos_q[bb1] = f4q(q1);
                    b.com[bb1] = f4(com1);
                    b.info[bb1] = b.info[bb1] | BI_CHANGED;
                }
                if (moved2) {
                    b.pos_t[bb2] = f4(t2);
                    b.pos_q[bb2] = f4q(q2);
                    b.com[bb2] = f4(com2);
                    b.info[bb2] = b.info[bb2] | BI_CHANGED;
                }
            }
            SYNC_OR_RETURN();
        }
    }
    stamp(w, p, 6);

    // ---- kinematic integration, update_dynamics, clear_forces, audit ------------------------
    double ke = 0.0;
    GRID_FOR(i, nb) {
        uint32_t info = b.info[i];
        if (!(info & BI_ALIVE)) continue;
        uint32_t st = bi_status(info);
        if (st == 3u) {
            body_integrate(b, i, dt);
            info = b.info[i];
        }
        if ((info & BI_CHANGED) && st == 2u) body_update_dynamics(b, i, dt);
        b.f_lin[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        b.f_ang[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        b.info[i] = b.info[i] & ~BI_CHANGED;
        if (st == 2u) {
            float4 l = b.lin[i], a = b.ang[i], tt = b.pos_t[i];
            if (!(isfinite(l.x) && isfinite(l.y) && isfinite(l.z) && isfinite(a.x) && isfinite(a.y) && isfinite(a.z) &&
                  isfinite(tt.x) && isfinite(tt.y) && isfinite(tt.z)))
                atomicOr(&w.ctl->err, ERRF_NAN);
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
    if (threadIdx.x == 0) atomicAdd(&w.ctl->kinetic_energy, tke);
    stamp(w, p, 7);
}

int solve_grid_size(int device) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve, kSolveThreads, 0);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

cudaError_t launch_solve(const World& w, const StepParams& p, int grid, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(&w.ctl->barrier_count, 0, 2 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    World wc = w;
    StepParams pc = p;
    void* args[] = {&wc, &pc};
    return cudaLaunchCooperativeKernel((const void*)k_solve, dim3(grid), dim3(kSolveThreads), args, 0, st);
}

}  // namespace npgpu_dev
