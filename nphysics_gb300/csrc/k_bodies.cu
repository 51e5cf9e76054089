// k_bodies.cu -- per-body kernels outside the solver: uploads from the host
// sets, the start of a step (update_dynamics / update_acceleration,
// src/world/mechanical_world.rs:225-245), applied forces, removals, and the
// gather of body state for the host.
#include "dyn.cuh"

namespace npgpu_dev {

constexpr int kThreads = 256;
static inline unsigned nblocks(uint32_t n) { return (n + kThreads - 1) / kThreads; }

__global__ void k_upload_bodies(World w, const BodyUpload* d, uint32_t n) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const BodyUpload u = d[t];
    const Bodies& b = w.b;
    uint32_t i = u.slot;
    b.gen[i] = u.gen;
    b.pos_t[i] = make_float4(u.pos[0], u.pos[1], u.pos[2], 0.0f);
    b.pos_q[i] = make_float4(u.pos[3], u.pos[4], u.pos[5], u.pos[6]);
    b.lin[i] = make_float4(u.vel[0], u.vel[1], u.vel[2], 0.0f);
    b.ang[i] = make_float4(u.vel[3], u.vel[4], u.vel[5], 0.0f);
    if (u.reset_energy) {
        // RigidBody::new / RigidBodyDesc::build (src/object/rigid_body.rs:54-83, 1064-1084).
        b.mass[i] = u.mass;
        for (int k = 0; k < 9; ++k) b.local_I[9 * i + k] = u.local_I[k];
        b.local_com[i] = make_float4(u.local_com[0], u.local_com[1], u.local_com[2], 0.0f);
        b.acc_lin[i] = b.acc_ang[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        b.f_lin[i] = b.f_ang[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        // ActivationStatus::new_active: 4 x the default threshold 0.01; a ground starts inactive.
        b.energy[i] = ((u.info >> BI_KIND_SHIFT) & 7u) == 1u ? 0.0f : 0.01f * 4.0f;
    }
    b.lin_damp[i] = u.lin_damp;
    b.ang_damp[i] = u.ang_damp;
    b.max_lin[i] = u.max_lin;
    b.max_ang[i] = u.max_ang;
    b.sleep_thr[i] = u.sleep_thr;
    b.world[i] = u.world;
    b.info[i] = u.info | BI_ALIVE | BI_CHANGED;
    np::Iso pose{v3(b.pos_t[i]), q4(b.pos_q[i])};
    b.com[i] = f4(np::iso_pt(pose, v3(b.local_com[i])));
    body_refresh_inertia(b, i);
}

__global__ void k_upload_colliders(World w, const ColliderUpload* d, uint32_t n) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const ColliderUpload u = d[t];
    const Colliders& c = w.c;
    uint32_t i = u.slot;
    c.body[i] = u.body;
    c.info[i] = u.info | CI_ALIVE;
    c.params[i] = make_float4(u.params[0], u.params[1], u.params[2], u.params[3]);
    c.wrt_t[i] = make_float4(u.wrt[0], u.wrt[1], u.wrt[2], 0.0f);
    c.wrt_q[i] = make_float4(u.wrt[3], u.wrt[4], u.wrt[5], u.wrt[6]);
    c.margin[i] = u.margin;
    c.lin_pred[i] = u.lin_pred;
    c.friction[i] = u.friction;
    c.restitution[i] = u.restitution;
    c.rank[i] = u.rank;
    c.aabb_min[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);   // a new DBVT proxy: no fat AABB yet
    c.aabb_max[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// RigidBody::add_local_inertia_and_com after the host folded the collider's
// mass properties into the local inertia (src/object/rigid_body.rs:747-766).
__global__ void k_mass_updates(World w, const MassUpdate* d, uint32_t n) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const MassUpdate u = d[t];
    const Bodies& b = w.b;
    uint32_t i = u.slot;
    if (u.activate & 1u) {   // the local inertia changed
        b.mass[i] = u.mass;
        for (int k = 0; k < 9; ++k) b.local_I[9 * i + k] = u.local_I[k];
        b.local_com[i] = make_float4(u.local_com[0], u.local_com[1], u.local_com[2], 0.0f);
        np::Iso pose{v3(b.pos_t[i]), q4(b.pos_q[i])};
        b.com[i] = f4(np::iso_pt(pose, v3(b.local_com[i])));
        body_refresh_inertia(b, i);
        b.info[i] |= BI_CHANGED;
    }
    if (u.activate & 2u) body_activate(b, i);   // Body::activate
}

// RigidBody::apply_force with ForceType::Force (rigid_body.rs:771-792).
__device__ __forceinline__ void apply_force(const Bodies& b, uint32_t i, const float* f, bool wake) {
    uint32_t info = b.info[i];
    if (bi_status(info) != 2u) return;
    if (wake) body_activate(b, i);
    np::V fl = np::mk(f[0] * body_mask(info, 0), f[1] * body_mask(info, 1), f[2] * body_mask(info, 2));
    np::V fa = np::mk(f[3] * body_mask(info, 3), f[4] * body_mask(info, 4), f[5] * body_mask(info, 5));
    b.f_lin[i] = f4(np::add(v3(b.f_lin[i]), fl));
    b.f_ang[i] = f4(np::add(v3(b.f_ang[i]), fa));
}

// Reads the batch from (h, f) (device memory, or page-locked host memory
// through its device-side address), keeps a copy in (hd, fd) when they
// differ, and checks it.
__global__ void k_force_check(World w, const npgpu_handle* h, const float* f, npgpu_handle* hd, float* fd, uint32_t n,
                              uint32_t batch, uint64_t cap) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const npgpu_handle ht = h[t];
    float ft[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) ft[e] = f[6 * (size_t)t + e];
    if (hd != h) {
        hd[t] = ht;
#pragma unroll
        for (int e = 0; e < 6; ++e) fd[6 * (size_t)t + e] = ft[e];
    }
    const uint64_t idx = ht.index;
    uint32_t fl = 0;
    if (idx >= cap || !(w.b.info[idx] & BI_ALIVE) || w.b.gen[idx] != ht.generation) fl |= 1u;
    else if (atomicExch(&w.b.fstamp[idx], batch) == batch) fl |= 4u;
#pragma unroll
    for (int e = 0; e < 6; ++e)
        if (!isfinite(ft[e])) fl |= 2u;
    if (fl) atomicOr(&w.ctl->force_flags, fl);
}

// One force per thread (the batch names each body once), or the whole batch
// in order on one thread.
__global__ void k_forces(World w, const npgpu_handle* h, const float* f, uint32_t n, bool wake, bool serial) {
    if (serial) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            for (uint32_t k = 0; k < n; ++k) apply_force(w.b, (uint32_t)h[k].index, f + 6 * (size_t)k, wake);
        return;
    }
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    apply_force(w.b, (uint32_t)h[t].index, f + 6 * (size_t)t, wake);
}

__global__ void k_kill(World w, const uint32_t* slots, uint32_t n, int colliders) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    uint32_t i = slots[t];
    if (colliders) w.c.info[i] &= ~CI_ALIVE;
    else w.b.info[i] &= ~BI_ALIVE;
}

// Drops the cached manifolds of colliders that were removed or replaced, and
// wakes the bodies touching a removed collider (geometrical_world.rs:152-177).
// flags[c]: 1 = replaced, 2 = removed.
__global__ void k_forget_pairs(World w, const uint8_t* flags) {
    uint32_t npairs = w.ctl->npairs;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x) {
        uint2 pr = w.cur.pair[p];
        if (pr.x == 0xffffffffu) continue;
        uint8_t f1 = flags[pr.x], f2 = flags[pr.y];
        if (!f1 && !f2) continue;
        if (w.cur.ncont[p] > 0) {
            if (f1 == 2 && !f2) body_activate(w.b, w.c.body[pr.y]);
            if (f2 == 2 && !f1) body_activate(w.b, w.c.body[pr.x]);
        }
        w.cur.pair[p] = make_uint2(0xffffffffu, 0xffffffffu);
        w.cur.ncont[p] = 0;
        w.cur.prox[p] = (uint8_t)PROX_DISJOINT;
    }
}

// Start of MechanicalWorld::step: update_dynamics for bodies whose state
// changed, then update_acceleration (mechanical_world.rs:225-245).
__global__ void k_body_start(World w, StepParams p) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) w.ctl->nevents = 0;   // MechanicalWorld::step clears the contact events first
    if (i >= w.nb_slots) return;
    uint32_t info = w.b.info[i];
    if (!(info & BI_ALIVE)) return;
    if ((info & BI_CHANGED) && bi_status(info) == 2u) body_update_dynamics(w.b, i, p.dt);
    body_update_acceleration(w.b, i, p);
}

__global__ void k_pack_bodies(World w, uint32_t first, uint32_t n, float* pos7, float* vel6, float* energy,
                              uint8_t* active) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    uint32_t i = first + t;
    const Bodies& b = w.b;
    if (pos7) {
        float4 a = b.pos_t[i], q = b.pos_q[i];
        float* o = pos7 + 7 * (size_t)t;
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = q.x; o[4] = q.y; o[5] = q.z; o[6] = q.w;
    }
    if (vel6) {
        float4 l = b.lin[i], a = b.ang[i];
        float* o = vel6 + 6 * (size_t)t;
        o[0] = l.x; o[1] = l.y; o[2] = l.z; o[3] = a.x; o[4] = a.y; o[5] = a.z;
    }
    if (energy) energy[t] = b.energy[i];
    if (active) active[t] = body_is_active(b.info[i], b.energy[i]) ? 1 : 0;
}

// Poses and velocities of slots [first, first + n) written straight into
// page-locked host arrays (their device-side addresses): each block packs
// its bodies in shared memory and writes contiguous runs, so the stores to
// host memory coalesce.
__global__ void k_pack_bodies_host(World w, uint32_t first, uint32_t n, float* pos7, float* vel6) {
    __shared__ float sp[kThreads * 7], sv[kThreads * 6];
    const uint32_t b0 = blockIdx.x * kThreads, t = threadIdx.x;
    const uint32_t cnt = n - b0 < (uint32_t)kThreads ? n - b0 : (uint32_t)kThreads;
    if (t < cnt) {
        const uint32_t i = first + b0 + t;
        const float4 a = w.b.pos_t[i], q = w.b.pos_q[i], l = w.b.lin[i], g = w.b.ang[i];
        float* o = sp + 7 * t;
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = q.x; o[4] = q.y; o[5] = q.z; o[6] = q.w;
        float* v = sv + 6 * t;
        v[0] = l.x; v[1] = l.y; v[2] = l.z; v[3] = g.x; v[4] = g.y; v[5] = g.z;
    }
    __syncthreads();
    if (pos7)
        for (uint32_t j = t; j < 7 * cnt; j += kThreads) pos7[7 * (size_t)b0 + j] = sp[j];
    if (vel6)
        for (uint32_t j = t; j < 6 * cnt; j += kThreads) vel6[6 * (size_t)b0 + j] = sv[j];
}

cudaError_t launch_pack_bodies_host(const World& w, uint32_t first, uint32_t n, float* pos7, float* vel6,
                                    cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_pack_bodies_host<<<nblocks(n), kThreads, 0, st>>>(w, first, n, pos7, vel6);
    return cudaGetLastError();
}

cudaError_t launch_upload_bodies(const World& w, const BodyUpload* d, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_upload_bodies<<<nblocks(n), kThreads, 0, st>>>(w, d, n);
    return cudaGetLastError();
}
cudaError_t launch_upload_colliders(const World& w, const ColliderUpload* d, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_upload_colliders<<<nblocks(n), kThreads, 0, st>>>(w, d, n);
    return cudaGetLastError();
}
cudaError_t launch_mass_updates(const World& w, const MassUpdate* d, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_mass_updates<<<nblocks(n), kThreads, 0, st>>>(w, d, n);
    return cudaGetLastError();
}
cudaError_t launch_force_check(const World& w, const npgpu_handle* h, const float* f, npgpu_handle* hd, float* fd,
                               uint32_t n, uint32_t batch, uint64_t cap, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_force_check<<<nblocks(n), kThreads, 0, st>>>(w, h, f, hd, fd, n, batch, cap);
    return cudaGetLastError();
}
cudaError_t launch_forces(const World& w, const npgpu_handle* h, const float* f, uint32_t n, bool wake, bool serial,
                          cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_forces<<<serial ? 1u : nblocks(n), kThreads, 0, st>>>(w, h, f, n, wake, serial);
    return cudaGetLastError();
}
__global__ void k_upload_joints(World w, const JointUpload* d, uint32_t n) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const JointUpload u = d[t];
    const uint32_t i = u.slot;
    const Joints& j = w.j;
    j.info[i] = u.info;
    j.body[2 * i] = u.body1;
    j.body[2 * i + 1] = u.body2;
    j.anchor[2 * i] = make_float4(u.anchor1[0], u.anchor1[1], u.anchor1[2], 0.0f);
    j.anchor[2 * i + 1] = make_float4(u.anchor2[0], u.anchor2[1], u.anchor2[2], 0.0f);
    j.frame[2 * i] = make_float4(u.frame1[0], u.frame1[1], u.frame1[2], u.frame1[3]);
    j.frame[2 * i + 1] = make_float4(u.frame2[0], u.frame2[1], u.frame2[2], u.frame2[3]);
    j.brk[i] = make_float2(u.brk_force2, u.brk_torque2);
    j.axis[3 * i] = make_float4(u.axis1[0], u.axis1[1], u.axis1[2], u.angle);
    j.axis[3 * i + 1] = make_float4(u.axis2[0], u.axis2[1], u.axis2[2], u.min_offset);
    j.axis[3 * i + 2] = make_float4(u.axis3[0], u.axis3[1], u.axis3[2], u.max_offset);
    if (u.reset) {
        j.imp[2 * i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        j.imp[2 * i + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        j.state[i] = 0u;
    }
}

cudaError_t launch_upload_joints(const World& w, const JointUpload* d, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_upload_joints<<<nblocks(n), kThreads, 0, st>>>(w, d, n);
    return cudaGetLastError();
}

cudaError_t launch_kill(const World& w, const uint32_t* slots, uint32_t n, int colliders, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_kill<<<nblocks(n), kThreads, 0, st>>>(w, slots, n, colliders);
    return cudaGetLastError();
}
cudaError_t launch_forget_pairs(const World& w, const uint8_t* flags, cudaStream_t st) {
    uint32_t blocks = nblocks(w.cap_pairs);
    if (blocks == 0) return cudaSuccess;
    if (blocks > 152u * 16u) blocks = 152u * 16u;
    k_forget_pairs<<<blocks, kThreads, 0, st>>>(w, flags);
    return cudaGetLastError();
}
cudaError_t launch_body_start(const World& w, const StepParams& p, cudaStream_t st) {
    if (w.nb_slots == 0) return cudaSuccess;
    k_body_start<<<nblocks(w.nb_slots), kThreads, 0, st>>>(w, p);
    return cudaGetLastError();
}
cudaError_t launch_pack_bodies(const World& w, uint32_t first, uint32_t n, float* pos7, float* vel6, float* energy,
                               uint8_t* active, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_pack_bodies<<<nblocks(n), kThreads, 0, st>>>(w, first, n, pos7, vel6, energy, active);
    return cudaGetLastError();
}

}  // namespace npgpu_dev
