// dyn.cuh -- per-body rigid-body dynamics on the device.
//
// RigidBody::update_dynamics / update_acceleration / integrate /
// apply_displacement (src/object/rigid_body.rs:371-381, 467-505, 558-619)
// and the activation helpers of src/object/body.rs:65-126, 335-340.
#pragma once
#include "world_dev.cuh"

namespace npgpu_dev {

__device__ __forceinline__ float np_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float np_min(float a, float b) { return (b < a) ? b : a; }

__device__ __forceinline__ np::V v3(float4 a) { return np::V{a.x, a.y, a.z}; }
__device__ __forceinline__ np::Q q4(float4 a) { return np::Q{a.x, a.y, a.z, a.w}; }
__device__ __forceinline__ float4 f4(np::V a, float w = 0.0f) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ float4 f4q(np::Q q) { return make_float4(q.i, q.j, q.k, q.w); }

__device__ __forceinline__ np::M load_m9(const float* p) {
    np::M m;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) m.m[a][c] = p[3 * a + c];
    return m;
}
__device__ __forceinline__ void store_m9(float* p, const np::M& m) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) p[3 * a + c] = m.m[a][c];
}

__device__ __forceinline__ bool body_is_active(uint32_t info, float energy) {
    uint32_t s = bi_status(info);
    if (s == 2u) return energy != 0.0f;   // NPGPU_BODY_DYNAMIC
    return s == 3u;                       // NPGPU_BODY_KINEMATIC
}
__device__ __forceinline__ bool body_can_sleep(uint32_t info) { return (bi_flags(info) & (1u << 7)) != 0; }
__device__ __forceinline__ float body_mask(uint32_t info, int k) {
    return (bi_flags(info) & (2u << k)) ? 0.0f : 1.0f;
}

// Body::activate.
__device__ __forceinline__ void body_activate(const Bodies& b, uint32_t i) {
    if (body_can_sleep(b.info[i])) b.energy[i] = b.sleep_thr[i] * 2.0f;
}

// R I R^-1 (Inertia3::transformed) of the angular part.
__device__ __forceinline__ np::M transformed_I(const np::M& local, np::Q q) {
    np::M rot = np::qmat(q);
    return np::mm(np::mm(rot, local), np::mtr(rot));
}

// RigidBody::update_dynamics for one body (assumes changed && dynamic).
__device__ __forceinline__ void body_update_dynamics(const Bodies& b, uint32_t i, float dt) {
    uint32_t info = b.info[i];
    if (!body_is_active(info, b.energy[i])) body_activate(b, i);
    np::Q q = q4(b.pos_q[i]);
    np::M I = transformed_I(load_m9(b.local_I + 9 * i), q);
    store_m9(b.I + 9 * i, I);
    np::V w = v3(b.ang[i]);
    np::V iw = np::mv(I, w);
    np::V w_dt = np::mul(w, dt);
    np::M wdc = np::cross_matrix(w_dt);
    np::M iwdc = np::cross_matrix(np::mul(iw, dt));
    np::M aug = np::madd(I, np::msub(np::mm(wdc, I), iwdc));
    float m = b.mass[i];
    b.inv_mass[i] = (m == 0.0f) ? 0.0f : 1.0f / m;
    store_m9(b.inv_I + 9 * i, np::minv_or_zero(aug));
}

// RigidBody::update_inertia_from_local_inertia (rigid_body.rs:266-271).
__device__ __forceinline__ void body_refresh_inertia(const Bodies& b, uint32_t i) {
    np::Q q = q4(b.pos_q[i]);
    np::M I = transformed_I(load_m9(b.local_I + 9 * i), q);
    store_m9(b.I + 9 * i, I);
    float m = b.mass[i];
    b.inv_mass[i] = (m == 0.0f) ? 0.0f : 1.0f / m;
    store_m9(b.inv_I + 9 * i, np::minv_or_zero(I));
}

// RigidBody::update_acceleration.
__device__ __forceinline__ void body_update_acceleration(const Bodies& b, uint32_t i, const StepParams& p) {
    uint32_t info = b.info[i];
    np::V al = np::mk(0.0f, 0.0f, 0.0f), aa = al;
    if (bi_status(info) == 2u) {
        np::M I = load_m9(b.I + 9 * i);
        np::M inv = load_m9(b.inv_I + 9 * i);
        np::V w = v3(b.ang[i]);
        np::V iw = np::mv(I, w);
        np::V gyro = np::neg(np::cross(w, iw));
        aa = np::mv(inv, gyro);
        float im = b.inv_mass[i];
        if (im != 0.0f && (bi_flags(info) & 1u)) al = np::mk(p.gx, p.gy, p.gz);
        al = np::add(al, np::mul(v3(b.f_lin[i]), im));
        aa = np::add(aa, np::mv(inv, v3(b.f_ang[i])));
        al = np::mk(al.x * body_mask(info, 0), al.y * body_mask(info, 1), al.z * body_mask(info, 2));
        aa = np::mk(aa.x * body_mask(info, 3), aa.y * body_mask(info, 4), aa.z * body_mask(info, 5));
    }
    b.acc_lin[i] = f4(al);
    b.acc_ang[i] = f4(aa);
}

// RigidBody::apply_displacement: pose <- T(com) exp(disp) T(-com) pose.
__device__ __forceinline__ void apply_displacement(np::V& pt, np::Q& pq, np::V& com, np::V local_com, np::V dlin,
                                                   np::V dang) {
    np::Q qd = np::qexp(dang);
    np::V t = np::add(np::add(com, dlin), np::qrot(qd, np::neg(com)));
    np::V nt = np::add(t, np::qrot(qd, pt));
    np::Q nq = np::qmul(qd, pq);
    pt = nt;
    pq = nq;
    np::Iso iso{pt, pq};
    com = np::iso_pt(iso, local_com);
}

__device__ __forceinline__ void body_apply_displacement(const Bodies& b, uint32_t i, np::V dlin, np::V dang) {
    np::V pt = v3(b.pos_t[i]);
    np::Q pq = q4(b.pos_q[i]);
    np::V com = v3(b.com[i]);
    apply_displacement(pt, pq, com, v3(b.local_com[i]), dlin, dang);
    b.pos_t[i] = f4(pt);
    b.pos_q[i] = f4q(pq);
    b.com[i] = f4(com);
    b.info[i] |= BI_CHANGED;
}

// RigidBody::integrate.
__device__ __forceinline__ void body_integrate(const Bodies& b, uint32_t i, float dt) {
    np::V lin = v3(b.lin[i]), ang = v3(b.ang[i]);
    lin = np::mul(lin, 1.0f / (1.0f + dt * b.lin_damp[i]));
    ang = np::mul(ang, 1.0f / (1.0f + dt * b.ang_damp[i]));
    float ml = b.max_lin[i], ma = b.max_ang[i];
    float ln = np::norm(lin);
    if (ln > ml) lin = (ml == 0.0f) ? np::mk(0.0f, 0.0f, 0.0f) : np::mul(lin, ml / ln);
    float an = np::norm(ang);
    if (an > ma) ang = (ma == 0.0f) ? np::mk(0.0f, 0.0f, 0.0f) : np::mul(ang, ma / an);
    b.lin[i] = f4(lin);
    b.ang[i] = f4(ang);
    body_apply_displacement(b, i, np::mul(lin, dt), np::mul(ang, dt));
}

}  // namespace npgpu_dev
