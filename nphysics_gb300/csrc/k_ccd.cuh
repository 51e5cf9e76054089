// k_ccd.cuh -- continuous collision detection: MechanicalWorld::solve_ccd
// (src/world/mechanical_world.rs:561-908) with predict_next_impacts
// (:400-559) and TOIEntry::try_from_colliders (:942-1031).
//
// Included once, by the translation unit of k_solve.cu that holds the
// solver's row and position helpers (NPGPU_EXCHANGE_TU = 0).
//
// One block per world that has a CCD collider (every world of a batch is its
// own MechanicalWorld: its own impacts, latest TOI and substeps). The loop of
// solve_ccd is sequential by nature (a priority queue of TOIs, bodies frozen
// at their first impact, resweeps, an island grown through contacts, a
// Gauss-Seidel solve in the reference's row order): thread 0 carries it, and
// the block shares the data-parallel parts: the swept boxes, the swept-box
// neighbour searches (ordered compactions over the world's colliders), every
// batch of TOI queries, the island's body preparation and contact updates,
// its rows, its colour-ordered solves and its integration. The interactions
// of a collider during CCD are its broad-phase pairs (fat AABBs overlapping,
// read from the step's pair list) and, where either collider has CCD
// enabled, the pairs whose boxes swept from the safe pose to the current one
// overlap; pairs are taken in collider-slot order and TOIs of equal time in
// the order they were found.

// The largest CCD block (a world's block has 128 or 256 threads).
constexpr int kCcdThreads = 256;
constexpr uint32_t kTocPopped = 1u << 30, kTocSuperseded = 1u << 31, kTocSeq = kTocPopped - 1u;

__device__ __forceinline__ uint32_t ccd_body_of(const World& w, uint32_t c) { return w.c.body[c]; }
__device__ __forceinline__ bool ccd_dynamic(const World& w, uint32_t b) { return bi_status(w.b.info[b]) == 2u; }
__device__ __forceinline__ bool ccd_enabled(const World& w, uint32_t c) { return (w.c.info[c] & CI_CCD) != 0u; }
__device__ __forceinline__ bool ccd_linear(const World& w, uint32_t b) {
    return (bi_flags(w.b.info[b]) & NPGPU_BODY_LINEAR_INTERP) != 0u;
}

// RigidBody::safe_position (rigid_body.rs:904-910).
__device__ __forceinline__ np::Iso ccd_safe_pose(const World& w, uint32_t b) {
    const np::V t0 = v3(w.ccd.pos0_t[b]);
    return ccd_linear(w, b) ? np::Iso{t0, q4(w.b.pos_q[b])} : np::Iso{t0, q4(w.ccd.pos0_q[b])};
}

// The loosened AABB (margin + linear prediction) of collider c at body pose P.
__device__ __forceinline__ void ccd_aabb(const World& w, uint32_t c, const np::Iso& P, float* mn, float* mx) {
    const np::Iso pose = np::iso_mul(P, np::Iso{v3(w.c.wrt_t[c]), q4(w.c.wrt_q[c])});
    const uint32_t shape = w.c.info[c] & 0xfu;
    const float4 prm = w.c.params[c];
    np::V half;
    if (shape == SHAPE_BALL) {
        half = np::mk(prm.x, prm.x, prm.x);
    } else if (shape == SHAPE_CAPSULE) {
        const np::M rot = np::qmat(pose.q);
        for (int a = 0; a < 3; ++a) np::setc(half, a, fabsf(rot.m[a][1]) * prm.y + prm.x);
    } else {
        const np::M rot = np::qmat(pose.q);
        for (int a = 0; a < 3; ++a)
            np::setc(half, a, fabsf(rot.m[a][0]) * prm.x + fabsf(rot.m[a][1]) * prm.y + fabsf(rot.m[a][2]) * prm.z);
    }
    const float ql = w.c.margin[c] + w.c.lin_pred[c];
    for (int a = 0; a < 3; ++a) {
        mn[a] = (np::comp(pose.t, a) - np::comp(half, a)) - ql;
        mx[a] = (np::comp(pose.t, a) + np::comp(half, a)) + ql;
    }
}

__device__ __forceinline__ void ccd_sweep_box(const World& w, uint32_t c) {
    const uint32_t b = ccd_body_of(w, c);
    float a0[3], b0[3], a1[3], b1[3];
    ccd_aabb(w, c, ccd_safe_pose(w, b), a0, b0);
    ccd_aabb(w, c, np::Iso{v3(w.b.pos_t[b]), q4(w.b.pos_q[b])}, a1, b1);
    w.ccd.sw_min[c] = make_float4(np_min(a0[0], a1[0]), np_min(a0[1], a1[1]), np_min(a0[2], a1[2]), 0.0f);
    w.ccd.sw_max[c] = make_float4(np_max(b0[0], b1[0]), np_max(b0[1], b1[1]), np_max(b0[2], b1[2]), 0.0f);
}

// The collider's core, pose on its body and reach from the body's centre of mass.
__device__ __forceinline__ ccd::Shape ccd_shape(const World& w, uint32_t c) {
    ccd::Shape s;
    const np::V zero = np::mk(0.0f, 0.0f, 0.0f);
    s.local.a = s.local.b = s.local.h = zero;
    s.local.q = np::Q{0.0f, 0.0f, 0.0f, 1.0f};
    s.wrt = np::Iso{v3(w.c.wrt_t[c]), q4(w.c.wrt_q[c])};
    const uint32_t shape = w.c.info[c] & 0xfu;
    const float4 prm = w.c.params[c];
    float extent;
    if (shape == SHAPE_BALL) {
        s.local.kind = ccd::CORE_POINT;
        s.local.radius = prm.x;
        extent = prm.x;
    } else if (shape == SHAPE_CAPSULE) {
        s.local.kind = ccd::CORE_SEGMENT;
        s.local.a = np::mk(0.0f, -prm.y, 0.0f);
        s.local.b = np::mk(0.0f, prm.y, 0.0f);
        s.local.radius = prm.x;
        extent = prm.y + prm.x;
    } else {
        s.local.kind = ccd::CORE_BOX;
        s.local.h = np::mk(prm.x, prm.y, prm.z);
        s.local.radius = 0.0f;
        extent = np::norm(s.local.h);
    }
    s.reach = np::norm(np::sub(s.wrt.t, v3(w.b.local_com[ccd_body_of(w, c)]))) + extent;
    return s;
}

// BodyPart::part_motion (rigid_body.rs:539-553) shifted by `by`, or the still
// pose of a frozen body (position0 displaced by `by`).
__device__ __forceinline__ ccd::Motion ccd_motion(const World& w, uint32_t b, bool frozen, float by) {
    ccd::Motion m;
    m.start = ccd_safe_pose(w, b);
    m.local_com = v3(w.b.local_com[b]);
    m.lin = v3(w.b.lin[b]);
    m.ang = v3(w.b.ang[b]);
    m.linear_only = ccd_linear(w, b);
    const bool still = m.lin.x == 0.0f && m.lin.y == 0.0f && m.lin.z == 0.0f &&
                       (m.linear_only || (m.ang.x == 0.0f && m.ang.y == 0.0f && m.ang.z == 0.0f));
    m.tau = frozen ? 0.0f : by;
    m.moving = !still;
    if (frozen) {
        if (m.moving) m.start = ccd::displace(m.start, m.local_com, np::mul(m.lin, by), np::mul(m.ang, by), m.linear_only);
        m.moving = false;
    }
    return m;
}

// TOIEntry::try_from_colliders with the search ending at end_time: t (from
// `start`, the later of the two bodies' times) or t = -1 when there is none.
__device__ __forceinline__ float2 ccd_toi(const World& w, const StepParams& p, uint32_t c1, uint32_t c2, float end_time) {
    const uint32_t b1 = ccd_body_of(w, c1), b2 = ccd_body_of(w, c2);
    const bool f1 = (w.ccd.bflag[b1] & 1u) != 0u, f2 = (w.ccd.bflag[b2] & 1u) != 0u;
    const float bt1 = w.ccd.btime[b1], bt2 = w.ccd.btime[b2];
    const float t1 = f1 ? w.ccd.ftime[b1] : bt1, t2 = f2 ? w.ccd.ftime[b2] : bt2;
    const float start = t1 < t2 ? t2 : t1;
    const ccd::Motion m1 = f1 ? ccd_motion(w, b1, true, t1 - bt1) : ccd_motion(w, b1, false, start - bt1);
    const ccd::Motion m2 = f2 ? ccd_motion(w, b2, true, t2 - bt2) : ccd_motion(w, b2, false, start - bt2);
    float t;
    const ccd::CaResult r = ccd::conservative_advancement(ccd_shape(w, c1), m1, ccd_shape(w, c2), m2,
                                                          end_time - start, p.allowed_linear_error, t);
    if (!r.some || (r.penetrating && !w.ccd.on_penetration)) return make_float2(-1.0f, start);
    return make_float2(t, start);
}

// The contacts of colliders c1 < c2 at their bodies' current poses into a
// pool manifold (the contact update of mechanical_world.rs:755-757).
__device__ __forceinline__ uint32_t ccd_contacts(const World& w, uint32_t c1, uint32_t c2, CcdManifold& m) {
    Shape s[2];
    const uint32_t cs[2] = {c1, c2};
    for (int k = 0; k < 2; ++k) {
        const uint32_t c = cs[k], b = ccd_body_of(w, c);
        const float4 prm = w.c.params[c];
        s[k].shape = w.c.info[c] & 0xfu;
        s[k].h = np::mk(prm.x, prm.y, prm.z);
        s[k].radius = prm.x;
        s[k].pose = np::iso_mul(np::Iso{v3(w.b.pos_t[b]), q4(w.b.pos_q[b])}, np::Iso{v3(w.c.wrt_t[c]), q4(w.c.wrt_q[c])});
    }
    const float prediction = (w.c.margin[c1] + w.c.lin_pred[c1]) + (w.c.margin[c2] + w.c.lin_pred[c2]);
    CandList out;
    int keep[kMaxContacts];
    const int nk = shape_pair_contacts(s[0], s[1], prediction, out, keep);
    const uint32_t nc = nk > kMaxContacts ? (uint32_t)kMaxContacts : (uint32_t)nk;
    const np::Q bq = q4(w.b.pos_q[ccd_body_of(w, c1)]);
    for (uint32_t k = 0; k < nc; ++k) {
        const Cand& cd = out.c[keep[k]];
        m.k[k].n = f4(cd.g.n, cd.g.depth);
        m.k[k].w1 = f4(cd.g.w1, __uint_as_float((uint32_t)(cd.f1 * 26 + cd.f2)));
        m.k[k].w2 = f4(cd.g.w2);
        m.k[k].nl = f4(np::qrot_inv(bq, cd.g.n));
    }
    m.c1 = c1;
    m.c2 = c2;
    m.nc = nc;
    return nc;
}

// RigidBody::advance then clamp_advancement (rigid_body.rs:521-537).
__device__ __forceinline__ void ccd_clamp(const World& w, uint32_t b) {
    const np::V t0 = v3(w.ccd.pos0_t[b]);
    const np::Q q = ccd_linear(w, b) ? q4(w.b.pos_q[b]) : q4(w.ccd.pos0_q[b]);
    w.b.pos_t[b] = f4(t0);
    w.b.pos_q[b] = f4q(q);
    w.b.com[b] = f4(np::iso_pt(np::Iso{t0, q}, v3(w.b.local_com[b])));
    w.b.info[b] |= BI_CHANGED;
}

// The preparation of an island body (mechanical_world.rs:681-713): forces
// cleared, dynamics for the substep, acceleration without gravity, moved back
// to `target` (its frozen time, or the latest TOI) and clamped there.
__device__ void ccd_prepare(const World& w, const StepParams& p0, uint32_t h, float dts, float last) {
    const Bodies& b = w.b;
    b.f_lin[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    b.f_ang[h] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (b.info[h] & BI_CHANGED) body_update_dynamics(b, h, dts);
    StepParams pz = p0;
    pz.gx = pz.gy = pz.gz = 0.0f;
    body_update_acceleration(b, h, pz);
    const float target = (w.ccd.bflag[h] & 1u) ? w.ccd.ftime[h] : last;
    const float by = target - w.ccd.btime[h];
    const np::Iso p0s = ccd::displace(ccd_safe_pose(w, h), v3(b.local_com[h]), np::mul(v3(b.lin[h]), by),
                                      np::mul(v3(b.ang[h]), by), ccd_linear(w, h));
    w.ccd.pos0_t[h] = f4(p0s.t);
    w.ccd.pos0_q[h] = f4q(p0s.q);
    ccd_clamp(w, h);
    w.ccd.btime[h] = last;
}

// The island's rows of one manifold (built in parallel after the island is
// complete): SignoriniCoulombPyramidModel's normal and friction rows for the
// substep, started from zero (warmstart_coeff 0).
__device__ void ccd_rows(const World& w, const StepParams& p, CcdManifold& m, float dts) {
    const Bodies& b = w.b;
    const Colliders& c = w.c;
    const uint32_t c1 = m.c1, c2 = m.c2, bb1 = ccd_body_of(w, c1), bb2 = ccd_body_of(w, c2);
    const BodyView v1 = load_view(b, bb1), v2 = load_view(b, bb2);
    const uint32_t ci1 = c.info[c1], ci2 = c.info[c2];
    m.mu = combine(c.friction[c1], (ci1 >> 4) & 0xfu, c.friction[c2], (ci2 >> 4) & 0xfu);
    const float e = combine(c.restitution[c1], (ci1 >> 8) & 0xfu, c.restitution[c2], (ci2 >> 8) & 0xfu);
    const float m1 = c.margin[c1], m2 = c.margin[c2];
    m.b1 = ccd_dynamic(w, bb1) ? (int)bb1 : -1;
    m.b2 = ccd_dynamic(w, bb2) ? (int)bb2 : -1;
    uint32_t mask = 0;
    if (m.b1 >= 0) mask |= ~(bi_flags(v1.info) >> 1) & 0x3fu;
    if (m.b2 >= 0) mask |= (~(bi_flags(v2.info) >> 1) & 0x3fu) << 8;
    m.mask = mask;
    const float inv_dt = dts == 0.0f ? 0.0f : 1.0f / dts;
    for (uint32_t k = 0; k < m.nc; ++k) {
        CcdContact& K = m.k[k];
        const np::V n = v3(K.n);
        const np::V center1 = np::add(v3(K.w1), np::mul(n, m1));
        const np::V center2 = np::sub(v3(K.w2), np::mul(n, m2));
        float rn[kRowFloats], rt[2][kRowFloats];
        make_row(rn, v1, v2, center1, center2, np::neg(n), dts);
        float rhs = rn[RF_RHS];
        if (rhs <= -p.restitution_threshold) rhs = rhs + e * rhs;
        const float depth = K.n.w + m1 + m2;
        if (depth < 0.0f) rhs = rhs + (-depth) * inv_dt;
        np::V t[2];
        tangent_basis(n, t[0], t[1]);
        for (int s = 0; s < 2; ++s) make_row(rt[s], v1, v2, center1, center2, t[s], dts);
        K.pos1 = f4(np::sub(center1, v1.com), rn[RF_R]);
        K.pos2 = f4(np::sub(center2, v2.com), rhs);
        K.rr = make_float4(rt[0][RF_R], rt[0][RF_RHS], rt[1][RF_R], rt[1][RF_RHS]);
        K.lam = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        K.t1 = f4(t[0]);
        K.t2 = f4(t[1]);
    }
}

// NonlinearSORProx::solve_unilateral for an island manifold's contacts in
// order (the position solver's contact arithmetic).
__device__ void ccd_position_manifold(const World& w, const StepParams& p, const CcdManifold& m) {
    const Bodies& b = w.b;
    const Colliders& c = w.c;
    const uint32_t bb1 = ccd_body_of(w, m.c1), bb2 = ccd_body_of(w, m.c2);
    const uint32_t i1 = b.info[bb1], i2 = b.info[bb2];
    const bool d1 = bi_status(i1) == 2u, d2 = bi_status(i2) == 2u;
    // The manifold's two bodies stay in registers over its contacts (no
    // other manifold of its colour moves them).
    np::V t1 = v3(b.pos_t[bb1]), t2 = v3(b.pos_t[bb2]);
    np::Q q1 = q4(b.pos_q[bb1]), q2 = q4(b.pos_q[bb2]);
    np::V com1 = v3(b.com[bb1]), com2 = v3(b.com[bb2]);
    const np::Iso wrt1{v3(c.wrt_t[m.c1]), q4(c.wrt_q[m.c1])}, wrt2{v3(c.wrt_t[m.c2]), q4(c.wrt_q[m.c2])};
    const uint32_t sh1 = c.info[m.c1] & 0xfu, sh2 = c.info[m.c2] & 0xfu;
    const float4 pp1 = c.params[m.c1], pp2 = c.params[m.c2];
    const float dil1 = (sh1 == SHAPE_BALL || sh1 == SHAPE_CAPSULE ? pp1.x : 0.0f) + c.margin[m.c1];
    const float dil2 = (sh2 == SHAPE_BALL || sh2 == SHAPE_CAPSULE ? pp2.x : 0.0f) + c.margin[m.c2];
    BodyView v1, v2;
    if (d1) {
        v1.inv_mass = b.inv_mass[bb1]; v1.inv_I = load_m9(b.inv_I + 9 * bb1); v1.info = i1;
        v1.lin = v1.ang = v1.acc_lin = v1.acc_ang = np::mk(0.0f, 0.0f, 0.0f);
    }
    if (d2) {
        v2.inv_mass = b.inv_mass[bb2]; v2.inv_I = load_m9(b.inv_I + 9 * bb2); v2.info = i2;
        v2.lin = v2.ang = v2.acc_lin = v2.acc_ang = np::mk(0.0f, 0.0f, 0.0f);
    }
    const np::V lc1 = d1 ? v3(b.local_com[bb1]) : np::mk(0.0f, 0.0f, 0.0f);
    const np::V lc2 = d2 ? v3(b.local_com[bb2]) : np::mk(0.0f, 0.0f, 0.0f);
    bool moved1 = false, moved2 = false;
    for (uint32_t kk = 0; kk < m.nc; ++kk) {
        const CcdContact& K = m.k[kk];
        const uint32_t key = __float_as_uint(K.w1.w);
        const int f1 = (int)(key / 26u), f2 = (int)(key % 26u);
        const np::Iso m1 = np::iso_mul(np::Iso{t1, q1}, wrt1), m2 = np::iso_mul(np::Iso{t2, q2}, wrt2);
        const np::V n0 = np::qrot(m1.q, v3(K.nl));
        const Geom g = kinematic_contact(feature_of(sh1, np::mk(pp1.x, pp1.y, pp1.z), f1), m1, dil1,
                                         feature_of(sh2, np::mk(pp2.x, pp2.y, pp2.z), f2), m2, dil2, n0);
        float rhs = (-g.depth + p.allowed_linear_error) * p.erp;
        const float lim = -p.max_linear_correction;
        rhs = (rhs < lim) ? lim : rhs;
        if (rhs >= 0.0f) continue;
        float inv_r = 0.0f, dummy = 0.0f;
        float J1[6], J2[6], W1[6], W2[6];
        if (d1) {
            v1.com = com1;
            fill_row_side(v1, g.w1, np::neg(g.n), J1, W1, inv_r, dummy, false, p.dt);
        }
        if (d2) {
            v2.com = com2;
            fill_row_side(v2, g.w2, g.n, J2, W2, inv_r, dummy, false, p.dt);
        }
        if (inv_r == 0.0f) continue;
        const float r = 1.0f / inv_r;
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
    if (moved1) {
        b.pos_t[bb1] = f4(t1);
        b.pos_q[bb1] = f4q(q1);
        b.com[bb1] = f4(com1);
        b.info[bb1] |= BI_CHANGED;
    }
    if (moved2) {
        b.pos_t[bb2] = f4(t2);
        b.pos_q[bb2] = f4q(q2);
        b.com[bb2] = f4(com2);
        b.info[bb2] |= BI_CHANGED;
    }
}

// One pass of an island manifold's rows (SORProx, sor_prox.rs:181-343):
// its friction rows (friction true) or its normal rows. Δv in Bodies::dv; two
// manifolds of one colour share no dynamic body, so a colour's manifolds run
// in parallel.
__device__ void ccd_manifold_velocity(const World& w, CcdManifold& m, bool friction) {
    const Bodies& b = w.b;
    const bool h1 = m.b1 >= 0, h2 = m.b2 >= 0;
    BodyMasses bm;
    const int sl[2] = {m.b1, m.b2};
    for (int s = 0; s < 2; ++s) {
        if (sl[s] < 0) continue;
        bm.s[s].im = b.inv_mass[sl[s]];
        bm.s[s].I = load_m9(b.inv_I + 9 * (size_t)sl[s]);
    }
    DV dv;
    for (int k = 0; k < 6; ++k) {
        if (h1) dv.a[k] = b.dv[6 * (size_t)m.b1 + k];
        if (h2) dv.b[k] = b.dv[6 * (size_t)m.b2 + k];
    }
    for (uint32_t k = 0; k < m.nc; ++k) {
        CcdContact& K = m.k[k];
        const np::V pos1 = v3(K.pos1), pos2 = v3(K.pos2);
        const float4 l = K.lam;
        if (friction) {
            const np::V t[2] = {v3(K.t1), v3(K.t2)};
            const float rr[2] = {K.rr.x, K.rr.z}, rh[2] = {K.rr.y, K.rr.w};
            float imps[2] = {l.y, l.z};
            const float li = l.x;
            for (int s = 0; s < 2; ++s) {
                const float imp = imps[s];
                if (li == 0.0f) {
                    if (imp != 0.0f) {
                        axpy(t[s], pos1, pos2, m.mask, bm, dv, -imp, h1, h2);
                        imps[s] = 0.0f;
                    }
                    continue;
                }
                const float mx = m.mu * li, mn = -mx;
                const float dimp = jdot(t[s], pos1, pos2, m.mask, dv, h1, h2) + rh[s];
                float ni = imp - rr[s] * dimp;
                if (ni < mn) ni = mn;
                else if (ni > mx) ni = mx;
                const float dl = ni - imp;
                imps[s] = ni;
                axpy(t[s], pos1, pos2, m.mask, bm, dv, dl, h1, h2);
            }
            K.lam = make_float4(li, imps[0], imps[1], 0.0f);
        } else {
            const np::V dn = np::neg(v3(K.n));
            const float imp = l.x;
            const float dimp = jdot(dn, pos1, pos2, m.mask, dv, h1, h2) + K.pos2.w;
            float ni = imp - K.pos1.w * dimp;
            ni = ni > 0.0f ? ni : 0.0f;
            const float dl = ni - imp;
            K.lam = make_float4(ni, l.y, l.z, 0.0f);
            axpy(dn, pos1, pos2, m.mask, bm, dv, dl, h1, h2);
        }
    }
    for (int k = 0; k < 6; ++k) {
        if (h1) b.dv[6 * (size_t)m.b1 + k] = dv.a[k];
        if (h2) b.dv[6 * (size_t)m.b2 + k] = dv.b[k];
    }
}

// Shared state of a world's CCD loop.
struct CcdState {
    float end_time, min_overstep, last;
    uint32_t last_iter, result, nheap, nimp, seq, nstack, nisland, nccdb, nm;
    uint32_t cur, n, stop, epoch, ncol, nnext, left;
    uint32_t cnt[kCcdThreads / 32];
    uint32_t part[kCcdThreads];
    uint32_t col_start[kCcdColours + 1];
    uint32_t col_fill[kCcdColours];
    unsigned long long t_mark, t_acc[4];
};

enum : int { CCD_T_TOI = 0, CCD_T_SOLVER = 1, CCD_T_BROAD = 2, CCD_T_NARROW = 3 };

// A world's CCD state between the pass and solve kernels (Ccd::wstate,
// kCcdStateWords words a world; the island's colour starts in Ccd::wcols).
constexpr int kCcdSolveThreads = 256;
enum : uint32_t {
    CS_END = 0, CS_DTS = 1, CS_LAST_ITER = 2, CS_DONE = 3, CS_PENDING = 4, CS_NM = 5, CS_NCOL = 6, CS_NISL = 7,
    CS_NCCDB = 8, CS_NIMP = 9, CS_TOTAL = 10   // CS_TOTAL, CS_TOTAL + 1: the world's CCD time (profile mode)
};
// Profile mode: ns of a world's CCD spent in `part`, and the world's total.
__device__ __forceinline__ void ccd_account(const World& w, uint32_t* S, int part, unsigned long long ns) {
    atomicAdd(&w.ctl->ccd_ns[part], ns);
    unsigned long long* total = reinterpret_cast<unsigned long long*>(S + CS_TOTAL);
    *total += ns;
    atomicMax(&w.ctl->ccd_max_ns, *total);
}
// Profile mode: the time since the last mark goes to `part` (thread 0 keeps
// the block's sums).
__device__ __forceinline__ void ccd_mark(CcdState& st, const StepParams& p, int part) {
    if (p.profile && threadIdx.x == 0) {
        const unsigned long long t = global_ns();
        st.t_acc[part] += t - st.t_mark;
        st.t_mark = t;
    }
}

// Exclusive prefix sums of a[0, n) in place, by the whole block; returns
// the total.
__device__ uint32_t block_scan(uint32_t* a, uint32_t n, CcdState& st) {
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t lo = threadIdx.x * per, hi = lo + per < n ? lo + per : n;
    uint32_t sum = 0;
    for (uint32_t i = lo; i < hi; ++i) sum += a[i];
    st.part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t k = 0; k < blockDim.x; ++k) {
            const uint32_t v = st.part[k];
            st.part[k] = run;
            run += v;
        }
        st.n = run;
    }
    __syncthreads();
    uint32_t run = st.part[threadIdx.x];
    for (uint32_t i = lo; i < hi; ++i) {
        const uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
    const uint32_t total = st.n;
    __syncthreads();
    return total;
}

// The Jones-Plassmann priority of an island manifold: a hash of its
// colliders' world-local slots, ties by the slots.
__device__ __forceinline__ unsigned long long ccd_priority(uint32_t base, const CcdManifold& m) {
    const uint32_t l1 = m.c1 - base, l2 = m.c2 - base;
    return ((unsigned long long)pair_hash22(l1, l2) << 42) | ((unsigned long long)l1 << 21) | (unsigned long long)l2;
}

// Is d (a collider of c's world) a swept-box partner of c: one of them with
// CCD, boxes apart now (so not in the step's pair list), swept boxes
// overlapping? The swept boxes are compared first: most colliders fail there.
__device__ __forceinline__ bool ccd_swept_partner(const World& w, uint32_t c, uint32_t bc, float4 smn, float4 smx,
                                                  uint32_t d) {
    const Ccd& cd = w.ccd;
    if (d == c) return false;
    const float4 tmn = cd.sw_min[d], tmx = cd.sw_max[d];
    if (!(smn.x <= tmx.x && tmn.x <= smx.x && smn.y <= tmx.y && tmn.y <= smx.y && smn.z <= tmx.z && tmn.z <= smx.z))
        return false;
    if (!(w.c.info[d] & CI_ALIVE)) return false;
    const uint32_t bd = ccd_body_of(w, d);
    if (bc == bd || w.b.world[bc] != w.b.world[bd]) return false;
    if (!ccd_dynamic(w, bc) && !ccd_dynamic(w, bd)) return false;
    if (!ccd_enabled(w, c) && !ccd_enabled(w, d)) return false;
    const float4 amn = w.c.aabb_min[c], amx = w.c.aabb_max[c], bmn = w.c.aabb_min[d], bmx = w.c.aabb_max[d];
    return !(amn.x <= bmx.x && bmn.x <= amx.x && amn.y <= bmx.y && bmn.y <= amx.y && amn.z <= bmx.z && bmn.z <= amx.z);
}

// Which of c's partners a TOI search takes: never a pair with a sensor; the
// first search takes a pair of two CCD colliders from the smaller one only;
// a resweep skips pairs without CCD and pairs of two still bodies.
enum : int { CAND_PREDICT = 0, CAND_RESWEEP = 1 };
__device__ __forceinline__ bool ccd_keep(const World& w, int mode, uint32_t c, uint32_t d) {
    if ((w.c.info[c] | w.c.info[d]) & CI_SENSOR) return false;   // proximity pairs take no part
    if (mode == CAND_PREDICT) return !(ccd_enabled(w, d) && d < c);
    const uint32_t ch1 = c < d ? c : d, ch2 = c < d ? d : c;
    const uint32_t x1 = ccd_body_of(w, ch1), x2 = ccd_body_of(w, ch2);
    const bool s1 = (w.ccd.bflag[x1] & 1u) || !ccd_dynamic(w, x1), s2 = (w.ccd.bflag[x2] & 1u) || !ccd_dynamic(w, x2);
    return !((!ccd_enabled(w, ch1) && !ccd_enabled(w, ch2)) || (s1 && s2));
}

// One warp: c's partners during CCD that `mode` keeps, counted, or with `out`
// written there as (c, d) in slot order of d. The partners are the step's
// broad-phase pairs of c and the swept-box partners, taken from the world's
// colliders when c has CCD, else from the world's CCD colliders.
__device__ uint32_t ccd_warp_partners(const World& w, uint32_t wd, uint32_t ws, uint32_t wn, uint32_t c, int mode,
                                      uint2* out) {
    const Ccd& cd = w.ccd;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t bc = ccd_body_of(w, c);
    uint32_t n = 0;
    const uint32_t a0 = cd.adj_start[c], a1 = cd.adj_start[c + 1];
    for (uint32_t base = a0; base < a1; base += 32u) {
        const uint32_t i = base + lane;
        uint32_t d = 0;
        bool f = false;
        if (i < a1) {
            d = cd.adj_list[i];
            f = ccd_keep(w, mode, c, d);
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, f);
        if (out && f) out[n + __popc(bal & ((1u << lane) - 1u))] = make_uint2(c, d);
        n += __popc(bal);
    }
    const float4 smn = cd.sw_min[c], smx = cd.sw_max[c];
    const bool all = ccd_enabled(w, c);
    const uint32_t* src = all ? cd.order + ws : cd.ccd_list + cd.ccd_wstart[wd];
    const uint32_t sn = all ? wn : cd.ccd_wstart[wd + 1] - cd.ccd_wstart[wd];
    for (uint32_t base = 0; base < sn; base += 32u) {
        const uint32_t i = base + lane;
        uint32_t d = 0;
        bool f = false;
        if (i < sn) {
            d = src[i];
            f = ccd_swept_partner(w, c, bc, smn, smx, d) && ccd_keep(w, mode, c, d);
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, f);
        if (out && f) out[n + __popc(bal & ((1u << lane) - 1u))] = make_uint2(c, d);
        n += __popc(bal);
    }
    if (out) {
        // Both runs are in slot order: merge them by insertion.
        __syncwarp();
        if (lane == 0)
            for (uint32_t a = 1; a < n; ++a) {
                const uint2 x = out[a];
                uint32_t b = a;
                while (b > 0 && out[b - 1].y > x.y) {
                    out[b] = out[b - 1];
                    --b;
                }
                out[b] = x;
            }
        __syncwarp();
    }
    return n;
}

// The pairs a TOI search takes for the colliders src[0, ns), in that order
// and each collider's partners in slot order, handed to `batch(cand, n)` in
// runs that fit `cap` (cand: the run, n: its length; every thread calls it).
// cnt: ns + 1 words of scratch. Returns false when one collider's pairs do
// not fit.
template <class Batch>
__device__ bool ccd_candidates(const World& w, uint32_t wd, uint32_t ws, uint32_t wn, const uint32_t* src, uint32_t ns,
                               int mode, uint32_t* cnt, uint2* cand, uint32_t cap, CcdState& st, Batch batch) {
    const uint32_t warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t k = warp; k < ns; k += nw) {
        const uint32_t n = ccd_warp_partners(w, wd, ws, wn, src[k], mode, nullptr);
        if ((threadIdx.x & 31u) == 0) cnt[k] = n;
    }
    if (threadIdx.x == 0) cnt[ns] = 0u;
    __syncthreads();
    block_scan(cnt, ns + 1, st);
    for (uint32_t k0 = 0; k0 < ns;) {
        if (threadIdx.x == 0) {
            uint32_t k1 = k0;
            while (k1 < ns && cnt[k1 + 1] - cnt[k0] <= cap) ++k1;
            st.n = k1;
        }
        __syncthreads();
        const uint32_t k1 = st.n;
        __syncthreads();
        if (k1 == k0) return false;
        for (uint32_t k = k0 + warp; k < k1; k += nw)
            ccd_warp_partners(w, wd, ws, wn, src[k], mode, cand + (cnt[k] - cnt[k0]));
        __syncthreads();
        batch(cand, cnt[k1] - cnt[k0]);
        k0 = k1;
    }
    return true;
}
enum : uint32_t { PRED_NONE = 0, PRED_IMPACTS = 1, PRED_AFTER = 2 };

// predict_next_impacts for the world: the impacts up to end_time in time
// order (st.nimp in `imp`), bodies frozen at their first impact (bflag bit 0,
// ftime), or PRED_NONE / PRED_AFTER with the smallest TOI beyond end_time in
// st.min_overstep.
__device__ void ccd_predict(const World& w, const StepParams& p, uint32_t wd, uint32_t ws, uint32_t wn, uint32_t rb,
                            uint32_t rcap, CcdState& st) {
    const Ccd& cd = w.ccd;
    float2* tres = cd.tres + rb;
    CcdToi* heap = cd.heap + rb;
    CcdToi* imp = cd.impacts + rb;
    for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) cd.bflag[ccd_body_of(w, cd.order[ws + i])] &= ~1u;
    if (threadIdx.x == 0) {
        st.nheap = st.nimp = st.seq = 0;
        st.min_overstep = p.dt;
        st.stop = 0;
    }
    __syncthreads();
    // The CCD colliders' pairs, each once, in slot order.
    uint2* cand = cd.res + rb;
    const bool fits = ccd_candidates(
        w, wd, ws, wn, cd.ccd_list + cd.ccd_wstart[wd], cd.ccd_wstart[wd + 1] - cd.ccd_wstart[wd], CAND_PREDICT,
        cd.nbr2 + rb, cand, rcap, st, [&](const uint2* cl, uint32_t n) {
            ccd_mark(st, p, CCD_T_BROAD);
            for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
                const uint32_t c = cl[j].x, d = cl[j].y;
                tres[j] = ccd_toi(w, p, c < d ? c : d, c < d ? d : c, p.dt);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                for (uint32_t j = 0; j < n && !st.stop; ++j) {
                    const float2 r = tres[j];
                    if (r.x < 0.0f) continue;
                    if (r.x > st.min_overstep - r.y) continue;   // beyond this search's end
                    const float toi = r.y + r.x;
                    if (toi > st.end_time) {
                        st.min_overstep = st.min_overstep < toi ? st.min_overstep : toi;
                    } else {
                        st.min_overstep = st.end_time;
                        if (st.nheap >= rcap) {
                            st.stop = 1;
                            break;
                        }
                        const uint32_t c = cl[j].x, d = cl[j].y;
                        heap[st.nheap++] = CcdToi{toi, c < d ? c : d, c < d ? d : c, st.seq++};
                    }
                }
            }
            __syncthreads();
            ccd_mark(st, p, CCD_T_TOI);
        });
    if (threadIdx.x == 0 && !fits) st.stop = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (st.stop) st.result = PRED_NONE;
        else if (st.min_overstep == p.dt && st.nheap == 0) st.result = PRED_NONE;
        else if (st.min_overstep > st.end_time) st.result = PRED_AFTER;
        else st.result = PRED_IMPACTS;
    }
    __syncthreads();
    if (st.result != PRED_IMPACTS) return;
    // The queue, earliest TOI first (ties: discovery order).
    for (;;) {
        if (threadIdx.x == 0) {
            uint32_t best = 0xffffffffu;
            for (uint32_t k = 0; k < st.nheap; ++k) {
                if (heap[k].seq & kTocPopped) continue;
                if (best == 0xffffffffu || heap[k].toi < heap[best].toi ||
                    (heap[k].toi == heap[best].toi && (heap[k].seq & kTocSeq) < (heap[best].seq & kTocSeq)))
                    best = k;
            }
            st.cur = best;
            if (best != 0xffffffffu) {
                heap[best].seq |= kTocPopped;
                const CcdToi e = heap[best];
                const uint32_t b1 = ccd_body_of(w, e.c1), b2 = ccd_body_of(w, e.c2);
                const bool fr1 = cd.bflag[b1] & 1u, fr2 = cd.bflag[b2] & 1u;
                if (e.seq & kTocSuperseded) {
                    st.cur = 0xfffffffeu;
                } else if (fr1 && fr2) {
                    const float t1 = cd.ftime[b1], t2 = cd.ftime[b2];
                    if (e.toi == (t1 < t2 ? t2 : t1) && st.nimp < rcap) imp[st.nimp++] = e;
                    st.cur = 0xfffffffeu;
                } else {
                    if (!fr1) {
                        cd.bflag[b1] |= 1u;
                        cd.ftime[b1] = e.toi;
                    }
                    if (!fr2) {
                        cd.bflag[b2] |= 1u;
                        cd.ftime[b2] = e.toi;
                    }
                }
            }
        }
        __syncthreads();
        const uint32_t cur = st.cur;
        __syncthreads();   // read by every thread before thread 0 writes it again
        if (cur == 0xffffffffu) break;
        if (cur == 0xfffffffeu) continue;
        const CcdToi e = heap[cur];
        // Resweep every pair of the frozen bodies' colliders.
        uint32_t* src = cd.stack + rb;
        if (threadIdx.x == 0) {
            uint32_t ns = 0;
            for (int side = 0; side < 2; ++side) {
                const uint32_t fb = ccd_body_of(w, side == 0 ? e.c1 : e.c2);
                if (!ccd_dynamic(w, fb)) continue;
                for (uint32_t q = cd.bc_start[fb]; q < cd.bc_start[fb + 1]; ++q) src[ns++] = cd.bc_list[q];
            }
            st.nstack = ns;
        }
        __syncthreads();
        ccd_mark(st, p, CCD_T_TOI);
        const bool ok = ccd_candidates(
            w, wd, ws, wn, src, st.nstack, CAND_RESWEEP, cd.nbr2 + rb, cand, rcap, st, [&](const uint2* cl, uint32_t n) {
                ccd_mark(st, p, CCD_T_BROAD);
                for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
                    const uint32_t c = cl[j].x, d = cl[j].y;
                    tres[j] = ccd_toi(w, p, c < d ? c : d, c < d ? d : c, st.end_time);
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    for (uint32_t j = 0; j < n && !st.stop; ++j) {
                        const float2 r = tres[j];
                        const uint32_t c = cl[j].x, d = cl[j].y;
                        const uint32_t ch1 = c < d ? c : d, ch2 = c < d ? d : c;
                        for (uint32_t k = 0; k < st.nheap; ++k)
                            if (heap[k].c1 == ch1 && heap[k].c2 == ch2) heap[k].seq |= kTocSuperseded;
                        if (r.x < 0.0f) continue;
                        if (st.nheap >= rcap) {
                            st.stop = 1;
                            break;
                        }
                        heap[st.nheap++] = CcdToi{r.y + r.x, ch1, ch2, st.seq++};
                    }
                }
                __syncthreads();
                ccd_mark(st, p, CCD_T_TOI);
            });
        if (threadIdx.x == 0 && !ok) st.stop = 1;
        __syncthreads();
        if (threadIdx.x == 0) {
            if (st.nimp < rcap) imp[st.nimp++] = e;
            else st.stop = 1;
        }
        __syncthreads();
        if (st.stop) break;
    }
    if (threadIdx.x == 0 && st.stop) {
        atomicOr(&w.ctl->err, ERRF_CCD_CAPACITY);
        st.nimp = 0;
    }
    __syncthreads();
}

// One substep (mechanical_world.rs:624-889): the island grown from the
// impacting bodies through contacts, moved back to the latest TOI, solved
// (MoreauJeanSolver::step_ccd, moreau_jean_solver.rs:94-127) and integrated
// over the rest of the step. The island is the closure through contacts,
// found level by level: a level's pairs are those of its colliders with
// colliders not explored before it (each pair once), its bodies are
// prepared first (forces cleared, dynamics over the substep, acceleration
// without gravity, moved back to the frozen time or the latest TOI), and a
// pair with contacts explores the colliders of its other body when that is
// dynamic. The manifolds are put in collider-pair order, coloured by
// Jones-Plassmann rounds and solved colour by colour.
__device__ void ccd_substep(const World& w, const StepParams& p, uint32_t wd, uint32_t ws, uint32_t wn, uint32_t rb,
                            uint32_t rcap, CcdState& st) {
    const Ccd& cd = w.ccd;
    uint32_t* front = cd.stack + rb;        // the level's colliders
    uint32_t* next = cd.nbr + rb;           // bodies the level explored
    uint32_t* island = cd.island + rb;
    uint32_t* ccdb = cd.ccdb + rb;
    uint32_t* mlist = cd.mlist + rb;
    uint32_t* mord = cd.mord + rb;
    uint2* pairs = cd.res + rb;
    const CcdToi* imp = cd.impacts + rb;
    for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) {
        const uint32_t c = cd.order[ws + i];
        cd.cflag[c] = 0u;
        cd.bflag[ccd_body_of(w, c)] &= ~6u;
    }
    __syncthreads();
    const float last = imp[st.nimp - 1].toi;
    const float dts = p.dt - last;
    if (threadIdx.x == 0) {
        st.last = last;
        st.nstack = st.nisland = st.nccdb = st.nm = 0;
        st.stop = 0;
        for (uint32_t k = 0; k < st.nimp && !st.stop; ++k) {
            const uint32_t bs[2] = {ccd_body_of(w, imp[k].c1), ccd_body_of(w, imp[k].c2)};
            for (int s = 0; s < 2; ++s) {
                if (st.nccdb >= rcap) st.stop = 1;
                else ccdb[st.nccdb++] = bs[s];
                if (cd.bflag[bs[s]] & 4u) continue;
                cd.bflag[bs[s]] |= 4u;
                for (uint32_t q = cd.bc_start[bs[s]]; q < cd.bc_start[bs[s] + 1]; ++q) {
                    const uint32_t c = cd.bc_list[q];
                    cd.cflag[c] |= 3u;
                    if (st.nstack >= rcap) st.stop = 1;
                    else front[st.nstack++] = c;
                }
            }
        }
    }
    __syncthreads();
    StepParams ps = p;
    ps.dt = dts;
    ps.inv_dt = dts == 0.0f ? 0.0f : 1.0f / dts;
    while (st.nstack > 0 && !st.stop) {
        const uint32_t nf = st.nstack;
        if (threadIdx.x == 0) st.n = 0;
        __syncthreads();
        // The level's pairs: a warp per frontier collider, its lanes over the
        // collider's step pairs and swept-box candidates.
        {
            const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
            for (uint32_t i = warp; i < nf; i += nw) {
                const uint32_t c = front[i];
                auto consider = [&](uint32_t d) {
                    if ((w.c.info[c] | w.c.info[d]) & CI_SENSOR) return;   // a proximity pair
                    const uint32_t f = cd.cflag[d];
                    if ((f & 1u) && !(f & 2u)) return;   // its pairs were a former level's
                    if ((f & 2u) && d < c) return;       // taken from d
                    const uint32_t at = atomicAdd(&st.n, 1u);
                    if (at < rcap) pairs[at] = make_uint2(c < d ? c : d, c < d ? d : c);
                };
                for (uint32_t q = cd.adj_start[c] + lane; q < cd.adj_start[c + 1]; q += 32u) consider(cd.adj_list[q]);
                const uint32_t bc = ccd_body_of(w, c);
                const float4 smn = cd.sw_min[c], smx = cd.sw_max[c];
                const bool all = ccd_enabled(w, c);
                const uint32_t* src = all ? cd.order + ws : cd.ccd_list + cd.ccd_wstart[wd];
                const uint32_t sn = all ? wn : cd.ccd_wstart[wd + 1] - cd.ccd_wstart[wd];
                for (uint32_t k = lane; k < sn; k += 32u)
                    if (ccd_swept_partner(w, c, bc, smn, smx, src[k])) consider(src[k]);
            }
        }
        __syncthreads();
        ccd_mark(st, p, CCD_T_BROAD);
        const uint32_t np_ = st.n;
        if (np_ > rcap) {
            if (threadIdx.x == 0) st.stop = 1;
            __syncthreads();
            break;
        }
        // Its bodies, each prepared once.
        for (uint32_t i = threadIdx.x; i < np_; i += blockDim.x) {
            const uint32_t xs[2] = {ccd_body_of(w, pairs[i].x), ccd_body_of(w, pairs[i].y)};
            for (int s = 0; s < 2; ++s) {
                if (!ccd_dynamic(w, xs[s]) || (atomicOr(&cd.bflag[xs[s]], 2u) & 2u)) continue;
                ccd_prepare(w, p, xs[s], dts, last);
                const uint32_t at = atomicAdd(&st.nisland, 1u);
                if (at < rcap) island[at] = xs[s];
                else st.stop = 1;
            }
        }
        if (threadIdx.x == 0) st.nnext = 0;
        __syncthreads();
        ccd_mark(st, p, CCD_T_SOLVER);
        // Its contacts; a pair with contacts explores its other body.
        for (uint32_t i = threadIdx.x; i < np_; i += blockDim.x) {
            const uint2 pr = pairs[i];
            CcdManifold mf;
            if (ccd_contacts(w, pr.x, pr.y, mf) == 0u) continue;
            const uint32_t slot = atomicAdd(&w.ctl->ccd_mcount, 1u);
            const uint32_t at = atomicAdd(&st.nm, 1u);
            if (slot >= cd.pool_cap || at >= rcap) {
                st.stop = 1;
                continue;
            }
            cd.pool[slot] = mf;
            mlist[at] = slot;
            const uint32_t other = (cd.cflag[pr.x] & 2u) ? pr.y : pr.x;
            const uint32_t xo = ccd_body_of(w, other);
            if ((cd.cflag[other] & 2u) || !ccd_dynamic(w, xo) || (atomicOr(&cd.bflag[xo], 4u) & 4u)) continue;
            const uint32_t k = atomicAdd(&st.nnext, 1u);
            if (k < rcap) next[k] = xo;
            else st.stop = 1;
        }
        __syncthreads();
        ccd_mark(st, p, CCD_T_NARROW);
        // The next level: the colliders of the bodies explored.
        for (uint32_t i = threadIdx.x; i < nf; i += blockDim.x) cd.cflag[front[i]] &= ~2u;
        if (threadIdx.x == 0) st.nstack = 0;
        __syncthreads();
        const uint32_t nn = st.nnext;
        for (uint32_t i = threadIdx.x; i < nn && i < rcap; i += blockDim.x) {
            const uint32_t b = next[i];
            for (uint32_t q = cd.bc_start[b]; q < cd.bc_start[b + 1]; ++q) {
                const uint32_t c = cd.bc_list[q];
                cd.cflag[c] |= 3u;
                const uint32_t at = atomicAdd(&st.nstack, 1u);
                if (at < rcap) front[at] = c;
                else st.stop = 1;
            }
        }
        __syncthreads();
    }
    if (st.stop) {
        if (threadIdx.x == 0) atomicOr(&w.ctl->err, ERRF_CCD_CAPACITY);
        __syncthreads();
        return;
    }
    const uint32_t nm = st.nm, nisl = st.nisland;
    // Collider-pair order: by the first collider's place in the world's
    // slot-ordered segment, then by the second collider.
    uint32_t* cnt = cd.nbr2 + rb;
    for (uint32_t i = threadIdx.x; i <= wn; i += blockDim.x) cnt[i] = 0u;
    __syncthreads();
    auto place = [&](uint32_t c) {
        uint32_t lo = 0, hi = wn;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (cd.order[ws + mid] < c) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    };
    for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) atomicAdd(&cnt[place(cd.pool[mlist[q]].c1)], 1u);
    __syncthreads();
    block_scan(cnt, wn + 1, st);
    uint32_t* cursor = cd.nbr + rb;
    for (uint32_t i = threadIdx.x; i <= wn; i += blockDim.x) cursor[i] = cnt[i];
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) {
        const uint32_t slot = mlist[q];
        mord[atomicAdd(&cursor[place(cd.pool[slot].c1)], 1u)] = slot;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) {
        uint32_t* l = mord + cnt[i];
        const uint32_t n = cnt[i + 1] - cnt[i];
        for (uint32_t a = 1; a < n; ++a) {
            const uint32_t x = l[a], kx = cd.pool[x].c2;
            uint32_t b = a;
            while (b > 0 && cd.pool[l[b - 1]].c2 > kx) {
                l[b] = l[b - 1];
                --b;
            }
            l[b] = x;
        }
    }
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) mlist[q] = mord[q];
    // The manifolds on each island body (CSR: bcount over the island's
    // bodies, numbered through bepoch).
    uint32_t* bstart = cd.nbr + rb;
    uint32_t* blist = reinterpret_cast<uint32_t*>(pairs);   // 2 rcap words
    // Per manifold (by place q): its priority, colour and island bodies.
    unsigned long long* prio = reinterpret_cast<unsigned long long*>(cd.tres + rb);
    uint32_t* mcol = reinterpret_cast<uint32_t*>(cd.heap + rb);          // rcap words
    uint2* mbody = reinterpret_cast<uint2*>(mcol + 2 * (size_t)rcap);   // rcap pairs
    const uint32_t base = cd.order[ws];
    for (uint32_t i = threadIdx.x; i < nisl; i += blockDim.x) {
        cd.bepoch[island[i]] = i;
        bstart[i] = 0u;
    }
    if (threadIdx.x == 0) bstart[nisl] = 0u;
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) {
        const CcdManifold& m = cd.pool[mlist[q]];
        prio[q] = ccd_priority(base, m);
        mcol[q] = 0xffffffffu;
        uint32_t k[2] = {0xffffffffu, 0xffffffffu};
        for (int s = 0; s < 2; ++s) {
            const uint32_t x = ccd_body_of(w, s == 0 ? m.c1 : m.c2);
            if (!ccd_dynamic(w, x)) continue;
            k[s] = cd.bepoch[x];
            atomicAdd(&bstart[k[s]], 1u);
        }
        mbody[q] = make_uint2(k[0], k[1]);
    }
    __syncthreads();
    block_scan(bstart, nisl + 1, st);
    uint32_t* bcur = cnt;
    for (uint32_t i = threadIdx.x; i <= nisl; i += blockDim.x) bcur[i] = bstart[i];
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) {
        const uint2 k = mbody[q];
        if (k.x != 0xffffffffu) blist[atomicAdd(&bcur[k.x], 1u)] = q;
        if (k.y != 0xffffffffu) blist[atomicAdd(&bcur[k.y], 1u)] = q;
    }
    if (threadIdx.x == 0) st.left = nm;
    __syncthreads();
    // Jones-Plassmann rounds: round r colours the manifolds whose priority
    // is above every uncoloured manifold's on a shared dynamic body.
    uint32_t ncol = 0;
    for (; st.left > 0 && ncol < kCcdColours; ++ncol) {
        for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) {
            mord[q] = 0u;
            if (mcol[q] != 0xffffffffu) continue;
            const unsigned long long pq = prio[q];
            const uint2 kb = mbody[q];
            bool top = true;
            for (int s = 0; s < 2 && top; ++s) {
                const uint32_t k = s == 0 ? kb.x : kb.y;
                if (k == 0xffffffffu) continue;
                for (uint32_t e = bstart[k]; e < bstart[k + 1]; ++e) {
                    const uint32_t o = blist[e];
                    if (o != q && mcol[o] == 0xffffffffu && prio[o] > pq) {
                        top = false;
                        break;
                    }
                }
            }
            mord[q] = top ? 1u : 0u;
        }
        __syncthreads();
        uint32_t taken = 0;
        for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x)
            if (mord[q]) {
                mcol[q] = ncol;
                ++taken;
            }
        atomicSub(&st.left, taken);
        __syncthreads();
    }
    if (st.left > 0) {
        if (threadIdx.x == 0) atomicOr(&w.ctl->err, ERRF_CCD_CAPACITY);
        __syncthreads();
        return;
    }
    // The manifolds by colour.
    for (uint32_t k = threadIdx.x; k <= kCcdColours; k += blockDim.x) {
        st.col_start[k] = 0u;
        if (k < kCcdColours) st.col_fill[k] = 0u;
    }
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) atomicAdd(&st.col_start[mcol[q]], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t k = 0; k <= kCcdColours; ++k) {
            const uint32_t v = st.col_start[k];
            st.col_start[k] = run;
            run += v;
        }
    }
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) {
        // Within a colour the manifolds share no dynamic body: any order.
        const uint32_t k = mcol[q];
        mord[st.col_start[k] + atomicAdd(&st.col_fill[k], 1u)] = mlist[q];
    }
    __syncthreads();
    // The island's solve runs in k_ccd_solve, with more threads a world.
    uint32_t* S = cd.wstate + kCcdStateWords * (size_t)wd;
    for (uint32_t k = threadIdx.x; k <= ncol; k += blockDim.x) cd.wcols[(kCcdColours + 1) * (size_t)wd + k] = st.col_start[k];
    ccd_mark(st, p, CCD_T_SOLVER);
    if (threadIdx.x == 0) {
        S[CS_DTS] = __float_as_uint(dts);
        S[CS_NM] = nm;
        S[CS_NCOL] = ncol;
        S[CS_NISL] = nisl;
        S[CS_NCCDB] = st.nccdb;
        S[CS_NIMP] = st.nimp;
        S[CS_PENDING] = 1u;
    }
    __syncthreads();
}

// step_ccd for a world whose pass prepared a substep island
// (MoreauJeanSolver::step_ccd, moreau_jean_solver.rs:94-127): the rows, the
// position solve, validate_advancement of the impacting bodies, the velocity
// solve, the island's integration and update_dynamics over the substep. A
// kernel of its own so that a world gets more threads than the pass kernel's
// registers allow.
__global__ void __launch_bounds__(kCcdSolveThreads, 2) k_ccd_solve(World w, StepParams p) {
    __shared__ uint32_t col_start[kCcdColours + 1];
    const Ccd& cd = w.ccd;
    const uint32_t wd = blockIdx.x;
    if (wd >= cd.n_worlds || !cd.wflag[wd]) return;
    uint32_t* S = cd.wstate + kCcdStateWords * (size_t)wd;
    if (!S[CS_PENDING]) return;
    const unsigned long long t0 = p.profile ? global_ns() : 0ull;
    const uint32_t ws = cd.wstart[wd], wn = cd.wstart[wd + 1] - ws;
    const uint32_t rb = kCcdRegion * ws + kCcdSlack * wd;
    const float dts = __uint_as_float(S[CS_DTS]);
    const uint32_t nm = S[CS_NM], ncol = S[CS_NCOL], nisl = S[CS_NISL], nccdb = S[CS_NCCDB], nimp = S[CS_NIMP];
    for (uint32_t k = threadIdx.x; k <= ncol; k += blockDim.x) col_start[k] = cd.wcols[(kCcdColours + 1) * (size_t)wd + k];
    const uint32_t* island = cd.island + rb;
    const uint32_t* ccdb = cd.ccdb + rb;
    const uint32_t* mlist = cd.mlist + rb;
    const uint32_t* mord = cd.mord + rb;
    StepParams ps = p;
    ps.dt = dts;
    ps.inv_dt = dts == 0.0f ? 0.0f : 1.0f / dts;
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < nm; q += blockDim.x) ccd_rows(w, ps, cd.pool[mlist[q]], dts);
    for (uint32_t i = threadIdx.x; i < nisl; i += blockDim.x)
        for (int k = 0; k < 6; ++k) w.b.dv[6 * (size_t)island[i] + k] = 0.0f;
    __syncthreads();
    for (uint32_t it = 0; it < cd.max_position_iterations; ++it)
        for (uint32_t k = 0; k < ncol; ++k) {
            for (uint32_t q = col_start[k] + threadIdx.x; q < col_start[k + 1]; q += blockDim.x) {
                ccd_position_manifold(w, ps, cd.pool[mord[q]]);
            }
            __syncthreads();
        }
    for (uint32_t k = threadIdx.x; k < nccdb; k += blockDim.x) {
        const uint32_t h = ccdb[k];
        cd.pos0_t[h] = w.b.pos_t[h];
        cd.pos0_q[h] = w.b.pos_q[h];
    }
    __syncthreads();
    for (uint32_t it = 0; it < p.max_velocity_iterations; ++it)
        for (int pass = 0; pass < 2; ++pass)
            for (uint32_t k = 0; k < ncol; ++k) {
                for (uint32_t q = col_start[k] + threadIdx.x; q < col_start[k + 1]; q += blockDim.x)
                    ccd_manifold_velocity(w, cd.pool[mord[q]], pass == 0);
                __syncthreads();
            }
    for (uint32_t i = threadIdx.x; i < nisl; i += blockDim.x) {
        const uint32_t h = island[i];
        const Bodies& b = w.b;
        const np::V el = np::mul(v3(b.acc_lin[h]), dts), ea = np::mul(v3(b.acc_ang[h]), dts);
        const float* d = b.dv + 6 * (size_t)h;
        b.lin[h] = f4(np::add(np::add(v3(b.lin[h]), el), np::mk(d[0], d[1], d[2])));
        b.ang[h] = f4(np::add(np::add(v3(b.ang[h]), ea), np::mk(d[3], d[4], d[5])));
        b.info[h] |= BI_CHANGED;
        body_integrate(b, h, dts);
    }
    __syncthreads();
    // update_dynamics over the substep for the world's changed bodies
    // (mechanical_world.rs:870-876), before anything moves them again;
    // bodies without colliders take it in k_ccd_finish.
    for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) {
        const uint32_t c = cd.order[ws + i], bb = ccd_body_of(w, c);
        if (cd.bc_list[cd.bc_start[bb]] != c) continue;   // one collider per body acts
        if ((w.b.info[bb] & BI_CHANGED) && ccd_dynamic(w, bb)) body_update_dynamics(w.b, bb, dts);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        w.ccd.wdts[wd] = dts;
        atomicAdd(&w.ctl->ccd_substeps, 1u);
        atomicAdd(&w.ctl->ccd_impacts, nimp);
        S[CS_PENDING] = 0u;
        if (p.profile) ccd_account(w, S, CCD_T_SOLVER, global_ns() - t0);
    }
}


// One pass of solve_ccd's loop for world blockIdx.x (at most
// max_ccd_substeps + 2 passes, one launch each): the swept boxes, the
// prediction, then either a substep's island for k_ccd_solve or, on the last
// pass, the clamp of the frozen bodies.
__global__ void __launch_bounds__(kCcdThreads) k_ccd_world(World w, StepParams p, uint32_t pass) {
    __shared__ CcdState st;
    const Ccd& cd = w.ccd;
    const uint32_t wd = blockIdx.x;
    if (wd >= cd.n_worlds) return;
    if (pass == 0 && threadIdx.x == 0) cd.wdts[wd] = -1.0f;   // no substep (yet) this step
    if (!cd.wflag[wd]) return;
    uint32_t* S = cd.wstate + kCcdStateWords * (size_t)wd;
    if (pass > 0 && S[CS_DONE]) return;
    const uint32_t ws = cd.wstart[wd], wn = cd.wstart[wd + 1] - ws;
    const uint32_t rb = kCcdRegion * ws + kCcdSlack * wd, rcap = kCcdRegion * wn + kCcdSlack;
    const float dt0 = p.dt;
    const float sub = dt0 / (float)cd.substeps;
    if (pass == 0)
        for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) {
            const uint32_t b = ccd_body_of(w, cd.order[ws + i]);
            cd.btime[b] = 0.0f;
            cd.bepoch[b] = 0u;
        }
    if (threadIdx.x == 0) {
        if (pass == 0) {
            S[CS_PENDING] = 0u;
            *reinterpret_cast<unsigned long long*>(S + CS_TOTAL) = 0ull;
        }
        st.end_time = pass == 0 ? 0.0f : __uint_as_float(S[CS_END]);
        st.last_iter = pass == 0 ? 0u : S[CS_LAST_ITER];
        st.epoch = 0;
        st.t_mark = p.profile ? global_ns() : 0ull;
        for (int k = 0; k < 4; ++k) st.t_acc[k] = 0ull;
        // Each pass either advances end_time by a substep or is the last.
        if (st.end_time < dt0) {
            const float e = st.end_time + sub;
            st.end_time = e < dt0 ? e : dt0;
        } else {
            st.last_iter = 1;
        }
    }
    for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) ccd_sweep_box(w, cd.order[ws + i]);
    __syncthreads();
    ccd_mark(st, p, CCD_T_BROAD);
    ccd_predict(w, p, wd, ws, wn, rb, rcap, st);
    if (st.result == PRED_AFTER) {
        if (threadIdx.x == 0) {
            const float e = floorf(st.min_overstep / sub) * sub + sub;
            st.end_time = e < dt0 ? e : dt0;
        }
        __syncthreads();
        ccd_predict(w, p, wd, ws, wn, rb, rcap, st);
        if (threadIdx.x == 0 && st.result != PRED_IMPACTS) st.nimp = 0;
        __syncthreads();
    } else if (st.result == PRED_NONE) {
        if (threadIdx.x == 0) st.nimp = 0;
        __syncthreads();
    }
    bool done = false;
    if (!st.last_iter && st.nimp > 0) {
        ccd_substep(w, p, wd, ws, wn, rb, rcap, st);
    } else {
        // The bodies frozen by the last prediction stay at their safe poses.
        for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) {
            const uint32_t c = cd.order[ws + i], b = ccd_body_of(w, c);
            if (cd.bc_list[cd.bc_start[b]] != c) continue;   // one collider per body acts
            if ((cd.bflag[b] & 1u) && bi_status(w.b.info[b]) != 1u) ccd_clamp(w, b);
        }
        done = true;
    }
    __syncthreads();
    ccd_mark(st, p, CCD_T_SOLVER);
    if (threadIdx.x == 0) {
        S[CS_END] = __float_as_uint(st.end_time);
        S[CS_LAST_ITER] = st.last_iter;
        S[CS_DONE] = done ? 1u : 0u;
        if (p.profile)
            for (int k = 0; k < 4; ++k) ccd_account(w, S, k, st.t_acc[k]);
    }
}

// The step's broad-phase pairs by collider (both ends), partners in slot
// order: counts, then (after an exclusive scan of the counts into adj_start)
// the lists, then each list sorted.
__global__ void k_ccd_adj_count(World w) {
    const uint32_t np_ = w.ctl->npairs < w.cap_pairs ? w.ctl->npairs : w.cap_pairs;
    GRID_FOR(q, np_) {
        const uint2 pr = w.cur.pair[q];
        atomicAdd(&w.ccd.adj_count[pr.x], 1u);
        atomicAdd(&w.ccd.adj_count[pr.y], 1u);
    }
}
__global__ void k_ccd_adj_fill(World w) {
    const uint32_t np_ = w.ctl->npairs < w.cap_pairs ? w.ctl->npairs : w.cap_pairs;
    GRID_FOR(q, np_) {
        const uint2 pr = w.cur.pair[q];
        w.ccd.adj_list[w.ccd.adj_start[pr.x] + atomicAdd(&w.ccd.adj_count[pr.x], 1u)] = pr.y;
        w.ccd.adj_list[w.ccd.adj_start[pr.y] + atomicAdd(&w.ccd.adj_count[pr.y], 1u)] = pr.x;
    }
}
__global__ void k_ccd_adj_sort(World w) {
    GRID_FOR(c, w.nc_slots) {
        uint32_t* l = w.ccd.adj_list + w.ccd.adj_start[c];
        const uint32_t n = w.ccd.adj_start[c + 1] - w.ccd.adj_start[c];
        for (uint32_t i = 1; i < n; ++i) {
            const uint32_t x = l[i];
            uint32_t j = i;
            while (j > 0 && l[j - 1] > x) {
                l[j] = l[j - 1];
                --j;
            }
            l[j] = x;
        }
    }
}

// Start of a step with CCD: position0 of every body (RigidBody::step_started,
// rigid_body.rs:517-519) and the step's CCD counters.
__global__ void k_ccd_begin(World w) {
    GRID_FOR(i, w.nb_slots) {
        w.ccd.pos0_t[i] = w.b.pos_t[i];
        w.ccd.pos0_q[i] = w.b.pos_q[i];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.ctl->ccd_mcount = 0;
        w.ctl->ccd_substeps = 0;
        w.ctl->ccd_impacts = 0;
        for (int k = 0; k < 4; ++k) w.ctl->ccd_ns[k] = 0ull;
        w.ctl->ccd_max_ns = 0ull;
    }
}

// After the worlds' CCD: update_dynamics over the last substep's length for
// the changed bodies without colliders of worlds that had one
// (mechanical_world.rs:870-876; their state does not change during CCD, so
// the last substep's update is theirs), the update flags cleared, and the
// kinetic-energy audit of the final state.
__global__ void k_ccd_finish(World w) {
    __shared__ double sh[32];
    const Bodies& b = w.b;
    double ke = 0.0;
    GRID_FOR(i, w.nb_slots) {
        const uint32_t info = b.info[i];
        if (!(info & BI_ALIVE)) continue;
        const uint32_t st = bi_status(info), wd = b.world[i];
        const float dts = wd < w.ccd.n_worlds ? w.ccd.wdts[wd] : -1.0f;
        if (dts >= 0.0f && (info & BI_CHANGED) && st == 2u && w.ccd.bc_start[i] == w.ccd.bc_start[i + 1])
            body_update_dynamics(b, i, dts);
        b.f_lin[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        b.f_ang[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        b.info[i] = b.info[i] & ~BI_CHANGED;
        if (st == 2u) {
            float4 l = b.lin[i], a = b.ang[i];
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
