// oracle_capi.cpp -- extern "C" face of the CPU oracle (test infrastructure only).
//
// Mirrors the npgpu_* entry points of include/npgpu.h so that a test can
// drive the oracle and the GPU world with the same calls. Loaded by the tests,
// the smoke check and the CPU-baseline leg of the benchmark, never by the product.
#include <cstring>
#include <memory>
#include <vector>
#include "ref_world.hpp"

using namespace oracle;

struct OracleBase {
    virtual ~OracleBase() {}
};
template <class R> struct OracleImpl : OracleBase {
    World<R> w;
    OracleImpl(const npgpu_params& p, const float g[3]) : w(p, g) {}
};

struct orc_world {
    int precision;
    std::unique_ptr<OracleBase> impl;
};

template <class R> static World<R>& W(orc_world* o) { return static_cast<OracleImpl<R>*>(o->impl.get())->w; }

#define DISPATCH(o, expr)                   \
    do {                                    \
        if ((o)->precision == 64) {         \
            auto& w = W<double>(o);         \
            expr;                           \
        } else {                            \
            auto& w = W<float>(o);          \
            expr;                           \
        }                                   \
    } while (0)

template <class R> static void contact_out(const World<R>& w, const Manifold<R>& m, const MContact<R>& k, npgpu_contact& o) {
    o.collider1 = m.c1;
    o.collider2 = m.c2;
    o.feature_key = k.key();
    Approx<R> a1 = w.feature(w.colliders[m.c1], k.fid1), a2 = w.feature(w.colliders[m.c2], k.fid2);
    o.kinematic = uint32_t(a1.kind) | (uint32_t(a2.kind) << 8);
    o.world1[0] = float(k.g.world1.x); o.world1[1] = float(k.g.world1.y); o.world1[2] = float(k.g.world1.z);
    o.world2[0] = float(k.g.world2.x); o.world2[1] = float(k.g.world2.y); o.world2[2] = float(k.g.world2.z);
    o.normal[0] = float(k.g.normal.x); o.normal[1] = float(k.g.normal.y); o.normal[2] = float(k.g.normal.z);
    o.depth = float(k.g.depth);
    for (int s = 0; s < 3; ++s) o.impulse[s] = float(k.impulse[s]);
    o.colour = m.colour;
}

extern "C" {

orc_world* orc_create(int precision, const npgpu_params* p, const float gravity[3]) {
    orc_world* o = new orc_world;
    o->precision = precision == 64 ? 64 : 32;
    if (o->precision == 64) o->impl.reset(new OracleImpl<double>(*p, gravity));
    else o->impl.reset(new OracleImpl<float>(*p, gravity));
    return o;
}

void orc_destroy(orc_world* o) { delete o; }

void orc_set_order(orc_world* o, int order) { DISPATCH(o, w.order = order); }
void orc_mlp_set(orc_world* o, const float* params, uint32_t n) { DISPATCH(o, w.set_mlp(params, n)); }

void orc_set_params(orc_world* o, const npgpu_params* p) { DISPATCH(o, w.params = *p); }

double orc_collider_distance(orc_world* o, uint32_t c1, uint32_t c2, double dir[3]) {
    double d = 0.0;
    DISPATCH(o, {
        auto v = decltype(w.bodies[0].lin){};
        d = double(w.collider_distance(c1, c2, v));
        dir[0] = double(v.x);
        dir[1] = double(v.y);
        dir[2] = double(v.z);
    });
    return d;
}

int orc_pair_toi(orc_world* o, uint32_t c1, uint32_t c2, double horizon, double* toi) {
    int r = -1;
    DISPATCH(o, {
        using Rw = decltype(w.cur_dt);
        Rw t = Rw(0);
        r = w.pair_toi(c1, c2, Rw(horizon), t);
        *toi = double(t);
    });
    return r;
}

int orc_upsert_bodies(orc_world* o, uint32_t n, const npgpu_handle* h, const npgpu_body_desc* d) {
    for (uint32_t i = 0; i < n; ++i) {
        int s = 0;
        DISPATCH(o, s = w.upsert_body(h[i], d[i]));
        if (s) return s;
    }
    return 0;
}

int orc_upsert_colliders(orc_world* o, uint32_t n, const npgpu_handle* h, const npgpu_collider_desc* d) {
    for (uint32_t i = 0; i < n; ++i) {
        int s = 0;
        DISPATCH(o, s = w.upsert_collider(h[i], d[i]));
        if (s) return s;
    }
    return 0;
}

int orc_remove_bodies(orc_world* o, uint32_t n, const npgpu_handle* h) {
    for (uint32_t i = 0; i < n; ++i) {
        int s = 0;
        DISPATCH(o, s = w.remove_body(h[i]));
        if (s) return s;
    }
    return 0;
}

int orc_remove_colliders(orc_world* o, uint32_t n, const npgpu_handle* h) {
    for (uint32_t i = 0; i < n; ++i) {
        int s = 0;
        DISPATCH(o, s = w.remove_collider(h[i]));
        if (s) return s;
    }
    return 0;
}

int orc_upsert_joints(orc_world* o, uint32_t n, const npgpu_handle* h, const npgpu_joint_desc* d) {
    for (uint32_t i = 0; i < n; ++i) {
        int s = 0;
        DISPATCH(o, s = w.upsert_joint(h[i], d[i]));
        if (s) return s;
    }
    return 0;
}

int orc_remove_joints(orc_world* o, uint32_t n, const npgpu_handle* h) {
    for (uint32_t i = 0; i < n; ++i) {
        int s = 0;
        DISPATCH(o, s = w.remove_joint(h[i]));
        if (s) return s;
    }
    return 0;
}

// Per joint: 7 impulses (f64: linear 3, angular 3, the limit's), then broken and active flags.
int orc_get_joints(orc_world* o, uint32_t n, const npgpu_handle* h, double* imp7, uint32_t* flags2) {
    int s = 0;
    DISPATCH(o, {
        for (uint32_t i = 0; i < n && !s; ++i) {
            if (h[i].index >= w.joints.size() || !w.joints[h[i].index].alive ||
                w.joints[h[i].index].generation != h[i].generation) {
                s = NPGPU_ERR_INVALID_HANDLE;
                break;
            }
            const auto& j = w.joints[h[i].index];
            for (int k = 0; k < 7; ++k) imp7[7 * i + k] = double(j.imp[k]);
            flags2[2 * i] = j.broken ? 1u : 0u;
            flags2[2 * i + 1] = j.active ? 1u : 0u;
        }
    });
    return s;
}

int orc_apply_forces(orc_world* o, uint32_t n, const npgpu_handle* h, const float* f, int wake) {
    for (uint32_t i = 0; i < n; ++i) {
        int s = 0;
        DISPATCH(o, s = w.apply_force(h[i], f + 6 * i, wake != 0));
        if (s) return s;
    }
    return 0;
}

int orc_step(orc_world* o, uint32_t nsteps) {
    for (uint32_t i = 0; i < nsteps; ++i) {
        int s = 0;
        DISPATCH(o, s = w.step());
        if (s) return s;
    }
    return 0;
}

// Runs only collision detection (sync, broad phase, narrow phase) on the
// current poses: used to compare pair sets and manifolds on given states.
void orc_collision_detection(orc_world* o) { DISPATCH(o, w.collision_detection()); }

// Positions / velocities as f64 (exact for both precisions).
int orc_download_bodies(orc_world* o, uint32_t first, uint32_t n, double* pos, double* vel, double* energy,
                        uint8_t* active) {
    DISPATCH(o, {
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t s = first + i;
            if (s >= w.bodies.size()) return NPGPU_ERR_INVALID_ARGUMENT;
            const auto& b = w.bodies[s];
            if (pos) {
                double* p = pos + 7 * i;
                p[0] = b.pos.t.x; p[1] = b.pos.t.y; p[2] = b.pos.t.z;
                p[3] = b.pos.q.i; p[4] = b.pos.q.j; p[5] = b.pos.q.k; p[6] = b.pos.q.w;
            }
            if (vel) {
                double* v = vel + 6 * i;
                v[0] = b.lin.x; v[1] = b.lin.y; v[2] = b.lin.z; v[3] = b.ang.x; v[4] = b.ang.y; v[5] = b.ang.z;
            }
            if (energy) energy[i] = double(b.energy);
            if (active) active[i] = b.is_active() ? 1 : 0;
        }
    });
    return 0;
}

int orc_download_mass_properties(orc_world* o, uint32_t first, uint32_t n, double* inertia7, double* com3) {
    DISPATCH(o, {
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t s = first + i;
            if (s >= w.bodies.size()) return NPGPU_ERR_INVALID_ARGUMENT;
            const auto& b = w.bodies[s];
            const auto& a = b.local_inertia.angular;
            double* I = inertia7 + 7 * i;
            I[0] = b.local_inertia.linear;
            I[1] = a.m[0][0]; I[2] = a.m[0][1]; I[3] = a.m[0][2]; I[4] = a.m[1][1]; I[5] = a.m[1][2]; I[6] = a.m[2][2];
            com3[3 * i + 0] = b.local_com.x; com3[3 * i + 1] = b.local_com.y; com3[3 * i + 2] = b.local_com.z;
        }
    });
    return 0;
}

// Sets pose and velocity of slots without touching anything else (state injection for tests).
int orc_set_body_state(orc_world* o, uint32_t first, uint32_t n, const float* pos, const float* vel) {
    DISPATCH(o, {
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t s = first + i;
            if (s >= w.bodies.size()) return NPGPU_ERR_INVALID_ARGUMENT;
            auto& b = w.bodies[s];
            if (pos) {
                const float* p = pos + 7 * i;
                b.pos.t.x = p[0]; b.pos.t.y = p[1]; b.pos.t.z = p[2];
                b.pos.q.i = p[3]; b.pos.q.j = p[4]; b.pos.q.k = p[5]; b.pos.q.w = p[6];
                b.com = iso_pt(b.pos, b.local_com);
            }
            if (vel) {
                const float* v = vel + 6 * i;
                b.lin.x = v[0]; b.lin.y = v[1]; b.lin.z = v[2];
                b.ang.x = v[3]; b.ang.y = v[4]; b.ang.z = v[5];
            }
            b.changed = true;
        }
        w.cd_dirty = true;
    });
    return 0;
}

uint32_t orc_get_pairs(orc_world* o, uint32_t* out, uint32_t max) {
    uint32_t n = 0;
    DISPATCH(o, {
        n = uint32_t(w.pairs.size());
        for (uint32_t i = 0; i < n && i < max; ++i) {
            out[2 * i] = uint32_t(w.pairs[i] >> 32);
            out[2 * i + 1] = uint32_t(w.pairs[i] & 0xffffffffu);
        }
    });
    return n;
}

// Contact events of the last step as (collider1, collider2, stopped), in the
// order the passes produced them.
void orc_record_events(orc_world* o, int on) {
    DISPATCH(o, {
        w.record_events = on != 0;
        w.events.clear();
        w.prox_events.clear();
    });
}
uint32_t orc_contact_events(orc_world* o, uint32_t* out3, uint32_t max) {
    uint32_t n = 0;
    DISPATCH(o, {
        n = uint32_t(w.events.size());
        for (uint32_t i = 0; i < n && i < max; ++i)
            for (int k = 0; k < 3; ++k) out3[3 * i + k] = w.events[i][k];
    });
    return n;
}

// Proximity events of the last step as (collider1, collider2, previous, new),
// in the order the passes produced them.
uint32_t orc_proximity_events(orc_world* o, uint32_t* out4, uint32_t max) {
    uint32_t n = 0;
    DISPATCH(o, {
        n = uint32_t(w.prox_events.size());
        for (uint32_t i = 0; i < n && i < max; ++i)
            for (int k = 0; k < 4; ++k) out4[4 * i + k] = w.prox_events[i][k];
    });
    return n;
}

// Ray queries by brute force over the alive colliders: (ray, collider, toi,
// nx, ny, nz) per hit as doubles, in ray then collider order.
uint32_t orc_rays(orc_world* o, uint32_t n, const float* rays6, const float* max_toi, uint32_t world, double* out6,
                  uint32_t max) {
    uint32_t cnt = 0;
    DISPATCH(o, {
        using R = typename std::remove_reference<decltype(w)>::type::Real;
        for (uint32_t r = 0; r < n; ++r) {
            V3<R> org = v3<R>(R(rays6[6 * r]), R(rays6[6 * r + 1]), R(rays6[6 * r + 2]));
            V3<R> dir = v3<R>(R(rays6[6 * r + 3]), R(rays6[6 * r + 4]), R(rays6[6 * r + 5]));
            for (uint32_t c = 0; c < w.colliders.size(); ++c) {
                const auto& col = w.colliders[c];
                if (!col.alive || !w.in_world(col, world)) continue;
                R toi;
                V3<R> nn;
                if (!w.ray_shape(col, org, dir, R(max_toi[r]), toi, nn)) continue;
                if (cnt < max) {
                    double* q = out6 + 6 * cnt;
                    q[0] = r; q[1] = c; q[2] = double(toi); q[3] = double(nn.x); q[4] = double(nn.y); q[5] = double(nn.z);
                }
                ++cnt;
            }
        }
    });
    return cnt;
}

// Point (kind 1) or fat-AABB (kind 2) queries: (query, collider) pairs.
uint32_t orc_overlaps(orc_world* o, int kind, uint32_t n, const float* q, uint32_t world, uint32_t* out2, uint32_t max) {
    uint32_t cnt = 0;
    DISPATCH(o, {
        using R = typename std::remove_reference<decltype(w)>::type::Real;
        for (uint32_t i = 0; i < n; ++i) {
            for (uint32_t c = 0; c < w.colliders.size(); ++c) {
                const auto& col = w.colliders[c];
                if (!col.alive || !w.in_world(col, world)) continue;
                bool hit;
                if (kind == 1) {
                    V3<R> p = v3<R>(R(q[3 * i]), R(q[3 * i + 1]), R(q[3 * i + 2]));
                    hit = col.has_fat && R(q[3 * i]) >= col.aabb_min[0] && R(q[3 * i]) <= col.aabb_max[0] &&
                          R(q[3 * i + 1]) >= col.aabb_min[1] && R(q[3 * i + 1]) <= col.aabb_max[1] &&
                          R(q[3 * i + 2]) >= col.aabb_min[2] && R(q[3 * i + 2]) <= col.aabb_max[2] &&
                          w.point_in_shape(col, p);
                } else {
                    hit = col.has_fat;
                    for (int a = 0; a < 3 && hit; ++a)
                        hit = R(q[6 * i + a]) <= col.aabb_max[a] && col.aabb_min[a] <= R(q[6 * i + 3 + a]);
                }
                if (!hit) continue;
                if (cnt < max) {
                    out2[2 * cnt] = i;
                    out2[2 * cnt + 1] = c;
                }
                ++cnt;
            }
        }
    });
    return cnt;
}

uint32_t orc_brute_force_pairs(orc_world* o, uint32_t* out, uint32_t max) {
    uint32_t n = 0;
    DISPATCH(o, {
        std::vector<uint64_t> p = w.broad_phase_brute_force();
        n = uint32_t(p.size());
        for (uint32_t i = 0; i < n && i < max; ++i) {
            out[2 * i] = uint32_t(p[i] >> 32);
            out[2 * i + 1] = uint32_t(p[i] & 0xffffffffu);
        }
    });
    return n;
}

int orc_get_aabbs(orc_world* o, uint32_t first, uint32_t n, double* out) {
    DISPATCH(o, {
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t s = first + i;
            if (s >= w.colliders.size()) return NPGPU_ERR_INVALID_ARGUMENT;
            for (int a = 0; a < 3; ++a) {
                out[6 * i + a] = w.colliders[s].aabb_min[a];
                out[6 * i + 3 + a] = w.colliders[s].aabb_max[a];
            }
        }
    });
    return 0;
}

uint32_t orc_get_contacts(orc_world* o, npgpu_contact* out, uint32_t max) {
    uint32_t n = 0;
    DISPATCH(o, {
        for (auto& kv : w.manifolds) {
            const auto& m = kv.second;
            for (const auto& k : m.contacts) {
                if (n < max) contact_out(w, m, k, out[n]);
                ++n;
            }
        }
    });
    return n;
}

// Contacts as f64: world1[3], world2[3], normal[3], depth, impulse[3] (13 doubles each).
uint32_t orc_get_contacts_f64(orc_world* o, double* out, uint32_t max) {
    uint32_t n = 0;
    DISPATCH(o, {
        for (auto& kv : w.manifolds) {
            for (const auto& k : kv.second.contacts) {
                if (n < max) {
                    double* p = out + 13 * n;
                    p[0] = k.g.world1.x; p[1] = k.g.world1.y; p[2] = k.g.world1.z;
                    p[3] = k.g.world2.x; p[4] = k.g.world2.y; p[5] = k.g.world2.z;
                    p[6] = k.g.normal.x; p[7] = k.g.normal.y; p[8] = k.g.normal.z;
                    p[9] = k.g.depth;
                    p[10] = k.impulse[0]; p[11] = k.impulse[1]; p[12] = k.impulse[2];
                }
                ++n;
            }
        }
    });
    return n;
}

void orc_get_counters(orc_world* o, npgpu_counters* c) { DISPATCH(o, *c = w.counters); }

const char* orc_last_error(orc_world* o) {
    const char* s = "";
    DISPATCH(o, s = w.last_error.c_str());
    return s;
}

}  // extern "C"
