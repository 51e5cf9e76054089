// npgpu_world.cu -- host side of the GPU mechanical world and the C ABI of
// include/npgpu.h.
//
// The host keeps what the reference's sets and GeometricalWorld keep on the
// CPU (handles, generations, the mass bookkeeping of collider insertion and
// removal, src/world/geometrical_world.rs:102-227); everything the step
// touches lives on the device (world_dev.cuh).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/npgpu.h"
#include "world_dev.cuh"
#include "mlp.cuh"

using namespace npgpu_dev;

namespace {

struct HostBody {
    bool alive = false;
    uint64_t gen = 0;
    uint32_t kind = 0, status = 0, flags = 0, world = 0;
    float mass = 0.0f;
    np::M local_I;
    np::V local_com{0.0f, 0.0f, 0.0f};
};

struct HostCollider {
    bool alive = false;
    bool registered = false;
    uint64_t gen = 0;
    npgpu_collider_desc desc;
};

struct HostJoint {
    bool alive = false;
    uint64_t gen = 0;
    npgpu_joint_desc desc;
};

bool finite_n(const float* v, int n) {
    for (int k = 0; k < n; ++k)
        if (!std::isfinite(v[k])) return false;
    return true;
}

// Volumetric::transformed_mass_properties for Ball / Cuboid / Capsule
// (src/volumetric/volumetric.rs:55-59, volumetric_ball.rs:8-47, volumetric_cuboid.rs:9-78,
// volumetric_capsule.rs:7-37 with volumetric_cylinder.rs:7-60).
void collider_mass_properties(const npgpu_collider_desc& d, np::V& com, float& mass, np::M& ang) {
    const float pi = 3.14159265358979323846f;
    np::M unit = np::mzero();
    if (d.shape == NPGPU_SHAPE_BALL) {
        float r = d.shape_params[0];
        float vol = pi * r * r * r * (float)(4.0 / 3.0);
        mass = vol * d.density;
        float diag = r * r * (float)(2.0 / 5.0);
        unit.m[0][0] = unit.m[1][1] = unit.m[2][2] = diag;
    } else if (d.shape == NPGPU_SHAPE_CAPSULE) {
        // capsule_volume = cylinder_volume + ball_volume; the unit inertia is
        // the cylinder's plus the ball's plus the hemispheres' parallel-axis
        // term on the two axes across the capsule.
        float r = d.shape_params[0], hh = d.shape_params[1];
        float vol = hh * r * r * pi * 2.0f + pi * r * r * r * (float)(4.0 / 3.0);
        mass = vol * d.density;
        float sq_radius = r * r;
        float sq_height = hh * hh * 4.0f;
        float off = (sq_radius * 3.0f + sq_height) / 12.0f;
        float diag = r * r * (float)(2.0 / 5.0);
        float h = hh * 2.0f;
        float extra = h * h * 0.5f + h * r * (float)(3.0 / 8.0);
        unit.m[0][0] = (off + diag) + extra;
        unit.m[1][1] = sq_radius / 2.0f + diag;
        unit.m[2][2] = (off + diag) + extra;
    } else {
        float vol = 1.0f;
        vol = vol * d.shape_params[0] * 2.0f;
        vol = vol * d.shape_params[1] * 2.0f;
        vol = vol * d.shape_params[2] * 2.0f;
        mass = vol * d.density;
        float w = (float)(1.0 / 12.0) * 2.0f * 2.0f;
        float ix = w * d.shape_params[0] * d.shape_params[0];
        float iy = w * d.shape_params[1] * d.shape_params[1];
        float iz = w * d.shape_params[2] * d.shape_params[2];
        unit.m[0][0] = iy + iz;
        unit.m[1][1] = ix + iz;
        unit.m[2][2] = ix + iy;
    }
    np::M local = np::mscale(unit, mass);
    np::Iso wrt{np::mk(d.position_wrt_body[0], d.position_wrt_body[1], d.position_wrt_body[2]),
                np::Q{d.position_wrt_body[3], d.position_wrt_body[4], d.position_wrt_body[5], d.position_wrt_body[6]}};
    com = np::iso_pt(wrt, np::mk(0.0f, 0.0f, 0.0f));
    np::M rot = np::qmat(wrt.q);
    ang = np::mm(np::mm(rot, local), np::mtr(rot));
}

// RigidBody::add_local_inertia_and_com, the part that does not need the pose
// (src/object/rigid_body.rs:747-766).
void add_local_inertia_and_com(HostBody& b, np::V com, float mass, const np::M& ang) {
    float mass_sum = b.mass + mass;
    if (mass_sum != 0.0f) b.local_com = np::divs(np::add(np::mul(b.local_com, b.mass), np::mul(com, mass)), mass_sum);
    else b.local_com = np::mk(0.0f, 0.0f, 0.0f);
    b.mass = b.mass + mass;
    b.local_I = np::madd(b.local_I, ang);
}

template <class T>
cudaError_t dalloc(T** p, size_t n, std::vector<void*>& owned) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
    if (e == cudaSuccess) {
        owned.push_back(*p);
        cudaMemset(*p, 0, sizeof(T) * n);
    }
    return e;
}

}  // namespace

struct npgpu_world {
    npgpu_params params;
    float gravity[3];
    uint32_t cap_b = 0, cap_c = 0, cap_p = 0;
    std::vector<HostBody> hb;
    std::vector<HostCollider> hc;
    uint32_t nb_slots = 0, nc_slots = 0, nc_alive = 0;
    World dw{};                          // value-initialised: pointers not allocated at creation stay null
    Pairs pa{}, pb{};
    Control* ctl = nullptr;
    cudaStream_t stream = nullptr;
    int device = 0;
    int solve_grid = 0;
    void* sort_temp = nullptr;
    size_t sort_bytes = 0;
    void* scan_temp = nullptr;
    size_t scan_bytes = 0;
    uint8_t* d_forget = nullptr;
    std::vector<uint8_t> forget;
    bool forget_pending = false;
    bool cd_dirty = true;
    std::vector<MassUpdate> pending_mass;
    // Staging.
    void* h_stage = nullptr;
    uint32_t* h_flags = nullptr;         // pinned: the device checks of a force batch
    size_t h_stage_bytes = 0;
    void* d_stage = nullptr;
    size_t d_stage_bytes = 0;
    cudaEvent_t ev_stage = nullptr;
    std::vector<void*> owned;
    std::string last_error;
    npgpu_counters counters;
    cudaEvent_t ev[8];
    cudaEvent_t ev_solver[7];
    SolverLaunch solver;
    bool ev_recorded = false;
    bool cd_start_ran = false;
    // Batched-world layout: recomputed when bodies are added, removed or
    // moved between worlds.
    bool layout_dirty = true;
    bool layout_ok = false;              // the worlds qualify for the per-world schedule
    uint32_t n_worlds = 0, max_world_bodies = 0, n_big_worlds = 0;
    uint32_t n_cluster_worlds = 0, cluster_shift = 0;   // worlds solved by a thread-block cluster
    uint32_t force_batch = 0;
    std::vector<uint32_t> world_start;   // n_worlds + 1 slot boundaries, then the n_worlds largest-first order
    uint32_t worlds_cap = 0;             // worlds the device bucket buffers hold
    bool layout_on_device = false;
    // Learned warm start.
    MlpDev* d_net = nullptr;             // inference copy (bf16 weights)
    float* d_prm = nullptr;              // fp32 parameters (NPGPU_MLP_PARAMS)
    float *d_m1 = nullptr, *d_m2 = nullptr, *d_grad = nullptr;   // Adam moments, gradient
    double* d_stats = nullptr;
    bool net_ready = false;
    uint32_t adam_t = 0;
    float* d_samples = nullptr;
    uint32_t sample_cap = 0;
    float* d_feat = nullptr;
    uint32_t max_world = 0;              // largest world index any body had (never lowered)
    // Geometric queries: device copies of a batch, per-query counts and
    // offsets, the hits; grown on demand, kept between calls.
    void* d_query = nullptr;
    size_t query_bytes = 0;
    bool local_dirty = true;             // colliders or worlds changed: the colliders' world-local slots
    std::vector<uint32_t> h_local;       // (Colliders::local) are recomputed before the next step
    std::vector<uint32_t> unregistered;  // colliders whose mass is not yet added to their body
    // CUDA graphs of one step (body start, solver, end-of-step collision
    // detection), one per parity of the double-buffered pair sets, keyed by
    // every value their launches bake in.
    struct GraphSlot {
        std::vector<uint8_t> key;
        cudaGraphExec_t exec = nullptr;
    } graphs[2];
    int graph_next = 0;
    bool graphs_broken = false;          // capture failed once: run eagerly from then on
    bool last_step_graphed = false;
    int grid_world = 0;
    // Joint constraints: the host mirror of the set, and device arrays grown
    // on demand (Joints, cap_j slots).
    std::vector<HostJoint> hj;
    uint32_t nj_slots = 0, nj_alive = 0, cap_j = 0;
    bool joints_local_dirty = false;     // the joints' world-local slots (Joints::local) need recomputing
    std::vector<uint32_t> h_jlocal;
    // Continuous collision detection: the colliders by (world, slot) and the
    // colliders of each body, rebuilt when colliders or worlds change, and the
    // device scratch (Ccd), allocated with the first CCD collider and grown
    // with the colliders and worlds.
    bool ccd_dirty = true;
    bool ccd_any = false;                // a CCD collider is alive
    bool last_step_ccd = false;
    size_t ccd_region = 0, ccd_worlds_cap = 0, ccd_bodies_cap = 0, ccd_colliders_cap = 0;
    std::vector<void*> ccd_fixed, ccd_grown;
    std::vector<uint32_t> h_ccd_order, h_ccd_wstart, h_ccd_wflag, h_bc_start, h_bc_list, h_ccd_list, h_ccd_lstart;
};

// The message of the last failure without a world (npgpu_create, the
// allocation-free pair finder), kept per host thread: a failing call on one
// thread never rewrites the string another thread is reading.
static thread_local std::string g_create_error;

namespace npgpu_dev {
size_t query_hit_bytes();
cudaError_t launch_query(const World& w, int kind, const float* qd, const float* max_toi, uint32_t nq, uint32_t world,
                         uint32_t* counts, uint32_t* offsets, void* scan_temp, size_t scan_bytes, void* out,
                         uint32_t cap_out, cudaStream_t st);
}

namespace npgpu_dev {
// Message returned by npgpu_last_error(NULL) for calls without a world.
void set_global_error(const std::string& msg) { g_create_error = msg; }
}  // namespace npgpu_dev

static npgpu_status fail(npgpu_world* w, npgpu_status s, const std::string& msg) {
    if (w) w->last_error = msg;
    else g_create_error = msg;
    return s;
}

static npgpu_status cuda_fail(npgpu_world* w, cudaError_t e, const char* what) {
    return fail(w, NPGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(expr, what)                                        \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return cuda_fail(w, _e, what); \
    } while (0)

static StepParams step_params(const npgpu_world* w) {
    const npgpu_params& p = w->params;
    StepParams s{};
    s.dt = p.dt;
    s.inv_dt = (p.dt == 0.0f) ? 0.0f : 1.0f / p.dt;
    s.erp = p.erp;
    s.warmstart_coeff = p.warmstart_coeff;
    s.restitution_threshold = p.restitution_velocity_threshold;
    s.allowed_linear_error = p.allowed_linear_error;
    s.max_linear_correction = p.max_linear_correction;
    s.activation_mix = p.activation_mix;
    s.broad_phase_margin = p.broad_phase_margin;
    s.gx = w->gravity[0];
    s.gy = w->gravity[1];
    s.gz = w->gravity[2];
    s.residual_tolerance = p.residual_tolerance;
    s.max_velocity_iterations = p.max_velocity_iterations;
    s.max_position_iterations = p.max_position_iterations;
    s.solve_to_tolerance = p.solve_to_tolerance;
    s.max_iterations_to_tolerance = p.max_iterations_to_tolerance;
    s.warmstart_mode = p.warmstart_mode;
    s.sweep_order = p.sweep_order;
    s.profile = p.profile;
    s.allowed_angular_error = p.allowed_angular_error;
    s.max_angular_correction = p.max_angular_correction;
    s.ccd = (w->ccd_any && p.max_ccd_substeps > 0 && p.dt > 0.0f) ? 1u : 0u;
    return s;
}

// The pinned host staging area, at least `bytes` long, once earlier uses of
// it are done; stage_commit then copies its first `bytes` to the device
// staging area and returns the device pointer.
// hptr null: only the device area is needed (the host side is read over
// the link from the caller's page-locked memory).
static npgpu_status stage_reserve(npgpu_world* w, size_t bytes, void** hptr) {
    CK(cudaEventSynchronize(w->ev_stage), "staging wait");
    if (hptr && bytes > w->h_stage_bytes) {
        if (w->h_stage) cudaFreeHost(w->h_stage);
        w->h_stage = nullptr;
        size_t nb = std::max(bytes, w->h_stage_bytes * 2);
        CK(cudaMallocHost(&w->h_stage, nb), "pinned staging");
        w->h_stage_bytes = nb;
    }
    if (bytes > w->d_stage_bytes) {
        if (w->d_stage) cudaFree(w->d_stage);
    if (w->d_query) cudaFree(w->d_query);
    if (w->dw.events) cudaFree(w->dw.events);
    for (void* p : {(void*)w->dw.j.info, (void*)w->dw.j.state, (void*)w->dw.j.body, (void*)w->dw.j.local,
                    (void*)w->dw.j.anchor, (void*)w->dw.j.frame, (void*)w->dw.j.imp, (void*)w->dw.j.brk,
                    (void*)w->dw.j.axis})
        cudaFree(p);
        w->d_stage = nullptr;
        size_t nb = std::max(bytes, w->d_stage_bytes * 2);
        CK(cudaMalloc(&w->d_stage, nb), "device staging");
        w->d_stage_bytes = nb;
    }
    if (hptr) *hptr = w->h_stage;
    return NPGPU_OK;
}

static npgpu_status stage_commit(npgpu_world* w, size_t bytes, void** dptr) {
    CK(cudaMemcpyAsync(w->d_stage, w->h_stage, bytes, cudaMemcpyHostToDevice, w->stream), "staging copy");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    *dptr = w->d_stage;
    return NPGPU_OK;
}

// Copies `bytes` from host memory to the device staging area (synchronously
// with respect to earlier uses of the staging area) and returns its device pointer.
static npgpu_status stage_upload(npgpu_world* w, const void* src, size_t bytes, void** dptr) {
    void* h = nullptr;
    npgpu_status st = stage_reserve(w, bytes, &h);
    if (st != NPGPU_OK) return st;
    std::memcpy(h, src, bytes);
    return stage_commit(w, bytes, dptr);
}

// True when `p` is page-locked host memory the copy engines can reach directly.
static bool host_pinned(const void* p) {
    if (!p) return true;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// The device-side address of page-locked host memory (null when there is none).
static void* host_device_ptr(void* p) {
    cudaPointerAttributes a{};
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

static void sync_world_view(npgpu_world* w) {
    w->dw.nb_slots = w->nb_slots;
    w->dw.nc_slots = w->nc_slots;
    w->dw.nc_alive = w->nc_alive;
    w->dw.nj_slots = w->nj_alive ? w->nj_slots : 0u;
    uint32_t wb = 0;
    while (wb < 16 && (w->max_world >> wb) != 0u) ++wb;
    w->dw.world_bits = wb;
}

// Finds each world's slot range. The per-world schedule needs the alive
// bodies' world indices non-decreasing in slot order (so a world is one run of
// slots). Worlds up to kMaxWorldBodies slots are solved by a block or a warp;
// wider ones by a thread-block cluster, up to its distributed shared-memory
// limit.
static void compute_layout(npgpu_world* w) {
    w->layout_dirty = false;
    w->layout_ok = false;
    uint32_t last = 0;
    bool any = false;
    for (uint32_t i = 0; i < w->nb_slots; ++i) {
        const HostBody& b = w->hb[i];
        if (!b.alive) continue;
        if (any && b.world < last) return;
        last = b.world;
        any = true;
    }
    if (!any) return;
    const uint32_t nw = last + 1;
    std::vector<uint32_t> st(nw + 1, 0xffffffffu);
    for (uint32_t i = 0; i < w->nb_slots; ++i) {
        const HostBody& b = w->hb[i];
        if (b.alive && st[b.world] == 0xffffffffu) st[b.world] = i;
    }
    st[nw] = w->nb_slots;
    for (uint32_t k = nw; k-- > 0;)
        if (st[k] == 0xffffffffu) st[k] = st[k + 1];
    st[0] = 0;
    uint32_t widest = 0, widest_block = 0, n_cluster = 0;
    for (uint32_t k = 0; k < nw; ++k) {
        const uint32_t wk = st[k + 1] - st[k];
        widest = std::max(widest, wk);
        if (wk > kMaxWorldBodies) ++n_cluster;
        else widest_block = std::max(widest_block, wk);
    }
    const uint32_t ctas = (uint32_t)w->solver.cluster_ctas;
    if (n_cluster > 0 && (ctas == 0 || widest > (ctas << kClusterShiftMax))) return;
    uint32_t shift = 0;
    while (n_cluster > 0 && (ctas << shift) < widest) ++shift;
    std::vector<uint32_t> order(nw);
    for (uint32_t k = 0; k < nw; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return st[a + 1] - st[a] > st[b + 1] - st[b]; });
    st.insert(st.end(), order.begin(), order.end());
    w->world_start.swap(st);
    w->n_worlds = nw;
    w->max_world_bodies = widest_block;
    w->n_cluster_worlds = n_cluster;
    w->cluster_shift = shift;
    w->n_big_worlds = 0;
    for (uint32_t k = 0; k < nw; ++k) {
        const uint32_t wk = w->world_start[k + 1] - w->world_start[k];
        w->n_big_worlds += (wk > kWarpWorldBodies && wk <= kMaxWorldBodies) ? 1u : 0u;
    }
    w->layout_ok = true;
}

// Chooses the schedule of this step and, for the per-world one, makes sure
// the bucket buffers hold every world and the world ranges are on the device.
static npgpu_status prepare_schedule(npgpu_world* w) {
    if (w->layout_dirty) {
        compute_layout(w);
        w->layout_on_device = false;
    }
    const uint32_t sched = w->params.solver_schedule;
    // The automatic choice keeps one grid for a single world and for batches
    // with cluster-sized worlds; the per-world schedule is theirs on request
    // (npgpu_autotune times it).
    const bool eligible = sched == NPGPU_SCHEDULE_WORLDS ||
                          (sched == NPGPU_SCHEDULE_AUTO && w->n_worlds >= 2 && w->n_cluster_worlds == 0);
    w->solver.batched = w->layout_ok && eligible && !w->params.solve_to_tolerance;
    if (!w->solver.batched) return NPGPU_OK;
    Solver& s = w->dw.s;
    const size_t nbk = (size_t)w->n_worlds * kMaxColours;
    if (w->n_worlds > w->worlds_cap) {
        CK(cudaStreamSynchronize(w->stream), "synchronize");
        cudaFree(s.world_start);
        cudaFree(s.bucket_count);
        cudaFree(s.bucket_start);
        s.world_start = s.world_order = s.bucket_count = s.bucket_start = s.bucket_cursor = nullptr;
        uint32_t cap = std::max(w->n_worlds, 2 * w->worlds_cap);
        size_t cbk = (size_t)cap * kMaxColours;
        CK(cudaMalloc(&s.world_start, sizeof(uint32_t) * (2 * (size_t)cap + 1)), "world ranges");
        CK(cudaMalloc(&s.bucket_count, sizeof(uint32_t) * (2 * cbk + 1)), "world buckets");
        CK(cudaMalloc(&s.bucket_start, sizeof(uint32_t) * (cbk + 1)), "world bucket starts");
        w->worlds_cap = cap;
        size_t need = scan_temp_bytes((uint32_t)(cbk + 1));
        if (need > w->scan_bytes) {
            void* old = w->scan_temp;
            CK(cudaMalloc(&w->scan_temp, need), "scan temp");
            for (void*& o : w->owned)
                if (o == old) o = w->scan_temp;
            cudaFree(old);
            w->scan_bytes = need;
            w->solver.scan_temp = w->scan_temp;
            w->solver.scan_bytes = w->scan_bytes;
        }
    }
    s.bucket_cursor = s.bucket_count + nbk + 1;
    s.world_order = s.world_start + w->n_worlds + 1;
    if (!w->layout_on_device) {
        w->layout_on_device = true;
        CK(cudaMemcpyAsync(s.world_start, w->world_start.data(), sizeof(uint32_t) * (2 * (size_t)w->n_worlds + 1),
                           cudaMemcpyHostToDevice, w->stream),
           "world ranges");
        w->solver.world_threads = 0;   // grid size below
    }
    const uint32_t wt = w->params.world_threads;
    const int threads = (wt == 64 || wt == 256) ? (int)wt : 128;
    if (threads != w->solver.world_threads) {
        w->grid_world = world_grid(w->device, w->max_world_bodies, w->n_worlds - w->n_cluster_worlds, threads);
        w->solver.world_threads = threads;
    }
    w->solver.n_worlds = w->n_worlds;
    w->solver.max_world_bodies = w->max_world_bodies;
    w->solver.n_big = w->n_big_worlds;
    w->solver.n_cluster = w->n_cluster_worlds;
    w->solver.cluster_shift = w->cluster_shift;
    w->solver.grid_world = w->grid_world;
    return NPGPU_OK;
}

extern "C" {

uint32_t npgpu_abi_version(void) { return NPGPU_ABI_VERSION; }

void npgpu_default_params(npgpu_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->dt = 1.0f / 60.0f;
    p->erp = 0.2f;
    p->warmstart_coeff = 1.0f;
    p->restitution_velocity_threshold = 1.0f;
    p->allowed_linear_error = 0.001f;
    p->allowed_angular_error = 0.001f;
    p->max_linear_correction = 0.2f;
    p->max_angular_correction = 0.2f;
    p->max_stabilization_multiplier = 0.2f;
    p->max_velocity_iterations = 8;
    p->max_position_iterations = 3;
    p->max_ccd_position_iterations = 10;
    p->max_ccd_substeps = 1;
    p->solve_to_tolerance = 0;
    p->residual_tolerance = 1e-4f;
    p->max_iterations_to_tolerance = 256;
    p->warmstart_mode = 0;
    p->broad_phase_margin = 0.01f;
    p->activation_mix = 0.01f;
    p->profile = 0;
    p->solver_schedule = NPGPU_SCHEDULE_AUTO;
    p->use_graph = 1;
    p->world_threads = 0;
    p->sweep_order = NPGPU_SWEEP_SEPARATE;
}

static npgpu_status create_buffers(npgpu_world* w) {
    auto& o = w->owned;
    uint32_t B = w->cap_b, Cn = w->cap_c, P = w->cap_p;
    Bodies& b = w->dw.b;
#define A(ptr, n) CK(dalloc(&(ptr), (n), o), "cudaMalloc")
    A(b.pos_t, B); A(b.pos_q, B); A(b.lin, B); A(b.ang, B); A(b.com, B); A(b.local_com, B);
    A(b.mass, B); A(b.local_I, 9 * (size_t)B); A(b.I, 9 * (size_t)B); A(b.inv_mass, B); A(b.inv_I, 9 * (size_t)B);
    A(b.acc_lin, B); A(b.acc_ang, B); A(b.f_lin, B); A(b.f_ang, B);
    A(b.lin_damp, B); A(b.ang_damp, B); A(b.max_lin, B); A(b.max_ang, B); A(b.sleep_thr, B); A(b.energy, B);
    A(b.info, B); A(b.world, B); A(b.gen, B); A(b.fstamp, B); A(b.dv, 6 * (size_t)B); A(b.sb, 3 * (size_t)B); A(b.dvf, 8 * (size_t)B); A(b.posef, 12 * (size_t)B); A(b.uf_parent, B); A(b.can_deact, B);
    A(b.cw, 2 * (size_t)B); A(b.adj_count, B); A(b.adj_start, B); A(b.adj_fill, B);
    Colliders& c = w->dw.c;
    A(c.body, Cn); A(c.local, Cn); A(c.info, Cn); A(c.params, Cn); A(c.wrt_t, Cn); A(c.wrt_q, Cn);
    A(c.margin, Cn); A(c.lin_pred, Cn); A(c.friction, Cn); A(c.restitution, Cn); A(c.rank, Cn);
    A(c.pose_t, Cn); A(c.pose_q, Cn); A(c.aabb_min, Cn); A(c.aabb_max, Cn);
    A(c.keys, Cn); A(c.keys_sorted, Cn); A(c.vals, Cn); A(c.vals_sorted, Cn);
    A(c.left, Cn); A(c.right, Cn); A(c.parent, 2 * (size_t)Cn); A(c.node_min, 2 * (size_t)Cn);
    A(c.node_max, 2 * (size_t)Cn); A(c.wide, 5 * (size_t)Cn); A(c.node_slot, 2 * (size_t)Cn); A(c.node_flag, Cn); A(c.leaf_count, Cn); A(c.leaf_offset, Cn);
    A(c.leaf_tmp, (size_t)kLeafCap * Cn);
    for (Pairs* pp : {&w->pa, &w->pb}) {
        A(pp->pair, P); A(pp->owner_start, Cn); A(pp->owner_count, Cn); A(pp->ncont, P); A(pp->prox, P);
        A(pp->key, 4 * (size_t)P); A(pp->w1, 4 * (size_t)P); A(pp->w2, 4 * (size_t)P); A(pp->n, 4 * (size_t)P);
        A(pp->imp, 4 * (size_t)P); A(pp->nl, 4 * (size_t)P);
    }
    Solver& s = w->dw.s;
    A(s.sm_list, P); A(s.sm_colour, P); A(s.sm_prank, P); A(s.sm_rk, P); A(s.sm_b1, P); A(s.sm_b2, P);
    A(s.sm_nc, P); A(s.con, (size_t)P * kMaxContacts * 4); A(s.lam, (size_t)P * kMaxContacts); A(s.sm_mask, P); A(s.pos_rec, (size_t)P * kPosRec); A(s.adj, 2 * (size_t)P); A(s.wm_order, P);
    A(s.perm, 5 * (size_t)P); A(s.tan, (size_t)P * kMaxContacts * 2);
    A(s.rows, (size_t)P * kMaxContacts * kRowsF4);
    A(w->ctl, 1);
    A(w->d_forget, Cn);
#undef A
    w->dw.ctl = w->ctl;
    w->dw.cur = w->pa;
    w->dw.prev = w->pb;
    w->dw.cap_pairs = P;
    w->sort_bytes = sort_temp_bytes(Cn);
    // Scans: leaf counts (colliders), adjacency counts (bodies), and the
    // per-world colour buckets (at most 128 per world, at most one world per body).
    w->scan_bytes = std::max({scan_temp_bytes(Cn), scan_temp_bytes(B), scan_temp_bytes(128u * B + 1u)});
    CK(cudaMalloc(&w->sort_temp, std::max<size_t>(w->sort_bytes, 16)), "sort temp");
    o.push_back(w->sort_temp);
    CK(cudaMalloc(&w->scan_temp, std::max<size_t>(w->scan_bytes, 16)), "scan temp");
    o.push_back(w->scan_temp);
    CK(cudaDeviceSynchronize(), "create");
    return NPGPU_OK;
}

npgpu_world* npgpu_create(const npgpu_params* params, const float gravity[3], uint32_t capacity_bodies,
                          uint32_t capacity_colliders, uint32_t capacity_pairs, npgpu_status* status) {
    npgpu_status st = NPGPU_OK;
    npgpu_world* w = nullptr;
    do {
        if (!params || !gravity) {
            st = fail(nullptr, NPGPU_ERR_INVALID_ARGUMENT, "params and gravity are required");
            break;
        }
        if (capacity_bodies >= (1u << 21) || capacity_colliders >= (1u << 21)) {
            st = fail(nullptr, NPGPU_ERR_CAPACITY, "at most 2^21 - 1 bodies and colliders per world");
            break;
        }
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            st = fail(nullptr, NPGPU_ERR_CUDA, "no CUDA device");
            break;
        }
        w = new npgpu_world;
        w->params = *params;
        std::memcpy(w->gravity, gravity, sizeof(w->gravity));
        w->cap_b = std::max(capacity_bodies, 1u);
        w->cap_c = std::max(capacity_colliders, 1u);
        w->cap_p = std::max(capacity_pairs, 1u);
        w->hb.resize(w->cap_b);
        w->hc.resize(w->cap_c);
        for (auto& b : w->hb) b.local_I = np::mzero();
        w->forget.assign(w->cap_c, 0);
        std::memset(&w->counters, 0, sizeof(w->counters));
        cudaGetDevice(&w->device);
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, w->device);
        if (!coop) {
            st = fail(nullptr, NPGPU_ERR_CUDA, "device does not support cooperative launches");
            break;
        }
        if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess) {
            st = fail(nullptr, NPGPU_ERR_CUDA, "stream creation failed");
            break;
        }
        cudaEventCreateWithFlags(&w->ev_stage, cudaEventDisableTiming);
        cudaEventRecord(w->ev_stage, w->stream);
        for (auto& e : w->ev) cudaEventCreate(&e);
        for (auto& e : w->ev_solver) cudaEventCreate(&e);
        st = create_buffers(w);
        if (st != NPGPU_OK) {
            g_create_error = w->last_error;
            break;
        }
        solver_grid_sizes(w->device, w->solver);
        w->solver.scan_temp = w->scan_temp;
        w->solver.scan_bytes = w->scan_bytes;
        w->solver.ev = nullptr;
    } while (0);
    if (status) *status = st;
    if (st != NPGPU_OK && w) {
        npgpu_destroy(w);
        w = nullptr;
    }
    return w;
}

void npgpu_destroy(npgpu_world* w) {
    if (!w) return;
    if (w->stream) cudaStreamSynchronize(w->stream);
    for (void* p : w->owned) cudaFree(p);
    for (void* p : w->ccd_fixed) cudaFree(p);
    for (void* p : w->ccd_grown) cudaFree(p);
    cudaFree(w->dw.s.world_start);
    cudaFree(w->dw.s.bucket_count);
    cudaFree(w->dw.s.bucket_start);
    for (auto& g : w->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (void* p : {(void*)w->d_net, (void*)w->d_prm, (void*)w->d_m1, (void*)w->d_m2, (void*)w->d_grad,
                    (void*)w->d_stats, (void*)w->d_samples, (void*)w->d_feat})
        cudaFree(p);
    if (w->d_stage) cudaFree(w->d_stage);
    if (w->d_query) cudaFree(w->d_query);
    if (w->dw.events) cudaFree(w->dw.events);
    if (w->h_flags) cudaFreeHost(w->h_flags);
    if (w->h_stage) cudaFreeHost(w->h_stage);
    if (w->ev_stage) cudaEventDestroy(w->ev_stage);
    for (auto& e : w->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : w->ev_solver)
        if (e) cudaEventDestroy(e);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
}

void* npgpu_stream(npgpu_world* w) { return w ? (void*)w->stream : nullptr; }

npgpu_status npgpu_set_params(npgpu_world* w, const npgpu_params* params) {
    if (!w || !params) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (!(params->dt >= 0.0f)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "dt must be >= 0");
    if (params->solver_schedule > NPGPU_SCHEDULE_WORLDS)
        return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "unknown solver_schedule");
    if (params->world_threads != 0 && params->world_threads != 64 && params->world_threads != 128 &&
        params->world_threads != 256)
        return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "world_threads must be 0, 64, 128 or 256");
    if (params->sweep_order > NPGPU_SWEEP_MANIFOLD)
        return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "unknown sweep_order");
    w->params = *params;
    return NPGPU_OK;
}

npgpu_status npgpu_set_gravity(npgpu_world* w, const float gravity[3]) {
    if (!w || !gravity) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (!finite_n(gravity, 3)) return fail(w, NPGPU_ERR_NAN, "gravity is not finite");
    std::memcpy(w->gravity, gravity, sizeof(w->gravity));
    return NPGPU_OK;
}

npgpu_status npgpu_upsert_bodies(npgpu_world* w, uint32_t n, const npgpu_handle* handles,
                                 const npgpu_body_desc* descs) {
    if (!w || (n && (!handles || !descs))) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<BodyUpload> up;
    up.reserve(n);
    for (uint32_t k = 0; k < n; ++k) {
        const npgpu_body_desc& d = descs[k];
        uint64_t slot = handles[k].index;
        if (d.kind != NPGPU_KIND_RIGID_BODY && d.kind != NPGPU_KIND_GROUND)
            return fail(w, NPGPU_ERR_UNSUPPORTED_BODY,
                        "only rigid bodies and grounds are supported (multibody / FEM / mass-spring bodies are rejected)");
        if (slot >= w->cap_b) return fail(w, NPGPU_ERR_CAPACITY, "body index beyond the world's capacity");
        if (d.status > NPGPU_BODY_KINEMATIC) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "invalid body status");
        if (!finite_n(d.position, 7) || !finite_n(d.velocity, 6) || !finite_n(d.local_inertia, 7) ||
            !finite_n(d.local_com, 3) || !std::isfinite(d.linear_damping) || !std::isfinite(d.angular_damping) ||
            std::isnan(d.max_linear_velocity) || std::isnan(d.max_angular_velocity) || !std::isfinite(d.sleep_threshold))
            return fail(w, NPGPU_ERR_NAN, "body description has a non-finite value");
        if (d.world >= 0xffffu) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "world index must be < 65535");
        HostBody& hb = w->hb[slot];
        bool is_new = !hb.alive;
        BodyUpload u;
        std::memset(&u, 0, sizeof(u));
        u.slot = (uint32_t)slot;
        uint32_t status = d.kind == NPGPU_KIND_GROUND ? (uint32_t)NPGPU_BODY_STATIC : d.status;
        u.info = status | (d.kind << BI_KIND_SHIFT) | ((d.flags & 0x1ffu) << BI_FLAGS_SHIFT);
        u.world = d.world;
        u.reset_energy = is_new ? 1u : 0u;
        std::memcpy(u.pos, d.position, sizeof(u.pos));
        std::memcpy(u.vel, d.velocity, sizeof(u.vel));
        if (d.kind == NPGPU_KIND_GROUND) {
            float id[7] = {0, 0, 0, 0, 0, 0, 1};
            std::memcpy(u.pos, id, sizeof(u.pos));
            std::memset(u.vel, 0, sizeof(u.vel));
        }
        if (is_new) {
            hb.mass = d.local_inertia[0];
            np::M a = np::mzero();
            a.m[0][0] = d.local_inertia[1];
            a.m[0][1] = a.m[1][0] = d.local_inertia[2];
            a.m[0][2] = a.m[2][0] = d.local_inertia[3];
            a.m[1][1] = d.local_inertia[4];
            a.m[1][2] = a.m[2][1] = d.local_inertia[5];
            a.m[2][2] = d.local_inertia[6];
            hb.local_I = a;
            hb.local_com = np::mk(d.local_com[0], d.local_com[1], d.local_com[2]);
        }
        u.mass = hb.mass;
        for (int r = 0; r < 3; ++r)
            for (int cc = 0; cc < 3; ++cc) u.local_I[3 * r + cc] = hb.local_I.m[r][cc];
        u.local_com[0] = hb.local_com.x;
        u.local_com[1] = hb.local_com.y;
        u.local_com[2] = hb.local_com.z;
        u.lin_damp = d.linear_damping;
        u.ang_damp = d.angular_damping;
        u.max_lin = d.max_linear_velocity;
        u.max_ang = d.max_angular_velocity;
        u.sleep_thr = d.sleep_threshold;
        if (!hb.alive || hb.world != d.world) w->layout_dirty = w->local_dirty = w->ccd_dirty = true;
        w->max_world = std::max(w->max_world, d.world);
        hb.alive = true;
        hb.gen = handles[k].generation;
        u.gen = handles[k].generation;
        hb.kind = d.kind;
        hb.status = status;
        hb.flags = d.flags;
        hb.world = d.world;
        w->nb_slots = std::max(w->nb_slots, (uint32_t)slot + 1);
        up.push_back(u);
    }
    if (up.empty()) return NPGPU_OK;
    void* dp = nullptr;
    npgpu_status st = stage_upload(w, up.data(), up.size() * sizeof(BodyUpload), &dp);
    if (st != NPGPU_OK) return st;
    sync_world_view(w);
    CK(launch_upload_bodies(w->dw, (const BodyUpload*)dp, (uint32_t)up.size(), w->stream), "upload bodies");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    w->cd_dirty = true;
    return NPGPU_OK;
}

static bool body_handle_ok(const npgpu_world* w, const npgpu_handle& h) {
    return h.index < w->cap_b && w->hb[h.index].alive && w->hb[h.index].gen == h.generation;
}

// Subtracts a registered collider's mass from its body and wakes the body
// (geometrical_world.rs:179-194).
static void unregister_collider_mass(npgpu_world* w, HostCollider& c, bool body_remains) {
    if (!body_remains || !c.registered) return;
    HostBody& b = w->hb[c.desc.body.index];
    MassUpdate u;
    std::memset(&u, 0, sizeof(u));
    u.slot = (uint32_t)c.desc.body.index;
    u.activate = 2u;   // bit 1: activate
    if (c.desc.density != 0.0f && b.kind == NPGPU_KIND_RIGID_BODY) {
        np::V com;
        float mass;
        np::M ang;
        collider_mass_properties(c.desc, com, mass, ang);
        add_local_inertia_and_com(b, np::neg(com), -mass, np::mscale(ang, -1.0f));
        u.activate |= 1u;   // bit 0: the mass changed
    }
    u.mass = b.mass;
    for (int r = 0; r < 3; ++r)
        for (int cc = 0; cc < 3; ++cc) u.local_I[3 * r + cc] = b.local_I.m[r][cc];
    u.local_com[0] = b.local_com.x;
    u.local_com[1] = b.local_com.y;
    u.local_com[2] = b.local_com.z;
    w->pending_mass.push_back(u);
}

npgpu_status npgpu_upsert_colliders(npgpu_world* w, uint32_t n, const npgpu_handle* handles,
                                    const npgpu_collider_desc* descs) {
    if (!w || (n && (!handles || !descs))) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<ColliderUpload> up;
    up.reserve(n);
    for (uint32_t k = 0; k < n; ++k) {
        const npgpu_collider_desc& d = descs[k];
        uint64_t slot = handles[k].index;
        if (d.shape != NPGPU_SHAPE_BALL && d.shape != NPGPU_SHAPE_CUBOID && d.shape != NPGPU_SHAPE_CAPSULE)
            return fail(w, NPGPU_ERR_UNSUPPORTED_SHAPE, "only Ball, Cuboid and Capsule shapes are supported");
        if (slot >= w->cap_c) return fail(w, NPGPU_ERR_CAPACITY, "collider index beyond the world's capacity");
        if (!body_handle_ok(w, d.body)) return fail(w, NPGPU_ERR_INVALID_HANDLE, "collider parent body handle is invalid");
        if (!finite_n(d.position_wrt_body, 7) || !finite_n(d.shape_params, 3) || !std::isfinite(d.margin) ||
            !std::isfinite(d.density) || !std::isfinite(d.linear_prediction) || !std::isfinite(d.friction) ||
            !std::isfinite(d.restitution))
            return fail(w, NPGPU_ERR_NAN, "collider description has a non-finite value");
        if (d.friction_combine > 3 || d.restitution_combine > 3)
            return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "invalid material combine mode");
        HostCollider& hc = w->hc[slot];
        if (hc.alive) {
            unregister_collider_mass(w, hc, true);
        } else {
            w->nc_alive += 1;
        }
        hc.alive = true;
        hc.registered = false;
        w->unregistered.push_back((uint32_t)slot);
        hc.gen = handles[k].generation;
        hc.desc = d;
        w->forget[slot] = std::max<uint8_t>(w->forget[slot], 1);
        w->forget_pending = true;
        ColliderUpload u;
        std::memset(&u, 0, sizeof(u));
        u.slot = (uint32_t)slot;
        u.body = (uint32_t)d.body.index;
        u.info = d.shape | (d.friction_combine << 4) | (d.restitution_combine << 8) | (d.ccd_enabled ? CI_CCD : 0u) |
                 (d.is_sensor ? CI_SENSOR : 0u);
        u.params[0] = d.shape_params[0];
        u.params[1] = d.shape_params[1];
        u.params[2] = d.shape_params[2];
        std::memcpy(u.wrt, d.position_wrt_body, sizeof(u.wrt));
        // A sensor's query limit is its linear prediction alone
        // (GeometricQueryType::Proximity, collider.rs:542-543).
        u.margin = d.is_sensor ? 0.0f : d.margin;
        u.lin_pred = d.linear_prediction;
        u.friction = d.friction;
        u.restitution = d.restitution;
        if (d.shape == NPGPU_SHAPE_BALL) u.rank = d.shape_params[0];
        else if (d.shape == NPGPU_SHAPE_CAPSULE) u.rank = d.shape_params[1] + d.shape_params[0];
        else u.rank = std::sqrt(d.shape_params[0] * d.shape_params[0] + d.shape_params[1] * d.shape_params[1] +
                                d.shape_params[2] * d.shape_params[2]);
        w->nc_slots = std::max(w->nc_slots, (uint32_t)slot + 1);
        up.push_back(u);
    }
    if (up.empty()) return NPGPU_OK;
    w->local_dirty = w->ccd_dirty = true;
    void* dp = nullptr;
    npgpu_status st = stage_upload(w, up.data(), up.size() * sizeof(ColliderUpload), &dp);
    if (st != NPGPU_OK) return st;
    sync_world_view(w);
    CK(launch_upload_colliders(w->dw, (const ColliderUpload*)dp, (uint32_t)up.size(), w->stream), "upload colliders");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    w->cd_dirty = true;
    return NPGPU_OK;
}

static npgpu_status kill_slots(npgpu_world* w, const std::vector<uint32_t>& slots, int colliders) {
    if (slots.empty()) return NPGPU_OK;
    void* dp = nullptr;
    npgpu_status st = stage_upload(w, slots.data(), slots.size() * sizeof(uint32_t), &dp);
    if (st != NPGPU_OK) return st;
    CK(launch_kill(w->dw, (const uint32_t*)dp, (uint32_t)slots.size(), colliders, w->stream), "kill");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    return NPGPU_OK;
}

// Body::activate of an alive body at the next step, keeping its mass state
// (the update carries it whole).
static void wake_body(npgpu_world* w, uint64_t slot) {
    if (slot >= w->cap_b || !w->hb[slot].alive) return;
    const HostBody& b = w->hb[slot];
    MassUpdate u;
    std::memset(&u, 0, sizeof(u));
    u.slot = (uint32_t)slot;
    u.activate = 2u;
    u.mass = b.mass;
    for (int r = 0; r < 3; ++r)
        for (int cc = 0; cc < 3; ++cc) u.local_I[3 * r + cc] = b.local_I.m[r][cc];
    u.local_com[0] = b.local_com.x;
    u.local_com[1] = b.local_com.y;
    u.local_com[2] = b.local_com.z;
    w->pending_mass.push_back(u);
}

// Device joint arrays for at least `need` slots; existing joints keep their
// description, impulses and state.
static npgpu_status ensure_joint_capacity(npgpu_world* w, uint32_t need) {
    if (need <= w->cap_j) return NPGPU_OK;
    uint32_t cap = std::max<uint32_t>(need, std::max<uint32_t>(64u, 2u * w->cap_j));
    Joints nj{};
    std::vector<void*> fresh;
    bool ok = true;
#define JA(ptr, n)                                                                                        \
    if (ok) {                                                                                             \
        void* p_ = nullptr;                                                                               \
        ok = cudaMalloc(&p_, std::max<size_t>((size_t)(n) * sizeof(*(ptr)), 16)) == cudaSuccess;          \
        if (ok) {                                                                                         \
            (ptr) = (decltype(ptr))p_;                                                                    \
            fresh.push_back(p_);                                                                          \
        }                                                                                                 \
    }
    JA(nj.info, cap) JA(nj.state, cap) JA(nj.body, 2 * (size_t)cap) JA(nj.local, cap)
    JA(nj.anchor, 2 * (size_t)cap) JA(nj.frame, 2 * (size_t)cap) JA(nj.imp, 2 * (size_t)cap) JA(nj.brk, cap)
    JA(nj.axis, 3 * (size_t)cap)
#undef JA
    if (!ok) {
        for (void* p : fresh) cudaFree(p);
        cudaGetLastError();
        return fail(w, NPGPU_ERR_CUDA, "joint arrays: cudaMalloc failed");
    }
    CK(cudaMemsetAsync(nj.info, 0, sizeof(uint32_t) * cap, w->stream), "joint arrays");
    CK(cudaMemsetAsync(nj.state, 0, sizeof(uint32_t) * cap, w->stream), "joint arrays");
    CK(cudaMemsetAsync(nj.imp, 0, sizeof(float4) * 2 * (size_t)cap, w->stream), "joint arrays");
    const Joints& oj = w->dw.j;
    const size_t n = w->cap_j;
    if (n) {
        CK(cudaMemcpyAsync(nj.info, oj.info, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
        CK(cudaMemcpyAsync(nj.state, oj.state, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
        CK(cudaMemcpyAsync(nj.body, oj.body, sizeof(uint32_t) * 2 * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
        CK(cudaMemcpyAsync(nj.local, oj.local, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
        CK(cudaMemcpyAsync(nj.anchor, oj.anchor, sizeof(float4) * 2 * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
        CK(cudaMemcpyAsync(nj.frame, oj.frame, sizeof(float4) * 2 * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
        CK(cudaMemcpyAsync(nj.imp, oj.imp, sizeof(float4) * 2 * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
        CK(cudaMemcpyAsync(nj.brk, oj.brk, sizeof(float2) * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
        CK(cudaMemcpyAsync(nj.axis, oj.axis, sizeof(float4) * 3 * n, cudaMemcpyDeviceToDevice, w->stream), "joints");
    }
    CK(cudaStreamSynchronize(w->stream), "joint arrays");
    for (void* p : {(void*)oj.info, (void*)oj.state, (void*)oj.body, (void*)oj.local, (void*)oj.anchor, (void*)oj.frame,
                    (void*)oj.imp, (void*)oj.brk, (void*)oj.axis})
        cudaFree(p);
    w->dw.j = nj;
    w->cap_j = cap;
    w->hj.resize(cap);
    return NPGPU_OK;
}

static npgpu_status upload_joints(npgpu_world* w, const std::vector<JointUpload>& up) {
    if (up.empty()) return NPGPU_OK;
    void* dp = nullptr;
    npgpu_status st = stage_upload(w, up.data(), up.size() * sizeof(JointUpload), &dp);
    if (st != NPGPU_OK) return st;
    CK(launch_upload_joints(w->dw, (const JointUpload*)dp, (uint32_t)up.size(), w->stream), "upload joints");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    return NPGPU_OK;
}

// Removes the joints in `slots` (alive), waking their bodies.
static npgpu_status drop_joints(npgpu_world* w, const std::vector<uint32_t>& slots) {
    std::vector<JointUpload> up;
    for (uint32_t j : slots) {
        HostJoint& hj = w->hj[j];
        hj.alive = false;
        w->nj_alive -= 1;
        wake_body(w, hj.desc.body1.index);
        wake_body(w, hj.desc.body2.index);
        JointUpload u;
        std::memset(&u, 0, sizeof(u));
        u.slot = j;
        u.reset = 1u;
        up.push_back(u);
    }
    w->joints_local_dirty = true;
    sync_world_view(w);
    return upload_joints(w, up);
}

npgpu_status npgpu_upsert_joints(npgpu_world* w, uint32_t n, const npgpu_handle* handles,
                                 const npgpu_joint_desc* descs) {
    if (!w || (n && (!handles || !descs))) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    for (uint32_t k = 0; k < n; ++k) {
        const npgpu_joint_desc& d = descs[k];
        if (handles[k].index >= (1u << 21) - 1u)
            return fail(w, NPGPU_ERR_CAPACITY, "joint index must be below 2^21 - 1");
        if (d.kind > NPGPU_JOINT_PIN_SLOT)
            return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "unknown joint kind");
        if ((d.limit_flags & NPGPU_JOINT_MIN_OFFSET) && (d.limit_flags & NPGPU_JOINT_MAX_OFFSET) &&
            !(d.min_offset <= d.max_offset))
            return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "a prismatic joint's min offset must not exceed its max offset");
        if (!body_handle_ok(w, d.body1) || !body_handle_ok(w, d.body2))
            return fail(w, NPGPU_ERR_INVALID_HANDLE, "joint body handle is invalid");
        if (d.body1.index == d.body2.index)
            return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "a joint needs two different bodies");
        if (w->hb[d.body1.index].world != w->hb[d.body2.index].world)
            return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "a joint's bodies must belong to the same world");
        if (!finite_n(d.anchor1, 3) || !finite_n(d.anchor2, 3) || !finite_n(d.frame1, 4) || !finite_n(d.frame2, 4) ||
            !finite_n(d.axis1, 3) || !finite_n(d.axis2, 3) || !finite_n(d.axis3, 3) || !std::isfinite(d.angle) ||
            !std::isfinite(d.min_offset) || !std::isfinite(d.max_offset) ||
            std::isnan(d.break_force) || std::isnan(d.break_torque))
            return fail(w, NPGPU_ERR_NAN, "joint description has a non-finite value");
    }
    uint32_t need = 0;
    for (uint32_t k = 0; k < n; ++k) need = std::max<uint32_t>(need, (uint32_t)handles[k].index + 1u);
    npgpu_status st = ensure_joint_capacity(w, need);
    if (st != NPGPU_OK) return st;
    std::vector<JointUpload> up;
    up.reserve(n);
    for (uint32_t k = 0; k < n; ++k) {
        const npgpu_joint_desc& d = descs[k];
        const uint32_t slot = (uint32_t)handles[k].index;
        HostJoint& hj = w->hj[slot];
        if (hj.alive) {
            wake_body(w, hj.desc.body1.index);
            wake_body(w, hj.desc.body2.index);
        } else {
            w->nj_alive += 1;
        }
        hj.alive = true;
        hj.gen = handles[k].generation;
        hj.desc = d;
        wake_body(w, d.body1.index);
        wake_body(w, d.body2.index);
        JointUpload u;
        std::memset(&u, 0, sizeof(u));
        u.slot = slot;
        u.info = d.kind | JI_ALIVE;
        u.body1 = (uint32_t)d.body1.index;
        u.body2 = (uint32_t)d.body2.index;
        u.reset = 1u;
        std::memcpy(u.anchor1, d.anchor1, sizeof(u.anchor1));
        std::memcpy(u.anchor2, d.anchor2, sizeof(u.anchor2));
        std::memcpy(u.frame1, d.frame1, sizeof(u.frame1));
        std::memcpy(u.frame2, d.frame2, sizeof(u.frame2));
        std::memcpy(u.axis1, d.axis1, sizeof(u.axis1));
        std::memcpy(u.axis2, d.axis2, sizeof(u.axis2));
        std::memcpy(u.axis3, d.axis3, sizeof(u.axis3));
        u.angle = d.angle;
        u.min_offset = d.min_offset;
        u.max_offset = d.max_offset;
        if (d.kind == NPGPU_JOINT_PRISMATIC) {
            if (d.limit_flags & NPGPU_JOINT_MIN_OFFSET) u.info |= JI_MIN_OFFSET;
            if (d.limit_flags & NPGPU_JOINT_MAX_OFFSET) u.info |= JI_MAX_OFFSET;
        }
        // set_break_force / set_break_torque keep the squares (f32).
        u.brk_force2 = d.break_force * d.break_force;
        u.brk_torque2 = d.break_torque * d.break_torque;
        w->nj_slots = std::max(w->nj_slots, slot + 1u);
        up.push_back(u);
    }
    if (up.empty()) return NPGPU_OK;
    w->joints_local_dirty = true;
    sync_world_view(w);
    return upload_joints(w, up);
}

static bool joint_handle_ok(const npgpu_world* w, const npgpu_handle& h) {
    return h.index < w->cap_j && w->hj[h.index].alive && w->hj[h.index].gen == h.generation;
}

npgpu_status npgpu_remove_joints(npgpu_world* w, uint32_t n, const npgpu_handle* handles) {
    if (!w || (n && !handles)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    for (uint32_t k = 0; k < n; ++k)
        if (!joint_handle_ok(w, handles[k])) return fail(w, NPGPU_ERR_INVALID_HANDLE, "invalid joint handle");
    std::vector<uint32_t> slots;
    for (uint32_t k = 0; k < n; ++k) slots.push_back((uint32_t)handles[k].index);
    std::sort(slots.begin(), slots.end());
    slots.erase(std::unique(slots.begin(), slots.end()), slots.end());
    return drop_joints(w, slots);
}

npgpu_status npgpu_get_joints(npgpu_world* w, uint32_t n, const npgpu_handle* handles, npgpu_joint_state* out) {
    if (!w || (n && (!handles || !out))) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    for (uint32_t k = 0; k < n; ++k)
        if (!joint_handle_ok(w, handles[k])) return fail(w, NPGPU_ERR_INVALID_HANDLE, "invalid joint handle");
    if (n == 0) return NPGPU_OK;
    CK(cudaStreamSynchronize(w->stream), "get joints");
    std::vector<float4> imp(2 * (size_t)w->nj_slots);
    std::vector<uint32_t> state(w->nj_slots);
    CK(cudaMemcpy(imp.data(), w->dw.j.imp, sizeof(float4) * imp.size(), cudaMemcpyDeviceToHost), "get joints");
    CK(cudaMemcpy(state.data(), w->dw.j.state, sizeof(uint32_t) * state.size(), cudaMemcpyDeviceToHost), "get joints");
    for (uint32_t k = 0; k < n; ++k) {
        const size_t j = handles[k].index;
        const float4 a = imp[2 * j], b = imp[2 * j + 1];
        const float v[6] = {a.x, a.y, a.z, b.x, b.y, b.z};
        std::memcpy(out[k].impulses, v, sizeof(v));
        out[k].limit_impulse = a.w;
        out[k].pad = 0;
        out[k].broken = (state[j] & JS_BROKEN) ? 1u : 0u;
        out[k].active = (state[j] & JS_ACTIVE) ? 1u : 0u;
    }
    return NPGPU_OK;
}

npgpu_status npgpu_remove_colliders(npgpu_world* w, uint32_t n, const npgpu_handle* handles) {
    if (!w || (n && !handles)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    for (uint32_t k = 0; k < n; ++k) {
        const npgpu_handle& h = handles[k];
        if (h.index >= w->cap_c || !w->hc[h.index].alive || w->hc[h.index].gen != h.generation)
            return fail(w, NPGPU_ERR_INVALID_HANDLE, "invalid collider handle");
    }
    std::vector<uint32_t> slots;
    for (uint32_t k = 0; k < n; ++k) {
        HostCollider& c = w->hc[handles[k].index];
        unregister_collider_mass(w, c, true);
        c.alive = false;
        w->nc_alive -= 1;
        w->forget[handles[k].index] = 2;
        slots.push_back((uint32_t)handles[k].index);
    }
    w->forget_pending = true;
    w->cd_dirty = true;
    w->local_dirty = w->ccd_dirty = true;
    return kill_slots(w, slots, 1);
}

npgpu_status npgpu_remove_bodies(npgpu_world* w, uint32_t n, const npgpu_handle* handles) {
    if (!w || (n && !handles)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    for (uint32_t k = 0; k < n; ++k)
        if (!body_handle_ok(w, handles[k])) return fail(w, NPGPU_ERR_INVALID_HANDLE, "invalid body handle");
    std::vector<uint32_t> bslots, cslots;
    for (uint32_t k = 0; k < n; ++k) {
        uint64_t bi = handles[k].index;
        for (uint32_t ci = 0; ci < w->nc_slots; ++ci) {
            HostCollider& c = w->hc[ci];
            if (c.alive && c.desc.body.index == bi) {
                c.alive = false;
                w->nc_alive -= 1;
                w->forget[ci] = 2;
                cslots.push_back(ci);
            }
        }
        w->hb[bi].alive = false;
        w->layout_dirty = w->local_dirty = w->ccd_dirty = true;
        bslots.push_back((uint32_t)bi);
    }
    // Joints with a removed body are removed, waking their other body
    // (mechanical_world.rs:141-165).
    std::vector<uint32_t> jslots;
    for (uint32_t j = 0; j < w->nj_slots; ++j) {
        HostJoint& hj = w->hj[j];
        if (!hj.alive) continue;
        const bool gone1 = !w->hb[hj.desc.body1.index].alive, gone2 = !w->hb[hj.desc.body2.index].alive;
        if (!gone1 && !gone2) continue;
        jslots.push_back(j);
    }
    if (!jslots.empty()) {
        npgpu_status sj = drop_joints(w, jslots);
        if (sj != NPGPU_OK) return sj;
    }
    w->forget_pending = true;
    w->cd_dirty = true;
    npgpu_status st = kill_slots(w, cslots, 1);
    if (st != NPGPU_OK) return st;
    return kill_slots(w, bslots, 0);
}

npgpu_status npgpu_apply_forces(npgpu_world* w, uint32_t n, const npgpu_handle* handles, const float* forces6,
                                int auto_wake_up) {
    if (!w || (n && (!handles || !forces6))) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) return NPGPU_OK;
    // The device checks the batch (handles against the slots' generations,
    // finite forces, a body named twice) as it copies it into the device
    // staging area, reading page-locked arrays over the host link itself and
    // pageable ones from the pinned staging area; the forces are applied from
    // that copy only if every handle and force is valid. The call returns once
    // the checks are known, so the caller may reuse its arrays.
    const size_t hb = sizeof(npgpu_handle) * (size_t)n, fb = 6 * sizeof(float) * (size_t)n;
    const npgpu_handle* src_h = (const npgpu_handle*)host_device_ptr((void*)handles);
    const float* src_f = (const float*)host_device_ptr((void*)forces6);
    const bool direct = src_h && src_f;
    void* hp = nullptr;
    npgpu_status st = stage_reserve(w, hb + fb, direct ? nullptr : &hp);
    if (st != NPGPU_OK) return st;
    void* dp = w->d_stage;
    if (!direct) {
        std::memcpy(hp, handles, hb);
        std::memcpy((char*)hp + hb, forces6, fb);
        st = stage_commit(w, hb + fb, &dp);
        if (st != NPGPU_OK) return st;
    }
    if (!w->h_flags) CK(cudaMallocHost(&w->h_flags, sizeof(uint32_t)), "pinned flags");
    if (++w->force_batch == 0) {
        CK(cudaMemsetAsync(w->dw.b.fstamp, 0, sizeof(uint32_t) * w->cap_b, w->stream), "force stamps");
        w->force_batch = 1;
    }
    npgpu_handle* dh = (npgpu_handle*)dp;
    float* df = (float*)((char*)dp + hb);
    CK(cudaMemsetAsync(&w->ctl->force_flags, 0, sizeof(uint32_t), w->stream), "force flags");
    CK(launch_force_check(w->dw, direct ? src_h : dh, direct ? src_f : df, dh, df, n, w->force_batch, w->cap_b,
                          w->stream),
       "force check");
    CK(cudaMemcpyAsync(w->h_flags, &w->ctl->force_flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream),
       "force flags");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    CK(cudaEventSynchronize(w->ev_stage), "force check");
    const uint32_t flags = *w->h_flags;
    if (flags & 1u) return fail(w, NPGPU_ERR_INVALID_HANDLE, "invalid body handle");
    if (flags & 2u) return fail(w, NPGPU_ERR_NAN, "force is not finite");
    CK(launch_forces(w->dw, dh, df, n, auto_wake_up != 0, (flags & 4u) != 0, w->stream), "apply forces");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    return NPGPU_OK;
}

// GeometricalWorld::maintain at the start of a step: register the colliders
// inserted since the last step, adding their mass to their body
// (geometrical_world.rs:102-143), and forget the manifolds of removed colliders.
static npgpu_status maintain(npgpu_world* w) {
    // Colliders inserted or replaced since the last step, in slot order.
    std::sort(w->unregistered.begin(), w->unregistered.end());
    w->unregistered.erase(std::unique(w->unregistered.begin(), w->unregistered.end()), w->unregistered.end());
    std::vector<uint32_t> todo;
    todo.swap(w->unregistered);
    for (uint32_t ci : todo) {
        HostCollider& c = w->hc[ci];
        if (!c.alive || c.registered) continue;
        c.registered = true;
        HostBody& b = w->hb[c.desc.body.index];
        if (c.desc.density != 0.0f && b.kind == NPGPU_KIND_RIGID_BODY) {
            np::V com;
            float mass;
            np::M ang;
            collider_mass_properties(c.desc, com, mass, ang);
            add_local_inertia_and_com(b, com, mass, ang);
            MassUpdate u;
            std::memset(&u, 0, sizeof(u));
            u.slot = (uint32_t)c.desc.body.index;
            u.activate = 1u;
            u.mass = b.mass;
            for (int r = 0; r < 3; ++r)
                for (int cc = 0; cc < 3; ++cc) u.local_I[3 * r + cc] = b.local_I.m[r][cc];
            u.local_com[0] = b.local_com.x;
            u.local_com[1] = b.local_com.y;
            u.local_com[2] = b.local_com.z;
            w->pending_mass.push_back(u);
        }
        w->cd_dirty = true;
    }
    if (!w->pending_mass.empty()) {
        // Each update carries the body's mass state after it was applied, so the
        // last update of a body supersedes the earlier ones; their flags are merged.
        std::vector<int32_t> last(w->nb_slots, -1);
        std::vector<MassUpdate> merged;
        for (const MassUpdate& u : w->pending_mass) {
            int32_t& l = last[u.slot];
            if (l < 0) {
                l = (int32_t)merged.size();
                merged.push_back(u);
            } else {
                uint32_t flags = merged[l].activate | u.activate;
                merged[l] = u;
                merged[l].activate = flags;
            }
        }
        void* dp = nullptr;
        npgpu_status st = stage_upload(w, merged.data(), merged.size() * sizeof(MassUpdate), &dp);
        if (st != NPGPU_OK) return st;
        CK(launch_mass_updates(w->dw, (const MassUpdate*)dp, (uint32_t)merged.size(), w->stream), "mass updates");
        CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
        w->pending_mass.clear();
    }
    if (w->forget_pending) {
        CK(cudaEventSynchronize(w->ev_stage), "staging wait");
        CK(cudaMemcpyAsync(w->d_forget, w->forget.data(), w->cap_c, cudaMemcpyHostToDevice, w->stream), "forget copy");
        CK(launch_forget_pairs(w->dw, w->d_forget, w->stream), "forget pairs");
        CK(cudaStreamSynchronize(w->stream), "forget");
        std::fill(w->forget.begin(), w->forget.end(), 0);
        w->forget_pending = false;
    }
    if (w->joints_local_dirty && w->nj_slots) {
        // World-local joint slots: slot minus the smallest alive joint slot
        // of the same world (the colouring priority of a joint hashes it).
        std::vector<uint32_t> base((size_t)w->max_world + 1, 0xffffffffu);
        for (uint32_t j = 0; j < w->nj_slots; ++j) {
            const HostJoint& hj = w->hj[j];
            if (!hj.alive) continue;
            uint32_t wd = w->hb[hj.desc.body1.index].world;
            if (wd < base.size()) base[wd] = std::min(base[wd], j);
        }
        w->h_jlocal.assign(w->nj_slots, 0u);
        for (uint32_t j = 0; j < w->nj_slots; ++j) {
            const HostJoint& hj = w->hj[j];
            uint32_t wd = hj.alive ? w->hb[hj.desc.body1.index].world : 0xffffffffu;
            w->h_jlocal[j] = (wd < base.size() && base[wd] <= j) ? j - base[wd] : j;
        }
        CK(cudaMemcpyAsync(w->dw.j.local, w->h_jlocal.data(), sizeof(uint32_t) * w->h_jlocal.size(),
                           cudaMemcpyHostToDevice, w->stream), "world-local joint slots");
        CK(cudaStreamSynchronize(w->stream), "world-local joint slots");
        w->joints_local_dirty = false;
    }
    if (w->local_dirty) {
        // World-local collider slots: slot minus the smallest alive collider
        // slot of the same world (the colouring priority's hash input).
        std::vector<uint32_t> base((size_t)w->max_world + 1, 0xffffffffu);
        for (uint32_t ci = 0; ci < w->nc_slots; ++ci) {
            const HostCollider& c = w->hc[ci];
            if (!c.alive) continue;
            uint32_t wd = w->hb[c.desc.body.index].world;
            if (wd < base.size()) base[wd] = std::min(base[wd], ci);
        }
        w->h_local.assign(std::max<uint32_t>(w->nc_slots, 1u), 0u);
        for (uint32_t ci = 0; ci < w->nc_slots; ++ci) {
            const HostCollider& c = w->hc[ci];
            uint32_t wd = c.alive ? w->hb[c.desc.body.index].world : 0xffffffffu;
            w->h_local[ci] = (wd < base.size() && base[wd] <= ci) ? ci - base[wd] : ci;
        }
        CK(cudaMemcpyAsync(w->dw.c.local, w->h_local.data(), sizeof(uint32_t) * w->h_local.size(),
                           cudaMemcpyHostToDevice, w->stream), "world-local collider slots");
        CK(cudaStreamSynchronize(w->stream), "world-local collider slots");
        w->local_dirty = false;
    }
    return NPGPU_OK;
}

// The CCD layout: alive colliders by (world, slot) with each world's range
// and whether it has a CCD collider, the colliders of each body in slot
// order, and the device scratch for them (Ccd). Run when colliders or worlds
// changed.
static npgpu_status ccd_layout(npgpu_world* w) {
    w->ccd_dirty = false;
    std::vector<std::pair<uint32_t, uint32_t>> by_world;
    bool any = false;
    uint32_t maxw = 0;
    for (uint32_t ci = 0; ci < w->nc_slots; ++ci) {
        const HostCollider& c = w->hc[ci];
        if (!c.alive) continue;
        const uint32_t wd = w->hb[c.desc.body.index].world;
        by_world.push_back({wd, ci});
        any = any || c.desc.ccd_enabled != 0;
        maxw = std::max(maxw, wd);
    }
    w->ccd_any = any;
    if (!any) {
        w->dw.ccd.n_worlds = 0;
        return NPGPU_OK;
    }
    std::sort(by_world.begin(), by_world.end());
    const uint32_t nw = maxw + 1, n = (uint32_t)by_world.size();
    w->h_ccd_order.resize(std::max<uint32_t>(n, 1u));
    w->h_ccd_wstart.assign(nw + 1, 0u);
    w->h_ccd_wflag.assign(nw, 0u);
    for (uint32_t i = 0; i < n; ++i) {
        w->h_ccd_order[i] = by_world[i].second;
        w->h_ccd_wstart[by_world[i].first + 1] += 1;
        if (w->hc[by_world[i].second].desc.ccd_enabled) w->h_ccd_wflag[by_world[i].first] = 1u;
    }
    for (uint32_t k = 0; k < nw; ++k) w->h_ccd_wstart[k + 1] += w->h_ccd_wstart[k];
    w->h_ccd_list.clear();
    w->h_ccd_lstart.assign(nw + 1, 0u);
    for (uint32_t i = 0; i < n; ++i)
        if (w->hc[by_world[i].second].desc.ccd_enabled) {
            w->h_ccd_list.push_back(by_world[i].second);
            w->h_ccd_lstart[by_world[i].first + 1] += 1;
        }
    for (uint32_t k = 0; k < nw; ++k) w->h_ccd_lstart[k + 1] += w->h_ccd_lstart[k];
    w->h_bc_start.assign(w->nb_slots + 1, 0u);
    for (uint32_t ci = 0; ci < w->nc_slots; ++ci)
        if (w->hc[ci].alive) w->h_bc_start[w->hc[ci].desc.body.index + 1] += 1;
    for (uint32_t b = 0; b < w->nb_slots; ++b) w->h_bc_start[b + 1] += w->h_bc_start[b];
    w->h_bc_list.assign(std::max<uint32_t>(w->h_bc_start[w->nb_slots], 1u), 0u);
    {
        std::vector<uint32_t> fill(w->h_bc_start.begin(), w->h_bc_start.end() - 1);
        for (uint32_t ci = 0; ci < w->nc_slots; ++ci)
            if (w->hc[ci].alive) w->h_bc_list[fill[w->hc[ci].desc.body.index]++] = ci;
    }
    Ccd& cd = w->dw.ccd;
    bool ok = true;
    auto alloc = [&](std::vector<void*>& owner, void** out, size_t bytes) {
        if (!ok) return;
        void* p = nullptr;
        ok = cudaMalloc(&p, std::max<size_t>(bytes, 16)) == cudaSuccess;
        if (ok) {
            *out = p;
            owner.push_back(p);
        }
    };
    // Per body and per collider: sized by the world's capacities, once.
    if (w->ccd_bodies_cap == 0) {
        const size_t B = w->cap_b + 1, C = w->cap_c;
        alloc(w->ccd_fixed, (void**)&cd.pos0_t, sizeof(float4) * B);
        alloc(w->ccd_fixed, (void**)&cd.pos0_q, sizeof(float4) * B);
        alloc(w->ccd_fixed, (void**)&cd.btime, sizeof(float) * B);
        alloc(w->ccd_fixed, (void**)&cd.ftime, sizeof(float) * B);
        alloc(w->ccd_fixed, (void**)&cd.bflag, sizeof(uint32_t) * B);
        alloc(w->ccd_fixed, (void**)&cd.bc_start, sizeof(uint32_t) * (B + 1));
        alloc(w->ccd_fixed, (void**)&cd.sw_min, sizeof(float4) * C);
        alloc(w->ccd_fixed, (void**)&cd.sw_max, sizeof(float4) * C);
        alloc(w->ccd_fixed, (void**)&cd.cflag, sizeof(uint32_t) * C);
        alloc(w->ccd_fixed, (void**)&cd.order, sizeof(uint32_t) * C);
        alloc(w->ccd_fixed, (void**)&cd.bc_list, sizeof(uint32_t) * C);
        alloc(w->ccd_fixed, (void**)&cd.ccd_list, sizeof(uint32_t) * C);
        alloc(w->ccd_fixed, (void**)&cd.adj_count, sizeof(uint32_t) * (C + 1));
        alloc(w->ccd_fixed, (void**)&cd.adj_start, sizeof(uint32_t) * (C + 1));
        alloc(w->ccd_fixed, (void**)&cd.adj_list, sizeof(uint32_t) * 2 * (size_t)w->cap_p);
        cd.adj_scan_bytes = scan_temp_bytes((uint32_t)C + 1u);
        alloc(w->ccd_fixed, (void**)&cd.adj_scan, cd.adj_scan_bytes);
        alloc(w->ccd_fixed, (void**)&cd.bepoch, sizeof(uint32_t) * B);
        alloc(w->ccd_fixed, (void**)&cd.bcol, sizeof(unsigned long long) * B);
        // The substeps' island manifolds: up to four a collider (a wall of
        // bricks has about three contact pairs a brick), 2^24 at most.
        cd.pool_cap = (uint32_t)std::min<size_t>(std::max<size_t>(4096, 4 * C), (size_t)1 << 24);
        alloc(w->ccd_fixed, (void**)&cd.pool, sizeof(CcdManifold) * cd.pool_cap);
        if (!ok) return fail(w, NPGPU_ERR_CUDA, "CCD arrays: cudaMalloc failed");
        CK(cudaMemsetAsync(cd.bflag, 0, sizeof(uint32_t) * B, w->stream), "CCD arrays");
        CK(cudaMemsetAsync(cd.cflag, 0, sizeof(uint32_t) * C, w->stream), "CCD arrays");
        w->ccd_bodies_cap = B;
        w->ccd_colliders_cap = C;
    }
    // Per world and the worlds' regions: grown with the worlds and colliders.
    const size_t region = (size_t)kCcdRegion * n + (size_t)kCcdSlack * nw;
    if (nw > w->ccd_worlds_cap || region > w->ccd_region) {
        CK(cudaStreamSynchronize(w->stream), "CCD arrays");
        for (void* p : w->ccd_grown) cudaFree(p);
        w->ccd_grown.clear();
        const size_t W = std::max<size_t>(nw, 2 * w->ccd_worlds_cap), R = std::max<size_t>(region, 2 * w->ccd_region);
        alloc(w->ccd_grown, (void**)&cd.wstart, sizeof(uint32_t) * (W + 1));
        alloc(w->ccd_grown, (void**)&cd.ccd_wstart, sizeof(uint32_t) * (W + 1));
        alloc(w->ccd_grown, (void**)&cd.wflag, sizeof(uint32_t) * W);
        alloc(w->ccd_grown, (void**)&cd.wdts, sizeof(float) * W);
        alloc(w->ccd_grown, (void**)&cd.wstate, sizeof(uint32_t) * kCcdStateWords * W);
        alloc(w->ccd_grown, (void**)&cd.wcols, sizeof(uint32_t) * (kCcdColours + 1) * W);
        alloc(w->ccd_grown, (void**)&cd.nbr, sizeof(uint32_t) * R);
        alloc(w->ccd_grown, (void**)&cd.nbr2, sizeof(uint32_t) * R);
        alloc(w->ccd_grown, (void**)&cd.mord, sizeof(uint32_t) * R);
        alloc(w->ccd_grown, (void**)&cd.res, sizeof(uint2) * R);
        alloc(w->ccd_grown, (void**)&cd.stack, sizeof(uint32_t) * R);
        alloc(w->ccd_grown, (void**)&cd.island, sizeof(uint32_t) * R);
        alloc(w->ccd_grown, (void**)&cd.ccdb, sizeof(uint32_t) * R);
        alloc(w->ccd_grown, (void**)&cd.mlist, sizeof(uint32_t) * R);
        alloc(w->ccd_grown, (void**)&cd.tres, sizeof(float2) * R);
        alloc(w->ccd_grown, (void**)&cd.heap, sizeof(CcdToi) * R);
        alloc(w->ccd_grown, (void**)&cd.impacts, sizeof(CcdToi) * R);
        if (!ok) {
            w->ccd_worlds_cap = w->ccd_region = 0;
            return fail(w, NPGPU_ERR_CUDA, "CCD scratch: cudaMalloc failed");
        }
        w->ccd_worlds_cap = W;
        w->ccd_region = R;
    }
    CK(cudaMemcpyAsync(cd.order, w->h_ccd_order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, w->stream),
       "CCD layout");
    CK(cudaMemcpyAsync(cd.wstart, w->h_ccd_wstart.data(), sizeof(uint32_t) * (nw + 1), cudaMemcpyHostToDevice,
                       w->stream), "CCD layout");
    CK(cudaMemcpyAsync(cd.wflag, w->h_ccd_wflag.data(), sizeof(uint32_t) * nw, cudaMemcpyHostToDevice, w->stream),
       "CCD layout");
    if (!w->h_ccd_list.empty())
        CK(cudaMemcpyAsync(cd.ccd_list, w->h_ccd_list.data(), sizeof(uint32_t) * w->h_ccd_list.size(),
                           cudaMemcpyHostToDevice, w->stream), "CCD layout");
    CK(cudaMemcpyAsync(cd.ccd_wstart, w->h_ccd_lstart.data(), sizeof(uint32_t) * (nw + 1), cudaMemcpyHostToDevice,
                       w->stream), "CCD layout");
    CK(cudaMemcpyAsync(cd.bc_start, w->h_bc_start.data(), sizeof(uint32_t) * (w->nb_slots + 1),
                       cudaMemcpyHostToDevice, w->stream), "CCD layout");
    CK(cudaMemcpyAsync(cd.bc_list, w->h_bc_list.data(), sizeof(uint32_t) * w->h_bc_list.size(),
                       cudaMemcpyHostToDevice, w->stream), "CCD layout");
    CK(cudaStreamSynchronize(w->stream), "CCD layout");
    cd.n_worlds = nw;
    return NPGPU_OK;
}

static npgpu_status run_cd(npgpu_world* w, const StepParams& sp) {
    std::swap(w->dw.cur, w->dw.prev);
    sync_world_view(w);
    CK(launch_sync_aabb(w->dw, sp, w->stream), "sync aabb");
    CK(launch_sort(w->dw, w->sort_temp, w->sort_bytes, w->stream), "radix sort");
    CK(launch_lbvh(w->dw, w->stream), "lbvh");
    CK(launch_pairs(w->dw, w->scan_temp, w->scan_bytes, w->stream), "pairs");
    if (w->params.profile) CK(cudaEventRecord(w->ev[5], w->stream), "event");
    CK(launch_narrow(w->dw, w->stream), "narrow phase");
    CK(launch_events(w->dw, w->stream), "contact events");
    return NPGPU_OK;
}

// Every value a step's launches bake in: the device view of the world, the
// step parameters and the solver's launch shape.
static std::vector<uint8_t> graph_key(const npgpu_world* w, const StepParams& sp) {
    std::vector<uint8_t> k;
    auto put = [&](const void* p, size_t n) {
        const uint8_t* b = (const uint8_t*)p;
        k.insert(k.end(), b, b + n);
    };
    put(&w->dw, sizeof(w->dw));
    put(&sp, sizeof(sp));
    const SolverLaunch& L = w->solver;
    int ints[7] = {L.grid_colour,      L.grid_velocity, L.grid_position,       L.grid_world,
                   L.batched ? 1 : 0, L.world_threads, L.grid_world_position};
    put(ints, sizeof(ints));
    put(&L.scan_temp, sizeof(L.scan_temp));
    put(&L.scan_bytes, sizeof(L.scan_bytes));
    put(&L.n_worlds, sizeof(L.n_worlds));
    put(&L.max_world_bodies, sizeof(L.max_world_bodies));
    put(&L.n_big, sizeof(L.n_big));
    put(&L.n_cluster, sizeof(L.n_cluster));
    put(&L.cluster_ctas, sizeof(L.cluster_ctas));
    put(&L.cluster_shift, sizeof(L.cluster_shift));
    put(&w->sort_temp, sizeof(w->sort_temp));
    put(&w->sort_bytes, sizeof(w->sort_bytes));
    return k;
}

// One step (body start, solver, end-of-step collision detection) from a CUDA
// graph: replayed when a graph with the same key exists, else captured from
// the stream and then launched. Sets last_step_graphed; when capture is not
// possible it leaves the step to the eager path and stops trying.
static npgpu_status step_graphed(npgpu_world* w, const StepParams& sp) {
    w->solver.ev = nullptr;
    std::vector<uint8_t> key = graph_key(w, sp);
    npgpu_world::GraphSlot* g = nullptr;
    for (auto& s : w->graphs)
        if (s.exec && s.key == key) g = &s;
    if (g) {
        std::swap(w->dw.cur, w->dw.prev);   // what run_cd does on the host side
        sync_world_view(w);
    } else {
        g = &w->graphs[w->graph_next];
        w->graph_next ^= 1;
        if (g->exec) cudaGraphExecDestroy(g->exec);
        g->exec = nullptr;
        g->key.clear();
        World before = w->dw;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e0 = sp.ccd ? launch_ccd_begin(w->dw, w->stream) : cudaSuccess;
            cudaError_t e1 = e0 == cudaSuccess ? launch_body_start(w->dw, sp, w->stream) : e0;
            cudaError_t e2 = e1 == cudaSuccess ? launch_solver(w->dw, sp, w->solver, w->stream) : e1;
            if (e2 == cudaSuccess && sp.ccd) e2 = launch_ccd(w->dw, sp, w->stream);
            npgpu_status s3 = e2 == cudaSuccess ? run_cd(w, sp) : NPGPU_ERR_CUDA;
            e = cudaStreamEndCapture(w->stream, &graph);
            if (s3 != NPGPU_OK && e == cudaSuccess) e = cudaErrorStreamCaptureInvalidated;
        }
        cudaGraphExec_t exec = nullptr;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            cudaGetLastError();
            w->graphs_broken = true;
            w->dw = before;                  // nothing ran: the eager path takes the step
            sync_world_view(w);
            return NPGPU_OK;
        }
        g->exec = exec;
        g->key = key;
    }
    CK(cudaGraphLaunch(g->exec, w->stream), "graph launch");
    w->last_step_graphed = true;
    return NPGPU_OK;
}

npgpu_status npgpu_step(npgpu_world* w, uint32_t nsteps, uint32_t num_joints, uint32_t num_force_generators) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    if (num_joints != w->nj_alive)
        return fail(w, NPGPU_ERR_NONEMPTY_JOINTS,
                    "the joint set's size differs from the joints uploaded with npgpu_upsert_joints");
    if (num_force_generators) return fail(w, NPGPU_ERR_NONEMPTY_FORCES, "force generators are not supported");
    if ((w->params.warmstart_mode == 2 || w->params.warmstart_mode == 3) && !w->net_ready)
        return fail(w, NPGPU_ERR_INVALID_ARGUMENT,
                    "warmstart_mode 2 and 3 need a network (npgpu_mlp_set or npgpu_mlp_train)");
    if (w->params.warmstart_mode > 3) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "unknown warmstart_mode");
    if (w->ccd_dirty) {
        npgpu_status st = ccd_layout(w);
        if (st != NPGPU_OK) return st;
    }
    w->dw.ccd.substeps = w->params.max_ccd_substeps;
    w->dw.ccd.on_penetration = w->params.ccd_on_penetration_enabled ? 1u : 0u;
    w->dw.ccd.max_position_iterations = w->params.max_ccd_position_iterations;
    StepParams sp = step_params(w);
    w->last_step_ccd = sp.ccd != 0u;
    for (uint32_t s = 0; s < nsteps; ++s) {
        npgpu_status st = maintain(w);
        if (st != NPGPU_OK) return st;
        sync_world_view(w);
        st = prepare_schedule(w);
        if (st != NPGPU_OK) return st;
        bool prof = w->params.profile != 0;
        w->last_step_graphed = false;
        if (!prof && w->params.use_graph && !w->cd_dirty && !w->graphs_broken) {
            st = step_graphed(w, sp);
            if (st != NPGPU_OK) return st;
            if (w->last_step_graphed) {
                w->cd_start_ran = false;
                w->counters.steps += 1;
                continue;
            }
        }
        if (prof) CK(cudaEventRecord(w->ev[0], w->stream), "event");
        if (sp.ccd) CK(launch_ccd_begin(w->dw, w->stream), "CCD begin");
        CK(launch_body_start(w->dw, sp, w->stream), "body start");
        w->cd_start_ran = w->cd_dirty;
        if (w->cd_dirty) {
            st = run_cd(w, sp);
            if (st != NPGPU_OK) return st;
            w->cd_dirty = false;
        }
        if (prof) CK(cudaEventRecord(w->ev[1], w->stream), "event");
        w->solver.ev = prof ? w->ev_solver : nullptr;
        CK(launch_solver(w->dw, sp, w->solver, w->stream), "solve");
        if (sp.ccd) CK(launch_ccd(w->dw, sp, w->stream), "CCD");
        if (prof) CK(cudaEventRecord(w->ev[2], w->stream), "event");
        st = run_cd(w, sp);
        if (st != NPGPU_OK) return st;
        if (prof) {
            CK(cudaEventRecord(w->ev[3], w->stream), "event");
            w->ev_recorded = true;
        }
        w->counters.steps += 1;
    }
    return NPGPU_OK;
}

npgpu_status npgpu_synchronize(npgpu_world* w) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    uint32_t err = 0;
    CK(cudaMemcpy(&err, &w->ctl->err, sizeof(err), cudaMemcpyDeviceToHost), "read error flag");
    if (err) {
        uint32_t zero = 0;
        cudaMemcpy(&w->ctl->err, &zero, sizeof(zero), cudaMemcpyHostToDevice);
        if (err & ERRF_TIMEOUT) return fail(w, NPGPU_ERR_TIMEOUT, "a bounded device wait gave up");
        if (err & ERRF_UNION_FIND) return fail(w, NPGPU_ERR_TIMEOUT, "island union-find did not converge");
        if (err & ERRF_NAN) return fail(w, NPGPU_ERR_NAN, "non-finite body state after the step");
        if (err & ERRF_PAIR_CAPACITY) return fail(w, NPGPU_ERR_CAPACITY, "pair capacity exceeded");
        if (err & ERRF_COLOURS) return fail(w, NPGPU_ERR_CAPACITY, "more than 112 solver colours needed");
        if (err & ERRF_TASKS)
            return fail(w, NPGPU_ERR_CAPACITY, "more solver manifolds than the cooperative grid holds (16 per thread)");
        if (err & ERRF_WORLD_RANGE) return fail(w, NPGPU_ERR_CUDA, "a solver manifold left its world's slot range");
        if (err & ERRF_CCD_CAPACITY)
            return fail(w, NPGPU_ERR_CAPACITY, "a world's CCD lists or the CCD island pool overflowed");
    }
    return NPGPU_OK;
}

npgpu_status npgpu_autotune(npgpu_world* w, uint32_t steps_per_candidate, uint32_t* schedule, uint32_t* world_threads,
                            float* ms_per_step) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    if (steps_per_candidate == 0) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "steps_per_candidate must be > 0");
    if (w->params.profile) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "autotune with profiling off");
    struct Cand {
        uint32_t schedule, threads;
    };
    // One step with the automatic schedule first: it gives the solver
    // manifold count the candidates are checked against. The one-grid
    // schedule is a candidate while that count fits its cooperative grid
    // (with a 2x margin for growth).
    {
        const npgpu_params saved = w->params;
        w->params.solver_schedule = NPGPU_SCHEDULE_AUTO;
        npgpu_status st0 = npgpu_step(w, 1, w->nj_alive, 0);
        if (st0 == NPGPU_OK) st0 = npgpu_synchronize(w);
        w->params = saved;
        if (st0 != NPGPU_OK) return st0;
    }
    uint32_t nsolver = 0;
    CK(cudaMemcpy(&nsolver, &w->ctl->nsolver, sizeof(nsolver), cudaMemcpyDeviceToHost), "solver manifolds");
    std::vector<Cand> cands;
    if (2ull * nsolver <= grid_task_capacity(w->solver)) cands.push_back({NPGPU_SCHEDULE_GRID, 0});
    if (w->layout_dirty) compute_layout(w), w->layout_on_device = false;
    if (w->layout_ok && !w->params.solve_to_tolerance) {
        // The block size only shapes the block and warp worlds' kernel.
        if (w->n_cluster_worlds == w->n_worlds) cands.push_back({NPGPU_SCHEDULE_WORLDS, 128u});
        else
            for (uint32_t t : {64u, 128u, 256u}) cands.push_back({NPGPU_SCHEDULE_WORLDS, t});
    }
    if (cands.empty()) cands.push_back({w->params.solver_schedule, w->params.world_threads});
    const npgpu_params saved = w->params;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    float best_ms = 0.0f;
    Cand best = cands[0];
    npgpu_status st = NPGPU_OK;
    for (const Cand& c : cands) {
        w->params.solver_schedule = c.schedule;
        w->params.world_threads = c.threads;
        st = npgpu_step(w, 1, w->nj_alive, 0);   // capture (when graphs are on) outside the timing
        if (st != NPGPU_OK) break;
        cudaEventRecord(e0, w->stream);
        st = npgpu_step(w, steps_per_candidate, w->nj_alive, 0);
        if (st != NPGPU_OK) break;
        cudaEventRecord(e1, w->stream);
        st = npgpu_synchronize(w);
        if (st != NPGPU_OK) break;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)steps_per_candidate;
        if (&c == &cands[0] || ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    w->params = saved;
    if (st != NPGPU_OK) return st;
    // Every candidate computes the same bits; only the launch shape is chosen.
    w->params.solver_schedule = best.schedule;
    w->params.world_threads = best.threads;
    if (schedule) *schedule = best.schedule;
    if (world_threads) *world_threads = best.threads;
    if (ms_per_step) *ms_per_step = best_ms;
    return NPGPU_OK;
}

npgpu_status npgpu_download_bodies(npgpu_world* w, uint32_t first, uint32_t n, float* position, float* velocity,
                                   float* energy, uint8_t* active) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    if ((uint64_t)first + n > w->cap_b) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "range beyond capacity");
    if (n == 0) return NPGPU_OK;
    size_t bytes = (size_t)n * (7 + 6 + 1) * sizeof(float) + n;
    CK(cudaEventSynchronize(w->ev_stage), "staging wait");
    if (!energy && !active && (position || velocity)) {
        // Page-locked destinations the device can address: the pack kernel
        // writes them over the host link itself, with no copy afterwards.
        float* dpos_h = (float*)host_device_ptr(position);
        float* dvel_h = (float*)host_device_ptr(velocity);
        if ((!position || dpos_h) && (!velocity || dvel_h)) {
            CK(launch_pack_bodies_host(w->dw, first, n, dpos_h, dvel_h, w->stream), "pack bodies");
            CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
            CK(cudaStreamSynchronize(w->stream), "download");
            return NPGPU_OK;
        }
    }
    if (bytes > w->d_stage_bytes) {
        if (w->d_stage) cudaFree(w->d_stage);
    if (w->d_query) cudaFree(w->d_query);
    if (w->dw.events) cudaFree(w->dw.events);
        w->d_stage = nullptr;
        CK(cudaMalloc(&w->d_stage, bytes), "device staging");
        w->d_stage_bytes = bytes;
    }
    if (bytes > w->h_stage_bytes) {
        if (w->h_stage) cudaFreeHost(w->h_stage);
        w->h_stage = nullptr;
        CK(cudaMallocHost(&w->h_stage, bytes), "pinned staging");
        w->h_stage_bytes = bytes;
    }
    float* dpos = (float*)w->d_stage;
    float* dvel = dpos + 7 * (size_t)n;
    float* den = dvel + 6 * (size_t)n;
    uint8_t* dact = (uint8_t*)(den + n);
    CK(launch_pack_bodies(w->dw, first, n, position ? dpos : nullptr, velocity ? dvel : nullptr, energy ? den : nullptr,
                          active ? dact : nullptr, w->stream),
       "pack bodies");
    if (host_pinned(position) && host_pinned(velocity) && host_pinned(energy) && host_pinned(active)) {
        // Page-locked destinations: the copy engines write them directly.
        if (position) CK(cudaMemcpyAsync(position, dpos, 7 * sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream), "d2h");
        if (velocity) CK(cudaMemcpyAsync(velocity, dvel, 6 * sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream), "d2h");
        if (energy) CK(cudaMemcpyAsync(energy, den, sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream), "d2h");
        if (active) CK(cudaMemcpyAsync(active, dact, n, cudaMemcpyDeviceToHost, w->stream), "d2h");
        CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
        CK(cudaStreamSynchronize(w->stream), "download");
        return NPGPU_OK;
    }
    char* h = (char*)w->h_stage;
    if (position) CK(cudaMemcpyAsync(h, dpos, 7 * sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream), "d2h");
    if (velocity)
        CK(cudaMemcpyAsync(h + 7 * sizeof(float) * n, dvel, 6 * sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream),
           "d2h");
    if (energy) CK(cudaMemcpyAsync(h + 13 * sizeof(float) * n, den, sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream), "d2h");
    if (active) CK(cudaMemcpyAsync(h + 14 * sizeof(float) * n, dact, n, cudaMemcpyDeviceToHost, w->stream), "d2h");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    CK(cudaStreamSynchronize(w->stream), "download");
    if (position) std::memcpy(position, h, 7 * sizeof(float) * n);
    if (velocity) std::memcpy(velocity, h + 7 * sizeof(float) * n, 6 * sizeof(float) * n);
    if (energy) std::memcpy(energy, h + 13 * sizeof(float) * n, sizeof(float) * n);
    if (active) std::memcpy(active, h + 14 * sizeof(float) * n, n);
    return NPGPU_OK;
}

npgpu_status npgpu_download_mass_properties(npgpu_world* w, uint32_t first, uint32_t n, float* local_inertia,
                                            float* local_com) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    if ((uint64_t)first + n > w->cap_b) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "range beyond capacity");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    std::vector<float> mass(n), I(9 * (size_t)n);
    std::vector<float4> com(n);
    if (n) {
        CK(cudaMemcpy(mass.data(), w->dw.b.mass + first, sizeof(float) * n, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(I.data(), w->dw.b.local_I + 9 * (size_t)first, sizeof(float) * 9 * n, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(com.data(), w->dw.b.local_com + first, sizeof(float4) * n, cudaMemcpyDeviceToHost), "d2h");
    }
    for (uint32_t k = 0; k < n; ++k) {
        if (local_inertia) {
            float* o = local_inertia + 7 * (size_t)k;
            const float* a = I.data() + 9 * (size_t)k;
            o[0] = mass[k]; o[1] = a[0]; o[2] = a[1]; o[3] = a[2]; o[4] = a[4]; o[5] = a[5]; o[6] = a[8];
        }
        if (local_com) {
            local_com[3 * k] = com[k].x;
            local_com[3 * k + 1] = com[k].y;
            local_com[3 * k + 2] = com[k].z;
        }
    }
    return NPGPU_OK;
}

static npgpu_status read_npairs(npgpu_world* w, uint32_t* np_) {
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    CK(cudaMemcpy(np_, &w->ctl->npairs, sizeof(uint32_t), cudaMemcpyDeviceToHost), "d2h");
    return NPGPU_OK;
}

npgpu_status npgpu_get_pairs(npgpu_world* w, uint32_t* pairs2, uint32_t max, uint32_t* count) {
    if (!w || !count) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    uint32_t np_ = 0;
    npgpu_status st = read_npairs(w, &np_);
    if (st != NPGPU_OK) return st;
    std::vector<uint2> pr(np_);
    if (np_) CK(cudaMemcpy(pr.data(), w->dw.cur.pair, sizeof(uint2) * np_, cudaMemcpyDeviceToHost), "d2h");
    std::vector<uint64_t> keys;
    keys.reserve(np_);
    for (auto& p : pr)
        if (p.x != 0xffffffffu) keys.push_back(((uint64_t)p.x << 32) | p.y);
    std::sort(keys.begin(), keys.end());
    *count = (uint32_t)keys.size();
    for (uint32_t k = 0; k < keys.size() && k < max && pairs2; ++k) {
        pairs2[2 * k] = (uint32_t)(keys[k] >> 32);
        pairs2[2 * k + 1] = (uint32_t)keys[k];
    }
    return NPGPU_OK;
}

npgpu_status npgpu_get_aabbs(npgpu_world* w, uint32_t first, uint32_t n, float* aabb6) {
    if (!w || (n && !aabb6)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    if ((uint64_t)first + n > w->cap_c) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "range beyond capacity");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    std::vector<float4> mn(n), mx(n);
    if (n) {
        CK(cudaMemcpy(mn.data(), w->dw.c.aabb_min + first, sizeof(float4) * n, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(mx.data(), w->dw.c.aabb_max + first, sizeof(float4) * n, cudaMemcpyDeviceToHost), "d2h");
    }
    for (uint32_t k = 0; k < n; ++k) {
        float* o = aabb6 + 6 * (size_t)k;
        o[0] = mn[k].x; o[1] = mn[k].y; o[2] = mn[k].z; o[3] = mx[k].x; o[4] = mx[k].y; o[5] = mx[k].z;
    }
    return NPGPU_OK;
}

npgpu_status npgpu_get_contacts(npgpu_world* w, npgpu_contact* out, uint32_t max, uint32_t* count) {
    if (!w || !count) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    uint32_t np_ = 0;
    npgpu_status st = read_npairs(w, &np_);
    if (st != NPGPU_OK) return st;
    const Pairs& P = w->dw.cur;
    std::vector<uint2> pr(np_);
    std::vector<uint8_t> nc(np_);
    size_t ns = 4 * (size_t)np_;
    std::vector<uint32_t> key(ns);
    std::vector<float4> w1(ns), w2(ns), nn(ns), imp(ns);
    if (np_) {
        CK(cudaMemcpy(pr.data(), P.pair, sizeof(uint2) * np_, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(nc.data(), P.ncont, np_, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(key.data(), P.key, 4 * ns, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(w1.data(), P.w1, 16 * ns, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(w2.data(), P.w2, 16 * ns, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(nn.data(), P.n, 16 * ns, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(imp.data(), P.imp, 16 * ns, cudaMemcpyDeviceToHost), "d2h");
    }
    std::vector<npgpu_contact> all;
    for (uint32_t p = 0; p < np_; ++p) {
        if (pr[p].x == 0xffffffffu) continue;
        for (uint32_t k = 0; k < nc[p]; ++k) {
            size_t s = 4 * (size_t)p + k;
            npgpu_contact c;
            std::memset(&c, 0, sizeof(c));
            c.collider1 = pr[p].x;
            c.collider2 = pr[p].y;
            c.feature_key = key[s];
            uint32_t f1 = key[s] / 26u, f2 = key[s] % 26u;
            auto kind = [](const HostCollider& hc, uint32_t f) -> uint32_t {
                if (hc.desc.shape == NPGPU_SHAPE_BALL) return 1u;
                return f < 8 ? 1u : (f < 20 ? 2u : 3u);
            };
            c.kinematic = kind(w->hc[c.collider1], f1) | (kind(w->hc[c.collider2], f2) << 8);
            c.world1[0] = w1[s].x; c.world1[1] = w1[s].y; c.world1[2] = w1[s].z;
            c.world2[0] = w2[s].x; c.world2[1] = w2[s].y; c.world2[2] = w2[s].z;
            c.normal[0] = nn[s].x; c.normal[1] = nn[s].y; c.normal[2] = nn[s].z;
            c.depth = w1[s].w;
            c.impulse[0] = imp[s].x; c.impulse[1] = imp[s].y; c.impulse[2] = imp[s].z;
            c.colour = 0xffffffffu;
            all.push_back(c);
        }
    }
    std::sort(all.begin(), all.end(), [](const npgpu_contact& a, const npgpu_contact& b) {
        if (a.collider1 != b.collider1) return a.collider1 < b.collider1;
        if (a.collider2 != b.collider2) return a.collider2 < b.collider2;
        return a.feature_key < b.feature_key;
    });
    *count = (uint32_t)all.size();
    if (out)
        for (uint32_t k = 0; k < all.size() && k < max; ++k) out[k] = all[k];
    return NPGPU_OK;
}

// ---------------------------------------------------------------- learned warm start
static_assert(NPGPU_MLP_PARAMS == (unsigned)kMlpParams, "parameter layout");
static_assert(NPGPU_MLP_TRAINABLE == (unsigned)kMlpTrainable, "parameter layout");
static_assert(NPGPU_MLP_SAMPLE_FLOATS == (unsigned)kMlpSampleFloats, "sample layout");

static npgpu_status mlp_alloc(npgpu_world* w) {
    if (w->d_net) return NPGPU_OK;
    CK(cudaMalloc(&w->d_net, sizeof(MlpDev)), "network");
    CK(cudaMalloc(&w->d_prm, sizeof(float) * kMlpParams), "network parameters");
    CK(cudaMalloc(&w->d_m1, sizeof(float) * kMlpTrainable), "adam");
    CK(cudaMalloc(&w->d_m2, sizeof(float) * kMlpTrainable), "adam");
    CK(cudaMalloc(&w->d_grad, sizeof(float) * kMlpTrainable), "gradient");
    CK(cudaMalloc(&w->d_stats, sizeof(double) * 2 * (kMlpIn + kMlpOut)), "statistics");
    // The starts that learned predictions replace, one per contact slot.
    CK(cudaMalloc(&w->dw.s.lam_alt, sizeof(float4) * kMaxContacts * (size_t)w->cap_p), "replaced starts");
    w->owned.push_back(w->dw.s.lam_alt);
    return NPGPU_OK;
}

static npgpu_status mlp_reset_adam(npgpu_world* w) {
    CK(cudaMemsetAsync(w->d_m1, 0, sizeof(float) * kMlpTrainable, w->stream), "adam");
    CK(cudaMemsetAsync(w->d_m2, 0, sizeof(float) * kMlpTrainable, w->stream), "adam");
    w->adam_t = 0;
    return NPGPU_OK;
}

static uint32_t mlp_count(npgpu_world* w) {
    uint32_t n = 0;
    if (cudaMemcpy(&n, &w->ctl->mlp_samples, sizeof(n), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
    return std::min(n, w->sample_cap);
}

npgpu_status npgpu_mlp_set(npgpu_world* w, const float* params, uint32_t n) {
    if (!w || !params) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (n != kMlpParams) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "expected NPGPU_MLP_PARAMS parameters");
    if (!finite_n(params, (int)n)) return fail(w, NPGPU_ERR_NAN, "network parameters are not finite");
    npgpu_status st = mlp_alloc(w);
    if (st != NPGPU_OK) return st;
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    CK(cudaMemcpy(w->d_prm, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice), "network upload");
    CK(mlp_upload(w->d_prm, w->d_net, w->stream), "network upload");
    st = mlp_reset_adam(w);
    if (st != NPGPU_OK) return st;
    w->net_ready = true;
    w->dw.mlp = w->d_net;
    return NPGPU_OK;
}

npgpu_status npgpu_mlp_get(npgpu_world* w, float* params, uint32_t n) {
    if (!w || !params) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (n < kMlpParams) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "buffer smaller than NPGPU_MLP_PARAMS");
    if (!w->net_ready) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "no network");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    CK(cudaMemcpy(params, w->d_prm, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost), "network download");
    return NPGPU_OK;
}

npgpu_status npgpu_mlp_record(npgpu_world* w, uint32_t capacity) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    if (capacity == 0) {
        w->dw.s.feat = nullptr;
        return NPGPU_OK;
    }
    if (!w->d_feat) CK(cudaMalloc(&w->d_feat, sizeof(float) * kMlpIn * kMaxContacts * (size_t)w->cap_p), "features");
    if (capacity > w->sample_cap) {
        cudaFree(w->d_samples);
        w->d_samples = nullptr;
        w->sample_cap = 0;
        CK(cudaMalloc(&w->d_samples, sizeof(float) * kMlpSampleFloats * (size_t)capacity), "samples");
    }
    w->sample_cap = capacity;
    uint32_t zero = 0;
    CK(cudaMemcpy(&w->ctl->mlp_samples, &zero, sizeof(zero), cudaMemcpyHostToDevice), "samples");
    w->dw.s.feat = w->d_feat;
    w->dw.s.samples = w->d_samples;
    w->dw.s.sample_cap = capacity;
    return NPGPU_OK;
}

npgpu_status npgpu_mlp_samples(npgpu_world* w, float* out, uint32_t max_samples, uint32_t* count) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    uint32_t n = w->d_samples ? mlp_count(w) : 0;
    if (count) *count = n;
    if (out && n) {
        uint32_t k = std::min(n, max_samples);
        CK(cudaMemcpy(out, w->d_samples, sizeof(float) * kMlpSampleFloats * (size_t)k, cudaMemcpyDeviceToHost),
           "samples download");
    }
    return NPGPU_OK;
}

npgpu_status npgpu_mlp_load_samples(npgpu_world* w, const float* samples, uint32_t n) {
    if (!w || (n && !samples)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (!finite_n(samples, (int)std::min<uint64_t>((uint64_t)n * kMlpSampleFloats, 0x7fffffffu)))
        return fail(w, NPGPU_ERR_NAN, "samples are not finite");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    w->dw.s.feat = nullptr;   // recording stops
    if (n > w->sample_cap || !w->d_samples) {
        cudaFree(w->d_samples);
        w->d_samples = nullptr;
        w->sample_cap = 0;
        CK(cudaMalloc(&w->d_samples, sizeof(float) * kMlpSampleFloats * (size_t)std::max(n, 1u)), "samples");
    }
    w->sample_cap = std::max(n, 1u);
    if (n) CK(cudaMemcpy(w->d_samples, samples, sizeof(float) * kMlpSampleFloats * (size_t)n, cudaMemcpyHostToDevice),
              "samples upload");
    CK(cudaMemcpy(&w->ctl->mlp_samples, &n, sizeof(n), cudaMemcpyHostToDevice), "samples");
    w->dw.s.samples = w->d_samples;
    w->dw.s.sample_cap = 0;
    return NPGPU_OK;
}

npgpu_status npgpu_mlp_train(npgpu_world* w, uint32_t steps, uint32_t batch, float lr, uint32_t seed, uint32_t flags,
                             float* final_loss) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    if (batch == 0 || batch % 64 != 0 || batch > (1u << 20))
        return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "batch must be a positive multiple of 64 (at most 2^20)");
    if (!(lr > 0.0f)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "lr must be positive");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    const uint32_t n = w->d_samples ? mlp_count(w) : 0;
    if (n == 0) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "no recorded samples (npgpu_mlp_record)");
    npgpu_status st = mlp_alloc(w);
    if (st != NPGPU_OK) return st;
    if ((flags & NPGPU_MLP_INIT) || !w->net_ready) {
        CK(mlp_init(w->d_prm, seed, w->stream), "network init");
        CK(mlp_normalise(w->d_samples, n, w->d_stats, w->d_prm, w->stream), "normalisation");
        CK(mlp_upload(w->d_prm, w->d_net, w->stream), "network upload");
        st = mlp_reset_adam(w);
        if (st != NPGPU_OK) return st;
        w->net_ready = true;
        w->dw.mlp = w->d_net;
    }
    const uint32_t bseed = (seed * 2654435761u) | 1u;   // non-zero: batches drawn by hash
    for (uint32_t k = 0; k < steps; ++k) {
        CK(mlp_grad(w->d_net, w->d_samples, n, batch, bseed, w->adam_t, w->d_grad, &w->ctl->mlp_loss, w->stream),
           "network gradient");
        CK(mlp_adam(w->d_prm, w->d_m1, w->d_m2, w->d_grad, lr, ++w->adam_t, w->d_net, w->stream), "adam");
    }
    CK(cudaStreamSynchronize(w->stream), "training");
    if (final_loss) {
        double l = 0.0;
        CK(cudaMemcpy(&l, &w->ctl->mlp_loss, sizeof(l), cudaMemcpyDeviceToHost), "loss");
        *final_loss = (float)l;
    }
    return NPGPU_OK;
}

npgpu_status npgpu_mlp_grad(npgpu_world* w, const float* samples, uint32_t n, float* grad, float* loss) {
    if (!w || !samples || !grad) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0 || n > 65536) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "1 <= n <= 65536 samples");
    if (!w->net_ready) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "no network");
    void* dp = nullptr;
    npgpu_status st = stage_upload(w, samples, sizeof(float) * kMlpSampleFloats * (size_t)n, &dp);
    if (st != NPGPU_OK) return st;
    CK(mlp_grad(w->d_net, (const float*)dp, n, n, 0u, 0u, w->d_grad, &w->ctl->mlp_loss, w->stream), "network gradient");
    CK(cudaEventRecord(w->ev_stage, w->stream), "staging event");
    CK(cudaStreamSynchronize(w->stream), "gradient");
    CK(cudaMemcpy(grad, w->d_grad, sizeof(float) * kMlpTrainable, cudaMemcpyDeviceToHost), "gradient download");
    if (loss) {
        double l = 0.0;
        CK(cudaMemcpy(&l, &w->ctl->mlp_loss, sizeof(l), cudaMemcpyDeviceToHost), "loss");
        *loss = (float)l;
    }
    return NPGPU_OK;
}

npgpu_status npgpu_get_counters(npgpu_world* w, npgpu_counters* out) {
    if (!w || !out) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    Control c;
    CK(cudaMemcpy(&c, w->ctl, sizeof(Control), cudaMemcpyDeviceToHost), "d2h");
    npgpu_counters& k = w->counters;
    k.num_pairs = c.npairs;
    k.num_manifolds = c.nmanifolds;
    k.num_contacts = c.ncontacts;
    k.num_solver_contacts = c.nsolver_contacts;
    k.num_constraints = 3 * c.nsolver_contacts;
    k.num_colours = c.ncolours;
    k.num_active_bodies = c.nactive;
    k.velocity_iterations = c.iterations;
    k.residual = c.residual;
    k.residual_initial = c.residual_initial;
    unsigned long long bits = c.max_pen_bits;
    if (c.ncontacts == 0 || bits == 0) {
        k.max_penetration = 0.0;
    } else {
        unsigned long long raw = (bits & 0x8000000000000000ull) ? (bits & ~0x8000000000000000ull) : ~bits;
        double v;
        std::memcpy(&v, &raw, sizeof(v));
        k.max_penetration = v;
    }
    k.kinetic_energy = c.kinetic_energy;
    k.learned_starts = c.learned_starts;
    k.learned_kept = c.learned_kept;
    k.graph_replay = w->last_step_graphed ? 1u : 0u;
    k.ccd_substeps = w->last_step_ccd ? c.ccd_substeps : 0u;
    k.ccd_impacts = w->last_step_ccd ? c.ccd_impacts : 0u;
    if (w->params.profile && w->ev_recorded) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, w->ev[0], w->ev[3]);
        k.step_time = ms;
        cudaEventElapsedTime(&ms, w->ev[1], w->ev[2]);
        k.solver_time = ms;
        cudaEventElapsedTime(&ms, w->ev[2], w->ev[3]);
        k.collision_detection_time = ms;
        cudaEventElapsedTime(&ms, w->ev[2], w->ev[5]);
        k.broad_phase_time = ms;
        cudaEventElapsedTime(&ms, w->ev[5], w->ev[3]);
        k.narrow_phase_time = ms;
        auto d = [&](int a, int b) {
            float t = 0.0f;
            cudaEventElapsedTime(&t, w->ev_solver[a], w->ev_solver[b]);
            return (double)t;
        };
        k.island_construction_time = d(0, 1);
        k.colouring_time = d(1, 2);
        k.assembly_time = d(2, 3);
        k.velocity_resolution_time = d(3, 4);
        k.velocity_update_time = d(4, 5);
        k.position_resolution_time = d(5, 6);
        k.velocity_task_ms = (double)c.task_ns * 1e-6;
        k.velocity_wait_ms = (double)c.wait_ns * 1e-6;
        k.velocity_kernel_ms = (double)c.t_phase[0] * 1e-6;
        k.velocity_tasks = c.tasks;
        if (w->last_step_ccd) {
            k.ccd_toi_computation_time = (double)c.ccd_ns[0] * 1e-6;
            k.ccd_solver_time = (double)c.ccd_ns[1] * 1e-6;
            k.ccd_broad_phase_time = (double)c.ccd_ns[2] * 1e-6;
            k.ccd_narrow_phase_time = (double)c.ccd_ns[3] * 1e-6;
            k.ccd_world_time_max = (double)c.ccd_max_ns * 1e-6;
        }
    }
    *out = k;
    return NPGPU_OK;
}

// ---------------------------------------------------------------- queries and events

struct HostHit {
    uint32_t q, collider;
    float toi, nx, ny, nz;
};

// Runs one batch of queries (kind 0 rays, 1 points, 2 boxes) and returns every
// hit sorted by (query, collider).
static npgpu_status run_queries(npgpu_world* w, int kind, uint32_t n, const float* qd, const float* max_toi,
                                uint32_t world, std::vector<HostHit>& hits) {
    hits.clear();
    if (n == 0 || w->nc_alive == 0) return NPGPU_OK;
    const int per = kind == 1 ? 3 : 6;
    if (!finite_n(qd, (int)std::min<uint64_t>((uint64_t)n * per, 0x7fffffffu)) ||
        (max_toi && !finite_n(max_toi, (int)n)))
        return fail(w, NPGPU_ERR_NAN, "query values are not finite");
    auto a256 = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t in_b = a256(sizeof(float) * per * (size_t)n), toi_b = a256(sizeof(float) * (size_t)n);
    const size_t cnt_b = a256(sizeof(uint32_t) * (size_t)n), scan_b = a256(scan_temp_bytes(n));
    size_t need = in_b + toi_b + 2 * cnt_b + scan_b;
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    if (need > w->query_bytes) {
        if (w->d_query) cudaFree(w->d_query);
        w->d_query = nullptr;
        w->query_bytes = 0;
        CK(cudaMalloc(&w->d_query, need), "query buffers");
        w->query_bytes = need;
    }
    unsigned char* base = (unsigned char*)w->d_query;
    float* d_in = (float*)base;
    float* d_toi = (float*)(base + in_b);
    uint32_t* d_cnt = (uint32_t*)(base + in_b + toi_b);
    uint32_t* d_off = (uint32_t*)(base + in_b + toi_b + cnt_b);
    void* d_scan = base + in_b + toi_b + 2 * cnt_b;
    CK(cudaMemcpy(d_in, qd, sizeof(float) * per * (size_t)n, cudaMemcpyHostToDevice), "query upload");
    if (max_toi) CK(cudaMemcpy(d_toi, max_toi, sizeof(float) * n, cudaMemcpyHostToDevice), "query upload");
    sync_world_view(w);
    CK(launch_query(w->dw, kind, d_in, d_toi, n, world, d_cnt, d_off, d_scan, scan_b, nullptr, 0, w->stream),
       "query count");
    uint32_t last_off = 0, last_cnt = 0;
    CK(cudaMemcpyAsync(&last_off, d_off + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream), "d2h");
    CK(cudaMemcpyAsync(&last_cnt, d_cnt + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream), "d2h");
    CK(cudaStreamSynchronize(w->stream), "query count");
    const uint32_t total = last_off + last_cnt;
    if (total == 0) return NPGPU_OK;
    void* d_out = nullptr;
    CK(cudaMalloc(&d_out, query_hit_bytes() * total), "query hits");
    cudaError_t e = launch_query(w->dw, kind, d_in, d_toi, n, world, d_cnt, d_off, d_scan, scan_b, d_out, total,
                                 w->stream);
    if (e == cudaSuccess) {
        hits.resize(total);
        e = cudaMemcpyAsync(hits.data(), d_out, sizeof(HostHit) * total, cudaMemcpyDeviceToHost, w->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
    cudaFree(d_out);
    if (e != cudaSuccess) return cuda_fail(w, e, "query hits");
    std::sort(hits.begin(), hits.end(),
              [](const HostHit& a, const HostHit& b) { return a.q != b.q ? a.q < b.q : a.collider < b.collider; });
    return NPGPU_OK;
}

npgpu_status npgpu_interferences_with_rays(npgpu_world* w, uint32_t n, const float* rays6, const float* max_toi,
                                           uint32_t world, npgpu_ray_hit* hits, uint32_t max_hits, uint32_t* count) {
    if (!w || !count || (n && (!rays6 || !max_toi)) || (max_hits && !hits))
        return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    static_assert(sizeof(HostHit) == 24, "hit record layout");
    std::vector<HostHit> h;
    npgpu_status st = run_queries(w, 0, n, rays6, max_toi, world, h);
    if (st != NPGPU_OK) return st;
    *count = (uint32_t)h.size();
    for (uint32_t k = 0; k < h.size() && k < max_hits; ++k) {
        hits[k].ray = h[k].q;
        hits[k].collider = h[k].collider;
        hits[k].toi = h[k].toi;
        hits[k].normal[0] = h[k].nx;
        hits[k].normal[1] = h[k].ny;
        hits[k].normal[2] = h[k].nz;
    }
    return NPGPU_OK;
}

static npgpu_status pair_queries(npgpu_world* w, int kind, uint32_t n, const float* q, uint32_t world, uint32_t* hits2,
                                 uint32_t max_hits, uint32_t* count) {
    if (!w || !count || (n && !q) || (max_hits && !hits2)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<HostHit> h;
    npgpu_status st = run_queries(w, kind, n, q, nullptr, world, h);
    if (st != NPGPU_OK) return st;
    *count = (uint32_t)h.size();
    for (uint32_t k = 0; k < h.size() && k < max_hits; ++k) {
        hits2[2 * k] = h[k].q;
        hits2[2 * k + 1] = h[k].collider;
    }
    return NPGPU_OK;
}

npgpu_status npgpu_interferences_with_points(npgpu_world* w, uint32_t n, const float* points3, uint32_t world,
                                             uint32_t* hits2, uint32_t max_hits, uint32_t* count) {
    return pair_queries(w, 1, n, points3, world, hits2, max_hits, count);
}

npgpu_status npgpu_interferences_with_aabbs(npgpu_world* w, uint32_t n, const float* aabbs6, uint32_t world,
                                            uint32_t* hits2, uint32_t max_hits, uint32_t* count) {
    return pair_queries(w, 2, n, aabbs6, world, hits2, max_hits, count);
}

npgpu_status npgpu_enable_contact_events(npgpu_world* w, uint32_t capacity) {
    if (!w) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null world");
    if (capacity && w->cap_c > (1u << 26))
        return fail(w, NPGPU_ERR_CAPACITY, "events need collider slots below 2^26");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    if (w->dw.events) cudaFree(w->dw.events);
    w->dw.events = nullptr;
    w->dw.events_cap = 0;
    if (capacity) {
        CK(cudaMalloc(&w->dw.events, sizeof(uint2) * (size_t)capacity), "contact events");
        w->dw.events_cap = capacity;
    }
    uint32_t zero = 0;
    CK(cudaMemcpy(&w->ctl->nevents, &zero, sizeof(zero), cudaMemcpyHostToDevice), "contact events");
    return NPGPU_OK;
}

// The step's recorded events in recording order (ev), and how many were
// emitted (n; above the capacity when some were lost).
static npgpu_status read_events(npgpu_world* w, std::vector<uint2>& ev, uint32_t& n) {
    if (!w->dw.events) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "events are off (npgpu_enable_contact_events)");
    CK(cudaStreamSynchronize(w->stream), "synchronize");
    n = 0;
    CK(cudaMemcpy(&n, &w->ctl->nevents, sizeof(n), cudaMemcpyDeviceToHost), "d2h");
    const uint32_t kept = std::min(n, w->dw.events_cap);
    ev.resize(kept);
    if (kept) CK(cudaMemcpy(ev.data(), w->dw.events, sizeof(uint2) * kept, cudaMemcpyDeviceToHost), "d2h");
    return NPGPU_OK;
}

npgpu_status npgpu_contact_events(npgpu_world* w, npgpu_contact_event* out, uint32_t max, uint32_t* count) {
    if (!w || !count || (max && !out)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<uint2> ev;
    uint32_t n = 0;
    npgpu_status st = read_events(w, ev, n);
    if (st != NPGPU_OK) return st;
    std::vector<uint64_t> keys;
    for (const uint2& e : ev)
        if (!(e.y & 0x40000000u))
            keys.push_back(((uint64_t)e.x << 33) | ((uint64_t)(e.y & 0x3fffffffu) << 1) | (e.y >> 31));
    std::sort(keys.begin(), keys.end());
    const uint32_t kept = (uint32_t)keys.size();
    *count = kept;
    for (uint32_t k = 0; k < kept && k < max; ++k) {
        out[k].collider1 = (uint32_t)(keys[k] >> 33);
        out[k].collider2 = (uint32_t)((keys[k] >> 1) & 0xffffffffu);
        out[k].stopped = (uint32_t)(keys[k] & 1u);
    }
    if (n > w->dw.events_cap)
        return fail(w, NPGPU_ERR_CAPACITY, "more contact events than the capacity given to npgpu_enable_contact_events");
    return NPGPU_OK;
}

npgpu_status npgpu_proximity_events(npgpu_world* w, npgpu_proximity_event* out, uint32_t max, uint32_t* count) {
    if (!w || !count || (max && !out)) return fail(w, NPGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<uint2> ev;
    uint32_t n = 0;
    npgpu_status st = read_events(w, ev, n);
    if (st != NPGPU_OK) return st;
    // Stable by pair: the passes append in order, and a pair has at most one
    // event a pass.
    std::vector<uint2> px;
    for (const uint2& e : ev)
        if (e.y & 0x40000000u) px.push_back(e);
    std::stable_sort(px.begin(), px.end(), [](const uint2& a, const uint2& b) {
        const uint32_t a2 = a.y & 0x03ffffffu, b2 = b.y & 0x03ffffffu;
        return a.x != b.x ? a.x < b.x : a2 < b2;
    });
    *count = (uint32_t)px.size();
    for (uint32_t k = 0; k < px.size() && k < max; ++k) {
        out[k].collider1 = px[k].x;
        out[k].collider2 = px[k].y & 0x03ffffffu;
        out[k].prev_status = (px[k].y >> 26) & 3u;
        out[k].new_status = (px[k].y >> 28) & 3u;
    }
    if (n > w->dw.events_cap)
        return fail(w, NPGPU_ERR_CAPACITY, "more events than the capacity given to npgpu_enable_contact_events");
    return NPGPU_OK;
}

const char* npgpu_last_error(const npgpu_world* w) {
    if (!w) return g_create_error.c_str();
    return w->last_error.c_str();
}

}  // extern "C"
