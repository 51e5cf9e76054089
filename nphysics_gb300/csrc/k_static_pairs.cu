// k_static_pairs.cu -- broad phase over caller-provided AABBs with no
// allocation: npgpu_find_pairs_static.
//
// Some callers cannot call cudaMalloc: real-time control loops that must not
// block on the allocator (cudaMalloc can synchronise the device and take
// milliseconds), and plugins hosted by an application that owns all device
// memory through its own pool and forbids allocations behind its back. For
// them this entry point runs the broad phase of the step (Morton keys, radix sort,
// linear BVH, owner traversal) on device buffers they already hold, with every
// piece of scratch memory taken from one file-scope __device__ array of fixed
// size (kScratchBytes, enough for kMaxAabbs boxes). Every GPU that loads the
// library holds that array until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and checks the scratch
// needs of the sort and scan; make that first call before any stream capture.
// The address belongs to the device's current context: after the context is
// destroyed and recreated (cudaDeviceReset), the next call sees a new
// context id and does the set-up again.
// Calls share the array: two calls whose work overlaps on the GPU (on
// different streams, or on the same stream from different threads before the
// first finishes) race on it.
#include <mutex>
#include <string>

#include "../../include/npgpu.h"
#include "sortscan.cuh"

namespace {

constexpr uint32_t kMaxAabbs = 32768;
constexpr size_t kScratchBytes = 8u << 20;

static __device__ __align__(256) unsigned char g_pair_scratch[kScratchBytes];

struct Layout {
    size_t keys, keys_sorted, vals, vals_sorted, left, right, parent, node_min, node_max, node_flag, leaf_count,
        leaf_offset, total, sort_temp, scan_temp, end;
    size_t sort_bytes, scan_bytes;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

Layout make_layout(uint32_t n) {
    Layout l;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    l.keys = take(8ull * n);
    l.keys_sorted = take(8ull * n);
    l.vals = take(4ull * n);
    l.vals_sorted = take(4ull * n);
    l.left = take(4ull * n);
    l.right = take(4ull * n);
    l.parent = take(8ull * n);
    l.node_min = take(32ull * n);
    l.node_max = take(32ull * n);
    l.node_flag = take(4ull * n);
    l.leaf_count = take(4ull * n);
    l.leaf_offset = take(4ull * n);
    l.total = take(16);
    l.sort_bytes = npgpu_dev::radix_sort_temp_bytes(n);
    l.scan_bytes = npgpu_dev::exclusive_scan_temp_bytes(n);
    l.sort_temp = take(l.sort_bytes);
    l.scan_temp = take(l.scan_bytes);
    l.end = o;
    return l;
}

std::mutex g_mu;
unsigned char* g_scratch_ptr[64];
unsigned long long g_ctx_id[64];
bool g_ready[64];

// Unique id of the calling thread's current CUDA context (cuCtxGetId, reached
// through the runtime's driver entry points so that the library needs no
// link-time dependency on the driver library), or 0 if it cannot be read.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (CtxGetCurrentFn)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (CtxGetIdFn)f;
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

__device__ __forceinline__ uint64_t expand16s(uint32_t v) {
    uint64_t x = v & 0xffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}
__device__ __forceinline__ uint32_t quantize_s(float c) {
    float q = floorf(c * 4.0f) + 32768.0f;
    q = q < 0.0f ? 0.0f : (q > 65535.0f ? 65535.0f : q);
    return (uint32_t)q;
}

struct Scratch {
    unsigned long long *keys, *keys_sorted;
    uint32_t *vals, *vals_sorted;
    int *left, *right, *parent;
    float4 *node_min, *node_max;
    int* node_flag;
    uint32_t *leaf_count, *leaf_offset, *total;
};

Scratch scratch_at(unsigned char* base, const Layout& l) {
    Scratch s;
    s.keys = (unsigned long long*)(base + l.keys);
    s.keys_sorted = (unsigned long long*)(base + l.keys_sorted);
    s.vals = (uint32_t*)(base + l.vals);
    s.vals_sorted = (uint32_t*)(base + l.vals_sorted);
    s.left = (int*)(base + l.left);
    s.right = (int*)(base + l.right);
    s.parent = (int*)(base + l.parent);
    s.node_min = (float4*)(base + l.node_min);
    s.node_max = (float4*)(base + l.node_max);
    s.node_flag = (int*)(base + l.node_flag);
    s.leaf_count = (uint32_t*)(base + l.leaf_count);
    s.leaf_offset = (uint32_t*)(base + l.leaf_offset);
    s.total = (uint32_t*)(base + l.total);
    return s;
}

__device__ __forceinline__ float4 box_min(const float* a, uint32_t i) {
    return make_float4(a[6 * i], a[6 * i + 1], a[6 * i + 2], 0.0f);
}
__device__ __forceinline__ float4 box_max(const float* a, uint32_t i) {
    return make_float4(a[6 * i + 3], a[6 * i + 4], a[6 * i + 5], 0.0f);
}
// Owner rank of a box: its extent sum (ties broken by index).
__device__ __forceinline__ float box_rank(const float* a, uint32_t i) {
    return (a[6 * i + 3] - a[6 * i]) + (a[6 * i + 4] - a[6 * i + 1]) + (a[6 * i + 5] - a[6 * i + 2]);
}

__global__ void ks_keys(Scratch s, const float* aabbs, const uint32_t* groups, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 mn = box_min(aabbs, i), mx = box_max(aabbs, i);
    float cx = 0.5f * (mn.x + mx.x), cy = 0.5f * (mn.y + mx.y), cz = 0.5f * (mn.z + mx.z);
    uint64_t morton = expand16s(quantize_s(cx)) | (expand16s(quantize_s(cy)) << 1) | (expand16s(quantize_s(cz)) << 2);
    uint64_t g = groups ? (groups[i] & 0xffffu) : 0u;
    s.keys[i] = (g << 48) | morton;
    s.vals[i] = i;
}

__device__ __forceinline__ int delta_s(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll((long long)(a ^ b));
}

__global__ void ks_build(Scratch s, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const unsigned long long* k = s.keys_sorted;
    int d = (delta_s(k, n, i, i + 1) - delta_s(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta_s(k, n, i, i - d);
    int lmax = 2;
    while (delta_s(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta_s(k, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta_s(k, n, i, j);
    int sp = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta_s(k, n, i, i + (sp + t) * d) > dnode) sp += t;
    } while (t > 1);
    int gamma = i + sp * d + (d < 0 ? d : 0);
    int lo = i < j ? i : j, hi = i < j ? j : i;
    int left = (lo == gamma) ? (n - 1 + gamma) : gamma;
    int right = (hi == gamma + 1) ? (n - 1 + gamma + 1) : (gamma + 1);
    s.left[i] = left;
    s.right[i] = right;
    s.parent[left] = i;
    s.parent[right] = i;
    if (i == 0) s.parent[0] = -1;
}

__global__ void ks_refit(Scratch s, const float* aabbs, int n, uint32_t* err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t bi = s.vals_sorted[k];
    int node = n - 1 + k;
    float4 mx = box_max(aabbs, bi);
    s.node_min[node] = box_min(aabbs, bi);
    s.node_max[node] = make_float4(mx.x, mx.y, mx.z, box_rank(aabbs, bi));
    if (n == 1) return;
    __threadfence();
    int p = s.parent[node];
    for (int guard = 0; p >= 0; ++guard) {
        if (guard > 256) {
            atomicOr(err, 1u);
            return;
        }
        if (atomicAdd(&s.node_flag[p], 1) == 0) return;
        int l = s.left[p], r = s.right[p];
        float4 a0 = __ldcg(&s.node_min[l]), a1 = __ldcg(&s.node_max[l]);
        float4 b0 = __ldcg(&s.node_min[r]), b1 = __ldcg(&s.node_max[r]);
        s.node_min[p] = make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), 0.0f);
        s.node_max[p] = make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), fmaxf(a1.w, b1.w));
        __threadfence();
        p = s.parent[p];
    }
}

template <bool WRITE>
__global__ void ks_traverse(Scratch s, const float* aabbs, const uint32_t* groups, int n, uint32_t* pairs,
                            uint32_t max_pairs, uint32_t* err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t a = s.vals_sorted[k];
    float4 amin = box_min(aabbs, a), amax = box_max(aabbs, a);
    float ra = box_rank(aabbs, a);
    uint32_t ga = groups ? groups[a] : 0u;
    uint32_t count = 0, base = WRITE ? s.leaf_offset[k] : 0u;
    if (n >= 2) {
        int stack[64];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            int node = stack[--sp];
            float4 nmin = s.node_min[node], nmax = s.node_max[node];
            if (nmax.w < ra) continue;
            if (!(amin.x <= nmax.x && nmin.x <= amax.x && amin.y <= nmax.y && nmin.y <= amax.y && amin.z <= nmax.z &&
                  nmin.z <= amax.z))
                continue;
            if (node >= n - 1) {
                uint32_t b = s.vals_sorted[node - (n - 1)];
                if (b == a) continue;
                float rb = box_rank(aabbs, b);
                bool own = ra < rb || (ra == rb && a < b);
                if (!own) continue;
                if (groups && groups[b] != ga) continue;
                if (WRITE) {
                    uint32_t slot = base + count;
                    if (slot < max_pairs) {
                        pairs[2 * slot] = a < b ? a : b;
                        pairs[2 * slot + 1] = a < b ? b : a;
                    }
                }
                ++count;
            } else if (sp < 62) {
                stack[sp++] = s.left[node];
                stack[sp++] = s.right[node];
            } else {
                atomicOr(err, 2u);
            }
        }
    }
    if (!WRITE) s.leaf_count[k] = count;
}

// Writes the pair count, or UINT32_MAX when a traversal or refit bound was hit.
__global__ void ks_total(Scratch s, int n, uint32_t* count_out, const uint32_t* err) {
    uint32_t total = n > 0 ? s.leaf_offset[n - 1] + s.leaf_count[n - 1] : 0u;
    *count_out = *err ? 0xffffffffu : total;
}

}  // namespace

namespace npgpu_dev {
void set_global_error(const std::string& msg);
}

extern "C" npgpu_status npgpu_find_pairs_static(const float* aabbs6, const uint32_t* groups, uint32_t n,
                                                uint32_t* pairs2, uint32_t max_pairs, uint32_t* count,
                                                void* stream) {
    if ((n && !aabbs6) || !count || (max_pairs && !pairs2)) {
        npgpu_dev::set_global_error("npgpu_find_pairs_static: null argument");
        return NPGPU_ERR_INVALID_ARGUMENT;
    }
    if (n > kMaxAabbs) {
        npgpu_dev::set_global_error("npgpu_find_pairs_static: at most " + std::to_string(kMaxAabbs) + " boxes per call");
        return NPGPU_ERR_CAPACITY;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        npgpu_dev::set_global_error("npgpu_find_pairs_static: no current CUDA device");
        return NPGPU_ERR_CUDA;
    }
    Layout layout = make_layout(kMaxAabbs);
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        // 0 when no context is current yet (before the runtime's lazy
        // initialisation): the set-up then runs and records the context the
        // symbol lookup made current.
        unsigned long long ctx = current_context_id();
        if (!g_ready[dev] || ctx != g_ctx_id[dev]) {
            // Set-up, once per device: the device address of the scratch array.
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_pair_scratch);
            if (e != cudaSuccess || p == nullptr) {
                npgpu_dev::set_global_error(std::string("npgpu_find_pairs_static: cudaGetSymbolAddress failed: ") +
                                 cudaGetErrorString(e));
                return NPGPU_ERR_CUDA;
            }
            if (layout.end > kScratchBytes) {
                npgpu_dev::set_global_error("npgpu_find_pairs_static: scratch array too small for the sort and scan");
                return NPGPU_ERR_CAPACITY;
            }
            g_scratch_ptr[dev] = (unsigned char*)p;
            g_ctx_id[dev] = current_context_id();
            g_ready[dev] = true;
        }
        base = g_scratch_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    Scratch s = scratch_at(base, layout);
    uint32_t* err = s.total + 1;
    cudaError_t e = cudaMemsetAsync(s.total, 0, 16, st);
    if (e == cudaSuccess && n == 0) e = cudaMemsetAsync(count, 0, sizeof(uint32_t), st);
    const int T = 256;
    unsigned nb = (n + T - 1) / T;
    if (e == cudaSuccess && n > 0) {
        ks_keys<<<nb, T, 0, st>>>(s, aabbs6, groups, n);
        size_t sb = layout.sort_bytes;
        // Without groups the keys' top 16 bits are zero: sort the 48 Morton bits only.
        e = npgpu_dev::radix_sort_pairs(base + layout.sort_temp, sb, s.keys, s.keys_sorted, s.vals, s.vals_sorted,
                                        n, groups ? 64 : 48, st);
        if (e == cudaSuccess && n >= 2) {
            e = cudaMemsetAsync(s.node_flag, 0, sizeof(int) * (size_t)(n - 1), st);
            ks_build<<<(n - 1 + T - 1) / T, T, 0, st>>>(s, (int)n);
        }
        if (e == cudaSuccess) {
            ks_refit<<<nb, T, 0, st>>>(s, aabbs6, (int)n, err);
            ks_traverse<false><<<nb, T, 0, st>>>(s, aabbs6, groups, (int)n, pairs2, max_pairs, err);
            size_t cb = layout.scan_bytes;
            e = npgpu_dev::exclusive_scan(base + layout.scan_temp, cb, s.leaf_count, s.leaf_offset, n, st);
        }
        if (e == cudaSuccess) {
            ks_traverse<true><<<nb, T, 0, st>>>(s, aabbs6, groups, (int)n, pairs2, max_pairs, err);
            ks_total<<<1, 1, 0, st>>>(s, (int)n, count, err);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        npgpu_dev::set_global_error(std::string("npgpu_find_pairs_static: ") + cudaGetErrorString(e));
        return NPGPU_ERR_CUDA;
    }
    return NPGPU_OK;
}
