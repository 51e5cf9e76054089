// sortscan.cu -- radix sort of (64-bit key, 32-bit value) pairs and exclusive
// prefix sums of 32-bit counts (the algorithms are described in sortscan.cuh).
#include "sortscan.cuh"

namespace npgpu_dev {
namespace {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortThreads = 256;                 // one thread per digit in the count/offset steps
constexpr int kSortWarps = kSortThreads / 32;
constexpr uint32_t kFull = 0xffffffffu;

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;   // 8192
constexpr int kScanPad = kScanTile + kScanTile / 32;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Items a sort tile holds: 256 threads x ITEMS. Small inputs use small tiles
// so that a pass still spreads over many SMs.
inline int sort_items(uint32_t n) { return n <= (1u << 17) ? 4 : 16; }
inline uint32_t sort_tiles(uint32_t n, int items) { return (n + kSortThreads * items - 1) / (kSortThreads * items); }

// ---------------------------------------------------------------- prefix sum
// Exclusive scan of the 1024 per-thread values of a block; returns this
// thread's exclusive prefix and writes the block total to *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
        uint32_t t = s;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(kFull, t, d);
            if (lane >= d) t += y;
        }
        warp_sums[lane] = t - s;   // exclusive prefix of each warp
        if (lane == 31) warp_sums[32] = t;
    }
    __syncthreads();
    uint32_t r = warp_sums[warp] + x - v;
    *total = warp_sums[32];
    __syncthreads();
    return r;
}

// Loads the block's tile coalesced into shared memory (padded against bank
// conflicts) and returns this thread's kScanItems consecutive items.
__device__ __forceinline__ void load_tile(const uint32_t* in, uint32_t n, uint32_t base, uint32_t* s, uint32_t* v) {
    for (int r = 0; r < kScanItems; ++r) {
        uint32_t i = (uint32_t)r * kScanThreads + threadIdx.x;
        s[i + (i >> 5)] = base + i < n ? in[base + i] : 0u;
    }
    __syncthreads();
    for (int j = 0; j < kScanItems; ++j) {
        uint32_t i = threadIdx.x * kScanItems + j;
        v[j] = s[i + (i >> 5)];
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* in, uint32_t n, uint32_t* bsum) {
    __shared__ uint32_t s[kScanPad];
    __shared__ uint32_t ws[33];
    uint32_t v[kScanItems];
    load_tile(in, n, blockIdx.x * (uint32_t)kScanTile, s, v);
    uint32_t t = 0;
    for (int j = 0; j < kScanItems; ++j) t += v[j];
    uint32_t total;
    block_exclusive(t, ws, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Scans tile blockIdx.x of `in` into `out`, adding offset[blockIdx.x] (or 0).
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* in, uint32_t n, uint32_t* out,
                                                             const uint32_t* offset) {
    __shared__ uint32_t s[kScanPad];
    __shared__ uint32_t ws[33];
    const uint32_t base = blockIdx.x * (uint32_t)kScanTile;
    uint32_t v[kScanItems];
    load_tile(in, n, base, s, v);
    uint32_t t = 0;
    for (int j = 0; j < kScanItems; ++j) t += v[j];
    uint32_t total;
    uint32_t run = block_exclusive(t, ws, &total) + (offset ? offset[blockIdx.x] : 0u);
    for (int j = 0; j < kScanItems; ++j) {
        uint32_t i = threadIdx.x * kScanItems + j;
        s[i + (i >> 5)] = run;
        run += v[j];
    }
    __syncthreads();
    for (int r = 0; r < kScanItems; ++r) {
        uint32_t i = (uint32_t)r * kScanThreads + threadIdx.x;
        if (base + i < n) out[base + i] = s[i + (i >> 5)];
    }
}

// ---------------------------------------------------------------- radix sort
// counts[d * tiles + tile] = items of the tile whose digit is d.
template <int ITEMS>
__global__ void __launch_bounds__(kSortThreads) k_radix_count(const unsigned long long* keys, uint32_t n, int shift,
                                                              uint32_t dmask, uint32_t* counts, uint32_t tiles) {
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t base = blockIdx.x * (uint32_t)(kSortThreads * ITEMS);
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
        uint32_t i = base + (uint32_t)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(uint32_t)(keys[i] >> shift) & dmask], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Writes each item of the tile to offsets[d * tiles + tile] + its stable rank
// among the tile's items of digit d. Warp w takes the tile's w-th run of
// 32 ITEMS items, 32 a round in order, so (warp, round, lane) is input order.
template <int ITEMS>
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const unsigned long long* keys_in,
                                                                const uint32_t* vals_in, unsigned long long* keys_out,
                                                                uint32_t* vals_out, uint32_t n, int shift,
                                                                uint32_t dmask, const uint32_t* offsets,
                                                                uint32_t tiles) {
    __shared__ uint32_t wc[kSortWarps][kRadix];   // per warp: items of each digit (then its exclusive prefix)
    __shared__ uint32_t toff[kRadix];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kSortWarps * kRadix; i += kSortThreads) (&wc[0][0])[i] = 0u;
    toff[threadIdx.x] = offsets[(size_t)threadIdx.x * tiles + blockIdx.x];
    __syncthreads();
    const uint32_t base = blockIdx.x * (uint32_t)(kSortThreads * ITEMS) + (uint32_t)warp * (32u * ITEMS);
    const uint32_t lt = (1u << lane) - 1u;
    unsigned long long k[ITEMS];
    uint32_t v[ITEMS], dig[ITEMS], rank[ITEMS];
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
        const uint32_t i = base + (uint32_t)r * 32u + (uint32_t)lane;
        const bool ok = i < n;
        k[r] = ok ? keys_in[i] : 0ull;
        v[r] = ok ? vals_in[i] : 0u;
        dig[r] = ok ? (uint32_t)(k[r] >> shift) & dmask : (uint32_t)kRadix + (uint32_t)lane;
        const uint32_t peers = __match_any_sync(kFull, dig[r]);
        const int leader = __ffs(peers) - 1;
        uint32_t before = 0u;
        if (ok && lane == leader) {
            before = wc[warp][dig[r]];
            wc[warp][dig[r]] = before + (uint32_t)__popc(peers);
        }
        before = __shfl_sync(kFull, before, leader);
        rank[r] = before + (uint32_t)__popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();
    {
        // Exclusive prefix over the warps, per digit (thread = digit).
        uint32_t s = 0u;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            uint32_t c = wc[w][threadIdx.x];
            wc[w][threadIdx.x] = s;
            s += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
        const uint32_t i = base + (uint32_t)r * 32u + (uint32_t)lane;
        if (i < n) {
            const uint32_t d = dig[r];
            const uint32_t at = toff[d] + wc[warp][d] + rank[r];
            keys_out[at] = k[r];
            vals_out[at] = v[r];
        }
    }
}

struct SortTemp {
    unsigned long long* keys;
    uint32_t* vals;
    uint32_t* counts;
    uint32_t* offsets;
    void* scan;
    size_t scan_bytes;
};

SortTemp sort_temp(void* temp, uint32_t n) {
    const uint32_t tiles = sort_tiles(n, sort_items(n));
    const uint32_t nc = tiles * (uint32_t)kRadix;
    unsigned char* p = (unsigned char*)temp;
    SortTemp t;
    size_t o = 0;
    t.keys = (unsigned long long*)(p + o);
    o = align256(o + 8ull * n);
    t.vals = (uint32_t*)(p + o);
    o = align256(o + 4ull * n);
    t.counts = (uint32_t*)(p + o);
    o = align256(o + 4ull * nc);
    t.offsets = (uint32_t*)(p + o);
    o = align256(o + 4ull * nc);
    t.scan = p + o;
    t.scan_bytes = exclusive_scan_temp_bytes(nc);
    return t;
}

template <int ITEMS>
cudaError_t sort_passes(const SortTemp& t, const unsigned long long* keys_in, unsigned long long* keys_out,
                        const uint32_t* vals_in, uint32_t* vals_out, uint32_t n, int end_bit, cudaStream_t st) {
    const uint32_t tiles = sort_tiles(n, ITEMS);
    const int passes = (end_bit + kRadixBits - 1) / kRadixBits;
    // Ping-pong between the output and the scratch copy so that the last pass
    // lands in the output.
    const unsigned long long* ks = keys_in;
    const uint32_t* vs = vals_in;
    for (int p = 0; p < passes; ++p) {
        const bool to_out = ((passes - 1 - p) & 1) == 0;
        unsigned long long* kd = to_out ? keys_out : t.keys;
        uint32_t* vd = to_out ? vals_out : t.vals;
        const int shift = p * kRadixBits;
        // The last pass looks only at the bits below end_bit.
        const int bits = end_bit - shift < kRadixBits ? end_bit - shift : kRadixBits;
        const uint32_t dmask = (1u << bits) - 1u;
        k_radix_count<ITEMS><<<tiles, kSortThreads, 0, st>>>(ks, n, shift, dmask, t.counts, tiles);
        cudaError_t e = exclusive_scan(t.scan, t.scan_bytes, t.counts, t.offsets, tiles * (uint32_t)kRadix, st);
        if (e != cudaSuccess) return e;
        k_radix_scatter<ITEMS><<<tiles, kSortThreads, 0, st>>>(ks, vs, kd, vd, n, shift, dmask, t.offsets, tiles);
        ks = kd;
        vs = vd;
    }
    return cudaGetLastError();
}

}  // namespace

size_t exclusive_scan_temp_bytes(uint32_t n) {
    const uint32_t blocks = (n + kScanTile - 1) / kScanTile;
    return blocks <= 1 ? 256 : 2 * align256(4ull * blocks);
}

cudaError_t exclusive_scan(void* temp, size_t temp_bytes, const uint32_t* in, uint32_t* out, uint32_t n,
                           cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + kScanTile - 1) / kScanTile;
    if (blocks == 1) {
        k_scan_tiles<<<1, kScanThreads, 0, st>>>(in, n, out, nullptr);
        return cudaGetLastError();
    }
    if (blocks > (uint32_t)kScanTile || temp_bytes < exclusive_scan_temp_bytes(n)) return cudaErrorInvalidValue;
    uint32_t* bsum = (uint32_t*)temp;
    uint32_t* boff = (uint32_t*)((unsigned char*)temp + align256(4ull * blocks));
    k_scan_reduce<<<blocks, kScanThreads, 0, st>>>(in, n, bsum);
    k_scan_tiles<<<1, kScanThreads, 0, st>>>(bsum, blocks, boff, nullptr);
    k_scan_tiles<<<blocks, kScanThreads, 0, st>>>(in, n, out, boff);
    return cudaGetLastError();
}

size_t radix_sort_temp_bytes(uint32_t n) {
    // Sized with the small tiles' count (never below the large tiles'), so
    // that the size grows with n and a buffer sized for a capacity serves
    // every n up to it.
    const uint32_t tiles = sort_tiles(n, 4);
    const uint32_t nc = tiles * (uint32_t)kRadix;
    return align256(8ull * n) + align256(4ull * n) + 2 * align256(4ull * nc) + exclusive_scan_temp_bytes(nc);
}

cudaError_t radix_sort_pairs(void* temp, size_t temp_bytes, const unsigned long long* keys_in,
                             unsigned long long* keys_out, const uint32_t* vals_in, uint32_t* vals_out, uint32_t n,
                             int end_bit, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    if (end_bit < 1 || end_bit > 64 || temp_bytes < radix_sort_temp_bytes(n)) return cudaErrorInvalidValue;
    const SortTemp t = sort_temp(temp, n);
    return sort_items(n) == 4 ? sort_passes<4>(t, keys_in, keys_out, vals_in, vals_out, n, end_bit, st)
                              : sort_passes<16>(t, keys_in, keys_out, vals_in, vals_out, n, end_bit, st);
}

}  // namespace npgpu_dev
