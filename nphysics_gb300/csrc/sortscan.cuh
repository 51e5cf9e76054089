// sortscan.cuh -- the step's own radix sort and prefix sum.
//
// The broad phase sorts 64-bit keys (world | static bit | Morton code) with
// 32-bit values, and several phases turn per-item counts into offsets with an
// exclusive prefix sum. Both are written here for sm_103a:
//
//  radix_sort_pairs   least-significant-digit radix sort, 8 bits a pass, over
//                     bits [0, end_bit). Each pass is three launches: per-tile
//                     digit counts, one exclusive prefix sum of the counts laid
//                     out digit-major (digit d, tile t -> d * tiles + t), so
//                     that every (digit, tile) gets its output base, and a
//                     scatter that ranks each tile's items stably
//                     (__match_any_sync per warp, then per-warp digit counts
//                     in shared memory). No pass waits on another block's
//                     progress, so nothing spins. The sort is stable, so it
//                     orders equal keys by input position, as any stable sort.
//  exclusive_scan     three launches: per-block sums of 8192 items, a scan of
//                     the block sums in one block, and the per-block scans
//                     offset by them (one launch when n <= 8192).
//
// Scratch memory is caller-provided; *_temp_bytes(n) gives its size.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace npgpu_dev {

size_t radix_sort_temp_bytes(uint32_t n);
// keys_in/vals_in are left unchanged; the sorted pairs land in keys_out/vals_out.
cudaError_t radix_sort_pairs(void* temp, size_t temp_bytes, const unsigned long long* keys_in,
                             unsigned long long* keys_out, const uint32_t* vals_in, uint32_t* vals_out, uint32_t n,
                             int end_bit, cudaStream_t st);

size_t exclusive_scan_temp_bytes(uint32_t n);
// out[i] = in[0] + ... + in[i - 1]; in and out may not overlap.
cudaError_t exclusive_scan(void* temp, size_t temp_bytes, const uint32_t* in, uint32_t* out, uint32_t n,
                           cudaStream_t st);

}  // namespace npgpu_dev
