// scan_sort.cuh -- device exclusive scan and stable LSD radix sort used by the
// cell-list build.  Hand-written for sm_103a: 256-thread blocks, 2048-item tiles,
// warp match-based stable ranking, digit-major tile histograms.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace dsph {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kTile = kScanThreads * kScanItems;  // 2048

// Scratch sizes (bytes) for the launchers below (constexpr, so fixed-size
// scratch arrays can be checked against them at compile time).
constexpr int64_t tiles_of(int64_t n) { return (n + kTile - 1) / kTile; }
constexpr size_t scan_scratch_bytes(int64_t n) { return sizeof(int32_t) * (size_t)(tiles_of(n) + 1); }
constexpr size_t radix_scratch_bytes(int64_t n) {
    return sizeof(int32_t) * (size_t)(256 * tiles_of(n) + tiles_of(256 * tiles_of(n)) + 2);
}

// out[i] = sum_{k<i} in[i]; out may alias in.  n <= 2^31 - 1.
// Returns the number of kernel launches issued.
int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, void* scratch,
                       cudaStream_t st);

// Stable sort of (key, value) pairs by the low `bits` bits of key (LSD, 8-bit
// digits).  If vals_in is null the values are the input positions 0..n-1.
// The sorted data ends up in keys_out / vals_out; keys_tmp / vals_tmp are
// ping-pong buffers of n entries.  Returns the number of launches.
int radix_sort_pairs(const uint32_t* keys_in, const int32_t* vals_in, uint32_t* keys_out,
                     int32_t* vals_out, uint32_t* keys_tmp, int32_t* vals_tmp, int64_t n, int bits,
                     void* scratch, cudaStream_t st);

}  // namespace dsph
