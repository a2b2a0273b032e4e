// prims.cuh — device-wide exclusive scan and stable LSD radix sort.
//
// Both take a host-side upper bound n_max (sizes the launch) and an optional
// device-resident element count n_dev (read by the kernels), so they can be
// issued without a host round trip and captured in a CUDA graph.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ibmdem {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096
constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;

// ints of scratch needed by scan_exclusive for n_max elements
long long scan_scratch_ints(long long n_max);
// ints of histogram scratch needed by radix_sort_pairs for n_max elements
long long sort_hist_ints(long long n_max);

// out[i] = sum(in[0..i)) for i < n; *total = sum(in[0..n)) if total != nullptr.
// out may alias in.  n = *n_dev when n_dev != nullptr, else n_max.
void scan_exclusive(const int* in, int* out, long long n_max, const int* n_dev, int* total, int* scratch,
                    cudaStream_t s, long long* launches);

// Stable sort of (keys, vals) by the low `bits` bits of keys.  The buffers are
// ping-ponged; on return keys/vals point at the sorted data and keys_alt/vals_alt
// at the scratch copies.
void radix_sort_pairs(uint32_t*& keys, uint32_t*& vals, uint32_t*& keys_alt, uint32_t*& vals_alt, long long n_max,
                      const int* n_dev, int bits, int* hist, int* scan_scratch, cudaStream_t s, long long* launches);

}  // namespace ibmdem
