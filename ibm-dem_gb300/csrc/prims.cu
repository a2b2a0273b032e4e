// prims.cu — device-wide exclusive scan and stable LSD radix sort (8-bit digits).
#include "prims.cuh"

namespace ibmdem {

namespace {

__device__ inline long long read_n(long long n_max, const int* n_dev) {
  if (!n_dev) return n_max;
  long long n = *n_dev;
  return n < n_max ? n : n_max;
}

// exclusive scan of one value per thread over a 256-thread block; returns the
// block total in *total (all threads).
__device__ inline int block_excl_scan(int v, int* sh_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? sh_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < 32) sh_warp[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  int warp_excl = warp ? sh_warp[warp - 1] : 0;
  *total = sh_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_excl + x - v;
}

__global__ void k_scan_reduce(const int* __restrict__ in, long long n_max, const int* n_dev, int* partial) {
  __shared__ int sh[32];
  long long n = read_n(n_max, n_dev);
  long long base = (long long)blockIdx.x * kScanTile;
  int s = 0;
  for (int it = 0; it < kScanItems; ++it) {
    long long e = base + it * kScanThreads + threadIdx.x;
    if (e < n) s += in[e];
  }
  int tot;
  block_excl_scan(s, sh, &tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// single block of 256 threads scans partial[0..nb) in place (exclusive)
__global__ void k_scan_spine(int* partial, long long nb, int* total) {
  __shared__ int sh[32];
  int carry = 0;
  for (long long base = 0; base < nb; base += kScanThreads * 4) {
    int v[4];
    int s = 0;
    for (int q = 0; q < 4; ++q) {
      long long e = base + threadIdx.x * 4 + q;
      v[q] = e < nb ? partial[e] : 0;
      s += v[q];
    }
    int tot;
    int ex = block_excl_scan(s, sh, &tot);
    int run = carry + ex;
    for (int q = 0; q < 4; ++q) {
      long long e = base + threadIdx.x * 4 + q;
      if (e < nb) partial[e] = run;
      run += v[q];
    }
    carry += tot;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

// tile slot of element idx: one pad word per 32, so that a thread's
// kScanItems consecutive elements (and a warp's 32 consecutive loads) fall in
// distinct banks
__device__ inline int padded(int idx) { return idx + (idx >> 5); }

__global__ void k_scan_down(const int* in, int* out, long long n_max, const int* n_dev, const int* partial) {
  __shared__ int tile[kScanTile + kScanTile / 32];
  __shared__ int sh[32];
  long long n = read_n(n_max, n_dev);
  long long base = (long long)blockIdx.x * kScanTile;
  if (base >= n) return;
  for (int it = 0; it < kScanItems; ++it) {
    int idx = it * kScanThreads + threadIdx.x;
    long long e = base + idx;
    tile[padded(idx)] = e < n ? in[e] : 0;
  }
  __syncthreads();
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    v[q] = tile[padded(threadIdx.x * kScanItems + q)];
    s += v[q];
  }
  int tot;
  int run = block_excl_scan(s, sh, &tot) + partial[blockIdx.x];
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    tile[padded(threadIdx.x * kScanItems + q)] = run;
    run += v[q];
  }
  __syncthreads();
  for (int it = 0; it < kScanItems; ++it) {
    int idx = it * kScanThreads + threadIdx.x;
    long long e = base + idx;
    if (e < n) out[e] = tile[padded(idx)];
  }
}

// ---- radix sort ----------------------------------------------------------
__global__ void k_rs_hist(const uint32_t* __restrict__ keys, long long n_max, const int* n_dev, int shift,
                          int* hist, long long nb) {
  __shared__ int sh[kRadix];
  long long n = read_n(n_max, n_dev);
  sh[threadIdx.x] = 0;
  __syncthreads();
  long long base = (long long)blockIdx.x * kSortTile;
  for (int it = 0; it < kSortItems; ++it) {
    long long e = base + it * kSortThreads + threadIdx.x;
    if (e < n) atomicAdd(&sh[(keys[e] >> shift) & (kRadix - 1)], 1);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * nb + blockIdx.x] = sh[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) k_rs_scatter(const uint32_t* __restrict__ kin,
                                                             const uint32_t* __restrict__ vin, uint32_t* kout,
                                                             uint32_t* vout, long long n_max, const int* n_dev,
                                                             int shift, const int* __restrict__ offs, long long nb) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ int wcnt[kWarps][kRadix];
  long long n = read_n(n_max, n_dev);
  long long base = (long long)blockIdx.x * kSortTile;
  if (base >= n) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = threadIdx.x; q < kWarps * kRadix; q += kSortThreads) (&wcnt[0][0])[q] = 0;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  uint32_t key[kSortItems], val[kSortItems];
  int rank[kSortItems];
  long long wbase = base + (long long)warp * 32 * kSortItems;
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    long long e = wbase + r * 32 + lane;
    bool ok = e < n;
    key[r] = ok ? kin[e] : 0u;
    val[r] = ok ? vin[e] : 0u;
    int d = ok ? (int)((key[r] >> shift) & (kRadix - 1)) : kRadix;  // kRadix marks an empty slot
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int leader = __ffs(peers) - 1;
    int before = __popc(peers & lt);
    int cnt_base = (ok ? wcnt[warp][d] : 0);
    __syncwarp();
    if (ok && lane == leader) wcnt[warp][d] = cnt_base + __popc(peers);
    __syncwarp();
    rank[r] = ok ? cnt_base + before : -1;
  }
  __syncthreads();
  // exclusive prefix over warps, per digit
  {
    int d = threadIdx.x;
    int run = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      int t = wcnt[w][d];
      wcnt[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    if (rank[r] < 0) continue;
    int d = (int)((key[r] >> shift) & (kRadix - 1));
    long long pos = (long long)offs[(long long)d * nb + blockIdx.x] + wcnt[warp][d] + rank[r];
    kout[pos] = key[r];
    vout[pos] = val[r];
  }
}

}  // namespace

long long scan_scratch_ints(long long n_max) { return (n_max + kScanTile - 1) / kScanTile + 1; }
long long sort_hist_ints(long long n_max) { return (long long)kRadix * ((n_max + kSortTile - 1) / kSortTile) + 1; }

void scan_exclusive(const int* in, int* out, long long n_max, const int* n_dev, int* total, int* scratch,
                    cudaStream_t s, long long* launches) {
  if (n_max <= 0) {
    if (total) cudaMemsetAsync(total, 0, sizeof(int), s);
    return;
  }
  long long nb = (n_max + kScanTile - 1) / kScanTile;
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n_max, n_dev, scratch);
  k_scan_spine<<<1, kScanThreads, 0, s>>>(scratch, nb, total);
  k_scan_down<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n_max, n_dev, scratch);
  if (launches) *launches += 3;
}

void radix_sort_pairs(uint32_t*& keys, uint32_t*& vals, uint32_t*& keys_alt, uint32_t*& vals_alt, long long n_max,
                      const int* n_dev, int bits, int* hist, int* scan_scratch, cudaStream_t s, long long* launches) {
  if (n_max <= 0) return;
  long long nb = (n_max + kSortTile - 1) / kSortTile;
  for (int shift = 0; shift < bits; shift += kRadixBits) {
    k_rs_hist<<<(unsigned)nb, kSortThreads, 0, s>>>(keys, n_max, n_dev, shift, hist, nb);
    scan_exclusive(hist, hist, (long long)kRadix * nb, nullptr, nullptr, scan_scratch, s, launches);
    k_rs_scatter<<<(unsigned)nb, kSortThreads, 0, s>>>(keys, vals, keys_alt, vals_alt, n_max, n_dev, shift, hist,
                                                       nb);
    if (launches) *launches += 2;
    uint32_t* t = keys;
    keys = keys_alt;
    keys_alt = t;
    t = vals;
    vals = vals_alt;
    vals_alt = t;
  }
}

}  // namespace ibmdem
