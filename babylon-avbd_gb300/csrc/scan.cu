// Device-wide exclusive prefix sum of int32 (three phases: per-tile scan with tile sums,
// recursive scan of the tile sums, uniform add). Tiles of 4096 elements: 1024 threads x 4.
// Used for the grid cell table, the per-body pair counts and the adjacency degrees.
#include "engine.cuh"

namespace avbd {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

static int tiles(int n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

size_t scan_temp_bytes(int n) {
  size_t bytes = 0;
  int m = n;
  while (m > SCAN_TILE) {
    m = tiles(m);
    bytes += size_t(m + 1) * sizeof(int);
  }
  return bytes + 256;
}

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total via *total.
__device__ __forceinline__ int block_excl_scan(int v, int* total) {
  __shared__ int warpSums[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = warp_incl_scan(v);
  if (lane == 31) warpSums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int s = lane < (SCAN_THREADS / 32) ? warpSums[lane] : 0;
    int si = warp_incl_scan(s);
    if (lane < (SCAN_THREADS / 32)) warpSums[lane] = si - s;
    if (lane == 31) *total = si;
  }
  __syncthreads();
  return incl - v + warpSums[warp];
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(int* data, int n, int* tileSums) {
  __shared__ int total;
  const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  int sum = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    v[i] = (base + i < n) ? data[base + i] : 0;
    sum += v[i];
  }
  int off = block_excl_scan(sum, &total);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    if (base + i < n) data[base + i] = off;
    off += v[i];
  }
  if (threadIdx.x == 0 && tileSums) tileSums[blockIdx.x] = total;
}

__global__ void k_scan_add(int* data, int n, const int* tileOffsets) {
  const long long i = (long long)blockIdx.x * SCAN_TILE + threadIdx.x;
  const int add = tileOffsets[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    long long j = i + (long long)k * SCAN_THREADS;
    if (j < n) data[j] += add;
  }
}

// total = exclusive-scanned last element + original last element; recorded before scanning.
__global__ void k_scan_save_last(const int* data, int n, int* last) { *last = n > 0 ? data[n - 1] : 0; }
__global__ void k_scan_total(const int* data, int n, const int* last, int* total) {
  *total = n > 0 ? data[n - 1] + *last : 0;
}

static void scan_rec(int* data, int n, int* temp, cudaStream_t s) {
  const int t = tiles(n);
  if (t <= 1) {
    k_scan_tiles<<<1, SCAN_THREADS, 0, s>>>(data, n, nullptr); note_launches(1);
    return;
  }
  int* sums = temp;
  k_scan_tiles<<<t, SCAN_THREADS, 0, s>>>(data, n, sums); note_launches(1);
  scan_rec(sums, t, temp + t + 1, s);
  k_scan_add<<<t, SCAN_THREADS, 0, s>>>(data, n, sums); note_launches(1);
}

void scan_exclusive(int* data, int n, int* total, void* temp, cudaStream_t s) {
  if (n <= 0) return;
  int* t = static_cast<int*>(temp);
  // the last slot of temp holds the original last element (temp is sized with 256 spare bytes)
  size_t words = (scan_temp_bytes(n) - 256) / sizeof(int);
  int* last = t + words;
  if (total) { k_scan_save_last<<<1, 1, 0, s>>>(data, n, last); note_launches(1); }
  scan_rec(data, n, t, s);
  if (total) { k_scan_total<<<1, 1, 0, s>>>(data, n, last, total); note_launches(1); }
}

int grid_blocks(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 0x7fffffffLL) b = 0x7fffffffLL;
  return int(b);
}

}  // namespace avbd

#include <atomic>

namespace avbd {
static std::atomic<int> g_sms[64];
int device_sms() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  int v = g_sms[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 1;
  g_sms[dev].store(v, std::memory_order_relaxed);
  return v;
}
static std::atomic<long long> g_launches{0};
void note_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_total() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace avbd
