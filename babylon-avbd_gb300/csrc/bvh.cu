// Bounding-volume hierarchy broadphase: Morton order, stable radix sort, hierarchical PLOC
// treelets, escape links, per-step refit (src/gpu/gpuHploc.js:62-380, src/gpu/hplocpp.wgsl,
// src/gpu/hplocSort.wgsl).
//
// A world that selects the BVH gets its own tree over its bodies' bounding-sphere boxes
// (centre +- radius), so the tree's candidates contain every pair the reference's predicate
// accepts (cpuPhysics3D.js:319-343) and the exact predicate then gives the same pair set as the
// grid. Build: leaf boxes and scene bounds, 30-bit Morton codes of the box centres, a stable LSD
// radix sort of (code, leaf) by 8-bit digits, then levels of treelets: each treelet takes 16
// consecutive clusters and merges mutual nearest neighbours by surface area until one cluster
// remains, which joins the next level. Parents and escape links ("ropes") give a stackless
// traversal. Between rebuilds the leaves and every treelet node are refitted in creation order.
// Nodes also keep the least body index below them, so a body looking for lower-index partners
// skips subtrees that cannot hold one.
#include <vector>

#include "engine.cuh"

namespace avbd {

namespace {

constexpr int RADIX_THREADS = 256;
constexpr int RADIX_ITEMS = 1024;  // keys per block (4 rounds of 256)

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
  uint32_t x = v & 1023u;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  return (x | (x << 2)) & 0x09249249u;
}

__device__ __forceinline__ float area(float3 lo, float3 hi) {
  const float dx = fminf(fmaxf(hi.x - lo.x, 0.f), 1e18f), dy = fminf(fmaxf(hi.y - lo.y, 0.f), 1e18f),
              dz = fminf(fmaxf(hi.z - lo.z, 0.f), 1e18f);
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ void store_node(float4* node, uint32_t id, float3 lo, uint32_t left, float3 hi, uint32_t right) {
  node[2 * size_t(id)] = make_float4(lo.x, lo.y, lo.z, __uint_as_float(left));
  node[2 * size_t(id) + 1] = make_float4(hi.x, hi.y, hi.z, __uint_as_float(right));
}

// Leaf boxes (bounding sphere of each body) and per-block scene bounds.
__global__ void k_bvh_leaves(const float4* __restrict__ pose, int bodyOff, int n, BvhPool b, int nodeOff, float4* blockBounds,
                             int withBounds) {
  __shared__ float3 slo[256], shi[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float3 lo = make_float3(3.402823e38f, 3.402823e38f, 3.402823e38f), hi = make_float3(-3.402823e38f, -3.402823e38f, -3.402823e38f);
  if (i < n) {
    const float4 p = pose[2 * size_t(bodyOff + i)];
    lo = make_float3(p.x - p.w, p.y - p.w, p.z - p.w);
    hi = make_float3(p.x + p.w, p.y + p.w, p.z + p.w);
    store_node(b.node, uint32_t(nodeOff + i), lo, uint32_t(i), hi, BVH_END);
    if (withBounds) b.minIdx[nodeOff + i] = uint32_t(i);
  }
  if (!withBounds) return;
  slo[threadIdx.x] = lo;
  shi[threadIdx.x] = hi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (int(threadIdx.x) < s) {
      const float3 a = slo[threadIdx.x + s], c = shi[threadIdx.x + s];
      slo[threadIdx.x] = make_float3(fminf(slo[threadIdx.x].x, a.x), fminf(slo[threadIdx.x].y, a.y), fminf(slo[threadIdx.x].z, a.z));
      shi[threadIdx.x] = make_float3(fmaxf(shi[threadIdx.x].x, c.x), fmaxf(shi[threadIdx.x].y, c.y), fmaxf(shi[threadIdx.x].z, c.z));
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    blockBounds[2 * blockIdx.x] = make_float4(slo[0].x, slo[0].y, slo[0].z, 0.f);
    blockBounds[2 * blockIdx.x + 1] = make_float4(shi[0].x, shi[0].y, shi[0].z, 0.f);
  }
}

// One block folds the per-block bounds into bounds[0], bounds[1].
__global__ void k_bvh_bounds(float4* blockBounds, int nblocks, float4* bounds) {
  __shared__ float3 slo[256], shi[256];
  float3 lo = make_float3(3.402823e38f, 3.402823e38f, 3.402823e38f), hi = make_float3(-3.402823e38f, -3.402823e38f, -3.402823e38f);
  for (int k = threadIdx.x; k < nblocks; k += blockDim.x) {
    const float4 a = blockBounds[2 * k], c = blockBounds[2 * k + 1];
    lo = make_float3(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z));
    hi = make_float3(fmaxf(hi.x, c.x), fmaxf(hi.y, c.y), fmaxf(hi.z, c.z));
  }
  slo[threadIdx.x] = lo;
  shi[threadIdx.x] = hi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (int(threadIdx.x) < s) {
      const float3 a = slo[threadIdx.x + s], c = shi[threadIdx.x + s];
      slo[threadIdx.x] = make_float3(fminf(slo[threadIdx.x].x, a.x), fminf(slo[threadIdx.x].y, a.y), fminf(slo[threadIdx.x].z, a.z));
      shi[threadIdx.x] = make_float3(fmaxf(shi[threadIdx.x].x, c.x), fmaxf(shi[threadIdx.x].y, c.y), fmaxf(shi[threadIdx.x].z, c.z));
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    bounds[0] = make_float4(slo[0].x, slo[0].y, slo[0].z, 0.f);
    bounds[1] = make_float4(shi[0].x, shi[0].y, shi[0].z, 0.f);
  }
}

// 30-bit Morton code of each leaf box's centre within the scene bounds (half scale keeps the
// extent finite for distant coordinates), keyed with the leaf index.
__global__ void k_bvh_morton(BvhPool b, int nodeOff, int n, const float4* __restrict__ bounds, uint2* keys) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = b.node[2 * size_t(nodeOff + i)], c = b.node[2 * size_t(nodeOff + i) + 1];
  const float4 lo = bounds[0], hi = bounds[1];
  const float ex = fmaxf(hi.x * 0.5f - lo.x * 0.5f, 1e-20f), ey = fmaxf(hi.y * 0.5f - lo.y * 0.5f, 1e-20f),
              ez = fmaxf(hi.z * 0.5f - lo.z * 0.5f, 1e-20f);
  const float px = fminf(fmaxf(((a.x * 0.25f + c.x * 0.25f) - lo.x * 0.5f) / ex, 0.f), 0.999999f);
  const float py = fminf(fmaxf(((a.y * 0.25f + c.y * 0.25f) - lo.y * 0.5f) / ey, 0.f), 0.999999f);
  const float pz = fminf(fmaxf(((a.z * 0.25f + c.z * 0.25f) - lo.z * 0.5f) / ez, 0.f), 0.999999f);
  const uint32_t code = (expand_bits(uint32_t(px * 1024.f)) << 2) | (expand_bits(uint32_t(py * 1024.f)) << 1) |
                        expand_bits(uint32_t(pz * 1024.f));
  keys[i] = make_uint2(code, uint32_t(i));
}

// Radix sort of the (code, leaf) keys by code, BITS bits per pass (4, 6 or 8: the autotuner's
// digit-width candidates; every width gives the same stable order).
// Pass 1: per-block digit counts, digit-major (hist[digit * blocks + block]).
template <int BITS>
__global__ void __launch_bounds__(RADIX_THREADS) k_radix_hist(const uint2* __restrict__ in, int n, int shift, int* hist) {
  constexpr int DIGITS = 1 << BITS;
  constexpr uint32_t MASK = DIGITS - 1;
  __shared__ int cnt[DIGITS];
  for (int q = threadIdx.x; q < DIGITS; q += RADIX_THREADS) cnt[q] = 0;
  __syncthreads();
  const int base = blockIdx.x * RADIX_ITEMS;
  for (int k = threadIdx.x; k < RADIX_ITEMS; k += RADIX_THREADS) {
    const int e = base + k;
    if (e < n) atomicAdd(&cnt[(in[e].x >> shift) & MASK], 1);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < DIGITS; q += RADIX_THREADS) hist[q * gridDim.x + blockIdx.x] = cnt[q];
}

// Pass 2: stable scatter. Each round ranks RADIX_THREADS consecutive keys (warp match for the rank
// inside a warp, per-warp digit counts for the warps before) after the block's earlier rounds,
// so equal digits keep their input order.
template <int BITS>
__global__ void __launch_bounds__(RADIX_THREADS) k_radix_scatter(const uint2* __restrict__ in, uint2* __restrict__ out, int n, int shift,
                                                                 const int* __restrict__ offsets) {
  constexpr int DIGITS = 1 << BITS;
  constexpr uint32_t MASK = DIGITS - 1;
  constexpr int WARPS = RADIX_THREADS / 32;
  __shared__ int warpCnt[WARPS][DIGITS];
  __shared__ int running[DIGITS];
  __shared__ int start[DIGITS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int q = threadIdx.x; q < DIGITS; q += RADIX_THREADS) {
    start[q] = offsets[q * gridDim.x + blockIdx.x];
    running[q] = 0;
    for (int w = 0; w < WARPS; w++) warpCnt[w][q] = 0;
  }
  __syncthreads();
  const int base = blockIdx.x * RADIX_ITEMS;
  for (int round = 0; round < RADIX_ITEMS / RADIX_THREADS; round++) {
    const int e = base + round * RADIX_THREADS + threadIdx.x;
    const bool valid = e < n;
    uint2 v = make_uint2(0u, 0u);
    uint32_t d = uint32_t(DIGITS);  // out-of-range keys form their own (unused) digit
    if (valid) {
      v = in[e];
      d = (v.x >> shift) & MASK;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rankInWarp = __popc(peers & ((1u << lane) - 1u));
    if (valid && rankInWarp == 0) warpCnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int before = running[d];
      for (int w = 0; w < warp; w++) before += warpCnt[w][d];
      out[start[d] + before + rankInWarp] = v;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < DIGITS; q += RADIX_THREADS) {
      int total = 0;
      for (int w = 0; w < WARPS; w++) {
        total += warpCnt[w][q];
        warpCnt[w][q] = 0;
      }
      running[q] += total;
    }
    __syncthreads();
  }
}

template <int BITS>
static int radix_passes(const uint2*& keysOut, BvhScratch sc, int n, int rb, void* scanTemp, cudaStream_t s) {
  constexpr int PASSES = (30 + BITS - 1) / BITS;  // codes have 30 bits
  for (int pass = 0; pass < PASSES; pass++) {
    const uint2* in = sc.keys[pass & 1];
    uint2* out = sc.keys[(pass & 1) ^ 1];
    k_radix_hist<BITS><<<rb, RADIX_THREADS, 0, s>>>(in, n, BITS * pass, sc.hist);
    scan_exclusive(sc.hist, (1 << BITS) * rb, nullptr, scanTemp, s);
    k_radix_scatter<BITS><<<rb, RADIX_THREADS, 0, s>>>(in, out, n, BITS * pass, sc.hist);
    note_launches(2);
  }
  keysOut = sc.keys[PASSES & 1];
  return PASSES;
}

__global__ void k_bvh_seed(const uint2* __restrict__ keys, int n, uint32_t* clusters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) clusters[i] = keys[i].y;
}

__global__ void k_bvh_init_links(BvhPool b, int nodeOff, int nodes) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nodes; i += gridDim.x * blockDim.x) {
    b.parent[nodeOff + i] = BVH_END;
    b.escape[nodeOff + i] = BVH_END;
  }
}

// One treelet per warp (lanes 0-15): merge mutual nearest neighbours (least union surface area,
// ties to the lower lane) until one cluster is left. Node ids are nodeBase + treelet * 15 + k
// in creation order, so children precede their parents. At least one mutual pair exists each
// round; if rounding ever left none, the two lowest live clusters merge, so the loop always
// ends within 15 rounds.
__global__ void __launch_bounds__(32) k_bvh_treelets(BvhPool b, int nodeOff, uint32_t* clusters, int inputOffset, int outputOffset,
                                                     int inputCount, int nodeBase) {
  const int t = blockIdx.x;
  const int lane = threadIdx.x;
  const int at = t * BVH_WIDTH + lane;
  bool alive = lane < BVH_WIDTH && at < inputCount;
  uint32_t cid = BVH_END, mn = BVH_END;
  float3 lo = make_float3(0.f, 0.f, 0.f), hi = make_float3(0.f, 0.f, 0.f);
  if (alive) {
    cid = clusters[inputOffset + at];
    const float4 a = b.node[2 * size_t(nodeOff + cid)], c = b.node[2 * size_t(nodeOff + cid) + 1];
    lo = make_float3(a.x, a.y, a.z);
    hi = make_float3(c.x, c.y, c.z);
    mn = b.minIdx[nodeOff + cid];
  }
  int created = 0;
  for (int round = 0; round < BVH_WIDTH; round++) {
    const unsigned live = __ballot_sync(0xffffffffu, alive);
    if (__popc(live) <= 1) break;
    float best = 3.402823e38f;
    int winner = -1;
    for (int j = 0; j < BVH_WIDTH; j++) {
      const float3 jl = make_float3(__shfl_sync(0xffffffffu, lo.x, j), __shfl_sync(0xffffffffu, lo.y, j), __shfl_sync(0xffffffffu, lo.z, j));
      const float3 jh = make_float3(__shfl_sync(0xffffffffu, hi.x, j), __shfl_sync(0xffffffffu, hi.y, j), __shfl_sync(0xffffffffu, hi.z, j));
      if (!alive || j == lane || !((live >> j) & 1u)) continue;
      const float cst = area(make_float3(fminf(lo.x, jl.x), fminf(lo.y, jl.y), fminf(lo.z, jl.z)),
                             make_float3(fmaxf(hi.x, jh.x), fmaxf(hi.y, jh.y), fmaxf(hi.z, jh.z)));
      if (cst < best) {
        best = cst;
        winner = j;
      }
    }
    const int partnerBest = __shfl_sync(0xffffffffu, winner, winner >= 0 ? winner : lane);
    bool merge = alive && winner > lane && partnerBest == lane;
    bool retire = alive && winner >= 0 && winner < lane && partnerBest == lane;
    unsigned mm = __ballot_sync(0xffffffffu, merge);
    int mate = winner;
    if (mm == 0u) {  // no mutual pair (only possible with non-finite boxes): merge the two lowest
      const int a = __ffs(live) - 1;
      const int c = __ffs(live & ~(1u << a)) - 1;
      merge = lane == a;
      retire = lane == c;
      mate = c;
      mm = 1u << a;
    }
    const int src = merge ? mate : lane;
    const float3 ml = make_float3(__shfl_sync(0xffffffffu, lo.x, src), __shfl_sync(0xffffffffu, lo.y, src), __shfl_sync(0xffffffffu, lo.z, src));
    const float3 mh = make_float3(__shfl_sync(0xffffffffu, hi.x, src), __shfl_sync(0xffffffffu, hi.y, src), __shfl_sync(0xffffffffu, hi.z, src));
    const uint32_t mcid = __shfl_sync(0xffffffffu, cid, src);
    const uint32_t mmn = __shfl_sync(0xffffffffu, mn, src);
    if (merge) {
      const uint32_t id = uint32_t(nodeBase + t * (BVH_WIDTH - 1) + created + __popc(mm & ((1u << lane) - 1u)));
      lo = make_float3(fminf(lo.x, ml.x), fminf(lo.y, ml.y), fminf(lo.z, ml.z));
      hi = make_float3(fmaxf(hi.x, mh.x), fmaxf(hi.y, mh.y), fmaxf(hi.z, mh.z));
      store_node(b.node, uint32_t(nodeOff) + id, lo, cid, hi, mcid);
      b.parent[nodeOff + cid] = id;
      b.parent[nodeOff + mcid] = id;
      mn = min(mn, mmn);
      b.minIdx[nodeOff + id] = mn;
      cid = id;
    }
    if (retire) alive = false;
    created += __popc(mm);
  }
  if (alive) clusters[outputOffset + t] = cid;
}

// Escape link of every node: the right sibling of the nearest ancestor reached from a left child.
__global__ void k_bvh_ropes(BvhPool b, int nodeOff, int nodes, uint32_t root) {
  for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nodes; id += gridDim.x * blockDim.x) {
    uint32_t at = uint32_t(id), escape = BVH_END;
    for (int depth = 0; depth < 4096; depth++) {  // depth <= 15 per level; bounded regardless
      if (at == root) break;
      const uint32_t p = b.parent[nodeOff + at];
      if (p == BVH_END) break;
      const uint32_t left = __float_as_uint(b.node[2 * size_t(nodeOff + p)].w);
      if (left == at) {
        escape = __float_as_uint(b.node[2 * size_t(nodeOff + p) + 1].w);
        break;
      }
      at = p;
    }
    b.escape[nodeOff + id] = escape;
  }
}

// Refit: a treelet's nodes in creation order (children first).
__global__ void k_bvh_refit_treelets(BvhPool b, int nodeOff, int inputCount, int nodeBase) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int first = t * BVH_WIDTH;
  if (first >= inputCount) return;
  const int count = min(BVH_WIDTH, inputCount - first);
  for (int j = 0; j + 1 < count; j++) {
    const uint32_t id = uint32_t(nodeOff + nodeBase + t * (BVH_WIDTH - 1) + j);
    const uint32_t l = __float_as_uint(b.node[2 * size_t(id)].w), r = __float_as_uint(b.node[2 * size_t(id) + 1].w);
    const float4 la = b.node[2 * size_t(nodeOff + l)], lb = b.node[2 * size_t(nodeOff + l) + 1];
    const float4 ra = b.node[2 * size_t(nodeOff + r)], rb = b.node[2 * size_t(nodeOff + r) + 1];
    store_node(b.node, id, make_float3(fminf(la.x, ra.x), fminf(la.y, ra.y), fminf(la.z, ra.z)), l,
               make_float3(fmaxf(lb.x, rb.x), fmaxf(lb.y, rb.y), fmaxf(lb.z, rb.z)), r);
  }
}

int blocks_of(long long n, int threads) { return int(n <= 0 ? 1 : (n + threads - 1) / threads); }

}  // namespace

// ---------------------------------------------------------------- host side

void bvh_layout(int n, BvhLayout& L) {
  L.levels.clear();
  L.root = n == 0 ? BVH_END : 0u;
  int inputCount = n, nodeBase = n, inputOffset = 0, outputOffset = n;
  while (inputCount > 1) {
    const int blocks = (inputCount + BVH_WIDTH - 1) / BVH_WIDTH;
    L.levels.push_back(BvhLevel{inputCount, nodeBase, inputOffset, outputOffset, blocks});
    if (blocks == 1) L.root = uint32_t(nodeBase + inputCount - 2);
    nodeBase += blocks * (BVH_WIDTH - 1);
    inputOffset = outputOffset;
    outputOffset += blocks;
    inputCount = blocks;
  }
  L.nodes = nodeBase;
  L.clusters = outputOffset;
}

size_t bvh_scratch_keys(int n) { return size_t(n > 0 ? n : 1); }
size_t bvh_scratch_hist(int n) { return size_t(256) * size_t(blocks_of(n, RADIX_ITEMS)); }
size_t bvh_scratch_bounds(int n) { return size_t(2) * size_t(blocks_of(n, 256)) + 2; }

void launch_bvh_build(const BodyPtrs& bd, int bodyOff, int n, BvhPool b, int nodeOff, const BvhLayout& L, BvhScratch sc,
                      void* scanTemp, int radixBits, cudaStream_t s) {
  if (n <= 0) return;
  const int lb = blocks_of(n, 256);
  k_bvh_init_links<<<blocks_of(L.nodes, 256) > device_sms() * 8 ? device_sms() * 8 : blocks_of(L.nodes, 256), 256, 0, s>>>(b, nodeOff, L.nodes);
  float4* bounds = sc.bounds + 2 * size_t(lb);
  k_bvh_leaves<<<lb, 256, 0, s>>>(bd.pose, bodyOff, n, b, nodeOff, sc.bounds, 1);
  k_bvh_bounds<<<1, 256, 0, s>>>(sc.bounds, lb, bounds);
  k_bvh_morton<<<lb, 256, 0, s>>>(b, nodeOff, n, bounds, sc.keys[0]);
  note_launches(4);
  const int rb = blocks_of(n, RADIX_ITEMS);
  const uint2* sorted = nullptr;
  if (radixBits == 4) radix_passes<4>(sorted, sc, n, rb, scanTemp, s);
  else if (radixBits == 6) radix_passes<6>(sorted, sc, n, rb, scanTemp, s);
  else radix_passes<8>(sorted, sc, n, rb, scanTemp, s);
  k_bvh_seed<<<lb, 256, 0, s>>>(sorted, n, sc.clusters);
  note_launches(1);
  for (const BvhLevel& v : L.levels) {
    k_bvh_treelets<<<v.blocks, 32, 0, s>>>(b, nodeOff, sc.clusters, v.inputOffset, v.outputOffset, v.inputCount, v.nodeBase);
    note_launches(1);
  }
  int rblocks = blocks_of(L.nodes, 256);
  if (rblocks > device_sms() * 8) rblocks = device_sms() * 8;
  k_bvh_ropes<<<rblocks, 256, 0, s>>>(b, nodeOff, L.nodes, L.root);
  note_launches(1);
}

void launch_bvh_refit(const BodyPtrs& bd, int bodyOff, int n, BvhPool b, int nodeOff, const BvhLayout& L, cudaStream_t s) {
  if (n <= 0) return;
  k_bvh_leaves<<<blocks_of(n, 256), 256, 0, s>>>(bd.pose, bodyOff, n, b, nodeOff, nullptr, 0);
  note_launches(1);
  for (const BvhLevel& v : L.levels) {
    k_bvh_refit_treelets<<<blocks_of(v.blocks, 64), 64, 0, s>>>(b, nodeOff, v.inputCount, v.nodeBase);
    note_launches(1);
  }
}

}  // namespace avbd
