// Collision stage: hashed-grid broadphase and narrowphase with warm-start matching.
//
// Compiled with -fmad=false: every product and sum is rounded separately, in the order of
// the reference's arithmetic, so pair sets and contact counts match its float32 results
// exactly.
//
// Broadphase. The pair predicate is the reference CPU's (src/native/cpu/cpuPhysics3D.js:319-343):
// A = the higher body index, B = the lower; bounding spheres overlap (|xA - xB|^2 <= (rA + rB)^2),
// not both static, collision masks agree, and no live joint/spring/ignore links the two. A hashed
// grid only narrows the candidates: per world, bodies with radius <= largeR go into cells of size
// cell >= 2 * max small radius keyed by (world, cell); each small body scans the 27 cells around
// its own for lower-index partners, every body scans its world's large-body list, and large
// bodies scan their world's lower-index small bodies. Two passes (count, then write after a
// prefix sum) give each body a private output range, which it sorts by partner: the pair list
// comes out sorted by (hi, lo) with no global sort and no atomics on the output.
//
// Narrowphase. One thread per candidate pair. Box-box: 15-axis SAT with the faceBias rule,
// reference-face clipping, up to 8 contacts (src/native/cpu/cpuBoxContacts3D.ts:409-499, the
// pinned reference/three-avbd/src/avbd3d/ref/collide.ts). Pairs with a sphere: the reference
// CPU's generic support-function SAT with one contact (src/native/cpu/cpuContacts3D.js:188-296).
// Warm start: the previous step's manifold of the same pair is found by binary search in the
// previous (sorted) pair list and its contacts are matched by feature key
// (src/native/cpu/cpuPhysics3D.js:76-147).
#include <float.h>

#include "engine.cuh"

namespace avbd {

// ------------------------------------------------------------------ grid

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ uint32_t cell_hash(int world, int cx, int cy, int cz) {
  uint32_t h = uint32_t(cx) * 73856093u;
  h ^= uint32_t(cy) * 19349663u;
  h ^= uint32_t(cz) * 83492791u;
  h ^= uint32_t(world) * 2654435761u;
  return mix32(h);
}

__device__ __forceinline__ int cell_coord(float x, float cell) { return __float2int_rd(x / cell); }

// The tick's active lists: bodies and joints of the active worlds (world by world) and the
// body -> list position map, from the active-world table (prefixes computed on the host).
__device__ __forceinline__ int active_world(const Tick& t, int k, int field) {
  int a = 0, b = t.nActive;  // last entry with prefix <= k
  while (b - a > 1) {
    const int m = (a + b) >> 1;
    if ((field == 0 ? t.active[m].y : t.active[m].z) <= k) a = m;
    else b = m;
  }
  return a;
}

__global__ void k_tick_lists(Tick t, const WorldDev* __restrict__ worlds, Topo topo) {
  const int total = max(t.nBodies, t.nJoints);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    if (k < t.nBodies) {
      const int a = active_world(t, k, 0);
      const int4 e = t.active[a];
      const int b = worlds[e.x].bodyOff + (k - e.y);
      t.bodies[k] = b;
      topo.activeIndex[b] = k;
    }
    if (k < t.nJoints) {
      const int a = active_world(t, k, 1);
      const int4 e = t.active[a];
      t.joints[k] = worlds[e.x].jointOff + (k - e.z);
    }
  }
}

__global__ void k_grid_count(const float4* __restrict__ pose, const int4* __restrict__ meta, const WorldDev* __restrict__ worlds,
                             Tick t, uint32_t mask, int* __restrict__ cellCount, int* __restrict__ bodyBucket) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += gridDim.x * blockDim.x) {
    const int i = t.bodies[k];
    const float4 p = pose[2 * size_t(i)];
    const int w = meta[i].x;
    const WorldDev& W = worlds[w];
    if (p.w > W.largeR || (W.flags & FLAG_BVH)) {  // large, or found through the world's tree
      bodyBucket[i] = -1;
      continue;
    }
    uint32_t b = cell_hash(w, cell_coord(p.x, W.cell), cell_coord(p.y, W.cell), cell_coord(p.z, W.cell)) & mask;
    bodyBucket[i] = int(b);
    atomicAdd(&cellCount[b], 1);
  }
}

// Bucket the small bodies; each bucket entry also records its body's cell and position, so the
// pair passes read candidates from contiguous memory and skip bodies of other cells or worlds
// that share a hash bucket.
__global__ void k_grid_scatter(const float4* __restrict__ pose, const int4* __restrict__ meta, const WorldDev* __restrict__ worlds,
                               Tick t, Grid g) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += gridDim.x * blockDim.x) {
    const int i = t.bodies[k];
    const int b = g.bodyBucket[i];
    if (b < 0) continue;
    const float4 p = pose[2 * size_t(i)];
    const int w = meta[i].x;
    const float cell = worlds[w].cell;
    const int slot = g.cellCount[b] + atomicAdd(&g.cellFill[b], 1);
    g.cellBodies[slot] = i;
    g.cellKey[slot] = make_int4(cell_coord(p.x, cell), cell_coord(p.y, cell), cell_coord(p.z, cell), w);
    g.cellPos[slot] = p;
  }
}

void launch_tick_begin(Tick t, Topo topo, const WorldDev* worlds, cudaStream_t s) {
  const int total = t.nBodies > t.nJoints ? t.nBodies : t.nJoints;
  if (total == 0) return;
  k_tick_lists<<<grid_blocks(total, 256), 256, 0, s>>>(t, worlds, topo); note_launches(1);
}

void launch_grid_build(const BodyPtrs& b, const WorldDev* worlds, Tick t, Grid g, void* scanTemp, cudaStream_t s) {
  const int table = int(g.tableMask) + 1;
  cudaMemsetAsync(g.cellCount, 0, sizeof(int) * (table + 1), s);
  cudaMemsetAsync(g.cellFill, 0, sizeof(int) * table, s);
  if (t.nBodies == 0) return;
  k_grid_count<<<grid_blocks(t.nBodies, 256), 256, 0, s>>>(b.pose, b.meta, worlds, t, g.tableMask, g.cellCount, g.bodyBucket); note_launches(1);
  scan_exclusive(g.cellCount, table + 1, nullptr, scanTemp, s);
  k_grid_scatter<<<grid_blocks(t.nBodies, 256), 256, 0, s>>>(b.pose, b.meta, worlds, t, g); note_launches(1);
}

// ------------------------------------------------------------------ pair predicate

struct PairCtx {
  const float4* __restrict__ pose;  // (pos, rot) pairs
  __device__ __forceinline__ float4 pos(int i) const { return pose[2 * size_t(i)]; }
  const float4* __restrict__ mass;
  const int4* __restrict__ meta;
  NoCollide nc;
  const int* __restrict__ jbroken;
};

__device__ __forceinline__ bool linked(const NoCollide& nc, const int* jbroken, int hi, int lo) {
  const unsigned long long key = (unsigned long long)(uint32_t)hi << 32 | (uint32_t)lo;
  int a = 0, b = nc.n;
  while (a < b) {
    int m = (a + b) >> 1;
    if (nc.keys[m] < key) a = m + 1;
    else b = m;
  }
  for (; a < nc.n && nc.keys[a] == key; a++) {
    int j = nc.jid[a];
    // 2: broken in the last step's dual or torn at this step's start, still joining the pair in
    // this broadphase (the reference drops a broken constraint from the bodies' lists after it)
    if (j < 0 || jbroken[j] != 1) return true;
  }
  return false;
}

// cpuPhysics3D.js:319-343 pair(): A = hi, B = lo. The conditions are independent, so the cheap
// distance test (on the partner's position pB) runs first.
__device__ __forceinline__ bool pair_test(const PairCtx& c, int hi, int lo, float4 pA, float4 pB, float mA, int4 metaA) {
  const float r = pA.w + pB.w;
  const V3 d = v3(pA) - v3(pB);
  if (!(dot(d, d) <= r * r)) return false;
  const float mB = c.mass[lo].x;
  if (mA <= 0.f && mB <= 0.f) return false;
  const int4 metaB = c.meta[lo];
  if (metaB.x != metaA.x) return false;
  if (!(uint32_t(metaA.z) & uint32_t(metaB.w)) || !(uint32_t(metaB.z) & uint32_t(metaA.w))) return false;
  if (c.nc.n > 0 && linked(c.nc, c.jbroken, hi, lo)) return false;
  return true;
}

// Lower-index partners from the world's tree: stackless traversal along escape links of every
// node whose box meets body i's (bounding sphere box, widened by a margin far above the rounding
// of the boxes) and whose subtree holds a lower index.
template <class Emit>
__device__ __forceinline__ void tree_partners(const PairCtx& c, const WorldDev& W, const Grid& g, int i, float4 pA, float mA, int4 metaA,
                                              Emit emit) {
  if (W.bvhRoot < 0) return;
  const uint32_t local = uint32_t(i - W.bodyOff);
  const float eps = 1e-3f + 1e-6f * (fabsf(pA.x) + fabsf(pA.y) + fabsf(pA.z));
  const float r = pA.w + eps;
  const float lx = pA.x - r, ly = pA.y - r, lz = pA.z - r, hx = pA.x + r, hy = pA.y + r, hz = pA.z + r;
  const float4* node = g.bvh.node + 2 * size_t(W.bvhNodeOff);
  const uint32_t* escape = g.bvh.escape + W.bvhNodeOff;
  const uint32_t* minIdx = g.bvh.minIdx + W.bvhNodeOff;
  uint32_t at = uint32_t(W.bvhRoot);
  // every node is entered at most once; the bound only guards against a damaged tree
  for (int guard = 4 * W.bodyCount + 8; at != BVH_END && guard > 0; guard--) {
    if (minIdx[at] >= local) {
      at = escape[at];
      continue;
    }
    const float4 lo = node[2 * size_t(at)], hi = node[2 * size_t(at) + 1];
    if (hi.x < lx || hi.y < ly || hi.z < lz || lo.x > hx || lo.y > hy || lo.z > hz) {
      at = escape[at];
      continue;
    }
    if (__float_as_uint(hi.w) == BVH_END) {  // leaf
      const int j = W.bodyOff + int(__float_as_uint(lo.w));
      if (pair_test(c, i, j, pA, c.pos(j), mA, metaA)) emit(j);
      at = escape[at];
    } else {
      at = __float_as_uint(lo.w);
    }
  }
}

// Enumerate the lower-index partners of body i; emit(j) for each pair (i, j).
template <class Emit>
__device__ __forceinline__ void for_each_partner(const PairCtx& c, const WorldDev* __restrict__ worlds, const Grid& g, int i, Emit emit) {
  const float4 pA = c.pos(i);
  const float mA = c.mass[i].x;
  const int4 metaA = c.meta[i];
  const int w = metaA.x;
  const WorldDev W = worlds[w];
  if (W.flags & FLAG_BVH) {
    tree_partners(c, W, g, i, pA, mA, metaA, emit);
    return;
  }
  const bool small = !(pA.w > W.largeR);
  if (small) {
    const int cx = cell_coord(pA.x, W.cell), cy = cell_coord(pA.y, W.cell), cz = cell_coord(pA.z, W.cell);
    // Only the neighbour cells within the body's reach: a partner is closer than rA + rB <= rA +
    // cell / 2 on every axis (cell >= 2 x the largest small radius); the reach is padded far
    // beyond the rounding of the coordinates, so no cell that can hold a partner is skipped.
    const float reach = pA.w + 0.501f * W.cell + 1e-5f * (fabsf(pA.x) + fabsf(pA.y) + fabsf(pA.z));
    const int x0 = cell_coord(pA.x - reach, W.cell) < cx ? -1 : 0, x1 = cell_coord(pA.x + reach, W.cell) > cx ? 1 : 0;
    const int y0 = cell_coord(pA.y - reach, W.cell) < cy ? -1 : 0, y1 = cell_coord(pA.y + reach, W.cell) > cy ? 1 : 0;
    const int z0 = cell_coord(pA.z - reach, W.cell) < cz ? -1 : 0, z1 = cell_coord(pA.z + reach, W.cell) > cz ? 1 : 0;
    for (int dz = z0; dz <= z1; dz++) {
      // the bucket ranges of this plane are loaded together (up to eighteen independent loads in
      // flight instead of two), then scanned
      int r0[9], r1[9];
#pragma unroll
      for (int q = 0; q < 9; q++) {
        const int dx = (q % 3) - 1, dy = (q / 3) - 1;
        r0[q] = r1[q] = 0;
        if (dx < x0 || dx > x1 || dy < y0 || dy > y1) continue;
        const uint32_t b = cell_hash(w, cx + dx, cy + dy, cz + dz) & g.tableMask;
        r0[q] = g.cellCount[b];
        r1[q] = g.cellCount[b + 1];
      }
#pragma unroll 1
      for (int q = 0; q < 9; q++) {
          const int nx = cx + (q % 3) - 1, ny = cy + (q / 3) - 1, nz = cz + dz;
          const int s0 = r0[q], s1 = r1[q];
          for (int s = s0; s < s1; s++) {
            // the distance test first: one load per entry, and the few entries that pass it read
            // their body index (the conditions are independent, so the pair set is the same)
            const float4 pB = g.cellPos[s];
            const float r = pA.w + pB.w;
            const V3 d = v3(pA) - v3(pB);
            if (!(dot(d, d) <= r * r)) continue;
            const int j = g.cellBodies[s];
            if (j >= i) continue;
            // only the entries of this very cell: a bucket shared by several neighbour cells (or
            // worlds) is scanned once per cell, and each body counts in its own cell only
            const int4 key = g.cellKey[s];
            if (key.x != nx || key.y != ny || key.z != nz || key.w != w) continue;
            if (pair_test(c, i, j, pA, pB, mA, metaA)) emit(j);
          }
      }
    }
  }
  for (int k = 0; k < W.largeCount; k++) {
    const int L = g.large[W.largeOff + k];
    if (L >= i) break;
    if (pair_test(c, i, L, pA, c.pos(L), mA, metaA)) emit(L);
  }
  if (!small) {
    for (int j = W.bodyOff; j < i; j++) {
      const float4 pB = c.pos(j);
      if (pB.w > W.largeR) continue;  // large partners came from the list above
      if (pair_test(c, i, j, pA, pB, mA, metaA)) emit(j);
    }
  }
}

// Pair passes over the tick's active bodies (k = list position). Each world writes its pairs into
// its own region of the buffer it does not hold its last state in; a world whose pairs exceed its
// region records how many it needs (the host grows the region and re-runs the tick).
__global__ void k_pair_count(PairCtx c, const WorldDev* __restrict__ worlds, Grid g, Tick t, int* __restrict__ pairCount) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= t.nBodies; k += gridDim.x * blockDim.x) {
    int cnt = 0;
    if (k < t.nBodies) {
      uint32_t* keep = g.pairTmp + k;  // column layout: partner m at keep[m * nBodies]
      for_each_partner(c, worlds, g, t.bodies[k], [&](int j) {
        if (cnt < PAIR_TMP) keep[size_t(cnt) * t.nBodies] = uint32_t(j);
        cnt++;
      });
    }
    pairCount[k] = cnt;
  }
}

// per active world: pairs found, region overflow, pair counts of the active-pair prefix
__global__ void k_pair_worlds(const WorldDev* __restrict__ worlds, Tick t, const int* __restrict__ pairStart, Counters* ctr) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < t.nActive; a += gridDim.x * blockDim.x) {
    const int4 e = t.active[a];
    const WorldDev& W = worlds[e.x];
    const int need = pairStart[e.y + W.bodyCount] - pairStart[e.y];
    const int cur = 1 - t.which[e.x];
    const int n = min(need, W.pairCap);
    t.pairN[cur * t.maxWorlds + e.x] = n;
    t.pairPrefix[a] = n;
    if (need > W.pairCap) {
      t.wover[e.x] = need;
      atomicAdd(&ctr->overflowWorlds, 1);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) t.pairPrefix[t.nActive] = 0;
}

// In-place heapsort of a (hi, lo) range by lo (the partners of one body are distinct).
__device__ void heapsort_by_partner(uint2* a, int n) {
  auto sift = [&](int root, int size) {
    const uint2 v = a[root];
    int at = root;
    while (true) {
      int child = 2 * at + 1;
      if (child >= size) break;
      if (child + 1 < size && a[child + 1].y > a[child].y) child++;
      if (a[child].y <= v.y) break;
      a[at] = a[child];
      at = child;
    }
    a[at] = v;
  };
  for (int r = n / 2 - 1; r >= 0; r--) sift(r, n);
  for (int size = n - 1; size > 0; size--) {
    const uint2 top = a[0];
    a[0] = a[size];
    a[size] = top;
    sift(0, size);
  }
}

__global__ void k_pair_write(PairCtx c, const WorldDev* __restrict__ worlds, Grid g, Tick t, const int* __restrict__ pairStart,
                             uint2* __restrict__ pairs) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += gridDim.x * blockDim.x) {
    const int i = t.bodies[k];
    const int w = c.meta[i].x;
    const WorldDev& W = worlds[w];
    const int4 e = t.active[t.wactive[w]];
    const int local = pairStart[k] - pairStart[e.y];
    const int cap = W.pairCap;
    uint2* out = pairs + (size_t)(1 - t.which[w]) * t.slotStride + W.pairOff;
    const int total = pairStart[k + 1] - pairStart[k];
    int n = 0;
    if (total <= PAIR_TMP) {  // the partners kept by the counting pass
      const uint32_t* keep = g.pairTmp + k;
      for (; n < total; n++)
        if (local + n < cap) out[local + n] = make_uint2(uint32_t(i), keep[size_t(n) * t.nBodies]);
    } else {
      for_each_partner(c, worlds, g, i, [&](int j) {
        const int slot = local + n++;
        if (slot < cap) out[slot] = make_uint2(uint32_t(i), uint32_t(j));
      });
    }
    // this body's range by partner: insertion sort for the usual few dozen partners, heapsort
    // beyond (a static or large body in a late slot can own a large share of its world's pairs)
    const int end = min(local + n, cap);
    if (end - local <= 64) {
      for (int a = local + 1; a < end; a++) {
        const uint2 v = out[a];
        int b = a;
        while (b > local && out[b - 1].y > v.y) {
          out[b] = out[b - 1];
          b--;
        }
        out[b] = v;
      }
    } else {
      heapsort_by_partner(out + local, end - local);
    }
  }
}

// active pair slots: the written part of each active world's region, world by world
__global__ void k_pair_slots(const WorldDev* __restrict__ worlds, Tick t, const Counters* __restrict__ ctr) {
  const int total = ctr->activePairs;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    int a = 0, b = t.nActive;
    while (b - a > 1) {
      const int m = (a + b) >> 1;
      if (t.pairPrefix[m] <= q) a = m;
      else b = m;
    }
    const int w = t.active[a].x;
    t.pairs[q] = (1 - t.which[w]) * t.slotStride + worlds[w].pairOff + (q - t.pairPrefix[a]);
  }
}

void launch_pairs(const BodyPtrs& b, const WorldDev* worlds, Tick t, Grid g, NoCollide nc, const int* jbroken, int* pairCount,
                  PairPtrs P, Counters* ctr, void* scanTemp, cudaStream_t s) {
  PairCtx c{b.pose, b.mass, b.meta, nc, jbroken};
  cudaMemsetAsync(ctr, 0, 2 * sizeof(int), s);  // activePairs, overflowWorlds
  if (t.nActive == 0) return;
  k_pair_count<<<grid_blocks(t.nBodies + 1, 128), 128, 0, s>>>(c, worlds, g, t, pairCount); note_launches(1);
  scan_exclusive(pairCount, t.nBodies + 1, nullptr, scanTemp, s);
  k_pair_worlds<<<grid_blocks(t.nActive, 128), 128, 0, s>>>(worlds, t, pairCount, ctr); note_launches(1);
  scan_exclusive(t.pairPrefix, t.nActive + 1, &ctr->activePairs, scanTemp, s);
  k_pair_write<<<grid_blocks(t.nBodies, 128), 128, 0, s>>>(c, worlds, g, t, pairCount, P.pair); note_launches(1);
  int blocks = grid_blocks(t.nBodies * 8LL, 256);
  if (blocks > device_sms() * 16) blocks = device_sms() * 16;
  k_pair_slots<<<blocks, 256, 0, s>>>(worlds, t, ctr); note_launches(1);
}

// ------------------------------------------------------------------ box-box (collide.ts)

namespace box {

constexpr float SAT_EPS = 1.0e-6f;
constexpr float PLANE_EPS = 1.0e-5f;
constexpr float MERGE_SQ = 1.0e-6f;
constexpr int MAX_POLY = 16;
constexpr int AXIS_FACE_A = 0, AXIS_FACE_B = 1, AXIS_EDGE = 2;

struct OBB {
  V3 c, h, ax[3];
};
struct Sat {
  int type, ia, ib;
  float sep;
  V3 n;
  bool valid;
};

__device__ __forceinline__ OBB make_obb(float4 p, float4 q, float4 size) {
  OBB o;
  o.c = v3(p);
  o.h = V3{size.x * 0.5f, size.y * 0.5f, size.z * 0.5f};
  o.ax[0] = rotate(q, V3{1.f, 0.f, 0.f});
  o.ax[1] = rotate(q, V3{0.f, 1.f, 0.f});
  o.ax[2] = rotate(q, V3{0.f, 0.f, 1.f});
  return o;
}

__device__ __forceinline__ float absdot(V3 a, V3 b) { return fabsf(dot(a, b)); }

__device__ __forceinline__ V3 support_point(const OBB& b, V3 dir) {
  float sx = dot(dir, b.ax[0]) >= 0 ? 1.f : -1.f;
  float sy = dot(dir, b.ax[1]) >= 0 ? 1.f : -1.f;
  float sz = dot(dir, b.ax[2]) >= 0 ? 1.f : -1.f;
  V3 p = madd(b.c, b.ax[0], b.h.x * sx);
  p = madd(p, b.ax[1], b.h.y * sy);
  return madd(p, b.ax[2], b.h.z * sz);
}

__device__ __forceinline__ bool test_axis(const OBB& A, const OBB& B, V3 delta, V3 axis, int type, int ia, int ib, Sat& best) {
  float l2 = len2(axis);
  if (l2 < SAT_EPS) return true;
  float inv = 1.f / sqrtf(l2);
  V3 n = axis * inv;
  if (dot(n, delta) < 0) n = -n;
  float distance = fabsf(dot(delta, n));
  float rA = A.h.x * absdot(n, A.ax[0]) + A.h.y * absdot(n, A.ax[1]) + A.h.z * absdot(n, A.ax[2]);
  float rB = B.h.x * absdot(n, B.ax[0]) + B.h.y * absdot(n, B.ax[1]) + B.h.z * absdot(n, B.ax[2]);
  float sep = distance - (rA + rB);
  if (sep > 0) return false;
  if (!best.valid || sep > best.sep) {
    best.valid = true;
    best.type = type;
    best.ia = ia;
    best.ib = ib;
    best.sep = sep;
    best.n = n;
  }
  return true;
}

__device__ __forceinline__ void face_axes(const OBB& b, int i, V3& u, V3& v, float& eu, float& ev) {
  if (i == 0) { u = b.ax[1]; v = b.ax[2]; eu = b.h.y; ev = b.h.z; }
  else if (i == 1) { u = b.ax[0]; v = b.ax[2]; eu = b.h.x; ev = b.h.z; }
  else { u = b.ax[0]; v = b.ax[1]; eu = b.h.x; ev = b.h.y; }
}

__device__ __forceinline__ int clip_polygon(const V3* in, int nin, V3* out, V3 n, float off) {
  int nout = 0;
  if (nin == 0) return 0;
  V3 a = in[nin - 1];
  float da = dot(n, a) - off;
  for (int k = 0; k < nin; k++) {
    V3 b = in[k];
    float db = dot(n, b) - off;
    bool aIn = da <= PLANE_EPS, bIn = db <= PLANE_EPS;
    if (aIn != bIn) {
      float t = 0.f;
      float denom = da - db;
      if (fabsf(denom) > SAT_EPS) t = clampr(da / denom, 0.f, 1.f);
      if (nout < MAX_POLY) out[nout++] = madd(a, b - a, t);
    }
    if (bIn && nout < MAX_POLY) out[nout++] = b;
    a = b;
    da = db;
  }
  return nout;
}

// ContactBuilder: merges near-duplicate midpoints, at most 8 contacts, anchors body-local.
struct Builder {
  V3 mids[MAX_CONTACTS];
  int n;
  float4 pA, qA, pB, qB;
  uint32_t* feat;
  V3* rA;
  V3* rB;
  __device__ __forceinline__ void add(V3 xA, V3 xB, uint32_t feature) {
    V3 mid = (xA + xB) * 0.5f;
    for (int k = 0; k < n; k++)
      if (len2(mid - mids[k]) < MERGE_SQ) return;
    if (n >= MAX_CONTACTS) return;
    feat[n] = feature;
    rA[n] = rotateInv(qA, xA - v3(pA));
    rB[n] = rotateInv(qB, xB - v3(pB));
    mids[n] = mid;
    n++;
  }
};

__device__ __forceinline__ void support_edge(const OBB& b, int i, V3 dir, V3& e0, V3& e1) {
  int a1 = (i + 1) % 3, a2 = (i + 2) % 3;
  float s1 = dot(dir, b.ax[a1]) >= 0 ? 1.f : -1.f;
  float s2 = dot(dir, b.ax[a2]) >= 0 ? 1.f : -1.f;
  V3 c = madd(b.c, b.ax[a1], comp(b.h, a1) * s1);
  c = madd(c, b.ax[a2], comp(b.h, a2) * s2);
  V3 e = b.ax[i] * comp(b.h, i);
  e0 = c - e;
  e1 = c + e;
}

__device__ __forceinline__ void closest_segments(V3 p0, V3 p1, V3 q0, V3 q1, V3& xA, V3& xB) {
  V3 d1 = p1 - p0, d2 = q1 - q0, r = p0 - q0;
  float a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
  float s = 0.f, t = 0.f;
  if (a <= SAT_EPS && e <= SAT_EPS) {
    xA = p0;
    xB = q0;
    return;
  }
  if (a <= SAT_EPS) {
    t = clampr(f / e, 0.f, 1.f);
  } else {
    float c = dot(d1, r);
    if (e <= SAT_EPS) {
      s = clampr(-c / a, 0.f, 1.f);
    } else {
      float b = dot(d1, d2);
      float denom = a * e - b * b;
      if (fabsf(denom) > SAT_EPS) s = clampr((b * f - c * e) / denom, 0.f, 1.f);
      t = (b * s + f) / e;
      if (t < 0) {
        t = 0.f;
        s = clampr(-c / a, 0.f, 1.f);
      } else if (t > 1) {
        t = 1.f;
        s = clampr((b - c) / a, 0.f, 1.f);
      }
    }
  }
  xA = madd(p0, d1, s);
  xB = madd(q0, d2, t);
}

__device__ void face_manifold(Builder& bld, const OBB& A, const OBB& B, bool refIsA, int refAxis, V3 nAB) {
  const OBB& R = refIsA ? A : B;
  const OBB& I = refIsA ? B : A;
  V3 refOut = refIsA ? nAB : -nAB;
  float sgn = dot(refOut, R.ax[refAxis]) >= 0 ? 1.f : -1.f;
  V3 rn = R.ax[refAxis] * sgn;
  V3 rc = madd(R.c, rn, comp(R.h, refAxis));
  V3 ru, rv;
  float reu, rev;
  face_axes(R, refAxis, ru, rv, reu, rev);
  // incident face: most anti-parallel axis of the other box
  int incAxis = 0;
  float best = -FLT_MAX;
  for (int k = 0; k < 3; k++) {
    float d = absdot(I.ax[k], rn);
    if (d > best) {
      best = d;
      incAxis = k;
    }
  }
  float isg = dot(I.ax[incAxis], rn) > 0 ? -1.f : 1.f;
  V3 fn = I.ax[incAxis] * isg;
  V3 fc = madd(I.c, fn, comp(I.h, incAxis));
  V3 iu, iv;
  float ieu, iev;
  face_axes(I, incAxis, iu, iv, ieu, iev);
  V3 bufA[MAX_POLY], bufB[MAX_POLY];
  bufA[0] = madd(madd(fc, iu, 1.f * ieu), iv, 1.f * iev);
  bufA[1] = madd(madd(fc, iu, -1.f * ieu), iv, 1.f * iev);
  bufA[2] = madd(madd(fc, iu, -1.f * ieu), iv, -1.f * iev);
  bufA[3] = madd(madd(fc, iu, 1.f * ieu), iv, -1.f * iev);
  int np = 4;
  V3 planes[4] = {ru, -ru, rv, -rv};
  float ext[4] = {reu, reu, rev, rev};
  V3* in = bufA;
  V3* out = bufB;
  for (int k = 0; k < 4; k++) {
    np = clip_polygon(in, np, out, planes[k], dot(planes[k], rc) + ext[k]);
    if (np == 0) return;
    V3* t = in;
    in = out;
    out = t;
  }
  const uint32_t prefix = (uint32_t(refIsA ? AXIS_FACE_A : AXIS_FACE_B) << 24) | (uint32_t(refAxis & 0xff) << 16) |
                          (uint32_t(incAxis & 0xff) << 8);
  for (int k = 0; k < np && bld.n < MAX_CONTACTS; k++) {
    V3 pI = in[k];
    float distance = dot(pI - rc, rn);
    if (distance > PLANE_EPS) continue;
    V3 pR = madd(pI, rn, -distance);
    if (refIsA) bld.add(pR, pI, prefix | uint32_t(k & 0xff));
    else bld.add(pI, pR, prefix | uint32_t(k & 0xff));
  }
  if (bld.n == 0) bld.add(support_point(A, nAB), support_point(B, -nAB), prefix);
}

__device__ void edge_contact(Builder& bld, const OBB& A, const OBB& B, int axA, int axB, V3 nAB) {
  V3 a0, a1, b0, b1, xA, xB;
  support_edge(A, axA, nAB, a0, a1);
  support_edge(B, axB, -nAB, b0, b1);
  closest_segments(a0, a1, b0, b1, xA, xB);
  const uint32_t key = (uint32_t(AXIS_EDGE) << 24) | (uint32_t(axA & 0xff) << 8) | uint32_t(axB & 0xff);
  bld.add(xA, xB, key);
  if (bld.n == 0) bld.add(support_point(A, nAB), support_point(B, -nAB), key);
}

// SAT over the 15 axes (collide.ts:312-338 with the faceBias rule); false when separated.
__device__ __forceinline__ bool sat(float4 pA, float4 qA, float4 sA, float4 pB, float4 qB, float4 sB, bool faceBias, Sat& best) {
  OBB A = make_obb(pA, qA, sA), B = make_obb(pB, qB, sB);
  V3 delta = B.c - A.c;
  Sat bf{AXIS_FACE_A, 0, 0, -FLT_MAX, V3{0, 0, 0}, false};
  Sat be{AXIS_EDGE, 0, 0, -FLT_MAX, V3{0, 0, 0}, false};
  for (int i = 0; i < 3; i++)
    if (!test_axis(A, B, delta, A.ax[i], AXIS_FACE_A, i, -1, bf)) return false;
  for (int i = 0; i < 3; i++)
    if (!test_axis(A, B, delta, B.ax[i], AXIS_FACE_B, -1, i, bf)) return false;
#pragma unroll 1
  for (int i = 0; i < 3; i++)
#pragma unroll 1
    for (int j = 0; j < 3; j++)
      if (!test_axis(A, B, delta, cross(A.ax[i], B.ax[j]), AXIS_EDGE, i, j, be)) return false;
  if (!bf.valid) return false;
  best = bf;
  if (be.valid) {
    const float rel = 0.95f, absT = 0.01f;
    bool edgeWins = !faceBias ? rel * be.sep > bf.sep + absT : be.sep > rel * bf.sep + absT;
    if (edgeWins) best = be;
  }
  return true;
}

// Contacts for the axis SAT chose (collide.ts:340-344); basis rows n (B to A), t1, t2.
__device__ __forceinline__ int contacts(Builder& bld, float4 pA, float4 qA, float4 sA, float4 pB, float4 qB, float4 sB, const Sat& best,
                                        M33& basis) {
  OBB A = make_obb(pA, qA, sA), B = make_obb(pB, qB, sB);
  basis = orthonormal(-best.n);
  if (best.type == AXIS_EDGE) edge_contact(bld, A, B, best.ia, best.ib, best.n);
  else if (best.type == AXIS_FACE_A) face_manifold(bld, A, B, true, best.ia, best.n);
  else face_manifold(bld, A, B, false, best.ib, best.n);
  return bld.n;
}

}  // namespace box

// ------------------------------------------------------------------ generic (cpuContacts3D.js)

namespace gen {

// Box faces (vertex indices) and outward normals, cpuContacts3D.js:26-41; vertex i has local
// coordinate size/2 * (bit k of i ? +1 : -1) on axis k.
__constant__ int kFaces[6][4] = {{1, 3, 7, 5}, {0, 4, 6, 2}, {2, 6, 7, 3}, {0, 1, 5, 4}, {4, 5, 7, 6}, {0, 2, 3, 1}};
__constant__ float kNormals[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
// Unique edges in the order geometry3D discovers them walking the faces (cpuContacts3D.js:73-86).
__constant__ int kEdges[12][2] = {{1, 3}, {3, 7}, {7, 5}, {5, 1}, {0, 4}, {4, 6}, {6, 2}, {2, 0}, {6, 7}, {3, 2}, {0, 1}, {5, 4}};

struct BoxGeo {
  V3 v[8];
  V3 n[6];
};

__device__ __forceinline__ float hyp(V3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ V3 unitv(V3 a) {
  float h = hyp(a);
  float s = 1.f / (h != 0.f ? h : 1.f);
  return a * s;
}

__device__ __forceinline__ void box_geo(BoxGeo& g, float4 p, float4 q, float4 size) {
  const V3 c = v3(p);
#pragma unroll
  for (int i = 0; i < 8; i++) {
    V3 l{(size.x / 2) * ((i & 1) ? 1.f : -1.f), (size.y / 2) * ((i & 2) ? 1.f : -1.f), (size.z / 2) * ((i & 4) ? 1.f : -1.f)};
    g.v[i] = c + rotate(q, l);
  }
#pragma unroll
  for (int f = 0; f < 6; f++) g.n[f] = rotate(q, V3{kNormals[f][0], kNormals[f][1], kNormals[f][2]});
}

// first vertex of greatest dot(v, n) (the running best is kept by value, not by index)
__device__ __forceinline__ V3 box_support(const BoxGeo& g, V3 n) {
  V3 best = g.v[0];
  float bestDot = dot(g.v[0], n);
#pragma unroll
  for (int i = 1; i < 8; i++) {
    const float d = dot(g.v[i], n);
    if (d > bestDot) {
      best = g.v[i];
      bestDot = d;
    }
  }
  return best;
}

// A round body's spine (cpuContacts3D.js:44-51): a capsule's segment along its local Y, of
// half-length height / 2 - r; a sphere's is its centre (both ends at a zero offset).
__device__ __forceinline__ void spine_of(float4 p, float4 q, float4 size, int shape, V3& s0, V3& s1) {
  const float r = size.x / 2;
  const float half = shape == SHAPE_CAPSULE ? fmaxf(0.f, size.y / 2 - r) : 0.f;
  const V3 c = v3(p);
  s0 = c + rotate(q, V3{0.f, -half, 0.f});
  s1 = c + rotate(q, V3{0.f, half, 0.f});
}

// support of a round body: the first spine end of greatest dot(v, n), pushed out by r
__device__ __forceinline__ V3 round_support(V3 s0, V3 s1, float r, V3 n) {
  const V3 p = dot(s1, n) > dot(s0, n) ? s1 : s0;
  return madd(p, n, r);
}

__device__ __forceinline__ void closest_seg(V3 p, V3 q, V3 r, V3 s, V3& oa, V3& ob) {
  V3 d1 = q - p, d2 = s - r, w = p - r;
  float a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, w);
  float u = 0.f, v = 0.f;
  if (a < 1e-16f) v = e > 1e-16f ? fmaxf(0.f, fminf(1.f, f / e)) : 0.f;
  else {
    float c = dot(d1, w);
    if (e < 1e-16f) u = fmaxf(0.f, fminf(1.f, -c / a));
    else {
      float b = dot(d1, d2), den = a * e - b * b;
      u = den > 1e-12f * a * e ? fmaxf(0.f, fminf(1.f, (b * f - c * e) / den)) : 0.f;
      v = (b * u + f) / e;
      if (v < 0) {
        v = 0.f;
        u = fmaxf(0.f, fminf(1.f, -c / a));
      } else if (v > 1) {
        v = 1.f;
        u = fmaxf(0.f, fminf(1.f, (b - c) / a));
      }
    }
  }
  oa = madd(p, d1, u);
  ob = madd(r, d2, v);
}

__device__ __forceinline__ V3 closest_triangle(V3 p, V3 a, V3 b, V3 c) {
  V3 ab = b - a, ac = c - a, ap = p - a;
  float d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0 && d2 <= 0) return a;
  V3 bp = p - b;
  float d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0 && d4 <= d3) return b;
  float vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) return madd(a, ab, d1 / (d1 - d3));
  V3 cp = p - c;
  float d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0 && d5 <= d6) return c;
  float vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) return madd(a, ac, d2 / (d2 - d6));
  float va = d3 * d6 - d5 * d4;
  if (va <= 0 && d4 - d3 >= 0 && d5 - d6 >= 0) return madd(b, c - b, (d4 - d3) / (d4 - d3 + d5 - d6));
  float den = 1.f / (va + vb + vc);
  return a + (ab * (vb * den) + ac * (vc * den));
}

__device__ __forceinline__ V3 closest_surface(const BoxGeo& g, V3 p) {
  float dist = INFINITY;
  V3 best = p;
  for (int f = 0; f < 6; f++)
    for (int i = 1; i < 3; i++) {
      V3 q = closest_triangle(p, g.v[kFaces[f][0]], g.v[kFaces[f][i]], g.v[kFaces[f][i + 1]]);
      V3 d = p - q;
      float dd = dot(d, d);
      if (dd < dist) {
        best = q;
        dist = dd;
      }
    }
  return best;
}

// At least one body is round, a sphere or a capsule (BOTH_ROUND: both are, and the box code
// compiles away). Returns the contact count (0 or 1).
template <bool BOTH_ROUND>
__device__ int collide(float4 pA, float4 qA, float4 sA, int shA, float4 pB, float4 qB, float4 sB, int shB, M33& basis,
                       V3& rA, V3& rB) {
  const bool roundA = BOTH_ROUND || shA != SHAPE_BOX, roundB = BOTH_ROUND || shB != SHAPE_BOX;
  BoxGeo box;
  const V3 cA = v3(pA), cB = v3(pB);
  V3 spA0{0.f, 0.f, 0.f}, spA1{0.f, 0.f, 0.f}, spB0{0.f, 0.f, 0.f}, spB1{0.f, 0.f, 0.f};
  if (roundA) spine_of(pA, qA, sA, shA, spA0, spA1);
  if (roundB) spine_of(pB, qB, sB, shB, spB0, spB1);
  const float radA = sA.x / 2, radB = sB.x / 2;
  if (!roundA) box_geo(box, pA, qA, sA);
  else if (!roundB) box_geo(box, pB, qB, sB);
  float gap = -INFINITY;
  V3 n{0.f, 0.f, 1.f};
  auto supA = [&](V3 d) { return roundA ? round_support(spA0, spA1, radA, d) : box_support(box, d); };
  auto supB = [&](V3 d) { return roundB ? round_support(spB0, spB1, radB, d) : box_support(box, d); };
  auto consider = [&](V3 axis) {
    if (hyp(axis) < 1e-9f) return;
    V3 v = unitv(axis);
    V3 nv = v * -1.f;
    float g = dot(supA(nv) - supB(v), v);
    float rev = dot(supB(nv) - supA(v), v);
    if (rev > g) {
      g = rev;
      v = v * -1.f;
    }
    if (g > gap + 1e-7f) {
      gap = g;
      n = v;
    }
  };
  // The gap only grows, and a positive final gap means no contact: stop at the first positive one.
  if (!roundA)
    for (int f = 0; f < 6; f++) {
      consider(box.n[f]);
      if (gap > 0) return 0;
    }
  if (!roundB)
    for (int f = 0; f < 6; f++) {
      consider(box.n[f]);
      if (gap > 0) return 0;
    }
  if (roundA && roundB) {
    V3 pa, pb;
    closest_seg(spA0, spA1, spB0, spB1, pa, pb);
    consider(pa - pb);
    if (gap > 0) return 0;
  }
  // [round, poly] = [A, B] then [B, A]
  for (int k = 0; k < 2; k++) {
    const bool roundIsA = k == 0;
    const bool isRound = roundIsA ? roundA : roundB;
    const bool polyIsBox = roundIsA ? !roundB : !roundA;
    if (!isRound || !polyIsBox) continue;
    const V3 s0 = roundIsA ? spA0 : spB0, s1 = roundIsA ? spA1 : spB1;
    const V3 e = s1 - s0;
    const float ee = dot(e, e);
    for (int i = 0; i < 8; i++) {  // vertex to its nearest spine point (cpuContacts3D.js nearest)
      V3 ap = box.v[i] - s0;
      float t = dot(ap, e) / (ee != 0.f ? ee : 1.f);
      t = fmaxf(0.f, fminf(1.f, t));
      consider(box.v[i] - madd(s0, e, t));
      if (gap > 0) return 0;
    }
    for (int i = 0; i < 12; i++) {
      V3 pa, pb;
      closest_seg(s0, s1, box.v[kEdges[i][0]], box.v[kEdges[i][1]], pa, pb);
      consider(pa - pb);
      if (gap > 0) return 0;
    }
  }
  if (gap == -INFINITY) consider(cA - cB);
  if (gap > 0) return 0;
  if (gap == -INFINITY) n = V3{0.f, 0.f, 1.f};
  V3 axisT = fabsf(n.x) < 0.7f ? V3{1.f, 0.f, 0.f} : V3{0.f, 1.f, 0.f};
  V3 tangent = unitv(cross(n, axisT));
  basis = M33{n, tangent, cross(n, tangent)};
  V3 xa, xb;
  if (roundA && roundB) {
    V3 pa, pb;
    closest_seg(spA0, spA1, spB0, spB1, pa, pb);
    xa = madd(pa, n, -radA);
    xb = madd(pb, n, radB);
  } else if (roundA) {
    xa = round_support(spA0, spA1, radA, n * -1.f);
    xb = closest_surface(box, xa);
  } else {
    xb = round_support(spB0, spB1, radB, n);
    xa = closest_surface(box, xb);
  }
  rA = rotateInv(qA, xa - cA);
  rB = rotateInv(qB, xb - cB);
  return 1;
}

}  // namespace gen

// ------------------------------------------------------------------ narrowphase kernel


// Warm start and store the contacts of pair p (cpuPhysics3D.js:108-145): match the previous
// step's contacts of the same pair by feature, keep sticking anchors (not for rolling pairs),
// C0 = basis (xA - xB) + margin, decayed lambda, clamped penalty, mass-penalty floor.
__device__ __forceinline__ void finish_pair(const BodyPtrs& bd, const WorldDev& W, const Tick& t, int w, PairPtrs& cur,
                                            int p, uint2 key, float4 pA, float4 qA, float4 sA, float4 pB, float4 qB, float4 sB,
                                            bool rolling, int n, const M33& basis, const uint32_t* feat, const V3* rA, const V3* rB) {
  const float friction = sqrtf(sA.w * sB.w);
  cur.count[p] = n;
  cur.basis[3 * p + 0] = f4(basis.r0, friction);
  cur.basis[3 * p + 1] = f4(basis.r1, W.alpha);  // the world's constants the solver kernels need
  cur.basis[3 * p + 2] = f4(basis.r2, W.betaLin);
  if (n == 0) return;
  // the world's previous pairs: its region in the buffer it holds its last state in
  const int pw = t.which[w];
  const int nprev = t.pairN[pw * t.maxWorlds + w];
  const int pp = nprev > 0 ? find_pair(cur.pair, pw * t.slotStride + W.pairOff, nprev, key) : -1;
  const int pn = pp >= 0 ? cur.count[pp] : 0;
  const float ag = W.alpha * W.gamma;
  float penFloor = 0.f;
  if (W.flags & FLAG_MASS_PENALTY) {
    const float mA = bd.mass[key.x].x, mB = bd.mass[key.y].x;
    const float mass = fminr(mA > 0.f ? mA : INFINITY, mB > 0.f ? mB : INFINITY);
    penFloor = fmaxf(PENALTY_MIN, fminf(PENALTY_MAX, mass / (W.dt * W.dt)));
  }
#pragma unroll 1
  for (int k = 0; k < n; k++) {
    V3 ra = rA[k], rb = rB[k];
    V3 pen{0.f, 0.f, 0.f}, lam{0.f, 0.f, 0.f};
    bool stick = false;
#pragma unroll 1
    for (int q = 0; q < pn; q++) {
      const float4* o = cur.ct + (size_t(pp) * MAX_CONTACTS + q) * 4;
      const float4 o0 = o[0];
      const uint32_t of = __float_as_uint(o0.w);
      if ((of & ~STICK_BIT) != feat[k]) continue;
      const float4 o1 = o[1], o2 = o[2], o3 = o[3];
      stick = (of & STICK_BIT) != 0;
      if (stick && !rolling) {
        ra = v3(o0);
        rb = v3(o1);
      }
      pen = v3(o2);
      lam = v3(o3);
      break;
    }
    const V3 d = xform(v3(pA), qA, ra) - xform(v3(pB), qB, rb);
    V3 C0 = mulv(basis, d);
    C0.x += COLLISION_MARGIN;
    lam = V3{lam.x * ag, lam.y * ag, lam.z * ag};
    pen = V3{clampr(pen.x * W.gamma, PENALTY_MIN, PENALTY_MAX), clampr(pen.y * W.gamma, PENALTY_MIN, PENALTY_MAX),
             clampr(pen.z * W.gamma, PENALTY_MIN, PENALTY_MAX)};
    if (W.flags & FLAG_MASS_PENALTY) pen.x = fmaxf(pen.x, penFloor);
    float4* o = cur.ct + (size_t(p) * MAX_CONTACTS + k) * 4;
    o[0] = f4(ra, __uint_as_float(feat[k] | (stick ? STICK_BIT : 0u)));
    o[1] = f4(rb, C0.x);
    o[2] = f4(pen, C0.y);
    o[3] = f4(lam, C0.z);
  }
}

// warp-aggregated append of `p` to list (count in *n)
__device__ __forceinline__ void append(int* list, int* n, int p, bool take) {
  const unsigned m = __ballot_sync(__activemask(), take);
  if (!take) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(n, __popc(m));
  base = __shfl_sync(m, base, leader);
  list[base + __popc(m & ((1u << lane) - 1))] = p;
}

// A sphere and a box clearly apart: the distance from the sphere's centre to the box exceeds its
// radius by far more than any rounding of the separating-axis search (1e-3 plus 1e-5 of the
// coordinates' size), so that search would end with a positive gap and no contact: skip it.
__device__ __forceinline__ bool sphere_box_apart(float4 pA, float4 qA, float4 sA, int shA, float4 pB, float4 qB, float4 sB,
                                                 int shB) {
  if (shA == SHAPE_CAPSULE || shB == SHAPE_CAPSULE) return false;  // capsules always run the search
  const bool sphereA = shA == SHAPE_SPHERE;
  const float4 pc = sphereA ? pA : pB, pbx = sphereA ? pB : pA, qbx = sphereA ? qB : qA, sbx = sphereA ? sB : sA;
  const float r = (sphereA ? sA : sB).x * 0.5f;
  const V3 l = rotateInv(qbx, v3(pc) - v3(pbx));
  const V3 h{sbx.x * 0.5f, sbx.y * 0.5f, sbx.z * 0.5f};
  const V3 o{fmaxf(fabsf(l.x) - h.x, 0.f), fmaxf(fabsf(l.y) - h.y, 0.f), fmaxf(fabsf(l.z) - h.z, 0.f)};
  const float margin = 1e-3f + 1e-5f * (fabsf(pc.x) + fabsf(pc.y) + fabsf(pc.z) + fabsf(pbx.x) + fabsf(pbx.y) + fabsf(pbx.z));
  const float reach = r + margin;
  return dot(o, o) > reach * reach;
}

// What finish_pair stores for a pair without contacts.
__device__ __forceinline__ void finish_empty(const WorldDev& W, PairPtrs& cur, int p, float4 sA, float4 sB) {
  cur.count[p] = 0;
  cur.basis[3 * p + 0] = make_float4(0.f, 0.f, 0.f, sqrtf(sA.w * sB.w));
  cur.basis[3 * p + 1] = make_float4(0.f, 0.f, 0.f, W.alpha);
  cur.basis[3 * p + 2] = make_float4(0.f, 0.f, 0.f, W.betaLin);
}

// Pass 1: box-box pairs run SAT; separated ones are finished here (no contacts), the others are
// queued with their chosen axis. Pairs with a sphere or a capsule are queued for the generic path,
// except sphere-box pairs clearly apart (sphere_box_apart), finished here too: the generic kernel
// then gets only pairs that run the full search, so its warps do not idle on finished lanes.
__global__ void __launch_bounds__(256) k_np_classify(BodyPtrs bd, const WorldDev* __restrict__ worlds, PairPtrs cur, Tick t,
                                                     const Counters* __restrict__ ctr, NarrowScratch ns) {
  const int np = ctr->activePairs;
  for (int base = blockIdx.x * blockDim.x; base < np; base += gridDim.x * blockDim.x) {
    const int q = base + threadIdx.x;
    const int p = q < np ? t.pairs[q] : 0;
    bool boxHit = false, sphere = false, bothRound = false;
    if (q < np) {
      const uint2 key = cur.pair[p];
      const int a = int(key.x), b = int(key.y);
      const int shA = bd.meta[a].y, shB = bd.meta[b].y;
      if (shA != SHAPE_BOX || shB != SHAPE_BOX) {  // a sphere or a capsule: the generic path
        sphere = true;
        bothRound = shA != SHAPE_BOX && shB != SHAPE_BOX;
        if (!bothRound) {
          const float4 sA = bd.size[a], sB = bd.size[b];
          if (sphere_box_apart(bd.pos(a), bd.rot(a), sA, shA, bd.pos(b), bd.rot(b), sB, shB)) {
            finish_empty(worlds[bd.meta[a].x], cur, p, sA, sB);
            sphere = false;
          }
        }
      } else {
        const WorldDev& W = worlds[bd.meta[a].x];
        box::Sat best;
        if (box::sat(bd.pos(a), bd.rot(a), bd.size[a], bd.pos(b), bd.rot(b), bd.size[b], (W.flags & FLAG_FACE_BIAS) != 0, best)) {
          boxHit = true;
          ns.sat[q] = make_float4(best.n.x, best.n.y, best.n.z, __int_as_float(best.type | ((best.ia & 0xff) << 8) | ((best.ib & 0xff) << 16)));
        } else {
          cur.count[p] = 0;
        }
      }
    }
    append(ns.boxList, &ns.ctr[0], q, boxHit);
    append(ns.sphereList, &ns.ctr[1], p, sphere && !bothRound);
    append(ns.sphere2List, &ns.ctr[2], p, sphere && bothRound);
  }
}

// Pass 2a: contacts of box-box pairs that SAT found overlapping.
#ifndef AVBD_NP_BOX_MINB
#define AVBD_NP_BOX_MINB 3  // blocks per SM the register allocation must allow
#endif
__global__ void __launch_bounds__(128, AVBD_NP_BOX_MINB) k_np_box(BodyPtrs bd, const WorldDev* __restrict__ worlds, PairPtrs cur, Tick t,
                                                NarrowScratch ns) {
  const int n = ns.ctr[0];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int q = ns.boxList[k];
    const int p = t.pairs[q];
    const uint2 key = cur.pair[p];
    const int a = int(key.x), b = int(key.y);
    const float4 pA = bd.pos(a), qA = bd.rot(a), sA = bd.size[a];
    const float4 pB = bd.pos(b), qB = bd.rot(b), sB = bd.size[b];
    const WorldDev& W = worlds[bd.meta[a].x];
    const float4 sr = ns.sat[q];
    const int code = __float_as_int(sr.w);
    box::Sat best;
    best.type = code & 0xff;
    best.ia = (code >> 8) & 0xff;
    best.ib = (code >> 16) & 0xff;
    best.n = v3(sr);
    best.valid = true;
    best.sep = 0.f;
    uint32_t feat[MAX_CONTACTS];
    V3 rA[MAX_CONTACTS], rB[MAX_CONTACTS];
    box::Builder bld;
    bld.n = 0;
    bld.pA = pA; bld.qA = qA; bld.pB = pB; bld.qB = qB;
    bld.feat = feat; bld.rA = rA; bld.rB = rB;
    M33 basis;
    const int nc = box::contacts(bld, pA, qA, sA, pB, qB, sB, best, basis);
    finish_pair(bd, W, t, bd.meta[a].x, cur, p, key, pA, qA, sA, pB, qB, sB, false, nc, basis, feat, rA, rB);
  }
}

// Pass 2b: pairs with a sphere (generic support-function SAT, one contact): sphere-box pairs,
// then sphere-sphere pairs in a lighter instance of the same code.
#ifndef AVBD_NP_SPHERE_MINB
#define AVBD_NP_SPHERE_MINB 5  // blocks per SM the register allocation must allow
#endif
template <bool BOTH_ROUND>
__global__ void __launch_bounds__(128, AVBD_NP_SPHERE_MINB) k_np_sphere(BodyPtrs bd, const WorldDev* __restrict__ worlds, PairPtrs cur, Tick t,
                                                   NarrowScratch ns) {
  const int n = ns.ctr[BOTH_ROUND ? 2 : 1];
  const int* list = BOTH_ROUND ? ns.sphere2List : ns.sphereList;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int p = list[k];
    const uint2 key = cur.pair[p];
    const int a = int(key.x), b = int(key.y);
    const float4 pA = bd.pos(a), qA = bd.rot(a), sA = bd.size[a];
    const float4 pB = bd.pos(b), qB = bd.rot(b), sB = bd.size[b];
    const int shA = bd.meta[a].y, shB = bd.meta[b].y;
    const WorldDev& W = worlds[bd.meta[a].x];
    M33 basis{V3{0, 0, 0}, V3{0, 0, 0}, V3{0, 0, 0}};
    uint32_t feat[1] = {1u};  // feature i + 1
    V3 rA[1], rB[1];
    const int nc = gen::collide<BOTH_ROUND>(pA, qA, sA, shA, pB, qB, sB, shB, basis, rA[0], rB[0]);
    finish_pair(bd, W, t, bd.meta[a].x, cur, p, key, pA, qA, sA, pB, qB, sB, true, nc, basis, feat, rA, rB);
  }
}

void launch_narrowphase(const BodyPtrs& b, const WorldDev* worlds, Tick t, PairPtrs P, NarrowScratch ns, const Counters* ctr,
                        int pairBudget, cudaStream_t s) {
  cudaMemsetAsync(ns.ctr, 0, 3 * sizeof(int), s);
  if (t.nActive == 0) return;
  int blocks = grid_blocks(pairBudget, 256);
  if (blocks > device_sms() * 16) blocks = device_sms() * 16;
  k_np_classify<<<blocks, 256, 0, s>>>(b, worlds, P, t, ctr, ns); note_launches(1);
  k_np_box<<<device_sms() * 16, 128, 0, s>>>(b, worlds, P, t, ns); note_launches(1);
  k_np_sphere<false><<<device_sms() * 16, 128, 0, s>>>(b, worlds, P, t, ns); note_launches(1);
  k_np_sphere<true><<<device_sms() * 16, 128, 0, s>>>(b, worlds, P, t, ns); note_launches(1);
}

}  // namespace avbd
