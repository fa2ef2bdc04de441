// Island sleeping after the step (src/native/cpu/sleeping.js CpuSleeping.after / wake), for the
// worlds of the tick with FLAG_SLEEP.
//
// Islands are the connected components of the dynamic bodies under every live constraint: unbroken
// joints and springs, ignore pairs, manifolds with contacts. A constraint to a static body, or a
// joint to the world, marks the dynamic body as support. An island is stable when it holds a
// support and each of its bodies allows sleep and moves no faster than the threshold, |(v, w)|
// as the square root of the left-to-right sum of the six squares. Each dynamic body's quiet time
// grows by dt while its island is stable and resets to 0 otherwise; at the delay the body sleeps
// with zero velocity. Finally a constraint joining a sleeping and an awake dynamic body wakes the
// whole world (every body awake, every quiet time 0).
//
// The components come from a concurrent union-find over global body indices: a root is only ever
// linked below a smaller root by compare-and-swap, and path halving only moves a pointer to an
// ancestor, so parent[x] <= x always and every find ends. The partition (all the outcome depends
// on) does not depend on the order of the unions. Kernels, each over the tick's lists:
//   k_sleep_init   parent = self, flags = 0 (bodies)
//   k_sleep_edges  mode 0: supports and unions; mode 1: mixed sleeping/awake edges -> wake[world]
//   k_sleep_roots  parent = root (bodies)
//   k_sleep_reduce island flags at the root: supported, unstable (dynamic bodies)
//   k_sleep_time   quiet time, falling asleep (dynamic bodies)
//   k_sleep_apply  wake the worlds flagged by mode 1 (bodies)
#include "engine.cuh"

namespace avbd {
namespace {

constexpr int F_SUPPORT = 1;      // the body touches a static body or hangs from the world
constexpr int F_ROOT_SUP = 2;     // (at a root) the island holds a support
constexpr int F_ROOT_UNSTABLE = 4;  // (at a root) some body of the island moves or may not sleep
constexpr int UNION_TRIES = 1 << 16;

__device__ __forceinline__ bool sleep_world(const BodyPtrs& bd, const WorldDev* worlds, int i) {
  return (worlds[bd.meta[i].x].flags & FLAG_SLEEP) != 0;
}

__device__ __forceinline__ int uf_find(int* parent, int x) {
  volatile int* par = parent;
  int p = par[x];
  while (p != x) {
    const int gp = par[p];
    if (gp != p) par[x] = gp;  // halving: x now points at an ancestor
    x = p;
    p = gp;
  }
  return x;
}

__device__ __forceinline__ void uf_union(int* parent, int a, int b, int* err) {
  for (int tries = 0; tries < UNION_TRIES; tries++) {
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    if (a == b) return;
    const int hi = a > b ? a : b, lo = a > b ? b : a;
    if (atomicCAS(&parent[hi], hi, lo) == hi) return;
  }
  atomicAdd(err, 1);
}

// The constraint q of the tick's edge list: joints, then active pair slots, then the no-collide
// list's ignore pairs. Returns false when q is not a live constraint of a sleeping world.
__device__ __forceinline__ bool sleep_edge(const BodyPtrs& bd, const WorldDev* worlds, const JointPtrs& J, const PairPtrs& P,
                                           const NoCollide& nc, const Tick& t, int np, int q, int& a, int& b, int& w) {
  if (q < t.nJoints) {
    const int j = t.joints[q];
    if (J.broken[j]) return false;
    const int2 ab = J.ab[j];
    a = ab.x;
    b = ab.y;
  } else if (q < t.nJoints + np) {
    const int p = t.pairs[q - t.nJoints];
    if (P.count[p] == 0) return false;
    const uint2 pr = P.pair[p];
    a = int(pr.x);
    b = int(pr.y);
  } else {
    const int e = q - t.nJoints - np;
    if (nc.jid[e] != -1) return false;  // a joint's own entry (the joint is the edge)
    const unsigned long long key = nc.keys[e];
    a = int(key >> 32);
    b = int(key & 0xffffffffull);
    if (t.wactive[bd.meta[b].x] < 0) return false;  // world not stepped this tick
  }
  if (trigger_pair(t.triggerBits, a, b)) return false;  // sleeping.js:54
  w = bd.meta[b].x;
  return (worlds[w].flags & FLAG_SLEEP) != 0;
}

__global__ void k_sleep_init(BodyPtrs bd, const WorldDev* __restrict__ worlds, Tick t, SleepBufs sb) {
  if (tick_held(t.ctl)) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += gridDim.x * blockDim.x) {
    const int i = t.bodies[k];
    if (!sleep_world(bd, worlds, i)) continue;
    sb.parent[i] = i;
    sb.flags[i] = 0;
  }
}

__global__ void k_sleep_edges(BodyPtrs bd, const WorldDev* __restrict__ worlds, JointPtrs J, PairPtrs P, NoCollide nc, Tick t,
                              const Counters* __restrict__ ctr, SleepBufs sb, int mode) {
  if (tick_held(t.ctl)) return;
  const int np = ctr->activePairs;
  const int total = t.nJoints + np + nc.n;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    int a, b, w;
    if (!sleep_edge(bd, worlds, J, P, nc, t, np, q, a, b, w)) continue;
    const bool dynB = bd.mass[b].x > 0.f;
    if (mode == 0) {
      if (a < 0 || !(bd.mass[a].x > 0.f)) atomicOr(&sb.flags[b], F_SUPPORT);
      else if (!dynB) atomicOr(&sb.flags[a], F_SUPPORT);
      else uf_union(sb.parent, a, b, sb.err);
    } else if (a >= 0 && bd.mass[a].x > 0.f && dynB &&
               ((bd.sleep[a] & SLEEP_ASLEEP) != 0) != ((bd.sleep[b] & SLEEP_ASLEEP) != 0)) {
      sb.wake[w] = 1;
    }
  }
}

__global__ void k_sleep_roots(BodyPtrs bd, const WorldDev* __restrict__ worlds, Tick t, SleepBufs sb) {
  if (tick_held(t.ctl)) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += gridDim.x * blockDim.x) {
    const int i = t.bodies[k];
    if (!sleep_world(bd, worlds, i)) continue;
    sb.parent[i] = uf_find(sb.parent, i);
  }
}

__device__ __forceinline__ float sleep_speed(float4 v, float4 w) {
  return sqrtf(((((v.x * v.x + v.y * v.y) + v.z * v.z) + w.x * w.x) + w.y * w.y) + w.z * w.z);
}

__global__ void k_sleep_reduce(BodyPtrs bd, const WorldDev* __restrict__ worlds, Tick t, SleepBufs sb) {
  if (tick_held(t.ctl)) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += gridDim.x * blockDim.x) {
    const int i = t.bodies[k];
    const WorldDev& W = worlds[bd.meta[i].x];
    if (!(W.flags & FLAG_SLEEP) || !(bd.mass[i].x > 0.f)) continue;
    const int r = sb.parent[i];
    if (sb.flags[i] & F_SUPPORT) atomicOr(&sb.flags[r], F_ROOT_SUP);
    const bool quiet = (bd.sleep[i] & SLEEP_ALLOW) && sleep_speed(bd.vel[i], bd.ang[i]) <= W.sleepSpeed;
    if (!quiet) atomicOr(&sb.flags[r], F_ROOT_UNSTABLE);
  }
}

__global__ void k_sleep_time(BodyPtrs bd, const WorldDev* __restrict__ worlds, Tick t, SleepBufs sb) {
  if (tick_held(t.ctl)) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += gridDim.x * blockDim.x) {
    const int i = t.bodies[k];
    const WorldDev& W = worlds[bd.meta[i].x];
    if (!(W.flags & FLAG_SLEEP) || !(bd.mass[i].x > 0.f)) continue;
    const int f = sb.flags[sb.parent[i]];
    const bool stable = (f & F_ROOT_SUP) && !(f & F_ROOT_UNSTABLE);
    const float time = stable ? bd.sleepTime[i] + W.dt : 0.f;
    bd.sleepTime[i] = time;
    if (time >= W.sleepDelay) {
      bd.sleep[i] |= SLEEP_ASLEEP;
      const float4 v = bd.vel[i], w = bd.ang[i];
      bd.vel[i] = make_float4(0.f, 0.f, 0.f, v.w);
      bd.ang[i] = make_float4(0.f, 0.f, 0.f, w.w);
    }
  }
}

__global__ void k_sleep_apply(BodyPtrs bd, const WorldDev* __restrict__ worlds, Tick t, SleepBufs sb) {
  if (tick_held(t.ctl)) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += gridDim.x * blockDim.x) {
    const int i = t.bodies[k];
    const int w = bd.meta[i].x;
    if (!(worlds[w].flags & FLAG_SLEEP) || !sb.wake[w]) continue;
    bd.sleep[i] &= ~SLEEP_ASLEEP;
    bd.sleepTime[i] = 0.f;
  }
}

__global__ void k_sleep_wake(BodyPtrs bd, int off, int n, const TickCtl* ctl) {
  if (tick_held(ctl)) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    bd.sleep[off + k] &= ~SLEEP_ASLEEP;
    bd.sleepTime[off + k] = 0.f;
  }
}

}  // namespace

void launch_sleep(const BodyPtrs& b, const WorldDev* worlds, JointPtrs J, PairPtrs P, NoCollide nc, Tick t,
                  const Counters* ctr, int pairBudget, SleepBufs sb, int maxWorlds, cudaStream_t s) {
  if (t.nBodies == 0) return;
  const int bblocks = grid_blocks(t.nBodies, 256);
  int eblocks = grid_blocks((long long)t.nJoints + pairBudget + nc.n, 256);
  if (eblocks > device_sms() * 8) eblocks = device_sms() * 8;
  if (eblocks < 1) eblocks = 1;
  cudaMemsetAsync(sb.wake, 0, sizeof(int) * size_t(maxWorlds), s);
  k_sleep_init<<<bblocks, 256, 0, s>>>(b, worlds, t, sb);
  k_sleep_edges<<<eblocks, 256, 0, s>>>(b, worlds, J, P, nc, t, ctr, sb, 0);
  k_sleep_roots<<<bblocks, 256, 0, s>>>(b, worlds, t, sb);
  k_sleep_reduce<<<bblocks, 256, 0, s>>>(b, worlds, t, sb);
  k_sleep_time<<<bblocks, 256, 0, s>>>(b, worlds, t, sb);
  k_sleep_edges<<<eblocks, 256, 0, s>>>(b, worlds, J, P, nc, t, ctr, sb, 1);
  k_sleep_apply<<<bblocks, 256, 0, s>>>(b, worlds, t, sb);
  note_launches(7);
}

void launch_sleep_wake(const BodyPtrs& b, int off, int n, const TickCtl* ctl, cudaStream_t s) {
  if (n <= 0) return;
  k_sleep_wake<<<grid_blocks(n, 256), 256, 0, s>>>(b, off, n, ctl);
  note_launches(1);
}

}  // namespace avbd
