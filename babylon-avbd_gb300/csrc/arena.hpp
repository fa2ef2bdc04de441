// The world arena: device arrays holding many worlds as self-contained segments, and the host
// logic that adds, steps, evicts and restores them. Shared by the world/batch ABI (engine.cu)
// and the server ABI (server.cu).
//
// An Arena holds worlds as self-contained segments of one set of device arrays (engine.cuh):
// a body range, a joint range and a pair-slot region per world, with range allocators on the
// host. A tick advances any subset of the resident worlds by one step, in one launch sequence
// over the bodies, joints and pairs of those worlds only:
//
//   collision   active lists -> grid -> pair count / scan / write into each world's region ->
//               narrowphase (SAT classification, per-type contacts) with warm-start matching
//   topology    constraint lists (CSR, sorted) -> Jones-Plassmann colouring -> buckets -> items
//   [one counter readback: pair-region overflow, colour sizes, work items]
//   solve       joint warm start -> body warm start -> iterations x (colours + dual) -> velocities
//
// Everything before the readback writes only the buffers the tick is filling (pairs, contacts,
// colours, lists); each world's previous state stays in the buffer named by which[w] until the
// tick completes. When a world's pair region overflows, the region grows and the tick re-runs
// from the same state, so capacities never alter a result. A world evolves the same way alone,
// in a batch, or parked between requests of a server, and can be evicted to host memory and
// restored exactly. The reference's counterpart is one WebGPU submission per world and step
// (src/gpu/gpuSolverStep.js:16-256).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/avbd_gb300.h"
#include "engine.cuh"
#include "angular.cuh"
#include "tuner.hpp"

using namespace avbd;

namespace avbd {

// Message of the last failed ABI call on this thread (avbd_last_error).
void set_error(const std::string& message);

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(call)                                                                                          \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess) throw Error(AVBD_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Every device allocation and free bumps this generation: a recorded launch sequence (a CUDA
// graph of a tick) is valid only while it is unchanged.
inline std::atomic<long long>& alloc_generation_counter() {
  static std::atomic<long long> g{0};
  return g;
}
inline long long alloc_generation() { return alloc_generation_counter().load(std::memory_order_relaxed); }

template <class T> inline T* dalloc(size_t n) {
  void* p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) throw Error(AVBD_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  alloc_generation_counter().fetch_add(1, std::memory_order_relaxed);
  return static_cast<T*>(p);
}

inline void dfree(void* p) {
  if (p) {
    cudaFree(p);
    alloc_generation_counter().fetch_add(1, std::memory_order_relaxed);
  }
}

// First-fit allocator of index ranges [0, cap).
struct RangeAlloc {
  int cap = 0;
  std::map<int, int> freeRanges;  // start -> length
  void init(int c) {
    cap = c;
    freeRanges.clear();
    if (c > 0) freeRanges[0] = c;
  }
  int find(int n) const {
    if (n == 0) return 0;
    for (auto& f : freeRanges)
      if (f.second >= n) return f.first;
    return -1;
  }
  int alloc(int n) {
    if (n == 0) return 0;
    for (auto it = freeRanges.begin(); it != freeRanges.end(); ++it) {
      if (it->second < n) continue;
      const int start = it->first, len = it->second;
      freeRanges.erase(it);
      if (len > n) freeRanges[start + n] = len - n;
      return start;
    }
    return -1;
  }
  void release(int start, int n) {
    if (n <= 0) return;
    auto it = freeRanges.emplace(start, n).first;
    auto next = std::next(it);
    if (next != freeRanges.end() && it->first + it->second == next->first) {
      it->second += next->second;
      freeRanges.erase(next);
    }
    if (it != freeRanges.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        freeRanges.erase(it);
      }
    }
  }
  void grow(int newCap) {
    if (newCap <= cap) return;
    const int old = cap;
    cap = newCap;
    release(old, newCap - old);
  }
};

}  // namespace avbd

struct avbd_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<void*> owned;  // Arenas created under this context
};

namespace avbd {

// World state kept on the host while a world is evicted (all indices world-local).
struct Snapshot {
  std::vector<float4> pose, pose0, poseY;          // (pos, rot) pairs
  std::vector<float4> vel, ang, vprev, size, mass;  // one per body
  std::vector<int4> meta;
  std::vector<float> restitution;
  std::vector<int> sleep;
  std::vector<float> sleepTime;
  std::vector<uint32_t> watch, watchPrev;
  std::vector<int2> jab;
  std::vector<float4> joint[10];  // rA rB stiff penLin penAng lamLin lamAng C0Lin C0Ang restQ
  std::vector<int> jbroken;
  std::vector<int> colors;
  std::vector<uint2> pairs;
  std::vector<int> counts;
  std::vector<float4> basis, ct;
};

struct WorldRec {
  bool live = false, resident = false;
  bool triggers = false;  // some body is a trigger (isTrigger)
  WorldDev dev{};
  int nBodies = 0, nJoints = 0;
  int which = 0;
  std::vector<std::pair<unsigned long long, int>> nc;  // local (hi << 32 | lo) -> local joint id or -1
  std::vector<int> largeLocal;
  long long pending = 0;
  unsigned long long lastUse = 0;
  std::unique_ptr<Snapshot> snap;
  // broadphase tree (FLAG_BVH): node range in the arena's pool, rebuilt every bvhRebuild steps
  bool bvh = false;
  BvhLayout tree;
  int bvhOff = 0, bvhRebuild = 16, sinceBuild = 0;
  bool built = false;
  std::vector<uint32_t> edits;  // body command records waiting for the next step (12 words each)
  bool wakePending = false;     // queued commands wake the world when they apply
  bool pinned = false;          // a held tick of this world is being re-run: not to be evicted
  long long steps = 0;          // steps taken
  // contact events (FLAG_EVENTS): device region of evCap events while resident, events already
  // drained to the host (12 words each), events dropped past the capacity
  int evCap = 0;
  float4* evDev = nullptr;
  std::vector<uint32_t> evHost;
  long long evDropped = 0;
};

// Solve schedule overrides from the environment (for tests and measurements): AVBD_SOLVE=queue|
// barrier, AVBD_SOLVE_WAVES, AVBD_SOLVE_BLOCKS, AVBD_SOLVE_WAIT_CYCLES (the tile queue's wait bound),
// AVBD_SOLVE_WAIT_PROBE (tests: the queue's waits run out on purpose, see SolveConfig::probe).
inline SolveConfig solve_config_from_env(SolveConfig c) {
  if (const char* v = std::getenv("AVBD_SOLVE")) c.queue = std::strcmp(v, "barrier") != 0;
  if (const char* v = std::getenv("AVBD_SOLVE_WAVES")) c.waves = std::max(1, std::atoi(v));
  if (const char* v = std::getenv("AVBD_SOLVE_BLOCKS")) c.blocks = std::max(0, std::atoi(v));
  if (const char* v = std::getenv("AVBD_SOLVE_TILE")) c.tile = std::atoi(v) == 256 ? 256 : 128;
  if (const char* v = std::getenv("AVBD_SOLVE_WAIT_CYCLES")) c.waitCycles = std::max(0LL, std::atoll(v));
  if (const char* v = std::getenv("AVBD_SOLVE_WAIT_PROBE")) c.probe = std::atoi(v) != 0;
  return c;
}

class Arena {
 public:
  avbd_ctx* ctx;
  cudaStream_t s;
  int bodyCap = 0, jointCap = 0, slotCap = 0, maxWorlds = 0;
  RangeAlloc bodyA, jointA, slotA;
  // tree pool of the worlds with FLAG_BVH, and the build scratch (sized for the largest tree)
  RangeAlloc bvhA;
  int bvhCap = 0;
  BvhScratch bsc{};
  size_t bscKeys = 0, bscHist = 0, bscClusters = 0, bscBounds = 0;
  BounceBufs BB{};  // bounce pass (FLAG_RESTITUTION), see ensureBounce
  SleepBufs SB{};   // island sleeping (FLAG_SLEEP), see ensureSleep
  EventBufs EV{};   // contact events (FLAG_EVENTS), per world; see watchContacts
  size_t evWorlds = 0;
  size_t sleepBodies = 0, sleepWorlds = 0;
  size_t bounceBodies = 0, bounceSlots = 0;
  std::vector<int> freeSlots;
  std::vector<WorldRec> W;
  // device
  WorldDev* worlds = nullptr;
  BodyPtrs B{};
  JointPtrs J{};
  PairPtrs P{};
  Grid G{};
  NarrowScratch NS{};
  NoCollide NC{};
  int ncCap = 0;
  Topo T{};
  int *which = nullptr, *pairN = nullptr, *wover = nullptr, *wactive = nullptr;
  int4* active = nullptr;
  int *activeBodies = nullptr, *activeJoints = nullptr, *activePairs = nullptr, *pairPrefix = nullptr, *pairCount = nullptr;
  Counters* ctr = nullptr;
  Counters* ctrHost = nullptr;
  int uploadedWorlds = 0;  // world capacity the device's active table was uploaded for
  void* scanTemp = nullptr;
  size_t scanBytes = 0;
  size_t itemCap = 0;
  int rounds = 64;
  bool tickTriggers = false;  // a world of the tick being built has trigger bodies
  int lastPairs = 0, lastJoints = 0;
  long long steps = 0, regrowths = 0, evictions = 0, restores = 0;
  bool haveStats = false;
  // profiling: event pairs per kernel class, harvested after each tick's counter readback
  enum { P_COLLIDE, P_TOPO, P_PRIMAL, P_DUAL, P_OTHER, P_CLASSES };
  struct Rec {
    int cls;
    cudaEvent_t a, b;
  };
  bool prof = false;
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  double profMs[P_CLASSES] = {0, 0, 0, 0, 0};
  long long profPrimalLaunches = 0;
  int profSteps = 0;
  double profBytes[3] = {0, 0, 0};
  unsigned long long* traffic = nullptr;  // device: primal, dual, collide bytes of one tick
  float4* poseStage = nullptr;

  // Called when a world's pair region must grow in a tick and the slot buffers cannot place
  // `slots` more: an owner with a memory budget may free slot ranges (evicting worlds that are
  // not being stepped) or grow the buffers itself; otherwise the buffers grow here.
  std::function<void(int slots)> onSlotPressure;

  // Host -> device uploads go through a pinned staging ring on the arena's stream: put() copies
  // the source into the ring (the caller's buffer is free at once, sources may be temporaries) and
  // queues the copy with an event behind it; a region of the ring is reused only once its event
  // has completed, so an upload waits for the device only when the ring is full.
  char* stage = nullptr;
  size_t stageCap = 0, stageHead = 0;
  struct StageRegion {
    size_t a, b;
    cudaEvent_t e;
  };
  std::deque<StageRegion> stageLive;
  std::vector<cudaEvent_t> stageEvents;

  void stageRetire(bool wait) {
    while (!stageLive.empty()) {
      cudaEvent_t e = stageLive.front().e;
      if (wait) CK(cudaEventSynchronize(e));
      else if (cudaEventQuery(e) != cudaSuccess) break;
      stageEvents.push_back(e);
      stageLive.pop_front();
    }
  }
  size_t stageAlloc(size_t bytes) {
    const size_t need = (bytes + 255) & ~size_t(255);
    if (need > stageCap / 2) {
      CK(cudaStreamSynchronize(s));
      stageRetire(true);
      if (stage) cudaFreeHost(stage);
      stage = nullptr;
      stageCap = 0;
      const size_t cap = std::max<size_t>(2 * need, size_t(8) << 20);
      CK(cudaHostAlloc((void**)&stage, cap, cudaHostAllocDefault));
      stageCap = cap;
      stageHead = 0;
    }
    for (;;) {
      stageRetire(false);
      if (stageLive.empty()) {
        stageHead = need;
        return 0;
      }
      const size_t start = stageHead + need <= stageCap ? stageHead : 0;
      const size_t tail = stageLive.front().a;
      // in use: [tail, head) when head > tail; [tail, cap) and [0, head) otherwise (head == tail:
      // the whole ring)
      const bool ok = stageHead > tail ? (start == stageHead || start + need <= tail) : (start == stageHead && start + need <= tail);
      if (ok) {
        stageHead = start + need;
        return start;
      }
      stageRetire(true);  // the ring is full: wait for its oldest upload
    }
  }
  void put(void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return;
    const size_t at = stageAlloc(bytes);
    std::memcpy(stage + at, src, bytes);
    CK(cudaMemcpyAsync(dst, stage + at, bytes, cudaMemcpyHostToDevice, s));
    cudaEvent_t e;
    if (!stageEvents.empty()) {
      e = stageEvents.back();
      stageEvents.pop_back();
    } else {
      CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    CK(cudaEventRecord(e, s));
    stageLive.push_back(StageRegion{at, at + ((bytes + 255) & ~size_t(255)), e});
  }
  // Wait until everything queued on the arena's stream has run.
  void flush() {
    CK(cudaStreamSynchronize(s));
    stageRetire(true);
  }
  // Device -> host copy after every queued tick is final (resolve): the result reflects every
  // step queued so far.
  void get(void* dst, const void* src, size_t bytes) {
    resolve();
    getRaw(dst, src, bytes);
  }
  void getRaw(void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }

  Arena(avbd_ctx* c, int bodies, int joints, int slots, int worldsMax) : ctx(c), s(c->stream) {
    prepare_launches();  // per-device launch geometry, looked up before any stream capture
    tickEvents.reserve(2 * MAX_IN_FLIGHT + 8);
    solveCfg = solve_config_from_env(solveCfg);
    tuner.init(solveCfg);
    allocate(std::max(bodies, 1), std::max(joints, 1), std::max(slots, 1024), std::max(worldsMax, 1));
  }
  ~Arena() {
    cudaStreamSynchronize(s);
    harvest();
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
    for (auto& r : stageLive) cudaEventDestroy(r.e);
    for (cudaEvent_t e : stageEvents) cudaEventDestroy(e);
    for (auto& t : tickLog)
      if (t.done) cudaEventDestroy(t.done);
    for (cudaEvent_t e : tickEvents) cudaEventDestroy(e);
    clearGraphs();
    release();
  }

  // ------------------------------------------------------------------ device memory
  void allocate(int nb, int nj, int slots, int nw) {
    bodyCap = nb;
    jointCap = nj;
    maxWorlds = nw;
    bodyA.init(nb);
    jointA.init(nj);
    W.resize(nw);
    for (int w = nw - 1; w >= 0; w--) freeSlots.push_back(w);
    const size_t N = size_t(nb), NJ = size_t(nj);
    for (float4** p : {&B.pose, &B.pose0, &B.poseY}) *p = dalloc<float4>(2 * N);
    for (float4** p : {&B.vel, &B.ang, &B.vprev, &B.size, &B.mass, &B.inert}) *p = dalloc<float4>(N);
    for (float4** p : {&B.pose0i, &B.poseYi}) *p = dalloc<float4>(2 * N);
    B.meta = dalloc<int4>(N);
    B.restitution = dalloc<float>(N);
    B.sleep = dalloc<int>(N);
    B.sleepTime = dalloc<float>(N);
    B.watch = dalloc<uint32_t>(N);
    B.watchPrev = dalloc<uint32_t>(N);
    J.ab = dalloc<int2>(NJ);
    for (float4** p : {&J.rA, &J.rB, &J.stiff, &J.penLin, &J.penAng, &J.lamLin, &J.lamAng, &J.C0Lin, &J.C0Ang, &J.restQ})
      *p = dalloc<float4>(NJ);
    J.broken = dalloc<int>(NJ);
    worlds = dalloc<WorldDev>(nw);
    which = dalloc<int>(nw);
    pairN = dalloc<int>(2 * size_t(nw));
    wover = dalloc<int>(nw);
    wactive = dalloc<int>(nw);
    active = dalloc<int4>(nw);
    CK(cudaMemset(which, 0, sizeof(int) * nw));
    CK(cudaMemset(pairN, 0, sizeof(int) * 2 * nw));
    CK(cudaMemset(wover, 0, sizeof(int) * nw));
    CK(cudaMemset(wactive, 0xff, sizeof(int) * nw));
    activeBodies = dalloc<int>(N);
    activeJoints = dalloc<int>(NJ);
    pairPrefix = dalloc<int>(size_t(nw) + 1);
    pairCount = dalloc<int>(N + 1);
    uint32_t table = 1024;
    while (table < 2u * uint32_t(N)) table <<= 1;
    G.tableMask = table - 1;
    G.cellCount = dalloc<int>(size_t(table) + 1);
    G.cellFill = dalloc<int>(table);
    G.cellBodies = dalloc<int>(N);
    G.cellKey = dalloc<int4>(N);
    G.cellPos = dalloc<float4>(N);
    G.pairTmp = dalloc<uint32_t>(N * PAIR_TMP);
    G.bodyBucket = dalloc<int>(N);
    G.large = dalloc<int>(size_t(nw) * MAX_LARGE);
    T.adjStart = dalloc<int>(N + 1);
    T.adjFill = dalloc<int>(std::max<size_t>(N + 1, MAX_COLORS));
    T.activeIndex = dalloc<int>(N);
    T.color = dalloc<int>(2 * N);
    T.won = dalloc<int>(N);
    T.pending = dalloc<unsigned char>(N);
    CK(cudaMemset(T.pending, 0, N));
    T.colorBodies = dalloc<int>(N);
    T.colorScan = dalloc<int>(color_scan_ints(N));
    T.slotRef = dalloc<int4>(N);
    T.itemStart = dalloc<int>(N + 1);
    ctr = dalloc<Counters>(1);
    CK(cudaMemset(ctr, 0, sizeof(Counters)));
    CK(cudaHostAlloc((void**)&ctrHost, sizeof(Counters), cudaHostAllocDefault));
    std::memset(ctrHost, 0, sizeof(Counters));
    queueScratch = dalloc<int>(solve_queue_ints(nw));
    ctl = dalloc<TickCtl>(1);
    CK(cudaMemset(ctl, 0, sizeof(TickCtl)));
    CK(cudaHostAlloc((void**)&ctlHost, sizeof(TickCtl), cudaHostAllocDefault));
    std::memset((void*)ctlHost, 0, sizeof(TickCtl));
    NC.keys = dalloc<unsigned long long>(1);
    NC.jid = dalloc<int>(1);
    ncCap = 1;
    slotCap = 0;
    allocSlots(slots);
  }

  void release() {
    void* ptrs[] = {B.pose, B.pose0, B.poseY, B.vel, B.ang, B.vprev, B.size, B.mass, B.pose0i, B.poseYi, B.inert, B.meta,
                    B.restitution, B.sleep,
                    B.sleepTime, B.watch, B.watchPrev, EV.region, EV.count, EV.cap, EV.step, SB.parent, SB.flags,
                    SB.wake, SB.err, BB.inVel,
                    BB.inAng, BB.ra, BB.rb, BB.nk, BB.delta, J.ab, J.rA,
                    J.rB, J.stiff, J.penLin, J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang, J.restQ, J.broken, worlds,
                    which, pairN, wover, wactive, active, activeBodies, activeJoints, pairPrefix, pairCount, G.cellCount,
                    G.cellFill, G.cellBodies, G.cellKey, G.cellPos, G.pairTmp, G.bodyBucket, G.large, T.adjStart, T.adjFill, T.activeIndex, T.color, T.won,
                    T.pending, T.colorBodies, T.colorScan, T.slotRef, T.itemStart, T.itemRef, ctr, NC.keys, NC.jid, scanTemp, traffic,
                    poseStage, P.pair, P.count, P.basis, P.ct, NS.sat, NS.boxList, NS.sphereList, NS.sphere2List, NS.ctr, activePairs,
                    T.adjList, T.adjOther, G.bvh.node, G.bvh.parent, G.bvh.escape, G.bvh.minIdx, bsc.keys[0], bsc.keys[1], bsc.hist,
                    bsc.clusters, bsc.bounds, editRec, editRanges, editTele, io, ctl, queueScratch, replySeg};
    for (void* p : ptrs) dfree(p);
    for (WorldRec& R : W) dfree(R.evDev);
    if (ctrHost) cudaFreeHost(ctrHost);
    if (ctlHost) cudaFreeHost(ctlHost);
    if (stage) cudaFreeHost(stage);
  }

  // Pair-slot buffers (both halves) and everything sized by them; keeps existing regions.
  void allocSlots(int cap) {
    PairPtrs np;
    np.pair = dalloc<uint2>(2 * size_t(cap));
    np.count = dalloc<int>(2 * size_t(cap));
    np.basis = dalloc<float4>(2 * size_t(cap) * 3);
    np.ct = dalloc<float4>(2 * size_t(cap) * MAX_CONTACTS * 4);
    if (slotCap > 0) {
      for (int k = 0; k < 2; k++) {
        const size_t o = size_t(k) * slotCap, n = size_t(k) * cap;
        CK(cudaMemcpyAsync(np.pair + n, P.pair + o, size_t(slotCap) * sizeof(uint2), cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(np.count + n, P.count + o, size_t(slotCap) * sizeof(int), cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(np.basis + 3 * n, P.basis + 3 * o, size_t(slotCap) * 3 * sizeof(float4), cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(np.ct + 32 * n, P.ct + 32 * o, size_t(slotCap) * 32 * sizeof(float4), cudaMemcpyDeviceToDevice, s));
      }
      CK(cudaStreamSynchronize(s));
    }
    for (void* p : {(void*)P.pair, (void*)P.count, (void*)P.basis, (void*)P.ct, (void*)NS.sat, (void*)NS.boxList,
                    (void*)NS.sphereList, (void*)NS.sphere2List, (void*)NS.ctr, (void*)activePairs, (void*)T.adjList,
                    (void*)T.adjOther})
      dfree(p);
    P = np;
    NS.sat = dalloc<float4>(cap);
    NS.boxList = dalloc<int>(cap);
    NS.sphereList = dalloc<int>(cap);
    NS.sphere2List = dalloc<int>(cap);
    NS.ctr = dalloc<int>(3);
    activePairs = dalloc<int>(cap);
    T.adjList = dalloc<uint32_t>(2 * (size_t(jointCap) + size_t(cap)) + 1);
    T.adjOther = dalloc<int>(2 * (size_t(jointCap) + size_t(cap)) + 1);
    if (slotCap == 0) slotA.init(cap);
    else slotA.grow(cap);
    slotCap = cap;
    statsValid = false;  // the last tick's pair list was in the buffers just replaced
    size_t need = std::max(scan_temp_bytes(int(G.tableMask) + 2), scan_temp_bytes(bodyCap + 2));
    need = std::max(need, scan_temp_bytes(maxWorlds + 2));
    need = std::max(need, scan_temp_bytes(int(color_scan_ints(size_t(bodyCap)))));
    if (need > scanBytes) {
      dfree(scanTemp);
      scanTemp = dalloc<char>(need);
      scanBytes = need;
    }
  }

  // Growth keeps every world's ranges (offsets are unchanged; new capacity is appended).
  template <class X> void regrow(X*& d, size_t keep, size_t m) {
    X* n = dalloc<X>(m);
    if (keep) CK(cudaMemcpyAsync(n, d, keep * sizeof(X), cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    dfree(d);
    d = n;
  }
  template <class X> void rescratch(X*& d, size_t m) {
    CK(cudaStreamSynchronize(s));  // queued work may still use the old buffer
    dfree(d);
    d = nullptr;
    d = dalloc<X>(m);
  }
  void ensureScan() {
    size_t need = std::max(scan_temp_bytes(int(G.tableMask) + 2), scan_temp_bytes(bodyCap + 2));
    need = std::max(need, scan_temp_bytes(maxWorlds + 2));
    need = std::max(need, scan_temp_bytes(int(color_scan_ints(size_t(bodyCap)))));
    if (need > scanBytes) {
      rescratch(reinterpret_cast<char*&>(scanTemp), need);
      scanBytes = need;
    }
  }

  static uint32_t tableFor(size_t n) {
    uint32_t table = 1024;
    while (table < 2u * uint32_t(n)) table <<= 1;
    return table;
  }

  void growBodies(int nb) {
    if (nb <= bodyCap) return;
    flush();
    const size_t o = size_t(bodyCap), N = size_t(nb);
    for (float4** p : {&B.pose, &B.pose0, &B.poseY}) regrow(*p, 2 * o, 2 * N);
    for (float4** p : {&B.vel, &B.ang, &B.vprev, &B.size, &B.mass}) regrow(*p, o, N);
    for (float4** p : {&B.pose0i, &B.poseYi, &B.inert}) {  // rewritten by every step's warm start
      cudaFree(*p);
      *p = dalloc<float4>(p == &B.inert ? N : 2 * N);
    }
    regrow(B.meta, o, N);
    regrow(B.restitution, o, N);
    regrow(B.sleep, o, N);
    regrow(B.sleepTime, o, N);
    regrow(B.watch, o, N);
    regrow(B.watchPrev, o, N);
    int* c = dalloc<int>(2 * N);  // both colour buffers, stride = capacity
    CK(cudaMemcpyAsync(c, T.color, o * 4, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(c + N, T.color + o, o * 4, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    dfree(T.color);
    T.color = c;
    rescratch(T.pending, N);
    CK(cudaMemset(T.pending, 0, N));
    for (int** p : {&T.activeIndex, &T.won, &T.colorBodies, &activeBodies, &G.cellBodies, &G.bodyBucket}) rescratch(*p, N);
    rescratch(T.colorScan, color_scan_ints(N));
    rescratch(T.slotRef, N);
    rescratch(G.cellKey, N);
    rescratch(G.cellPos, N);
    rescratch(G.pairTmp, N * PAIR_TMP);
    for (int** p : {&T.itemStart, &T.adjStart, &pairCount}) rescratch(*p, N + 1);
    rescratch(T.adjFill, std::max<size_t>(N + 1, MAX_COLORS));
    const uint32_t table = tableFor(N);
    if (table != G.tableMask + 1) {
      G.tableMask = table - 1;
      rescratch(G.cellCount, size_t(table) + 1);
      rescratch(G.cellFill, size_t(table));
    }
    bodyA.grow(nb);
    bodyCap = nb;
    ensureScan();
  }

  void growJoints(int nj) {
    if (nj <= jointCap) return;
    flush();
    const size_t o = size_t(jointCap), N = size_t(nj);
    regrow(J.ab, o, N);
    for (float4** p : {&J.rA, &J.rB, &J.stiff, &J.penLin, &J.penAng, &J.lamLin, &J.lamAng, &J.C0Lin, &J.C0Ang, &J.restQ})
      regrow(*p, o, N);
    regrow(J.broken, o, N);
    rescratch(activeJoints, N);
    rescratch(T.adjList, 2 * (N + size_t(slotCap)) + 1);
    rescratch(T.adjOther, 2 * (N + size_t(slotCap)) + 1);
    jointA.grow(nj);
    jointCap = nj;
  }

  void growWorlds(int nw) {
    if (nw <= maxWorlds) return;
    flush();
    const size_t o = size_t(maxWorlds), N = size_t(nw);
    regrow(worlds, o, N);
    regrow(which, o, N);
    regrow(wover, o, N);
    CK(cudaMemset(which + o, 0, (N - o) * 4));
    CK(cudaMemset(wover + o, 0, (N - o) * 4));
    int* pn = dalloc<int>(2 * N);  // pairN: both buffers, stride = world capacity
    CK(cudaMemset(pn, 0, 2 * N * 4));
    CK(cudaMemcpyAsync(pn, pairN, o * 4, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(pn + N, pairN + o, o * 4, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    dfree(pairN);
    pairN = pn;
    regrow(G.large, o * MAX_LARGE, N * MAX_LARGE);
    rescratch(wactive, N);
    rescratch(active, N);
    rescratch(pairPrefix, N + 1);
    actUploaded.clear();  // the active table is uploaded again at the next tick
    rescratch(queueScratch, solve_queue_ints(int(N)));
    W.resize(N);
    for (int w = nw - 1; w >= int(o); w--) freeSlots.insert(freeSlots.begin(), w);
    maxWorlds = nw;
    ensureScan();
  }

  // Device bytes of an arena with these capacities: the arrays above and the pair-slot buffers.
  // The per-tick work-item scratch (scratchBytes) comes on top; it grows with the contacts of
  // the worlds being stepped (about 0.2 KB per body in settled piles; the reserve doubles that).
  size_t scratchBytes() const { return itemCap * sizeof(int4); }
  static size_t scratchReserve(long long nb) { return size_t(nb) * 512; }
  size_t footprint(long long nb, long long nj, long long slots, long long nw) const {
    const size_t perBody = 17 * 16 + 2 * 4 + 1 + 16 * 4 + 32 + 4 * PAIR_TMP + 1 + 8;
    const size_t perJoint = 8 + 10 * 16 + 4 + 4 + 8;
    const size_t perSlot = 2 * (8 + 4 + 3 * 16 + MAX_CONTACTS * 64) + 16 + 4 * 4 + 8;
    const size_t perWorld = sizeof(WorldDev) + 4 * 4 + 16 + 4 + MAX_LARGE * 4;
    return size_t(nb) * perBody + size_t(tableFor(size_t(nb))) * 8 + size_t(nj) * perJoint + size_t(slots) * perSlot +
           size_t(nw) * perWorld + size_t(ncCap) * 12 + scanBytes + size_t(bvhCap) * (32 + 12) +
           (2 * bscKeys * sizeof(uint2) + bscHist * 4 + bscClusters * 4 + bscBounds * 16) +
           (bounceBodies * 32 + bounceSlots * 52) + (sleepBodies * 8 + sleepWorlds * 4 + 4) + evWorlds * 20 +
           eventBytes();
  }
  size_t deviceBytes() const { return footprint(bodyCap, jointCap, slotCap, maxWorlds) + scratchBytes(); }

  // Capacities after making room for one more world of (nb, nj, slots): each array that cannot
  // place it grows by at least half.
  void plannedCaps(int nb, int nj, int slots, long long caps[4], bool minimal, bool newWorld = true) const {
    auto next = [&](const RangeAlloc& a, int cap, int need) -> long long {
      if (a.find(need) >= 0) return cap;
      // the trailing free range (if any) merges with the growth
      int tail = 0;
      if (!a.freeRanges.empty()) {
        auto last = std::prev(a.freeRanges.end());
        if (last->first + last->second == a.cap) tail = last->second;
      }
      const long long exact = (long long)cap + (need - tail);
      return minimal ? exact : std::max<long long>(exact, (long long)cap + cap / 2);
    };
    caps[0] = next(bodyA, bodyCap, nb);
    caps[1] = next(jointA, jointCap, nj);
    caps[2] = next(slotA, slotCap, slots);
    caps[3] = newWorld && freeSlots.empty() ? (minimal ? maxWorlds + 1 : maxWorlds + std::max(16, maxWorlds / 2)) : maxWorlds;
  }
  void growTo(const long long caps[4]) {
    if (caps[0] > 0x3fffffffLL || caps[2] > 0x3fffffffLL || caps[1] > 0x3fffffffLL) throw Error(AVBD_E_CAPACITY, "arena index space exhausted");
    growBodies(int(caps[0]));
    growJoints(int(caps[1]));
    if (caps[2] > slotCap) allocSlots(int(caps[2]));
    growWorlds(int(caps[3]));
  }
  // Make room for one more world (without a budget): grow what does not fit.
  void ensureRoom(int nb, int nj, int slots, bool newWorld = true) {
    long long caps[4];
    plannedCaps(nb, nj, slots, caps, false, newWorld);
    growTo(caps);
  }

  Tick tick(int nActive, int nb, int nj) {
    Tick t;
    t.active = active;
    t.nActive = nActive;
    t.wactive = wactive;
    t.which = which;
    t.bodies = activeBodies;
    t.nBodies = nb;
    t.joints = activeJoints;
    t.nJoints = nj;
    t.pairs = activePairs;
    t.pairPrefix = pairPrefix;
    t.pairN = pairN;
    t.wover = wover;
    t.maxWorlds = maxWorlds;
    t.slotStride = slotCap;
    t.bodyStride = bodyCap;
    t.triggerBits = tickTriggers ? B.sleep : nullptr;
    t.ctl = ctl;
    return t;
  }

  // ------------------------------------------------------------------ worlds
  static void validate(const avbd_scene_desc& d, const avbd_params& p) {
    if (d.n_bodies < 0 || d.n_cons < 0) throw Error(AVBD_E_INVALID, "negative body or constraint count");
    if (d.n_bodies > 0 && (!d.position || !d.size || !d.mass || !d.moment || !d.friction || !d.radius || !d.shape))
      throw Error(AVBD_E_INVALID, "scene is missing a required body array");
    if (d.n_cons > 0 && (!d.cons_kind || !d.cons_a || !d.cons_b || !d.cons_ra || !d.cons_rb || !d.cons_p0 || !d.cons_p1 || !d.cons_p2))
      throw Error(AVBD_E_INVALID, "scene is missing a required constraint array");
    if (!(p.dt > 0.f) || !std::isfinite(p.dt)) throw Error(AVBD_E_INVALID, "timeStep must be positive");
    if (p.iterations <= 0) throw Error(AVBD_E_INVALID, "iterations must be a positive integer");
    if (!std::isfinite(p.gravity)) throw Error(AVBD_E_INVALID, "gravity must be finite");
    for (int i = 0; i < d.n_bodies; i++) {
      if (d.shape[i] != AVBD_SHAPE_BOX && d.shape[i] != AVBD_SHAPE_SPHERE && d.shape[i] != AVBD_SHAPE_CAPSULE)
        throw Error(AVBD_E_INVALID, "unknown body shape");
      for (int k = 0; k < 3; k++) {
        if (!std::isfinite(d.position[3 * i + k])) throw Error(AVBD_E_INVALID, "position must be finite");
        if (!(d.size[3 * i + k] > 0.f)) throw Error(AVBD_E_INVALID, "size must be positive");
      }
    }
    for (int c = 0; c < d.n_cons; c++) {
      int k = d.cons_kind[c];
      if (k != AVBD_CONS_JOINT && k != AVBD_CONS_SPRING && k != AVBD_CONS_IGNORE && k != AVBD_CONS_MOTOR && k != AVBD_CONS_LIMIT)
        throw Error(AVBD_E_INVALID, "unknown constraint kind");
      int a = d.cons_a[c], b = d.cons_b[c];
      if (b < 0 || b >= d.n_bodies || a < -1 || a >= d.n_bodies || a == b) throw Error(AVBD_E_INVALID, "constraint bodies out of range");
      if (a < 0 && (k == AVBD_CONS_SPRING || k == AVBD_CONS_IGNORE)) throw Error(AVBD_E_INVALID, "only joints may attach to the world");
      if (k == AVBD_CONS_MOTOR || k == AVBD_CONS_LIMIT) checkAngular(k, d.cons_ra + 3 * c, d.cons_rb + 3 * c, d.cons_p0[c], d.cons_p1[c]);
    }
  }

  // angularConstraintOptions (src/gpu/angularConstraints.js:87-120): finite nonzero axes; a
  // finite motor speed and a nonnegative finite torque bound; limits ordered within [-pi, pi].
  static void checkAngular(int k, const float* ra, const float* rb, float p0, float p1) {
    for (const float* v : {ra, rb}) {
      if (!(std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2])) ||
          !(double(v[0]) * v[0] + double(v[1]) * v[1] + double(v[2]) * v[2] >= 1e-16))
        throw Error(AVBD_E_INVALID, "Angular axis requires three finite, nonzero components");
    }
    if (k == AVBD_CONS_MOTOR) {
      if (!std::isfinite(p0) || !std::isfinite(p1) || p1 < 0.f)
        throw Error(AVBD_E_INVALID, "Motor speed must be finite and maxTorque nonnegative");
    } else if (!(p0 >= -ANG_PI && p1 <= ANG_PI && p0 <= p1)) {
      throw Error(AVBD_E_INVALID, "Hinge angles must be ordered within -PI..PI radians");
    }
  }

  // A spring's breakStrain / breakForce (src/gpu/springMaterial.js): zero, negative or infinite
  // means unbreakable, held as INFINITY.
  static float springLimit(float x) { return x > 0.f && std::isfinite(x) ? x : INFINITY; }

  static int jointsOf(const avbd_scene_desc& d) {
    int nj = 0;
    for (int c = 0; c < d.n_cons; c++) nj += d.cons_kind[c] != AVBD_CONS_IGNORE;
    return nj;
  }
  static int initialPairCap(int n) { return 8 * n + 32; }

  bool fits(int nb, int nj, int slots) const { return bodyA.find(nb) >= 0 && jointA.find(nj) >= 0 && slotA.find(slots) >= 0; }

  // World parameters, large bodies (radius > 2 x median, at most 64) and the grid cell.
  static void worldParams(const avbd_scene_desc& d, const avbd_params& p, WorldRec& R) {
    WorldDev& Wd = R.dev;
    std::memset(&Wd, 0, sizeof(Wd));
    Wd.dt = p.dt;
    Wd.gravity = p.gravity;
    Wd.alpha = p.alpha;
    Wd.gamma = p.gamma;
    Wd.betaLin = p.beta_lin;
    Wd.betaAng = p.beta_ang;
    Wd.up0 = p.up[0];
    Wd.up1 = p.up[1];
    Wd.up2 = p.up[2];
    Wd.iterations = p.iterations;
    Wd.flags = (p.mass_penalty ? FLAG_MASS_PENALTY : 0) | (p.face_bias ? FLAG_FACE_BIAS : 0);
    if (d.restitution)
      for (int i = 0; i < d.n_bodies; i++)
        if (d.restitution[i] > 0.f) {
          Wd.flags |= FLAG_RESTITUTION;
          break;
        }
    if (p.sleeping) Wd.flags |= FLAG_SLEEP;
    Wd.sleepSpeed = p.sleep_speed > 0.f ? p.sleep_speed : 0.08f;
    Wd.sleepDelay = p.sleep_time > 0.f ? p.sleep_time : 0.6f;
    Wd.bodyCount = d.n_bodies;
    R.largeLocal.clear();
    float largeR = INFINITY;
    if (d.n_bodies > 0) {
      std::vector<float> sorted(d.radius, d.radius + d.n_bodies);
      std::sort(sorted.begin(), sorted.end());
      float thr = 2.f * sorted[sorted.size() / 2];
      int nl = 0;
      for (float r : sorted) nl += r > thr;
      if (nl > MAX_LARGE) thr = sorted[sorted.size() - (MAX_LARGE + 1)];
      float maxSmall = 0.f;
      for (float r : sorted)
        if (!(r > thr)) maxSmall = std::max(maxSmall, r);
      largeR = thr;
      Wd.cell = std::max(2.f * maxSmall * 1.001f, 1e-3f);
      for (int i = 0; i < d.n_bodies; i++)
        if (d.radius[i] > largeR) R.largeLocal.push_back(i);
    } else {
      Wd.cell = 1.f;
    }
    Wd.largeR = largeR;
    Wd.largeCount = int(R.largeLocal.size());
    R.nBodies = d.n_bodies;
    R.nJoints = jointsOf(d);
    Wd.jointCount = R.nJoints;
    R.bvh = p.broadphase == AVBD_BROADPHASE_HPLOC || (p.broadphase == AVBD_BROADPHASE_AUTO && treeSuits(d, R.nJoints, Wd.cell));
    if (R.bvh) Wd.flags |= FLAG_BVH;
    R.bvhRebuild = p.bvh_rebuild > 0 ? p.bvh_rebuild : 16;
    Wd.bvhRoot = -1;
    R.nc.clear();
    int j = 0;
    for (int c = 0; c < d.n_cons; c++) {
      const int kind = d.cons_kind[c];
      const int jid = kind != AVBD_CONS_IGNORE ? j++ : -1;
      const int a = d.cons_a[c], b = d.cons_b[c];
      if (a >= 0) R.nc.push_back({(unsigned long long)(uint32_t)std::max(a, b) << 32 | (uint32_t)std::min(a, b), jid});
    }
  }

  // "auto" broadphase (src/gpu/appGpuSolver3D.js:333-398): the tree for >= 10,000 bodies when the
  // grid cell is at least 4x twice the median radius, or for a jointed sheet of thin plates.
  static bool treeSuits(const avbd_scene_desc& d, int joints, float cell) {
    const int n = d.n_bodies;
    if (n < 10000) return false;
    std::vector<float> radii;
    radii.reserve(n);
    int dynamicCount = 0, thin = 0;
    for (int i = 0; i < n; i++) {
      if (d.radius[i] > 0.f) radii.push_back(d.radius[i]);
      if (!(d.mass[i] > 0.f)) continue;
      dynamicCount++;
      const float a = d.size[3 * i], b = d.size[3 * i + 1], c = d.size[3 * i + 2];
      const float lo = std::min(a, std::min(b, c)), hi = std::max(a, std::max(b, c)), mid = a + b + c - lo - hi;
      if (d.shape[i] == AVBD_SHAPE_BOX && lo <= 0.4f * mid && mid >= 0.5f * hi) thin++;
    }
    float median = 1.f;
    if (!radii.empty()) {
      std::nth_element(radii.begin(), radii.begin() + radii.size() / 2, radii.end());
      median = radii[radii.size() / 2];
    }
    const double cellRatio = double(cell) / (2.0 * double(median));
    const bool sheet = joints >= n && dynamicCount > 0 && double(thin) / dynamicCount >= 0.25;
    return cellRatio >= 4.0 || sheet;
  }

  // ------------------------------------------------------------------ trees
  void growBvhPool(int cap) {
    if (cap <= bvhCap) return;
    flush();
    const size_t o = size_t(bvhCap), N = size_t(cap);
    regrow(G.bvh.node, 2 * o, 2 * N);
    regrow(G.bvh.parent, o, N);
    regrow(G.bvh.escape, o, N);
    regrow(G.bvh.minIdx, o, N);
    if (bvhCap == 0) bvhA.init(cap);
    else bvhA.grow(cap);
    bvhCap = cap;
  }
  void ensureBvhScratch(const WorldRec& R) {
    const int n = R.nBodies;
    if (bvh_scratch_keys(n) > bscKeys) {
      bscKeys = bvh_scratch_keys(n);
      rescratch(bsc.keys[0], bscKeys);
      rescratch(bsc.keys[1], bscKeys);
    }
    if (bvh_scratch_hist(n) > bscHist) {
      bscHist = bvh_scratch_hist(n);
      rescratch(bsc.hist, bscHist);
    }
    if (size_t(R.tree.clusters) > bscClusters) {
      bscClusters = size_t(R.tree.clusters);
      rescratch(bsc.clusters, bscClusters);
    }
    if (bvh_scratch_bounds(n) > bscBounds) {
      bscBounds = bvh_scratch_bounds(n);
      rescratch(bsc.bounds, bscBounds);
    }
    const size_t need = scan_temp_bytes(int(bscHist) + 2);
    if (need > scanBytes) {
      rescratch(reinterpret_cast<char*&>(scanTemp), need);
      scanBytes = need;
    }
  }
  void placeBvh(WorldRec& R) {
    if (!R.bvh) return;
    bvh_layout(R.nBodies, R.tree);
    const int need = std::max(R.tree.nodes, 1);
    int off = bvhA.alloc(need);
    if (off < 0) {
      growBvhPool(std::max(bvhCap + need, bvhCap + bvhCap / 2));
      off = bvhA.alloc(need);
    }
    if (off < 0) throw Error(AVBD_E_NOMEM, "tree pool exhausted");
    R.bvhOff = off;
    R.dev.bvhNodeOff = off;
    R.dev.bvhRoot = R.tree.root == BVH_END ? -1 : int(R.tree.root);
    R.built = false;
    R.sinceBuild = 0;
  }
  void freeBvh(WorldRec& R) {
    if (R.bvh) bvhA.release(R.bvhOff, std::max(R.tree.nodes, 1));
  }

  int takeSlot() {
    if (freeSlots.empty()) throw Error(AVBD_E_CAPACITY, "world table full");
    int w = freeSlots.back();
    freeSlots.pop_back();
    return w;
  }

  void placeRanges(WorldRec& R, int slotsWanted) {
    const int bo = bodyA.alloc(R.nBodies);
    if (bo < 0) throw Error(AVBD_E_NOMEM, "body capacity of the arena exhausted");
    const int jo = jointA.alloc(R.nJoints);
    if (jo < 0) {
      bodyA.release(bo, R.nBodies);
      throw Error(AVBD_E_NOMEM, "joint capacity of the arena exhausted");
    }
    const int po = slotA.alloc(slotsWanted);
    if (po < 0) {
      bodyA.release(bo, R.nBodies);
      jointA.release(jo, R.nJoints);
      throw Error(AVBD_E_NOMEM, "pair-slot capacity of the arena exhausted");
    }
    R.dev.bodyOff = bo;
    R.dev.jointOff = jo;
    R.dev.pairOff = po;
    R.dev.pairCap = slotsWanted;
  }

  void uploadWorldDev(int w) { put(worlds + w, &W[w].dev, sizeof(WorldDev)); }

  void uploadLarge(int w) {
    std::vector<int> L(MAX_LARGE, 0);
    for (size_t k = 0; k < W[w].largeLocal.size(); k++) L[k] = W[w].dev.bodyOff + W[w].largeLocal[k];
    put(G.large + size_t(w) * MAX_LARGE, L.data(), sizeof(int) * MAX_LARGE);
  }

  void rebuildNoCollide() {
    std::vector<std::pair<unsigned long long, int>> all;
    for (int w = 0; w < maxWorlds; w++) {
      const WorldRec& R = W[w];
      if (!R.live || !R.resident) continue;
      const unsigned long long off = (unsigned long long)R.dev.bodyOff;
      for (auto& e : R.nc) {
        unsigned long long hi = (e.first >> 32) + off, lo = (e.first & 0xffffffffull) + off;
        all.push_back({hi << 32 | lo, e.second >= 0 ? R.dev.jointOff + e.second : -1});
      }
    }
    std::sort(all.begin(), all.end());
    if (int(all.size()) > ncCap) {
      CK(cudaStreamSynchronize(s));  // queued ticks still read the old arrays
      dfree(NC.keys);
      dfree(NC.jid);
      NC.keys = nullptr;
      NC.jid = nullptr;
      ncCap = int(all.size()) + int(all.size()) / 2 + 16;
      NC.keys = dalloc<unsigned long long>(ncCap);
      NC.jid = dalloc<int>(ncCap);
    }
    NC.n = int(all.size());
    if (!all.empty()) {
      std::vector<unsigned long long> k(all.size());
      std::vector<int> id(all.size());
      for (size_t i = 0; i < all.size(); i++) { k[i] = all[i].first; id[i] = all[i].second; }
      put(NC.keys, k.data(), k.size() * 8);
      put(NC.jid, id.data(), id.size() * 4);
    }
  }

  // Add a world (with rebuild = false, call rebuildNoCollide after a batch of additions).
  // Queued ticks need not finish first: the new world's uploads go to unused ranges in stream order
  // behind them, and growth waits for the stream before it moves any array.
  int addWorld(const avbd_scene_desc& d, const avbd_params& p, bool rebuild = true) {
    validate(d, p);
    ensureRoom(d.n_bodies, jointsOf(d), initialPairCap(d.n_bodies));  // may move W: before any reference into it
    const int w = takeSlot();
    WorldRec& R = W[w];
    bool placed = false;
    try {
      worldParams(d, p, R);
      R.dev.largeOff = w * MAX_LARGE;
      placeRanges(R, initialPairCap(d.n_bodies));
      placed = true;
      placeBvh(R);
    } catch (...) {
      if (placed) freeRanges(R);
      R = WorldRec();
      freeSlots.push_back(w);
      throw;
    }
    R.live = true;
    R.resident = true;
    R.which = 0;
    R.pending = 0;
    rounds = std::max(rounds, p.color_rounds > 0 ? p.color_rounds : 64);
    // bodies
    const size_t n = size_t(d.n_bodies), off = size_t(R.dev.bodyOff);
    if (n) {
      std::vector<float4> pos(n), rot(n), vel(n), ang(n), vprev(n), size(n), mass(n);
      std::vector<int4> meta(n);
      std::vector<float> rest(n);
      std::vector<int> sleepBits(n);
      auto v3at = [&](const float* a, size_t k) { return a ? make_float4(a[3 * k], a[3 * k + 1], a[3 * k + 2], 0.f) : make_float4(0, 0, 0, 0); };
      for (size_t i = 0; i < n; i++) {
        pos[i] = v3at(d.position, i);
        pos[i].w = d.radius[i];
        rot[i] = d.rotation ? make_float4(d.rotation[4 * i], d.rotation[4 * i + 1], d.rotation[4 * i + 2], d.rotation[4 * i + 3])
                            : make_float4(0, 0, 0, 1);
        vel[i] = v3at(d.velocity, i);
        ang[i] = v3at(d.angular_velocity, i);
        vprev[i] = v3at(d.prev_velocity, i);
        size[i] = v3at(d.size, i);
        size[i].w = d.friction[i];
        mass[i] = make_float4(d.mass[i], d.moment[3 * i], d.moment[3 * i + 1], d.moment[3 * i + 2]);
        rest[i] = d.restitution ? d.restitution[i] : 0.f;
        sleepBits[i] = (d.allow_sleep && d.allow_sleep[i] == 0) ? 0 : SLEEP_ALLOW;
        if (d.is_trigger && d.is_trigger[i]) {
          sleepBits[i] |= BODY_TRIGGER;
          R.triggers = true;
        }
        const uint32_t grp = d.group ? d.group[i] : 0xffffffffu, msk = d.collides_with ? d.collides_with[i] : 0xffffffffu;
        meta[i] = make_int4(w, d.shape[i], int(grp), int(msk));
      }
      std::vector<float4> pose(2 * n);
      for (size_t i = 0; i < n; i++) {
        pose[2 * i] = pos[i];
        pose[2 * i + 1] = rot[i];
      }
      for (float4* d : {B.pose, B.pose0, B.poseY}) put(d + 2 * off, pose.data(), 2 * n * 16);
      const float4* src[5] = {vel.data(), ang.data(), vprev.data(), size.data(), mass.data()};
      float4* dst[5] = {B.vel, B.ang, B.vprev, B.size, B.mass};
      for (int k = 0; k < 5; k++) put(dst[k] + off, src[k], n * 16);
      put(B.meta + off, meta.data(), n * 16);
      put(B.restitution + off, rest.data(), n * 4);
      put(B.sleep + off, sleepBits.data(), n * 4);
      std::vector<float> zeros(n, 0.f);
      put(B.sleepTime + off, zeros.data(), n * 4);
      put(B.watch + off, zeros.data(), n * 4);
      put(B.watchPrev + off, zeros.data(), n * 4);
      std::vector<int> minus(n, -1);
      put(T.color + off, minus.data(), n * 4);
      put(T.color + bodyCap + off, minus.data(), n * 4);
    }
    // joints and springs (global body ids)
    const size_t nj = size_t(R.nJoints), joff = size_t(R.dev.jointOff);
    if (nj) {
      std::vector<int2> jab(nj);
      std::vector<float4> jra(nj), jrb(nj), jst(nj), jz(nj, make_float4(0, 0, 0, 0)), jq(nj, make_float4(0, 0, 0, 1));
      std::vector<float4> jpl(nj, make_float4(0, 0, 0, 0));
      std::vector<int> jbr(nj, 0);
      size_t j = 0;
      for (int c = 0; c < d.n_cons; c++) {
        const int kind = d.cons_kind[c];
        if (kind == AVBD_CONS_IGNORE) continue;
        const int a = d.cons_a[c] >= 0 ? int(off) + d.cons_a[c] : -1;
        const int b = int(off) + d.cons_b[c];
        jab[j] = make_int2(a, b);
        const bool angular = kind == AVBD_CONS_MOTOR || kind == AVBD_CONS_LIMIT;
        int kk = kind == AVBD_CONS_JOINT ? KIND_JOINT
                 : kind == AVBD_CONS_SPRING ? KIND_SPRING
                 : kind == AVBD_CONS_MOTOR  ? KIND_MOTOR
                                            : KIND_LIMIT;
        float kf;
        std::memcpy(&kf, &kk, 4);
        jra[j] = make_float4(d.cons_ra[3 * c], d.cons_ra[3 * c + 1], d.cons_ra[3 * c + 2], kf);
        jrb[j] = make_float4(d.cons_rb[3 * c], d.cons_rb[3 * c + 1], d.cons_rb[3 * c + 2], kind == AVBD_CONS_SPRING ? d.cons_p1[c] : 0.f);
        jst[j] = kind == AVBD_CONS_JOINT ? make_float4(d.cons_p0[c], d.cons_p1[c], d.cons_p2[c], 0.f)
                 : angular               ? make_float4(d.cons_p0[c], d.cons_p1[c], INFINITY, 0.f)
                                         : make_float4(d.cons_p0[c], springLimit(d.cons_p3 ? d.cons_p3[c] : 0.f),
                                                       springLimit(d.cons_p2[c]), 0.f);
        if (angular) jpl[j] = make_float4(ANGULAR_PENALTY0, ANGULAR_PENALTY0, 0.f, 0.f);
        j++;
      }
      put(J.ab + joff, jab.data(), nj * 8);
      put(J.rA + joff, jra.data(), nj * 16);
      put(J.rB + joff, jrb.data(), nj * 16);
      put(J.stiff + joff, jst.data(), nj * 16);
      put(J.penLin + joff, jpl.data(), nj * 16);
      for (float4* q : {J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang}) put(q + joff, jz.data(), nj * 16);
      put(J.restQ + joff, jq.data(), nj * 16);
      put(J.broken + joff, jbr.data(), nj * 4);
    }
    const int zero = 0;
    put(which + w, &zero, 4);
    put(pairN + w, &zero, 4);
    put(pairN + maxWorlds + w, &zero, 4);
    put(wover + w, &zero, 4);
    uploadLarge(w);
    uploadWorldDev(w);
    launch_joint_prepare(B, J, R.dev.jointOff, R.dev.jointOff + R.nJoints, s);
    if (rebuild) rebuildNoCollide();
    return w;
  }

  void freeRanges(WorldRec& R) {
    bodyA.release(R.dev.bodyOff, R.nBodies);
    jointA.release(R.dev.jointOff, R.nJoints);
    slotA.release(R.dev.pairOff, R.dev.pairCap);
  }
  // everything a resident world holds in the arena
  void freeResident(WorldRec& R) {
    freeRanges(R);
    freeBvh(R);
  }

  void removeWorld(int w) {
    resolve();
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    CK(cudaStreamSynchronize(s));
    WorldRec& R = W[w];
    if (R.resident) freeResident(R);
    dfree(R.evDev);
    R = WorldRec();
    freeSlots.push_back(w);
    rebuildNoCollide();
    flush();
  }

  template <class X> void getRange(std::vector<X>& out, const X* d, size_t off, size_t n) {
    out.resize(n);
    get(out.data(), d + off, n * sizeof(X));
  }
  template <class X> void putRange(X* d, size_t off, const std::vector<X>& in) {
    put(d + off, in.data(), in.size() * sizeof(X));
  }

  int prevPairs(int w) {
    int n = 0;
    get(&n, pairN + size_t(W[w].which) * maxWorlds + w, 4);
    return n;
  }

  // Move a resident world's state to host memory and free its ranges.
  void evict(int w) {
    resolve();
    WorldRec& R = W[w];
    if (!R.live || !R.resident) throw Error(AVBD_E_INVALID, "world is not resident");
    CK(cudaStreamSynchronize(s));
    auto S = std::make_unique<Snapshot>();
    const size_t off = R.dev.bodyOff, n = R.nBodies, joff = R.dev.jointOff, nj = R.nJoints;
    getRange(S->pose, B.pose, 2 * off, 2 * n);
    getRange(S->pose0, B.pose0, 2 * off, 2 * n);
    getRange(S->poseY, B.poseY, 2 * off, 2 * n);
    getRange(S->vel, B.vel, off, n);
    getRange(S->ang, B.ang, off, n);
    getRange(S->vprev, B.vprev, off, n);
    getRange(S->size, B.size, off, n);
    getRange(S->mass, B.mass, off, n);
    getRange(S->meta, B.meta, off, n);
    getRange(S->restitution, B.restitution, off, n);
    getRange(S->sleep, B.sleep, off, n);
    getRange(S->sleepTime, B.sleepTime, off, n);
    getRange(S->watch, B.watch, off, n);
    getRange(S->watchPrev, B.watchPrev, off, n);
    drainEvents(w);
    dfree(R.evDev);
    R.evDev = nullptr;
    getRange(S->jab, J.ab, joff, nj);
    for (auto& ab : S->jab) {
      if (ab.x >= 0) ab.x -= int(off);
      ab.y -= int(off);
    }
    const float4* jsrc[10] = {J.rA, J.rB, J.stiff, J.penLin, J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang, J.restQ};
    for (int k = 0; k < 10; k++) getRange(S->joint[k], jsrc[k], joff, nj);
    getRange(S->jbroken, J.broken, joff, nj);
    getRange(S->colors, T.color, size_t(R.which) * bodyCap + off, n);
    const int np = prevPairs(w);
    const size_t base = size_t(R.which) * slotCap + R.dev.pairOff;
    getRange(S->pairs, P.pair, base, np);
    for (auto& pr : S->pairs) {
      pr.x -= uint32_t(off);
      pr.y -= uint32_t(off);
    }
    getRange(S->counts, P.count, base, np);
    getRange(S->basis, P.basis, 3 * base, 3 * size_t(np));
    getRange(S->ct, P.ct, 32 * base, 32 * size_t(np));
    freeResident(R);
    R.resident = false;
    R.snap = std::move(S);
    evictions++;
    rebuildNoCollide();
    flush();
  }

  // Bring an evicted world back (into any free ranges); its state continues exactly.
  int restoreSlots(int w) const {
    const int np = int(W[w].snap->pairs.size());
    return std::max(initialPairCap(W[w].nBodies), np + np / 4 + 64);
  }
  void restore(int w) {
    resolve();
    if (w < 0 || w >= maxWorlds || !W[w].live || W[w].resident || !W[w].snap) throw Error(AVBD_E_INVALID, "world is not evicted");
    ensureRoom(W[w].nBodies, W[w].nJoints, restoreSlots(w), false);  // may move W: before any reference into it
    WorldRec& R = W[w];
    Snapshot& S = *R.snap;
    const int np = int(S.pairs.size());
    placeRanges(R, restoreSlots(w));
    placeBvh(R);  // the tree is rebuilt at the next step (it only shapes the candidate search)
    const size_t off = R.dev.bodyOff, joff = R.dev.jointOff;
    putRange(B.pose, 2 * off, S.pose);
    putRange(B.pose0, 2 * off, S.pose0);
    putRange(B.poseY, 2 * off, S.poseY);
    putRange(B.vel, off, S.vel);
    putRange(B.ang, off, S.ang);
    putRange(B.vprev, off, S.vprev);
    putRange(B.size, off, S.size);
    putRange(B.mass, off, S.mass);
    putRange(B.meta, off, S.meta);
    putRange(B.restitution, off, S.restitution);
    putRange(B.sleep, off, S.sleep);
    putRange(B.sleepTime, off, S.sleepTime);
    putRange(B.watch, off, S.watch);
    putRange(B.watchPrev, off, S.watchPrev);
    if (R.dev.flags & FLAG_EVENTS) placeEvents(w);
    for (auto& ab : S.jab) {
      if (ab.x >= 0) ab.x += int(off);
      ab.y += int(off);
    }
    putRange(J.ab, joff, S.jab);
    float4* jdst[10] = {J.rA, J.rB, J.stiff, J.penLin, J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang, J.restQ};
    for (int k = 0; k < 10; k++) putRange(jdst[k], joff, S.joint[k]);
    putRange(J.broken, joff, S.jbroken);
    putRange(T.color, off, S.colors);
    for (auto& pr : S.pairs) {
      pr.x += uint32_t(off);
      pr.y += uint32_t(off);
    }
    const size_t base = R.dev.pairOff;  // buffer 0
    putRange(P.pair, base, S.pairs);
    putRange(P.count, base, S.counts);
    putRange(P.basis, 3 * base, S.basis);
    putRange(P.ct, 32 * base, S.ct);
    R.which = 0;
    const int zero = 0;
    put(which + w, &zero, 4);
    put(pairN + w, &np, 4);
    put(pairN + maxWorlds + w, &zero, 4);
    put(wover + w, &zero, 4);
    uploadLarge(w);
    uploadWorldDev(w);
    R.resident = true;
    R.snap.reset();
    restores++;
    rebuildNoCollide();
    flush();
  }

  // A world's pair region overflowed: give it `need` slots (+25 %), keeping its previous state.
  void growRegion(int w, int need) {
    const int cap = need + need / 4 + 64;
    int po = slotA.alloc(cap);
    if (po < 0 && onSlotPressure) {
      onSlotPressure(cap);
      po = slotA.alloc(cap);
    }
    if (po < 0) {
      allocSlots(std::max(slotCap + cap + 1024, slotCap + slotCap / 2));
      po = slotA.alloc(cap);
    }
    WorldRec& R = W[w];
    const int np = prevPairs(w);
    const size_t k = size_t(R.which) * slotCap;
    const size_t src = k + R.dev.pairOff, dst = k + po;
    if (np) {
      CK(cudaMemcpyAsync(P.pair + dst, P.pair + src, size_t(np) * sizeof(uint2), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(P.count + dst, P.count + src, size_t(np) * sizeof(int), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(P.basis + 3 * dst, P.basis + 3 * src, size_t(np) * 3 * sizeof(float4), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(P.ct + 32 * dst, P.ct + 32 * src, size_t(np) * 32 * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    }
    slotA.release(R.dev.pairOff, R.dev.pairCap);
    R.dev.pairOff = po;
    R.dev.pairCap = cap;
    uploadWorldDev(w);
    flush();
    regrowths++;
  }

  // ------------------------------------------------------------------ call scratch
  // One grow-only device buffer for the arguments and results of the read/write entry points
  // (indices, velocities, poses), so they allocate nothing once warm; uploads go through the
  // pinned stager on the arena's stream, so a write returns without waiting for the device.
  char* io = nullptr;
  size_t ioCap = 0;
  char* ioBuffer(size_t bytes) {
    resolve();
    if (bytes > ioCap) {
      CK(cudaStreamSynchronize(s));  // earlier calls may still read the old buffer
      ioCap = bytes + bytes / 2 + 4096;
      rescratch(io, ioCap);
    }
    return io;
  }
  static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

  // ------------------------------------------------------------------ body commands
  uint32_t* editRec = nullptr;
  int2* editRanges = nullptr;
  uint32_t* editTele = nullptr;
  size_t editCap = 0;

  // Validate n 12-word records (src/native/runtime.js:59-167 stages the same checks) and queue
  // them for world w's next step. Nothing reaches the device here: the records (and the wake that
  // queued commands cause, src/native/cpu/world.js:132-133) apply at the world's next step, or at
  // a read or flushEdits, before anything else touches its state.
  void queueEdits(int w, const uint32_t* rec, int n) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (n < 0) throw Error(AVBD_E_INVALID, "negative record count");
    const WorldRec& R = W[w];
    for (int k = 0; k < n; k++) {
      const uint32_t* u = rec + 12 * size_t(k);
      if (u[0] >= uint32_t(R.nBodies)) throw Error(AVBD_E_INVALID, "body index out of range");
      if (u[1] > 6u) throw Error(AVBD_E_INVALID, "unknown body command kind");
      float f[8];
      std::memcpy(f, u + 4, sizeof(f));
      for (int i = 0; i < 8; i++)
        if (!std::isfinite(f[i])) throw Error(AVBD_E_INVALID, "body command values must be finite");
      if (u[1] == 4u && u[2] != 0u && f[4] == 0.f && f[5] == 0.f && f[6] == 0.f && f[7] == 0.f)
        throw Error(AVBD_E_INVALID, "rotation must be nonzero");
    }
    W[w].edits.insert(W[w].edits.end(), rec, rec + 12 * size_t(n));
    if (n > 0) W[w].wakePending = true;
  }

  // Upload records (word 0: body index relative to bodyOff) grouped by body in record order and
  // apply them, one thread per body (k_apply_edits).
  void uploadCommands(const std::vector<uint32_t>& recs, int bodyOff) {
    const int n = int(recs.size() / 12);
    if (n == 0) return;
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return recs[12 * size_t(a)] < recs[12 * size_t(b)]; });
    std::vector<uint32_t> sorted(recs.size());
    std::vector<int2> ranges;
    for (int k = 0; k < n; k++) {
      const uint32_t* u = recs.data() + 12 * size_t(order[k]);
      std::memcpy(sorted.data() + 12 * size_t(k), u, 48);
      if (ranges.empty() || sorted[12 * size_t(ranges.back().x)] != u[0]) ranges.push_back(make_int2(k, 0));
      ranges.back().y++;
    }
    if (size_t(n) > editCap) {
      editCap = size_t(n) + size_t(n) / 2 + 64;
      rescratch(editRec, 12 * editCap);
      rescratch(editRanges, editCap);
      rescratch(editTele, editCap);
    }
    put(editRec, sorted.data(), sorted.size() * 4);
    put(editRanges, ranges.data(), ranges.size() * sizeof(int2));
    launch_apply_edits(B, editRec, editRanges, int(ranges.size()), bodyOff, ctl, s);
  }
  // Teleported bodies of world w (records with world-local indices) lose the warm start of their
  // pairs in the world's last pair region.
  void dropTeleported(int w, const std::vector<uint32_t>& recs) {
    std::vector<uint32_t> tele;
    for (size_t k = 0; k < recs.size() / 12; k++)
      if (recs[12 * k + 1] == 4u) tele.push_back(recs[12 * k]);
    if (tele.empty()) return;
    std::sort(tele.begin(), tele.end());
    tele.erase(std::unique(tele.begin(), tele.end()), tele.end());
    const WorldRec& R = W[w];
    if (tele.size() > editCap) {
      editCap = tele.size() + tele.size() / 2 + 64;
      rescratch(editRec, 12 * editCap);
      rescratch(editRanges, editCap);
      rescratch(editTele, editCap);
    }
    put(editTele, tele.data(), tele.size() * 4);
    launch_drop_contacts(P, size_t(R.which) * slotCap + R.dev.pairOff, pairN + size_t(R.which) * maxWorlds + w, R.dev.pairCap,
                         editTele, int(tele.size()), R.dev.bodyOff, ctl, s);
  }

  // Every queued tick final, then world w's queued commands applied: the start of every call
  // that reads or changes world w's state outside a step.
  void touch(int w) {
    resolve();
    flushEdits(w);
  }

  // Apply world w's queued records now (the reference applies them at its next step, or at
  // flushEdits and before reads, src/native/cpu/world.js:566-575): grouped by body in record order,
  // one thread per body; teleported bodies lose the warm start of their pairs.
  void flushEdits(int w) {
    WorldRec& R = W[w];
    if (R.edits.empty() && !R.wakePending) return;
    if (!R.resident) throw Error(AVBD_E_STATE, "world is evicted");
    resolve();
    if (R.wakePending && (R.dev.flags & FLAG_SLEEP) && R.nBodies) launch_sleep_wake(B, R.dev.bodyOff, R.nBodies, ctl, s);
    R.wakePending = false;
    std::vector<uint32_t> recs;
    recs.swap(R.edits);
    uploadCommands(recs, R.dev.bodyOff);
    dropTeleported(w, recs);
    CK(cudaGetLastError());
  }

  // ------------------------------------------------------------------ profiling
  cudaEvent_t event() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    return e;
  }
  cudaEvent_t mark() {
    cudaEvent_t e = event();
    CK(cudaEventRecord(e, s));
    return e;
  }
  void span(int cls, cudaEvent_t a, cudaEvent_t b) { recs.push_back(Rec{cls, a, b}); }
  void harvest() {
    for (const Rec& r : recs) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) profMs[r.cls] += ms;
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    recs.clear();
  }
  void profile(bool on) {
    resolve();
    CK(cudaStreamSynchronize(s));
    harvest();
    prof = on;
    for (double& v : profMs) v = 0;
    for (double& v : profBytes) v = 0;
    profPrimalLaunches = 0;
    profSteps = 0;
    if (!traffic) traffic = dalloc<unsigned long long>(3);
  }
  void profileRead(avbd_profile* o) {
    resolve();
    CK(cudaStreamSynchronize(s));
    harvest();
    std::memset(o, 0, sizeof(*o));
    o->steps = profSteps;
    o->ms_collide = profMs[P_COLLIDE];
    o->ms_topology = profMs[P_TOPO];
    o->ms_primal = profMs[P_PRIMAL];
    o->ms_dual = profMs[P_DUAL];
    o->ms_other = profMs[P_OTHER];
    o->primal_launches = profPrimalLaunches;
    o->launches = launches_total();
    o->bytes_primal = profBytes[0];
    o->bytes_dual = profBytes[1];
    o->bytes_collide = profBytes[2];
    o->graph_captures = graphCaptures;
    o->graph_replays = graphReplays;
    o->graphs_on = graphsOn ? 1 : 0;
    o->ticks_held = int32_t(ticksHeld);
    std::vector<cudaEvent_t> freed;
    tuner.harvest(true, freed);
    for (cudaEvent_t ev : freed) pool.push_back(ev);
    o->tuned = lastTuned ? 1 : 0;
    o->solve_queue = solveCfg.queue;
    o->solve_waves = solveCfg.waves;
    o->solve_blocks = solveCfg.blocks;
    o->radix_bits = radixBits;
    o->solve_tile = solveCfg.tile;
  }

  // ------------------------------------------------------------------ ticks
  // bounce-pass scratch (worlds with FLAG_RESTITUTION): incoming velocities per body, state per
  // active pair; allocated on first use at the arena's capacities
  // island-sleeping scratch (worlds with FLAG_SLEEP), allocated on first use
  void ensureSleep() {
    if (sleepBodies < size_t(bodyCap)) {
      CK(cudaStreamSynchronize(s));
      rescratch(SB.parent, size_t(bodyCap));
      rescratch(SB.flags, size_t(bodyCap));
      sleepBodies = size_t(bodyCap);
    }
    if (sleepWorlds < size_t(maxWorlds)) {
      CK(cudaStreamSynchronize(s));
      rescratch(SB.wake, size_t(maxWorlds));
      sleepWorlds = size_t(maxWorlds);
    }
    if (!SB.err) {
      SB.err = dalloc<int>(1);
      CK(cudaMemsetAsync(SB.err, 0, sizeof(int), s));
    }
  }

  // Wake every body of world w (src/native/cpu/sleeping.js wake): queued commands, pose and
  // velocity writes and sleep settings do this, as the reference's world does.
  void wakeWorld(int w) {
    WorldRec& R = W[w];
    if (!(R.dev.flags & FLAG_SLEEP) || R.nBodies == 0) return;
    if (R.resident) {
      resolve();
      launch_sleep_wake(B, R.dev.bodyOff, R.nBodies, ctl, s);
      CK(cudaGetLastError());
    } else if (R.snap) {
      for (int& b : R.snap->sleep) b &= ~SLEEP_ASLEEP;
      std::fill(R.snap->sleepTime.begin(), R.snap->sleepTime.end(), 0.f);
    }
  }

  // Sleeping on/off for world w (enableSleeping / disableSleeping of src/native/cpu/world.js:
  // 869-878); turning it off or changing the thresholds wakes the world first.
  void setSleeping(int w, bool on, float speed, float delay) {
    resolve();
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (on && (!(speed > 0.f) || !(delay > 0.f) || !std::isfinite(speed) || !std::isfinite(delay)))
      throw Error(AVBD_E_INVALID, "Sleep thresholds must be positive and finite");
    wakeWorld(w);
    WorldDev& D = W[w].dev;
    D.flags = on ? (D.flags | FLAG_SLEEP) : (D.flags & ~FLAG_SLEEP);
    if (on) {
      D.sleepSpeed = speed;
      D.sleepDelay = delay;
    }
    if (W[w].resident) uploadWorldDev(w);
  }

  // allowSleep of one body (setSleepEnabled, src/native/cpu/world.js:859-867): enabling it turns
  // sleeping on with the default thresholds if it was off; the world wakes.
  void setSleepAllowed(int w, int body, bool allowed) {
    resolve();
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    WorldRec& R = W[w];
    if (body < 0 || body >= R.nBodies) throw Error(AVBD_E_INVALID, "body index out of range");
    if (allowed && !(R.dev.flags & FLAG_SLEEP)) setSleeping(w, true, 0.08f, 0.6f);
    if (R.resident) {
      int bits = 0;
      get(&bits, B.sleep + R.dev.bodyOff + body, 4);
      bits = allowed ? (bits | SLEEP_ALLOW) : (bits & ~SLEEP_ALLOW);
      put(B.sleep + R.dev.bodyOff + body, &bits, 4);
    } else if (R.snap) {
      int& bits = R.snap->sleep[body];
      bits = allowed ? (bits | SLEEP_ALLOW) : (bits & ~SLEEP_ALLOW);
    }
    wakeWorld(w);
  }

  // Per-body sleep flags (1: asleep) and quiet times of world w; returns the sleeping count.
  int sleepState(int w, int32_t* asleep, float* time) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    WorldRec& R = W[w];
    if (R.resident) touch(w);  // queued commands (and the wake they cause) apply before a read
    const size_t n = size_t(R.nBodies);
    std::vector<int> bits(n);
    std::vector<float> t(n);
    if (R.resident) {
      if (n) {
        get(bits.data(), B.sleep + R.dev.bodyOff, n * 4);
        get(t.data(), B.sleepTime + R.dev.bodyOff, n * 4);
      }
    } else if (R.snap) {
      bits = R.snap->sleep;
      t = R.snap->sleepTime;
    }
    int count = 0;
    for (size_t i = 0; i < n; i++) {
      const int a = (bits[i] & SLEEP_ASLEEP) ? 1 : 0;
      count += a;
      if (asleep) asleep[i] = a;
      if (time) time[i] = t[i];
    }
    return count;
  }

  // Load per-body sleep flags and quiet times into world w (state import for tests and tools).
  void setSleepState(int w, const int32_t* asleep, const float* time) {
    const WorldRec& R = resident(w);
    const size_t n = size_t(R.nBodies);
    if (!n) return;
    std::vector<int> bits(n);
    get(bits.data(), B.sleep + R.dev.bodyOff, n * 4);
    for (size_t i = 0; i < n; i++) {
      if (asleep) bits[i] = asleep[i] ? (bits[i] | SLEEP_ASLEEP) : (bits[i] & ~SLEEP_ASLEEP);
    }
    put(B.sleep + R.dev.bodyOff, bits.data(), n * 4);
    if (time) put(B.sleepTime + R.dev.bodyOff, time, n * 4);
    flush();
  }

  // ---------------------------------------------------------------- contact events
  size_t eventBytes() const {
    size_t b = 0;
    for (const WorldRec& R : W)
      if (R.evDev) b += size_t(R.evCap) * EVENT_FLOAT4 * 16;
    return b;
  }
  // per-world event arrays at the arena's world capacity
  void ensureEventArrays() {
    if (evWorlds >= size_t(maxWorlds)) return;
    const size_t o = evWorlds, nw = size_t(maxWorlds);
    if (o == 0) {
      EV.region = dalloc<float4*>(nw);
      EV.count = dalloc<int>(nw);
      EV.cap = dalloc<int>(nw);
      EV.step = dalloc<int>(nw);
    } else {
      regrow(EV.region, o, nw);
      regrow(EV.count, o, nw);
      regrow(EV.cap, o, nw);
      regrow(EV.step, o, nw);
    }
    evWorlds = nw;
  }
  // device region of a resident world with events on; its counters restart
  void placeEvents(int w) {
    WorldRec& R = W[w];
    ensureEventArrays();
    if (!R.evDev) R.evDev = dalloc<float4>(size_t(R.evCap) * EVENT_FLOAT4);
    const int zero = 0, step = int(R.steps);
    put(EV.region + w, &R.evDev, sizeof(float4*));
    put(EV.count + w, &zero, 4);
    put(EV.cap + w, &R.evCap, 4);
    put(EV.step + w, &step, 4);
  }
  // watchContacts (src/native/solver3D.js:256-284): the first call turns events on with room for
  // maxEvents per read and watches every body unless `select`; with `select`, exactly the given
  // bodies are watched. A newly watched body begins its current contacts at the next step.
  void watchContacts(int w, const uint32_t* idx, int n, int maxEvents, bool select) {
    resolve();
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (maxEvents < 1) throw Error(AVBD_E_INVALID, "Contact capacities must be positive integers");
    WorldRec& R = W[w];
    for (int k = 0; select && k < n; k++)
      if (idx[k] >= uint32_t(R.nBodies)) throw Error(AVBD_E_INVALID, "body index out of range");
    const bool first = !(R.dev.flags & FLAG_EVENTS);
    if (!first && !select) return;
    const size_t nb = size_t(R.nBodies);
    std::vector<uint32_t> words(nb), prev(nb);
    if (R.resident) {
      if (nb) get(words.data(), B.watch + R.dev.bodyOff, nb * 4);
    } else {
      words = R.snap->watch;
    }
    std::vector<char> on(nb, select ? 0 : 1);
    for (int k = 0; select && k < n; k++) on[idx[k]] = 1;
    for (size_t i = 0; i < nb; i++) words[i] = (words[i] & ~WATCH_ON) | (on[i] ? WATCH_ON : 0u);
    if (first) {
      R.evCap = maxEvents;
      R.dev.flags |= FLAG_EVENTS;
      if (R.resident) {
        placeEvents(w);
        uploadWorldDev(w);
      }
    }
    if (R.resident) {
      if (nb) put(B.watch + R.dev.bodyOff, words.data(), nb * 4);
      if (first && nb) put(B.watchPrev + R.dev.bodyOff, prev.data(), nb * 4);
      flush();
    } else {
      R.snap->watch = words;
      if (first) R.snap->watchPrev = prev;
    }
  }
  // resetContactHistory (src/vendor/three-avbd-lib/contacts.ts resetBodies): new lifetimes for
  // the given bodies (ascending, unique): their contacts begin afresh, none of the old ones end.
  void resetContactHistory(int w, const uint32_t* idx, int n) {
    resolve();
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    WorldRec& R = W[w];
    long long prev = -1;
    for (int k = 0; k < n; k++) {
      if ((long long)idx[k] <= prev || idx[k] >= uint32_t(R.nBodies))
        throw Error(AVBD_E_INVALID, "Contact reset slots must be unique, ascending and in range");
      prev = idx[k];
    }
    if (n == 0) return;
    const size_t nb = size_t(R.nBodies);
    std::vector<uint32_t> words(nb);
    if (R.resident) get(words.data(), B.watch + R.dev.bodyOff, nb * 4);
    else words = R.snap->watch;
    for (int k = 0; k < n; k++) words[idx[k]] += 2u;
    if (R.resident) {
      put(B.watch + R.dev.bodyOff, words.data(), nb * 4);
      flush();
    } else {
      R.snap->watch = words;
    }
  }
  void drainEvents(int w) {
    WorldRec& R = W[w];
    if (!(R.dev.flags & FLAG_EVENTS) || !R.resident || !R.evDev) return;
    int cnt = 0;
    get(&cnt, EV.count + w, 4);
    const int n = std::min(cnt, R.evCap);
    if (n > 0) {
      const size_t at = R.evHost.size();
      R.evHost.resize(at + 12 * size_t(n));
      get(R.evHost.data() + at, R.evDev, size_t(n) * EVENT_FLOAT4 * 16);
    }
    R.evDropped += cnt - n;
    const int zero = 0;
    put(EV.count + w, &zero, 4);
    flush();
  }
  // readContactEvents: the events since the last read in step order (within a step: begins then
  // ends, each by (a, b)), 12 words each: kind, a, b, step, point xyz, impulse, normal xyz, 0.
  // With out == nullptr or cap too small only the count is returned and nothing is consumed.
  long long readEvents(int w, uint32_t* out, long long cap, long long* dropped) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    drainEvents(w);
    WorldRec& R = W[w];
    const long long n = (long long)(R.evHost.size() / 12);
    if (dropped) *dropped = R.evDropped;
    if (!out || cap < n) return n;
    std::vector<long long> order(static_cast<size_t>(n));
    for (long long k = 0; k < n; k++) order[size_t(k)] = k;
    const uint32_t* e = R.evHost.data();
    std::stable_sort(order.begin(), order.end(), [&](long long x, long long y) {
      const uint32_t* a = e + 12 * x;
      const uint32_t* b = e + 12 * y;
      if (a[3] != b[3]) return a[3] < b[3];
      if (a[0] != b[0]) return a[0] < b[0];
      if (a[1] != b[1]) return a[1] < b[1];
      return a[2] < b[2];
    });
    for (long long k = 0; k < n; k++) std::memcpy(out + 12 * k, e + 12 * order[size_t(k)], 48);
    R.evHost.clear();
    R.evDropped = 0;
    return n;
  }

  // ---------------------------------------------------------------- joints and filters
  // readJoints (src/vendor/three-avbd-lib/solver3D.ts:1456-1458, record layout
  // avbd3d/gpu/layout.ts:27-36, infinities as +-3e38 as src/native/cpu/world.js:603-660): 32 floats
  // per joint or spring in creation order: penalty lin (w: linear stiffness, 0 once broken),
  // penalty ang (w: angular stiffness, 0 once broken), lambda lin (w: fracture), lambda ang
  // (w: torque arm), C0 lin, C0 ang, rA (w: spring rest length), rB.
  void readJoints(int w, float* out) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    touch(w);
    const WorldRec& R = resident(w);
    const size_t nj = size_t(R.nJoints), off = size_t(R.dev.jointOff);
    if (!nj) return;
    std::vector<float4> f[10];
    const float4* src[10] = {J.rA, J.rB, J.stiff, J.penLin, J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang, J.restQ};
    for (int k = 0; k < 9; k++) getRange(f[k], src[k], off, nj);
    std::vector<int> broken;
    getRange(broken, J.broken, off, nj);
    auto fin = [](float x) { return x == INFINITY ? 3e38f : (x == -INFINITY ? -3e38f : x); };
    for (size_t j = 0; j < nj; j++) {
      float* o = out + 32 * j;
      const float4 ra = f[0][j], rb = f[1][j], st = f[2][j];
      int kind;
      std::memcpy(&kind, &ra.w, 4);
      if (kind == KIND_MOTOR || kind == KIND_LIMIT) {  // src/native/cpu/world.js:622-636
        const float4 pl = f[3][j], ll = f[5][j], c0 = f[7][j], c1 = f[8][j];
        const float rec[32] = {pl.x, pl.y, 0.f, broken[j] ? 0.f : 1.f, 0.f, 0.f, 0.f, 0.f,
                               ll.x, ll.y, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f,
                               c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w,
                               ra.x, ra.y, ra.z, st.x, rb.x, rb.y, rb.z, st.y};
        std::memcpy(o, rec, sizeof(rec));
        continue;
      }
      const float4 blocks[6] = {f[3][j], f[4][j], f[5][j], f[6][j], f[7][j], f[8][j]};
      for (int b = 0; b < 6; b++) {
        o[4 * b] = blocks[b].x;
        o[4 * b + 1] = blocks[b].y;
        o[4 * b + 2] = blocks[b].z;
        o[4 * b + 3] = 0.f;
      }
      o[3] = broken[j] ? 0.f : fin(st.x);
      o[7] = broken[j] ? 0.f : fin(st.y);
      o[11] = fin(st.z);
      o[15] = st.w;
      if (kind == KIND_SPRING) {  // stiffness; strain and tension limits (0: none) as appGpuSolver3D.js:826-833
        o[7] = 0.f;
        o[11] = st.y < INFINITY ? st.y : 0.f;
        o[15] = st.z < INFINITY ? st.z : 0.f;
      }
      o[24] = ra.x; o[25] = ra.y; o[26] = ra.z; o[27] = rb.w;
      o[28] = rb.x; o[29] = rb.y; o[30] = rb.z; o[31] = 0.f;
    }
  }

  // setFilters (src/native/cpu/world.js:327-341): collision group and collidesWith of the given
  // bodies; the world wakes.
  void setFilters(int w, const uint32_t* idx, int n, const uint32_t* groups, const uint32_t* masks) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (n < 0) throw Error(AVBD_E_INVALID, "negative count");
    const WorldRec& R = resident(w);
    for (int k = 0; k < n; k++)
      if (idx[k] >= uint32_t(R.nBodies)) throw Error(AVBD_E_INVALID, "body index out of range");
    if (n == 0) return;
    const size_t nb = size_t(R.nBodies), off = size_t(R.dev.bodyOff);
    std::vector<int4> meta;
    getRange(meta, B.meta, off, nb);
    for (int k = 0; k < n; k++) {
      meta[idx[k]].z = int(groups[k]);
      meta[idx[k]].w = int(masks[k]);
    }
    putRange(B.meta, off, meta);
    flush();
    wakeWorld(w);
  }

  // setRestitution (src/native/cpu/world.js:343-351): restitution 0..1 of the given bodies; the
  // bounce pass runs while any body of the world has restitution > 0; the world wakes.
  void setRestitution(int w, const uint32_t* idx, int n, const float* values) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (n < 0) throw Error(AVBD_E_INVALID, "negative count");
    const WorldRec& R = resident(w);
    for (int k = 0; k < n; k++) {
      if (idx[k] >= uint32_t(R.nBodies)) throw Error(AVBD_E_INVALID, "body index out of range");
      if (!(values[k] >= 0.f && values[k] <= 1.f)) throw Error(AVBD_E_INVALID, "restitution must be between 0 and 1");
    }
    if (n == 0) return;
    const size_t nb = size_t(R.nBodies), off = size_t(R.dev.bodyOff);
    std::vector<float> e;
    getRange(e, B.restitution, off, nb);
    for (int k = 0; k < n; k++) e[idx[k]] = values[k];
    putRange(B.restitution, off, e);
    bool any = false;
    for (float x : e) any |= x > 0.f;
    WorldDev& D = W[w].dev;
    D.flags = any ? (D.flags | FLAG_RESTITUTION) : (D.flags & ~FLAG_RESTITUTION);
    uploadWorldDev(w);
    flush();
    wakeWorld(w);
  }

  // setMotor (src/gpu/appGpuSolver3D.js:547-562, src/native/cpu/world.js:360-388): a new speed
  // and/or torque bound of motor `slot` (joint index); the world wakes. mask bit 0: speed, bit 1:
  // torque bound.
  void setMotor(int w, int slot, int mask, float speed, float maxTorque) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    touch(w);
    const WorldRec& R = resident(w);
    if (slot < 0 || slot >= R.nJoints) throw Error(AVBD_E_INVALID, "Motor needs an active motor slot");
    const size_t j = size_t(R.dev.jointOff) + size_t(slot);
    const float4 ra = fetch(J.rA, j, 1)[0];
    float4 st = fetch(J.stiff, j, 1)[0];
    int kind;
    std::memcpy(&kind, &ra.w, 4);
    if (kind != KIND_MOTOR) throw Error(AVBD_E_INVALID, "Motor needs an active motor slot");
    if ((mask & 1) && !std::isfinite(speed)) throw Error(AVBD_E_INVALID, "Motor speed must be finite");
    if ((mask & 2) && !(std::isfinite(maxTorque) && maxTorque >= 0.f)) throw Error(AVBD_E_INVALID, "maxTorque must be nonnegative");
    if (mask & 1) st.x = speed;
    if (mask & 2) st.y = maxTorque;
    put(J.stiff + j, &st, 16);
    flush();
    wakeWorld(w);
  }

  // setSensor (src/native/cpu/world.js:342-350): the bodies become (enabled) or stop being
  // triggers; the world wakes.
  void setSensor(int w, const uint32_t* idx, int n, bool enabled) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (n < 0) throw Error(AVBD_E_INVALID, "negative count");
    touch(w);
    WorldRec& R = W[w];
    resident(w);
    for (int k = 0; k < n; k++)
      if (idx[k] >= uint32_t(R.nBodies)) throw Error(AVBD_E_INVALID, "A live body index is required");
    if (n == 0) return;
    const size_t nb = size_t(R.nBodies), off = size_t(R.dev.bodyOff);
    std::vector<int> bits;
    getRange(bits, B.sleep, off, nb);
    for (int k = 0; k < n; k++) bits[idx[k]] = enabled ? (bits[idx[k]] | BODY_TRIGGER) : (bits[idx[k]] & ~BODY_TRIGGER);
    putRange(B.sleep, off, bits);
    R.triggers = false;
    for (int b : bits) R.triggers |= (b & BODY_TRIGGER) != 0;
    flush();
    wakeWorld(w);
  }

  // setSpringMaterial (src/gpu/appGpuSolver3D.js:810-835, src/native/cpu/world.js:495-501): the
  // strain and tension limits of the live spring `slot` (positive, or INFINITY: none); the world
  // wakes. mask bit 0: breakStrain, bit 1: breakForce.
  void setSpringMaterial(int w, int slot, int mask, float breakStrain, float breakForce) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    for (int k = 0; k < 2; k++) {
      const float v = k ? breakForce : breakStrain;
      if ((mask >> k & 1) && !(v > 0.f)) throw Error(AVBD_E_INVALID, k ? "breakForce must be positive or Infinity" : "breakStrain must be positive or Infinity");
    }
    touch(w);
    const WorldRec& R = resident(w);
    if (slot < 0 || slot >= R.nJoints) throw Error(AVBD_E_INVALID, "Spring material requires an active spring slot");
    const size_t j = size_t(R.dev.jointOff) + size_t(slot);
    const float4 ra = fetch(J.rA, j, 1)[0];
    float4 st = fetch(J.stiff, j, 1)[0];
    int kind;
    std::memcpy(&kind, &ra.w, 4);
    if (kind != KIND_SPRING || fetch(J.broken, j, 1)[0]) throw Error(AVBD_E_INVALID, "Spring material requires an active spring slot");
    if (mask & 1) st.y = breakStrain;
    if (mask & 2) st.z = breakForce;
    put(J.stiff + j, &st, 16);
    flush();
    wakeWorld(w);
  }

  // setWorldAnchor (src/gpu/appGpuSolver3D.js:928-941): the world point of the live world joint
  // `slot` (a joint whose first body is the world) moves to `point`; the world wakes.
  void setWorldAnchor(int w, int slot, const float* point) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (!(std::isfinite(point[0]) && std::isfinite(point[1]) && std::isfinite(point[2])))
      throw Error(AVBD_E_INVALID, "A world joint and finite xyz anchor are required");
    touch(w);
    const WorldRec& R = resident(w);
    if (slot < 0 || slot >= R.nJoints) throw Error(AVBD_E_INVALID, "A world joint and finite xyz anchor are required");
    const size_t j = size_t(R.dev.jointOff) + size_t(slot);
    float4 ra = fetch(J.rA, j, 1)[0];
    int kind;
    std::memcpy(&kind, &ra.w, 4);
    if (kind != KIND_JOINT || fetch(J.ab, j, 1)[0].x >= 0) throw Error(AVBD_E_INVALID, "A world joint and finite xyz anchor are required");
    ra.x = point[0];
    ra.y = point[1];
    ra.z = point[2];
    put(J.rA + j, &ra, 16);
    flush();
    wakeWorld(w);
  }

  // captureConstraintFrames (src/native/cpu/world.js:474-492): for each entry, the live joint's
  // rest rotation (spring = 0) or the live spring's rest length (spring = 1) taken again from the
  // current poses, after queued commands apply; the world wakes.
  void captureFrames(int w, const int32_t* slots, const int32_t* spring, int n) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (n < 0) throw Error(AVBD_E_INVALID, "negative count");
    const WorldRec& R = resident(w);
    if (n == 0) return;
    const size_t off = size_t(R.dev.jointOff), nj = size_t(R.nJoints);
    std::vector<float4> ra;
    std::vector<int> broken;
    getRange(ra, J.rA, off, nj);
    getRange(broken, J.broken, off, nj);
    for (int k = 0; k < n; k++) {
      int kind = -1;
      if (slots[k] >= 0 && size_t(slots[k]) < nj) std::memcpy(&kind, &ra[slots[k]].w, 4);
      if (kind != (spring[k] ? KIND_SPRING : KIND_JOINT) || broken[slots[k]])
        throw Error(AVBD_E_INVALID, "A live spring or joint slot is required");
    }
    touch(w);
    for (int k = 0; k < n; k++) launch_joint_capture(B, J, int(off) + slots[k], spring[k] ? 1 : 0, s);
    CK(cudaGetLastError());
    flush();
    wakeWorld(w);
  }

  // releaseJoints (src/native/cpu/world.js:397-410, src/vendor/three-avbd-lib/solver3D.ts:1173-1193):
  // the joints, springs or angular rows at `slots` stop acting for good: marked broken (no rows,
  // no island link, their bodies collide again from the next step) with their penalties and
  // lambdas zeroed; the world wakes.
  void releaseJoints(int w, const int32_t* slots, int n) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (n < 0) throw Error(AVBD_E_INVALID, "negative count");
    touch(w);
    const WorldRec& R = resident(w);
    for (int k = 0; k < n; k++)
      if (slots[k] < 0 || slots[k] >= R.nJoints) throw Error(AVBD_E_INVALID, "A live constraint slot is required");
    if (n == 0) return;
    const size_t off = size_t(R.dev.jointOff), nj = size_t(R.nJoints);
    std::vector<int> broken;
    getRange(broken, J.broken, off, nj);
    for (float4* a : {J.penLin, J.penAng, J.lamLin, J.lamAng}) {
      std::vector<float4> v;
      getRange(v, a, off, nj);
      for (int k = 0; k < n; k++) v[slots[k]] = make_float4(0.f, 0.f, 0.f, 0.f);
      putRange(a, off, v);
    }
    for (int k = 0; k < n; k++) broken[slots[k]] = 1;
    putRange(J.broken, off, broken);
    flush();
    wakeWorld(w);
  }

  // ---------------------------------------------------------------- shape casts
  // raycastAll / sphereCastAll against world w's current poses; queued commands apply first
  // (src/native/solver3D.js:244-251). queries: 8 floats each (origin, max distance, direction,
  // radius); hits: 8 floats each (normal, distance or -1, body index as bits, 0, 0, 0).
  void cast(int w, const float* queries, int n, const avbd_cast_filter& filt, float* hits) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (n < 0) throw Error(AVBD_E_INVALID, "negative count");
    if (filt.n_ignore < 0 || filt.n_ignore > 16) throw Error(AVBD_E_INVALID, "Queries can ignore up to 16 live body indices");
    const WorldRec& R0 = W[w];
    for (int k = 0; k < filt.n_ignore; k++)
      if (filt.ignore[k] >= uint32_t(R0.nBodies)) throw Error(AVBD_E_INVALID, "Queries can ignore up to 16 live body indices");
    std::vector<CastQuery> qs(static_cast<size_t>(n));
    for (int k = 0; k < n; k++) {
      const float* q = queries + 8 * size_t(k);
      for (int j = 0; j < 8; j++)
        if (!std::isfinite(q[j])) throw Error(AVBD_E_INVALID, "A query requires finite components and a nonzero direction");
      const double len = std::sqrt(double(q[4]) * q[4] + double(q[5]) * q[5] + double(q[6]) * q[6]);
      if (!(len > 0)) throw Error(AVBD_E_INVALID, "A query requires finite components and a nonzero direction");
      if (q[7] < 0.f || q[3] < 0.f) throw Error(AVBD_E_INVALID, "Query radius and maximum distance must be finite and nonnegative");
      qs[k].o = make_float4(q[0], q[1], q[2], q[3]);
      qs[k].d = make_float4(float(q[4] / len), float(q[5] / len), float(q[6] / len), q[7]);
    }
    if (n == 0) return;
    touch(w);
    const WorldRec& R = resident(w);
    CastFilter f{};
    f.collidesWith = filt.collides_with;
    f.membership = filt.membership;
    f.hasMembership = filt.has_membership != 0;
    f.includeTriggers = filt.include_triggers != 0;
    f.nIgnore = filt.n_ignore;
    for (int k = 0; k < filt.n_ignore; k++) f.ignore[k] = filt.ignore[k];
    const size_t qb = align256(size_t(n) * sizeof(CastQuery)), bb = align256(size_t(n) * 8);
    char* io = ioBuffer(qb + bb + size_t(n) * 32);
    CastQuery* dq = reinterpret_cast<CastQuery*>(io);
    unsigned long long* best = reinterpret_cast<unsigned long long*>(io + qb);
    float4* out = reinterpret_cast<float4*>(io + qb + bb);
    put(dq, qs.data(), size_t(n) * sizeof(CastQuery));
    launch_cast(B, R.dev.bodyOff, R.nBodies, dq, n, f, best, out, s);
    CK(cudaGetLastError());
    get(hits, out, size_t(n) * 32);
  }

  void ensureBounce() {
    if (bounceBodies < size_t(bodyCap)) {
      CK(cudaStreamSynchronize(s));
      rescratch(BB.inVel, size_t(bodyCap));
      rescratch(BB.inAng, size_t(bodyCap));
      bounceBodies = size_t(bodyCap);
    }
    if (bounceSlots < size_t(slotCap)) {
      CK(cudaStreamSynchronize(s));
      rescratch(BB.ra, size_t(slotCap));
      rescratch(BB.rb, size_t(slotCap));
      rescratch(BB.nk, size_t(slotCap));
      rescratch(BB.delta, size_t(slotCap));
      bounceSlots = size_t(slotCap);
    }
  }

  // ------------------------------------------------------------------ tick protocol
  // A tick is queued without waiting for the device (the reference's step never waits either,
  // src/native/solver3D.js:350-359). Its capacities (pair regions, work items) are chosen on the
  // host before it is queued; its gate holds it on the device when they do not suffice (TickCtl).
  // Every queued tick stays in tickLog, with the host state its worlds had before it, until it is
  // known to have completed: resolve() waits for the stream, and when a tick was held it grows the
  // capacities and queues the held ticks again from that state, so the results are those of a
  // run with enough room from the start. Reads and every other call that touches world state
  // resolve first.
  TickCtl* ctl = nullptr;      // device
  TickCtl* ctlHost = nullptr;  // pinned mirror, written by the last copy of every tick
  struct TickPre {  // a stepped world's host state before the tick, and the commands queued for it
    int w = 0, which = 0, sinceBuild = 0;
    long long steps = 0;
    bool built = false, wake = false;
    std::vector<uint32_t> edits;
  };
  // Poses of some stepped worlds right after a tick, gathered on the device and copied to pinned
  // host memory in stream order (an owner's replies to requests that the tick completes); the
  // tags are reported (confirmedTags) once the tick is confirmed, and a held tick's gather is
  // queued again with it.
  struct TickReply {
    std::vector<int4> seg;  // (first body, bodies, first row, 0), ascending rows
    int rows = 0;
    float4* dev = nullptr;   // 2 per row
    float4* host = nullptr;  // pinned, 2 per row
    std::vector<long long> tags;
  };
  struct TickLog {
    std::vector<int> act;
    std::vector<TickPre> pre;
    TickReply reply;
    cudaEvent_t done = nullptr;
  };
  std::vector<long long> confirmedTags;  // tags of confirmed ticks' replies, in order
  int4* replySeg = nullptr;
  size_t replySegCap = 0;
  std::deque<TickLog> tickLog;  // queued ticks not yet confirmed, in queue order
  long long logBase = 0;        // TickCtl::ticksDone before the first entry of tickLog
  static constexpr size_t MAX_IN_FLIGHT = 24;
  std::vector<cudaEvent_t> tickEvents;
  bool statsValid = false;  // the last tick's active-pair list still indexes the pair buffers
  SolveConfig solveCfg;          // the solve loop's schedule (solve.cu launch_solve)
  int radixBits = 8;             // digit width of the tree builds' Morton sort
  Tuner tuner;                   // run-time choice of both (tuner.hpp)
  bool lastTuned = false;        // the last tick's class had its choices
  int* queueScratch = nullptr;   // the tile queue's per-world counters (solve_queue_ints)

  bool hostHeld() const { return *(volatile const int*)&ctlHost->held != 0; }
  cudaEvent_t tickEvent() {
    if (!tickEvents.empty()) {
      cudaEvent_t e = tickEvents.back();
      tickEvents.pop_back();
      return e;
    }
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return e;
  }
  void dropLogFront() {  // the front tick is confirmed (or the log is abandoned after an error)
    const TickLog& f = tickLog.front();
    confirmedTags.insert(confirmedTags.end(), f.reply.tags.begin(), f.reply.tags.end());
    if (tickLog.front().done) tickEvents.push_back(tickLog.front().done);
    tickLog.pop_front();
    logBase++;
  }

  // Work items of a tick: grown ahead when the largest need seen comes close to the capacity
  // (a tick that still overflows is held and re-run).
  void growItems(size_t cap) {
    if (cap <= itemCap) return;
    CK(cudaStreamSynchronize(s));
    dfree(T.itemRef);
    T.itemRef = nullptr;
    T.itemRef = dalloc<int4>(cap);
    itemCap = cap;
  }
  void ensureItems(int nb) {
    const size_t seen = size_t(std::max(ctlHost->itemsNeed, 0));
    if (itemCap < size_t(16) * size_t(nb) + 1024) growItems(size_t(16) * size_t(nb) + 1024);
    if (seen > itemCap - itemCap / 5) growItems(seen + seen / 2 + 1024);
  }

  // Confirmed ticks (completed, no hold seen) leave the log; with MAX_IN_FLIGHT ticks queued the
  // host waits for the oldest (the reference's queue is bounded by its device the same way).
  void trimLog() {
    while (!tickLog.empty()) {
      cudaEvent_t d = tickLog.front().done;
      if (cudaEventQuery(d) != cudaSuccess) {
        if (tickLog.size() < MAX_IN_FLIGHT) break;
        CK(cudaEventSynchronize(d));
      }
      if (hostHeld()) {  // the mirror is at least as new as this tick's last copy
        resolve();
        return;
      }
      dropLogFront();
    }
  }

  // Wait for every queued tick without growing anything: false when a tick was held (making it
  // final needs growth, which allocates).
  bool settle() {
    CK(cudaStreamSynchronize(s));
    if (hostHeld()) return false;
    while (!tickLog.empty()) dropLogFront();
    logBase = ctlHost->ticksDone;
    return true;
  }

  // Make every queued tick final: wait for the stream; if a tick was held, grow what overflowed
  // and queue the held ticks again (bounded: a capacity that fails to converge is an error).
  void resolve() {
    if (tickLog.empty() && !hostHeld()) return;
    for (int round = 0;; round++) {
      CK(cudaStreamSynchronize(s));
      stageRetire(true);
      TickCtl c;
      std::memcpy(&c, (const void*)ctlHost, sizeof(c));
      if (c.waitFail) {
        // a bounded wait of the tile queue ran out: the tick's solve is incomplete; the flag stays
        // set (ticks keep stopping at it) and every later call reports it
        while (!tickLog.empty()) dropLogFront();
        logBase = c.ticksDone;
        throw Error(AVBD_E_STATE, "the persistent solve's wait limit ran out (TickCtl::waitFail); the world state is not valid");
      }
      if (!c.held) {
        while (!tickLog.empty()) dropLogFront();
        logBase = c.ticksDone;
        break;
      }
      if (round >= 8) throw Error(AVBD_E_CAPACITY, "pair regions or work items did not converge");
      // timings of held ticks (whose solve did nothing) must not reach the autotuner
      {
        std::vector<cudaEvent_t> freed;
        tuner.discard(freed);
        for (cudaEvent_t ev : freed) pool.push_back(ev);
      }
      const long long good = c.ticksDone - logBase;
      ticksHeld += (long long)tickLog.size() - good;
      if (good < 0 || good >= (long long)tickLog.size()) throw Error(AVBD_E_STATE, "tick protocol out of step");
      for (long long k = 0; k < good; k++) dropLogFront();
      std::vector<TickLog> again;
      while (!tickLog.empty()) {
        again.push_back(std::move(tickLog.front()));
        tickLog.pop_front();
      }
      // the held ticks' worlds go back to their state before the first held tick that stepped them
      for (auto it = again.rbegin(); it != again.rend(); ++it)
        for (const TickPre& pr : it->pre) {
          WorldRec& R = W[pr.w];
          R.which = pr.which;
          R.steps = pr.steps;
          R.sinceBuild = pr.sinceBuild;
          R.built = pr.built;
        }
      // the first held tick's commands ran before its gate held it: they are not applied again
      for (TickPre& pr : again.front().pre) {
        pr.edits.clear();
        pr.wake = false;
      }
      // clear the hold before growing (growth may read the device, which resolves: nothing is
      // queued now)
      TickCtl reset = c;
      reset.held = 0;
      reset.itemsNeed = 0;
      CK(cudaMemcpyAsync(ctl, &reset, sizeof(TickCtl), cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));
      std::memcpy((void*)ctlHost, &reset, sizeof(reset));
      logBase = c.ticksDone;
      for (const TickLog& e : again)
        for (const TickPre& pr : e.pre) W[pr.w].pinned = true;
      std::vector<int> over(maxWorlds);
      getRaw(over.data(), wover, sizeof(int) * maxWorlds);
      for (int w = 0; w < maxWorlds; w++)
        if (over[w] > 0 && W[w].live && W[w].resident) {
          growRegion(w, over[w]);
          const int zero = 0;
          put(wover + w, &zero, 4);
        }
      if (size_t(c.itemsNeed) > itemCap) growItems(size_t(c.itemsNeed) + size_t(c.itemsNeed) / 4 + 1024);
      for (const TickLog& e : again)
        for (const TickPre& pr : e.pre) W[pr.w].pinned = false;
      regrowths++;
      for (TickLog& e : again) {
        if (e.done) tickEvents.push_back(e.done);
        e.done = nullptr;
        tickLog.push_back(std::move(e));
        queueTick(tickLog.back());
      }
    }
  }

  // CUDA graphs of tick launch sequences. A sequence depends only on host values fixed when it is
  // queued (the active table, sizes, capacities, flags, tree rebuilds) and on the device buffers;
  // a graph is replayed while all of those are unchanged (any allocation drops every graph).
  struct TickPlan {
    Tick t{};
    int na = 0, nb = 0, nj = 0, maxIter = 0, pairBudget = 0;
    long long itemCap = 0;
    bool bounce = false, sleeping = false, events = false, sleepy = false;
    int radixBits = 8;
    cudaEvent_t tune[4] = {nullptr, nullptr, nullptr, nullptr};  // autotuner timing: solve (0, 1), tree builds (2, 3)
    int* tuneItems = nullptr;  // autotuner: page-locked slot for the solve's work-item count
    std::vector<std::pair<int, int>> trees;  // (world, rebuild)
  };
  struct GraphEntry {
    std::vector<long long> key;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
    unsigned long long use = 0;
    char* table = nullptr;  // pinned: the tick's active table and world map, copied in by the graph itself
  };
  std::map<std::vector<long long>, int> graphSightings;  // keys seen, for capture on the second sighting
  std::vector<GraphEntry> graphs;
  bool graphsOn = true;
  std::string graphsOff;  // why graphs were turned off
  long long graphGen = -1;
  unsigned long long graphClock = 0;
  long long graphReplays = 0, graphCaptures = 0, ticksHeld = 0;
  std::vector<int> actUploaded;  // the active worlds whose table the device holds

  void clearGraphs() {
    if (!graphs.empty()) cudaStreamSynchronize(s);  // replays in flight may still read the tables
    for (GraphEntry& g : graphs) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      if (g.table) cudaFreeHost(g.table);
    }
    graphs.clear();
    graphSightings.clear();
  }
  std::vector<long long> planKey(const TickPlan& p, const std::vector<int>& act) const {
    std::vector<long long> k = {p.na, p.nb, p.nj, p.maxIter, p.pairBudget, p.itemCap,
                                (p.bounce ? 1 : 0) | (p.sleeping ? 2 : 0) | (p.events ? 4 : 0) | (p.sleepy ? 8 : 0) |
                                    (p.t.triggerBits ? 16 : 0),
                                rounds, slotCap, bodyCap, maxWorlds, solveCfg.queue, solveCfg.blocks, solveCfg.waves,
                                solveCfg.tile, solveCfg.waitCycles, solveCfg.probe, p.radixBits};
    for (auto& tr : p.trees) {
      k.push_back(tr.first);
      k.push_back(tr.second);
    }
    k.insert(k.end(), act.begin(), act.end());
    return k;
  }

  // The tick's active table (per active world: world, first body and joint position) and the
  // world -> active index map, as the device holds them.
  void activeTables(const std::vector<int>& act, std::vector<int4>& table, std::vector<int>& wtab) const {
    const int na = int(act.size());
    table.assign(size_t(std::max(na, 1)), make_int4(0, 0, 0, 0));
    wtab.assign(size_t(maxWorlds), -1);
    int b0 = 0, j0 = 0;
    for (int a = 0; a < na; a++) {
      table[a] = make_int4(act[a], b0, j0, 0);
      wtab[act[a]] = a;
      b0 += W[act[a]].nBodies;
      j0 += W[act[a]].nJoints;
    }
  }
  void uploadActive(const std::vector<int>& act) {
    if (act == actUploaded && uploadedWorlds == maxWorlds) return;
    std::vector<int4> table;
    std::vector<int> wtab;
    activeTables(act, table, wtab);
    if (!act.empty()) put(active, table.data(), sizeof(int4) * act.size());
    put(wactive, wtab.data(), sizeof(int) * maxWorlds);
    actUploaded = act;
    uploadedWorlds = maxWorlds;
  }

  // The launch sequence of one tick (direct, or recorded into a graph by stream capture).
  void launchTick(const TickPlan& p) {
    const Tick& t = p.t;
    cudaEvent_t b0 = (prof && !p.trees.empty()) ? mark() : nullptr;
    if (p.tune[2]) CK(cudaEventRecord(p.tune[2], s));
    for (auto& tr : p.trees) {
      WorldRec& R = W[tr.first];
      if (tr.second) launch_bvh_build(B, R.dev.bodyOff, R.nBodies, G.bvh, R.bvhOff, R.tree, bsc, scanTemp, p.radixBits, s);
      else launch_bvh_refit(B, R.dev.bodyOff, R.nBodies, G.bvh, R.bvhOff, R.tree, s);
    }
    if (p.tune[3]) CK(cudaEventRecord(p.tune[3], s));
    if (b0) span(P_COLLIDE, b0, mark());
    cudaEvent_t e0 = prof ? mark() : nullptr;
    launch_tick_begin(t, T, worlds, s);
    launch_grid_build(B, worlds, t, G, scanTemp, s);
    launch_pairs(B, worlds, t, G, NC, J.broken, pairCount, P, ctr, scanTemp, s);
    launch_narrowphase(B, worlds, t, P, NS, ctr, p.pairBudget, s);
    // every span owns its two events (the pool recycles each event exactly once)
    cudaEvent_t e1 = prof ? mark() : nullptr;
    cudaEvent_t e1b = prof ? mark() : nullptr;
    launch_spring_tear(B, J, t, s);
    launch_adjacency(B, J, P, t, ctr, T, p.pairBudget, scanTemp, s);
    launch_coloring(B, worlds, J, P, t, T, rounds, ctr, scanTemp, s);
    launch_items_count(P, t, T, ctr, scanTemp, s);
    launch_tick_gate(t, ctr, p.itemCap, s);
    if (prof) {
      cudaEvent_t e2 = mark();
      span(P_COLLIDE, e0, e1);
      span(P_TOPO, e1b, e2);
    }
    launch_items_fill(B, worlds, P, t, T, ctr, s);
    cudaEvent_t o0 = prof ? mark() : nullptr;
    launch_joint_retire(J, t, s);
    launch_joint_warmstart(B, worlds, J, t, s);
    launch_body_warmstart(B, worlds, t, s);
    if (prof) span(P_OTHER, o0, mark());
    cudaEvent_t a = prof ? mark() : nullptr;
    if (p.tuneItems) CK(cudaMemcpyAsync(p.tuneItems, &ctr->itemsTotal, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (p.tune[0]) CK(cudaEventRecord(p.tune[0], s));
    CK(launch_solve(B, worlds, J, P, t, T, ctr, p.maxIter, p.nb, p.sleepy, solveCfg, queueScratch, s));
    if (p.tune[1]) CK(cudaEventRecord(p.tune[1], s));
    if (prof) {
      span(P_PRIMAL, a, mark());
      profPrimalLaunches += 1;
    }
    cudaEvent_t v0 = prof ? mark() : nullptr;
    if (p.bounce) launch_bounce_capture(B, t, BB, s);
    launch_velocities(B, worlds, t, s);
    if (p.bounce) launch_bounce(B, P, t, T, ctr, p.pairBudget, BB, worlds, s);
    if (p.sleeping) launch_sleep(B, worlds, J, P, NC, t, ctr, p.pairBudget, SB, maxWorlds, s);
    if (p.events) launch_events(B, worlds, P, t, ctr, p.pairBudget, EV, s);
    if (prof) span(P_OTHER, v0, mark());
    launch_tick_end(t, s);
    CK(cudaMemcpyAsync(ctlHost, ctl, sizeof(TickCtl), cudaMemcpyDeviceToHost, s));
  }

  // Direct launches for a launch sequence seen once; on its second sighting it is recorded into a
  // graph (which copies its own active table in first) and replayed from then on.
  void runTick(const TickPlan& p, const std::vector<int>& act) {
    if (prof || !graphsOn || p.tune[0] || p.tune[2]) {
      uploadActive(act);
      launchTick(p);
      return;
    }
    if (graphGen != alloc_generation()) {
      clearGraphs();
      graphGen = alloc_generation();
    }
    const std::vector<long long> key = planKey(p, act);
    GraphEntry* hit = nullptr;
    for (GraphEntry& g : graphs)
      if (g.key == key) hit = &g;
    if (!hit) {
      if (graphSightings.size() > 256) graphSightings.clear();
      if (++graphSightings[key] < 2) {
        uploadActive(act);
        launchTick(p);
        return;
      }
      std::vector<int4> table;
      std::vector<int> wtab;
      activeTables(act, table, wtab);
      const size_t tb = sizeof(int4) * table.size(), wb = sizeof(int) * wtab.size();
      char* host = nullptr;
      CK(cudaHostAlloc((void**)&host, tb + wb, cudaHostAllocDefault));
      std::memcpy(host, table.data(), tb);
      std::memcpy(host + tb, wtab.data(), wb);
      const long long before = launches_total();
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      try {
        CK(cudaMemcpyAsync(active, host, tb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(wactive, host + tb, wb, cudaMemcpyHostToDevice, s));
        launchTick(p);
      } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        cudaFreeHost(host);
        throw;
      }
      cudaError_t e = cudaStreamEndCapture(s, &g);
      cudaGraphExec_t x = nullptr;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
      if (g) cudaGraphDestroy(g);
      const long long n = launches_total() - before;
      note_launches(int(-n));  // recorded, not run
      if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFreeHost(host);
        graphsOn = false;
        graphsOff = std::string("graph capture failed: ") + cudaGetErrorString(e);
        std::fprintf(stderr, "avbd_gb300: %s; ticks are launched directly\n", graphsOff.c_str());
        uploadActive(act);
        launchTick(p);
        return;
      }
      if (graphs.size() >= 32) {
        auto lru = std::min_element(graphs.begin(), graphs.end(), [](const GraphEntry& a, const GraphEntry& b) { return a.use < b.use; });
        CK(cudaStreamSynchronize(s));  // a replay in flight may still read its table
        cudaGraphExecDestroy(lru->exec);
        cudaFreeHost(lru->table);
        graphs.erase(lru);
      }
      graphs.push_back(GraphEntry{key, x, n, 0, host});
      hit = &graphs.back();
      graphCaptures++;
    } else {
      graphReplays++;
    }
    hit->use = ++graphClock;
    CK(cudaGraphLaunch(hit->exec, s));
    note_launches(int(hit->launches));
    actUploaded = act;  // the graph copied its table in
    uploadedWorlds = maxWorlds;
  }

  // Body commands and wakes queued for the tick's worlds (kernels that do nothing when held):
  // one upload and one launch for all of them, records addressed by global body index.
  void applyTickCommands(const TickLog& e) {
    for (const TickPre& pr : e.pre) {
      const WorldRec& R = W[pr.w];
      if (pr.wake && (R.dev.flags & FLAG_SLEEP) && R.nBodies) launch_sleep_wake(B, R.dev.bodyOff, R.nBodies, ctl, s);
    }
    size_t total = 0;
    for (const TickPre& pr : e.pre) total += pr.edits.size() / 12;
    if (total == 0) return;
    std::vector<uint32_t> recs;
    recs.reserve(12 * total);
    for (const TickPre& pr : e.pre) {
      const uint32_t off = uint32_t(W[pr.w].dev.bodyOff);
      const size_t n = pr.edits.size() / 12;
      for (size_t k = 0; k < n; k++) {
        const uint32_t* u = pr.edits.data() + 12 * k;
        recs.insert(recs.end(), u, u + 12);
        recs[recs.size() - 12] = u[0] + off;
      }
    }
    uploadCommands(recs, 0);
    for (const TickPre& pr : e.pre) dropTeleported(pr.w, pr.edits);
  }

  // One step of the given resident worlds, queued on the arena's stream without waiting.
  void stepWorlds(std::vector<int> act, TickReply* reply = nullptr) {
    std::sort(act.begin(), act.end(), [&](int a, int b) { return W[a].dev.bodyOff < W[b].dev.bodyOff; });
    act.erase(std::unique(act.begin(), act.end()), act.end());
    for (int w : act)
      if (w < 0 || w >= maxWorlds || !W[w].live || !W[w].resident) throw Error(AVBD_E_INVALID, "stepping a world that is not resident");
    if (hostHeld()) resolve();  // a held tick: grow and re-run it before queueing more
    trimLog();
    TickLog e;
    e.act = act;
    e.pre.reserve(act.size());
    for (int w : act) {
      WorldRec& R = W[w];
      TickPre pr;
      pr.w = w;
      pr.which = R.which;
      pr.sinceBuild = R.sinceBuild;
      pr.steps = R.steps;
      pr.built = R.built;
      pr.wake = R.wakePending;
      pr.edits.swap(R.edits);
      R.wakePending = false;
      e.pre.push_back(std::move(pr));
    }
    if (reply) e.reply = std::move(*reply);
    tickLog.push_back(std::move(e));
    queueTick(tickLog.back());
  }

  void queueTick(TickLog& e) {
    const std::vector<int>& act = e.act;
    applyTickCommands(e);
    int nb = 0, nj = 0, maxIter = 0;
    tickTriggers = false;
    TickPlan p;
    for (int w : act) {
      const WorldRec& R = W[w];
      tickTriggers |= R.triggers;
      nb += R.nBodies;
      nj += R.nJoints;
      maxIter = std::max(maxIter, R.dev.iterations);
      p.bounce |= (R.dev.flags & FLAG_RESTITUTION) != 0;
      p.sleeping |= (R.dev.flags & FLAG_SLEEP) != 0;
      p.events |= (R.dev.flags & FLAG_EVENTS) != 0;
    }
    p.sleepy = p.sleeping;
    const int na = int(act.size());
    long long budget = 0;
    for (int w : act) budget += W[w].dev.pairCap;
    ensureItems(nb);
    if (p.bounce) ensureBounce();
    if (p.sleeping) ensureSleep();
    for (int w : act) {
      WorldRec& R = W[w];
      if (!R.bvh || R.nBodies == 0) continue;
      const bool rebuild = !R.built || R.sinceBuild >= R.bvhRebuild;
      if (rebuild) ensureBvhScratch(R);
      p.trees.push_back({w, rebuild ? 1 : 0});
    }
    // the autotuner's choice for this class of tick (or a candidate to time)
    {
      std::vector<cudaEvent_t> freed;
      tuner.harvest(false, freed);
      for (cudaEvent_t ev : freed) pool.push_back(ev);
      bool rebuild = false;
      for (auto& tr : p.trees) rebuild |= tr.second != 0;
      int sizeLog2 = 0;
      while ((1LL << sizeLog2) < (long long)std::max(nb, 1)) sizeLog2++;
      const TuneKey key{ctx->device, sizeLog2, nj > 0 ? 1 : 0, maxIter};
      int sc = -1, rc = -1;
      if (tuner.needsHarvest(key)) {  // every candidate issued: wait for their timings, settle
        std::vector<cudaEvent_t> more;
        tuner.harvest(true, more);
        for (cudaEvent_t ev : more) pool.push_back(ev);
      }
      tuner.pick(key, rebuild, device_sms(), solveCfg, radixBits, sc, rc, !prof);
      p.radixBits = radixBits;
      if ((sc >= 0 || rc >= 0) && !prof) {
        int slot = -1;
        if (sc >= 0) {
          p.tune[0] = event();
          p.tune[1] = event();
          p.tuneItems = tuner.itemSlot(slot);
        }
        if (rc >= 0) {
          p.tune[2] = event();
          p.tune[3] = event();
        }
        tuner.pending.push_back(Tuner::Pending{key, sc, rc, p.tune[0], p.tune[1], p.tune[2], p.tune[3], slot, nb});
      }
      lastTuned = tuner.settled(key, !p.trees.empty());
    }
    p.t = tick(na, nb, nj);
    p.na = na;
    p.nb = nb;
    p.nj = nj;
    p.maxIter = maxIter;
    p.pairBudget = int(std::min<long long>(budget, slotCap));
    p.itemCap = (long long)itemCap;
    // host state of the stepped worlds after this tick
    for (auto& tr : p.trees) {
      WorldRec& R = W[tr.first];
      if (tr.second) {
        R.built = true;
        R.sinceBuild = 0;
      }
      R.sinceBuild++;
    }
    for (int w : act) {
      W[w].which ^= 1;
      W[w].steps++;
    }
    runTick(p, act);
    if (e.reply.rows > 0) {  // the tick's replies: gather, then copy to the owner's pinned block
      if (e.reply.seg.size() > replySegCap) {
        replySegCap = e.reply.seg.size() + e.reply.seg.size() / 2 + 64;
        rescratch(replySeg, replySegCap);
      }
      put(replySeg, e.reply.seg.data(), e.reply.seg.size() * sizeof(int4));
      launch_gather_poses(B, replySeg, int(e.reply.seg.size()), e.reply.rows, e.reply.dev, ctl, s);
      CK(cudaMemcpyAsync(e.reply.host, e.reply.dev, size_t(e.reply.rows) * 2 * sizeof(float4), cudaMemcpyDeviceToHost, s));
    }
    e.done = tickEvent();
    CK(cudaEventRecord(e.done, s));
    if (prof) {  // the tick's algorithmic bytes (profiling runs only)
      CK(cudaMemsetAsync(traffic, 0, 3 * sizeof(unsigned long long), s));
      launch_traffic(B, J, P, p.t, T, ctr, p.pairBudget, traffic, s);
      unsigned long long tb[3];
      CK(cudaMemcpyAsync(tb, traffic, sizeof(tb), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      harvest();
      profBytes[0] += double(tb[0]) * maxIter;
      profBytes[1] += double(tb[1]) * maxIter;
      profBytes[2] += double(tb[2]);
      profSteps++;
    }
    lastJoints = nj;
    statsValid = true;
    steps++;
    haveStats = false;
    CK(cudaGetLastError());
  }

  // ------------------------------------------------------------------ reads
  void syncStats() {
    resolve();
    if (haveStats) return;
    int np = 0;
    getRaw(&np, &ctr->activePairs, sizeof(int));
    lastPairs = statsValid ? np : 0;
    launch_count_active(J, P, activePairs, lastPairs, activeJoints, lastJoints, ctr, s);
    CK(cudaMemcpyAsync(ctrHost, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    haveStats = true;
  }

  void counters(avbd_counters* o) {
    syncStats();
    o->pairs = lastPairs;
    o->manifolds = ctrHost->manifolds;
    o->contacts = ctrHost->contacts;
    o->joints = ctrHost->joints;
    o->colors = ctrHost->ncolors;
    o->conflicts = ctrHost->conflicts;
    o->overflow = int32_t(regrowths);
    o->steps = int32_t(steps);
  }

  template <class X> std::vector<X> fetch(const X* d, size_t off, size_t n) {
    resolve();
    std::vector<X> h(n);
    if (n) CK(cudaMemcpyAsync(h.data(), d + off, n * sizeof(X), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return h;
  }

  const WorldRec& resident(int w) const {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    if (!W[w].resident) throw Error(AVBD_E_STATE, "world is evicted");
    return W[w];
  }

  void readState(int w, float* position, float* rotation, float* velocity, float* angular, float* prevVel) {
    const WorldRec& R = resident(w);
    touch(w);  // queued commands apply before a read (src/native/solver3D.js:223-227,245,249)
    const size_t off = R.dev.bodyOff, n = R.nBodies;
    auto put3 = [&](float* out, const float4* d) {
      if (!out) return;
      auto h = fetch(d, off, n);
      for (size_t i = 0; i < n; i++) { out[3 * i] = h[i].x; out[3 * i + 1] = h[i].y; out[3 * i + 2] = h[i].z; }
    };
    put3(velocity, B.vel);
    put3(angular, B.ang);
    put3(prevVel, B.vprev);
    if (position || rotation) {
      auto h = fetch(B.pose, 2 * off, 2 * n);
      for (size_t i = 0; i < n; i++) {
        const float4 p = h[2 * i], q = h[2 * i + 1];
        if (position) { position[3 * i] = p.x; position[3 * i + 1] = p.y; position[3 * i + 2] = p.z; }
        if (rotation) { rotation[4 * i] = q.x; rotation[4 * i + 1] = q.y; rotation[4 * i + 2] = q.z; rotation[4 * i + 3] = q.w; }
      }
    }
  }

  // the world's pairs of its last completed step (its region in buffer which[w]); global ids
  void lastPairsOf(int w, std::vector<uint2>& pairs, std::vector<int>* counts, std::vector<float4>* ct) {
    const WorldRec& R = resident(w);
    const int np = prevPairs(w);
    const size_t base = size_t(R.which) * slotCap + R.dev.pairOff;
    pairs = fetch(P.pair, base, np);
    if (counts) *counts = fetch(P.count, base, np);
    if (ct) *ct = fetch(P.ct, 32 * base, 32 * size_t(np));
  }
};

}  // namespace avbd

// ABI helpers: every entry point runs inside API_BEGIN/API_END, so no C++ exception crosses it.
#define API_BEGIN try {
#define API_END                                  \
  }                                              \
  catch (const avbd::Error& e) {                 \
    avbd::set_error(e.what());                   \
    return e.code;                               \
  }                                              \
  catch (const std::bad_alloc&) {                \
    avbd::set_error("host allocation failed");   \
    return AVBD_E_NOMEM;                         \
  }                                              \
  catch (const std::exception& e) {              \
    avbd::set_error(e.what());                   \
    return AVBD_E_STATE;                         \
  }                                              \
  return AVBD_OK;

#define REQUIRE(cond, msg) \
  if (!(cond)) throw avbd::Error(AVBD_E_INVALID, msg)
