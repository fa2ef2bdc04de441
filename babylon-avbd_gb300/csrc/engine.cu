// Host orchestration of the AVBD engine and the C ABI (include/avbd_gb300.h).
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
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/avbd_gb300.h"
#include "engine.cuh"

using namespace avbd;

namespace {

thread_local std::string g_error;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(call)                                                                                          \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess) throw Error(AVBD_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T> T* dalloc(size_t n) {
  void* p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) throw Error(AVBD_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return static_cast<T*>(p);
}

void dfree(void* p) {
  if (p) cudaFree(p);
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

}  // namespace

struct avbd_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<void*> owned;  // Arenas created under this context
};

namespace avbd {

// World state kept on the host while a world is evicted (all indices world-local).
struct Snapshot {
  std::vector<float4> body[11];  // pos rot pos0 rot0 posY rotY vel ang vprev size mass
  std::vector<int4> meta;
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
  WorldDev dev{};
  int nBodies = 0, nJoints = 0;
  int which = 0;
  std::vector<std::pair<unsigned long long, int>> nc;  // local (hi << 32 | lo) -> local joint id or -1
  std::vector<int> largeLocal;
  long long pending = 0;
  unsigned long long lastUse = 0;
  std::unique_ptr<Snapshot> snap;
};

class Arena {
 public:
  avbd_ctx* ctx;
  cudaStream_t s;
  int bodyCap = 0, jointCap = 0, slotCap = 0, maxWorlds = 0;
  RangeAlloc bodyA, jointA, slotA;
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
  int4* activeHost = nullptr;
  int* wactiveHost = nullptr;
  void* scanTemp = nullptr;
  size_t scanBytes = 0;
  size_t itemCap = 0;
  int rounds = 64;
  // the last tick (its lists stay valid until the next tick)
  std::vector<int> lastActive;
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

  // Host -> device uploads of world set-up go through one pinned staging buffer on the arena's
  // stream (sources may be temporaries); flush() waits for them and recycles the buffer.
  char* stage = nullptr;
  size_t stageCap = 0, stageUsed = 0;

  void put(void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return;
    if (stageUsed + bytes > stageCap) {
      flush();
      if (bytes > stageCap) {
        if (stage) cudaFreeHost(stage);
        stage = nullptr;
        stageCap = 0;
        const size_t cap = std::max<size_t>(bytes, size_t(4) << 20);
        CK(cudaHostAlloc((void**)&stage, cap, cudaHostAllocDefault));
        stageCap = cap;
      }
    }
    std::memcpy(stage + stageUsed, src, bytes);
    CK(cudaMemcpyAsync(dst, stage + stageUsed, bytes, cudaMemcpyHostToDevice, s));
    stageUsed += (bytes + 255) & ~size_t(255);
  }
  void flush() {
    CK(cudaStreamSynchronize(s));
    stageUsed = 0;
  }
  void get(void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    stageUsed = 0;
  }

  Arena(avbd_ctx* c, int bodies, int joints, int slots, int worldsMax) : ctx(c), s(c->stream) {
    allocate(std::max(bodies, 1), std::max(joints, 1), std::max(slots, 1024), std::max(worldsMax, 1));
  }
  ~Arena() {
    cudaStreamSynchronize(s);
    harvest();
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
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
    for (float4** p : {&B.pos, &B.rot, &B.pos0, &B.rot0, &B.posY, &B.rotY, &B.vel, &B.ang, &B.vprev, &B.size, &B.mass})
      *p = dalloc<float4>(N);
    B.meta = dalloc<int4>(N);
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
    CK(cudaHostAlloc((void**)&activeHost, sizeof(int4) * nw, cudaHostAllocDefault));
    CK(cudaHostAlloc((void**)&wactiveHost, sizeof(int) * nw, cudaHostAllocDefault));
    for (int w = 0; w < nw; w++) wactiveHost[w] = -1;
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
    T.itemStart = dalloc<int>(N + 1);
    ctr = dalloc<Counters>(1);
    CK(cudaMemset(ctr, 0, sizeof(Counters)));
    CK(cudaHostAlloc((void**)&ctrHost, sizeof(Counters), cudaHostAllocDefault));
    std::memset(ctrHost, 0, sizeof(Counters));
    NC.keys = dalloc<unsigned long long>(1);
    NC.jid = dalloc<int>(1);
    ncCap = 1;
    slotCap = 0;
    allocSlots(slots);
  }

  void release() {
    void* ptrs[] = {B.pos, B.rot, B.pos0, B.rot0, B.posY, B.rotY, B.vel, B.ang, B.vprev, B.size, B.mass, B.meta, J.ab, J.rA,
                    J.rB, J.stiff, J.penLin, J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang, J.restQ, J.broken, worlds,
                    which, pairN, wover, wactive, active, activeBodies, activeJoints, pairPrefix, pairCount, G.cellCount,
                    G.cellFill, G.cellBodies, G.bodyBucket, G.large, T.adjStart, T.adjFill, T.activeIndex, T.color, T.won,
                    T.pending, T.colorBodies, T.itemStart, T.itemRef, T.contrib, ctr, NC.keys, NC.jid, scanTemp, traffic,
                    poseStage, P.pair, P.count, P.basis, P.ct, NS.sat, NS.boxList, NS.sphereList, NS.ctr, activePairs,
                    T.adjList};
    for (void* p : ptrs) dfree(p);
    if (ctrHost) cudaFreeHost(ctrHost);
    if (activeHost) cudaFreeHost(activeHost);
    if (wactiveHost) cudaFreeHost(wactiveHost);
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
                    (void*)NS.sphereList, (void*)NS.ctr, (void*)activePairs, (void*)T.adjList})
      dfree(p);
    P = np;
    NS.sat = dalloc<float4>(cap);
    NS.boxList = dalloc<int>(cap);
    NS.sphereList = dalloc<int>(cap);
    NS.ctr = dalloc<int>(2);
    activePairs = dalloc<int>(cap);
    T.adjList = dalloc<uint32_t>(2 * (size_t(jointCap) + size_t(cap)) + 1);
    if (slotCap == 0) slotA.init(cap);
    else slotA.grow(cap);
    slotCap = cap;
    lastPairs = 0;  // the last tick's pair list was in the buffers just replaced
    size_t need = std::max(scan_temp_bytes(int(G.tableMask) + 2), scan_temp_bytes(bodyCap + 2));
    need = std::max(need, scan_temp_bytes(maxWorlds + 2));
    if (need > scanBytes) {
      dfree(scanTemp);
      scanTemp = dalloc<char>(need);
      scanBytes = need;
    }
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
      if (d.shape[i] != AVBD_SHAPE_BOX && d.shape[i] != AVBD_SHAPE_SPHERE) throw Error(AVBD_E_INVALID, "unknown body shape");
      for (int k = 0; k < 3; k++) {
        if (!std::isfinite(d.position[3 * i + k])) throw Error(AVBD_E_INVALID, "position must be finite");
        if (!(d.size[3 * i + k] > 0.f)) throw Error(AVBD_E_INVALID, "size must be positive");
      }
    }
    for (int c = 0; c < d.n_cons; c++) {
      int k = d.cons_kind[c];
      if (k != AVBD_CONS_JOINT && k != AVBD_CONS_SPRING && k != AVBD_CONS_IGNORE) throw Error(AVBD_E_INVALID, "unknown constraint kind");
      int a = d.cons_a[c], b = d.cons_b[c];
      if (b < 0 || b >= d.n_bodies || a < -1 || a >= d.n_bodies || a == b) throw Error(AVBD_E_INVALID, "constraint bodies out of range");
      if (a < 0 && k != AVBD_CONS_JOINT) throw Error(AVBD_E_INVALID, "only joints may attach to the world");
    }
  }

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
    R.nc.clear();
    int j = 0;
    for (int c = 0; c < d.n_cons; c++) {
      const int kind = d.cons_kind[c];
      const int jid = kind != AVBD_CONS_IGNORE ? j++ : -1;
      const int a = d.cons_a[c], b = d.cons_b[c];
      if (a >= 0) R.nc.push_back({(unsigned long long)(uint32_t)std::max(a, b) << 32 | (uint32_t)std::min(a, b), jid});
    }
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
    int po = slotA.alloc(slotsWanted);
    if (po < 0) {
      allocSlots(std::max(slotCap + slotsWanted + 1024, slotCap + slotCap / 2));
      po = slotA.alloc(slotsWanted);
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
  int addWorld(const avbd_scene_desc& d, const avbd_params& p, bool rebuild = true) {
    validate(d, p);
    const int w = takeSlot();
    WorldRec& R = W[w];
    try {
      worldParams(d, p, R);
      R.dev.largeOff = w * MAX_LARGE;
      placeRanges(R, initialPairCap(d.n_bodies));
    } catch (...) {
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
        const uint32_t grp = d.group ? d.group[i] : 0xffffffffu, msk = d.collides_with ? d.collides_with[i] : 0xffffffffu;
        meta[i] = make_int4(w, d.shape[i], int(grp), int(msk));
      }
      const float4* src[11] = {pos.data(), rot.data(), pos.data(), rot.data(), pos.data(), rot.data(), vel.data(), ang.data(),
                               vprev.data(), size.data(), mass.data()};
      float4* dst[11] = {B.pos, B.rot, B.pos0, B.rot0, B.posY, B.rotY, B.vel, B.ang, B.vprev, B.size, B.mass};
      for (int k = 0; k < 11; k++) put(dst[k] + off, src[k], n * 16);
      put(B.meta + off, meta.data(), n * 16);
      std::vector<int> minus(n, -1);
      put(T.color + off, minus.data(), n * 4);
      put(T.color + bodyCap + off, minus.data(), n * 4);
    }
    // joints and springs (global body ids)
    const size_t nj = size_t(R.nJoints), joff = size_t(R.dev.jointOff);
    if (nj) {
      std::vector<int2> jab(nj);
      std::vector<float4> jra(nj), jrb(nj), jst(nj), jz(nj, make_float4(0, 0, 0, 0)), jq(nj, make_float4(0, 0, 0, 1));
      std::vector<int> jbr(nj, 0);
      size_t j = 0;
      for (int c = 0; c < d.n_cons; c++) {
        const int kind = d.cons_kind[c];
        if (kind == AVBD_CONS_IGNORE) continue;
        const int a = d.cons_a[c] >= 0 ? int(off) + d.cons_a[c] : -1;
        const int b = int(off) + d.cons_b[c];
        jab[j] = make_int2(a, b);
        int kk = kind == AVBD_CONS_JOINT ? KIND_JOINT : KIND_SPRING;
        float kf;
        std::memcpy(&kf, &kk, 4);
        jra[j] = make_float4(d.cons_ra[3 * c], d.cons_ra[3 * c + 1], d.cons_ra[3 * c + 2], kf);
        jrb[j] = make_float4(d.cons_rb[3 * c], d.cons_rb[3 * c + 1], d.cons_rb[3 * c + 2], kind == AVBD_CONS_SPRING ? d.cons_p1[c] : 0.f);
        jst[j] = kind == AVBD_CONS_JOINT ? make_float4(d.cons_p0[c], d.cons_p1[c], d.cons_p2[c], 0.f)
                                         : make_float4(d.cons_p0[c], 0.f, INFINITY, 0.f);
        j++;
      }
      put(J.ab + joff, jab.data(), nj * 8);
      put(J.rA + joff, jra.data(), nj * 16);
      put(J.rB + joff, jrb.data(), nj * 16);
      put(J.stiff + joff, jst.data(), nj * 16);
      for (float4* q : {J.penLin, J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang}) put(q + joff, jz.data(), nj * 16);
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
    flush();
    return w;
  }

  void freeRanges(WorldRec& R) {
    bodyA.release(R.dev.bodyOff, R.nBodies);
    jointA.release(R.dev.jointOff, R.nJoints);
    slotA.release(R.dev.pairOff, R.dev.pairCap);
  }

  void removeWorld(int w) {
    if (w < 0 || w >= maxWorlds || !W[w].live) throw Error(AVBD_E_INVALID, "no such world");
    CK(cudaStreamSynchronize(s));
    WorldRec& R = W[w];
    if (R.resident) freeRanges(R);
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
    WorldRec& R = W[w];
    if (!R.live || !R.resident) throw Error(AVBD_E_INVALID, "world is not resident");
    CK(cudaStreamSynchronize(s));
    auto S = std::make_unique<Snapshot>();
    const size_t off = R.dev.bodyOff, n = R.nBodies, joff = R.dev.jointOff, nj = R.nJoints;
    const float4* bsrc[11] = {B.pos, B.rot, B.pos0, B.rot0, B.posY, B.rotY, B.vel, B.ang, B.vprev, B.size, B.mass};
    for (int k = 0; k < 11; k++) getRange(S->body[k], bsrc[k], off, n);
    getRange(S->meta, B.meta, off, n);
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
    freeRanges(R);
    R.resident = false;
    R.snap = std::move(S);
    evictions++;
    rebuildNoCollide();
    flush();
  }

  // Bring an evicted world back (into any free ranges); its state continues exactly.
  void restore(int w) {
    WorldRec& R = W[w];
    if (!R.live || R.resident || !R.snap) throw Error(AVBD_E_INVALID, "world is not evicted");
    Snapshot& S = *R.snap;
    const int np = int(S.pairs.size());
    placeRanges(R, std::max(initialPairCap(R.nBodies), np + np / 4 + 64));
    const size_t off = R.dev.bodyOff, joff = R.dev.jointOff;
    float4* bdst[11] = {B.pos, B.rot, B.pos0, B.rot0, B.posY, B.rotY, B.vel, B.ang, B.vprev, B.size, B.mass};
    for (int k = 0; k < 11; k++) putRange(bdst[k], off, S.body[k]);
    putRange(B.meta, off, S.meta);
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
    WorldRec& R = W[w];
    const int cap = need + need / 4 + 64;
    int po = slotA.alloc(cap);
    if (po < 0) {
      allocSlots(std::max(slotCap + cap + 1024, slotCap + slotCap / 2));
      po = slotA.alloc(cap);
    }
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
  }

  // ------------------------------------------------------------------ ticks
  void ensureItems() {
    const size_t need = size_t(std::max(ctrHost->itemsTotal, 1));
    int maxColor = 1;
    for (int c = 0; c < MAX_COLORS; c++) maxColor = std::max(maxColor, ctrHost->colorItems[c]);
    if (need > itemCap) {
      CK(cudaStreamSynchronize(s));
      const size_t cap = need + need / 4 + 1024;
      dfree(T.itemRef);
      T.itemRef = nullptr;
      T.itemRef = dalloc<int2>(cap);
      itemCap = cap;
    }
    if (maxColor > T.contribCap) {
      CK(cudaStreamSynchronize(s));
      const int ccap = maxColor + maxColor / 4 + 1024;
      dfree(T.contrib);
      T.contrib = nullptr;
      T.contrib = dalloc<float4>(size_t(ccap) * 7);
      T.contribCap = ccap;
    }
  }

  // One step of the given resident worlds.
  void stepWorlds(std::vector<int> act) {
    std::sort(act.begin(), act.end(), [&](int a, int b) { return W[a].dev.bodyOff < W[b].dev.bodyOff; });
    act.erase(std::unique(act.begin(), act.end()), act.end());
    for (int w : act)
      if (w < 0 || w >= maxWorlds || !W[w].live || !W[w].resident) throw Error(AVBD_E_INVALID, "stepping a world that is not resident");
    for (int w : lastActive) wactiveHost[w] = -1;
    lastActive.clear();
    int nb = 0, nj = 0, maxIter = 0;
    for (size_t a = 0; a < act.size(); a++) {
      const WorldRec& R = W[act[a]];
      activeHost[a] = make_int4(act[a], nb, nj, 0);
      wactiveHost[act[a]] = int(a);
      nb += R.nBodies;
      nj += R.nJoints;
      maxIter = std::max(maxIter, R.dev.iterations);
    }
    const int na = int(act.size());
    if (na) CK(cudaMemcpyAsync(active, activeHost, sizeof(int4) * na, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(wactive, wactiveHost, sizeof(int) * maxWorlds, cudaMemcpyHostToDevice, s));
    lastActive = act;
    long long budget = 0;
    for (int attempt = 0;; attempt++) {
      budget = 0;
      for (int w : act) budget += W[w].dev.pairCap;
      const int pairBudget = int(std::min<long long>(budget, slotCap));
      Tick t = tick(na, nb, nj);
      cudaEvent_t e0 = prof ? mark() : nullptr;
      launch_tick_begin(t, T, worlds, s);
      launch_grid_build(B, worlds, t, G, scanTemp, s);
      launch_pairs(B, worlds, t, G, NC, J.broken, pairCount, P, ctr, scanTemp, s);
      launch_narrowphase(B, worlds, t, P, NS, ctr, pairBudget, s);
      // every span owns its two events (the pool recycles each event exactly once)
      cudaEvent_t e1 = prof ? mark() : nullptr;
      cudaEvent_t e1b = prof ? mark() : nullptr;
      launch_adjacency(B, J, P, t, ctr, T, pairBudget, scanTemp, s);
      launch_coloring(B, worlds, J, P, t, T, rounds, ctr, s);
      launch_items_count(P, t, T, ctr, scanTemp, s);
      if (prof) {
        cudaEvent_t e2 = mark();
        span(P_COLLIDE, e0, e1);
        span(P_TOPO, e1b, e2);
      }
      CK(cudaMemcpyAsync(ctrHost, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      CK(cudaGetLastError());
      if (prof) harvest();
      if (ctrHost->overflowWorlds == 0) break;
      if (attempt > 8) throw Error(AVBD_E_CAPACITY, "pair regions did not converge");
      std::vector<int> over(maxWorlds);
      get(over.data(), wover, sizeof(int) * maxWorlds);
      for (int w : act)
        if (over[w] > 0) {
          growRegion(w, over[w]);
          const int zero = 0;
          put(wover + w, &zero, 4);
        }
    }
    const int pairBudget = int(std::min<long long>(budget, slotCap));
    Tick t = tick(na, nb, nj);
    ensureItems();
    launch_items_fill(P, t, T, ctr, s);
    cudaEvent_t o0 = prof ? mark() : nullptr;
    launch_joint_warmstart(B, worlds, J, t, s);
    launch_body_warmstart(B, worlds, t, s);
    if (prof) span(P_OTHER, o0, mark());
    const int ncolors = ctrHost->ncolors;
    for (int it = 0; it < maxIter; it++) {
      for (int c = 0; c < ncolors; c++) {
        const int cnt = ctrHost->colorCount[c];
        if (!cnt) continue;
        cudaEvent_t a = prof ? mark() : nullptr;
        launch_primal(B, worlds, J, P, t, T, ctr, c, it, cnt, ctrHost->colorItems[c], s);
        if (prof) {
          span(P_PRIMAL, a, mark());
          profPrimalLaunches += ctrHost->colorItems[c] > 0 ? 2 : 1;
        }
      }
      cudaEvent_t d = prof ? mark() : nullptr;
      launch_dual(B, worlds, J, P, t, ctr, pairBudget, it, s);
      if (prof) span(P_DUAL, d, mark());
    }
    cudaEvent_t v0 = prof ? mark() : nullptr;
    launch_velocities(B, worlds, t, s);
    if (prof) span(P_OTHER, v0, mark());
    if (prof) {
      CK(cudaMemsetAsync(traffic, 0, 3 * sizeof(unsigned long long), s));
      launch_traffic(B, J, P, t, T, ctr, pairBudget, traffic, s);
      unsigned long long tb[3];
      CK(cudaMemcpyAsync(tb, traffic, sizeof(tb), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      profBytes[0] += double(tb[0]) * maxIter;
      profBytes[1] += double(tb[1]) * maxIter;
      profBytes[2] += double(tb[2]);
      profSteps++;
    }
    launch_tick_end(t, s);
    for (int w : act) W[w].which ^= 1;
    lastPairs = ctrHost->activePairs;
    lastJoints = nj;
    steps++;
    haveStats = false;
    CK(cudaGetLastError());
  }

  // ------------------------------------------------------------------ reads
  void syncStats() {
    if (haveStats) return;
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
    const size_t off = R.dev.bodyOff, n = R.nBodies;
    auto put3 = [&](float* out, const float4* d) {
      if (!out) return;
      auto h = fetch(d, off, n);
      for (size_t i = 0; i < n; i++) { out[3 * i] = h[i].x; out[3 * i + 1] = h[i].y; out[3 * i + 2] = h[i].z; }
    };
    put3(position, B.pos);
    put3(velocity, B.vel);
    put3(angular, B.ang);
    put3(prevVel, B.vprev);
    if (rotation) {
      auto h = fetch(B.rot, off, n);
      for (size_t i = 0; i < n; i++) { rotation[4 * i] = h[i].x; rotation[4 * i + 1] = h[i].y; rotation[4 * i + 2] = h[i].z; rotation[4 * i + 3] = h[i].w; }
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

struct avbd_world {
  Arena* A;
  int w;
};
struct avbd_batch {
  Arena* A;
  std::vector<int> worlds;
  int64_t bodies;
};

// ---------------------------------------------------------------- device helpers for the ABI

namespace avbd {

// 40-float body records of src/native/cpu/world.js:503-561 (or 8-float poses)
__global__ void k_read_selected(BodyPtrs bd, const WorldDev* __restrict__ worlds, const uint32_t* __restrict__ idx, int n, int off,
                                int posesOnly, float* __restrict__ out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int i = off + int(idx[k]);
    const float4 p = bd.pos[i], q = bd.rot[i], sz = bd.size[i];
    if (posesOnly) {
      float* o = out + size_t(k) * 8;
      o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = sz.w;
      o[4] = q.x; o[5] = q.y; o[6] = q.z; o[7] = q.w;
      continue;
    }
    float* o = out + size_t(k) * 40;
    const float4 p0 = bd.pos0[i], q0 = bd.rot0[i], m = bd.mass[i], py = bd.posY[i], qy = bd.rotY[i];
    const float4 v = bd.vel[i], w = bd.ang[i], vp = bd.vprev[i];
    const int4 meta = bd.meta[i];
    const WorldDev& W = worlds[meta.x];
    o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = sz.w;
    o[4] = q.x; o[5] = q.y; o[6] = q.z; o[7] = q.w;
    o[8] = p0.x; o[9] = p0.y; o[10] = p0.z; o[11] = 0.f;
    o[12] = q0.x; o[13] = q0.y; o[14] = q0.z; o[15] = q0.w;
    o[16] = sz.x; o[17] = sz.y; o[18] = sz.z; o[19] = m.x;
    o[20] = m.y; o[21] = m.z; o[22] = m.w; o[23] = p.w;
    o[24] = py.x; o[25] = py.y; o[26] = py.z; o[27] = 0.f;
    o[28] = qy.x; o[29] = qy.y; o[30] = qy.z; o[31] = qy.w;
    o[32] = v.x; o[33] = v.y; o[34] = v.z; o[35] = (vp.x * W.up0 + vp.y * W.up1) + vp.z * W.up2;
    o[36] = w.x; o[37] = w.y; o[38] = w.z; o[39] = float(meta.y);
  }
}

__global__ void k_set_poses(BodyPtrs bd, const uint32_t* __restrict__ idx, int n, int off, const float* __restrict__ pos,
                            const float* __restrict__ rot) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int i = off + int(idx[k]);
    const float r = bd.pos[i].w;
    bd.pos[i] = make_float4(pos[3 * k], pos[3 * k + 1], pos[3 * k + 2], r);
    if (rot) bd.rot[i] = qnormalize(make_float4(rot[4 * k], rot[4 * k + 1], rot[4 * k + 2], rot[4 * k + 3]));
  }
}

__global__ void k_set_velocities(BodyPtrs bd, const uint32_t* __restrict__ idx, int n, int off, const float* __restrict__ vel,
                                 const float* __restrict__ ang) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int i = off + int(idx[k]);
    if (vel) bd.vel[i] = make_float4(vel[3 * k], vel[3 * k + 1], vel[3 * k + 2], 0.f);
    if (ang) bd.ang[i] = make_float4(ang[3 * k], ang[3 * k + 1], ang[3 * k + 2], 0.f);
  }
}

__global__ void k_read_poses(const float4* __restrict__ pos, const float4* __restrict__ rot, const float4* __restrict__ size, int n,
                             float4* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pos[i];
    out[2 * i] = make_float4(p.x, p.y, p.z, size[i].w);
    out[2 * i + 1] = rot[i];
  }
}

}  // namespace avbd

// ---------------------------------------------------------------- C ABI

#define API_BEGIN try {
#define API_END                                  \
  }                                              \
  catch (const Error& e) {                       \
    g_error = e.what();                          \
    return e.code;                               \
  }                                              \
  catch (const std::bad_alloc&) {                \
    g_error = "host allocation failed";          \
    return AVBD_E_NOMEM;                         \
  }                                              \
  catch (const std::exception& e) {              \
    g_error = e.what();                          \
    return AVBD_E_STATE;                         \
  }                                              \
  return AVBD_OK;

#define REQUIRE(cond, msg) \
  if (!(cond)) throw Error(AVBD_E_INVALID, msg)

namespace {

void bind(avbd_ctx* c) { CK(cudaSetDevice(c->device)); }

// Stage host bytes into a temporary device buffer; freed by the caller via the returned pointer.
template <class X> X* upload(const X* h, size_t n, cudaStream_t s) {
  X* d = dalloc<X>(n);
  CK(cudaMemcpyAsync(d, h, n * sizeof(X), cudaMemcpyHostToDevice, s));
  return d;
}

void forget(avbd_ctx* ctx, Arena* A) {
  auto& v = ctx->owned;
  v.erase(std::remove(v.begin(), v.end(), (void*)A), v.end());
}

// Arena for a fixed set of worlds, sized to fit them.
Arena* arenaFor(avbd_ctx* ctx, const avbd_scene_desc* scenes, const avbd_params* params, int n, std::vector<int>& slots) {
  long long nb = 0, nj = 0, np = 0;
  for (int i = 0; i < n; i++) {
    Arena::validate(scenes[i], params[i]);
    nb += scenes[i].n_bodies;
    nj += Arena::jointsOf(scenes[i]);
    np += Arena::initialPairCap(scenes[i].n_bodies);
  }
  if (nb > 0x3fffffffLL || np > 0x3fffffffLL) throw Error(AVBD_E_CAPACITY, "too many bodies for one arena");
  auto* A = new Arena(ctx, int(nb), int(nj), int(np), n);
  try {
    for (int i = 0; i < n; i++) slots.push_back(A->addWorld(scenes[i], params[i], false));
    A->rebuildNoCollide();
    A->flush();
  } catch (...) {
    delete A;
    throw;
  }
  ctx->owned.push_back(A);
  return A;
}

void readSelected(Arena& A, int w, const uint32_t* indices, int n, int posesOnly, float* out) {
  const WorldRec& R = A.resident(w);
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(R.nBodies), "body index out of range");
  if (n == 0) return;
  const int stride = posesOnly ? 8 : 40;
  uint32_t* di = upload(indices, size_t(n), A.s);
  float* dout = dalloc<float>(size_t(n) * stride);
  k_read_selected<<<grid_blocks(n, 128), 128, 0, A.s>>>(A.B, A.worlds, di, n, R.dev.bodyOff, posesOnly, dout); note_launches(1);
  cudaError_t e = cudaMemcpyAsync(out, dout, size_t(n) * stride * 4, cudaMemcpyDeviceToHost, A.s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(A.s);
  dfree(di);
  dfree(dout);
  if (e != cudaSuccess) throw Error(AVBD_E_CUDA, cudaGetErrorString(e));
}

void setVelocities(Arena& A, int off, int limit, const uint32_t* indices, int n, const float* velocity, const float* angular) {
  REQUIRE(n == 0 || indices, "null argument");
  REQUIRE(n >= 0, "negative count");
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(limit), "body index out of range");
  for (int k = 0; velocity && k < 3 * n; k++) REQUIRE(std::isfinite(velocity[k]), "velocities must be finite");
  for (int k = 0; angular && k < 3 * n; k++) REQUIRE(std::isfinite(angular[k]), "velocities must be finite");
  if (n == 0 || (!velocity && !angular)) return;
  uint32_t* di = upload(indices, size_t(n), A.s);
  float* dv = velocity ? upload(velocity, size_t(n) * 3, A.s) : nullptr;
  float* da = angular ? upload(angular, size_t(n) * 3, A.s) : nullptr;
  k_set_velocities<<<grid_blocks(n, 128), 128, 0, A.s>>>(A.B, di, n, off, dv, da); note_launches(1);
  cudaError_t e = cudaStreamSynchronize(A.s);
  dfree(di);
  dfree(dv);
  dfree(da);
  if (e != cudaSuccess) throw Error(AVBD_E_CUDA, cudaGetErrorString(e));
}

}  // namespace

extern "C" {

const char* avbd_last_error(void) { return g_error.c_str(); }
const char* avbd_version(void) { return "avbd_gb300 0.2.0 (sm_103a)"; }

int avbd_ctx_create(int device, avbd_ctx** out) {
  API_BEGIN
  REQUIRE(out, "out is null");
  int count = 0;
  CK(cudaGetDeviceCount(&count));
  REQUIRE(device >= 0 && device < count, "no such CUDA device");
  auto* c = new avbd_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    throw Error(AVBD_E_CUDA, std::string("context: ") + cudaGetErrorString(e));
  }
  *out = c;
  API_END
}

int avbd_ctx_stream(avbd_ctx* ctx, void** stream) {
  API_BEGIN
  REQUIRE(ctx && stream, "null argument");
  *stream = (void*)ctx->stream;
  API_END
}

int avbd_ctx_synchronize(avbd_ctx* ctx) {
  API_BEGIN
  REQUIRE(ctx, "null context");
  bind(ctx);
  CK(cudaStreamSynchronize(ctx->stream));
  API_END
}

int avbd_ctx_destroy(avbd_ctx* ctx) {
  API_BEGIN
  if (!ctx) return AVBD_OK;
  bind(ctx);
  for (void* p : ctx->owned) delete static_cast<Arena*>(p);
  ctx->owned.clear();
  cudaStreamSynchronize(ctx->stream);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  API_END
}

// ---------------------------------------------------------------- plain worlds

int avbd_world_create(avbd_ctx* ctx, const avbd_scene_desc* scene, const avbd_params* params, avbd_world** out) {
  API_BEGIN
  REQUIRE(ctx && scene && params && out, "null argument");
  bind(ctx);
  std::vector<int> slots;
  Arena* A = arenaFor(ctx, scene, params, 1, slots);
  *out = new avbd_world{A, slots[0]};
  API_END
}

int avbd_world_destroy(avbd_world* w) {
  API_BEGIN
  if (!w) return AVBD_OK;
  avbd_ctx* ctx = w->A->ctx;
  bind(ctx);
  forget(ctx, w->A);
  delete w->A;
  delete w;
  API_END
}

int avbd_world_step(avbd_world* w, int32_t steps) {
  API_BEGIN
  REQUIRE(w, "null world");
  REQUIRE(steps >= 0, "steps must be non-negative");
  bind(w->A->ctx);
  for (int i = 0; i < steps; i++) w->A->stepWorlds({w->w});
  API_END
}

int avbd_world_read_state(avbd_world* w, float* position, float* rotation, float* velocity, float* angular, float* prev_velocity) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->readState(w->w, position, rotation, velocity, angular, prev_velocity);
  API_END
}

int avbd_world_read_selected(avbd_world* w, const uint32_t* indices, int32_t n, int32_t poses_only, float* out) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (indices && out)), "null argument");
  REQUIRE(n >= 0, "negative count");
  bind(w->A->ctx);
  readSelected(*w->A, w->w, indices, n, poses_only, out);
  API_END
}

}  // extern "C"

// ---------------------------------------------------------------- allocation-free selected reads
// Staging for avbd_world_read_selected_noalloc: indices in the first
// AVBD_NOALLOC_MAX_SELECTED words, then AVBD_NOALLOC_MAX_SELECTED records of 40 floats (the
// record region starts 32 KB in, a multiple of 256 bytes). Nothing in it is read before the
// call that uses it has written it, so no part needs clearing between calls.
static __device__ __align__(256) float g_select_scratch[AVBD_NOALLOC_MAX_SELECTED * 41];

namespace {

std::mutex g_select_mutex;
float* g_select_ptr[256] = {};

// Device address of g_select_scratch on `device` (which must be current): looked up once per
// device. In host code the symbol itself is only a host-side stand-in for the device array.
float* select_scratch(int device) {
  std::lock_guard<std::mutex> lock(g_select_mutex);
  if (device < 0 || device >= 256) throw Error(AVBD_E_INVALID, "device index out of range");
  if (!g_select_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_select_scratch);
    if (e != cudaSuccess) throw Error(AVBD_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_select_ptr[device] = static_cast<float*>(p);
  }
  return g_select_ptr[device];
}

}  // namespace

extern "C" {

int avbd_world_read_selected_noalloc(avbd_world* w, const uint32_t* indices, int32_t n, int32_t poses_only, float* out) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (indices && out)), "null argument");
  REQUIRE(n >= 0, "negative count");
  if (n > AVBD_NOALLOC_MAX_SELECTED)
    throw Error(AVBD_E_CAPACITY, "avbd_world_read_selected_noalloc: at most " + std::to_string(AVBD_NOALLOC_MAX_SELECTED) +
                                     " bodies per call (" + std::to_string(n) + " requested)");
  Arena& A = *w->A;
  bind(A.ctx);
  const WorldRec& R = A.resident(w->w);
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(R.nBodies), "body index out of range");
  if (n == 0) return AVBD_OK;
  float* scratch = select_scratch(A.ctx->device);
  uint32_t* dIdx = reinterpret_cast<uint32_t*>(scratch);
  float* dOut = scratch + AVBD_NOALLOC_MAX_SELECTED;
  const size_t stride = poses_only ? 8 : 40;
  CK(cudaMemcpyAsync(dIdx, indices, size_t(n) * 4, cudaMemcpyHostToDevice, A.s));
  k_read_selected<<<grid_blocks(n, 128), 128, 0, A.s>>>(A.B, A.worlds, dIdx, n, R.dev.bodyOff, poses_only, dOut); note_launches(1);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dOut, size_t(n) * stride * 4, cudaMemcpyDeviceToHost, A.s));
  CK(cudaStreamSynchronize(A.s));
  API_END
}

int avbd_world_set_poses(avbd_world* w, const uint32_t* indices, int32_t n, const float* position, const float* rotation) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (indices && position)), "null argument");
  REQUIRE(n >= 0, "negative count");
  Arena& A = *w->A;
  bind(A.ctx);
  const WorldRec& R = A.resident(w->w);
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(R.nBodies), "body index out of range");
  for (int k = 0; k < 3 * n; k++) REQUIRE(std::isfinite(position[k]), "positions must be finite");
  if (rotation)
    for (int k = 0; k < n; k++) {
      const float* q = rotation + 4 * k;
      REQUIRE(std::isfinite(q[0]) && std::isfinite(q[1]) && std::isfinite(q[2]) && std::isfinite(q[3]) &&
                  (q[0] != 0 || q[1] != 0 || q[2] != 0 || q[3] != 0),
              "rotations must be finite and nonzero");
    }
  if (n == 0) return AVBD_OK;
  uint32_t* di = upload(indices, size_t(n), A.s);
  float* dp = upload(position, size_t(n) * 3, A.s);
  float* dr = rotation ? upload(rotation, size_t(n) * 4, A.s) : nullptr;
  k_set_poses<<<grid_blocks(n, 128), 128, 0, A.s>>>(A.B, di, n, R.dev.bodyOff, dp, dr); note_launches(1);
  cudaError_t e = cudaStreamSynchronize(A.s);
  dfree(di);
  dfree(dp);
  dfree(dr);
  if (e != cudaSuccess) throw Error(AVBD_E_CUDA, cudaGetErrorString(e));
  API_END
}

int avbd_world_set_velocities(avbd_world* w, const uint32_t* indices, int32_t n, const float* velocity, const float* angular) {
  API_BEGIN
  REQUIRE(w, "null argument");
  Arena& A = *w->A;
  bind(A.ctx);
  const WorldRec& R = A.resident(w->w);
  setVelocities(A, R.dev.bodyOff, R.nBodies, indices, n, velocity, angular);
  API_END
}

int avbd_world_counters(avbd_world* w, avbd_counters* out) {
  API_BEGIN
  REQUIRE(w && out, "null argument");
  bind(w->A->ctx);
  w->A->counters(out);
  API_END
}

int avbd_world_pairs(avbd_world* w, uint32_t* out, int64_t cap, int64_t* n) {
  API_BEGIN
  REQUIRE(w && n, "null argument");
  bind(w->A->ctx);
  std::vector<uint2> pairs;
  w->A->lastPairsOf(w->w, pairs, nullptr, nullptr);
  *n = int64_t(pairs.size());
  const int64_t k = std::min<int64_t>(int64_t(pairs.size()), cap);
  const uint32_t off = uint32_t(w->A->W[w->w].dev.bodyOff);
  for (int64_t i = 0; out && i < k; i++) {
    out[2 * i] = pairs[i].x - off;
    out[2 * i + 1] = pairs[i].y - off;
  }
  API_END
}

int avbd_world_pair_contacts(avbd_world* w, int32_t* out, int64_t cap, int64_t* n) {
  API_BEGIN
  REQUIRE(w && n, "null argument");
  bind(w->A->ctx);
  std::vector<uint2> pairs;
  std::vector<int> counts;
  w->A->lastPairsOf(w->w, pairs, &counts, nullptr);
  *n = int64_t(counts.size());
  const int64_t k = std::min<int64_t>(int64_t(counts.size()), cap);
  if (out && k > 0) std::memcpy(out, counts.data(), size_t(k) * 4);
  API_END
}

int avbd_world_colors(avbd_world* w, int32_t* out) {
  API_BEGIN
  REQUIRE(w && out, "null argument");
  Arena& A = *w->A;
  bind(A.ctx);
  const WorldRec& R = A.resident(w->w);
  auto c = A.fetch(A.T.color, size_t(R.which) * A.bodyCap + R.dev.bodyOff, size_t(R.nBodies));
  if (!c.empty()) std::memcpy(out, c.data(), c.size() * 4);
  API_END
}

int avbd_world_state_sizes(avbd_world* w, int32_t* n_joints, int64_t* n_manifolds, int64_t* n_contacts) {
  API_BEGIN
  REQUIRE(w && n_joints && n_manifolds && n_contacts, "null argument");
  bind(w->A->ctx);
  std::vector<uint2> pairs;
  std::vector<int> counts;
  w->A->lastPairsOf(w->w, pairs, &counts, nullptr);
  int64_t m = 0, c = 0;
  for (int v : counts) { m += v > 0; c += v; }
  *n_joints = w->A->W[w->w].nJoints;
  *n_manifolds = m;
  *n_contacts = c;
  API_END
}

int avbd_world_export_state(avbd_world* w, float* jpen_lin, float* jpen_ang, float* jlam_lin, float* jlam_ang, int32_t* jbroken,
                            uint32_t* mpairs, int32_t* mcount, uint32_t* cfeature, float* cra, float* crb, float* cpen, float* clam,
                            int32_t* cstick) {
  API_BEGIN
  REQUIRE(w, "null world");
  Arena& A = *w->A;
  bind(A.ctx);
  const WorldRec& R = A.resident(w->w);
  const int nj = R.nJoints;
  const size_t joff = R.dev.jointOff;
  auto put3 = [&](float* o, const float4* d) {
    auto h = A.fetch(d, joff, size_t(nj));
    for (int i = 0; i < nj; i++) { o[3 * i] = h[i].x; o[3 * i + 1] = h[i].y; o[3 * i + 2] = h[i].z; }
  };
  if (nj) {
    REQUIRE(jpen_lin && jpen_ang && jlam_lin && jlam_ang && jbroken, "null joint buffer");
    put3(jpen_lin, A.J.penLin);
    put3(jpen_ang, A.J.penAng);
    put3(jlam_lin, A.J.lamLin);
    put3(jlam_ang, A.J.lamAng);
    auto b = A.fetch(A.J.broken, joff, size_t(nj));
    std::memcpy(jbroken, b.data(), size_t(nj) * 4);
  }
  std::vector<uint2> pairs;
  std::vector<int> counts;
  std::vector<float4> ct;
  A.lastPairsOf(w->w, pairs, &counts, &ct);
  const uint32_t off = uint32_t(R.dev.bodyOff);
  int64_t m = 0, c = 0;
  for (size_t p = 0; p < pairs.size(); p++) {
    if (counts[p] == 0) continue;
    mpairs[2 * m] = pairs[p].x - off;
    mpairs[2 * m + 1] = pairs[p].y - off;
    mcount[m] = counts[p];
    m++;
    for (int k = 0; k < counts[p]; k++, c++) {
      const float4* o = &ct[(p * MAX_CONTACTS + k) * 4];
      uint32_t key;
      std::memcpy(&key, &o[0].w, 4);
      cfeature[c] = key & ~STICK_BIT;
      cstick[c] = (key & STICK_BIT) ? 1 : 0;
      cra[3 * c] = o[0].x; cra[3 * c + 1] = o[0].y; cra[3 * c + 2] = o[0].z;
      crb[3 * c] = o[1].x; crb[3 * c + 1] = o[1].y; crb[3 * c + 2] = o[1].z;
      cpen[3 * c] = o[2].x; cpen[3 * c + 1] = o[2].y; cpen[3 * c + 2] = o[2].z;
      clam[3 * c] = o[3].x; clam[3 * c + 1] = o[3].y; clam[3 * c + 2] = o[3].z;
    }
  }
  API_END
}

int avbd_world_profile(avbd_world* w, int32_t enable) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->profile(enable != 0);
  API_END
}

int avbd_world_profile_read(avbd_world* w, avbd_profile* out) {
  API_BEGIN
  REQUIRE(w && out, "null argument");
  bind(w->A->ctx);
  w->A->profileRead(out);
  API_END
}

// ---------------------------------------------------------------- batches

int avbd_batch_create(avbd_ctx* ctx, const avbd_scene_desc* scenes, const avbd_params* params, int32_t n_worlds, avbd_batch** out) {
  API_BEGIN
  REQUIRE(ctx && scenes && params && out, "null argument");
  REQUIRE(n_worlds > 0, "need at least one world");
  bind(ctx);
  std::vector<int> slots;
  Arena* A = arenaFor(ctx, scenes, params, n_worlds, slots);
  int64_t nb = 0;
  for (int i = 0; i < n_worlds; i++) nb += scenes[i].n_bodies;
  *out = new avbd_batch{A, slots, nb};
  API_END
}

int avbd_batch_destroy(avbd_batch* b) {
  API_BEGIN
  if (!b) return AVBD_OK;
  avbd_ctx* ctx = b->A->ctx;
  bind(ctx);
  forget(ctx, b->A);
  delete b->A;
  delete b;
  API_END
}

int avbd_batch_step(avbd_batch* b, int32_t steps) {
  API_BEGIN
  REQUIRE(b, "null batch");
  REQUIRE(steps >= 0, "steps must be non-negative");
  bind(b->A->ctx);
  for (int i = 0; i < steps; i++) b->A->stepWorlds(b->worlds);
  API_END
}

int avbd_batch_world_count(avbd_batch* b, int32_t* n_worlds, int64_t* n_bodies) {
  API_BEGIN
  REQUIRE(b, "null batch");
  if (n_worlds) *n_worlds = int32_t(b->worlds.size());
  if (n_bodies) *n_bodies = b->bodies;
  API_END
}

int avbd_batch_read_state(avbd_batch* b, int32_t world, float* position, float* rotation, float* velocity, float* angular,
                          float* prev_velocity) {
  API_BEGIN
  REQUIRE(b, "null batch");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  bind(b->A->ctx);
  b->A->readState(b->worlds[world], position, rotation, velocity, angular, prev_velocity);
  API_END
}

int avbd_batch_read_poses(avbd_batch* b, float* out) {
  API_BEGIN
  REQUIRE(b && out, "null argument");
  Arena& A = *b->A;
  bind(A.ctx);
  const int n = int(b->bodies);  // the batch's worlds occupy bodies [0, n) in creation order
  if (n == 0) return AVBD_OK;
  if (!A.poseStage) A.poseStage = dalloc<float4>(size_t(n) * 2);
  int blocks = grid_blocks(n, 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_read_poses<<<blocks, 256, 0, A.s>>>(A.B.pos, A.B.rot, A.B.size, n, A.poseStage); note_launches(1);
  CK(cudaMemcpyAsync(out, A.poseStage, size_t(n) * 32, cudaMemcpyDeviceToHost, A.s));
  CK(cudaStreamSynchronize(A.s));
  API_END
}

int avbd_batch_set_velocities(avbd_batch* b, const uint32_t* indices, int32_t n, const float* velocity, const float* angular) {
  API_BEGIN
  REQUIRE(b, "null batch");
  bind(b->A->ctx);
  setVelocities(*b->A, 0, int(b->bodies), indices, n, velocity, angular);
  API_END
}

int avbd_batch_profile(avbd_batch* b, int32_t enable) {
  API_BEGIN
  REQUIRE(b, "null batch");
  bind(b->A->ctx);
  b->A->profile(enable != 0);
  API_END
}

int avbd_batch_profile_read(avbd_batch* b, avbd_profile* out) {
  API_BEGIN
  REQUIRE(b && out, "null argument");
  bind(b->A->ctx);
  b->A->profileRead(out);
  API_END
}

int avbd_batch_counters(avbd_batch* b, avbd_counters* out) {
  API_BEGIN
  REQUIRE(b && out, "null argument");
  bind(b->A->ctx);
  b->A->counters(out);
  API_END
}

}  // extern "C"
