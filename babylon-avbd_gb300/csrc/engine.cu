// Host orchestration of the AVBD engine and the C ABI (include/avbd_gb300.h).
//
// A WorldSet holds one or many independent worlds in one set of device arrays (bodies,
// joints and pairs concatenated, each world a contiguous range). One step is one launch
// sequence over every body of every world:
//
//   collision   grid build -> pair count / scan / write -> narrowphase + warm-start match
//   topology    constraint lists (CSR, sorted) -> Jones-Plassmann colouring -> colour buckets
//   [one 600-byte counter readback: pair overflow check, colour sizes]
//   solve       joint warm start -> body warm start -> iterations x (colours + dual) -> velocities
//
// Everything before the readback writes only this step's buffers (pairs, contacts, lists,
// colours); the previous step's manifolds and colours are kept until the step completes. When
// the pair capacity overflows, the buffers grow and the step is re-run from the same state,
// so a capacity change never alters the result. The reference's counterpart is
// src/gpu/gpuSolverStep.js:16-256 (one WebGPU submission per step with held steps on overflow).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/avbd_gb300.h"
#include "engine.cuh"

namespace avbd {
void launch_joint_prepare(const BodyPtrs& b, JointPtrs j, int nJoints, cudaStream_t s);
}

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

}  // namespace

struct avbd_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<void*> owned;  // WorldSets created under this context
};

namespace avbd {

class WorldSet {
 public:
  avbd_ctx* ctx;
  cudaStream_t s;
  int nBodies = 0, nJoints = 0, nWorlds = 0;
  std::vector<WorldDev> worldsHost;
  WorldDev* worlds = nullptr;
  BodyPtrs B{};
  JointPtrs J{};
  PairPtrs P[2]{};
  int* pairN[2] = {nullptr, nullptr};
  int cur = 0;
  int capacity = 0;
  Grid G{};
  NarrowScratch NS{};
  NoCollide NC{};
  Topo T{};
  int* pairCount = nullptr;
  int* pairStart = nullptr;
  Counters* ctr = nullptr;
  Counters* ctrHost = nullptr;
  void* scanTemp = nullptr;
  size_t scanBytes = 0;
  int maxIter = 0, rounds = 64;
  size_t itemCap = 0;
  int steps = 0, regrowths = 0;
  bool haveStats = false;
  // profiling: event pairs per kernel class, harvested after each step's counter readback
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
  unsigned long long* traffic = nullptr;  // device: primal, dual, collide bytes (accumulated)
  uint4* poseStage = nullptr;             // batch pose readback staging

  WorldSet(avbd_ctx* c, const avbd_scene_desc* scenes, const avbd_params* params, int n) : ctx(c), s(c->stream) {
    build(scenes, params, n);
  }
  ~WorldSet() {
    harvest();
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
    release();
  }

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
  // all recorded events have completed (called after a stream synchronisation)
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
    profPrimalLaunches = 0;
    profSteps = 0;
    if (!traffic) traffic = dalloc<unsigned long long>(3);
    CK(cudaMemset(traffic, 0, 3 * sizeof(unsigned long long)));
  }
  void profileRead(avbd_profile* o) {
    CK(cudaStreamSynchronize(s));
    harvest();
    unsigned long long t[3] = {0, 0, 0};
    if (traffic) CK(cudaMemcpy(t, traffic, sizeof(t), cudaMemcpyDeviceToHost));
    std::memset(o, 0, sizeof(*o));
    o->steps = profSteps;
    o->ms_collide = profMs[P_COLLIDE];
    o->ms_topology = profMs[P_TOPO];
    o->ms_primal = profMs[P_PRIMAL];
    o->ms_dual = profMs[P_DUAL];
    o->ms_other = profMs[P_OTHER];
    o->primal_launches = profPrimalLaunches;
    o->launches = launches_total();
    // traffic holds per-iteration primal/dual bytes summed over steps; scale by iterations
    o->bytes_primal = double(t[0]) * maxIter;
    o->bytes_dual = double(t[1]) * maxIter;
    o->bytes_collide = double(t[2]);
  }

  void release() {
    void* ptrs[] = {worlds, B.pos, B.rot, B.pos0, B.rot0, B.posY, B.rotY, B.vel, B.ang, B.vprev, B.size, B.mass, B.meta,
                    J.ab, J.rA, J.rB, J.stiff, J.penLin, J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang, J.restQ, J.broken,
                    G.cellCount, G.cellFill, G.cellBodies, G.bodyBucket, G.large, NC.keys, NC.jid, T.adjStart, T.adjFill,
                    T.colorPrev, T.color, T.won, T.pending, T.colorBodies, T.itemStart, T.itemRef, T.contrib, pairCount,
                    pairStart, ctr, scanTemp, traffic, poseStage};
    for (void* p : ptrs) dfree(p);
    freePairs();
    if (ctrHost) cudaFreeHost(ctrHost);
    ctrHost = nullptr;
  }

  void freePairs() {
    for (int k = 0; k < 2; k++) {
      dfree(P[k].pair);
      dfree(P[k].count);
      dfree(P[k].basis);
      dfree(P[k].ct);
      dfree(pairN[k]);
      P[k] = PairPtrs{};
      pairN[k] = nullptr;
    }
    dfree(T.adjList);
    T.adjList = nullptr;
    dfree(NS.sat);
    dfree(NS.boxList);
    dfree(NS.sphereList);
    dfree(NS.ctr);
    NS = NarrowScratch{};
  }

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

  void build(const avbd_scene_desc* scenes, const avbd_params* params, int n) {
    if (n <= 0) throw Error(AVBD_E_INVALID, "need at least one world");
    nWorlds = n;
    for (int w = 0; w < n; w++) validate(scenes[w], params[w]);
    // ---------------- ranges
    worldsHost.resize(n);
    std::vector<int> largeAll;
    int bodyOff = 0, jointOff = 0;
    for (int w = 0; w < n; w++) {
      const avbd_scene_desc& d = scenes[w];
      const avbd_params& p = params[w];
      WorldDev& W = worldsHost[w];
      std::memset(&W, 0, sizeof(W));
      W.dt = p.dt;
      W.gravity = p.gravity;
      W.alpha = p.alpha;
      W.gamma = p.gamma;
      W.betaLin = p.beta_lin;
      W.betaAng = p.beta_ang;
      W.up0 = p.up[0];
      W.up1 = p.up[1];
      W.up2 = p.up[2];
      W.iterations = p.iterations;
      W.flags = (p.mass_penalty ? FLAG_MASS_PENALTY : 0) | (p.face_bias ? FLAG_FACE_BIAS : 0);
      W.bodyOff = bodyOff;
      W.bodyCount = d.n_bodies;
      int nj = 0;
      for (int c = 0; c < d.n_cons; c++) nj += d.cons_kind[c] != AVBD_CONS_IGNORE;
      W.jointOff = jointOff;
      W.jointCount = nj;
      // large bodies: radius > 2 x median, at most 64 of them (the largest)
      std::vector<float> radii(d.radius, d.radius + d.n_bodies);
      float largeR = INFINITY;
      if (d.n_bodies > 0) {
        std::vector<float> sorted = radii;
        std::sort(sorted.begin(), sorted.end());
        float med = sorted[sorted.size() / 2];
        float thr = 2.f * med;
        int nl = 0;
        for (float r : sorted) nl += r > thr;
        if (nl > 64) thr = sorted[sorted.size() - 65];
        float maxSmall = 0.f;
        for (float r : sorted)
          if (!(r > thr)) maxSmall = std::max(maxSmall, r);
        largeR = thr;
        W.cell = std::max(2.f * maxSmall * 1.001f, 1e-3f);
      } else {
        W.cell = 1.f;
      }
      W.largeR = largeR;
      W.largeOff = int(largeAll.size());
      for (int i = 0; i < d.n_bodies; i++)
        if (d.radius[i] > largeR) largeAll.push_back(bodyOff + i);
      W.largeCount = int(largeAll.size()) - W.largeOff;
      maxIter = std::max(maxIter, p.iterations);
      rounds = std::max(rounds, p.color_rounds > 0 ? p.color_rounds : 64);
      bodyOff += d.n_bodies;
      jointOff += nj;
    }
    nBodies = bodyOff;
    nJoints = jointOff;
    // ---------------- bodies
    const size_t N = size_t(std::max(nBodies, 1));
    std::vector<float4> pos(N), rot(N), zero(N, make_float4(0, 0, 0, 0)), vel(N), ang(N), vprev(N), size(N), mass(N);
    std::vector<int4> meta(N);
    for (int w = 0; w < n; w++) {
      const avbd_scene_desc& d = scenes[w];
      const int off = worldsHost[w].bodyOff;
      for (int i = 0; i < d.n_bodies; i++) {
        const int g = off + i;
        auto v3at = [&](const float* a, int k) { return a ? make_float4(a[3 * k], a[3 * k + 1], a[3 * k + 2], 0.f) : make_float4(0, 0, 0, 0); };
        pos[g] = v3at(d.position, i);
        pos[g].w = d.radius[i];
        rot[g] = d.rotation ? make_float4(d.rotation[4 * i], d.rotation[4 * i + 1], d.rotation[4 * i + 2], d.rotation[4 * i + 3])
                            : make_float4(0, 0, 0, 1);
        vel[g] = v3at(d.velocity, i);
        ang[g] = v3at(d.angular_velocity, i);
        vprev[g] = v3at(d.prev_velocity, i);
        size[g] = v3at(d.size, i);
        size[g].w = d.friction[i];
        mass[g] = make_float4(d.mass[i], d.moment[3 * i], d.moment[3 * i + 1], d.moment[3 * i + 2]);
        uint32_t grp = d.group ? d.group[i] : 0xffffffffu, msk = d.collides_with ? d.collides_with[i] : 0xffffffffu;
        meta[g] = make_int4(w, d.shape[i], int(grp), int(msk));
      }
    }
    B.pos = dalloc<float4>(N); B.rot = dalloc<float4>(N); B.pos0 = dalloc<float4>(N); B.rot0 = dalloc<float4>(N);
    B.posY = dalloc<float4>(N); B.rotY = dalloc<float4>(N); B.vel = dalloc<float4>(N); B.ang = dalloc<float4>(N);
    B.vprev = dalloc<float4>(N); B.size = dalloc<float4>(N); B.mass = dalloc<float4>(N); B.meta = dalloc<int4>(N);
    CK(cudaMemcpy(B.pos, pos.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.rot, rot.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.pos0, pos.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.rot0, rot.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.posY, pos.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.rotY, rot.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.vel, vel.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.ang, ang.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.vprev, vprev.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.size, size.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.mass, mass.data(), N * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.meta, meta.data(), N * 16, cudaMemcpyHostToDevice));
    worlds = dalloc<WorldDev>(n);
    CK(cudaMemcpy(worlds, worldsHost.data(), sizeof(WorldDev) * n, cudaMemcpyHostToDevice));
    // ---------------- joints, springs, no-collide pairs
    const size_t NJ = size_t(std::max(nJoints, 1));
    std::vector<int2> jab(NJ);
    std::vector<float4> jra(NJ), jrb(NJ), jst(NJ), jz(NJ, make_float4(0, 0, 0, 0)), jq(NJ, make_float4(0, 0, 0, 1));
    std::vector<int> jbroken(NJ, 0);
    std::vector<std::pair<unsigned long long, int>> nc;
    for (int w = 0; w < n; w++) {
      const avbd_scene_desc& d = scenes[w];
      const int off = worldsHost[w].bodyOff;
      int j = worldsHost[w].jointOff;
      for (int c = 0; c < d.n_cons; c++) {
        const int kind = d.cons_kind[c];
        const int a = d.cons_a[c] >= 0 ? off + d.cons_a[c] : -1;
        const int b = off + d.cons_b[c];
        int jid = -1;
        if (kind != AVBD_CONS_IGNORE) {
          jid = j++;
          jab[jid] = make_int2(a, b);
          int kk = kind == AVBD_CONS_JOINT ? KIND_JOINT : KIND_SPRING;
          float kf;
          std::memcpy(&kf, &kk, 4);
          jra[jid] = make_float4(d.cons_ra[3 * c], d.cons_ra[3 * c + 1], d.cons_ra[3 * c + 2], kf);
          jrb[jid] = make_float4(d.cons_rb[3 * c], d.cons_rb[3 * c + 1], d.cons_rb[3 * c + 2], kind == AVBD_CONS_SPRING ? d.cons_p1[c] : 0.f);
          jst[jid] = kind == AVBD_CONS_JOINT ? make_float4(d.cons_p0[c], d.cons_p1[c], d.cons_p2[c], 0.f)
                                             : make_float4(d.cons_p0[c], 0.f, INFINITY, 0.f);
        }
        if (a >= 0) nc.push_back({(unsigned long long)(uint32_t)std::max(a, b) << 32 | (uint32_t)std::min(a, b), jid});
      }
    }
    std::sort(nc.begin(), nc.end());
    J.ab = dalloc<int2>(NJ); J.rA = dalloc<float4>(NJ); J.rB = dalloc<float4>(NJ); J.stiff = dalloc<float4>(NJ);
    J.penLin = dalloc<float4>(NJ); J.penAng = dalloc<float4>(NJ); J.lamLin = dalloc<float4>(NJ); J.lamAng = dalloc<float4>(NJ);
    J.C0Lin = dalloc<float4>(NJ); J.C0Ang = dalloc<float4>(NJ); J.restQ = dalloc<float4>(NJ); J.broken = dalloc<int>(NJ);
    CK(cudaMemcpy(J.ab, jab.data(), NJ * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J.rA, jra.data(), NJ * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J.rB, jrb.data(), NJ * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J.stiff, jst.data(), NJ * 16, cudaMemcpyHostToDevice));
    for (float4* p : {J.penLin, J.penAng, J.lamLin, J.lamAng, J.C0Lin, J.C0Ang})
      CK(cudaMemcpy(p, jz.data(), NJ * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J.restQ, jq.data(), NJ * 16, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J.broken, jbroken.data(), NJ * 4, cudaMemcpyHostToDevice));
    NC.n = int(nc.size());
    NC.keys = dalloc<unsigned long long>(std::max<size_t>(nc.size(), 1));
    NC.jid = dalloc<int>(std::max<size_t>(nc.size(), 1));
    {
      std::vector<unsigned long long> k(nc.size());
      std::vector<int> id(nc.size());
      for (size_t i = 0; i < nc.size(); i++) { k[i] = nc[i].first; id[i] = nc[i].second; }
      if (!nc.empty()) {
        CK(cudaMemcpy(NC.keys, k.data(), k.size() * 8, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(NC.jid, id.data(), id.size() * 4, cudaMemcpyHostToDevice));
      }
    }
    launch_joint_prepare(B, J, nJoints, s);
    // ---------------- grid
    uint32_t table = 1024;
    while (table < 2u * uint32_t(N)) table <<= 1;
    G.tableMask = table - 1;
    G.cellCount = dalloc<int>(table + 1);
    G.cellFill = dalloc<int>(table);
    G.cellBodies = dalloc<int>(N);
    G.bodyBucket = dalloc<int>(N);
    G.large = dalloc<int>(std::max<size_t>(largeAll.size(), 1));
    if (!largeAll.empty()) CK(cudaMemcpy(G.large, largeAll.data(), largeAll.size() * 4, cudaMemcpyHostToDevice));
    // ---------------- topology
    T.adjStart = dalloc<int>(N + 1);
    T.adjFill = dalloc<int>(std::max<size_t>(N + 1, MAX_COLORS));
    T.colorPrev = dalloc<int>(N);
    T.color = dalloc<int>(N);
    T.won = dalloc<int>(N);
    T.pending = dalloc<unsigned char>(N);
    T.colorBodies = dalloc<int>(N);
    T.itemStart = dalloc<int>(N + 1);
    std::vector<int> minus(N, -1);
    CK(cudaMemcpy(T.colorPrev, minus.data(), N * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(T.color, minus.data(), N * 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(T.pending, 0, N));
    pairCount = dalloc<int>(N);
    pairStart = dalloc<int>(N);
    ctr = dalloc<Counters>(1);
    CK(cudaMemset(ctr, 0, sizeof(Counters)));
    CK(cudaHostAlloc((void**)&ctrHost, sizeof(Counters), cudaHostAllocDefault));
    std::memset(ctrHost, 0, sizeof(Counters));
    // ---------------- pairs
    allocPairs(std::max(1024, 6 * nBodies), false);
    CK(cudaStreamSynchronize(s));
  }

  size_t scanNeed() const {
    size_t a = scan_temp_bytes(int(G.tableMask) + 2);
    size_t b = scan_temp_bytes(nBodies + 1);
    return std::max(a, b);
  }

  void allocPairs(int cap, bool keepPrev) {
    PairPtrs old = P[cur ^ 1];
    int* oldN = pairN[cur ^ 1];
    const int oldCap = capacity;
    PairPtrs np[2];
    int* nn[2];
    for (int k = 0; k < 2; k++) {
      np[k].pair = dalloc<uint2>(cap);
      np[k].count = dalloc<int>(cap);
      np[k].basis = dalloc<float4>(size_t(cap) * 3);
      np[k].ct = dalloc<float4>(size_t(cap) * MAX_CONTACTS * 4);
      nn[k] = dalloc<int>(1);
      CK(cudaMemsetAsync(nn[k], 0, sizeof(int), s));
    }
    const int prevIdx = cur ^ 1;
    if (keepPrev && old.pair) {
      CK(cudaMemcpyAsync(np[prevIdx].pair, old.pair, size_t(oldCap) * sizeof(uint2), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(np[prevIdx].count, old.count, size_t(oldCap) * sizeof(int), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(np[prevIdx].basis, old.basis, size_t(oldCap) * 3 * sizeof(float4), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(np[prevIdx].ct, old.ct, size_t(oldCap) * MAX_CONTACTS * 4 * sizeof(float4), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(nn[prevIdx], oldN, sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
    CK(cudaStreamSynchronize(s));
    freePairs();
    for (int k = 0; k < 2; k++) {
      P[k] = np[k];
      pairN[k] = nn[k];
    }
    capacity = cap;
    T.adjList = dalloc<uint32_t>(2 * (size_t(nJoints) + size_t(cap)) + 1);
    NS.sat = dalloc<float4>(cap);
    NS.boxList = dalloc<int>(cap);
    NS.sphereList = dalloc<int>(cap);
    NS.ctr = dalloc<int>(2);
    size_t need = scanNeed();
    if (need > scanBytes) {
      dfree(scanTemp);
      scanTemp = dalloc<char>(need);
      scanBytes = need;
    }
  }

  // item lists and the per-colour contribution planes, sized from this step's counts
  void ensureItems() {
    size_t need = size_t(std::max(ctrHost->itemsTotal, 1));
    int maxColor = 1;
    for (int c = 0; c < MAX_COLORS; c++) maxColor = std::max(maxColor, ctrHost->colorItems[c]);
    if (need > itemCap || maxColor > T.contribCap) {
      CK(cudaStreamSynchronize(s));
      size_t cap = std::max(need, itemCap);
      cap = cap + cap / 4 + 1024;
      dfree(T.itemRef);
      T.itemRef = nullptr;
      T.itemRef = dalloc<int2>(cap);
      itemCap = cap;
      int ccap = std::max(maxColor, T.contribCap);
      ccap = ccap + ccap / 4 + 1024;
      dfree(T.contrib);
      T.contrib = nullptr;
      T.contrib = dalloc<float4>(size_t(ccap) * 7);
      T.contribCap = ccap;
    }
  }

  // ------------------------------------------------------------------ step
  void collideAndColor() {
    PairPtrs& C = P[cur];
    PairPtrs& Pv = P[cur ^ 1];
    cudaEvent_t e0 = prof ? mark() : nullptr;
    launch_grid_build(B, worlds, nBodies, G, scanTemp, s);
    launch_pairs(B, worlds, nBodies, G, NC, J.broken, pairCount, pairStart, C.pair, capacity, ctr, scanTemp, s);
    CK(cudaMemcpyAsync(pairN[cur], &ctr->npairs, sizeof(int), cudaMemcpyDeviceToDevice, s));
    launch_narrowphase(B, worlds, C, Pv, pairN[cur ^ 1], pairN[cur], capacity, NS, s);
    // every span owns its two events (the pool recycles each event exactly once)
    cudaEvent_t e1 = prof ? mark() : nullptr;
    cudaEvent_t e1b = prof ? mark() : nullptr;
    launch_adjacency(B, J, nJoints, C, pairN[cur], capacity, T, nBodies, scanTemp, s);
    launch_coloring(B, worlds, J, C, T, nBodies, rounds, ctr, s);
    launch_items_count(C, T, nBodies, ctr, scanTemp, s);
    if (prof) {
      cudaEvent_t e2 = mark();
      span(P_COLLIDE, e0, e1);
      span(P_TOPO, e1b, e2);
    }
    CK(cudaMemcpyAsync(ctrHost, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    if (prof) harvest();
  }

  void step() {
    for (int attempt = 0;; attempt++) {
      collideAndColor();
      if (ctrHost->pairsNeeded <= capacity) break;
      if (attempt > 8) throw Error(AVBD_E_CAPACITY, "pair capacity did not converge");
      long long want = (long long)ctrHost->pairsNeeded * 5 / 4 + 1024;
      if (want > 0x7fffffffLL / (MAX_CONTACTS * 4)) throw Error(AVBD_E_CAPACITY, "pair capacity limit exceeded");
      allocPairs(int(want), true);
      regrowths++;
    }
    PairPtrs& C = P[cur];
    ensureItems();
    launch_items_fill(C, T, nBodies, ctr, s);
    cudaEvent_t o0 = prof ? mark() : nullptr;
    launch_joint_warmstart(B, worlds, J, nJoints, ctr, s);
    launch_body_warmstart(B, worlds, nBodies, s);
    if (prof) span(P_OTHER, o0, mark());
    const int ncolors = ctrHost->ncolors;
    for (int it = 0; it < maxIter; it++) {
      for (int c = 0; c < ncolors; c++) {
        const int cnt = ctrHost->colorCount[c];
        if (!cnt) continue;
        cudaEvent_t a = prof ? mark() : nullptr;
        launch_primal(B, worlds, J, C, T, ctr, c, it, cnt, ctrHost->colorItems[c], s);
        if (prof) {
          span(P_PRIMAL, a, mark());
          profPrimalLaunches++;
        }
      }
      cudaEvent_t d = prof ? mark() : nullptr;
      launch_dual(B, worlds, J, nJoints, C, pairN[cur], capacity, it, s);
      if (prof) span(P_DUAL, d, mark());
    }
    cudaEvent_t v0 = prof ? mark() : nullptr;
    launch_velocities(B, worlds, nBodies, s);
    if (prof) {
      span(P_OTHER, v0, mark());
      launch_traffic(B, J, nJoints, C, pairN[cur], capacity, T, nBodies, traffic, s);
      profSteps++;
    }
    std::swap(T.colorPrev, T.color);
    cur ^= 1;
    steps++;
    haveStats = false;
    CK(cudaGetLastError());
  }

  void syncStats() {
    if (haveStats) return;
    // stats of the last step: its pairs are now the "previous" buffer
    launch_count_active(J, nJoints, P[cur ^ 1], pairN[cur ^ 1], capacity, ctr, s);
    CK(cudaMemcpyAsync(ctrHost, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    haveStats = true;
  }

  void counters(avbd_counters* o) {
    syncStats();
    o->pairs = ctrHost->npairs;
    o->manifolds = ctrHost->manifolds;
    o->contacts = ctrHost->contacts;
    o->joints = ctrHost->joints;
    o->colors = ctrHost->ncolors;
    o->conflicts = ctrHost->conflicts;
    o->overflow = regrowths;
    o->steps = steps;
  }

  // ------------------------------------------------------------------ reads
  template <class T> std::vector<T> fetch(const T* d, size_t off, size_t n) {
    std::vector<T> h(n);
    if (n) CK(cudaMemcpyAsync(h.data(), d + off, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return h;
  }

  void readState(int world, float* position, float* rotation, float* velocity, float* angular, float* prevVel) {
    const WorldDev& W = worldsHost[world];
    const size_t off = W.bodyOff, n = W.bodyCount;
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
};

}  // namespace avbd

struct avbd_world {
  WorldSet* set;
};
struct avbd_batch {
  WorldSet* set;
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
template <class T> T* upload(const T* h, size_t n, cudaStream_t s) {
  T* d = dalloc<T>(n);
  CK(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
  return d;
}

}  // namespace

extern "C" {

const char* avbd_last_error(void) { return g_error.c_str(); }
const char* avbd_version(void) { return "avbd_gb300 0.1.0 (sm_103a)"; }

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
  for (void* p : ctx->owned) delete static_cast<WorldSet*>(p);
  ctx->owned.clear();
  cudaStreamSynchronize(ctx->stream);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  API_END
}

int avbd_world_create(avbd_ctx* ctx, const avbd_scene_desc* scene, const avbd_params* params, avbd_world** out) {
  API_BEGIN
  REQUIRE(ctx && scene && params && out, "null argument");
  bind(ctx);
  auto* set = new WorldSet(ctx, scene, params, 1);
  ctx->owned.push_back(set);
  *out = new avbd_world{set};
  API_END
}

static void forget(avbd_ctx* ctx, WorldSet* set) {
  auto& v = ctx->owned;
  v.erase(std::remove(v.begin(), v.end(), (void*)set), v.end());
}

int avbd_world_destroy(avbd_world* w) {
  API_BEGIN
  if (!w) return AVBD_OK;
  avbd_ctx* ctx = w->set->ctx;
  bind(ctx);
  forget(ctx, w->set);
  delete w->set;
  delete w;
  API_END
}

int avbd_world_step(avbd_world* w, int32_t steps) {
  API_BEGIN
  REQUIRE(w, "null world");
  REQUIRE(steps >= 0, "steps must be non-negative");
  bind(w->set->ctx);
  for (int i = 0; i < steps; i++) w->set->step();
  API_END
}

int avbd_world_read_state(avbd_world* w, float* position, float* rotation, float* velocity, float* angular, float* prev_velocity) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->set->ctx);
  w->set->readState(0, position, rotation, velocity, angular, prev_velocity);
  API_END
}

int avbd_world_read_selected(avbd_world* w, const uint32_t* indices, int32_t n, int32_t poses_only, float* out) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (indices && out)), "null argument");
  REQUIRE(n >= 0, "negative count");
  WorldSet& S = *w->set;
  bind(S.ctx);
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(S.worldsHost[0].bodyCount), "body index out of range");
  if (n == 0) return AVBD_OK;
  const int stride = poses_only ? 8 : 40;
  uint32_t* di = upload(indices, size_t(n), S.s);
  float* dout = dalloc<float>(size_t(n) * stride);
  k_read_selected<<<grid_blocks(n, 128), 128, 0, S.s>>>(S.B, S.worlds, di, n, 0, poses_only, dout); note_launches(1);
  cudaError_t e = cudaMemcpyAsync(out, dout, size_t(n) * stride * 4, cudaMemcpyDeviceToHost, S.s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(S.s);
  dfree(di);
  dfree(dout);
  if (e != cudaSuccess) throw Error(AVBD_E_CUDA, cudaGetErrorString(e));
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
  WorldSet& S = *w->set;
  bind(S.ctx);
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(S.worldsHost[0].bodyCount), "body index out of range");
  if (n == 0) return AVBD_OK;
  float* scratch = select_scratch(S.ctx->device);
  uint32_t* dIdx = reinterpret_cast<uint32_t*>(scratch);
  float* dOut = scratch + AVBD_NOALLOC_MAX_SELECTED;
  const size_t stride = poses_only ? 8 : 40;
  CK(cudaMemcpyAsync(dIdx, indices, size_t(n) * 4, cudaMemcpyHostToDevice, S.s));
  k_read_selected<<<grid_blocks(n, 128), 128, 0, S.s>>>(S.B, S.worlds, dIdx, n, 0, poses_only, dOut); note_launches(1);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dOut, size_t(n) * stride * 4, cudaMemcpyDeviceToHost, S.s));
  CK(cudaStreamSynchronize(S.s));
  API_END
}

int avbd_world_set_poses(avbd_world* w, const uint32_t* indices, int32_t n, const float* position, const float* rotation) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (indices && position)), "null argument");
  WorldSet& S = *w->set;
  bind(S.ctx);
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(S.worldsHost[0].bodyCount), "body index out of range");
  for (int k = 0; k < 3 * n; k++) REQUIRE(std::isfinite(position[k]), "positions must be finite");
  if (rotation)
    for (int k = 0; k < n; k++) {
      const float* q = rotation + 4 * k;
      REQUIRE(std::isfinite(q[0]) && std::isfinite(q[1]) && std::isfinite(q[2]) && std::isfinite(q[3]) &&
                  (q[0] != 0 || q[1] != 0 || q[2] != 0 || q[3] != 0),
              "rotations must be finite and nonzero");
    }
  if (n == 0) return AVBD_OK;
  uint32_t* di = upload(indices, size_t(n), S.s);
  float* dp = upload(position, size_t(n) * 3, S.s);
  float* dr = rotation ? upload(rotation, size_t(n) * 4, S.s) : nullptr;
  k_set_poses<<<grid_blocks(n, 128), 128, 0, S.s>>>(S.B, di, n, 0, dp, dr); note_launches(1);
  cudaError_t e = cudaStreamSynchronize(S.s);
  dfree(di);
  dfree(dp);
  dfree(dr);
  if (e != cudaSuccess) throw Error(AVBD_E_CUDA, cudaGetErrorString(e));
  API_END
}

int avbd_world_set_velocities(avbd_world* w, const uint32_t* indices, int32_t n, const float* velocity, const float* angular) {
  API_BEGIN
  REQUIRE(w && (n == 0 || indices), "null argument");
  WorldSet& S = *w->set;
  bind(S.ctx);
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(S.worldsHost[0].bodyCount), "body index out of range");
  for (int k = 0; velocity && k < 3 * n; k++) REQUIRE(std::isfinite(velocity[k]), "velocities must be finite");
  for (int k = 0; angular && k < 3 * n; k++) REQUIRE(std::isfinite(angular[k]), "velocities must be finite");
  if (n == 0 || (!velocity && !angular)) return AVBD_OK;
  uint32_t* di = upload(indices, size_t(n), S.s);
  float* dv = velocity ? upload(velocity, size_t(n) * 3, S.s) : nullptr;
  float* da = angular ? upload(angular, size_t(n) * 3, S.s) : nullptr;
  k_set_velocities<<<grid_blocks(n, 128), 128, 0, S.s>>>(S.B, di, n, 0, dv, da); note_launches(1);
  cudaError_t e = cudaStreamSynchronize(S.s);
  dfree(di);
  dfree(dv);
  dfree(da);
  if (e != cudaSuccess) throw Error(AVBD_E_CUDA, cudaGetErrorString(e));
  API_END
}

int avbd_world_counters(avbd_world* w, avbd_counters* out) {
  API_BEGIN
  REQUIRE(w && out, "null argument");
  bind(w->set->ctx);
  w->set->counters(out);
  API_END
}

int avbd_world_pairs(avbd_world* w, uint32_t* out, int64_t cap, int64_t* n) {
  API_BEGIN
  REQUIRE(w && n, "null argument");
  WorldSet& S = *w->set;
  bind(S.ctx);
  const int prev = S.cur ^ 1;
  int cnt = 0;
  CK(cudaMemcpy(&cnt, S.pairN[prev], 4, cudaMemcpyDeviceToHost));
  *n = cnt;
  const int64_t k = std::min<int64_t>(cnt, cap);
  if (k > 0 && out) CK(cudaMemcpy(out, S.P[prev].pair, size_t(k) * 8, cudaMemcpyDeviceToHost));
  API_END
}

int avbd_world_pair_contacts(avbd_world* w, int32_t* out, int64_t cap, int64_t* n) {
  API_BEGIN
  REQUIRE(w && n, "null argument");
  WorldSet& S = *w->set;
  bind(S.ctx);
  const int prev = S.cur ^ 1;
  int cnt = 0;
  CK(cudaMemcpy(&cnt, S.pairN[prev], 4, cudaMemcpyDeviceToHost));
  *n = cnt;
  const int64_t k = std::min<int64_t>(cnt, cap);
  if (k > 0 && out) CK(cudaMemcpy(out, S.P[prev].count, size_t(k) * 4, cudaMemcpyDeviceToHost));
  API_END
}

int avbd_world_colors(avbd_world* w, int32_t* out) {
  API_BEGIN
  REQUIRE(w && out, "null argument");
  WorldSet& S = *w->set;
  bind(S.ctx);
  if (S.nBodies) CK(cudaMemcpy(out, S.T.colorPrev, size_t(S.nBodies) * 4, cudaMemcpyDeviceToHost));
  API_END
}

int avbd_world_state_sizes(avbd_world* w, int32_t* n_joints, int64_t* n_manifolds, int64_t* n_contacts) {
  API_BEGIN
  REQUIRE(w && n_joints && n_manifolds && n_contacts, "null argument");
  WorldSet& S = *w->set;
  bind(S.ctx);
  const int prev = S.cur ^ 1;
  int cnt = 0;
  CK(cudaMemcpy(&cnt, S.pairN[prev], 4, cudaMemcpyDeviceToHost));
  auto counts = S.fetch(S.P[prev].count, 0, size_t(cnt));
  int64_t m = 0, c = 0;
  for (int v : counts) { m += v > 0; c += v; }
  *n_joints = S.nJoints;
  *n_manifolds = m;
  *n_contacts = c;
  API_END
}

int avbd_world_export_state(avbd_world* w, float* jpen_lin, float* jpen_ang, float* jlam_lin, float* jlam_ang, int32_t* jbroken,
                            uint32_t* mpairs, int32_t* mcount, uint32_t* cfeature, float* cra, float* crb, float* cpen, float* clam,
                            int32_t* cstick) {
  API_BEGIN
  REQUIRE(w, "null world");
  WorldSet& S = *w->set;
  bind(S.ctx);
  const int nj = S.nJoints;
  auto put3 = [&](float* o, const float4* d) {
    auto h = S.fetch(d, 0, size_t(nj));
    for (int i = 0; i < nj; i++) { o[3 * i] = h[i].x; o[3 * i + 1] = h[i].y; o[3 * i + 2] = h[i].z; }
  };
  if (nj) {
    REQUIRE(jpen_lin && jpen_ang && jlam_lin && jlam_ang && jbroken, "null joint buffer");
    put3(jpen_lin, S.J.penLin);
    put3(jpen_ang, S.J.penAng);
    put3(jlam_lin, S.J.lamLin);
    put3(jlam_ang, S.J.lamAng);
    auto b = S.fetch(S.J.broken, 0, size_t(nj));
    std::memcpy(jbroken, b.data(), size_t(nj) * 4);
  }
  const int prev = S.cur ^ 1;
  int cnt = 0;
  CK(cudaMemcpy(&cnt, S.pairN[prev], 4, cudaMemcpyDeviceToHost));
  auto pairs = S.fetch(S.P[prev].pair, 0, size_t(cnt));
  auto counts = S.fetch(S.P[prev].count, 0, size_t(cnt));
  auto ct = S.fetch(S.P[prev].ct, 0, size_t(cnt) * MAX_CONTACTS * 4);
  int64_t m = 0, c = 0;
  for (int p = 0; p < cnt; p++) {
    if (counts[p] == 0) continue;
    mpairs[2 * m] = pairs[p].x;
    mpairs[2 * m + 1] = pairs[p].y;
    mcount[m] = counts[p];
    m++;
    for (int k = 0; k < counts[p]; k++, c++) {
      const float4* o = &ct[(size_t(p) * MAX_CONTACTS + k) * 4];
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

int avbd_batch_create(avbd_ctx* ctx, const avbd_scene_desc* scenes, const avbd_params* params, int32_t n_worlds, avbd_batch** out) {
  API_BEGIN
  REQUIRE(ctx && scenes && params && out, "null argument");
  REQUIRE(n_worlds > 0, "need at least one world");
  bind(ctx);
  auto* set = new WorldSet(ctx, scenes, params, n_worlds);
  ctx->owned.push_back(set);
  *out = new avbd_batch{set};
  API_END
}

int avbd_batch_destroy(avbd_batch* b) {
  API_BEGIN
  if (!b) return AVBD_OK;
  avbd_ctx* ctx = b->set->ctx;
  bind(ctx);
  forget(ctx, b->set);
  delete b->set;
  delete b;
  API_END
}

int avbd_batch_step(avbd_batch* b, int32_t steps) {
  API_BEGIN
  REQUIRE(b, "null batch");
  REQUIRE(steps >= 0, "steps must be non-negative");
  bind(b->set->ctx);
  for (int i = 0; i < steps; i++) b->set->step();
  API_END
}

int avbd_batch_world_count(avbd_batch* b, int32_t* n_worlds, int64_t* n_bodies) {
  API_BEGIN
  REQUIRE(b, "null batch");
  if (n_worlds) *n_worlds = b->set->nWorlds;
  if (n_bodies) *n_bodies = b->set->nBodies;
  API_END
}

int avbd_batch_read_state(avbd_batch* b, int32_t world, float* position, float* rotation, float* velocity, float* angular,
                          float* prev_velocity) {
  API_BEGIN
  REQUIRE(b, "null batch");
  REQUIRE(world >= 0 && world < b->set->nWorlds, "world index out of range");
  bind(b->set->ctx);
  b->set->readState(world, position, rotation, velocity, angular, prev_velocity);
  API_END
}

int avbd_batch_read_poses(avbd_batch* b, float* out) {
  API_BEGIN
  REQUIRE(b && out, "null argument");
  WorldSet& S = *b->set;
  bind(S.ctx);
  if (S.nBodies == 0) return AVBD_OK;
  if (!S.poseStage) S.poseStage = reinterpret_cast<uint4*>(dalloc<float4>(size_t(S.nBodies) * 2));
  float4* st = reinterpret_cast<float4*>(S.poseStage);
  int blocks = grid_blocks(S.nBodies, 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_read_poses<<<blocks, 256, 0, S.s>>>(S.B.pos, S.B.rot, S.B.size, S.nBodies, st); note_launches(1);
  CK(cudaMemcpyAsync(out, st, size_t(S.nBodies) * 32, cudaMemcpyDeviceToHost, S.s));
  CK(cudaStreamSynchronize(S.s));
  API_END
}

int avbd_batch_set_velocities(avbd_batch* b, const uint32_t* indices, int32_t n, const float* velocity, const float* angular) {
  API_BEGIN
  REQUIRE(b && (n == 0 || indices), "null argument");
  REQUIRE(n >= 0, "negative count");
  WorldSet& S = *b->set;
  bind(S.ctx);
  for (int k = 0; k < n; k++) REQUIRE(indices[k] < uint32_t(S.nBodies), "body index out of range");
  for (int k = 0; velocity && k < 3 * n; k++) REQUIRE(std::isfinite(velocity[k]), "velocities must be finite");
  for (int k = 0; angular && k < 3 * n; k++) REQUIRE(std::isfinite(angular[k]), "velocities must be finite");
  if (n == 0 || (!velocity && !angular)) return AVBD_OK;
  uint32_t* di = upload(indices, size_t(n), S.s);
  float* dv = velocity ? upload(velocity, size_t(n) * 3, S.s) : nullptr;
  float* da = angular ? upload(angular, size_t(n) * 3, S.s) : nullptr;
  k_set_velocities<<<grid_blocks(n, 128), 128, 0, S.s>>>(S.B, di, n, 0, dv, da); note_launches(1);
  cudaError_t e = cudaStreamSynchronize(S.s);
  dfree(di);
  dfree(dv);
  dfree(da);
  if (e != cudaSuccess) throw Error(AVBD_E_CUDA, cudaGetErrorString(e));
  API_END
}

int avbd_world_profile(avbd_world* w, int32_t enable) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->set->ctx);
  w->set->profile(enable != 0);
  API_END
}

int avbd_world_profile_read(avbd_world* w, avbd_profile* out) {
  API_BEGIN
  REQUIRE(w && out, "null argument");
  bind(w->set->ctx);
  w->set->profileRead(out);
  API_END
}

int avbd_batch_profile(avbd_batch* b, int32_t enable) {
  API_BEGIN
  REQUIRE(b, "null batch");
  bind(b->set->ctx);
  b->set->profile(enable != 0);
  API_END
}

int avbd_batch_profile_read(avbd_batch* b, avbd_profile* out) {
  API_BEGIN
  REQUIRE(b && out, "null argument");
  bind(b->set->ctx);
  b->set->profileRead(out);
  API_END
}

int avbd_batch_counters(avbd_batch* b, avbd_counters* out) {
  API_BEGIN
  REQUIRE(b && out, "null argument");
  bind(b->set->ctx);
  b->set->counters(out);
  API_END
}

}  // extern "C"
