// Run-time autotuner of the tick's launch schedule.
//
// The reference chooses kernel variants at run time from the device and the scene
// (src/gpu/solverPolicy.js:15-52, src/gpu/appGpuSolver3D.js:1024-1050). Here every candidate
// gives the same bits (tests/test_gpu_async.py), so candidates can be timed on the live ticks of
// the workload itself: the first ticks of a workload class on a device each run one candidate
// (direct launches, CUDA events around the timed stage), in rotation, and once every candidate
// has its samples the fastest is kept for that class on that device for the rest of the process.
// The work of those ticks drifts (piles settle, contacts grow), so a solve sample is its time
// per unit of the tick's work (bodies plus contact work items, the items read back with it).
//
// Tuned parameters:
//   solve    schedule (tile queue / colour barriers), chunks per block and colour (the width of a
//            colour-bucket chunk, i.e. bodies per block), work items per shared-memory tile (128 or
//            256), persistent grid size (all resident blocks, or a quarter of the SMs for small
//            ticks);
//   radix    digit width of the tree build's Morton-code sort (4, 6 or 8 bits), on rebuild ticks.
// A workload class is (device, log2 of the tick's bodies, whether it has joints, iterations).
// Environment overrides (AVBD_SOLVE*, AVBD_RADIX_BITS) pin a parameter; AVBD_TUNE=0 keeps the
// defaults.
#pragma once
#include <cuda_runtime.h>

#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "engine.cuh"

namespace avbd {

struct TuneKey {
  int device, sizeLog2, joints, iterations;
  bool operator<(const TuneKey& o) const {
    return std::tie(device, sizeLog2, joints, iterations) < std::tie(o.device, o.sizeLog2, o.joints, o.iterations);
  }
};

// Choices kept for the process, per device and workload class.
struct TuneCache {
  std::mutex m;
  std::map<TuneKey, SolveConfig> solve;
  std::map<TuneKey, int> radix;
  // page-locked slots for the work items of timed ticks (read back in stream order)
  static constexpr int ITEM_SLOTS = 256;
  int* items = nullptr;
  std::vector<int> freeItems;
  static TuneCache& get() {
    static TuneCache c;
    return c;
  }
  int takeItemSlot() {  // with m held; -1 when none is free
    if (!items) {
      if (cudaHostAlloc(reinterpret_cast<void**>(&items), ITEM_SLOTS * sizeof(int), cudaHostAllocPortable) != cudaSuccess) {
        items = nullptr;
        cudaGetLastError();
        return -1;
      }
      for (int k = ITEM_SLOTS - 1; k >= 0; k--) freeItems.push_back(k);
    }
    if (freeItems.empty()) return -1;
    const int k = freeItems.back();
    freeItems.pop_back();
    return k;
  }
};

class Tuner {
 public:
  static constexpr int SAMPLES = 2;  // timed ticks per candidate (the fastest counts)

  bool enabled = true;
  bool solvePinned = false, radixPinned = false;
  SolveConfig base;     // the defaults (with any environment overrides)
  int baseRadix = 8;

  void init(const SolveConfig& cfg) {
    base = cfg;
    const char* t = std::getenv("AVBD_TUNE");
    enabled = !(t && std::atoi(t) == 0);
    solvePinned = std::getenv("AVBD_SOLVE") || std::getenv("AVBD_SOLVE_WAVES") || std::getenv("AVBD_SOLVE_BLOCKS") ||
                  std::getenv("AVBD_SOLVE_TILE") || std::getenv("AVBD_SOLVE_WAIT_PROBE");
    if (const char* r = std::getenv("AVBD_RADIX_BITS")) {
      const int v = std::atoi(r);
      baseRadix = (v == 4 || v == 6) ? v : 8;
      radixPinned = true;
    }
  }

  static std::vector<SolveConfig> solveCandidates(const SolveConfig& b, int sms, int sizeLog2) {
    std::vector<SolveConfig> c;
    auto add = [&](int queue, int waves, int blocks, int tile) {
      SolveConfig x = b;
      x.queue = queue;
      x.waves = waves;
      x.blocks = blocks;
      x.tile = tile;
      c.push_back(x);
    };
    for (int tile : {128, 256}) {
      add(1, 1, 0, tile);
      add(1, 2, 0, tile);
      add(0, 1, 0, tile);
      add(0, 2, 0, tile);
    }
    add(1, 4, 0, 128);
    if (sizeLog2 <= 16) add(0, 1, sms / 4 > 8 ? sms / 4 : 8, 128);  // small ticks: fewer blocks make each colour barrier cheaper
    return c;
  }
  static std::vector<int> radixCandidates() { return {8, 6, 4}; }

  // The configuration for a tick of this class; `timed` tells whether the tick should be timed
  // for the tuner (candidate index in *solveCand / *radixCand, -1 otherwise).
  void pick(const TuneKey& key, bool rebuild, int sms, SolveConfig& solve, int& radix, int& solveCand, int& radixCand,
            bool measure = true) {
    solve = base;
    radix = baseRadix;
    solveCand = radixCand = -1;
    if (!enabled) return;
    if (!measure) {  // no timing possible: the class's choices if known, else the defaults
      TuneCache& C = TuneCache::get();
      std::lock_guard<std::mutex> lock(C.m);
      auto it = C.solve.find(key);
      if (it != C.solve.end() && !solvePinned) solve = it->second;
      auto jt = C.radix.find(key);
      if (jt != C.radix.end() && !radixPinned) radix = jt->second;
      return;
    }
    TuneCache& C = TuneCache::get();
    std::lock_guard<std::mutex> lock(C.m);
    if (!solvePinned) {
      auto it = C.solve.find(key);
      if (it != C.solve.end()) {
        solve = it->second;
      } else {
        auto& st = state(key);
        if (st.solveCands.empty()) {
          st.solveCands = solveCandidates(base, sms, key.sizeLog2);
          st.solveBest.assign(st.solveCands.size(), 1e30f);
          st.solveSeen.assign(st.solveCands.size(), 0);
        }
        solveCand = int(st.solveTurn++ % st.solveCands.size());
        solve = st.solveCands[solveCand];
      }
    }
    if (!radixPinned && rebuild) {
      auto it = C.radix.find(key);
      if (it != C.radix.end()) {
        radix = it->second;
      } else {
        auto& st = state(key);
        if (st.radixCands.empty()) {
          st.radixCands = radixCandidates();
          st.radixBest.assign(st.radixCands.size(), 1e30f);
          st.radixSeen.assign(st.radixCands.size(), 0);
        }
        radixCand = int(st.radixTurn++ % st.radixCands.size());
        radix = st.radixCands[radixCand];
      }
    } else if (!radixPinned) {
      auto it = C.radix.find(key);
      if (it != C.radix.end()) radix = it->second;
    }
  }

  // A timed tick: events (a, b) around the solve and (c, d) around the tree builds (null when not
  // timed), harvested once they complete.
  struct Pending {
    TuneKey key;
    int solveCand, radixCand;
    cudaEvent_t a, b, c, d;
    int itemSlot, bodies;  // the tick's work: bodies, and its items in TuneCache::items[itemSlot] (-1: none)
  };

  // The page-locked slot a timed tick copies its work-item count into (null when none is free).
  int* itemSlot(int& slot) {
    TuneCache& C = TuneCache::get();
    std::lock_guard<std::mutex> lock(C.m);
    slot = C.takeItemSlot();
    return slot >= 0 ? C.items + slot : nullptr;
  }
  // Drop pending timings (held ticks), returning their events and item slots.
  void discard(std::vector<cudaEvent_t>& freed) {
    TuneCache& C = TuneCache::get();
    std::lock_guard<std::mutex> lock(C.m);
    for (auto& pt : pending) {
      for (cudaEvent_t ev : {pt.a, pt.b, pt.c, pt.d})
        if (ev) freed.push_back(ev);
      if (pt.itemSlot >= 0) C.freeItems.push_back(pt.itemSlot);
    }
    pending.clear();
  }
  std::vector<Pending> pending;

  // Harvest completed measurements (wait = true: wait for them); returns events to recycle.
  void harvest(bool wait, std::vector<cudaEvent_t>& freed) {
    TuneCache& C = TuneCache::get();
    std::lock_guard<std::mutex> lock(C.m);
    size_t keep = 0;
    for (size_t i = 0; i < pending.size(); i++) {
      Pending& p = pending[i];
      cudaEvent_t last = p.b ? p.b : p.d;  // the solve (a, b) runs after the tree builds (c, d) in a tick
      if (!wait && cudaEventQuery(last) != cudaSuccess) {
        pending[keep++] = p;
        continue;
      }
      if (wait) cudaEventSynchronize(last);
      auto& st = state(p.key);
      float ms = 0.f;
      if (p.solveCand >= 0 && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess && size_t(p.solveCand) < st.solveBest.size()) {
        // time per unit of work (the item count was copied before event b in stream order)
        const double work = double(p.bodies) + (p.itemSlot >= 0 ? double(C.items[p.itemSlot]) : 0.0);
        const float score = work > 0.0 ? float(double(ms) * 1e6 / work) : ms;
        st.solveBest[p.solveCand] = std::min(st.solveBest[p.solveCand], score);
        st.solveSeen[p.solveCand]++;
      }
      if (p.itemSlot >= 0) C.freeItems.push_back(p.itemSlot);
      if (p.radixCand >= 0 && p.c && cudaEventElapsedTime(&ms, p.c, p.d) == cudaSuccess && size_t(p.radixCand) < st.radixBest.size()) {
        st.radixBest[p.radixCand] = std::min(st.radixBest[p.radixCand], ms);
        st.radixSeen[p.radixCand]++;
      }
      for (cudaEvent_t e : {p.a, p.b, p.c, p.d})
        if (e) freed.push_back(e);
      settle(p.key, st);
    }
    pending.resize(keep);
  }

  // True when every candidate of the class has been issued its samples but the class is not
  // settled yet: the caller waits for the timings (ticks run ahead of the host) before the next.
  bool needsHarvest(const TuneKey& key) {
    if (!enabled || pending.empty()) return false;
    TuneCache& C = TuneCache::get();
    std::lock_guard<std::mutex> lock(C.m);
    auto it = states.find(key);
    if (it == states.end()) return false;
    const State& st = it->second;
    const bool solveDue = !solvePinned && !C.solve.count(key) && !st.solveCands.empty() &&
                          st.solveTurn >= (unsigned long long)(SAMPLES * st.solveCands.size());
    const bool radixDue = !radixPinned && !C.radix.count(key) && !st.radixCands.empty() &&
                          st.radixTurn >= (unsigned long long)st.radixCands.size();
    return solveDue || radixDue;
  }

  // True once the class has its choices (nothing left to time for it).
  bool settled(const TuneKey& key, bool trees) {
    if (!enabled) return true;
    TuneCache& C = TuneCache::get();
    std::lock_guard<std::mutex> lock(C.m);
    return (solvePinned || C.solve.count(key)) && (radixPinned || !trees || C.radix.count(key));
  }

  static bool lookup(const TuneKey& key, SolveConfig& solve, int& radix, bool& haveRadix) {
    TuneCache& C = TuneCache::get();
    std::lock_guard<std::mutex> lock(C.m);
    auto it = C.solve.find(key);
    auto jt = C.radix.find(key);
    haveRadix = jt != C.radix.end();
    if (haveRadix) radix = jt->second;
    if (it == C.solve.end()) return false;
    solve = it->second;
    return true;
  }

 private:
  struct State {
    std::vector<SolveConfig> solveCands;
    std::vector<float> solveBest;
    std::vector<int> solveSeen;
    unsigned long long solveTurn = 0;
    std::vector<int> radixCands;
    std::vector<float> radixBest;
    std::vector<int> radixSeen;
    unsigned long long radixTurn = 0;
  };
  std::map<TuneKey, State> states;
  State& state(const TuneKey& k) { return states[k]; }

  void settle(const TuneKey& key, State& st) {
    TuneCache& C = TuneCache::get();
    if (!st.solveCands.empty() && !C.solve.count(key)) {
      bool all = true;
      for (int n : st.solveSeen) all &= n >= SAMPLES;
      if (all) {
        size_t best = 0;
        for (size_t i = 1; i < st.solveBest.size(); i++)
          if (st.solveBest[i] < st.solveBest[best]) best = i;
        C.solve[key] = st.solveCands[best];
      }
    }
    if (!st.radixCands.empty() && !C.radix.count(key)) {
      bool all = true;
      for (int n : st.radixSeen) all &= n >= 1;
      if (all) {
        size_t best = 0;
        for (size_t i = 1; i < st.radixBest.size(); i++)
          if (st.radixBest[i] < st.radixBest[best]) best = i;
        C.radix[key] = st.radixCands[best];
      }
    }
  }
};

}  // namespace avbd
