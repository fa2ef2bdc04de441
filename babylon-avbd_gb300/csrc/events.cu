// Contact begin/end events after the step (src/vendor/three-avbd-lib/contacts.ts ContactWatch),
// for the worlds of the tick with FLAG_EVENTS.
//
// A pair is touching in a step when its manifold has contacts and one of its bodies is watched.
// It begins when it touches now but did not in the world's previous step, and ends when it
// touched then but does not now; a body whose watch word changed since the previous step (newly
// watched, or its history reset) begins its current contacts afresh and ends none of the old.
// The reference keeps two hash sets of touching pairs; here both steps' pairs are already sorted
// by (hi, lo) in the world's two pair regions, so "touched in the other step" is a binary search
// of the other region, and no set (and no set capacity) is needed.
//
// A begin carries where (the mean of the contact points, anchor rA turned by A's rotation plus
// A's position, summed then divided), how hard (|sum of the contacts' normal lambda| x dt) and
// the manifold normal (from B to A); an end carries zeros. Events go to the world's region by an
// atomic counter (written past the capacity: dropped). Bodies are world-local, a > b.
//   k_events_begin  per active pair slot: begins
//   k_events_end    per active world (one block), over its previous region: ends
//   k_events_commit watch words become the previous ones; the worlds' step counters advance
#include "engine.cuh"

namespace avbd {
namespace {

__device__ __forceinline__ void emit(const EventBufs& ev, int w, uint32_t kind, int a, int b, int step, V3 point,
                                     float impulse, V3 n, bool trigger) {
  const int e = atomicAdd(&ev.count[w], 1);
  if (e >= ev.cap[w]) return;
  float4* r = ev.region[w] + size_t(EVENT_FLOAT4) * e;
  r[0] = make_float4(__uint_as_float(kind), __uint_as_float(uint32_t(a)), __uint_as_float(uint32_t(b)),
                     __uint_as_float(uint32_t(step)));
  r[1] = f4(point, impulse);
  r[2] = f4(n, trigger ? 1.f : 0.f);  // isTrigger
}

__global__ void k_events_begin(BodyPtrs bd, const WorldDev* __restrict__ worlds, PairPtrs P, Tick t,
                               const Counters* __restrict__ ctr, EventBufs ev) {
  if (tick_held(t.ctl)) return;
  const int np = ctr->activePairs;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
    const int p = t.pairs[q];
    const int nc = P.count[p];
    if (nc == 0) continue;
    const uint2 pr = P.pair[p];
    const int a = int(pr.x), b = int(pr.y);
    const int w = bd.meta[b].x;
    const WorldDev& W = worlds[w];
    if (!(W.flags & FLAG_EVENTS)) continue;
    const uint32_t wa = bd.watch[a], wb = bd.watch[b];
    if (!((wa | wb) & WATCH_ON)) continue;
    if (wa == bd.watchPrev[a] && wb == bd.watchPrev[b]) {
      const int pw = t.which[w];
      const int nprev = t.pairN[pw * t.maxWorlds + w];
      const int pp = nprev > 0 ? find_pair(P.pair, pw * t.slotStride + W.pairOff, nprev, pr) : -1;
      if (pp >= 0 && P.count[pp] > 0) continue;  // touching in the previous step too
    }
    const float4 pA = bd.pos(a), qA = bd.rot(a);
    V3 point{0.f, 0.f, 0.f};
    float force = 0.f;
    for (int c = 0; c < nc; c++) {
      const float4* c4 = P.ct + (size_t(p) * MAX_CONTACTS + c) * 4;
      point = point + (rotate(qA, v3(c4[0])) + v3(pA));
      force += c4[3].x;
    }
    // a trigger pair reports no impulse (src/native/cpu/world.js:757-762)
    const bool trig = ((bd.sleep[a] | bd.sleep[b]) & BODY_TRIGGER) != 0;
    emit(ev, w, EVENT_BEGIN, a - W.bodyOff, b - W.bodyOff, ev.step[w] + 1, vdiv(point, float(nc)),
         trig ? 0.f : fabsf(force) * W.dt, v3(P.basis[3 * p]), trig);
  }
}

__global__ void k_events_end(BodyPtrs bd, const WorldDev* __restrict__ worlds, PairPtrs P, Tick t, EventBufs ev) {
  if (tick_held(t.ctl)) return;
  for (int a0 = blockIdx.x; a0 < t.nActive; a0 += gridDim.x) {
    const int w = t.active[a0].x;
    const WorldDev& W = worlds[w];
    if (!(W.flags & FLAG_EVENTS)) continue;
    const int pw = t.which[w], cw = 1 - pw;
    const int nprev = t.pairN[pw * t.maxWorlds + w], ncur = t.pairN[cw * t.maxWorlds + w];
    const int prevBase = pw * t.slotStride + W.pairOff, curBase = cw * t.slotStride + W.pairOff;
    for (int k = threadIdx.x; k < nprev; k += blockDim.x) {
      const int pp = prevBase + k;
      if (P.count[pp] == 0) continue;
      const uint2 pr = P.pair[pp];
      const int a = int(pr.x), b = int(pr.y);
      const uint32_t pa = bd.watchPrev[a], pb = bd.watchPrev[b];
      if (!((pa | pb) & WATCH_ON)) continue;               // not touching-and-watched then
      if (bd.watch[a] != pa || bd.watch[b] != pb) continue;  // history restarted
      const int cp = ncur > 0 ? find_pair(P.pair, curBase, ncur, pr) : -1;
      if (cp >= 0 && P.count[cp] > 0) continue;  // still touching
      emit(ev, w, EVENT_END, a - W.bodyOff, b - W.bodyOff, ev.step[w] + 1, V3{0.f, 0.f, 0.f}, 0.f, V3{0.f, 0.f, 0.f},
             ((bd.sleep[a] | bd.sleep[b]) & BODY_TRIGGER) != 0);
    }
  }
}

__global__ void k_events_commit(BodyPtrs bd, const WorldDev* __restrict__ worlds, Tick t, EventBufs ev) {
  if (tick_held(t.ctl)) return;
  const int stride = gridDim.x * blockDim.x;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < t.nBodies; k += stride) {
    const int i = t.bodies[k];
    if (worlds[bd.meta[i].x].flags & FLAG_EVENTS) bd.watchPrev[i] = bd.watch[i];
  }
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < t.nActive; a += stride) {
    const int w = t.active[a].x;
    if (worlds[w].flags & FLAG_EVENTS) ev.step[w] += 1;
  }
}

}  // namespace

void launch_events(const BodyPtrs& b, const WorldDev* worlds, PairPtrs P, Tick t, const Counters* ctr, int pairBudget,
                   EventBufs ev, cudaStream_t s) {
  if (t.nActive == 0) return;
  int pb = grid_blocks(pairBudget > 0 ? pairBudget : 1, 256);
  const int cap = device_sms() * 8;
  if (pb > cap) pb = cap;
  int wb = t.nActive < cap ? t.nActive : cap;
  const int total = t.nBodies > t.nActive ? t.nBodies : t.nActive;
  k_events_begin<<<pb, 256, 0, s>>>(b, worlds, P, t, ctr, ev);
  k_events_end<<<wb, 256, 0, s>>>(b, worlds, P, t, ev);
  k_events_commit<<<grid_blocks(total, 256), 256, 0, s>>>(b, worlds, t, ev);
  note_launches(3);
}

}  // namespace avbd
