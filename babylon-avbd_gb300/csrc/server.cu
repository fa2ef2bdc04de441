// Serving entry points of the C ABI (avbd_server_*): continuous batching of many worlds over
// one arena (arena.hpp), with admission under a device-memory budget and LRU eviction.
//
// A world's queued steps run one per tick; every tick steps all worlds that have queued steps,
// in one launch sequence. Tickets record the step count at which an advance request is done.
// When a world must be admitted or restored and the arena cannot place it, the arena grows
// while its footprint stays within the budget; past that, idle worlds (nothing queued) are
// evicted to host memory, least recently used first. Eviction and restoring move a world's
// complete state (bodies, joints, carried colours, last contacts), so served results equal
// those of a world stepped on its own.
#include <deque>
#include <set>
#include <unordered_map>

#include "arena.hpp"

using namespace avbd;

namespace {

struct Ticket {
  long long target;  // the world's step count at which the request is done
  int64_t id;
};

struct Served {
  int slot = -1;
  int nBodies = 0;
  long long queued = 0;
  long long done = 0;
  unsigned long long lastUse = 0;
  std::deque<Ticket> tickets;
};

}  // namespace

struct avbd_server {
  avbd_ctx* ctx = nullptr;
  Arena* A = nullptr;
  int64_t budget = 0;
  size_t peak = 0;
  std::unordered_map<int64_t, Served> worlds;
  std::set<int64_t> busy;  // worlds with queued steps
  int64_t nextId = 1, nextTicket = 1;
  unsigned long long clock = 0;
  std::deque<int64_t> completed;
  long long admitted = 0, rejected = 0, ticks = 0, bodySteps = 0, completedCount = 0;
  int4* segDev = nullptr;
  size_t segCap = 0;
  float4* poseDev = nullptr;
  size_t poseCap = 0;
  // Replies captured with the ticks (tick_steps with replies): rows (2 float4 per body) of one
  // device and one pinned buffer, a row range per ticket until the reply is taken.
  float4* replyDev = nullptr;
  float4* replyHost = nullptr;
  int replyCap = 0;
  RangeAlloc replyRows;
  std::unordered_map<int64_t, std::pair<int, int>> replyOf;  // ticket -> (first row, rows)
  std::deque<int64_t> ready;                                // tickets whose reply has arrived

  // Rows for a reply: grows both buffers (waiting for every queued tick first, whose replies
  // point into the old ones) when the free ranges cannot place it.
  int replyAlloc(int rows) {
    int at = replyRows.alloc(rows);
    if (at >= 0) return at;
    A->resolve();
    const int cap = std::max(replyCap + rows + 4096, replyCap * 2);
    float4* d = dalloc<float4>(2 * size_t(cap));
    float4* h = nullptr;
    CK(cudaHostAlloc((void**)&h, 2 * size_t(cap) * sizeof(float4), cudaHostAllocDefault));
    if (replyHost) std::memcpy(h, replyHost, 2 * size_t(replyCap) * sizeof(float4));
    if (replyHost) cudaFreeHost(replyHost);
    dfree(replyDev);
    replyDev = d;
    replyHost = h;
    if (replyCap == 0) replyRows.init(cap);
    else replyRows.grow(cap);
    replyCap = cap;
    notePeak();
    return replyRows.alloc(rows);
  }

  // Bytes held against the budget: the arena's arrays, its work-item scratch (at least the
  // reserve for its body capacity) and the pose-read buffers.
  size_t accounted(long long nb, long long nj, long long slots, long long nw) const {
    return A->footprint(nb, nj, slots, nw) + std::max(A->scratchBytes(), Arena::scratchReserve(nb)) + segCap * sizeof(int4) +
           poseCap * 2 * sizeof(float4) + size_t(replyCap) * 2 * sizeof(float4);
  }
  size_t deviceBytes() const { return accounted(A->bodyCap, A->jointCap, A->slotCap, A->maxWorlds); }
  void notePeak() { peak = std::max(peak, deviceBytes()); }

  Served& get(int64_t id) {
    auto it = worlds.find(id);
    if (it == worlds.end()) throw Error(AVBD_E_INVALID, "no such world");
    return it->second;
  }

  // The least recently used resident world with nothing queued (other than `keepSlot`).
  int lruIdle(int keepSlot) const {
    int best = -1;
    unsigned long long bestUse = ~0ull;
    for (auto& kv : worlds) {
      const Served& w = kv.second;
      if (w.queued > 0 || w.slot == keepSlot || !A->W[w.slot].resident || A->W[w.slot].pinned) continue;
      if (w.lastUse < bestUse) {
        bestUse = w.lastUse;
        best = w.slot;
      }
    }
    return best;
  }

  // Room for one world of (nb, nj, slots) (newWorld: and a world-table entry): grow within the
  // budget, else evict idle worlds.
  bool makeRoom(int nb, int nj, int slots, int keepSlot, bool newWorld = true) {
    for (;;) {
      if (A->fits(nb, nj, slots) && (!newWorld || !A->freeSlots.empty())) return true;
      long long caps[4];
      bool grown = false;
      for (bool minimal : {false, true}) {
        A->plannedCaps(nb, nj, slots, caps, minimal, newWorld);
        if (accounted(caps[0], caps[1], caps[2], caps[3]) <= size_t(budget)) {
          A->growTo(caps);
          notePeak();
          grown = true;
          break;
        }
      }
      if (grown) continue;
      const int victim = lruIdle(keepSlot);
      if (victim < 0) return false;
      A->evict(victim);
    }
  }

  void ensurePoseBuffers(size_t nseg, size_t bodies) {
    if (nseg > segCap) {
      dfree(segDev);
      segDev = nullptr;
      segCap = nseg + nseg / 2 + 64;
      segDev = dalloc<int4>(segCap);
    }
    if (bodies > poseCap) {
      dfree(poseDev);
      poseDev = nullptr;
      poseCap = bodies + bodies / 2 + 1024;
      poseDev = dalloc<float4>(2 * poseCap);
    }
    notePeak();
  }
};

namespace {

void forget(avbd_ctx* ctx, Arena* A) {
  auto& v = ctx->owned;
  v.erase(std::remove(v.begin(), v.end(), (void*)A), v.end());
}

void bind(avbd_ctx* c) { CK(cudaSetDevice(c->device)); }

}  // namespace

extern "C" {

int avbd_server_create(avbd_ctx* ctx, const avbd_server_desc* desc, avbd_server** out) {
  API_BEGIN
  REQUIRE(ctx && desc && out, "null argument");
  REQUIRE(desc->budget_bytes > 0, "budget_bytes must be positive");
  REQUIRE(desc->initial_bodies >= 0 && desc->initial_worlds >= 0, "negative initial capacity");
  bind(ctx);
  const int nb = std::max(desc->initial_bodies, 1024);
  const int nw = std::max(desc->initial_worlds, 16);
  auto* S = new avbd_server();
  S->ctx = ctx;
  S->budget = desc->budget_bytes;
  try {
    S->A = new Arena(ctx, nb, std::max(nb / 16, 64), Arena::initialPairCap(nb), nw);
  } catch (...) {
    delete S;
    throw;
  }
  if (S->A->deviceBytes() > size_t(S->budget)) {
    delete S->A;
    delete S;
    throw Error(AVBD_E_CAPACITY, "the initial capacities alone exceed budget_bytes");
  }
  ctx->owned.push_back(S->A);
  // a pair region outgrowing the slot buffers mid-tick: stay within the budget by evicting idle
  // worlds (never one being stepped: those have queued steps) before the buffers grow
  S->A->onSlotPressure = [S](int slots) { S->makeRoom(0, 0, slots, -1, false); };
  S->notePeak();
  *out = S;
  API_END
}

int avbd_server_destroy(avbd_server* s) {
  API_BEGIN
  if (!s) return AVBD_OK;
  bind(s->ctx);
  forget(s->ctx, s->A);
  delete s->A;
  dfree(s->segDev);
  dfree(s->poseDev);
  dfree(s->replyDev);
  if (s->replyHost) cudaFreeHost(s->replyHost);
  delete s;
  API_END
}

int avbd_server_admit(avbd_server* s, const avbd_scene_desc* scene, const avbd_params* params, int64_t* world_id) {
  API_BEGIN
  REQUIRE(s && scene && params && world_id, "null argument");
  Arena::validate(*scene, *params);
  bind(s->ctx);
  const int nb = scene->n_bodies, nj = Arena::jointsOf(*scene);
  if (!s->makeRoom(nb, nj, Arena::initialPairCap(nb), -1)) {
    s->rejected++;
    throw Error(AVBD_E_CAPACITY, "world of " + std::to_string(nb) + " bodies does not fit in the device budget (" +
                                     std::to_string(s->budget) + " bytes) with every idle world evicted");
  }
  const int slot = s->A->addWorld(*scene, *params);
  const int64_t id = s->nextId++;
  Served w;
  w.slot = slot;
  w.nBodies = nb;
  w.lastUse = ++s->clock;
  s->worlds.emplace(id, std::move(w));
  s->admitted++;
  s->notePeak();
  *world_id = id;
  API_END
}

int avbd_server_advance(avbd_server* s, int64_t world_id, int32_t steps, int64_t* ticket) {
  API_BEGIN
  REQUIRE(s && ticket, "null argument");
  REQUIRE(steps >= 0, "steps must be non-negative");
  Served& w = s->get(world_id);
  const int64_t t = s->nextTicket++;
  w.queued += steps;
  w.lastUse = ++s->clock;
  if (steps == 0 && w.tickets.empty()) {
    s->completed.push_back(t);  // nothing to wait for
    s->completedCount++;
  } else {
    w.tickets.push_back(Ticket{w.done + w.queued, t});
  }
  if (w.queued > 0) s->busy.insert(world_id);
  *ticket = t;
  API_END
}

int avbd_server_tick_steps(avbd_server* s, int32_t max_steps, int32_t replies, int32_t* n_stepped) {
  API_BEGIN
  REQUIRE(s, "null server");
  REQUIRE(max_steps >= 1, "max_steps must be positive");
  bind(s->ctx);
  Arena& A = *s->A;
  s->clock++;
  // restore evicted worlds that have work, least recently used first, while room allows
  std::vector<std::pair<unsigned long long, int64_t>> waiting;
  for (int64_t id : s->busy) {
    const Served& w = s->worlds.at(id);
    if (!A.W[w.slot].resident) waiting.push_back({w.lastUse, id});
  }
  std::sort(waiting.begin(), waiting.end());
  for (auto& e : waiting) {
    Served& w = s->worlds.at(e.second);
    const WorldRec& R = A.W[w.slot];
    if (!s->makeRoom(R.nBodies, R.nJoints, A.restoreSlots(w.slot), w.slot, false)) break;
    A.restore(w.slot);
  }
  int32_t stepped = 0;
  for (int step = 0; step < max_steps; step++) {
    std::vector<int> act;
    std::vector<int64_t> ids;
    for (int64_t id : s->busy) {
      const Served& w = s->worlds.at(id);
      if (A.W[w.slot].resident) {
        act.push_back(w.slot);
        ids.push_back(id);
      }
    }
    if (act.empty()) break;
    // the tickets this step completes, and (with replies) their worlds' poses after it
    Arena::TickReply reply;
    std::vector<std::pair<int64_t, int64_t>> finishing;  // (world id, ticket)
    for (int64_t id : ids) {
      const Served& w = s->worlds.at(id);
      for (const Ticket& t : w.tickets) {
        if (t.target > w.done + 1) break;
        finishing.push_back({id, t.id});
      }
    }
    if (replies && !finishing.empty()) {
      int rows = 0;
      for (auto& f : finishing) rows += s->worlds.at(f.first).nBodies;
      const int at = s->replyAlloc(rows);
      reply.rows = rows;
      reply.dev = s->replyDev + 2 * size_t(at);
      reply.host = s->replyHost + 2 * size_t(at);
      int row = 0;
      for (auto& f : finishing) {
        const Served& w = s->worlds.at(f.first);
        reply.seg.push_back(make_int4(A.W[w.slot].dev.bodyOff, w.nBodies, row, 0));
        reply.tags.push_back(f.second);
        s->replyOf[f.second] = {at + row, w.nBodies};
        row += w.nBodies;
      }
    }
    A.stepWorlds(act, reply.rows > 0 ? &reply : nullptr);
    for (int64_t id : ids) {
      Served& w = s->worlds.at(id);
      w.queued--;
      w.done++;
      w.lastUse = s->clock;
      s->bodySteps += w.nBodies;
      while (!w.tickets.empty() && w.tickets.front().target <= w.done) {
        if (!replies) {  // with replies a ticket completes once its tick is confirmed (avbd_server_ready)
          s->completed.push_back(w.tickets.front().id);
          s->completedCount++;
        }
        w.tickets.pop_front();
      }
      if (w.queued == 0) s->busy.erase(id);
    }
    stepped += int32_t(act.size());
    s->ticks++;
  }
  s->notePeak();
  if (n_stepped) *n_stepped = stepped;
  API_END
}

int avbd_server_tick(avbd_server* s, int32_t* n_stepped) { return avbd_server_tick_steps(s, 1, 0, n_stepped); }

int avbd_server_ready(avbd_server* s, int64_t* tickets, int32_t cap, int32_t wait, int32_t* n) {
  API_BEGIN
  REQUIRE(s && n && (cap == 0 || tickets), "null argument");
  REQUIRE(cap >= 0, "negative capacity");
  bind(s->ctx);
  Arena& A = *s->A;
  if (wait) A.resolve();
  else A.trimLog();
  for (long long t : A.confirmedTags) {
    s->ready.push_back(t);
    s->completedCount++;
  }
  A.confirmedTags.clear();
  int k = 0;
  while (k < cap && !s->ready.empty()) {
    tickets[k++] = s->ready.front();
    s->ready.pop_front();
  }
  *n = k;
  API_END
}

int avbd_server_take_reply(avbd_server* s, int64_t ticket, float* out, int64_t cap_bodies, int32_t* n_bodies) {
  API_BEGIN
  REQUIRE(s && n_bodies, "null argument");
  auto it = s->replyOf.find(ticket);
  REQUIRE(it != s->replyOf.end(), "no reply for this ticket (not captured, or already taken)");
  const int first = it->second.first, rows = it->second.second;
  *n_bodies = rows;
  if (!out || cap_bodies < rows) return AVBD_OK;  // size query
  std::memcpy(out, s->replyHost + 2 * size_t(first), size_t(rows) * 2 * sizeof(float4));
  s->replyRows.release(first, rows);
  s->replyOf.erase(it);
  API_END
}

int avbd_server_completed(avbd_server* s, int64_t* tickets, int32_t cap, int32_t* n) {
  API_BEGIN
  REQUIRE(s && n && (cap == 0 || tickets), "null argument");
  REQUIRE(cap >= 0, "negative capacity");
  int k = 0;
  while (k < cap && !s->completed.empty()) {
    tickets[k++] = s->completed.front();
    s->completed.pop_front();
  }
  *n = k;
  API_END
}

int avbd_server_read_poses(avbd_server* s, const int64_t* world_ids, int32_t n, float* out) {
  API_BEGIN
  REQUIRE(s && (n == 0 || (world_ids && out)), "null argument");
  REQUIRE(n >= 0, "negative count");
  bind(s->ctx);
  Arena& A = *s->A;
  std::vector<int4> seg;
  std::vector<std::pair<int, size_t>> hostRows;  // (slot, first output body) of evicted worlds
  size_t total = 0;
  for (int k = 0; k < n; k++) {
    const Served& w = s->get(world_ids[k]);
    const WorldRec& R = A.W[w.slot];
    if (total + size_t(R.nBodies) > size_t(0x7fffffff)) throw Error(AVBD_E_CAPACITY, "too many bodies in one read");
    if (R.resident) {
      A.flushEdits(w.slot);  // queued commands apply before a read
      seg.push_back(make_int4(R.dev.bodyOff, R.nBodies, int(total), 0));
    }
    else {
      seg.push_back(make_int4(0, 0, int(total), 0));
      hostRows.push_back({w.slot, total});
    }
    total += size_t(R.nBodies);
  }
  A.resolve();
  if (total == 0) return AVBD_OK;
  s->ensurePoseBuffers(seg.size(), total);
  A.put(s->segDev, seg.data(), seg.size() * sizeof(int4));
  int blocks = grid_blocks((long long)total, 256);
  if (blocks > device_sms() * 8) blocks = device_sms() * 8;
  launch_gather_poses(A.B, s->segDev, int(seg.size()), int(total), s->poseDev, nullptr, A.s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, s->poseDev, total * 2 * sizeof(float4), cudaMemcpyDeviceToHost, A.s));
  A.flush();
  for (auto& h : hostRows) {
    const WorldRec& R = A.W[h.first];
    const Snapshot& S = *R.snap;
    for (int i = 0; i < R.nBodies; i++) {
      float* o = out + (h.second + size_t(i)) * 8;
      const float4 p = S.pose[2 * size_t(i)], q = S.pose[2 * size_t(i) + 1], sz = S.size[i];
      o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = sz.w;
      o[4] = q.x; o[5] = q.y; o[6] = q.z; o[7] = q.w;
    }
  }
  API_END
}

int avbd_server_read_state(avbd_server* s, int64_t world_id, float* position, float* rotation, float* velocity, float* angular,
                           float* prev_velocity) {
  API_BEGIN
  REQUIRE(s, "null server");
  bind(s->ctx);
  const Served& w = s->get(world_id);
  const WorldRec& R = s->A->W[w.slot];
  if (R.resident) {
    s->A->readState(w.slot, position, rotation, velocity, angular, prev_velocity);
    return AVBD_OK;
  }
  const Snapshot& S = *R.snap;
  auto put3 = [&](float* o, const std::vector<float4>& v) {
    if (!o) return;
    for (int i = 0; i < R.nBodies; i++) { o[3 * i] = v[i].x; o[3 * i + 1] = v[i].y; o[3 * i + 2] = v[i].z; }
  };
  put3(velocity, S.vel);
  put3(angular, S.ang);
  put3(prev_velocity, S.vprev);
  if (position)
    for (int i = 0; i < R.nBodies; i++) {
      const float4 p = S.pose[2 * size_t(i)];
      position[3 * i] = p.x; position[3 * i + 1] = p.y; position[3 * i + 2] = p.z;
    }
  if (rotation)
    for (int i = 0; i < R.nBodies; i++) {
      const float4 q = S.pose[2 * size_t(i) + 1];
      rotation[4 * i] = q.x; rotation[4 * i + 1] = q.y; rotation[4 * i + 2] = q.z; rotation[4 * i + 3] = q.w;
    }
  API_END
}

int avbd_server_world_info(avbd_server* s, int64_t world_id, int32_t* n_bodies, int64_t* queued, int64_t* steps_done,
                           int32_t* resident) {
  API_BEGIN
  REQUIRE(s, "null server");
  const Served& w = s->get(world_id);
  if (n_bodies) *n_bodies = w.nBodies;
  if (queued) *queued = w.queued;
  if (steps_done) *steps_done = w.done;
  if (resident) *resident = s->A->W[w.slot].resident ? 1 : 0;
  API_END
}

int avbd_server_edit(avbd_server* s, int64_t world_id, const uint32_t* records, int32_t n) {
  API_BEGIN
  REQUIRE(s && (n == 0 || records), "null argument");
  bind(s->ctx);
  const Served& w = s->get(world_id);
  s->A->queueEdits(w.slot, records, n);
  API_END
}

int avbd_server_watch_contacts(avbd_server* s, int64_t world_id, const uint32_t* indices, int32_t n, int32_t max_pairs,
                               int32_t max_events) {
  API_BEGIN
  REQUIRE(s, "null server");
  REQUIRE(max_pairs >= 1 && max_events >= 1, "Contact capacities must be positive integers");
  REQUIRE(!indices || n >= 0, "negative count");
  bind(s->ctx);
  const Served& w = s->get(world_id);
  s->A->watchContacts(w.slot, indices, n, max_events, indices != nullptr);
  API_END
}

int avbd_server_contact_events(avbd_server* s, int64_t world_id, uint32_t* out, int64_t cap, int64_t* n, int64_t* dropped,
                               int32_t* full) {
  API_BEGIN
  REQUIRE(s && n, "null argument");
  bind(s->ctx);
  const Served& w = s->get(world_id);
  long long d = 0;
  *n = s->A->readEvents(w.slot, out, cap, &d);
  if (dropped) *dropped = d;
  if (full) *full = d > 0;
  API_END
}

int avbd_server_cast(avbd_server* s, int64_t world_id, const float* queries, int32_t n, const avbd_cast_filter* filter,
                     float* hits) {
  API_BEGIN
  REQUIRE(s && (n == 0 || (queries && hits)), "null argument");
  bind(s->ctx);
  const Served& w = s->get(world_id);
  REQUIRE(s->A->W[w.slot].resident, "world is evicted: advance it before casting");
  avbd_cast_filter all{0xffffffffu, 0u, 0, 1, 0, {0}};
  s->A->cast(w.slot, queries, n, filter ? *filter : all, hits);
  API_END
}

int avbd_server_sleep_state(avbd_server* s, int64_t world_id, int32_t* asleep, float* quiet_time, int32_t* n_sleeping) {
  API_BEGIN
  REQUIRE(s, "null server");
  bind(s->ctx);
  const Served& w = s->get(world_id);
  const int c = s->A->sleepState(w.slot, asleep, quiet_time);
  if (n_sleeping) *n_sleeping = c;
  API_END
}

int avbd_server_evict(avbd_server* s, int64_t world_id) {
  API_BEGIN
  REQUIRE(s, "null server");
  bind(s->ctx);
  const Served& w = s->get(world_id);
  if (!s->A->W[w.slot].resident) return AVBD_OK;
  s->A->evict(w.slot);
  API_END
}

int avbd_server_release(avbd_server* s, int64_t world_id) {
  API_BEGIN
  REQUIRE(s, "null server");
  bind(s->ctx);
  const Served& w = s->get(world_id);
  s->A->removeWorld(w.slot);
  s->busy.erase(world_id);
  s->worlds.erase(world_id);
  API_END
}

int avbd_server_read_stats(avbd_server* s, avbd_server_stats* out) {
  API_BEGIN
  REQUIRE(s && out, "null argument");
  std::memset(out, 0, sizeof(*out));
  out->budget_bytes = s->budget;
  out->device_bytes = int64_t(s->deviceBytes());
  out->peak_device_bytes = int64_t(s->peak);
  out->live_worlds = int64_t(s->worlds.size());
  for (auto& kv : s->worlds) {
    const WorldRec& R = s->A->W[kv.second.slot];
    if (R.resident) {
      out->resident_worlds++;
      out->resident_bodies += R.nBodies;
    } else {
      out->evicted_worlds++;
    }
  }
  out->pending_worlds = int64_t(s->busy.size());
  out->admitted = s->admitted;
  out->rejected = s->rejected;
  out->evictions = s->A->evictions;
  out->restores = s->A->restores;
  out->ticks = s->ticks;
  out->body_steps = s->bodySteps;
  out->completed = s->completedCount;
  API_END
}

}  // extern "C"
