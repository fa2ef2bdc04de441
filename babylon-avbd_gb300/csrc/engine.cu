// World and batch entry points of the C ABI (include/avbd_gb300.h) over the arena (arena.hpp).
#include "arena.hpp"

using namespace avbd;

namespace avbd {

namespace {
thread_local std::string g_error;
}

void set_error(const std::string& message) { g_error = message; }

}  // namespace avbd

struct avbd_world {
  Arena* A;
  int w;
};
struct avbd_batch {
  Arena* A;
  std::vector<int> worlds;
  int64_t bodies;
  std::vector<std::pair<long long, int>> starts;  // (first body, world slot), ascending
  long long nextTag = 1;                          // tags of avbd_batch_step_read, in queue order
  long long doneUpTo = 0;                         // every tag up to this one is confirmed
};

// ---------------------------------------------------------------- device helpers for the ABI

namespace avbd {

// 40-float body records of src/native/cpu/world.js:503-561 (or 8-float poses)
__global__ void k_read_selected(BodyPtrs bd, const WorldDev* __restrict__ worlds, const uint32_t* __restrict__ idx, int n, int off,
                                int posesOnly, float* __restrict__ out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int i = off + int(idx[k]);
    const float4 p = bd.pos(i), q = bd.rot(i), sz = bd.size[i];
    if (posesOnly) {
      float* o = out + size_t(k) * 8;
      o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = sz.w;
      o[4] = q.x; o[5] = q.y; o[6] = q.z; o[7] = q.w;
      continue;
    }
    float* o = out + size_t(k) * 40;
    const float4 p0 = bd.pos0(i), q0 = bd.rot0(i), m = bd.mass[i], py = bd.posY(i), qy = bd.rotY(i);
    const float4 v = bd.vel[i], w = bd.ang[i], vp = bd.vprev[i];
    const int4 meta = bd.meta[i];
    const WorldDev& W = worlds[meta.x];
    o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = sz.w;
    o[4] = q.x; o[5] = q.y; o[6] = q.z; o[7] = q.w;
    o[8] = p0.x; o[9] = p0.y; o[10] = p0.z; o[11] = (bd.sleep[i] & BODY_TRIGGER) ? 1.f : 0.f;  // isTrigger
    o[12] = q0.x; o[13] = q0.y; o[14] = q0.z; o[15] = q0.w;
    o[16] = sz.x; o[17] = sz.y; o[18] = sz.z; o[19] = (bd.sleep[i] & SLEEP_ASLEEP) ? 0.f : m.x;  // effective mass
    o[20] = m.y; o[21] = m.z; o[22] = m.w; o[23] = p.w;
    o[24] = py.x; o[25] = py.y; o[26] = py.z; o[27] = 0.f;
    o[28] = qy.x; o[29] = qy.y; o[30] = qy.z; o[31] = qy.w;
    o[32] = v.x; o[33] = v.y; o[34] = v.z; o[35] = (vp.x * W.up0 + vp.y * W.up1) + vp.z * W.up2;
    // shape code of world.js:543-551: box 0, sphere 1, capsule -1
    o[36] = w.x; o[37] = w.y; o[38] = w.z; o[39] = meta.y == SHAPE_CAPSULE ? -1.f : float(meta.y);
  }
}

__global__ void k_set_poses(BodyPtrs bd, const uint32_t* __restrict__ idx, int n, int off, const float* __restrict__ pos,
                            const float* __restrict__ rot) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int i = off + int(idx[k]);
    const float r = bd.pos(i).w;
    bd.pos(i) = make_float4(pos[3 * k], pos[3 * k + 1], pos[3 * k + 2], r);
    if (rot) bd.rot(i) = qnormalize(make_float4(rot[4 * k], rot[4 * k + 1], rot[4 * k + 2], rot[4 * k + 3]));
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

__global__ void k_read_poses(const float4* __restrict__ pose, const float4* __restrict__ size, int n, float4* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pose[2 * size_t(i)];
    out[2 * size_t(i)] = make_float4(p.x, p.y, p.z, size[i].w);
    out[2 * size_t(i) + 1] = pose[2 * size_t(i) + 1];
  }
}

}  // namespace avbd

// ---------------------------------------------------------------- C ABI

namespace {

void bind(avbd_ctx* c) { CK(cudaSetDevice(c->device)); }


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
  A.flushEdits(w);  // queued commands apply before a read (src/native/solver3D.js:223-227,245,249)
  if (n == 0) return;
  const int stride = posesOnly ? 8 : 40;
  const size_t ib = Arena::align256(size_t(n) * 4);
  char* io = A.ioBuffer(ib + size_t(n) * stride * 4);
  uint32_t* di = reinterpret_cast<uint32_t*>(io);
  float* dout = reinterpret_cast<float*>(io + ib);
  A.put(di, indices, size_t(n) * 4);
  k_read_selected<<<grid_blocks(n, 128), 128, 0, A.s>>>(A.B, A.worlds, di, n, R.dev.bodyOff, posesOnly, dout); note_launches(1);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout, size_t(n) * stride * 4, cudaMemcpyDeviceToHost, A.s));
  A.flush();
}

// setVelocities / setLinearVelocities / setAngularVelocities (src/native/runtime.js:354-380):
// like the reference's velocity batches, the writes are queued in stream order with the steps:
// body commands of kind 0 (linear) and 1 (angular) for the world's next step or read. `indices`
// are global to the worlds listed in `starts` (first body index of each, ascending).
void setVelocities(Arena& A, const std::vector<std::pair<long long, int>>& starts, long long limit, const uint32_t* indices, int n,
                   const float* velocity, const float* angular) {
  REQUIRE(n == 0 || indices, "null argument");
  REQUIRE(n >= 0, "negative count");
  for (int k = 0; k < n; k++) REQUIRE((long long)indices[k] < limit, "body index out of range");
  for (int k = 0; velocity && k < 3 * n; k++) REQUIRE(std::isfinite(velocity[k]), "velocities must be finite");
  for (int k = 0; angular && k < 3 * n; k++) REQUIRE(std::isfinite(angular[k]), "velocities must be finite");
  if (n == 0 || (!velocity && !angular)) return;
  // (start index, k) in index order: each world's records stay in call order (stable sort)
  std::vector<std::pair<int, int>> order(n);
  for (int k = 0; k < n; k++) {
    const auto it = std::upper_bound(starts.begin(), starts.end(), std::make_pair((long long)indices[k], INT32_MAX)) - 1;
    order[k] = {int(it - starts.begin()), k};
  }
  std::stable_sort(order.begin(), order.end(), [](const std::pair<int, int>& x, const std::pair<int, int>& y) { return x.first < y.first; });
  std::vector<uint32_t> r;
  for (size_t a = 0; a < order.size();) {
    const int si = order[a].first;
    r.clear();
    for (; a < order.size() && order[a].first == si; a++) {
      const int k = order[a].second;
      const uint32_t local = uint32_t((long long)indices[k] - starts[size_t(si)].first);
      for (int kind = 0; kind < 2; kind++) {
        const float* v = kind == 0 ? velocity : angular;
        if (!v) continue;
        uint32_t rec[12] = {local, uint32_t(kind), 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        std::memcpy(rec + 4, v + 3 * size_t(k), 12);
        r.insert(r.end(), rec, rec + 12);
      }
    }
    A.queueEdits(starts[size_t(si)].second, r.data(), int(r.size() / 12));
  }
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
  for (void* p : ctx->owned) static_cast<Arena*>(p)->resolve();  // queued steps final (held ones re-run)
  CK(cudaStreamSynchronize(ctx->stream));
  API_END
}

struct avbd_fence {
  int device = 0;
  cudaEvent_t ev = nullptr;
};

int avbd_ctx_fence(avbd_ctx* ctx, avbd_fence** out) {
  API_BEGIN
  REQUIRE(ctx && out, "null argument");
  bind(ctx);
  auto* f = new avbd_fence;
  f->device = ctx->device;
  if (cudaEventCreateWithFlags(&f->ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventRecord(f->ev, ctx->stream) != cudaSuccess) {
    if (f->ev) cudaEventDestroy(f->ev);
    delete f;
    throw avbd::Error(AVBD_E_CUDA, "cannot record a fence");
  }
  *out = f;
  API_END
}

int avbd_fence_wait(avbd_fence* f) {
  API_BEGIN
  REQUIRE(f, "null fence");
  CK(cudaSetDevice(f->device));
  CK(cudaEventSynchronize(f->ev));
  API_END
}

int avbd_fence_query(avbd_fence* f, int32_t* done) {
  API_BEGIN
  REQUIRE(f && done, "null argument");
  CK(cudaSetDevice(f->device));
  const cudaError_t e = cudaEventQuery(f->ev);
  if (e != cudaSuccess && e != cudaErrorNotReady) CK(e);
  *done = e == cudaSuccess;
  API_END
}

int avbd_fence_destroy(avbd_fence* f) {
  API_BEGIN
  if (!f) return AVBD_OK;
  CK(cudaSetDevice(f->device));
  cudaEventDestroy(f->ev);
  delete f;
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

// Device address of g_select_scratch on `device` (which must be current). In host code the
// symbol itself is only a host-side stand-in for the device array. The address is looked up on
// every call (a cheap query that allocates nothing), so a primary context that was reset in
// between (cudaDeviceReset) never leaves a stale address behind.
float* select_scratch(int device) {
  if (device < 0) throw Error(AVBD_E_INVALID, "device index out of range");
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_select_scratch);
  if (e != cudaSuccess) throw Error(AVBD_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  return static_cast<float*>(p);
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
  // A read sees the queued body commands applied (src/native/solver3D.js:223-227). Applying them
  // can grow the command buffers, which allocates, so this entry point refuses instead.
  if (!R.edits.empty() || R.wakePending)
    throw Error(AVBD_E_STATE, "avbd_world_read_selected_noalloc: the world has queued body commands; apply them first "
                              "(avbd_world_flush_edits or a step)");
  // Steps still queued must be final; one that overflowed needs buffer growth (an allocation), so
  // this entry point refuses then too.
  if (!A.settle())
    throw Error(AVBD_E_STATE, "avbd_world_read_selected_noalloc: a queued step needs more buffer room; make it final first "
                              "(any other read, or avbd_ctx_synchronize)");
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
  const size_t ib = Arena::align256(size_t(n) * 4), pb = Arena::align256(size_t(n) * 12);
  char* io = A.ioBuffer(ib + pb + size_t(n) * 16);
  uint32_t* di = reinterpret_cast<uint32_t*>(io);
  float* dp = reinterpret_cast<float*>(io + ib);
  float* dr = rotation ? reinterpret_cast<float*>(io + ib + pb) : nullptr;
  A.put(di, indices, size_t(n) * 4);
  A.put(dp, position, size_t(n) * 12);
  if (dr) A.put(dr, rotation, size_t(n) * 16);
  k_set_poses<<<grid_blocks(n, 128), 128, 0, A.s>>>(A.B, di, n, R.dev.bodyOff, dp, dr); note_launches(1);
  CK(cudaGetLastError());
  A.wakeWorld(w->w);  // setPoses wakes the world (src/native/cpu/world.js:165-170)
  API_END
}

int avbd_world_set_velocities(avbd_world* w, const uint32_t* indices, int32_t n, const float* velocity, const float* angular) {
  API_BEGIN
  REQUIRE(w, "null argument");
  Arena& A = *w->A;
  bind(A.ctx);
  const WorldRec& R = A.resident(w->w);
  setVelocities(A, {{0LL, w->w}}, R.nBodies, indices, n, velocity, angular);
  API_END
}

int avbd_world_counters(avbd_world* w, avbd_counters* out) {
  API_BEGIN
  REQUIRE(w && out, "null argument");
  bind(w->A->ctx);
  w->A->counters(out);
  API_END
}

int avbd_world_edit(avbd_world* w, const uint32_t* records, int32_t n) {
  API_BEGIN
  REQUIRE(w && (n == 0 || records), "null argument");
  bind(w->A->ctx);
  w->A->queueEdits(w->w, records, n);
  API_END
}

int avbd_world_set_sleeping(avbd_world* w, int32_t enabled, float speed_threshold, float time_threshold) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->setSleeping(w->w, enabled != 0, speed_threshold, time_threshold);
  API_END
}

int avbd_world_set_sleep_enabled(avbd_world* w, int32_t body, int32_t enabled) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->setSleepAllowed(w->w, body, enabled != 0);
  API_END
}

int avbd_world_wake_all(avbd_world* w) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->wakeWorld(w->w);
  API_END
}

int avbd_world_sleep_state(avbd_world* w, int32_t* asleep, float* quiet_time, int32_t* n_sleeping) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  const int c = w->A->sleepState(w->w, asleep, quiet_time);
  if (n_sleeping) *n_sleeping = c;
  API_END
}

int avbd_world_watch_contacts(avbd_world* w, const uint32_t* indices, int32_t n, int32_t max_pairs, int32_t max_events) {
  API_BEGIN
  REQUIRE(w, "null world");
  REQUIRE(max_pairs >= 1 && max_events >= 1, "Contact capacities must be positive integers");
  REQUIRE(!indices || n >= 0, "negative count");
  bind(w->A->ctx);
  w->A->watchContacts(w->w, indices, n, max_events, indices != nullptr);
  API_END
}

int avbd_world_reset_contact_history(avbd_world* w, const uint32_t* indices, int32_t n) {
  API_BEGIN
  REQUIRE(w && (n == 0 || indices), "null argument");
  REQUIRE(n >= 0, "negative count");
  bind(w->A->ctx);
  w->A->resetContactHistory(w->w, indices, n);
  API_END
}

int avbd_world_contact_events(avbd_world* w, uint32_t* out, int64_t cap, int64_t* n, int64_t* dropped, int32_t* full) {
  API_BEGIN
  REQUIRE(w && n, "null argument");
  bind(w->A->ctx);
  long long d = 0;
  *n = w->A->readEvents(w->w, out, cap, &d);
  if (dropped) *dropped = d;
  if (full) *full = d > 0;
  API_END
}

int avbd_world_read_joints(avbd_world* w, float* out) {
  API_BEGIN
  REQUIRE(w && out, "null argument");
  bind(w->A->ctx);
  w->A->readJoints(w->w, out);
  API_END
}

int avbd_world_set_filters(avbd_world* w, const uint32_t* indices, int32_t n, const uint32_t* groups,
                           const uint32_t* collides_with) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (indices && groups && collides_with)), "null argument");
  bind(w->A->ctx);
  w->A->setFilters(w->w, indices, n, groups, collides_with);
  API_END
}

int avbd_world_set_restitution(avbd_world* w, const uint32_t* indices, int32_t n, const float* values) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (indices && values)), "null argument");
  bind(w->A->ctx);
  w->A->setRestitution(w->w, indices, n, values);
  API_END
}

int avbd_world_set_sensor(avbd_world* w, const uint32_t* indices, int32_t n, int32_t enabled) {
  API_BEGIN
  REQUIRE(w && (n == 0 || indices), "null argument");
  bind(w->A->ctx);
  w->A->setSensor(w->w, indices, n, enabled != 0);
  API_END
}

int avbd_world_set_motor(avbd_world* w, int32_t slot, int32_t mask, float speed, float max_torque) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->setMotor(w->w, slot, mask, speed, max_torque);
  API_END
}

int avbd_world_release_joints(avbd_world* w, const int32_t* slots, int32_t n) {
  API_BEGIN
  REQUIRE(w && (n == 0 || slots), "null argument");
  bind(w->A->ctx);
  w->A->releaseJoints(w->w, slots, n);
  API_END
}

int avbd_world_set_spring_material(avbd_world* w, int32_t slot, int32_t mask, float break_strain, float break_force) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->setSpringMaterial(w->w, slot, mask, break_strain, break_force);
  API_END
}

int avbd_world_set_world_anchor(avbd_world* w, int32_t slot, const float* point) {
  API_BEGIN
  REQUIRE(w && point, "null argument");
  bind(w->A->ctx);
  w->A->setWorldAnchor(w->w, slot, point);
  API_END
}

int avbd_world_capture_frames(avbd_world* w, const int32_t* slots, const int32_t* spring, int32_t n) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (slots && spring)), "null argument");
  bind(w->A->ctx);
  w->A->captureFrames(w->w, slots, spring, n);
  API_END
}

int avbd_world_cast(avbd_world* w, const float* queries, int32_t n, const avbd_cast_filter* filter, float* hits) {
  API_BEGIN
  REQUIRE(w && (n == 0 || (queries && hits)), "null argument");
  bind(w->A->ctx);
  avbd_cast_filter all{0xffffffffu, 0u, 0, 1, 0, {0}};
  w->A->cast(w->w, queries, n, filter ? *filter : all, hits);
  API_END
}

int avbd_world_import_sleep_state(avbd_world* w, const int32_t* asleep, const float* quiet_time) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->setSleepState(w->w, asleep, quiet_time);
  API_END
}

int avbd_world_flush_edits(avbd_world* w) {
  API_BEGIN
  REQUIRE(w, "null world");
  bind(w->A->ctx);
  w->A->flushEdits(w->w);
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
  auto* b = new avbd_batch{A, slots, nb, {}, 1, 0};
  for (int w : b->worlds) b->starts.emplace_back((long long)A->W[w].dev.bodyOff, w);
  std::sort(b->starts.begin(), b->starts.end());
  *out = b;
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
  if (n == 0) {
    A.resolve();
    return AVBD_OK;
  }
  if (!A.poseStage) {
    A.resolve();  // the allocation waits for the device anyway
    A.poseStage = dalloc<float4>(size_t(n) * 2);
  }
  int blocks = grid_blocks(n, 256);
  if (blocks > device_sms() * 8) blocks = device_sms() * 8;
  // the read is queued behind the steps in flight and waited for with them (one wait); if one of
  // those steps held itself, resolve() re-ran it after the read, which is then made again
  const long long held = A.ticksHeld;
  for (int pass = 0; pass < 2; pass++) {
    k_read_poses<<<blocks, 256, 0, A.s>>>(A.B.pose, A.B.size, n, A.poseStage); note_launches(1);
    CK(cudaMemcpyAsync(out, A.poseStage, size_t(n) * 32, cudaMemcpyDeviceToHost, A.s));
    A.resolve();
    CK(cudaStreamSynchronize(A.s));
    if (A.ticksHeld == held) break;
  }
  API_END
}

int avbd_batch_step_read(avbd_batch* b, int32_t steps, float* out, int64_t* tag) {
  API_BEGIN
  REQUIRE(b && out && tag, "null argument");
  REQUIRE(steps >= 1, "steps must be positive");
  Arena& A = *b->A;
  bind(A.ctx);
  cudaPointerAttributes at{};
  REQUIRE(cudaPointerGetAttributes(&at, out) == cudaSuccess && at.type == cudaMemoryTypeHost,
          "out must be page-locked host memory (avbd_pinned_alloc, cudaHostAlloc or cudaHostRegister)");
  const int n = int(b->bodies);
  if (!A.poseStage && n > 0) {
    A.resolve();
    A.poseStage = dalloc<float4>(size_t(n) * 2);
  }
  for (int i = 0; i + 1 < steps; i++) A.stepWorlds(b->worlds);
  Arena::TickReply reply;
  const long long t = b->nextTag++;
  if (n > 0) {
    reply.rows = n;
    reply.dev = A.poseStage;
    reply.host = reinterpret_cast<float4*>(out);
    reply.seg.push_back(make_int4(0, n, 0, 0));  // the batch's bodies are [0, n) of its arena
  }
  reply.tags.push_back(t);
  A.stepWorlds(b->worlds, &reply);
  *tag = t;
  API_END
}

int avbd_batch_read_done(avbd_batch* b, int64_t tag, int32_t wait, int32_t* done) {
  API_BEGIN
  REQUIRE(b && done, "null argument");
  REQUIRE(tag > 0 && tag < b->nextTag, "no such read");
  Arena& A = *b->A;
  bind(A.ctx);
  // ticks are confirmed in queue order and tags grow with it
  auto collect = [&] {
    for (long long c : A.confirmedTags) b->doneUpTo = std::max(b->doneUpTo, c);
    A.confirmedTags.clear();
  };
  A.trimLog();
  collect();
  if (tag > b->doneUpTo && wait) {
    for (const auto& e : A.tickLog)  // wait for that tick only, not for the ticks queued after it
      if (std::find(e.reply.tags.begin(), e.reply.tags.end(), (long long)tag) != e.reply.tags.end()) {
        CK(cudaEventSynchronize(e.done));
        break;
      }
    A.trimLog();
    collect();
    if (tag > b->doneUpTo) {  // held and queued again: make every queued tick final
      A.resolve();
      collect();
    }
  }
  *done = tag <= b->doneUpTo ? 1 : 0;
  API_END
}

int avbd_pinned_alloc(int64_t bytes, void** out) {
  API_BEGIN
  REQUIRE(out && bytes > 0, "bad argument");
  *out = nullptr;
  CK(cudaHostAlloc(out, size_t(bytes), cudaHostAllocDefault));
  API_END
}

int avbd_pinned_free(void* p) {
  API_BEGIN
  if (p) CK(cudaFreeHost(p));
  API_END
}

int avbd_check_division(int32_t device, int64_t n, uint32_t seed, int64_t* reciprocal_mismatches,
                        int64_t* quotient_mismatches) {
  API_BEGIN
  REQUIRE(reciprocal_mismatches && quotient_mismatches && n >= 0, "bad argument");
  int count = 0;
  CK(cudaGetDeviceCount(&count));
  REQUIRE(device >= 0 && device < count, "no such CUDA device");
  CK(cudaSetDevice(device));
  unsigned long long* bad = dalloc<unsigned long long>(2);
  cudaError_t e = cudaMemset(bad, 0, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = launch_check_division(n, seed, bad);
  unsigned long long h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  CK(e);
  *reciprocal_mismatches = int64_t(h[0]);
  *quotient_mismatches = int64_t(h[1]);
  API_END
}

int avbd_batch_set_velocities(avbd_batch* b, const uint32_t* indices, int32_t n, const float* velocity, const float* angular) {
  API_BEGIN
  REQUIRE(b, "null batch");
  bind(b->A->ctx);
  // batch body index (the arena's body slot) -> (world, local index)
  setVelocities(*b->A, b->starts, b->bodies, indices, n, velocity, angular);
  API_END
}

int avbd_batch_edit(avbd_batch* b, int32_t world, const uint32_t* records, int32_t n) {
  API_BEGIN
  REQUIRE(b && (n == 0 || records), "null argument");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  bind(b->A->ctx);
  b->A->queueEdits(b->worlds[world], records, n);
  API_END
}

int avbd_batch_watch_contacts(avbd_batch* b, int32_t world, const uint32_t* indices, int32_t n, int32_t max_pairs,
                              int32_t max_events) {
  API_BEGIN
  REQUIRE(b, "null batch");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  REQUIRE(max_pairs >= 1 && max_events >= 1, "Contact capacities must be positive integers");
  REQUIRE(!indices || n >= 0, "negative count");
  bind(b->A->ctx);
  b->A->watchContacts(b->worlds[world], indices, n, max_events, indices != nullptr);
  API_END
}

int avbd_batch_contact_events(avbd_batch* b, int32_t world, uint32_t* out, int64_t cap, int64_t* n, int64_t* dropped,
                              int32_t* full) {
  API_BEGIN
  REQUIRE(b && n, "null argument");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  bind(b->A->ctx);
  long long d = 0;
  *n = b->A->readEvents(b->worlds[world], out, cap, &d);
  if (dropped) *dropped = d;
  if (full) *full = d > 0;
  API_END
}

int avbd_batch_read_joints(avbd_batch* b, int32_t world, float* out) {
  API_BEGIN
  REQUIRE(b && out, "null argument");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  bind(b->A->ctx);
  b->A->readJoints(b->worlds[world], out);
  API_END
}

int avbd_batch_set_motor(avbd_batch* b, int32_t world, int32_t slot, int32_t mask, float speed, float max_torque) {
  API_BEGIN
  REQUIRE(b, "null batch");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  bind(b->A->ctx);
  b->A->setMotor(b->worlds[world], slot, mask, speed, max_torque);
  API_END
}

int avbd_batch_release_joints(avbd_batch* b, int32_t world, const int32_t* slots, int32_t n) {
  API_BEGIN
  REQUIRE(b && (n == 0 || slots), "null argument");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  bind(b->A->ctx);
  b->A->releaseJoints(b->worlds[world], slots, n);
  API_END
}

#define BATCH_WORLD(b, world)                                                   \
  REQUIRE(b, "null batch");                                                     \
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range"); \
  bind(b->A->ctx)

int avbd_batch_set_filters(avbd_batch* b, int32_t world, const uint32_t* indices, int32_t n, const uint32_t* groups,
                           const uint32_t* collides_with) {
  API_BEGIN
  BATCH_WORLD(b, world);
  REQUIRE(n == 0 || (indices && groups && collides_with), "null argument");
  b->A->setFilters(b->worlds[world], indices, n, groups, collides_with);
  API_END
}

int avbd_batch_set_restitution(avbd_batch* b, int32_t world, const uint32_t* indices, int32_t n, const float* values) {
  API_BEGIN
  BATCH_WORLD(b, world);
  REQUIRE(n == 0 || (indices && values), "null argument");
  b->A->setRestitution(b->worlds[world], indices, n, values);
  API_END
}

int avbd_batch_set_sensor(avbd_batch* b, int32_t world, const uint32_t* indices, int32_t n, int32_t enabled) {
  API_BEGIN
  BATCH_WORLD(b, world);
  REQUIRE(n == 0 || indices, "null argument");
  b->A->setSensor(b->worlds[world], indices, n, enabled != 0);
  API_END
}

int avbd_batch_set_sleep_enabled(avbd_batch* b, int32_t world, int32_t body, int32_t enabled) {
  API_BEGIN
  BATCH_WORLD(b, world);
  b->A->setSleepAllowed(b->worlds[world], body, enabled != 0);
  API_END
}

int avbd_batch_set_spring_material(avbd_batch* b, int32_t world, int32_t slot, int32_t mask, float break_strain,
                                   float break_force) {
  API_BEGIN
  BATCH_WORLD(b, world);
  b->A->setSpringMaterial(b->worlds[world], slot, mask, break_strain, break_force);
  API_END
}

int avbd_batch_set_world_anchor(avbd_batch* b, int32_t world, int32_t slot, const float* point) {
  API_BEGIN
  BATCH_WORLD(b, world);
  REQUIRE(point, "null argument");
  b->A->setWorldAnchor(b->worlds[world], slot, point);
  API_END
}

int avbd_batch_capture_frames(avbd_batch* b, int32_t world, const int32_t* slots, const int32_t* spring, int32_t n) {
  API_BEGIN
  BATCH_WORLD(b, world);
  REQUIRE(n == 0 || (slots && spring), "null argument");
  b->A->captureFrames(b->worlds[world], slots, spring, n);
  API_END
}

int avbd_batch_cast(avbd_batch* b, int32_t world, const float* queries, int32_t n, const avbd_cast_filter* filter,
                    float* hits) {
  API_BEGIN
  REQUIRE(b && (n == 0 || (queries && hits)), "null argument");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  bind(b->A->ctx);
  avbd_cast_filter all{0xffffffffu, 0u, 0, 1, 0, {0}};
  b->A->cast(b->worlds[world], queries, n, filter ? *filter : all, hits);
  API_END
}

int avbd_batch_sleep_state(avbd_batch* b, int32_t world, int32_t* asleep, float* quiet_time, int32_t* n_sleeping) {
  API_BEGIN
  REQUIRE(b, "null batch");
  REQUIRE(world >= 0 && world < int32_t(b->worlds.size()), "world index out of range");
  bind(b->A->ctx);
  const int c = b->A->sleepState(b->worlds[world], asleep, quiet_time);
  if (n_sleeping) *n_sleeping = c;
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
