// Node-API addon over the engine's C ABI (include/avbd_gb300.h): the native side of a "gb300"
// backend for createSolverPipeline (src/native/pipeline.js:14-92). Every entry point validates
// nothing itself beyond argument shapes: the library validates and reports through
// avbd_last_error(), which becomes a synchronous JS exception here, where the reference throws.
// Handles are externals; typed arrays are borrowed for the duration of one call.
//
// Build where Node headers exist (node-gyp with binding.gyp beside this file), with
// libavbd_gb300.so on the library path. The JS side is index.js.
#include <node_api.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "avbd_gb300.h"

namespace {

napi_value Throw(napi_env env, const char* msg) {
  napi_throw_error(env, nullptr, msg);
  return nullptr;
}
napi_value ThrowLast(napi_env env) { return Throw(env, avbd_last_error()); }
#define CALL(expr)                 \
  do {                             \
    if ((expr) != AVBD_OK) return ThrowLast(env); \
  } while (0)

template <size_t N> bool Args(napi_env env, napi_callback_info info, napi_value (&argv)[N], size_t need) {
  size_t argc = N;
  if (napi_get_cb_info(env, info, &argc, argv, nullptr, nullptr) != napi_ok || argc < need) {
    napi_throw_type_error(env, nullptr, "missing arguments");
    return false;
  }
  return true;
}

template <class T> T* External(napi_env env, napi_value v) {
  void* p = nullptr;
  if (napi_get_value_external(env, v, &p) != napi_ok || !p) {
    napi_throw_type_error(env, nullptr, "expected a handle");
    return nullptr;
  }
  return static_cast<T*>(p);
}

bool IsNullish(napi_env env, napi_value v) {
  napi_valuetype t;
  napi_typeof(env, v, &t);
  return t == napi_undefined || t == napi_null;
}

// A typed array's data and element count (nullptr, 0 for undefined/null).
template <class T> bool Typed(napi_env env, napi_value v, const T** data, size_t* n) {
  *data = nullptr;
  *n = 0;
  if (IsNullish(env, v)) return true;
  napi_typedarray_type type;
  void* p = nullptr;
  napi_value ab;
  size_t off = 0, len = 0;
  if (napi_get_typedarray_info(env, v, &type, &len, &p, &ab, &off) != napi_ok) {
    napi_throw_type_error(env, nullptr, "expected a typed array");
    return false;
  }
  *data = static_cast<const T*>(p);
  *n = len;
  return true;
}

template <class T> const T* Field(napi_env env, napi_value obj, const char* key, size_t* n = nullptr) {
  napi_value v;
  bool has = false;
  napi_has_named_property(env, obj, key, &has);
  if (!has) return nullptr;
  napi_get_named_property(env, obj, key, &v);
  const T* d = nullptr;
  size_t len = 0;
  Typed<T>(env, v, &d, &len);
  if (n) *n = len;
  return d;
}

double Number(napi_env env, napi_value obj, const char* key, double fallback) {
  bool has = false;
  napi_has_named_property(env, obj, key, &has);
  if (!has) return fallback;
  napi_value v;
  napi_get_named_property(env, obj, key, &v);
  double d = fallback;
  if (napi_get_value_double(env, v, &d) != napi_ok) {
    bool b = false;
    if (napi_get_value_bool(env, v, &b) == napi_ok) return b ? 1.0 : 0.0;
  }
  return d;
}

int32_t Int(napi_env env, napi_value v) {
  int32_t i = 0;
  napi_get_value_int32(env, v, &i);
  return i;
}
int64_t Id(napi_env env, napi_value v) {
  double d = 0;
  napi_get_value_double(env, v, &d);
  return int64_t(d);
}
napi_value Num(napi_env env, double d) {
  napi_value v;
  napi_create_double(env, d, &v);
  return v;
}
napi_value Float32(napi_env env, size_t n, float** data) {
  void* p = nullptr;
  napi_value buf, arr;
  napi_create_arraybuffer(env, n * 4, &p, &buf);
  napi_create_typedarray(env, napi_float32_array, n, buf, 0, &arr);
  *data = static_cast<float*>(p);
  return arr;
}
napi_value Uint32(napi_env env, size_t n, uint32_t** data) {
  void* p = nullptr;
  napi_value buf, arr;
  napi_create_arraybuffer(env, n * 4, &p, &buf);
  napi_create_typedarray(env, napi_uint32_array, n, buf, 0, &arr);
  *data = static_cast<uint32_t*>(p);
  return arr;
}
void Set(napi_env env, napi_value obj, const char* key, napi_value v) { napi_set_named_property(env, obj, key, v); }

// The structure-of-arrays scene (packScene in index.js) and solver parameters.
bool Scene(napi_env env, napi_value s, napi_value p, avbd_scene_desc* d, avbd_params* q) {
  std::memset(d, 0, sizeof(*d));
  std::memset(q, 0, sizeof(*q));
  size_t n = 0, nc = 0;
  d->mass = Field<float>(env, s, "mass", &n);
  d->n_bodies = int32_t(n);
  d->position = Field<float>(env, s, "position");
  d->rotation = Field<float>(env, s, "rotation");
  d->size = Field<float>(env, s, "size");
  d->velocity = Field<float>(env, s, "velocity");
  d->angular_velocity = Field<float>(env, s, "angularVelocity");
  d->prev_velocity = Field<float>(env, s, "prevVelocity");
  d->moment = Field<float>(env, s, "moment");
  d->friction = Field<float>(env, s, "friction");
  d->radius = Field<float>(env, s, "radius");
  d->shape = Field<int32_t>(env, s, "shape");
  d->group = Field<uint32_t>(env, s, "group");
  d->collides_with = Field<uint32_t>(env, s, "collidesWith");
  d->cons_kind = Field<int32_t>(env, s, "consKind", &nc);
  d->n_cons = int32_t(nc);
  d->cons_a = Field<int32_t>(env, s, "consA");
  d->cons_b = Field<int32_t>(env, s, "consB");
  d->cons_ra = Field<float>(env, s, "consRA");
  d->cons_rb = Field<float>(env, s, "consRB");
  d->cons_p0 = Field<float>(env, s, "consP0");
  d->cons_p1 = Field<float>(env, s, "consP1");
  d->cons_p2 = Field<float>(env, s, "consP2");
  d->restitution = Field<float>(env, s, "restitution");
  d->allow_sleep = Field<int32_t>(env, s, "allowSleep");
  d->cons_p3 = Field<float>(env, s, "consP3");
  d->is_trigger = Field<int32_t>(env, s, "isTrigger");
  q->dt = float(Number(env, p, "dt", 1.0 / 60.0));
  q->gravity = float(Number(env, p, "gravity", -10.0));
  const float* up = Field<float>(env, p, "up");
  q->up[0] = up ? up[0] : 0.f;
  q->up[1] = up ? up[1] : 1.f;
  q->up[2] = up ? up[2] : 0.f;
  q->iterations = int32_t(Number(env, p, "iterations", 10));
  q->alpha = float(Number(env, p, "alpha", 0.99));
  q->beta_lin = float(Number(env, p, "betaLin", 10000.0));
  q->beta_ang = float(Number(env, p, "betaAng", 100.0));
  q->gamma = float(Number(env, p, "gamma", 0.999));
  q->mass_penalty = int32_t(Number(env, p, "massPenalty", 1));
  q->face_bias = int32_t(Number(env, p, "faceBias", 1));
  q->color_rounds = int32_t(Number(env, p, "colorRounds", 64));
  q->broadphase = int32_t(Number(env, p, "broadphase", AVBD_BROADPHASE_AUTO));
  q->bvh_rebuild = int32_t(Number(env, p, "bvhRebuild", 16));
  q->sleeping = int32_t(Number(env, p, "sleeping", 0));
  q->sleep_speed = float(Number(env, p, "sleepSpeed", 0.08));
  q->sleep_time = float(Number(env, p, "sleepTime", 0.6));
  return true;
}

// ---------------------------------------------------------------- context
napi_value CreateContext(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  if (!Args(env, info, argv, 1)) return nullptr;
  avbd_ctx* ctx = nullptr;
  CALL(avbd_ctx_create(Int(env, argv[0]), &ctx));
  napi_value out;
  napi_create_external(env, ctx, nullptr, nullptr, &out);
  return out;
}
napi_value DestroyContext(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  if (!Args(env, info, argv, 1)) return nullptr;
  auto* ctx = External<avbd_ctx>(env, argv[0]);
  if (!ctx) return nullptr;
  CALL(avbd_ctx_destroy(ctx));
  return nullptr;
}
napi_value Synchronize(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  if (!Args(env, info, argv, 1)) return nullptr;
  auto* ctx = External<avbd_ctx>(env, argv[0]);
  if (!ctx) return nullptr;
  CALL(avbd_ctx_synchronize(ctx));
  return nullptr;
}

// ---------------------------------------------------------------- worlds
napi_value CreateWorld(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  if (!Args(env, info, argv, 3)) return nullptr;
  auto* ctx = External<avbd_ctx>(env, argv[0]);
  if (!ctx) return nullptr;
  avbd_scene_desc d;
  avbd_params q;
  Scene(env, argv[1], argv[2], &d, &q);
  avbd_world* w = nullptr;
  CALL(avbd_world_create(ctx, &d, &q, &w));
  napi_value out;
  napi_create_external(env, w, nullptr, nullptr, &out);
  return out;
}
#define WORLD_ARG(k)                                   \
  napi_value argv[k];                                  \
  if (!Args(env, info, argv, 1)) return nullptr;       \
  auto* w = External<avbd_world>(env, argv[0]);        \
  if (!w) return nullptr

napi_value DestroyWorld(napi_env env, napi_callback_info info) {
  WORLD_ARG(1);
  CALL(avbd_world_destroy(w));
  return nullptr;
}
napi_value Step(napi_env env, napi_callback_info info) {
  WORLD_ARG(2);
  CALL(avbd_world_step(w, Int(env, argv[1])));
  return nullptr;
}
napi_value Edit(napi_env env, napi_callback_info info) {  // (w, Uint32Array of 12-word records)
  WORLD_ARG(2);
  const uint32_t* rec;
  size_t n;
  if (!Typed(env, argv[1], &rec, &n)) return nullptr;
  CALL(avbd_world_edit(w, rec, int32_t(n / 12)));
  return nullptr;
}
napi_value FlushEdits(napi_env env, napi_callback_info info) {
  WORLD_ARG(1);
  CALL(avbd_world_flush_edits(w));
  return nullptr;
}
napi_value ReadSelected(napi_env env, napi_callback_info info) {  // (w, Uint32Array, posesOnly)
  WORLD_ARG(3);
  const uint32_t* idx;
  size_t n;
  if (!Typed(env, argv[1], &idx, &n)) return nullptr;
  bool poses = false;
  napi_get_value_bool(env, argv[2], &poses);
  float* out;
  napi_value arr = Float32(env, n * (poses ? 8 : 40), &out);
  CALL(avbd_world_read_selected(w, idx, int32_t(n), poses ? 1 : 0, out));
  return arr;
}
napi_value ReadState(napi_env env, napi_callback_info info) {  // (w, bodyCount)
  WORLD_ARG(2);
  const size_t n = size_t(Int(env, argv[1]));
  float *p, *q, *v, *a, *pv;
  napi_value obj;
  napi_create_object(env, &obj);
  Set(env, obj, "position", Float32(env, 3 * n, &p));
  Set(env, obj, "rotation", Float32(env, 4 * n, &q));
  Set(env, obj, "velocity", Float32(env, 3 * n, &v));
  Set(env, obj, "angular", Float32(env, 3 * n, &a));
  Set(env, obj, "prevVelocity", Float32(env, 3 * n, &pv));
  CALL(avbd_world_read_state(w, p, q, v, a, pv));
  return obj;
}
napi_value SetPoses(napi_env env, napi_callback_info info) {  // (w, Uint32Array, Float32Array, Float32Array?)
  WORLD_ARG(4);
  const uint32_t* idx;
  const float *pos, *rot;
  size_t n, np, nr;
  if (!Typed(env, argv[1], &idx, &n) || !Typed(env, argv[2], &pos, &np) || !Typed(env, argv[3], &rot, &nr)) return nullptr;
  if (np != 3 * n || (rot && nr != 4 * n)) return Throw(env, "pose arrays must match the indices");
  CALL(avbd_world_set_poses(w, idx, int32_t(n), pos, rot));
  return nullptr;
}
napi_value SetVelocities(napi_env env, napi_callback_info info) {  // (w, Uint32Array, linear?, angular?)
  WORLD_ARG(4);
  const uint32_t* idx;
  const float *lin, *ang;
  size_t n, nl, na;
  if (!Typed(env, argv[1], &idx, &n) || !Typed(env, argv[2], &lin, &nl) || !Typed(env, argv[3], &ang, &na)) return nullptr;
  if ((lin && nl != 3 * n) || (ang && na != 3 * n)) return Throw(env, "velocity arrays must match the indices");
  CALL(avbd_world_set_velocities(w, idx, int32_t(n), lin, ang));
  return nullptr;
}
napi_value ReadCounters(napi_env env, napi_callback_info info) {
  WORLD_ARG(1);
  avbd_counters c;
  CALL(avbd_world_counters(w, &c));
  napi_value obj;
  napi_create_object(env, &obj);
  Set(env, obj, "pairs", Num(env, double(c.pairs)));
  Set(env, obj, "manifolds", Num(env, double(c.manifolds)));
  Set(env, obj, "contacts", Num(env, double(c.contacts)));
  Set(env, obj, "joints", Num(env, double(c.joints)));
  Set(env, obj, "colors", Num(env, c.colors));
  Set(env, obj, "clashes", Num(env, c.conflicts));
  Set(env, obj, "overflow", Num(env, c.overflow));
  return obj;
}
napi_value ReadJoints(napi_env env, napi_callback_info info) {  // (w, jointCount)
  WORLD_ARG(2);
  float* out;
  napi_value arr = Float32(env, size_t(Int(env, argv[1])) * 32, &out);
  CALL(avbd_world_read_joints(w, out));
  return arr;
}
napi_value SetFilters(napi_env env, napi_callback_info info) {  // (w, indices, groups, masks) Uint32Arrays
  WORLD_ARG(4);
  const uint32_t *idx, *g, *m;
  size_t n, ng, nm;
  if (!Typed(env, argv[1], &idx, &n) || !Typed(env, argv[2], &g, &ng) || !Typed(env, argv[3], &m, &nm)) return nullptr;
  if (ng != n || nm != n) return Throw(env, "filter arrays must match the indices");
  CALL(avbd_world_set_filters(w, idx, int32_t(n), g, m));
  return nullptr;
}
napi_value SetRestitution(napi_env env, napi_callback_info info) {  // (w, Uint32Array, Float32Array)
  WORLD_ARG(3);
  const uint32_t* idx;
  const float* e;
  size_t n, ne;
  if (!Typed(env, argv[1], &idx, &n) || !Typed(env, argv[2], &e, &ne)) return nullptr;
  if (ne != n) return Throw(env, "restitution values must match the indices");
  CALL(avbd_world_set_restitution(w, idx, int32_t(n), e));
  return nullptr;
}
napi_value SetSensor(napi_env env, napi_callback_info info) {  // (w, Uint32Array, enabled)
  WORLD_ARG(3);
  const uint32_t* idx;
  size_t n;
  if (!Typed(env, argv[1], &idx, &n)) return nullptr;
  CALL(avbd_world_set_sensor(w, idx, int32_t(n), Int(env, argv[2])));
  return nullptr;
}
napi_value SetMotor(napi_env env, napi_callback_info info) {  // (w, slot, speed|undefined, maxTorque|undefined)
  WORLD_ARG(4);
  int32_t mask = 0;
  double speed = 0, torque = 0;
  napi_valuetype t;
  napi_typeof(env, argv[2], &t);
  if (t == napi_number) { napi_get_value_double(env, argv[2], &speed); mask |= 1; }
  napi_typeof(env, argv[3], &t);
  if (t == napi_number) { napi_get_value_double(env, argv[3], &torque); mask |= 2; }
  CALL(avbd_world_set_motor(w, Int(env, argv[1]), mask, float(speed), float(torque)));
  return nullptr;
}
napi_value SetSpringMaterial(napi_env env, napi_callback_info info) {  // (w, slot, breakStrain|undefined, breakForce|undefined)
  WORLD_ARG(4);
  int32_t mask = 0;
  double v[2] = {0, 0};
  for (int k = 0; k < 2; k++) {
    napi_valuetype t;
    napi_typeof(env, argv[2 + k], &t);
    if (t == napi_number) { napi_get_value_double(env, argv[2 + k], &v[k]); mask |= 1 << k; }
  }
  CALL(avbd_world_set_spring_material(w, Int(env, argv[1]), mask, float(v[0]), float(v[1])));
  return nullptr;
}
napi_value SetWorldAnchor(napi_env env, napi_callback_info info) {  // (w, slot, Float32Array(3))
  WORLD_ARG(3);
  const float* p;
  size_t n;
  if (!Typed(env, argv[2], &p, &n)) return nullptr;
  if (n != 3) return Throw(env, "A world joint and finite xyz anchor are required");
  CALL(avbd_world_set_world_anchor(w, Int(env, argv[1]), p));
  return nullptr;
}
napi_value CaptureFrames(napi_env env, napi_callback_info info) {  // (w, Int32Array slots, Int32Array spring)
  WORLD_ARG(3);
  const int32_t *slots, *spring;
  size_t n, ns;
  if (!Typed(env, argv[1], &slots, &n) || !Typed(env, argv[2], &spring, &ns)) return nullptr;
  if (ns != n) return Throw(env, "one spring flag per slot");
  CALL(avbd_world_capture_frames(w, slots, spring, int32_t(n)));
  return nullptr;
}
napi_value ReleaseJoints(napi_env env, napi_callback_info info) {  // (w, Int32Array of joint slots)
  WORLD_ARG(2);
  const int32_t* slots;
  size_t n;
  if (!Typed(env, argv[1], &slots, &n)) return nullptr;
  CALL(avbd_world_release_joints(w, slots, int32_t(n)));
  return nullptr;
}
napi_value WatchContacts(napi_env env, napi_callback_info info) {  // (w, Uint32Array|null, maxPairs, maxEvents)
  WORLD_ARG(4);
  const uint32_t* idx;
  size_t n;
  if (!Typed(env, argv[1], &idx, &n)) return nullptr;
  CALL(avbd_world_watch_contacts(w, idx, int32_t(n), Int(env, argv[2]), Int(env, argv[3])));
  return nullptr;
}
napi_value ReadContactEvents(napi_env env, napi_callback_info info) {  // -> {records, dropped, full}
  WORLD_ARG(1);
  int64_t n = 0, dropped = 0;
  int32_t full = 0;
  CALL(avbd_world_contact_events(w, nullptr, 0, &n, &dropped, &full));
  uint32_t* out;
  napi_value arr = Uint32(env, size_t(n) * 12, &out);
  CALL(avbd_world_contact_events(w, out, n, &n, &dropped, &full));
  napi_value obj, b;
  napi_create_object(env, &obj);
  Set(env, obj, "records", arr);
  Set(env, obj, "dropped", Num(env, double(dropped)));
  napi_get_boolean(env, full != 0, &b);
  Set(env, obj, "full", b);
  return obj;
}
napi_value ResetContactHistory(napi_env env, napi_callback_info info) {
  WORLD_ARG(2);
  const uint32_t* idx;
  size_t n;
  if (!Typed(env, argv[1], &idx, &n)) return nullptr;
  CALL(avbd_world_reset_contact_history(w, idx, int32_t(n)));
  return nullptr;
}
napi_value Cast(napi_env env, napi_callback_info info) {  // (w, Float32Array 8/query, filter{}) -> hits
  WORLD_ARG(3);
  const float* q;
  size_t n;
  if (!Typed(env, argv[1], &q, &n)) return nullptr;
  avbd_cast_filter f{0xffffffffu, 0u, 0, 1, 0, {0}};
  if (!IsNullish(env, argv[2])) {
    f.collides_with = uint32_t(Number(env, argv[2], "collidesWith", 4294967295.0));
    bool hasMembership = false;
    napi_has_named_property(env, argv[2], "membership", &hasMembership);
    if (hasMembership) {
      f.has_membership = 1;
      f.membership = uint32_t(Number(env, argv[2], "membership", 0));
    }
    size_t ni = 0;
    const uint32_t* ign = Field<uint32_t>(env, argv[2], "ignore", &ni);
    if (ni > 16) return Throw(env, "Queries can ignore up to 16 live body indices");
    f.n_ignore = int32_t(ni);
    for (size_t k = 0; k < ni; k++) f.ignore[k] = ign[k];
  }
  float* out;
  napi_value arr = Float32(env, n, &out);
  CALL(avbd_world_cast(w, q, int32_t(n / 8), &f, out));
  return arr;
}
napi_value SetSleeping(napi_env env, napi_callback_info info) {  // (w, enabled, speed, time)
  WORLD_ARG(4);
  bool on = false;
  napi_get_value_bool(env, argv[1], &on);
  double speed = 0.08, time = 0.6;
  napi_get_value_double(env, argv[2], &speed);
  napi_get_value_double(env, argv[3], &time);
  CALL(avbd_world_set_sleeping(w, on ? 1 : 0, float(speed), float(time)));
  return nullptr;
}
napi_value SetSleepEnabled(napi_env env, napi_callback_info info) {  // (w, body, enabled)
  WORLD_ARG(3);
  bool on = false;
  napi_get_value_bool(env, argv[2], &on);
  CALL(avbd_world_set_sleep_enabled(w, Int(env, argv[1]), on ? 1 : 0));
  return nullptr;
}
napi_value WakeAll(napi_env env, napi_callback_info info) {
  WORLD_ARG(1);
  CALL(avbd_world_wake_all(w));
  return nullptr;
}
napi_value SleepStats(napi_env env, napi_callback_info info) {
  WORLD_ARG(1);
  int32_t n = 0;
  CALL(avbd_world_sleep_state(w, nullptr, nullptr, &n));
  return Num(env, n);
}

// ---------------------------------------------------------------- servers
napi_value CreateServer(napi_env env, napi_callback_info info) {  // (ctx, budgetBytes, bodies, worlds)
  napi_value argv[4];
  if (!Args(env, info, argv, 2)) return nullptr;
  auto* ctx = External<avbd_ctx>(env, argv[0]);
  if (!ctx) return nullptr;
  avbd_server_desc d{Id(env, argv[1]), 0, 0};
  if (!IsNullish(env, argv[2])) d.initial_bodies = Int(env, argv[2]);
  if (!IsNullish(env, argv[3])) d.initial_worlds = Int(env, argv[3]);
  avbd_server* s = nullptr;
  CALL(avbd_server_create(ctx, &d, &s));
  napi_value out;
  napi_create_external(env, s, nullptr, nullptr, &out);
  return out;
}
#define SERVER_ARG(k)                                  \
  napi_value argv[k];                                  \
  if (!Args(env, info, argv, 1)) return nullptr;       \
  auto* s = External<avbd_server>(env, argv[0]);       \
  if (!s) return nullptr

napi_value DestroyServer(napi_env env, napi_callback_info info) {
  SERVER_ARG(1);
  CALL(avbd_server_destroy(s));
  return nullptr;
}
napi_value Admit(napi_env env, napi_callback_info info) {  // (s, scene, params) -> world id
  SERVER_ARG(3);
  avbd_scene_desc d;
  avbd_params q;
  Scene(env, argv[1], argv[2], &d, &q);
  int64_t id = 0;
  CALL(avbd_server_admit(s, &d, &q, &id));
  return Num(env, double(id));
}
napi_value Advance(napi_env env, napi_callback_info info) {  // (s, id, steps) -> ticket
  SERVER_ARG(3);
  int64_t ticket = 0;
  CALL(avbd_server_advance(s, Id(env, argv[1]), Int(env, argv[2]), &ticket));
  return Num(env, double(ticket));
}
napi_value Tick(napi_env env, napi_callback_info info) {
  SERVER_ARG(1);
  int32_t n = 0;
  CALL(avbd_server_tick(s, &n));
  return Num(env, n);
}
napi_value Completed(napi_env env, napi_callback_info info) {  // -> Float64Array of tickets
  SERVER_ARG(1);
  std::vector<int64_t> t(65536);
  int32_t n = 0;
  CALL(avbd_server_completed(s, t.data(), int32_t(t.size()), &n));
  void* p = nullptr;
  napi_value buf, arr;
  napi_create_arraybuffer(env, size_t(n) * 8, &p, &buf);
  napi_create_typedarray(env, napi_float64_array, size_t(n), buf, 0, &arr);
  for (int32_t k = 0; k < n; k++) static_cast<double*>(p)[k] = double(t[size_t(k)]);
  return arr;
}
napi_value ServerReadPoses(napi_env env, napi_callback_info info) {  // (s, Float64Array ids, bodies) -> Float32Array
  SERVER_ARG(3);
  const double* ids;
  size_t n;
  if (!Typed(env, argv[1], &ids, &n)) return nullptr;
  std::vector<int64_t> w(n);
  for (size_t k = 0; k < n; k++) w[k] = int64_t(ids[k]);
  float* out;
  napi_value arr = Float32(env, size_t(Int(env, argv[2])) * 8, &out);
  CALL(avbd_server_read_poses(s, w.data(), int32_t(n), out));
  return arr;
}
napi_value ServerEdit(napi_env env, napi_callback_info info) {  // (s, id, Uint32Array records)
  SERVER_ARG(3);
  const uint32_t* rec;
  size_t n;
  if (!Typed(env, argv[2], &rec, &n)) return nullptr;
  CALL(avbd_server_edit(s, Id(env, argv[1]), rec, int32_t(n / 12)));
  return nullptr;
}
napi_value Evict(napi_env env, napi_callback_info info) {
  SERVER_ARG(2);
  CALL(avbd_server_evict(s, Id(env, argv[1])));
  return nullptr;
}
napi_value Release(napi_env env, napi_callback_info info) {
  SERVER_ARG(2);
  CALL(avbd_server_release(s, Id(env, argv[1])));
  return nullptr;
}
napi_value ServerStats(napi_env env, napi_callback_info info) {
  SERVER_ARG(1);
  avbd_server_stats st;
  CALL(avbd_server_read_stats(s, &st));
  napi_value obj;
  napi_create_object(env, &obj);
  Set(env, obj, "deviceBytes", Num(env, double(st.device_bytes)));
  Set(env, obj, "peakDeviceBytes", Num(env, double(st.peak_device_bytes)));
  Set(env, obj, "liveWorlds", Num(env, double(st.live_worlds)));
  Set(env, obj, "evictedWorlds", Num(env, double(st.evicted_worlds)));
  Set(env, obj, "pendingWorlds", Num(env, double(st.pending_worlds)));
  Set(env, obj, "admitted", Num(env, double(st.admitted)));
  Set(env, obj, "rejected", Num(env, double(st.rejected)));
  Set(env, obj, "evictions", Num(env, double(st.evictions)));
  Set(env, obj, "restores", Num(env, double(st.restores)));
  Set(env, obj, "bodySteps", Num(env, double(st.body_steps)));
  return obj;
}

napi_value TickSteps(napi_env env, napi_callback_info info) {  // (s, maxSteps, replies) -> steps taken
  SERVER_ARG(3);
  bool replies = false;
  napi_get_value_bool(env, argv[2], &replies);
  int32_t n = 0;
  CALL(avbd_server_tick_steps(s, Int(env, argv[1]), replies ? 1 : 0, &n));
  return Num(env, n);
}

// Every reply that has arrived, taken out of the server: [{ticket, poses: Float32Array}, ...].
// Main thread only. Returns nullptr with *status set when a call fails.
napi_value TakeReplies(napi_env env, avbd_server* s, int* status) {
  std::vector<int64_t> tickets;
  int64_t t[1024];
  for (int32_t n = 1024; n == 1024;) {
    if ((*status = avbd_server_ready(s, t, 1024, 0, &n)) != AVBD_OK) return nullptr;
    tickets.insert(tickets.end(), t, t + n);
  }
  napi_value arr;
  napi_create_array_with_length(env, tickets.size(), &arr);
  for (size_t k = 0; k < tickets.size(); k++) {
    int32_t rows = 0;
    if ((*status = avbd_server_take_reply(s, tickets[k], nullptr, 0, &rows)) != AVBD_OK) return nullptr;
    float* out;
    napi_value poses = Float32(env, size_t(rows) * 8, &out);
    if ((*status = avbd_server_take_reply(s, tickets[k], out, rows, &rows)) != AVBD_OK) return nullptr;
    napi_value item;
    napi_create_object(env, &item);
    Set(env, item, "ticket", Num(env, double(tickets[k])));
    Set(env, item, "poses", poses);
    napi_set_element(env, arr, uint32_t(k), item);
  }
  return arr;
}
napi_value Ready(napi_env env, napi_callback_info info) {  // (s) -> [{ticket, poses}] without waiting
  SERVER_ARG(1);
  int status = AVBD_OK;
  napi_value arr = TakeReplies(env, s, &status);
  if (status != AVBD_OK) return ThrowLast(env);
  return arr;
}

// ---------------------------------------------------------------- asynchronous serving
// The Node event loop must not block on the device. A worker thread of libuv waits on a fence
// (avbd_fence_wait touches nothing but the fence, the one thread-safe entry point); the completion
// then runs on the main thread, where every other library call is made, and finds the work done.
struct FenceWork {
  avbd_server* server = nullptr;
  avbd_fence* fence = nullptr;
  napi_deferred deferred = nullptr;
  napi_async_work work = nullptr;
  int status = AVBD_OK;
  std::string error;
  int32_t stepped = 0;         // tickAsync: steps queued by the tick
  bool only = false;           // fence: nothing to do after the wait
  bool read = false;           // readPosesAsync: the worlds to read and their total bodies
  std::vector<int64_t> ids;
  size_t bodies = 0;
};

void FenceExecute(napi_env, void* data) {  // worker thread
  auto* f = static_cast<FenceWork*>(data);
  if ((f->status = avbd_fence_wait(f->fence)) != AVBD_OK) f->error = avbd_last_error();
}

void FenceComplete(napi_env env, napi_status, void* data) {  // main thread
  auto* f = static_cast<FenceWork*>(data);
  avbd_fence_destroy(f->fence);
  napi_value result = nullptr;
  if (f->status == AVBD_OK && f->only) {
    napi_get_undefined(env, &result);
  } else if (f->status == AVBD_OK) {
    if (f->read) {
      float* out;
      result = Float32(env, f->bodies * 8, &out);
      f->status = avbd_server_read_poses(f->server, f->ids.data(), int32_t(f->ids.size()), out);
    } else {
      napi_value replies = TakeReplies(env, f->server, &f->status);
      napi_create_object(env, &result);
      Set(env, result, "stepped", Num(env, f->stepped));
      if (replies) Set(env, result, "replies", replies);
    }
    if (f->status != AVBD_OK) f->error = avbd_last_error();
  }
  if (f->status == AVBD_OK) {
    napi_resolve_deferred(env, f->deferred, result);
  } else {
    napi_value msg, err;
    napi_create_string_utf8(env, f->error.c_str(), NAPI_AUTO_LENGTH, &msg);
    napi_create_error(env, nullptr, msg, &err);
    napi_reject_deferred(env, f->deferred, err);
  }
  napi_delete_async_work(env, f->work);
  delete f;
}

// Queue the fence wait of f on a libuv worker; returns the promise.
napi_value QueueFence(napi_env env, avbd_ctx* ctx, FenceWork* f) {
  napi_value promise, name;
  if (avbd_ctx_fence(ctx, &f->fence) != AVBD_OK) {
    delete f;
    return ThrowLast(env);
  }
  napi_create_promise(env, &f->deferred, &promise);
  napi_create_string_utf8(env, "avbd_gb300.fence", NAPI_AUTO_LENGTH, &name);
  napi_create_async_work(env, nullptr, name, FenceExecute, FenceComplete, f, &f->work);
  napi_queue_async_work(env, f->work);
  return promise;
}

// (ctx) -> Promise<undefined>, settled once the device has run everything queued before the call
// (the reference's device.queue.onSubmittedWorkDone()). A read made after it finds the steps done,
// so the event loop never waits on the device: the world's async reads await it first.
napi_value Fence(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  if (!Args(env, info, argv, 1)) return nullptr;
  auto* ctx = External<avbd_ctx>(env, argv[0]);
  if (!ctx) return nullptr;
  auto* f = new FenceWork;
  f->only = true;
  return QueueFence(env, ctx, f);
}

// (ctx, s, maxSteps) -> Promise<{stepped, replies: [{ticket, poses}]}>: one multi-step tick with
// captured replies, queued without waiting; the promise settles once the device has run it (and
// carries every reply that arrived by then). The caller may queue further ticks, admissions and
// edits meanwhile: tick after tick stays in flight, as in avbd_server_tick_steps.
napi_value TickAsync(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  if (!Args(env, info, argv, 3)) return nullptr;
  auto* ctx = External<avbd_ctx>(env, argv[0]);
  auto* s = External<avbd_server>(env, argv[1]);
  if (!ctx || !s) return nullptr;
  auto* f = new FenceWork;
  f->server = s;
  if (avbd_server_tick_steps(s, Int(env, argv[2]), 1, &f->stepped) != AVBD_OK) {
    delete f;
    return ThrowLast(env);
  }
  return QueueFence(env, ctx, f);
}

// (ctx, s, Float64Array ids, bodies) -> Promise<Float32Array>: the listed worlds' poses, read once
// the device has run every tick queued before the call (steps queued after it may be included).
napi_value ReadPosesAsync(napi_env env, napi_callback_info info) {
  napi_value argv[4];
  if (!Args(env, info, argv, 4)) return nullptr;
  auto* ctx = External<avbd_ctx>(env, argv[0]);
  auto* s = External<avbd_server>(env, argv[1]);
  if (!ctx || !s) return nullptr;
  const double* ids;
  size_t n;
  if (!Typed(env, argv[2], &ids, &n)) return nullptr;
  auto* f = new FenceWork;
  f->server = s;
  f->read = true;
  f->ids.assign(n, 0);
  for (size_t k = 0; k < n; k++) f->ids[k] = int64_t(ids[k]);
  f->bodies = size_t(Int(env, argv[3]));
  return QueueFence(env, ctx, f);
}

napi_value Init(napi_env env, napi_value exports) {
  const struct {
    const char* name;
    napi_callback fn;
  } fns[] = {{"createContext", CreateContext}, {"destroyContext", DestroyContext}, {"synchronize", Synchronize},
             {"createWorld", CreateWorld},     {"destroyWorld", DestroyWorld},     {"step", Step},
             {"edit", Edit},                   {"flushEdits", FlushEdits},         {"readSelected", ReadSelected},
             {"readState", ReadState},         {"setPoses", SetPoses},             {"setVelocities", SetVelocities},
             {"readCounters", ReadCounters},   {"readJoints", ReadJoints},         {"setFilters", SetFilters},
             {"setRestitution", SetRestitution}, {"setSensor", SetSensor},       {"setMotor", SetMotor},         {"releaseJoints", ReleaseJoints},
             {"setSpringMaterial", SetSpringMaterial}, {"setWorldAnchor", SetWorldAnchor},
             {"captureFrames", CaptureFrames},
             {"watchContacts", WatchContacts}, {"readContactEvents", ReadContactEvents},
             {"resetContactHistory", ResetContactHistory}, {"cast", Cast},         {"setSleeping", SetSleeping},
             {"setSleepEnabled", SetSleepEnabled}, {"wakeAll", WakeAll},           {"sleepStats", SleepStats},
             {"createServer", CreateServer},   {"destroyServer", DestroyServer},   {"admit", Admit},
             {"advance", Advance},             {"tick", Tick},                     {"completed", Completed},
             {"serverReadPoses", ServerReadPoses}, {"serverEdit", ServerEdit},     {"evict", Evict},
             {"release", Release},             {"serverStats", ServerStats},       {"tickSteps", TickSteps},
             {"ready", Ready},                 {"tickAsync", TickAsync},           {"readPosesAsync", ReadPosesAsync},
             {"fence", Fence}};
  for (const auto& f : fns) {
    napi_value v;
    napi_create_function(env, f.name, NAPI_AUTO_LENGTH, f.fn, nullptr, &v);
    napi_set_named_property(env, exports, f.name, v);
  }
  napi_value ver;
  napi_create_string_utf8(env, avbd_version(), NAPI_AUTO_LENGTH, &ver);
  napi_set_named_property(env, exports, "version", ver);
  return exports;
}

}  // namespace

NAPI_MODULE(NODE_GYP_MODULE_NAME, Init)
