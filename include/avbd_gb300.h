/*
 * avbd_gb300 -- C ABI of the GB300 (sm_103a) AVBD rigid-body engine.
 *
 * This is the boundary a host binding (the reference's Node world API through an N-API addon,
 * or Python ctypes) calls. Plain C types only: pointers, sizes, status codes. Every function
 * returns 0 on success or a negative AVBD_E_* code; avbd_last_error() then describes the
 * failure (thread-local string). No C++ exception crosses this boundary. Caller buffers are
 * borrowed for the duration of the call only. One host thread per context (or external
 * locking).
 *
 * Each entry point names the reference interface it replaces (paths in joshbrew/babylon-avbd).
 */
#ifndef AVBD_GB300_H
#define AVBD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AVBD_OK 0
#define AVBD_E_INVALID (-1)   /* bad argument (validated before any work is queued) */
#define AVBD_E_CUDA (-2)      /* CUDA runtime error */
#define AVBD_E_NOMEM (-3)     /* device or host allocation failed / over budget */
#define AVBD_E_STATE (-4)     /* call not valid in the object's current state */
#define AVBD_E_CAPACITY (-5)  /* a fixed capacity was exceeded */

typedef struct avbd_ctx avbd_ctx;
typedef struct avbd_world avbd_world;
typedef struct avbd_batch avbd_batch;

/* Shapes and constraint kinds (src/native/scenes.js addBox/addSphere, addJoint/addSpring). */
#define AVBD_SHAPE_BOX 0
#define AVBD_SHAPE_SPHERE 1
/* addCapsule (src/native/scenes.js:180-193, src/gpu/capsuleShape.js): along local Y, size =
 * (2 radius, tip-to-tip height, 2 radius), bounding radius height / 2. */
#define AVBD_SHAPE_CAPSULE 2
#define AVBD_CONS_JOINT 0
#define AVBD_CONS_SPRING 1
#define AVBD_CONS_IGNORE 2
/* Angular rows about a hinge axis (scenes.js:575-630 addMotor / addHinge minAngle, maxAngle;
 * src/gpu/angularConstraints.js info types 3 and 4): cons_ra / cons_rb carry the unit axis in the
 * frames of a and b (a = -1: world frame); a motor's cons_p0 / cons_p1 are its speed (rad/s) and
 * torque bound, a limit's the lower and upper angle within [-pi, pi]. */
#define AVBD_CONS_MOTOR 3
#define AVBD_CONS_LIMIT 4

/* Solver parameters: reference/three-avbd/src/avbd3d/ref/solver.ts:347-359 and
 * src/native/cpu/cpuSolver3D.ts:46-79 (massPenalty, faceBias, up). */
typedef struct avbd_params {
  float dt;
  float gravity;
  float up[3];
  int32_t iterations;
  float alpha;
  float beta_lin;
  float beta_ang;
  float gamma;
  int32_t mass_penalty; /* contact normal penalty floor min(mA, mB)/dt^2 */
  int32_t face_bias;    /* prefer face axes in box-box SAT (cpuBoxContacts3D.ts:457-466) */
  int32_t color_rounds; /* Jones-Plassmann round budget per step */
  int32_t broadphase;   /* options.broadphase (src/native/scenes.d.ts:299-300): AVBD_BROADPHASE_* */
  int32_t bvh_rebuild;  /* options.bvh.rebuildInterval: steps between tree rebuilds; <= 0: 16 */
  int32_t sleeping;     /* options.sleeping / a body's allowSleep: true (src/native/cpu/world.js:103-108):
                           island sleeping after each step (src/native/cpu/sleeping.js) */
  float sleep_speed;    /* speedThreshold, |(v, w)| in m/s [0.08] */
  float sleep_time;     /* timeThreshold, seconds of quiet before sleeping [0.6] */
} avbd_params;

/* Candidate search. Both give the same pair set; the tree (hierarchical PLOC, src/gpu/gpuHploc.js)
 * suits large worlds whose grid cells would be large against most bodies. AUTO follows
 * src/gpu/appGpuSolver3D.js:333-398: the tree for >= 10,000 bodies when the grid cell is >= 4x
 * twice the median radius or the world is a jointed sheet of thin plates. */
#define AVBD_BROADPHASE_GRID 0
#define AVBD_BROADPHASE_HPLOC 1
#define AVBD_BROADPHASE_AUTO 2

/* A built scene as flat structure-of-arrays in creation order (what AvbdScene3D holds,
 * src/native/scenes.js:107-698). Optional arrays may be NULL (defaults in brackets). */
typedef struct avbd_scene_desc {
  int32_t n_bodies;
  const float* position;         /* 3n */
  const float* rotation;         /* 4n (x, y, z, w) [identity] */
  const float* size;             /* 3n full extents; spheres 2r */
  const float* velocity;         /* 3n [0] */
  const float* angular_velocity; /* 3n [0] */
  const float* prev_velocity;    /* 3n [0] */
  const float* mass;             /* n; <= 0 is static */
  const float* moment;           /* 3n principal moments */
  const float* friction;         /* n */
  const float* radius;           /* n bounding radius */
  const int32_t* shape;          /* n AVBD_SHAPE_* (sphere and capsule: the spine/radius shapes) */
  const uint32_t* group;         /* n [0xffffffff] */
  const uint32_t* collides_with; /* n [0xffffffff] */
  int32_t n_cons;
  const int32_t* cons_kind;      /* n_cons AVBD_CONS_* in creation order */
  const int32_t* cons_a;         /* -1 = world (joints) */
  const int32_t* cons_b;
  const float* cons_ra;          /* 3 n_cons body-local anchor (world point when a = -1); motor/limit: axis */
  const float* cons_rb;          /* 3 n_cons */
  const float* cons_p0;          /* joint: linear stiffness (INFINITY = hard); spring: stiffness;
                                    motor: speed; limit: lower angle */
  const float* cons_p1;          /* joint: angular stiffness; spring: rest length (-1: current);
                                    motor: torque bound; limit: upper angle */
  const float* cons_p2;          /* joint: fracture threshold on |lambda_ang|; spring: breakForce,
                                    the tension limit (<= 0 or INFINITY: none) */
  const float* restitution;      /* n [0] restitution 0..1 (addBox/addSphere option; the velocity
                                    bounce pass of src/native/cpu/restitution.js runs when > 0) */
  const int32_t* allow_sleep;    /* n [1] allowSleep option (scenes.js:235-240): 0 keeps the body's
                                    island awake */
  const float* cons_p3;          /* n_cons [none] spring: breakStrain, the strain limit (<= 0 or
                                    INFINITY: none). A spring past either limit at the start of
                                    a step tears for good (src/gpu/springMaterial.js) */
  const int32_t* is_trigger;     /* n [0] isTrigger option (scenes.js:69-75): its contacts are
                                    reported (events, readSelectedBodies word 11) but apply no
                                    forces, bounce or sleep links (cpuPhysics3D.js:148-156) */
} avbd_scene_desc;

/* readCounters() of src/vendor/three-avbd-lib/solver3D.ts:1460-1463 plus engine state. */
typedef struct avbd_counters {
  int64_t pairs;      /* candidate pairs (bounding spheres overlap) */
  int64_t manifolds;  /* pairs with at least one contact */
  int64_t contacts;
  int64_t joints;     /* unbroken joints and springs */
  int32_t colors;     /* colours used by the last step (max over worlds) */
  int32_t conflicts;  /* bodies left sharing a colour with a neighbour */
  int32_t overflow;   /* capacity regrowths so far */
  int32_t steps;      /* steps taken */
} avbd_counters;

/* Per-kernel-class device time (CUDA events on the engine's stream) and algorithmic bytes,
 * accumulated over the steps taken while profiling is on (the reference's timestamp phases,
 * src/vendor/three-avbd-lib/solver3D.ts:1332-1447, profileDetailedNextStep). */
typedef struct avbd_profile {
  int32_t steps;
  int32_t pad;
  double ms_collide;   /* grid build, pair passes, narrowphase */
  double ms_topology;  /* constraint lists, colouring, colour buckets */
  double ms_primal;    /* every per-colour primal launch */
  double ms_dual;
  double ms_other;     /* joint/body warm start, velocities */
  int64_t primal_launches;
  int64_t launches;    /* kernel launches issued by the library since it was loaded */
  double bytes_primal; /* algorithmic bytes (see the engine's traffic accounting) */
  double bytes_dual;
  double bytes_collide;
  int64_t graph_captures; /* ticks recorded into a CUDA graph (then launched) */
  int64_t graph_replays;  /* ticks launched by replaying a recorded graph */
  int32_t graphs_on;      /* 0 when graph capture failed on this device (ticks launch directly) */
  int32_t ticks_held;     /* ticks held on the device for growth and run again */
  /* The run-time autotuner's choice for the last tick's class (device, size, joints, iterations):
   * tuned = 1 once every candidate was timed; the solve loop's schedule (1: tile queue, 0: colour
   * barriers), chunks per block and colour, persistent blocks (0: all resident), and the digit
   * width of the tree builds' Morton sort. */
  int32_t tuned;
  int32_t solve_queue;
  int32_t solve_waves;
  int32_t solve_blocks;
  int32_t radix_bits;
  int32_t solve_tile;  /* work items per shared-memory tile of the solve (128 or 256) */
} avbd_profile;

/* ---------------------------------------------------------------- context */

/* createSolverPipeline({backend}) (src/native/pipeline.js:14-92): binds a device and stream. */
int avbd_ctx_create(int device, avbd_ctx** out);
/* pipeline.destroy (src/native/pipeline.js:82-90): frees every world/batch it owns. */
int avbd_ctx_destroy(avbd_ctx* ctx);
/* Failure details of the last call on this thread. */
const char* avbd_last_error(void);
/* Library version string. */
const char* avbd_version(void);
/* The CUDA stream all of this context's work is queued on (cudaStream_t), so a host binding can
 * order its own work or timing events after the engine's (the reference's device queue). */
int avbd_ctx_stream(avbd_ctx* ctx, void** stream);
/* Wait until all queued work of the context has finished (the reference's
 * device.queue.onSubmittedWorkDone). */
int avbd_ctx_synchronize(avbd_ctx* ctx);
/* A fence after the work queued so far on the context's stream: onSubmittedWorkDone as a value
 * that another thread can wait on. avbd_fence_wait and avbd_fence_query touch only the fence, so
 * a host binding's worker thread may wait on it while the calling thread keeps queuing work (the
 * Node addon's asynchronous reads: wait on a worker, then read on the main thread, which finds the
 * work done). Every other entry point stays single-threaded per context. */
typedef struct avbd_fence avbd_fence;
int avbd_ctx_fence(avbd_ctx* ctx, avbd_fence** out);
/* Block the calling thread until the device has passed the fence. Thread-safe. */
int avbd_fence_wait(avbd_fence* fence);
/* *done = 1 when the device has passed the fence, else 0. Thread-safe. */
int avbd_fence_query(avbd_fence* fence, int32_t* done);
int avbd_fence_destroy(avbd_fence* fence);

/* ---------------------------------------------------------------- plain worlds */

/* pipeline.createSolver(scene, options) (src/native/pipeline.js:52-81). */
int avbd_world_create(avbd_ctx* ctx, const avbd_scene_desc* scene, const avbd_params* params, avbd_world** out);
/* world.destroy() */
int avbd_world_destroy(avbd_world* w);
/* world.step() repeated `steps` times (src/native/solver3D.js:350-359 -> AppGpuSolver3D.step,
 * src/gpu/appGpuSolver3D.js:403-442 / CpuSolver3D.step, src/native/cpu/cpuSolver3D.ts:144-281). */
int avbd_world_step(avbd_world* w, int32_t steps);
/* world.readBodyState / readBodies: poses and velocities of all bodies (host arrays, any may
 * be NULL): position 3n, rotation 4n, velocity 3n, angular 3n, prev_velocity 3n. */
int avbd_world_read_state(avbd_world* w, float* position, float* rotation, float* velocity, float* angular, float* prev_velocity);
/* world.readSelectedBodies(indices, {posesOnly}) (src/native/cpu/world.js:503-571):
 * 8 floats per body (pos.xyz, friction, quat) when poses_only, else 40 (the 160-byte body
 * record of reference/three-avbd/src/avbd3d/gpu/layout.ts:8-25). */
int avbd_world_read_selected(avbd_world* w, const uint32_t* indices, int32_t n, int32_t poses_only, float* out);
/* Allocation-free variant of avbd_world_read_selected. No counterpart in the reference.
 * For hosts that must not allocate device memory while they run: a render or input loop that
 * reads poses every frame (cudaMalloc and cudaFree can block until the whole device is idle, which
 * stalls the frame), a serving process that has committed its device-memory budget to world state,
 * or a JavaScript binding that must not block its event loop. The staging for the indices and the
 * records lives in one fixed per-GPU device buffer of AVBD_NOALLOC_MAX_SELECTED records (about
 * 1.3 MB, held by every GPU that loads the library until the process exits). Every call looks that
 * buffer's device address up (make the first call before any stream capture). Requests with
 * n > AVBD_NOALLOC_MAX_SELECTED fail with AVBD_E_CAPACITY. A world with queued body commands
 * (avbd_world_edit) fails with AVBD_E_STATE: applying them can allocate, so apply them first with
 * avbd_world_flush_edits or a step. Every call shares the buffer, which keeps the last call's
 * contents: calls whose work overlaps on the GPU (different threads or streams) race; serialise
 * them. Output is identical to avbd_world_read_selected. */
#define AVBD_NOALLOC_MAX_SELECTED 8192
int avbd_world_read_selected_noalloc(avbd_world* w, const uint32_t* indices, int32_t n, int32_t poses_only, float* out);
/* world.setPoses / setVelocities (src/native/runtime.js, scenes.d.ts:317-454); rotation or
 * angular may be NULL. */
int avbd_world_set_poses(avbd_world* w, const uint32_t* indices, int32_t n, const float* position, const float* rotation);
int avbd_world_set_velocities(avbd_world* w, const uint32_t* indices, int32_t n, const float* velocity, const float* angular);
/* world.readCounters() (src/vendor/three-avbd-lib/solver3D.ts:1460-1463). */
int avbd_world_counters(avbd_world* w, avbd_counters* out);

/* Body commands: world.editBodies(edits) / flushEdits() (src/native/runtime.js:46-167,
 * src/native/cpu/world.js:229-300). n records of 12 32-bit words, the layout of the reference's
 * command staging (src/gpu/bodyCommands2D.js:46-55): word 0 body index, 1 kind, 2 has-point,
 * 3 zero, 4-7 value (float), 8-11 point (float). Kinds: 0 set linear velocity, 1 set angular
 * velocity, 2 impulse (at point when has-point), 3 force (value.w = dt), 4 teleport (value.xyz =
 * position, point = unit quaternion when has-point; the body's contacts lose their warm start),
 * 5 angular impulse, 6 torque (value.w = dt). Records are validated, queued, and applied in order
 * at the next step (or at avbd_world_flush_edits). */
int avbd_world_edit(avbd_world* w, const uint32_t* records, int32_t n);
int avbd_world_flush_edits(avbd_world* w);

/* Parity dumps (readPairs / readContactList, solver3D.ts:1466-1506). Each writes at most `cap`
 * records and stores the full count in *n. */
/* Candidate pairs of the last step, sorted ascending by (hi, lo): 2 uint32 per pair. */
int avbd_world_pairs(avbd_world* w, uint32_t* out, int64_t cap, int64_t* n);
/* Contact count of each candidate pair of the last step (same order as avbd_world_pairs). */
int avbd_world_pair_contacts(avbd_world* w, int32_t* out, int64_t cap, int64_t* n);
/* Jones-Plassmann colour of each body after the last step (-1: static / none). */
int avbd_world_colors(avbd_world* w, int32_t* out);

/* Full solver state for one-step parity (the GpuSolver3D.seedFrom counterpart,
 * src/vendor/three-avbd-lib/solver3D.ts:942-979): joint warm-start state (3 floats each, jid
 * order), the live manifolds (pairs with contacts, sorted) and their contacts. Sizes first:
 * call avbd_world_state_sizes, then avbd_world_export_state with buffers of those sizes. */
int avbd_world_state_sizes(avbd_world* w, int32_t* n_joints, int64_t* n_manifolds, int64_t* n_contacts);
int avbd_world_export_state(avbd_world* w, float* jpen_lin, float* jpen_ang, float* jlam_lin, float* jlam_ang,
                            int32_t* jbroken, uint32_t* mpairs, int32_t* mcount, uint32_t* cfeature, float* cra,
                            float* crb, float* cpen, float* clam, int32_t* cstick);

/* Island sleeping (src/native/cpu/sleeping.js; world API of src/native/cpu/world.js:859-890).
 * enableSleeping / disableSleeping: enabled != 0 turns it on with the given thresholds
 * (speedThreshold |(v, w)| m/s, timeThreshold s; both > 0), 0 turns it off; either wakes the
 * world. setSleepEnabled (allowSleep of one body; enabling turns sleeping on with the defaults
 * 0.08 / 0.6 if it was off; wakes the world). wakeAll. Queued body commands, setPoses and
 * setVelocities also wake the world. Sleep state per body: 1 = asleep, and the seconds its island
 * has been quiet; n_sleeping = readSleepStats().sleeping. Any output pointer may be NULL. */
int avbd_world_set_sleeping(avbd_world* w, int32_t enabled, float speed_threshold, float time_threshold);
int avbd_world_set_sleep_enabled(avbd_world* w, int32_t body, int32_t enabled);
int avbd_world_wake_all(avbd_world* w);
int avbd_world_sleep_state(avbd_world* w, int32_t* asleep, float* quiet_time, int32_t* n_sleeping);
/* Contact events (src/native/solver3D.js:256-310 watchContacts / readContactEvents /
 * resetContactHistory; src/vendor/three-avbd-lib/contacts.ts). watch_contacts: the first call turns
 * events on, with room for max_events events between reads, watching every body when indices is
 * NULL; with indices, exactly those n bodies are watched. max_pairs is validated (>= 1) but not a
 * limit here: touching pairs are found in the world's own sorted pair lists, not a bounded set.
 * contact_events: the events since the last read, 12 words each: kind (1 begin, 2 end), body a,
 * body b (world-local, a > b), step (1-based count of the world's steps), point xyz, impulse
 * (|sum of normal lambda| x dt), normal xyz (from b to a), 0 -- floats as bits; in step order,
 * within a step begins then ends, each by (a, b). With out NULL or cap < *n only *n is set and
 * nothing is consumed. dropped = events past the capacity since the last read; full = dropped > 0.
 * reset_contact_history: new lifetimes for the bodies (ascending, unique): their contacts begin
 * afresh at the next step and none of the old ones end. */
int avbd_world_watch_contacts(avbd_world* w, const uint32_t* indices, int32_t n, int32_t max_pairs, int32_t max_events);
int avbd_world_reset_contact_history(avbd_world* w, const uint32_t* indices, int32_t n);
int avbd_world_contact_events(avbd_world* w, uint32_t* out, int64_t cap, int64_t* n, int64_t* dropped, int32_t* full);

/* Shape casts: raycastAll / sphereCastAll (src/native/solver3D.js:244-251, the GPU backend's
 * src/gpu/shapeQueries.js cast): the nearest body each ray (radius 0) or swept sphere hits, against
 * the current poses after queued commands apply. queries: n x 8 floats (origin xyz, max distance,
 * direction xyz (any nonzero length), radius); hits: n x 8 floats (normal xyz, distance (-1: no
 * hit), body index (uint32 bits), 0, 0, 0). Ties in distance go to the lowest body index. The
 * center of the hit sphere is origin + distance x unit direction, the touching point center -
 * radius x normal. filter NULL: every body. */
typedef struct avbd_cast_filter {
  uint32_t collides_with;   /* bodies whose group & collides_with != 0 [0xffffffff] */
  uint32_t membership;      /* with has_membership: bodies whose collidesWith & membership != 0 */
  int32_t has_membership;
  int32_t include_triggers; /* trigger bodies are skipped unless nonzero [1 without a filter] */
  int32_t n_ignore;         /* <= 16 body indices skipped */
  uint32_t ignore[16];
} avbd_cast_filter;
int avbd_world_cast(avbd_world* w, const float* queries, int32_t n, const avbd_cast_filter* filter, float* hits);

/* readJoints() (src/vendor/three-avbd-lib/solver3D.ts:1456-1458): 32 floats per joint or spring in
 * creation order, the reference's record (avbd3d/gpu/layout.ts:27-36): penalty lin (w: linear
 * stiffness, 0 once broken), penalty ang (w: angular stiffness, 0 once broken), lambda lin
 * (w: fracture threshold), lambda ang (w: torque arm), C0 lin, C0 ang, rA (w: spring rest
 * length), rB; infinities as +-3e38. Queued commands apply first. */
int avbd_world_read_joints(avbd_world* w, float* out);
/* setFilters(indices, groups, collidesWith) (src/native/scenes.d.ts:414-418): new collision
 * filters for the given bodies; the world wakes. */
int avbd_world_set_filters(avbd_world* w, const uint32_t* indices, int32_t n, const uint32_t* groups,
                           const uint32_t* collides_with);
/* setRestitution per body (src/native/cpu/world.js:343-351; editBodies' restitution property):
 * values in [0, 1]; the world wakes. */
int avbd_world_set_restitution(avbd_world* w, const uint32_t* indices, int32_t n, const float* values);
/* setSensor(index, enabled) (src/native/cpu/world.js:342-350; editBodies' isTrigger property): the
 * bodies become (enabled != 0) or stop being triggers; the world wakes. */
int avbd_world_set_sensor(avbd_world* w, const uint32_t* indices, int32_t n, int32_t enabled);
/* setMotor(slot, {speed, maxTorque}) (src/gpu/appGpuSolver3D.js:547-562, src/native/cpu/world.js:
 * 360-388): slot is the joint index of an AVBD_CONS_MOTOR constraint; mask bit 0 sets the speed,
 * bit 1 the torque bound (finite, >= 0). The world wakes. */
int avbd_world_set_motor(avbd_world* w, int32_t slot, int32_t mask, float speed, float max_torque);
/* releaseJoints(slots) (src/native/cpu/world.js:397-410; src/vendor/three-avbd-lib/solver3D.ts:
 * 1173-1193): the joints, springs or angular rows at the given joint indices stop acting (their
 * records read as released, their bodies collide again); the world wakes. */
int avbd_world_release_joints(avbd_world* w, const int32_t* slots, int32_t n);
/* setSpringMaterial(slot, {breakStrain, breakForce}) (src/gpu/appGpuSolver3D.js:810-835): limits
 * of a live spring (positive, or INFINITY: none); mask bit 0 sets breakStrain, bit 1 breakForce.
 * The world wakes. */
int avbd_world_set_spring_material(avbd_world* w, int32_t slot, int32_t mask, float break_strain, float break_force);
/* setWorldAnchor(slot, point) (src/gpu/appGpuSolver3D.js:928-941): moves the world point of a live
 * joint attached to the world (a grab handle); the world wakes. */
int avbd_world_set_world_anchor(avbd_world* w, int32_t slot, const float* point);
/* captureConstraintFrames(entries) (src/native/cpu/world.js:474-492): per entry, a live joint's rest
 * rotation (spring[k] = 0) or a live spring's rest length (spring[k] != 0) is taken again from the
 * current poses, after queued commands; the world wakes. */
int avbd_world_capture_frames(avbd_world* w, const int32_t* slots, const int32_t* spring, int32_t n);

/* Load per-body sleep flags and quiet times (state import for one-step comparisons; NULL skips). */
int avbd_world_import_sleep_state(avbd_world* w, const int32_t* asleep, const float* quiet_time);

/* ---------------------------------------------------------------- batched worlds */

/* Many independent worlds stepped together: one launch sequence per step covers every world
 * (no counterpart in the reference, which creates one solver per world:
 * src/native/pipeline.js:52-81). World w of the batch keeps its own parameters. */
int avbd_batch_create(avbd_ctx* ctx, const avbd_scene_desc* scenes, const avbd_params* params, int32_t n_worlds,
                      avbd_batch** out);
int avbd_batch_destroy(avbd_batch* b);
/* Advance every world of the batch by `steps`. */
int avbd_batch_step(avbd_batch* b, int32_t steps);
int avbd_batch_world_count(avbd_batch* b, int32_t* n_worlds, int64_t* n_bodies);
/* State of world `world` of the batch (as avbd_world_read_state). */
int avbd_batch_read_state(avbd_batch* b, int32_t world, float* position, float* rotation, float* velocity,
                          float* angular, float* prev_velocity);
int avbd_batch_counters(avbd_batch* b, avbd_counters* out);
/* Poses of every body of every world, 8 floats each (pos.xyz, friction, quat), world by world
 * in creation order (readSelectedBodies(.., {posesOnly: true}) over the whole batch). */
int avbd_batch_read_poses(avbd_batch* b, float* out);
/* Pipelined reads (the WebGPU backend's reads are asynchronous too: mapAsync): queue `steps`
 * steps of every world and, right after the last one, a copy of every body's pose (the layout of
 * avbd_batch_read_poses) into `out`, then return at once with a tag. `out` must be page-locked host
 * memory (avbd_pinned_alloc, cudaHostAlloc or cudaHostRegister) and stay valid until the read is
 * done; the copy runs in stream order behind the steps and is made again if one of them had to be
 * re-run. avbd_batch_read_done: *done = 1 once the read has landed (wait = 1: block until then,
 * without waiting for steps queued after it). Typical loop: step_read into one of two buffers,
 * then read_done on the other, so the host never stalls the device. No counterpart in the
 * reference's CPU path. */
int avbd_batch_step_read(avbd_batch* b, int32_t steps, float* out, int64_t* tag);
int avbd_batch_read_done(avbd_batch* b, int64_t tag, int32_t wait, int32_t* done);
/* Page-locked host memory for avbd_batch_step_read (cudaHostAlloc / cudaFreeHost). */
int avbd_pinned_alloc(int64_t bytes, void** out);
int avbd_pinned_free(void* p);
/* setVelocities for bodies given by batch-global index (world offset + body index). */
int avbd_batch_set_velocities(avbd_batch* b, const uint32_t* indices, int32_t n, const float* velocity, const float* angular);
/* Body commands (as avbd_world_edit) for world `world` of the batch (world-local body indices). */
int avbd_batch_edit(avbd_batch* b, int32_t world, const uint32_t* records, int32_t n);
/* Joint records of world `world` of the batch (as avbd_world_read_joints). */
int avbd_batch_read_joints(avbd_batch* b, int32_t world, float* out);
/* setMotor for world `world` of the batch (as avbd_world_set_motor). */
int avbd_batch_set_motor(avbd_batch* b, int32_t world, int32_t slot, int32_t mask, float speed, float max_torque);
/* releaseJoints for world `world` of the batch (as avbd_world_release_joints). */
int avbd_batch_release_joints(avbd_batch* b, int32_t world, const int32_t* slots, int32_t n);
/* The world-local property and constraint edits for world `world` of the batch (as the
 * avbd_world_* forms: set_filters, set_restitution, set_sensor, set_spring_material,
 * set_world_anchor, capture_frames). */
int avbd_batch_set_filters(avbd_batch* b, int32_t world, const uint32_t* indices, int32_t n, const uint32_t* groups,
                           const uint32_t* collides_with);
int avbd_batch_set_restitution(avbd_batch* b, int32_t world, const uint32_t* indices, int32_t n, const float* values);
int avbd_batch_set_sensor(avbd_batch* b, int32_t world, const uint32_t* indices, int32_t n, int32_t enabled);
int avbd_batch_set_sleep_enabled(avbd_batch* b, int32_t world, int32_t body, int32_t enabled);
int avbd_batch_set_spring_material(avbd_batch* b, int32_t world, int32_t slot, int32_t mask, float break_strain,
                                   float break_force);
int avbd_batch_set_world_anchor(avbd_batch* b, int32_t world, int32_t slot, const float* point);
int avbd_batch_capture_frames(avbd_batch* b, int32_t world, const int32_t* slots, const int32_t* spring, int32_t n);
/* Shape casts against world `world` of the batch (as avbd_world_cast). */
int avbd_batch_cast(avbd_batch* b, int32_t world, const float* queries, int32_t n, const avbd_cast_filter* filter,
                    float* hits);
/* Contact events of world `world` of the batch (as avbd_world_watch_contacts / _contact_events). */
int avbd_batch_watch_contacts(avbd_batch* b, int32_t world, const uint32_t* indices, int32_t n, int32_t max_pairs,
                              int32_t max_events);
int avbd_batch_contact_events(avbd_batch* b, int32_t world, uint32_t* out, int64_t cap, int64_t* n, int64_t* dropped,
                              int32_t* full);
/* Sleep state of world `world` of the batch (as avbd_world_sleep_state). */
int avbd_batch_sleep_state(avbd_batch* b, int32_t world, int32_t* asleep, float* quiet_time, int32_t* n_sleeping);

/* Profiling (see avbd_profile): enable resets the accumulators; read returns them. */
int avbd_world_profile(avbd_world* w, int32_t enable);
int avbd_world_profile_read(avbd_world* w, avbd_profile* out);
int avbd_batch_profile(avbd_batch* b, int32_t enable);
int avbd_batch_profile_read(avbd_batch* b, avbd_profile* out);

/* ---------------------------------------------------------------- serving */

/* A world server: worlds are admitted and released at any time, advance requests queue steps,
 * and each tick steps every world with queued steps in one launch sequence (continuous
 * batching). Device memory is held under a byte budget: when a new or restored world does not
 * fit, the least recently used idle world (no queued steps) is evicted to host memory and
 * restored when work for it arrives. A world's results do not depend on what else is served,
 * on ticks it waits, or on eviction: K steps give the same bits as avbd_world_step(w, K) on
 * the same scene. No counterpart in the reference (one solver per world, stepped by its owner:
 * src/native/pipeline.js:52-81, src/native/runtime.js:255-272). World ids and tickets are
 * positive and never reused. */
typedef struct avbd_server avbd_server;

typedef struct avbd_server_desc {
  int64_t budget_bytes;   /* device bytes the server's arrays may occupy (> 0) */
  int32_t initial_bodies; /* initial capacities (grown on demand within the budget) */
  int32_t initial_worlds;
} avbd_server_desc;

typedef struct avbd_server_stats {
  int64_t budget_bytes, device_bytes, peak_device_bytes;
  int64_t live_worlds, resident_worlds, evicted_worlds, pending_worlds;
  int64_t resident_bodies, admitted, rejected, evictions, restores, ticks, body_steps, completed;
} avbd_server_stats;

int avbd_server_create(avbd_ctx* ctx, const avbd_server_desc* desc, avbd_server** out);
int avbd_server_destroy(avbd_server* s);
/* Admit a world (as avbd_world_create). AVBD_E_CAPACITY when it cannot fit in the budget even
 * after evicting every idle world; nothing changes then. */
int avbd_server_admit(avbd_server* s, const avbd_scene_desc* scene, const avbd_params* params, int64_t* world_id);
/* Queue `steps` steps of a world; *ticket completes once they have run. */
int avbd_server_advance(avbd_server* s, int64_t world_id, int32_t steps, int64_t* ticket);
/* One step of every world with queued steps (evicted ones are restored first, room
 * permitting). *n_stepped = worlds stepped (may be 0). */
int avbd_server_tick(avbd_server* s, int32_t* n_stepped);
/* Up to max_steps steps of every world with queued steps, queued back to back on the device
 * without waiting (each step is a tick over the worlds that still have steps: the same bits as
 * max_steps calls of avbd_server_tick), so a request for K steps completes in one call. With
 * replies, the poses of every world whose request a step completes are gathered right after that
 * step and copied to pinned host memory in stream order; those tickets are then reported by
 * avbd_server_ready (once their step has run on the device), not by avbd_server_completed, and
 * avbd_server_take_reply hands out the poses. No counterpart in the reference (which has no
 * server). */
int avbd_server_tick_steps(avbd_server* s, int32_t max_steps, int32_t replies, int32_t* n_stepped);
/* Tickets whose replies have arrived (wait = 0: without waiting for the device). */
int avbd_server_ready(avbd_server* s, int64_t* tickets, int32_t cap, int32_t wait, int32_t* n);
/* The reply of a ready ticket: its world's poses after the completing step, 8 floats per body
 * (pos, friction, quat), n_bodies rows; with out NULL or cap_bodies < n_bodies only the size is
 * returned. A reply is handed out once. */
int avbd_server_take_reply(avbd_server* s, int64_t ticket, float* out, int64_t cap_bodies, int32_t* n_bodies);
/* Drain up to `cap` completed tickets (oldest first); *n = number written. */
int avbd_server_completed(avbd_server* s, int64_t* tickets, int32_t cap, int32_t* n);
/* Poses of every body of each listed world, 8 floats each (pos.xyz, friction, quat), world
 * after world in list order; evicted worlds are read from their host copy. */
int avbd_server_read_poses(avbd_server* s, const int64_t* world_ids, int32_t n, float* out);
/* Full state of one world (as avbd_world_read_state); any pointer may be null. */
int avbd_server_read_state(avbd_server* s, int64_t world_id, float* position, float* rotation, float* velocity,
                           float* angular, float* prev_velocity);
/* World facts: bodies, queued steps, steps done, resident (1) or evicted (0). */
int avbd_server_world_info(avbd_server* s, int64_t world_id, int32_t* n_bodies, int64_t* queued, int64_t* steps_done,
                           int32_t* resident);
/* Body commands (as avbd_world_edit), applied before the world's next step. */
int avbd_server_edit(avbd_server* s, int64_t world_id, const uint32_t* records, int32_t n);
/* Shape casts against a resident served world (as avbd_world_cast). */
int avbd_server_cast(avbd_server* s, int64_t world_id, const float* queries, int32_t n, const avbd_cast_filter* filter,
                     float* hits);
/* Contact events of a served world (as avbd_world_watch_contacts / _contact_events); events of an
 * evicted world wait on the host. */
int avbd_server_watch_contacts(avbd_server* s, int64_t world_id, const uint32_t* indices, int32_t n, int32_t max_pairs,
                               int32_t max_events);
int avbd_server_contact_events(avbd_server* s, int64_t world_id, uint32_t* out, int64_t cap, int64_t* n, int64_t* dropped,
                               int32_t* full);
/* Sleep state of a served world, resident or evicted (as avbd_world_sleep_state). */
int avbd_server_sleep_state(avbd_server* s, int64_t world_id, int32_t* asleep, float* quiet_time, int32_t* n_sleeping);
/* Evict a world now (its queued steps wait for a restore). */
int avbd_server_evict(avbd_server* s, int64_t world_id);
/* Drop a world; its outstanding tickets never complete. */
int avbd_server_release(avbd_server* s, int64_t world_id);
int avbd_server_read_stats(avbd_server* s, avbd_server_stats* out);

/* ---- diagnostics (no reference counterpart) */
/* The solve's LDL^T factorisation divides by each pivot through its reciprocal (one Newton step on
 * rcp.approx) and Markstein's fused-multiply-add correction, which must give the bits of the IEEE
 * division wherever it is used. This checks the reciprocal against 1/d for every float of its
 * range (both signs) and the quotients on n seeded operand pairs, on `device`, and counts the
 * results that differ in any bit. */
int avbd_check_division(int32_t device, int64_t n, uint32_t seed, int64_t* reciprocal_mismatches,
                        int64_t* quotient_mismatches);

#ifdef __cplusplus
}
#endif
#endif /* AVBD_GB300_H */
