// Internal interface of the AVBD engine: device layouts shared by the kernel translation units
// and the host orchestration (engine.cu). Not part of the C ABI.
//
// Every world is a self-contained segment of one arena in HBM:
//   bodies   a contiguous range of the body arrays: poses as (pos(xyz, bounding radius), rot)
//            pairs for the current, step-start (x-) and inertial poses, then one float4 per field:
//            vel ang vprev size(xyz, friction) mass(m, Ix, Iy, Iz) meta(world, shape, group, mask)
//   joints   a contiguous range of the joint arrays: body pair, rA(xyz, kind) rB(xyz, rest)
//            stiff(lin, ang, fracture, torqueArm) penLin penAng lamLin lamAng C0Lin C0Ang restQ, broken
//            (a spring: stiff(stiffness, strain limit, tension limit, torqueArm), rest length in rB.w;
//            motors and limits: angular.cuh)
//   pairs    a region of pair slots, present in two buffers (slot + k * slotStride, k = 0, 1): the
//            world's previous state lives in buffer which[w], a step writes the other buffer and
//            flips which[w]. Per slot: (hi, lo) sorted ascending within the world, contact count,
//            basis rows n(w: friction), t1(w: the world's alpha), t2(w: its beta_lin), and 8
//            contact slots of 4 float4: rA(xyz, feature|stick) rB(xyz, C0.n) pen(xyz, C0.t1)
//            lam(xyz, C0.t2).
//   colours  two buffers of per-body colour state, selected like the pairs.
// A step (a "tick") runs over an explicit list of active worlds: the bodies, joints and pair slots
// of those worlds only. Worlds not stepped keep their state untouched, so a world evolves the
// same way whether it is stepped alone, in a batch, or parked between requests.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "avbd_math.cuh"

namespace avbd {

constexpr int MAX_CONTACTS = 8;
constexpr int MAX_COLORS = 64;
constexpr int MAX_LARGE = 64;  // large-body slots per world
constexpr float PENALTY_MIN = 1.0f;
constexpr float PENALTY_MAX = 1e10f;
constexpr float COLLISION_MARGIN = 0.01f;
constexpr float STICK_THRESH = 0.00001f;
constexpr uint32_t STICK_BIT = 0x80000000u;
constexpr uint32_t JOINT_BIT = 0x80000000u;  // constraint-list entry is a joint id
constexpr int SHAPE_BOX = 0;
constexpr int SHAPE_SPHERE = 1;
constexpr int SHAPE_CAPSULE = 2;  // along local Y; size (2r, height, 2r) (src/gpu/capsuleShape.js)
constexpr int KIND_JOINT = 0;
constexpr int KIND_SPRING = 1;
// Angular rows about a hinge axis (src/gpu/angularConstraints.js info types 3 and 4): a motor
// driving the twist at a speed under a torque bound, or lower/upper angle stops. Their records
// live in the joint arrays (angular.cuh gives the field map).
constexpr int KIND_MOTOR = 3;
constexpr int KIND_LIMIT = 4;

constexpr int FLAG_MASS_PENALTY = 1;
constexpr int FLAG_FACE_BIAS = 2;
constexpr int FLAG_BVH = 4;  // broadphase by the world's bounding-volume hierarchy (bvh.cu)
constexpr int FLAG_RESTITUTION = 8;  // some body has restitution > 0: run the bounce pass
constexpr int FLAG_SLEEP = 16;       // island sleeping after each step (sleep.cu)
constexpr int SLEEP_ASLEEP = 1;      // the body sleeps: the solve leaves it where it is
constexpr int SLEEP_ALLOW = 2;       // allowSleep (a body without it keeps its island awake)
constexpr int BODY_TRIGGER = 4;      // isTrigger: its contacts are reported but apply no forces
constexpr int FLAG_EVENTS = 32;      // contact begin/end events after each step (events.cu)
// A pair with a trigger body (src/native/cpu/cpuPhysics3D.js:148-156, sleeping.js:54,
// restitution.js:68): its manifold and contacts exist (events, queries) but it joins no constraint
// list (no primal or dual rows, no colouring edge, no bounce) and links no sleeping island.
__host__ __device__ __forceinline__ bool trigger_pair(const int* bits, int a, int b) {
  return bits && (((a >= 0 ? bits[a] : 0) | bits[b]) & BODY_TRIGGER);
}
// A watch word: bit 0 = the body reports its contacts; the bits above count its lifetimes
// (resetContactHistory adds 2), so a changed word restarts the body's contact history.
constexpr uint32_t WATCH_ON = 1u;
constexpr uint32_t EVENT_BEGIN = 1u, EVENT_END = 2u;
constexpr int EVENT_FLOAT4 = 3;  // per event: (kind, a, b, step) bits; (point, impulse); (normal, 0)

// Per-world parameters and ranges (96 bytes).
struct WorldDev {
  float dt, gravity, alpha, gamma;
  float betaLin, betaAng, cell, largeR;
  float up0, up1, up2;
  int iterations;
  int flags, bodyOff, bodyCount, largeOff;
  int largeCount, jointOff, jointCount, pairOff;
  int pairCap, bvhNodeOff, bvhRoot, pad0;  // bvhRoot: local node id (-1: empty tree)
  float sleepSpeed, sleepDelay;            // FLAG_SLEEP: |(v, w)| threshold, seconds of quiet
  int pad1, pad2;
};

// Poses are stored as interleaved pairs (pos, rot) of 32 bytes: a gather of a body's pose, or of
// its pose and step-start pose, touches one (two) 32-byte sectors instead of two (four).
struct BodyPtrs {
  float4 *pose, *pose0, *poseY;  // (pos, rot) at [2i], [2i + 1]: current, step start (x-), inertial
  float4 *vel, *ang, *vprev, *size, *mass;
  // set by each step's warm start for the solve and the velocity update (step-constant there):
  // (pos, qinverse(rot)) of the step-start and inertial poses at [2i], [2i + 1] (one 32-byte
  // sector per body read), and (mass, inertia) / dt^2
  float4 *pose0i, *poseYi, *inert;
  int4* meta;
  float* restitution;  // per body (0 for most)
  int* sleep;          // per body: SLEEP_ASLEEP | SLEEP_ALLOW | BODY_TRIGGER
  float* sleepTime;    // per body: seconds its island has been quiet (FLAG_SLEEP worlds)
  uint32_t *watch, *watchPrev;  // per body: contact-event watch word now and at the last event pass
  __host__ __device__ __forceinline__ float4& pos(int i) const { return pose[2 * size_t(i)]; }
  __host__ __device__ __forceinline__ float4& rot(int i) const { return pose[2 * size_t(i) + 1]; }
  __host__ __device__ __forceinline__ float4& pos0(int i) const { return pose0[2 * size_t(i)]; }
  __host__ __device__ __forceinline__ float4& rot0(int i) const { return pose0[2 * size_t(i) + 1]; }
  __host__ __device__ __forceinline__ float4& posY(int i) const { return poseY[2 * size_t(i)]; }
  __host__ __device__ __forceinline__ float4& rotY(int i) const { return poseY[2 * size_t(i) + 1]; }
};

struct JointPtrs {
  int2* ab;
  float4 *rA, *rB, *stiff, *penLin, *penAng, *lamLin, *lamAng, *C0Lin, *C0Ang, *restQ;
  int* broken;  // 0 live; 1 gone; 2 broken or torn this step, still joining its pair in the broadphase
};

// Both pair buffers (slots [0, slotStride) and [slotStride, 2 slotStride)).
struct PairPtrs {
  uint2* pair;     // (hi, lo)
  int* count;      // contacts (0: no manifold)
  float4* basis;   // 3 per slot
  float4* ct;      // 4 per contact, 8 contacts per slot
};

// Control block of the tick protocol (one per arena, device memory). A tick never waits for
// the host: its capacities are chosen before it is queued, and its gate (k_tick_gate, after the
// constraint lists and colours, before anything that changes a world's state) checks them. A
// tick whose pair regions or work items overflowed sets `held`; from then on every kernel that
// would change state, in that tick and in every tick queued after it, returns at once, so the
// worlds stay exactly as the last good tick left them. The host sees `held` later, grows the
// capacities and queues the held ticks again (the reference's protectSolverStep, which turns the
// solve of an overflowing step into no-ops, src/gpu/gpuSolverKernels.js:72-102, with adapt's
// growth, src/vendor/three-avbd-lib/solver3D.ts:1515-1559; here the held steps are re-run so
// capacities never change a result).
struct TickCtl {
  int held;       // 1: a tick overflowed; state-changing kernels do nothing until the host clears it
  int ticksDone;  // ticks completed (not held), counted by k_tick_end
  int itemsNeed;  // largest number of contact work items a tick needed
  int waitFail;   // a bounded wait of the persistent solve gave up (an error, never expected)
};

// The active set of one tick.
struct Tick {
  const int4* active;   // per active world, by body offset: (world, bodyPrefix, jointPrefix, -)
  int nActive;
  const int* wactive;   // world -> index in `active` (-1: not stepped)
  int* which;           // world -> buffer holding its last completed state
  int* bodies;          // active bodies, world by world
  int nBodies;
  int* joints;          // active joints
  int nJoints;
  int* pairs;           // active pair slots (count in Counters::activePairs)
  int* pairPrefix;      // [nActive + 1] scanned pair counts of the active worlds
  int* pairN;           // [2 * maxWorlds]: pairs of world w in buffer k at [k * maxWorlds + w]
  int* wover;           // world -> pair slots needed when its region overflowed (0: fits)
  const int* triggerBits;  // the per-body words when a stepped world has trigger bodies, else null
  int maxWorlds;
  int slotStride;       // pair slots per buffer
  int bodyStride;       // colour entries per buffer
  TickCtl* ctl;         // the arena's tick control block
};

// A held tick (TickCtl::held): the kernels that change world state return at once.
__device__ __forceinline__ bool tick_held(const TickCtl* c) { return *(volatile const int*)&c->held != 0; }

// Device counters (one block of ints, reset each tick where noted).
struct Counters {
  int activePairs;      // pair slots written this tick (all active worlds)
  int overflowWorlds;   // worlds whose pair region overflowed
  int remaining;        // colouring: bodies still pending
  int ncolors;
  int conflicts;
  int manifolds;
  int contacts;
  int joints;
  int colorCount[MAX_COLORS];
  int colorStart[MAX_COLORS + 1];
  int itemsTotal;
  int colorItems[MAX_COLORS];
};

constexpr int PAIR_TMP = 16;  // partners a body keeps from the enumerating pass (more: enumerated again)

// Bounding-volume hierarchies of the worlds that use one, in one pool of nodes (each world a
// range starting at WorldDev::bvhNodeOff; node ids below are local to the range). A node is two
// float4: (lo.xyz, left) and (hi.xyz, right); a leaf has right == BVH_END and left = its body's
// local index.
constexpr uint32_t BVH_END = 0xffffffffu;
constexpr int BVH_WIDTH = 16;  // clusters per treelet
struct BvhPool {
  float4* node;      // 2 per node
  uint32_t* parent;  // per node (BVH_END: root or unused)
  uint32_t* escape;  // per node: where traversal continues after its subtree (BVH_END: done)
  uint32_t* minIdx;  // per node: least local body index below it
};

struct Grid {
  uint32_t tableMask;  // hash table size - 1 (power of two)
  int* cellCount;      // table + 1 (scanned in place to starts)
  int* cellFill;
  int* cellBodies;     // small bodies bucketed
  int4* cellKey;       // per bucketed entry: its cell (x, y, z, world)
  float4* cellPos;     // per bucketed entry: position and bounding radius
  int* bodyBucket;     // per body (-1: large)
  int* large;          // MAX_LARGE slots per world: its large bodies, ascending
  uint32_t* pairTmp;   // PAIR_TMP partners per active body: partner m of list position k at m * nBodies + k
  BvhPool bvh;         // trees of the worlds with FLAG_BVH
};

// Narrowphase scratch (per tick), indexed by position q in the tick's active pair list: SAT
// results of overlapping box pairs, the queued lists (box hits by q, sphere pairs by slot) and
// their counts (ctr[0] box hits, ctr[1] sphere-box pairs, ctr[2] sphere-sphere pairs).
struct NarrowScratch {
  float4* sat;
  int* boxList;
  int* sphereList;   // pairs of a sphere and a box
  int* sphere2List;  // pairs of two spheres
  int* ctr;
};

struct NoCollide {
  unsigned long long* keys;  // (hi << 32 | lo), sorted
  int* jid;                  // joint/spring id (broken ones stop blocking), -1 for ignore pairs
  int n;
};

// Per-tick topology, indexed by a body's position k in the tick's active body list.
struct Topo {
  int* adjStart;   // nBodies + 1
  int* adjFill;    // nBodies
  uint32_t* adjList;
  int* adjOther;     // per constraint-list entry: the other body if it is dynamic, else -1
  int* activeIndex;  // body -> k (valid for active bodies)
  int* color;        // both colour buffers, 2 * bodyStride entries (see Tick::which)
  int* won;          // round scratch, per body
  unsigned char* pending;  // per body
  int* colorBodies;  // active indices k, bucketed by colour, ascending within a bucket
  int* colorScan;    // colour scatter scratch: (colour, block of 256 positions) counts, scanned
  int4* slotRef;     // per bucket slot: (body, list position k, world, iterations | asleep << 30), written with the work items
  // manifold-contact work items of the dynamic bodies, bucket order (see primal_chunk):
  int* itemStart;  // per bucket slot, nBodies + 1 (exclusive scan of item counts)
  int4* itemRef;   // item -> (pair slot, item code (item_code), body A, body B)
};

// ---------------------------------------------------------------- launchers
// scan.cu
size_t scan_temp_bytes(int n);
// exclusive scan of n ints in place; writes the total to *total (device) if non-null
void scan_exclusive(int* data, int n, int* total, void* temp, cudaStream_t s);
int grid_blocks(long long n, int threads);
// Streaming multiprocessors of the current device (looked up once per device): grids of the
// grid-stride kernels are capped at a multiple of it.
int device_sms();
// Looks up the per-device launch geometry (call before capturing launches into a graph).
void prepare_launches();
// Kernel launches issued by this library (host counter, for the benchmark's launch count).
void note_launches(int n);
long long launches_total();

// collide.cu
void launch_tick_begin(Tick t, Topo topo, const WorldDev* worlds, cudaStream_t s);
void launch_grid_build(const BodyPtrs& b, const WorldDev* worlds, Tick t, Grid g, void* scanTemp, cudaStream_t s);
void launch_pairs(const BodyPtrs& b, const WorldDev* worlds, Tick t, Grid g, NoCollide nc, const int* jbroken, int* pairCount,
                  PairPtrs P, Counters* ctr, void* scanTemp, cudaStream_t s);
void launch_narrowphase(const BodyPtrs& b, const WorldDev* worlds, Tick t, PairPtrs P, NarrowScratch ns, const Counters* ctr,
                        int pairBudget, cudaStream_t s);

// bvh.cu
struct BvhLevel {
  int inputCount, nodeBase, inputOffset, outputOffset, blocks;
};
struct BvhLayout {
  std::vector<BvhLevel> levels;
  uint32_t root = BVH_END;
  int nodes = 0;     // node ids in use: [0, nodes)
  int clusters = 0;  // cluster-list entries the build needs
};
struct BvhScratch {
  uint2* keys[2];     // Morton keys, ping-pong
  int* hist;          // radix digit counts
  uint32_t* clusters;
  float4* bounds;     // per-block bounds, then the scene bounds
};
void bvh_layout(int n, BvhLayout& L);
size_t bvh_scratch_keys(int n);
size_t bvh_scratch_hist(int n);
size_t bvh_scratch_bounds(int n);
// radixBits: digit width of the Morton-code sort (4, 6 or 8; same order for every width)
void launch_bvh_build(const BodyPtrs& b, int bodyOff, int n, BvhPool pool, int nodeOff, const BvhLayout& L, BvhScratch sc,
                      void* scanTemp, int radixBits, cudaStream_t s);
void launch_bvh_refit(const BodyPtrs& b, int bodyOff, int n, BvhPool pool, int nodeOff, const BvhLayout& L, cudaStream_t s);

// solve.cu
void launch_joint_prepare(const BodyPtrs& b, JointPtrs j, int j0, int j1, cudaStream_t s);
void launch_joint_capture(const BodyPtrs& b, JointPtrs j, int slot, int spring, cudaStream_t s);
void launch_spring_tear(const BodyPtrs& b, JointPtrs j, Tick t, cudaStream_t s);
void launch_joint_retire(JointPtrs j, Tick t, cudaStream_t s);
void launch_joint_warmstart(const BodyPtrs& b, const WorldDev* worlds, JointPtrs j, Tick t, cudaStream_t s);
void launch_body_warmstart(const BodyPtrs& b, const WorldDev* worlds, Tick t, cudaStream_t s);
void launch_adjacency(const BodyPtrs& b, JointPtrs j, PairPtrs P, Tick t, const Counters* ctr, Topo topo, int pairBudget,
                      void* scanTemp, cudaStream_t s);
void launch_coloring(const BodyPtrs& b, const WorldDev* worlds, JointPtrs j, PairPtrs P, Tick t, Topo topo, int rounds,
                     Counters* ctr, void* scanTemp, cudaStream_t s);
// scratch ints of the colour scatter for a tick of n bodies
inline size_t color_scan_ints(size_t n) { return size_t(MAX_COLORS) * ((n + 255) / 256 + 1) + 1; }
// Per tick, before the counter readback: per-body manifold-contact item counts, their scan and
// the per-colour item totals. After the readback (with itemRef large enough): fill.
void launch_items_count(PairPtrs P, Tick t, Topo topo, Counters* ctr, void* scanTemp, cudaStream_t s);
void launch_items_fill(const BodyPtrs& b, const WorldDev* worlds, PairPtrs P, Tick t, Topo topo, const Counters* ctr,
                       cudaStream_t s);
// The tick's gate (TickCtl): after the items count, holds the tick when a world's pair region
// overflowed or the work items exceed itemCap.
void launch_tick_gate(Tick t, const Counters* ctr, long long itemCap, cudaStream_t s);

// Work-item code: contact index (3 bits), side (0: body A, 1: body B), whether this item runs the
// contact's dual update (the item of the body solved last in an iteration: the other body is
// static or has a lower colour; side 0 breaks a tie), and the world's iteration count (the solver
// kernels need no world lookup).
__host__ __device__ __forceinline__ int item_code(int contact, int side, bool dualOwner, int iterations) {
  return contact | (side << 3) | (dualOwner ? 16 : 0) | (iterations << 5);
}
__host__ __device__ __forceinline__ int item_contact(int code) { return code & 7; }
__host__ __device__ __forceinline__ int item_side(int code) { return (code >> 3) & 1; }
__host__ __device__ __forceinline__ bool item_dual_owner(int code) { return (code & 16) != 0; }
__host__ __device__ __forceinline__ int item_iterations(int code) { return code >> 5; }
// The solve loop of a tick (every iteration, colour and chunk, with the contact and joint duals
// fused) in one persistent launch, chosen at run time (the autotuner's candidates):
//   queue   tiles (iteration, colour, chunk) drained in order; a tile waits only for its own
//           worlds' earlier stages (k_solve_queue);
//   barrier colour by colour with a grid barrier between colours (k_solve_coop).
// Both give the same bits. sleepy: some stepped world has sleeping on (rows of sleeping bodies
// are skipped: nobody reads them).
struct SolveConfig {
  int queue = 1;                     // 1: tile queue, 0: barrier per colour
  int blocks = 0;                    // persistent blocks (0: every resident block)
  int waves = 2;                     // chunks per block and colour (chunk size = colour / (blocks * waves))
  int tile = 128;                    // work items per shared-memory tile: 128 (one per thread) or 256
  long long waitCycles = 4000000000LL;  // bound of one wait of the tile queue (SM cycles, ~2 s)
  int probe = 0;                     // tests: every wait past the first stage runs out (see k_solve_queue)
};
// ints of the tile queue's scratch for a world table of maxWorlds entries
size_t solve_queue_ints(int maxWorlds);
cudaError_t launch_solve(const BodyPtrs& b, const WorldDev* worlds, JointPtrs j, PairPtrs P, Tick t, Topo topo, const Counters* ctr,
                         int maxIter, int nBodies, bool sleepy, const SolveConfig& cfg, int* queueScratch, cudaStream_t s);
void launch_velocities(const BodyPtrs& b, const WorldDev* worlds, Tick t, cudaStream_t s);
// Contact events (FLAG_EVENTS worlds), per world: its event region, events written since the
// last read (may pass the capacity), the capacity, and the steps it has taken.
struct EventBufs {
  float4** region;
  int* count;
  int* cap;
  int* step;
};
void launch_events(const BodyPtrs& b, const WorldDev* worlds, PairPtrs P, Tick t, const Counters* ctr, int pairBudget,
                   EventBufs ev, cudaStream_t s);

// Shape casts (queries.cu): per query origin.xyz + maximum distance, unit direction.xyz +
// radius (0: a ray); the body filter of the query.
struct CastQuery {
  float4 o, d;
};
struct CastFilter {
  uint32_t collidesWith, membership;
  int hasMembership, nIgnore, includeTriggers;
  uint32_t ignore[16];
};
// nearest hit of each query among bodies [off, off + nb): out[2q] = (normal, distance or -1),
// out[2q + 1].x = body (local index, as bits); best: n 64-bit scratch words
void launch_cast(const BodyPtrs& b, int off, int nb, const CastQuery* qs, int n, const CastFilter& f,
                 unsigned long long* best, float4* out, cudaStream_t s);

// Slot of pair `key` in the sorted region [base, base + n) of a pair buffer, or -1.
__device__ __forceinline__ int find_pair(const uint2* __restrict__ pairs, int base, int n, uint2 key) {
  const unsigned long long k = (unsigned long long)key.x << 32 | key.y;
  pairs += base;
  int a = 0, b = n;
  while (a < b) {
    int m = (a + b) >> 1;
    uint2 p = pairs[m];
    unsigned long long pk = (unsigned long long)p.x << 32 | p.y;
    if (pk < k) a = m + 1;
    else b = m;
  }
  if (a < n) {
    uint2 p = pairs[a];
    if (p.x == key.x && p.y == key.y) return base + a;
  }
  return -1;
}

// Restitution (src/native/cpu/restitution.js): per active pair q the bounce state: ra (xyz,
// target speed), rb (xyz, accumulated impulse), nk (normal, effective mass k; k == 0: inactive),
// delta (this round's impulse change); incoming velocities per body.
struct BounceBufs {
  float4 *inVel, *inAng;
  float4 *ra, *rb, *nk;
  float* delta;
};
void launch_bounce_capture(const BodyPtrs& b, Tick t, BounceBufs bb, cudaStream_t s);
void launch_bounce(const BodyPtrs& b, PairPtrs P, Tick t, Topo topo, const Counters* ctr, int pairBudget, BounceBufs bb,
                   const WorldDev* worlds, cudaStream_t s);
// Island sleeping (sleep.cu): union-find parents and island flags per body, a wake flag per
// world, an error counter (union retries that ran out).
struct SleepBufs {
  int* parent;
  int* flags;
  int* wake;
  int* err;
};
void launch_sleep(const BodyPtrs& b, const WorldDev* worlds, JointPtrs J, PairPtrs P, NoCollide nc, Tick t,
                  const Counters* ctr, int pairBudget, SleepBufs sb, int maxWorlds, cudaStream_t s);
// wake every body of bodies [off, off + n): asleep cleared, quiet time 0
void launch_sleep_wake(const BodyPtrs& b, int off, int n, const TickCtl* ctl, cudaStream_t s);
// Body command records of one world (sorted by body, ranges per body; see k_apply_edits), and
// the warm-start drop of teleported bodies (sorted local indices) in its last pair region.
// Both do nothing while a tick is held (ctl); the world's last pair count is read from the device
// (*np, at most npMax).
void launch_apply_edits(const BodyPtrs& b, const uint32_t* rec, const int2* ranges, int nranges, int bodyOff, const TickCtl* ctl,
                        cudaStream_t s);
void launch_drop_contacts(PairPtrs P, size_t base, const int* np, int npMax, const uint32_t* tele, int ntele, int bodyOff,
                          const TickCtl* ctl, cudaStream_t s);
void launch_tick_end(Tick t, cudaStream_t s);
// Poses of listed worlds into rows of `out` (2 float4 per body); seg = (first body, bodies, first
// row, -) ascending by row. With ctl, nothing is written while a tick is held.
void launch_gather_poses(const BodyPtrs& b, const int4* seg, int nseg, int total, float4* out, const TickCtl* ctl, cudaStream_t s);
void launch_count_active(JointPtrs j, PairPtrs P, const int* slots, int nSlots, const int* joints, int nJoints, Counters* out,
                         cudaStream_t s);

// The LDL^T solve's shared-reciprocal division against the IEEE division: bad[0] += reciprocals that
// differ (every float of the range), bad[1] += quotients that differ (n seeded operand pairs).
cudaError_t launch_check_division(long long n, uint32_t seed, unsigned long long* bad);

// Algorithmic bytes of one tick's kernels from its live counts (the bytes each kernel must
// move at minimum; see launch_traffic): out3 = {primal per iteration, dual per iteration, collision}.
void launch_traffic(const BodyPtrs& b, JointPtrs j, PairPtrs P, Tick t, Topo topo, const Counters* ctr, int pairBudget,
                    unsigned long long* out3, cudaStream_t s);

}  // namespace avbd
