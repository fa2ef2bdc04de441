// Internal interface of the AVBD engine: device layouts shared by the kernel translation units
// and the host orchestration (engine.cu). Not part of the C ABI.
//
// Layout in HBM (structure of arrays, one float4 per field, all worlds of a set concatenated):
//   bodies   pos(xyz, bounding radius) rot  pos0(x-) rot0  posY(inertial) rotY
//            vel  ang  vprev  size(xyz, friction)  mass(m, Ix, Iy, Iz)  meta(world, shape, group, mask)
//   joints   body pair, rA(xyz, kind) rB(xyz, rest) stiff(lin, ang, fracture, torqueArm)
//            penLin penAng lamLin lamAng C0Lin C0Ang restQ, broken flag
//   pairs    (hi, lo) sorted ascending; per pair: contact count, basis rows n(w: friction), t1, t2,
//            and 8 contact slots of 4 float4: rA(xyz, feature|stick) rB(xyz, C0.n) pen(xyz, C0.t1)
//            lam(xyz, C0.t2). Two pair buffers (previous step, this step) swap every step.
//   topology per-body constraint lists (CSR), Jones-Plassmann colour state, colour buckets.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "avbd_math.cuh"

namespace avbd {

constexpr int MAX_CONTACTS = 8;
constexpr int MAX_COLORS = 64;
constexpr float PENALTY_MIN = 1.0f;
constexpr float PENALTY_MAX = 1e10f;
constexpr float COLLISION_MARGIN = 0.01f;
constexpr float STICK_THRESH = 0.00001f;
constexpr uint32_t STICK_BIT = 0x80000000u;
constexpr uint32_t JOINT_BIT = 0x80000000u;  // constraint-list entry is a joint id
constexpr int SHAPE_BOX = 0;
constexpr int SHAPE_SPHERE = 1;
constexpr int KIND_JOINT = 0;
constexpr int KIND_SPRING = 1;

constexpr int FLAG_MASS_PENALTY = 1;
constexpr int FLAG_FACE_BIAS = 2;

// Per-world parameters and ranges (80 bytes).
struct WorldDev {
  float dt, gravity, alpha, gamma;
  float betaLin, betaAng, cell, largeR;
  float up0, up1, up2;
  int iterations;
  int flags, bodyOff, bodyCount, largeOff;
  int largeCount, jointOff, jointCount, pad;
};

struct BodyPtrs {
  float4 *pos, *rot, *pos0, *rot0, *posY, *rotY, *vel, *ang, *vprev, *size, *mass;
  int4* meta;
};

struct JointPtrs {
  int2* ab;
  float4 *rA, *rB, *stiff, *penLin, *penAng, *lamLin, *lamAng, *C0Lin, *C0Ang, *restQ;
  int* broken;
};

struct PairPtrs {
  uint2* pair;     // (hi, lo)
  int* count;      // contacts (0: no manifold)
  float4* basis;   // 3 per pair
  float4* ct;      // 4 per contact slot, 8 slots per pair
};

// Device counters (one block of ints, reset each step where noted).
struct Counters {
  int npairs;      // candidate pairs written
  int pairsNeeded; // candidate pairs found (> capacity: overflow)
  int remaining;   // colouring: bodies still pending
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

struct Grid {
  uint32_t tableMask;  // hash table size - 1 (power of two)
  int* cellCount;      // table + 1 (scanned in place to starts)
  int* cellFill;
  int* cellBodies;     // small bodies bucketed
  int* bodyBucket;     // per body (-1: large)
  int* large;          // large bodies of each world, global ids, ascending
};

// Narrowphase scratch (per step): SAT results of overlapping box pairs, the queued pair lists
// and their counts (ctr[0] box hits, ctr[1] sphere pairs).
struct NarrowScratch {
  float4* sat;
  int* boxList;
  int* sphereList;
  int* ctr;
};

struct NoCollide {
  unsigned long long* keys;  // (hi << 32 | lo), sorted
  int* jid;                  // joint/spring id (broken ones stop blocking), -1 for ignore pairs
  int n;
};

struct Topo {
  int* adjStart;  // N + 1
  int* adjFill;   // N
  uint32_t* adjList;
  int* colorPrev;  // colour state carried from the previous step
  int* color;      // this step's colours
  int* won;        // round scratch
  unsigned char* pending;
  int* colorBodies;
  // manifold-contact work items of the dynamic bodies, bucket order (see launch_primal):
  int* itemStart;  // per bucket slot, N + 1 (exclusive scan of item counts)
  int2* itemRef;   // item -> (pair, contact | side << 3)
  float4* contrib; // per item of the current colour: 7 planes of `contribCap` float4
  int contribCap;
};

// ---------------------------------------------------------------- launchers
// scan.cu
size_t scan_temp_bytes(int n);
// exclusive scan of n ints in place; writes the total to *total (device) if non-null
void scan_exclusive(int* data, int n, int* total, void* temp, cudaStream_t s);

// collide.cu
void launch_grid_build(const BodyPtrs& b, const WorldDev* worlds, int nBodies, Grid g, void* scanTemp, cudaStream_t s);
void launch_pairs(const BodyPtrs& b, const WorldDev* worlds, int nBodies, Grid g, NoCollide nc, const int* jbroken,
                  int* pairCount, int* pairStart, uint2* pairsOut, int capacity, Counters* ctr, void* scanTemp,
                  cudaStream_t s);
void launch_narrowphase(const BodyPtrs& b, const WorldDev* worlds, PairPtrs cur, PairPtrs prev, const int* prevN,
                        const int* curN, int capacity, NarrowScratch ns, cudaStream_t s);

// solve.cu
void launch_joint_warmstart(const BodyPtrs& b, const WorldDev* worlds, JointPtrs j, int nJoints, Counters* ctr, cudaStream_t s);
void launch_body_warmstart(const BodyPtrs& b, const WorldDev* worlds, int nBodies, cudaStream_t s);
void launch_adjacency(const BodyPtrs& b, JointPtrs j, int nJoints, PairPtrs cur, const int* npairs, int capacity,
                      Topo t, int nBodies, void* scanTemp, cudaStream_t s);
void launch_coloring(const BodyPtrs& b, const WorldDev* worlds, JointPtrs j, PairPtrs cur, Topo t, int nBodies, int rounds,
                     Counters* ctr, cudaStream_t s);
// Per step, before the counter readback: per-body manifold-contact item counts, their scan and
// the per-colour item totals. After the readback (with itemRef/contrib large enough): fill.
void launch_items_count(PairPtrs cur, Topo t, int nBodies, Counters* ctr, void* scanTemp, cudaStream_t s);
void launch_items_fill(PairPtrs cur, Topo t, int nBodies, const Counters* ctr, cudaStream_t s);
void launch_primal(const BodyPtrs& b, const WorldDev* worlds, JointPtrs j, PairPtrs cur, Topo t, const Counters* ctr,
                   int color, int iteration, int nBodiesColor, int nItemsColor, cudaStream_t s);
void launch_dual(const BodyPtrs& b, const WorldDev* worlds, JointPtrs j, int nJoints, PairPtrs cur, const int* npairs,
                 int capacity, int iteration, cudaStream_t s);
void launch_velocities(const BodyPtrs& b, const WorldDev* worlds, int nBodies, cudaStream_t s);
void launch_count_active(JointPtrs j, int nJoints, PairPtrs cur, const int* npairs, int capacity, Counters* ctr, cudaStream_t s);

int grid_blocks(long long n, int threads);

// Kernel launches issued by this library (host counter, for the benchmark's launch count).
void note_launches(int n);
long long launches_total();

// Algorithmic bytes of one step's kernels, from the step's live counts (the bytes each kernel
// must move at minimum; see launch_traffic).
struct Traffic {
  unsigned long long primalPerIter;  // all colours of one iteration
  unsigned long long dualPerIter;
  unsigned long long collide;        // grid + pairs + narrowphase
};
void launch_traffic(const BodyPtrs& b, JointPtrs j, int nJoints, PairPtrs cur, const int* npairs, int capacity, Topo t,
                    int nBodies, unsigned long long* out3, cudaStream_t s);

}  // namespace avbd
