// AVBD CPU ORACLE -- test infrastructure only.
//
// A C++ restatement of babylon-avbd's CPU rigid-body path, used to check the CUDA engine.
// Nothing in the product links or calls this code: only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg load it, as the checker or as the timed CPU baseline.
//
// It follows, operation for operation (double precision reproduces the reference bit for bit
// where the reference is itself pinned):
//   reference/three-avbd/src/avbd3d/ref/math.ts      vector/quaternion/3x3 helpers, solve6
//   reference/three-avbd/src/avbd3d/ref/body.ts      Rigid, constants
//   reference/three-avbd/src/avbd3d/ref/manifold.ts  Manifold initialize/evaluate/primal/dual
//   reference/three-avbd/src/avbd3d/ref/forces.ts    Joint, Spring, IgnoreCollision
//   reference/three-avbd/src/avbd3d/ref/collide.ts   box-box SAT + clipping (pinned edge rule)
//   reference/three-avbd/src/avbd3d/ref/solver.ts    Solver.step (Z-up "ref" mode)
//   src/native/cpu/cpuSolver3D.ts:144-281            CpuSolver3D.step ("app" mode: up vector)
//   src/native/cpu/cpuPhysics3D.js:67-156,304-363    CpuManifold3D.initialize, cpuBroadphase3D
//   src/native/cpu/cpuBoxContacts3D.ts:409-499       collide() with the faceBias rule
//   src/native/cpu/cpuContacts3D.js:43-296           generic (sphere) narrowphase
//   reference/three-avbd/src/avbd3d/shapes.ts:28-36  sphere mass properties
//   reference/three-avbd/src/avbd2d/soa/coloring.ts  Jones-Plassmann colouring
//
// Parity of "ref" mode is pinned by the reference's 14 C++ golden trajectories
// (reference/three-avbd/tests/fixtures/oracle3d, copied to tests/golden/oracle3d). "app" mode
// extensions (up vector, grid broadphase, faceBias, massPenalty, spheres) have no golden
// vectors in the reference; they are restated from the cited source.
//
// Besides the faithful sequential newest-first Gauss-Seidel order, Solver::colored = true runs
// the primal in the GPU engine's order: Jones-Plassmann colours ascending, and each body's
// constraints stamped joints-first by id, then manifolds by the other body's index. This is
// the order the CUDA engine uses, so one step of both can be compared directly.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <tuple>
#include <unordered_map>
#include <vector>

namespace avbd_oracle {

constexpr double PENALTY_MIN = 1.0;
constexpr double PENALTY_MAX = 10000000000.0;
constexpr double COLLISION_MARGIN = 0.01;
constexpr double STICK_THRESH = 0.00001;

// ---------------------------------------------------------------- math.ts
template <class R> struct M {
  static R mn(R a, R b) { return a < b ? a : b; }
  static R mx(R a, R b) { return a > b ? a : b; }
  static R clamp(R x, R a, R b) { return mx(a, mn(b, x)); }
  static R sign(R x) { return x < 0 ? R(-1) : x > 0 ? R(1) : R(0); }
  static R dot(const R* a, const R* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
  static R lengthSq(const R* v) { return dot(v, v); }
  static R length(const R* v) { return std::sqrt(lengthSq(v)); }
  static void set3(R* o, R x, R y, R z) { o[0] = x; o[1] = y; o[2] = z; }
  static void add3(R* o, const R* a, const R* b) { set3(o, a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
  static void sub3(R* o, const R* a, const R* b) { set3(o, a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
  static void scale3(R* o, const R* a, R s) { set3(o, a[0] * s, a[1] * s, a[2] * s); }
  static void div3(R* o, const R* a, R s) { set3(o, a[0] / s, a[1] / s, a[2] / s); }
  static void neg3(R* o, const R* a) { set3(o, -a[0], -a[1], -a[2]); }
  static void abs3(R* o, const R* a) { set3(o, std::fabs(a[0]), std::fabs(a[1]), std::fabs(a[2])); }
  // out = a + b*s
  static void addScaled3(R* o, const R* a, const R* b, R s) { set3(o, a[0] + b[0] * s, a[1] + b[1] * s, a[2] + b[2] * s); }
  static void normalize3(R* o, const R* v) { div3(o, v, length(v)); }
  static void cross(R* o, const R* a, const R* b) {
    set3(o, a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
  }
  static void set4(R* o, R x, R y, R z, R w) { o[0] = x; o[1] = y; o[2] = z; o[3] = w; }
  static void qmul(R* o, const R* a, const R* b) {
    R ax = a[0], ay = a[1], az = a[2], aw = a[3];
    R bx = b[0], by = b[1], bz = b[2], bw = b[3];
    set4(o, aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
         aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz);
  }
  static void conjugate(R* o, const R* q) { set4(o, -q[0], -q[1], -q[2], q[3]); }
  static R qlengthSq(const R* q) { return lengthSq(q) + q[3] * q[3]; }
  static void qinverse(R* o, const R* q) {
    R l = qlengthSq(q);
    set4(o, -q[0] / l, -q[1] / l, -q[2] / l, q[3] / l);
  }
  static void qnormalize(R* o, const R* q) {
    R l = std::sqrt(qlengthSq(q));
    set4(o, q[0] / l, q[1] / l, q[2] / l, q[3] / l);
  }
  // rotation vector taking b to a: 2*vec(a * b^-1)
  static void qsub(R* o, const R* a, const R* b) {
    R inv[4], t[4];
    qinverse(inv, b);
    qmul(t, a, inv);
    set3(o, t[0] * 2, t[1] * 2, t[2] * 2);
  }
  // normalize(a + (b,0)*a*0.5)
  static void qaddv(R* o, const R* a, const R* b) {
    R t[4] = {b[0], b[1], b[2], 0};
    R s[4];
    qmul(s, t, a);
    R u[4] = {a[0] + s[0] * R(0.5), a[1] + s[1] * R(0.5), a[2] + s[2] * R(0.5), a[3] + s[3] * R(0.5)};
    qnormalize(o, u);
  }
  static void rotate(R* o, const R* q, const R* v) {
    R ux = q[0], uy = q[1], uz = q[2], w = q[3];
    R tx = (uy * v[2] - uz * v[1]) * 2;
    R ty = (uz * v[0] - ux * v[2]) * 2;
    R tz = (ux * v[1] - uy * v[0]) * 2;
    set3(o, v[0] + tx * w + (uy * tz - uz * ty), v[1] + ty * w + (uz * tx - ux * tz), v[2] + tz * w + (ux * ty - uy * tx));
  }
  static void transform(R* o, const R* p, const R* q, const R* v) {
    R t[3];
    rotate(t, q, v);
    add3(o, t, p);
  }
  static void rotateInv(R* o, const R* q, const R* v) {
    R c[4];
    conjugate(c, q);
    rotate(o, c, v);
  }
  // 3x3 row-major
  static void diagonal(R* o, R a, R b, R c) {
    for (int i = 0; i < 9; i++) o[i] = 0;
    o[0] = a; o[4] = b; o[8] = c;
  }
  static void skew(R* o, const R* r) {
    o[0] = 0; o[1] = -r[2]; o[2] = r[1];
    o[3] = r[2]; o[4] = 0; o[5] = -r[0];
    o[6] = -r[1]; o[7] = r[0]; o[8] = 0;
  }
  static void transpose(R* o, const R* a) {
    R t[9];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) t[i * 3 + j] = a[j * 3 + i];
    std::memcpy(o, t, sizeof(t));
  }
  static void mul(R* o, const R* a, const R* b) {
    R t[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) t[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
    std::memcpy(o, t, sizeof(t));
  }
  static void mulv(R* o, const R* a, const R* v) {
    R x = v[0], y = v[1], z = v[2];
    set3(o, a[0] * x + a[1] * y + a[2] * z, a[3] * x + a[4] * y + a[5] * z, a[6] * x + a[7] * y + a[8] * z);
  }
  static void addm(R* o, const R* a) { for (int i = 0; i < 9; i++) o[i] += a[i]; }
  static void scalem(R* o, const R* a, R s) { for (int i = 0; i < 9; i++) o[i] = a[i] * s; }
  static void negm(R* o, const R* a) { for (int i = 0; i < 9; i++) o[i] = -a[i]; }
  // rows b*a.x, b*a.y, b*a.z
  static void outer(R* o, const R* a, const R* b) {
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o[i * 3 + j] = b[j] * a[i];
  }
  static void diagonalize(R* o, const R* m) {
    R c0 = std::sqrt(m[0] * m[0] + m[3] * m[3] + m[6] * m[6]);
    R c1 = std::sqrt(m[1] * m[1] + m[4] * m[4] + m[7] * m[7]);
    R c2 = std::sqrt(m[2] * m[2] + m[5] * m[5] + m[8] * m[8]);
    diagonal(o, c0, c1, c2);
  }
  static void orthonormal(R* o, const R* n) {
    R t1[3];
    if (std::fabs(n[0]) > std::fabs(n[2])) set3(t1, -n[1], n[0], 0);
    else set3(t1, 0, -n[2], n[1]);
    normalize3(t1, t1);
    R t2[3];
    cross(t2, n, t1);
    o[0] = n[0]; o[1] = n[1]; o[2] = n[2];
    o[3] = t1[0]; o[4] = t1[1]; o[5] = t1[2];
    o[6] = t2[0]; o[7] = t2[1]; o[8] = t2[2];
  }
  // LDL^T of [aLin aCross^T; aCross aAng] (lower triangle), math.ts:227-285
  static void solve6(const R* aLin, const R* aAng, const R* aCross, const R* bLin, const R* bAng, R* xLin, R* xAng) {
    R A11 = aLin[0];
    R A21 = aLin[3], A22 = aLin[4];
    R A31 = aLin[6], A32 = aLin[7], A33 = aLin[8];
    R A41 = aCross[0], A42 = aCross[1], A43 = aCross[2], A44 = aAng[0];
    R A51 = aCross[3], A52 = aCross[4], A53 = aCross[5], A54 = aAng[3], A55 = aAng[4];
    R A61 = aCross[6], A62 = aCross[7], A63 = aCross[8], A64 = aAng[6], A65 = aAng[7], A66 = aAng[8];
    R L21 = A21 / A11, L31 = A31 / A11, L41 = A41 / A11, L51 = A51 / A11, L61 = A61 / A11;
    R D1 = A11;
    R D2 = A22 - L21 * L21 * D1;
    R L32 = (A32 - L21 * L31 * D1) / D2;
    R L42 = (A42 - L21 * L41 * D1) / D2;
    R L52 = (A52 - L21 * L51 * D1) / D2;
    R L62 = (A62 - L21 * L61 * D1) / D2;
    R D3 = A33 - (L31 * L31 * D1 + L32 * L32 * D2);
    R L43 = (A43 - L31 * L41 * D1 - L32 * L42 * D2) / D3;
    R L53 = (A53 - L31 * L51 * D1 - L32 * L52 * D2) / D3;
    R L63 = (A63 - L31 * L61 * D1 - L32 * L62 * D2) / D3;
    R D4 = A44 - (L41 * L41 * D1 + L42 * L42 * D2 + L43 * L43 * D3);
    R L54 = (A54 - L41 * L51 * D1 - L42 * L52 * D2 - L43 * L53 * D3) / D4;
    R L64 = (A64 - L41 * L61 * D1 - L42 * L62 * D2 - L43 * L63 * D3) / D4;
    R D5 = A55 - (L51 * L51 * D1 + L52 * L52 * D2 + L53 * L53 * D3 + L54 * L54 * D4);
    R L65 = (A65 - L51 * L61 * D1 - L52 * L62 * D2 - L53 * L63 * D3 - L54 * L64 * D4) / D5;
    R D6 = A66 - (L61 * L61 * D1 + L62 * L62 * D2 + L63 * L63 * D3 + L64 * L64 * D4 + L65 * L65 * D5);
    R y1 = bLin[0];
    R y2 = bLin[1] - L21 * y1;
    R y3 = bLin[2] - L31 * y1 - L32 * y2;
    R y4 = bAng[0] - L41 * y1 - L42 * y2 - L43 * y3;
    R y5 = bAng[1] - L51 * y1 - L52 * y2 - L53 * y3 - L54 * y4;
    R y6 = bAng[2] - L61 * y1 - L62 * y2 - L63 * y3 - L64 * y4 - L65 * y5;
    R z1 = y1 / D1, z2 = y2 / D2, z3 = y3 / D3, z4 = y4 / D4, z5 = y5 / D5, z6 = y6 / D6;
    xAng[2] = z6;
    xAng[1] = z5 - L65 * xAng[2];
    xAng[0] = z4 - L54 * xAng[1] - L64 * xAng[2];
    xLin[2] = z3 - L43 * xAng[0] - L53 * xAng[1] - L63 * xAng[2];
    xLin[1] = z2 - L32 * xLin[2] - L42 * xAng[0] - L52 * xAng[1] - L62 * xAng[2];
    xLin[0] = z1 - L21 * xLin[1] - L31 * xLin[2] - L41 * xAng[0] - L51 * xAng[1] - L61 * xAng[2];
  }
};

// SHAPE_CAPSULE: along local Y, size = (2r, height, 2r) (src/gpu/capsuleShape.js)
enum Shape : int { SHAPE_BOX = 0, SHAPE_SPHERE = 1, SHAPE_CAPSULE = 2 };
enum ForceType : int { F_MANIFOLD = 0, F_JOINT = 1, F_SPRING = 2, F_IGNORE = 3 };

template <class R> struct Body {
  R pos[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1};
  R x0[3] = {0, 0, 0}, q0[4] = {0, 0, 0, 1};
  R y[3] = {0, 0, 0}, qy[4] = {0, 0, 0, 1};
  R v[3] = {0, 0, 0}, w[3] = {0, 0, 0}, vprev[3] = {0, 0, 0};
  R size[3] = {1, 1, 1};
  R mass = 0, moment[3] = {0, 0, 0}, friction = 0, radius = 0, restitution = 0;
  int shape = SHAPE_BOX;
  bool sleeping = false, allowSleep = true;  // sleeping: skipped by the solve, as a static body
  bool isTrigger = false;  // contacts reported, no forces (cpuPhysics3D.js:148-156)
  uint32_t group = 0xffffffffu, mask = 0xffffffffu;
  std::vector<int> forces;  // force ids, in link order (newest last)
};

template <class R> struct Contact {
  uint32_t feature = 0;
  R rA[3] = {0, 0, 0}, rB[3] = {0, 0, 0};
  R C0[3] = {0, 0, 0}, pen[3] = {0, 0, 0}, lam[3] = {0, 0, 0};
  bool stick = false;
};

template <class R> struct Force {
  int type = F_MANIFOLD;
  int a = -1, b = -1;  // a = -1: world joint
  int jid = -1;        // creation order among joints and springs (the engine's joint id)
  // manifold
  std::vector<Contact<R>> contacts;
  R basis[9] = {0};
  R friction = 0;
  // joint / spring
  R rA[3] = {0, 0, 0}, rB[3] = {0, 0, 0};
  R C0Lin[3] = {0, 0, 0}, C0Ang[3] = {0, 0, 0};
  R penLin[3] = {0, 0, 0}, penAng[3] = {0, 0, 0}, lamLin[3] = {0, 0, 0}, lamAng[3] = {0, 0, 0};
  R stiffLin = std::numeric_limits<R>::infinity(), stiffAng = 0, fracture = std::numeric_limits<R>::infinity();
  R torqueArm = 0;
  bool broken = false;
  bool restFrame = false;  // app mode: angular rows relative to the captured rest rotation
  R restQ[4] = {0, 0, 0, 1};
  R rest = 0, stiffness = 0;  // spring
  // angular rows (src/gpu/angularConstraints.js): 3 motor, 4 limit, 0 none. rA / rB hold the axis
  // in A's / B's frame; p0, p1 the speed and torque bound (motor) or the lower and upper angle
  // (limit); ta, tb the reference tangents; c0 the rows' step-start values; penLin[0..1] and
  // lamLin[0..1] the rows' penalty and lambda.
  // spring fracture (src/gpu/springMaterial.js): strain and tension limits, infinite for none
  R breakStrain = std::numeric_limits<R>::infinity(), breakForce = std::numeric_limits<R>::infinity();
  int angular = 0;
  R p0 = 0, p1 = 0;
  R ta[3] = {0, 0, 0}, tb[3] = {0, 0, 0};
  R c0[2] = {0, 0};
};

struct RawContactD;  // fwd

// JP colouring (coloring.ts), shared by the colour-ordered step
inline uint32_t jp_priority(uint32_t i) {
  uint32_t x = i + 0x9e3779b9u;
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
inline bool jp_beats(uint32_t pi, int i, uint32_t pj, int j) { return pi > pj || (pi == pj && i > j); }
constexpr int MAX_COLORS = 64;

template <class R> class Solver {
 public:
  using Mt = M<R>;
  // parameters (defaults of solver.ts / cpuSolver3D.ts)
  R dt = R(1.0 / 60.0), gravity = -10;
  int iterations = 10;
  R alpha = R(0.99), betaLin = 10000, betaAng = 100, gamma = R(0.999);
  bool app = false;         // false: ref/solver.ts; true: cpuSolver3D.ts + cpuPhysics3D.js
  bool massPenalty = true;  // app only
  bool faceBias = true;     // app only
  R up[3] = {0, 0, 1};      // app only
  bool colored = false;     // GPU order (see header)
  int colorRounds = 64;
  // island sleeping (src/native/cpu/sleeping.js): off unless enabled
  bool sleepOn = false;
  R sleepSpeed = R(0.08), sleepDelay = R(0.6);
  std::vector<R> sleepTime;

  std::vector<Body<R>> bodies;
  std::vector<std::unique_ptr<Force<R>>> store;
  std::vector<int> forces;  // solver force list, creation order
  int nextJid = 0;

  // colouring state (persists across steps, as the GPU's)
  std::vector<int> colors;
  int lastNumColors = 0, lastConflicts = 0;

  int addBody(const Body<R>& b) {
    bodies.push_back(b);
    bodies.back().forces.clear();
    return int(bodies.size()) - 1;
  }
  int newForce(int type, int a, int b) {
    store.emplace_back(new Force<R>());
    int id = int(store.size()) - 1;
    Force<R>& f = *store[id];
    f.type = type;
    f.a = a;
    f.b = b;
    forces.push_back(id);
    if (a >= 0) bodies[a].forces.push_back(id);
    bodies[b].forces.push_back(id);
    if (type == F_JOINT || type == F_SPRING) f.jid = nextJid++;
    return id;
  }
  void unlinkFromBodies(int id) {
    Force<R>& f = *store[id];
    for (int body : {f.a, f.b}) {
      if (body < 0) continue;
      auto& l = bodies[body].forces;
      auto it = std::find(l.begin(), l.end(), id);
      if (it != l.end()) l.erase(it);
    }
  }
  // forces.ts:86-104
  int addJoint(int a, int b, const R* rA, const R* rB, R stiffLin, R stiffAng, R fracture) {
    int id = newForce(F_JOINT, a, b);
    Force<R>& f = *store[id];
    for (int i = 0; i < 3; i++) { f.rA[i] = rA[i]; f.rB[i] = rB[i]; }
    f.stiffLin = stiffLin;
    f.stiffAng = stiffAng;
    f.fracture = fracture;
    R s[3] = {0, 0, 0};
    if (a >= 0) for (int i = 0; i < 3; i++) s[i] = bodies[a].size[i];
    R t[3] = {s[0] + bodies[b].size[0], s[1] + bodies[b].size[1], s[2] + bodies[b].size[2]};
    f.torqueArm = Mt::lengthSq(t);
    return id;
  }
  // forces.ts:247-258
  int addSpring(int a, int b, const R* rA, const R* rB, R stiffness, R rest) {
    int id = newForce(F_SPRING, a, b);
    Force<R>& f = *store[id];
    for (int i = 0; i < 3; i++) { f.rA[i] = rA[i]; f.rB[i] = rB[i]; }
    f.stiffness = stiffness;
    f.rest = rest;
    if (f.rest < 0) {
      R pA[3], pB[3], d[3];
      Mt::transform(pA, bodies[a].pos, bodies[a].q, f.rA);
      Mt::transform(pB, bodies[b].pos, bodies[b].q, f.rB);
      Mt::sub3(d, pA, pB);
      f.rest = Mt::length(d);
    }
    return id;
  }
  int addIgnore(int a, int b) { return newForce(F_IGNORE, a, b); }
  // addMotor / the limit row of addHinge (scenes.js:575-630) as src/gpu/appGpuSolver3D.js:500-526
  // installs them: initial row penalties 1000, frames captured from the poses at creation.
  int addAngular(int a, int b, int kind, const R* axisA, const R* axisB, R p0, R p1) {
    int id = newForce(F_JOINT, a, b);
    Force<R>& f = *store[id];
    f.angular = kind;
    for (int i = 0; i < 3; i++) { f.rA[i] = axisA[i]; f.rB[i] = axisB[i]; }
    f.p0 = p0;
    f.p1 = p1;
    f.penLin[0] = f.penLin[1] = R(1000);
    angularCapture(f);
    return id;
  }

  // cpuPhysics3D.js:47-66 (captureCpuFrame3D) applied by prepareCpuForces3D to joints with
  // angular stiffness > 0: angular rows measure rotation relative to the captured rest frame.
  void prepareApp() {
    for (int id : forces) {
      Force<R>& f = *store[id];
      if (f.type == F_JOINT && f.stiffAng > 0) {
        R qa[4] = {0, 0, 0, 1};
        if (f.a >= 0) std::memcpy(qa, bodies[f.a].q, sizeof(qa));
        R inv[4];
        Mt::qinverse(inv, qa);
        Mt::qmul(f.restQ, inv, bodies[f.b].q);
        f.restFrame = true;
      }
    }
  }

  bool constrainedTo(int i, int j) const {
    for (int id : bodies[i].forces) {
      const Force<R>& f = *store[id];
      if ((f.a == i && f.b == j) || (f.a == j && f.b == i)) return true;
    }
    return false;
  }

  // ------------------------------------------------------------ joints (forces.ts)
  void jointEvalLin(const Force<R>& f, R* out) const {
    R pA[3], pB[3];
    if (f.a >= 0) Mt::transform(pA, bodies[f.a].pos, bodies[f.a].q, f.rA);
    else std::memcpy(pA, f.rA, sizeof(pA));
    Mt::transform(pB, bodies[f.b].pos, bodies[f.b].q, f.rB);
    Mt::sub3(out, pA, pB);
  }
  void jointEvalAng(const Force<R>& f, R* out) const {
    static const R IDENTITY[4] = {0, 0, 0, 1};
    const R* qa = f.a >= 0 ? bodies[f.a].q : IDENTITY;
    if (f.restFrame) {
      R target[4];
      Mt::qmul(target, qa, f.restQ);
      Mt::qsub(out, target, bodies[f.b].q);
      for (int i = 0; i < 3; i++) out[i] *= f.torqueArm;
    } else {
      Mt::qsub(out, qa, bodies[f.b].q);
      Mt::scale3(out, out, f.torqueArm);
    }
  }
  bool jointInitialize(Force<R>& f) {
    if (f.angular) return angularInitialize(f);
    jointEvalLin(f, f.C0Lin);
    jointEvalAng(f, f.C0Ang);
    for (int i = 0; i < 3; i++) {
      f.lamLin[i] = f.lamLin[i] * alpha * gamma;
      f.lamAng[i] = f.lamAng[i] * alpha * gamma;
      f.penLin[i] = Mt::clamp(f.penLin[i] * gamma, R(PENALTY_MIN), R(PENALTY_MAX));
      f.penAng[i] = Mt::clamp(f.penAng[i] * gamma, R(PENALTY_MIN), R(PENALTY_MAX));
    }
    for (int i = 0; i < 3; i++) f.penLin[i] = Mt::mn(f.penLin[i], f.stiffLin);
    for (int i = 0; i < 3; i++) f.penAng[i] = Mt::mn(f.penAng[i], f.stiffAng);
    return !f.broken;
  }
  static void geometricStiffnessBallSocket(R* out, int k, const R* v) {
    Mt::diagonal(out, -v[k], -v[k], -v[k]);
    out[k] += v[0];
    out[3 + k] += v[1];
    out[6 + k] += v[2];
  }
  struct Sys { R lhsLin[9], lhsAng[9], lhsCross[9], rhsLin[3], rhsAng[3]; };
  static bool isInf(R x) { return std::isinf(x) && x > 0; }

  void jointPrimal(const Force<R>& f, int body, Sys& sys) const {
    if (f.angular) {
      angularPrimal(f, body, sys);
      return;
    }
    const bool isA = body == f.a;
    R K[9], C[3], F[3], r[3], jLin[9], jAng[9], jLinT[9], jAngT[9], jAngTk[9], tmp[9], H[9], gs[9];
    if (Mt::lengthSq(f.penLin) > 0) {
      Mt::diagonal(K, f.penLin[0], f.penLin[1], f.penLin[2]);
      jointEvalLin(f, C);
      if (isInf(f.stiffLin)) Mt::addScaled3(C, C, f.C0Lin, -alpha);
      Mt::mulv(F, K, C);
      Mt::addScaled3(F, F, f.lamLin, 1);
      R sgn = isA ? 1 : -1;
      Mt::diagonal(jLin, sgn, sgn, sgn);
      if (isA) {
        Mt::rotate(r, bodies[f.a].q, f.rA);
        Mt::neg3(r, r);
        Mt::skew(jAng, r);
      } else {
        Mt::rotate(r, bodies[f.b].q, f.rB);
        Mt::skew(jAng, r);
      }
      Mt::transpose(jLinT, jLin);
      Mt::transpose(jAngT, jAng);
      Mt::mul(jAngTk, jAngT, K);
      Mt::mul(tmp, jLinT, K);
      Mt::mul(tmp, tmp, jLin);
      Mt::addm(sys.lhsLin, tmp);
      Mt::mul(tmp, jAngTk, jAng);
      Mt::addm(sys.lhsAng, tmp);
      Mt::mul(tmp, jAngTk, jLin);
      Mt::addm(sys.lhsCross, tmp);
      if (isA) Mt::rotate(r, bodies[f.a].q, f.rA);
      else {
        Mt::rotate(r, bodies[f.b].q, f.rB);
        Mt::neg3(r, r);
      }
      geometricStiffnessBallSocket(gs, 0, r);
      Mt::scalem(H, gs, F[0]);
      geometricStiffnessBallSocket(gs, 1, r);
      Mt::scalem(gs, gs, F[1]);
      Mt::addm(H, gs);
      geometricStiffnessBallSocket(gs, 2, r);
      Mt::scalem(gs, gs, F[2]);
      Mt::addm(H, gs);
      Mt::diagonalize(tmp, H);
      Mt::addm(sys.lhsAng, tmp);
      Mt::mulv(r, jLinT, F);
      Mt::addScaled3(sys.rhsLin, sys.rhsLin, r, 1);
      Mt::mulv(r, jAngT, F);
      Mt::addScaled3(sys.rhsAng, sys.rhsAng, r, 1);
    }
    if (Mt::lengthSq(f.penAng) > 0) {
      Mt::diagonal(K, f.penAng[0], f.penAng[1], f.penAng[2]);
      jointEvalAng(f, C);
      if (isInf(f.stiffAng)) Mt::addScaled3(C, C, f.C0Ang, -alpha);
      Mt::mulv(F, K, C);
      Mt::addScaled3(F, F, f.lamAng, 1);
      R s = (isA ? R(1) : R(-1)) * f.torqueArm;
      Mt::diagonal(jAng, s, s, s);
      Mt::transpose(jAngT, jAng);
      Mt::mul(tmp, jAngT, K);
      Mt::mul(tmp, tmp, jAng);
      Mt::addm(sys.lhsAng, tmp);
      Mt::mulv(r, jAngT, F);
      Mt::addScaled3(sys.rhsAng, sys.rhsAng, r, 1);
    }
  }
  void jointDual(Force<R>& f) {
    if (f.angular) {
      angularDual(f);
      return;
    }
    R K[9], C[3], F[3], r[3];
    if (Mt::lengthSq(f.penLin) > 0) {
      Mt::diagonal(K, f.penLin[0], f.penLin[1], f.penLin[2]);
      jointEvalLin(f, C);
      if (isInf(f.stiffLin)) {
        Mt::addScaled3(C, C, f.C0Lin, -alpha);
        Mt::mulv(F, K, C);
        Mt::addScaled3(f.lamLin, F, f.lamLin, 1);
      }
      Mt::abs3(r, C);
      Mt::addScaled3(f.penLin, f.penLin, r, betaLin);
      R cap = Mt::mn(f.stiffLin, R(PENALTY_MAX));
      for (int i = 0; i < 3; i++) f.penLin[i] = Mt::mn(f.penLin[i], cap);
    }
    if (Mt::lengthSq(f.penAng) > 0) {
      Mt::diagonal(K, f.penAng[0], f.penAng[1], f.penAng[2]);
      jointEvalAng(f, C);
      if (isInf(f.stiffAng)) {
        Mt::addScaled3(C, C, f.C0Ang, -alpha);
        Mt::mulv(F, K, C);
        Mt::addScaled3(f.lamAng, F, f.lamAng, 1);
      }
      Mt::abs3(r, C);
      Mt::addScaled3(f.penAng, f.penAng, r, betaAng);
      R cap = Mt::mn(f.stiffAng, R(PENALTY_MAX));
      for (int i = 0; i < 3; i++) f.penAng[i] = Mt::mn(f.penAng[i], cap);
    }
    if (Mt::lengthSq(f.lamAng) > f.fracture * f.fracture) {
      for (int i = 0; i < 3; i++) f.penLin[i] = f.penAng[i] = f.lamLin[i] = f.lamAng[i] = 0;
      f.broken = true;
    }
  }
  // setMotor (src/native/cpu/world.js:360-388) of the motor with joint id `jid`; mask bit 0:
  // speed, bit 1: torque bound. Returns false when jid is not a motor.
  bool setMotor(int jid, int mask, R speed, R torque) {
    for (auto& p : store) {
      Force<R>& f = *p;
      if (f.jid != jid || f.angular != 3) continue;
      if (mask & 1) f.p0 = speed;
      if (mask & 2) f.p1 = torque;
      return true;
    }
    return false;
  }
  // releaseJoints (src/native/cpu/world.js:397-410): the constraint with joint id `jid` stops
  // acting at once (broken, state zeroed, gone from the body and solver lists).
  void releaseJoint(int jid) {
    for (size_t id = 0; id < store.size(); id++) {
      Force<R>& f = *store[id];
      if (f.jid != jid || f.broken) continue;
      f.broken = true;
      for (int i = 0; i < 3; i++) f.penLin[i] = f.penAng[i] = f.lamLin[i] = f.lamAng[i] = 0;
      unlinkFromBodies(int(id));
      forces.erase(std::remove(forces.begin(), forces.end(), int(id)), forces.end());
    }
  }
  // ------------------------------------------------------------ angular rows
  // (src/gpu/angularConstraints.js:16-64, frames of src/gpu/angularFrames.wgsl)
  // atan2 from the half-angle identity atan(t) = 2 atan(t / (1 + sqrt(1 + t^2))) applied twice
  // (|t| <= tan(pi/16) after it) and the odd Taylor series of atan through t^9; +, -, *, / and
  // sqrt only, so the float instance repeats the engine's bits.
  static R angleAtan2(R y, R x) {
    const R ax = std::fabs(x), ay = std::fabs(y);
    const R hi = Mt::mx(ax, ay), lo = Mt::mn(ax, ay);
    if (!(hi > 0)) return 0;
    const R one = 1, t = lo / hi;
    const R u = t / (one + std::sqrt(one + t * t));
    const R v = u / (one + std::sqrt(one + u * u));
    const R w = v * v;
    const R s = v * (one + w * (R(-1) / R(3) + w * (R(1) / R(5) + w * (R(-1) / R(7) + w * (R(1) / R(9))))));
    R a = R(4) * s;
    if (ay > ax) a = R(1.57079632679489661923) - a;
    if (x < 0) a = R(3.14159265358979323846) - a;
    return y < 0 ? -a : a;
  }
  // atan2(sin d, cos d) for d in [-2 pi, 2 pi]
  static R angleWrap(R d) {
    const R pi = R(3.14159265358979323846), twoPi = R(6.28318530717958647692);
    return d > pi ? d - twoPi : (d < -pi ? d + twoPi : d);
  }
  static void angleTangent(R* o, const R* n) {
    R t[3];
    if (std::fabs(n[0]) > std::fabs(n[2])) Mt::set3(t, -n[1], n[0], 0);
    else Mt::set3(t, 0, -n[2], n[1]);
    Mt::div3(o, t, Mt::length(t));
  }
  const R* rotOfA(const Force<R>& f) const {
    static const R IDENTITY[4] = {0, 0, 0, 1};
    return f.a >= 0 ? bodies[f.a].q : IDENTITY;
  }
  void angularCapture(Force<R>& f) {
    angleTangent(f.ta, f.rA);
    R world[3], nb[3], t[3], p[3];
    Mt::rotate(world, rotOfA(f), f.ta);
    Mt::div3(nb, f.rB, Mt::length(f.rB));
    Mt::rotateInv(t, bodies[f.b].q, world);
    Mt::scale3(p, nb, Mt::dot(t, nb));
    Mt::sub3(t, t, p);
    if (Mt::length(t) < R(1.0e-6)) {
      if (std::fabs(nb[0]) > std::fabs(nb[2])) Mt::set3(t, -nb[1], nb[0], 0);
      else Mt::set3(t, 0, -nb[2], nb[1]);
    }
    Mt::div3(f.tb, t, Mt::length(t));
  }
  R angularAngle(const Force<R>& f, R* axis) const {
    const R* qa = rotOfA(f);
    R wa[3], wb[3], c[3];
    Mt::rotate(axis, qa, f.rA);
    Mt::rotate(wa, qa, f.ta);
    Mt::rotate(wb, bodies[f.b].q, f.tb);
    Mt::cross(c, wa, wb);
    return angleAtan2(Mt::dot(axis, c), Mt::dot(wa, wb));
  }
  void angularRows(const Force<R>& f, R angle, R* C) const {
    if (f.angular == 3) {
      C[0] = angleWrap(angle - f.c0[0]) - f.p0 * dt;
      C[1] = 0;
    } else {
      C[0] = (angle - f.p0) - alpha * f.c0[0];
      C[1] = (angle - f.p1) - alpha * f.c0[1];
    }
  }
  void angularForce(const Force<R>& f, const R* C, R* F) const {
    const R fx = f.penLin[0] * C[0] + f.lamLin[0], fy = f.penLin[1] * C[1] + f.lamLin[1];
    if (f.angular == 3) {
      F[0] = Mt::clamp(fx, -f.p1, f.p1);
      F[1] = 0;
    } else {
      F[0] = Mt::mn(R(0), fx);
      F[1] = Mt::mx(R(0), fy);
    }
  }
  bool angularInitialize(Force<R>& f) {
    R axis[3];
    const R angle = angularAngle(f, axis);
    const bool motor = f.angular == 3;
    f.c0[0] = motor ? angle : Mt::mn(R(0), angle - f.p0);
    f.c0[1] = motor ? R(0) : Mt::mx(R(0), angle - f.p1);
    const R decay = alpha * gamma;
    for (int i = 0; i < 2; i++) {
      f.lamLin[i] = f.lamLin[i] * decay;
      f.penLin[i] = Mt::clamp(f.penLin[i] * gamma, R(PENALTY_MIN), R(PENALTY_MAX));
    }
    return !f.broken;
  }
  void angularPrimal(const Force<R>& f, int body, Sys& sys) const {
    const bool motor = f.angular == 3;
    if (motor && f.p1 == 0) return;
    R axis[3], C[2], F[2];
    const R angle = angularAngle(f, axis);
    angularRows(f, angle, C);
    angularForce(f, C, F);
    if (body == f.a) Mt::neg3(axis, axis);
    for (int r = 0; r < 2; r++) {
      const bool on = r == 0 ? (motor || F[0] != 0) : (!motor && F[1] != 0);
      if (!on) continue;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) sys.lhsAng[i * 3 + j] += (axis[i] * axis[j]) * f.penLin[r];
      for (int i = 0; i < 3; i++) sys.rhsAng[i] += axis[i] * F[r];
    }
  }
  void angularDual(Force<R>& f) {
    const bool motor = f.angular == 3;
    R axis[3], C[2], F[2];
    const R angle = angularAngle(f, axis);
    angularRows(f, angle, C);
    angularForce(f, C, F);
    f.lamLin[0] = F[0];
    f.lamLin[1] = F[1];
    const R vx = motor ? std::fabs(C[0]) : Mt::mx(R(0), -C[0]), vy = motor ? std::fabs(C[1]) : Mt::mx(R(0), C[1]);
    f.penLin[0] = Mt::mn(f.penLin[0] + vx * betaAng, R(PENALTY_MAX));
    f.penLin[1] = Mt::mn(f.penLin[1] + vy * betaAng, R(PENALTY_MAX));
  }
  // ------------------------------------------------------------ springs (forces.ts:260-296)
  // Tensile fracture at the step start (cpuPhysics3D.js:276-299): a spring stretched past its
  // strain or tension limit tears for good.
  bool springInitialize(Force<R>& f) {
    if (f.broken) return false;
    if (f.breakStrain < std::numeric_limits<R>::infinity() || f.breakForce < std::numeric_limits<R>::infinity()) {
      R pA[3], pB[3], d[3];
      Mt::transform(pA, bodies[f.a].pos, bodies[f.a].q, f.rA);
      Mt::transform(pB, bodies[f.b].pos, bodies[f.b].q, f.rB);
      Mt::sub3(d, pA, pB);
      const R ext = Mt::mx(R(0), Mt::length(d) - f.rest);
      if (ext / Mt::mx(f.rest, R(1.0e-6)) > f.breakStrain || ext * f.stiffness > f.breakForce) {
        f.broken = true;
        return false;
      }
    }
    return true;
  }
  // setSpringMaterial / setWorldAnchor / captureConstraintFrames by joint id (world.js:474-501,
  // appGpuSolver3D.js:810-841). Each returns false when jid is not a live constraint of that kind.
  Force<R>* liveJid(int jid) {
    for (auto& p : store)
      if (p->jid == jid && !p->broken) return p.get();
    return nullptr;
  }
  bool setSpringMaterial(int jid, int mask, R strain, R force) {
    Force<R>* f = liveJid(jid);
    if (!f || f->type != F_SPRING) return false;
    if (mask & 1) f->breakStrain = strain;
    if (mask & 2) f->breakForce = force;
    return true;
  }
  bool setWorldAnchor(int jid, const R* point) {
    Force<R>* f = liveJid(jid);
    if (!f || f->type != F_JOINT || f->angular || f->a >= 0) return false;
    for (int i = 0; i < 3; i++) f->rA[i] = point[i];
    return true;
  }
  bool captureFrame(int jid, bool spring) {
    Force<R>* f = liveJid(jid);
    if (!f || f->angular || f->type != (spring ? F_SPRING : F_JOINT)) return false;
    if (spring) {
      R pA[3], pB[3], d[3];
      Mt::transform(pA, bodies[f->a].pos, bodies[f->a].q, f->rA);
      Mt::transform(pB, bodies[f->b].pos, bodies[f->b].q, f->rB);
      Mt::sub3(d, pA, pB);
      f->rest = Mt::length(d);
    } else {
      static const R IDENTITY[4] = {0, 0, 0, 1};
      R inv[4];
      Mt::qinverse(inv, f->a >= 0 ? bodies[f->a].q : IDENTITY);
      Mt::qmul(f->restQ, inv, bodies[f->b].q);
    }
    return true;
  }
  void springPrimal(const Force<R>& f, int body, Sys& sys) const {
    const Body<R>& A = bodies[f.a];
    const Body<R>& B = bodies[f.b];
    R pA[3], pB[3], d[3], n[3], r[3], jl[3], ja[3], tmp[9];
    Mt::transform(pA, A.pos, A.q, f.rA);
    Mt::transform(pB, B.pos, B.q, f.rB);
    Mt::sub3(d, pA, pB);
    R dLen = Mt::length(d);
    if (dLen <= R(1.0e-6)) return;
    Mt::div3(n, d, dLen);
    R c = dLen - f.rest;
    R fo = f.stiffness * c;
    if (body == f.a) {
      Mt::rotate(r, A.q, f.rA);
      std::memcpy(jl, n, sizeof(jl));
      Mt::cross(ja, r, n);
    } else {
      Mt::rotate(r, B.q, f.rB);
      Mt::neg3(jl, n);
      Mt::cross(ja, r, n);
      Mt::neg3(ja, ja);
    }
    Mt::outer(tmp, jl, jl); Mt::scalem(tmp, tmp, f.stiffness); Mt::addm(sys.lhsLin, tmp);
    Mt::outer(tmp, ja, ja); Mt::scalem(tmp, tmp, f.stiffness); Mt::addm(sys.lhsAng, tmp);
    Mt::outer(tmp, ja, jl); Mt::scalem(tmp, tmp, f.stiffness); Mt::addm(sys.lhsCross, tmp);
    Mt::scale3(r, jl, fo); Mt::addScaled3(sys.rhsLin, sys.rhsLin, r, 1);
    Mt::scale3(r, ja, fo); Mt::addScaled3(sys.rhsAng, sys.rhsAng, r, 1);
  }

  // ------------------------------------------------------------ manifolds (manifold.ts)
  struct Eval { R jBLin[9], jAAng[9], jBAng[9], K[9], C[3], F[3], frictionScale, bounds; };
  struct Disp { R dqALin[3], dqAAng[3], dqBLin[3], dqBAng[3]; };
  static void angularJacobian(R* out, const R* r, const R* lin) {
    for (int k = 0; k < 3; k++) {
      R row[3] = {lin[k * 3], lin[k * 3 + 1], lin[k * 3 + 2]};
      R c[3];
      Mt::cross(c, r, row);
      out[k * 3] = c[0]; out[k * 3 + 1] = c[1]; out[k * 3 + 2] = c[2];
    }
  }
  void computeDisplacements(const Force<R>& f, Disp& d) const {
    const Body<R>& A = bodies[f.a];
    const Body<R>& B = bodies[f.b];
    Mt::sub3(d.dqALin, A.pos, A.x0);
    Mt::qsub(d.dqAAng, A.q, A.q0);
    Mt::sub3(d.dqBLin, B.pos, B.x0);
    Mt::qsub(d.dqBAng, B.q, B.q0);
  }
  void evaluate(const Force<R>& f, const Contact<R>& c, const Disp& d, Eval& e) const {
    const Body<R>& A = bodies[f.a];
    const Body<R>& B = bodies[f.b];
    R rAW[3], rBW[3], v[3];
    Mt::rotate(rAW, A.q, c.rA);
    Mt::rotate(rBW, B.q, c.rB);
    Mt::negm(e.jBLin, f.basis);
    angularJacobian(e.jAAng, rAW, f.basis);
    angularJacobian(e.jBAng, rBW, e.jBLin);
    Mt::diagonal(e.K, c.pen[0], c.pen[1], c.pen[2]);
    Mt::scale3(e.C, c.C0, 1 - alpha);
    Mt::mulv(v, f.basis, d.dqALin); Mt::addScaled3(e.C, e.C, v, 1);
    Mt::mulv(v, e.jBLin, d.dqBLin); Mt::addScaled3(e.C, e.C, v, 1);
    Mt::mulv(v, e.jAAng, d.dqAAng); Mt::addScaled3(e.C, e.C, v, 1);
    Mt::mulv(v, e.jBAng, d.dqBAng); Mt::addScaled3(e.C, e.C, v, 1);
    Mt::mulv(e.F, e.K, e.C);
    Mt::addScaled3(e.F, e.F, c.lam, 1);
    e.F[0] = Mt::mn(e.F[0], R(0));
    e.bounds = std::fabs(e.F[0]) * f.friction;
    e.frictionScale = std::sqrt(e.F[1] * e.F[1] + e.F[2] * e.F[2]);
    if (e.frictionScale > e.bounds && e.frictionScale > 0) {
      e.F[1] *= e.bounds / e.frictionScale;
      e.F[2] *= e.bounds / e.frictionScale;
    }
  }
  void manifoldPrimal(const Force<R>& f, int body, Sys& sys) const {
    if (triggerForce(f)) return;
    Disp d;
    computeDisplacements(f, d);
    const bool isA = body == f.a;
    Eval e;
    R jLinT[9], jAngT[9], jAngTk[9], tmp[9], v[3];
    for (const Contact<R>& c : f.contacts) {
      evaluate(f, c, d, e);
      const R* jLin = isA ? f.basis : e.jBLin;
      const R* jAng = isA ? e.jAAng : e.jBAng;
      Mt::transpose(jLinT, jLin);
      Mt::transpose(jAngT, jAng);
      Mt::mul(jAngTk, jAngT, e.K);
      Mt::mul(tmp, jLinT, e.K);
      Mt::mul(tmp, tmp, jLin);
      Mt::addm(sys.lhsLin, tmp);
      Mt::mul(tmp, jAngTk, jAng);
      Mt::addm(sys.lhsAng, tmp);
      Mt::mul(tmp, jAngTk, jLin);
      Mt::addm(sys.lhsCross, tmp);
      Mt::mulv(v, jLinT, e.F); Mt::addScaled3(sys.rhsLin, sys.rhsLin, v, 1);
      Mt::mulv(v, jAngT, e.F); Mt::addScaled3(sys.rhsAng, sys.rhsAng, v, 1);
    }
  }
  void manifoldDual(Force<R>& f) {
    if (triggerForce(f)) return;
    Disp d;
    computeDisplacements(f, d);
    Eval e;
    for (Contact<R>& c : f.contacts) {
      evaluate(f, c, d, e);
      std::memcpy(c.lam, e.F, sizeof(c.lam));
      if (e.F[0] < 0) c.pen[0] = Mt::mn(c.pen[0] + betaLin * std::fabs(e.C[0]), R(PENALTY_MAX));
      if (e.frictionScale <= e.bounds) {
        c.pen[1] = Mt::mn(c.pen[1] + betaLin * std::fabs(e.C[1]), R(PENALTY_MAX));
        c.pen[2] = Mt::mn(c.pen[2] + betaLin * std::fabs(e.C[2]), R(PENALTY_MAX));
        c.stick = std::sqrt(e.C[1] * e.C[1] + e.C[2] * e.C[2]) < R(STICK_THRESH);
      }
    }
  }

  // ------------------------------------------------------------ narrowphase
  struct Raw { uint32_t feature; R rA[3], rB[3]; };
  std::vector<Raw> collide(int ia, int ib, R* basis) const;         // box-box (collide.ts)
  std::vector<Raw> collideGeneric(int ia, int ib, R* basis) const;  // cpuContacts3D.js
  std::vector<Raw> narrowphase(int ia, int ib, R* basis) const {
    if (!app || (bodies[ia].shape == SHAPE_BOX && bodies[ib].shape == SHAPE_BOX)) return collide(ia, ib, basis);
    return collideGeneric(ia, ib, basis);
  }

  // manifold.ts:95-133 (ref) and cpuPhysics3D.js:68-147 (app)
  bool manifoldInitialize(Force<R>& f) {
    const Body<R>& A = bodies[f.a];
    const Body<R>& B = bodies[f.b];
    if (app && (!(A.group & B.mask) || !(B.group & A.mask))) return false;
    // spheres and capsules roll (cpuPhysics3D.js:77): their anchors are not kept while sticking
    const bool rolling = app && (A.shape != SHAPE_BOX || B.shape != SHAPE_BOX);
    f.friction = std::sqrt(A.friction * B.friction);
    std::vector<Contact<R>> old;
    old.swap(f.contacts);
    std::vector<Raw> raw = narrowphase(f.a, f.b, f.basis);
    for (const Raw& rc : raw) {
      const Contact<R>* prev = nullptr;
      for (const Contact<R>& o : old)
        if (o.feature == rc.feature) { prev = &o; break; }
      Contact<R> c;
      c.feature = rc.feature;
      const bool keep = prev && prev->stick && !rolling;
      std::memcpy(c.rA, keep ? prev->rA : rc.rA, sizeof(c.rA));
      std::memcpy(c.rB, keep ? prev->rB : rc.rB, sizeof(c.rB));
      if (prev) {
        std::memcpy(c.pen, prev->pen, sizeof(c.pen));
        std::memcpy(c.lam, prev->lam, sizeof(c.lam));
        c.stick = prev->stick;
      }
      f.contacts.push_back(c);
    }
    for (Contact<R>& c : f.contacts) {
      R xA[3], xB[3], v[3];
      Mt::transform(xA, A.pos, A.q, c.rA);
      Mt::transform(xB, B.pos, B.q, c.rB);
      Mt::sub3(v, xA, xB);
      Mt::mulv(c.C0, f.basis, v);
      c.C0[0] += R(COLLISION_MARGIN);
      for (int i = 0; i < 3; i++) {
        if (app) c.lam[i] *= alpha * gamma;
        else c.lam[i] = c.lam[i] * alpha * gamma;
        c.pen[i] = Mt::clamp(c.pen[i] * gamma, R(PENALTY_MIN), R(PENALTY_MAX));
      }
      if (app && massPenalty) {
        R inf = std::numeric_limits<R>::infinity();
        R mass = Mt::mn(A.mass > 0 ? A.mass : inf, B.mass > 0 ? B.mass : inf);
        // Math.max/min with clamp(mass / dt ** 2, PENALTY_MIN, PENALTY_MAX)
        R floorPen = std::max(R(PENALTY_MIN), std::min(R(PENALTY_MAX), mass / (dt * dt)));
        c.pen[0] = std::max(c.pen[0], floorPen);
      }
    }
    return !f.contacts.empty();
  }

  // ------------------------------------------------------------ broadphase
  void broadphaseRef() {  // solver.ts:443-452
    const int n = int(bodies.size());
    for (int i = n - 1; i >= 0; i--) {
      for (int j = i - 1; j >= 0; j--) {
        R dp[3];
        Mt::sub3(dp, bodies[i].pos, bodies[j].pos);
        R r = bodies[i].radius + bodies[j].radius;
        if (Mt::dot(dp, dp) <= r * r && !constrainedTo(i, j)) newForce(F_MANIFOLD, i, j);
      }
    }
  }
  // cpuPhysics3D.js:304-363
  void broadphaseApp() {
    const int n = int(bodies.size());
    std::vector<double> radii;
    for (int i = 0; i < n && int(radii.size()) < 1024; i++)
      if (bodies[i].mass > 0) radii.push_back(double(bodies[i].radius));
    std::sort(radii.begin(), radii.end());
    double med = radii.empty() ? 1.0 : radii[radii.size() / 2];
    double cell = std::max(0.1, med * 2);
    struct KeyHash {
      size_t operator()(const std::tuple<long long, long long, long long>& k) const {
        return size_t(std::get<0>(k) * 73856093LL) ^ size_t(std::get<1>(k) * 19349663LL) ^ size_t(std::get<2>(k) * 83492791LL);
      }
    };
    std::unordered_map<std::tuple<long long, long long, long long>, std::vector<int>, KeyHash> bins;
    std::vector<int> large;
    std::vector<uint64_t> seenv;
    std::unordered_map<uint64_t, char> seen;
    auto pair = [&](int a, int b) {
      if (a == b || (bodies[a].mass <= 0 && bodies[b].mass <= 0)) return;
      int hi = std::max(a, b), lo = std::min(a, b);
      uint64_t key = uint64_t(hi) * uint64_t(n) + uint64_t(lo);
      if (seen.count(key)) return;
      seen[key] = 1;
      const Body<R>& A = bodies[hi];
      const Body<R>& B = bodies[lo];
      if (!(A.group & B.mask) || !(B.group & A.mask)) return;
      R r = A.radius + B.radius;
      R d[3];
      Mt::sub3(d, A.pos, B.pos);
      if (Mt::dot(d, d) <= r * r && !constrainedTo(hi, lo)) newForce(F_MANIFOLD, hi, lo);
    };
    for (int i = 0; i < n; i++) {
      const Body<R>& b = bodies[i];
      long long lo[3], hi[3];
      for (int k = 0; k < 3; k++) {
        lo[k] = (long long)std::floor((double(b.pos[k]) - double(b.radius)) / cell);
        hi[k] = (long long)std::floor((double(b.pos[k]) + double(b.radius)) / cell);
      }
      if ((hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) > 128) {
        large.push_back(i);
        continue;
      }
      for (long long x = lo[0]; x <= hi[0]; x++)
        for (long long y = lo[1]; y <= hi[1]; y++)
          for (long long z = lo[2]; z <= hi[2]; z++) {
            auto& list = bins[std::make_tuple(x, y, z)];
            for (int j : list) pair(i, j);
            list.push_back(i);
          }
    }
    // The reference pairs every large body with all n bodies in ascending order. Only bodies
    // whose bounding spheres can overlap matter (pair() creates nothing for the others, and
    // skipping a pair that cannot overlap leaves `seen` without effect), so the candidates come
    // from a coarse grid of bodies up to radius R0 plus an explicit list of the bodies above it,
    // and are visited in the same ascending order: identical forces in identical creation order,
    // without the n x large scan (10,000 bricks of the joint-heavy scene each scanned 75,000
    // bodies).
    if (large.empty()) return;
    std::vector<double> rs(n);
    for (int j = 0; j < n; j++) rs[j] = double(bodies[j].radius);
    std::vector<double> sortedR(rs);
    std::sort(sortedR.begin(), sortedR.end());
    const double R0 = n > 256 ? sortedR[size_t(n) - 257] : sortedR.back();
    const double h = std::max(2.0 * R0, 1e-3);
    std::vector<int> big;
    std::unordered_map<std::tuple<long long, long long, long long>, std::vector<int>, KeyHash> coarse;
    std::vector<int> gridded;
    for (int j = 0; j < n; j++) {
      if (rs[j] > R0) {
        big.push_back(j);
        continue;
      }
      gridded.push_back(j);
      coarse[std::make_tuple((long long)std::floor(double(bodies[j].pos[0]) / h), (long long)std::floor(double(bodies[j].pos[1]) / h),
                             (long long)std::floor(double(bodies[j].pos[2]) / h))]
          .push_back(j);
    }
    std::vector<int> cand;
    for (int i : large) {
      cand.assign(big.begin(), big.end());
      // conservative reach: |pi - pj| <= ri + rj <= ri + R0, widened far beyond the rounding
      // of the float predicate (the slack only adds candidates)
      const double reach = (rs[i] + R0) * 1.001 + 1e-3;
      long long lo[3], hi[3];
      long long cells = 1;
      for (int k = 0; k < 3; k++) {
        lo[k] = (long long)std::floor((double(bodies[i].pos[k]) - reach) / h);
        hi[k] = (long long)std::floor((double(bodies[i].pos[k]) + reach) / h);
        cells *= hi[k] - lo[k] + 1;
      }
      if (cells > (long long)coarse.size()) {
        cand.insert(cand.end(), gridded.begin(), gridded.end());
      } else {
        for (long long x = lo[0]; x <= hi[0]; x++)
          for (long long y = lo[1]; y <= hi[1]; y++)
            for (long long z = lo[2]; z <= hi[2]; z++) {
              auto it = coarse.find(std::make_tuple(x, y, z));
              if (it != coarse.end()) cand.insert(cand.end(), it->second.begin(), it->second.end());
            }
      }
      std::sort(cand.begin(), cand.end());
      for (int j : cand) pair(i, j);
    }
  }

  // ------------------------------------------------------------ colouring (coloring.ts)
  struct Graph { std::vector<int> start, nbr; };
  // Dynamic-neighbour graph and the canonical per-body constraint order (joints by jid, then
  // manifolds by the other body), the order the GPU engine stamps in.
  // A constraint touching a trigger body (its manifolds apply no forces, no constraint joins a
  // sleeping island through it; cpuPhysics3D.js:148-156, sleeping.js:54, restitution.js:68).
  bool triggerForce(const Force<R>& f) const {
    return (f.a >= 0 && bodies[f.a].isTrigger) || (f.b >= 0 && bodies[f.b].isTrigger);
  }
  void canonicalLists(std::vector<std::vector<int>>& lists) const {
    const int n = int(bodies.size());
    lists.assign(n, {});
    for (int id : forces) {
      const Force<R>& f = *store[id];
      if (f.type == F_IGNORE) continue;
      if (f.type == F_MANIFOLD && triggerForce(f)) continue;
      for (int body : {f.a, f.b})
        if (body >= 0 && bodies[body].mass > 0) lists[body].push_back(id);
    }
    for (int b = 0; b < n; b++) {
      auto key = [&](int id) {
        const Force<R>& f = *store[id];
        if (f.type != F_MANIFOLD) return std::make_pair(0LL, (long long)f.jid);
        int other = f.a == b ? f.b : f.a;
        return std::make_pair((long long)other + 2, 0LL);
      };
      std::stable_sort(lists[b].begin(), lists[b].end(), [&](int x, int y) { return key(x) < key(y); });
    }
  }
  void jpColor(const std::vector<std::vector<int>>& lists) {
    const int n = int(bodies.size());
    if (int(colors.size()) != n) colors.assign(n, -1);
    std::vector<int> next(n);
    std::vector<char> pending(n, 0);
    auto dyn = [&](int i) { return i >= 0 && bodies[i].mass > 0; };
    auto other = [&](int id, int b) {
      const Force<R>& f = *store[id];
      int o = f.a == b ? f.b : f.a;
      return dyn(o) ? o : -1;
    };
    auto smallestFree = [&](int b, bool skipPending) {
      uint64_t used = 0;
      for (int id : lists[b]) {
        int j = other(id, b);
        if (j < 0 || (skipPending && pending[j])) continue;
        int col = colors[j];
        if (col < 0) continue;
        used |= 1ull << col;
      }
      if (~used == 0) return MAX_COLORS - 1;
      int c = 0;
      while (used & (1ull << c)) c++;
      return c;
    };
    for (int b = 0; b < n; b++) {
      next[b] = colors[b];
      if (!dyn(b) || colors[b] < 0) continue;
      bool isMax = true;
      for (int id : lists[b]) {
        int j = other(id, b);
        if (j >= 0 && !jp_beats(jp_priority(b), b, jp_priority(j), j)) { isMax = false; break; }
      }
      if (isMax) next[b] = std::min(colors[b], smallestFree(b, false));
    }
    colors = next;
    auto markPending = [&]() {
      int count = 0;
      for (int b = 0; b < n; b++) {
        pending[b] = 0;
        if (!dyn(b)) continue;
        if (colors[b] < 0) pending[b] = 1;
        else
          for (int id : lists[b]) {
            int j = other(id, b);
            if (j >= 0 && colors[j] == colors[b] && jp_beats(jp_priority(j), j, jp_priority(b), b)) { pending[b] = 1; break; }
          }
        count += pending[b];
      }
      return count;
    };
    int remaining = markPending();
    int rounds = 0;
    while (remaining > 0 && rounds < colorRounds) {
      rounds++;
      for (int b = 0; b < n; b++) {
        next[b] = -2;
        if (!pending[b]) continue;
        bool isMax = true;
        for (int id : lists[b]) {
          int j = other(id, b);
          if (j >= 0 && pending[j] && !jp_beats(jp_priority(b), b, jp_priority(j), j)) { isMax = false; break; }
        }
        if (isMax) next[b] = smallestFree(b, true);
      }
      for (int b = 0; b < n; b++) {
        if (next[b] == -2) continue;
        colors[b] = next[b];
        pending[b] = 0;
        remaining--;
      }
    }
    lastConflicts = 0;
    if (remaining > 0) {
      for (int b = 0; b < n; b++)
        if (pending[b] && colors[b] < 0) colors[b] = 0;
      lastConflicts = markPending();
    }
    lastNumColors = 0;
    for (int b = 0; b < n; b++)
      if (dyn(b)) lastNumColors = std::max(lastNumColors, colors[b] + 1);
  }

  // ------------------------------------------------------------ step
  void solveBody(int bi, const std::vector<int>& order, bool reverse) {
    Body<R>& body = bodies[bi];
    Sys sys;
    R m = body.mass;
    const R* I = body.moment;
    Mt::diagonal(sys.lhsLin, m / (dt * dt), m / (dt * dt), m / (dt * dt));
    Mt::diagonal(sys.lhsAng, I[0] / (dt * dt), I[1] / (dt * dt), I[2] / (dt * dt));
    for (int i = 0; i < 9; i++) sys.lhsCross[i] = 0;
    R dp[3];
    Mt::sub3(dp, body.pos, body.y);
    Mt::mulv(sys.rhsLin, sys.lhsLin, dp);
    Mt::qsub(dp, body.q, body.qy);
    Mt::mulv(sys.rhsAng, sys.lhsAng, dp);
    const int nf = int(order.size());
    for (int k = 0; k < nf; k++) {
      const Force<R>& f = *store[order[reverse ? nf - 1 - k : k]];
      if (f.type == F_MANIFOLD) manifoldPrimal(f, bi, sys);
      else if (f.type == F_JOINT) jointPrimal(f, bi, sys);
      else if (f.type == F_SPRING) springPrimal(f, bi, sys);
    }
    const bool point = app && body.moment[0] == 0 && body.moment[1] == 0 && body.moment[2] == 0;
    if (point) {
      Mt::diagonal(sys.lhsAng, 1, 1, 1);
      for (int i = 0; i < 9; i++) sys.lhsCross[i] = 0;
      sys.rhsAng[0] = sys.rhsAng[1] = sys.rhsAng[2] = 0;
    }
    R bl[3], ba[3], dxL[3], dxA[3];
    Mt::neg3(bl, sys.rhsLin);
    Mt::neg3(ba, sys.rhsAng);
    Mt::solve6(sys.lhsLin, sys.lhsAng, sys.lhsCross, bl, ba, dxL, dxA);
    Mt::addScaled3(body.pos, body.pos, dxL, 1);
    if (!point) Mt::qaddv(body.q, body.q, dxA);
  }

  // Step part 1: broadphase and force initialisation (the "collision" half).
  void stepCollide() {
    if (app) broadphaseApp();
    else broadphaseRef();
    std::vector<int> kept;
    for (int id : forces) {
      Force<R>& f = *store[id];
      bool keep = true;
      if (f.type == F_MANIFOLD) keep = manifoldInitialize(f);
      else if (f.type == F_JOINT) keep = jointInitialize(f);
      else if (f.type == F_SPRING) keep = springInitialize(f);
      if (keep) kept.push_back(id);
      else unlinkFromBodies(id);
    }
    forces.swap(kept);
  }
  // Velocity-level restitution after the solve (src/native/cpu/restitution.js, with the GPU
  // backend's arrangement, src/gpu/restitution.js: manifold centroids summed then divided, an
  // impact threshold of 1 m/s, 12 Jacobi rounds relaxed by the larger constraint-list length of
  // the two bodies, each body's velocity change summed in its constraint-list order). Constraint
  // lists hold dynamic bodies only, as the GPU backend's adjacency does, so a static body's
  // degree is 0 (the CPU world counts a static body's forces too).
  struct Bounce {
    int a, b;
    R n[3], ra[3], rb[3], k, target, impulse, delta;
  };
  // a sleeping body takes no impulse (restitution.js inverseMass)
  R invMass(int i) const { return bodies[i].mass > 0 && !bodies[i].sleeping ? R(1) / bodies[i].mass : R(0); }
  void invInertia(R* o, int i, const R* t) const {
    const Body<R>& bd = bodies[i];
    if (!(bd.mass > 0) || bd.sleeping) {
      Mt::set3(o, 0, 0, 0);
      return;
    }
    R c[4] = {-bd.q[0], -bd.q[1], -bd.q[2], bd.q[3]}, local[3];
    Mt::rotate(local, c, t);
    for (int k = 0; k < 3; k++) local[k] = bd.moment[k] > 0 ? local[k] / bd.moment[k] : R(0);
    Mt::rotate(o, bd.q, local);
  }
  static void pointVelocity(R* o, const R* v, const R* w, const R* r) {
    R c[3];
    Mt::cross(c, w, r);
    Mt::add3(o, v, c);
  }
  void bounce(const std::vector<R>& inV, const std::vector<R>& inW, const std::vector<std::vector<int>>& lists) {
    std::vector<int> slot(store.size(), -1);
    std::vector<Bounce> bs;
    for (int id : forces) {
      const Force<R>& f = *store[id];
      if (f.type != F_MANIFOLD || f.contacts.empty() || triggerForce(f)) continue;
      const R e = std::max(bodies[f.a].restitution, bodies[f.b].restitution);
      if (!(e > 0)) continue;
      Bounce B;
      B.a = f.a;
      B.b = f.b;
      for (int k = 0; k < 3; k++) B.n[k] = f.basis[k];
      R sa[3] = {0, 0, 0}, sb[3] = {0, 0, 0}, t[3];
      for (const Contact<R>& c : f.contacts) {
        Mt::rotate(t, bodies[f.a].q, c.rA);
        Mt::add3(sa, sa, t);
        Mt::rotate(t, bodies[f.b].q, c.rB);
        Mt::add3(sb, sb, t);
      }
      const R cnt = R(f.contacts.size());
      for (int k = 0; k < 3; k++) { B.ra[k] = sa[k] / cnt; B.rb[k] = sb[k] / cnt; }
      R pa[3], pb[3], d[3];
      pointVelocity(pa, &inV[3 * f.a], &inW[3 * f.a], B.ra);
      pointVelocity(pb, &inV[3 * f.b], &inW[3 * f.b], B.rb);
      Mt::sub3(d, pa, pb);
      const R vn = Mt::dot(B.n, d);
      if (vn >= R(-1)) continue;
      R ta[3], tb[3], ia[3], ib[3];
      Mt::cross(ta, B.ra, B.n);
      Mt::cross(tb, B.rb, B.n);
      invInertia(ia, f.a, ta);
      invInertia(ib, f.b, tb);
      B.k = ((invMass(f.a) + invMass(f.b)) + Mt::dot(ta, ia)) + Mt::dot(tb, ib);
      if (!(B.k > 0)) continue;
      B.target = -e * vn;
      B.impulse = 0;
      B.delta = 0;
      slot[id] = int(bs.size());
      bs.push_back(B);
    }
    if (bs.empty()) return;
    auto degree = [&](int i) { return bodies[i].mass > 0 ? int(lists[i].size()) : 0; };
    for (int round = 0; round < 12; round++) {
      for (Bounce& B : bs) {
        R pa[3], pb[3], d[3];
        pointVelocity(pa, bodies[B.a].v, bodies[B.a].w, B.ra);
        pointVelocity(pb, bodies[B.b].v, bodies[B.b].w, B.rb);
        Mt::sub3(d, pa, pb);
        const R vn = Mt::dot(B.n, d);
        const int deg = std::max(1, std::max(degree(B.a), degree(B.b)));
        const R imp = std::max(R(0), B.impulse + (B.target - vn) / (B.k * R(deg)));
        B.delta = imp - B.impulse;
        B.impulse = imp;
      }
      std::vector<R> dvs(3 * bodies.size(), R(0)), dws(3 * bodies.size(), R(0));
      for (int i = 0; i < int(bodies.size()); i++) {
        if (!(bodies[i].mass > 0) || bodies[i].sleeping) continue;
        R dv[3] = {0, 0, 0}, dw[3] = {0, 0, 0};
        for (int id : lists[i]) {
          if (id >= int(slot.size()) || slot[id] < 0) continue;
          const Bounce& B = bs[slot[id]];
          const bool isA = i == B.a;
          R imp[3], t[3], di[3];
          for (int k = 0; k < 3; k++) imp[k] = (B.n[k] * B.delta) * (isA ? R(1) : R(-1));
          for (int k = 0; k < 3; k++) dv[k] += imp[k] * invMass(i);
          Mt::cross(t, isA ? B.ra : B.rb, imp);
          invInertia(di, i, t);
          Mt::add3(dw, dw, di);
        }
        for (int k = 0; k < 3; k++) { dvs[3 * i + k] = dv[k]; dws[3 * i + k] = dw[k]; }
      }
      for (int i = 0; i < int(bodies.size()); i++) {
        if (!(bodies[i].mass > 0) || bodies[i].sleeping) continue;
        for (int k = 0; k < 3; k++) { bodies[i].v[k] += dvs[3 * i + k]; bodies[i].w[k] += dws[3 * i + k]; }
      }
    }
  }

  // Step part 2: body warm start, iterations, velocities.
  void stepSolve() {
    const int n = int(bodies.size());
    bool bounceOn = false;
    for (const Body<R>& b : bodies) bounceOn |= b.restitution > 0;
    std::vector<R> inV, inW;
    std::vector<std::vector<int>> bounceLists;
    if (bounceOn) {
      inV.resize(3 * size_t(n));
      inW.resize(3 * size_t(n));
      for (int b = 0; b < n; b++)
        for (int k = 0; k < 3; k++) { inV[3 * b + k] = bodies[b].v[k]; inW[3 * b + k] = bodies[b].w[k]; }
      canonicalLists(bounceLists);
    }
    for (int b = n - 1; b >= 0; b--) {
      Body<R>& body = bodies[b];
      R t[3], accel[3];
      if (app) {
        Mt::addScaled3(body.y, body.pos, body.v, dt);
        if (body.mass > 0) Mt::addScaled3(body.y, body.y, up, gravity * dt * dt);
        Mt::scale3(t, body.w, dt);
        Mt::qaddv(body.qy, body.q, t);
        Mt::sub3(accel, body.v, body.vprev);
        Mt::div3(accel, accel, dt);
        R accelExt = Mt::dot(accel, up) * Mt::sign(gravity);
        R accelWeight = Mt::clamp(accelExt / std::fabs(gravity), 0, 1);
        if (!std::isfinite(accelWeight)) accelWeight = 0;
        std::memcpy(body.x0, body.pos, sizeof(body.x0));
        std::memcpy(body.q0, body.q, sizeof(body.q0));
        if (body.mass > 0 && !body.sleeping) {
          Mt::addScaled3(body.pos, body.pos, body.v, dt);
          Mt::addScaled3(body.pos, body.pos, up, gravity * accelWeight * dt * dt);
          Mt::scale3(t, body.w, dt);
          Mt::qaddv(body.q, body.q, t);
        }
      } else {
        Mt::addScaled3(body.y, body.pos, body.v, dt);
        if (body.mass > 0) body.y[2] += gravity * (dt * dt);
        Mt::scale3(t, body.w, dt);
        Mt::qaddv(body.qy, body.q, t);
        Mt::sub3(accel, body.v, body.vprev);
        Mt::div3(accel, accel, dt);
        R accelExt = accel[2] * Mt::sign(gravity);
        R accelWeight = Mt::clamp(accelExt / std::fabs(gravity), 0, 1);
        if (!std::isfinite(accelWeight)) accelWeight = 0;
        std::memcpy(body.x0, body.pos, sizeof(body.x0));
        std::memcpy(body.q0, body.q, sizeof(body.q0));
        if (body.mass > 0 && !body.sleeping) {
          Mt::addScaled3(body.pos, body.pos, body.v, dt);
          body.pos[2] += gravity * (accelWeight * dt * dt);
          Mt::scale3(t, body.w, dt);
          Mt::qaddv(body.q, body.q, t);
        }
      }
    }
    std::vector<std::vector<int>> lists;
    std::vector<std::vector<int>> buckets;
    if (colored) {
      canonicalLists(lists);
      jpColor(lists);
      buckets.assign(MAX_COLORS, {});
      for (int b = 0; b < n; b++)
        if (bodies[b].mass > 0) buckets[colors[b]].push_back(b);
    }
    for (int it = 0; it < iterations; it++) {
      if (colored) {
        for (int c = 0; c < MAX_COLORS; c++)
          for (int b : buckets[c])
            if (!bodies[b].sleeping) solveBody(b, lists[b], false);
      } else {
        for (int b = n - 1; b >= 0; b--) {
          if (bodies[b].mass <= 0 || bodies[b].sleeping) continue;
          solveBody(b, bodies[b].forces, true);
        }
      }
      for (int id : forces) {
        Force<R>& f = *store[id];
        if (f.type == F_MANIFOLD) manifoldDual(f);
        else if (f.type == F_JOINT) jointDual(f);
      }
    }
    for (Body<R>& body : bodies) {
      std::memcpy(body.vprev, body.v, sizeof(body.v));
      if (body.mass > 0 && !body.sleeping) {
        R t[3];
        Mt::sub3(t, body.pos, body.x0);
        Mt::div3(body.v, t, dt);
        Mt::qsub(t, body.q, body.q0);
        Mt::div3(body.w, t, dt);
      }
    }
    if (bounceOn) bounce(inV, inW, bounceLists);
  }
  void step() {
    stepCollide();
    stepSolve();
    if (sleepOn) sleepAfter();
  }

  // Island sleeping after the step (src/native/cpu/sleeping.js:26-108). Islands: dynamic bodies
  // joined by any live constraint (joint, spring, ignore pair, manifold with contacts); an
  // island is supported when one of its bodies touches a static body or hangs from the world.
  // A supported island whose bodies all allow sleep and move no faster than the threshold
  // (|(v, w)|, the 6-vector) accumulates time; each body whose time reaches the delay sleeps
  // with zero velocity. A live constraint between a sleeping and an awake dynamic body wakes
  // the whole world before the next step. The speed is sqrt of the left-to-right sum of the six
  // squares, in the solver's precision.
  void wakeAll() {
    for (Body<R>& b : bodies) b.sleeping = false;
    std::fill(sleepTime.begin(), sleepTime.end(), R(0));
  }
  static R sleepSpeedOf(const Body<R>& b) {
    const R s = ((((b.v[0] * b.v[0] + b.v[1] * b.v[1]) + b.v[2] * b.v[2]) + b.w[0] * b.w[0]) + b.w[1] * b.w[1]) +
                b.w[2] * b.w[2];
    return std::sqrt(s);
  }
  void sleepAfter() {
    const int n = int(bodies.size());
    if (int(sleepTime.size()) != n) sleepTime.assign(n, R(0));
    std::vector<int> root(n);
    for (int i = 0; i < n; i++) root[i] = i;
    auto find = [&](int i) {
      while (root[i] != i) {
        root[i] = root[root[i]];
        i = root[i];
      }
      return i;
    };
    std::vector<char> support(n, 0);
    std::vector<std::pair<int, int>> edges;
    auto dyn = [&](int i) { return bodies[i].mass > 0; };
    for (int id : forces) {
      const Force<R>& f = *store[id];
      if (f.broken || triggerForce(f)) continue;
      if (f.type == F_MANIFOLD && f.contacts.empty()) continue;
      const int a = f.a, b = f.b;
      if (a < 0) support[b] = 1;
      else if (!dyn(a)) support[b] = 1;
      else if (!dyn(b)) support[a] = 1;
      else root[find(a)] = find(b);
      edges.emplace_back(a, b);
    }
    std::vector<char> supported(n, 0), stable(n, 1);
    for (int i = 0; i < n; i++)
      if (support[i]) supported[find(i)] = 1;
    for (int i = 0; i < n; i++)
      if (dyn(i) && !(bodies[i].allowSleep && sleepSpeedOf(bodies[i]) <= sleepSpeed)) stable[find(i)] = 0;
    for (int i = 0; i < n; i++) {
      if (!dyn(i)) continue;
      const int r = find(i);
      sleepTime[i] = supported[r] && stable[r] ? sleepTime[i] + dt : R(0);
      if (sleepTime[i] >= sleepDelay) {
        Body<R>& b = bodies[i];
        b.sleeping = true;
        Mt::set3(b.v, 0, 0, 0);
        Mt::set3(b.w, 0, 0, 0);
      }
    }
    for (const auto& e : edges)
      if (e.first >= 0 && dyn(e.first) && dyn(e.second) && bodies[e.first].sleeping != bodies[e.second].sleeping) {
        wakeAll();
        break;
      }
  }
  int forceCount() const { return int(forces.size()); }

  // Body commands in the 12-word records of src/gpu/bodyCommands2D.js:46-55 (index, kind,
  // hasPoint, 0, value[4], point[4]) with the semantics of src/native/cpu/world.js:229-300
  // (flushEdits): 0 set linear velocity, 1 set angular velocity, 2 impulse (at point), 3 force
  // (value.w = dt), 4 teleport (position, rotation = point; step-start and inertial poses follow;
  // the body's manifolds are dropped), 5 angular impulse, 6 torque (value.w = dt).
  void applyEdits(const uint32_t* rec, int n) {
    if (n > 0 && sleepOn) wakeAll();  // queued body commands wake the world (world.js:132-133)
    for (int k = 0; k < n; k++) {
      const uint32_t* u = rec + 12 * size_t(k);
      float f[12];
      std::memcpy(f, u, sizeof(f));
      const int id = int(u[0]), kind = int(u[1]);
      const bool point = u[2] != 0;
      Body<R>& b = bodies[id];
      auto angular = [&](const R* v) {
        if (b.mass <= 0) return;
        R c[4] = {-b.q[0], -b.q[1], -b.q[2], b.q[3]}, local[3], delta[3];
        Mt::rotate(local, c, v);
        for (int i = 0; i < 3; i++) local[i] = local[i] / std::max(R(1e-10), b.moment[i]);
        Mt::rotate(delta, b.q, local);
        for (int i = 0; i < 3; i++) b.w[i] += delta[i];
      };
      if (kind == 0) {
        for (int i = 0; i < 3; i++) b.v[i] = R(f[4 + i]);
      } else if (kind == 1) {
        for (int i = 0; i < 3; i++) b.w[i] = R(f[4 + i]);
      } else if (kind == 4) {
        for (int i = 0; i < 3; i++) b.pos[i] = R(f[4 + i]);
        if (point)
          for (int i = 0; i < 4; i++) b.q[i] = R(f[8 + i]);
        std::memcpy(b.x0, b.pos, sizeof(b.x0));
        std::memcpy(b.y, b.pos, sizeof(b.y));
        std::memcpy(b.q0, b.q, sizeof(b.q0));
        std::memcpy(b.qy, b.q, sizeof(b.qy));
        std::vector<int> kept;
        for (int fid : forces) {
          Force<R>& fo = *store[fid];
          if (fo.type == F_MANIFOLD && (fo.a == id || fo.b == id)) unlinkFromBodies(fid);
          else kept.push_back(fid);
        }
        forces.swap(kept);
      } else if (kind == 2 || kind == 3) {
        if (b.mass <= 0) continue;
        R imp[3];
        for (int i = 0; i < 3; i++) imp[i] = kind == 3 ? R(f[4 + i]) * R(f[7]) : R(f[4 + i]);
        for (int i = 0; i < 3; i++) b.v[i] += imp[i] / b.mass;
        if (point) {
          R r[3], t[3];
          for (int i = 0; i < 3; i++) r[i] = R(f[8 + i]) - b.pos[i];
          Mt::cross(t, r, imp);
          angular(t);
        }
      } else if (kind == 5 || kind == 6) {
        R t[3];
        for (int i = 0; i < 3; i++) t[i] = kind == 6 ? R(f[4 + i]) * R(f[7]) : R(f[4 + i]);
        angular(t);
      }
    }
  }
};

// ---------------------------------------------------------------- collide.ts (box-box)
template <class R> struct BoxCollide {
  using Mt = M<R>;
  static constexpr int MAX_CONTACTS = 8;
  static constexpr int MAX_POLY_VERTS = 16;
  static constexpr int AXIS_FACE_A = 0, AXIS_FACE_B = 1, AXIS_EDGE = 2;
  struct V { R v[3]; };
  struct OBB { R center[3]; R half[3]; R axis[3][3]; };
  struct SatAxis { int type, indexA, indexB; R separation; R normalAB[3]; bool valid; };
  using Raw = typename Solver<R>::Raw;
  static R SAT_EPS() { return R(1.0e-6); }
  static R PLANE_EPS() { return R(1.0e-5); }
  static R MERGE_SQ() { return R(1.0e-6); }

  static OBB makeOBB(const Body<R>& b) {
    OBB o;
    std::memcpy(o.center, b.pos, sizeof(o.center));
    Mt::scale3(o.half, b.size, R(0.5));
    static const R ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0}, ez[3] = {0, 0, 1};
    Mt::rotate(o.axis[0], b.q, ex);
    Mt::rotate(o.axis[1], b.q, ey);
    Mt::rotate(o.axis[2], b.q, ez);
    return o;
  }
  static R absDot(const R* a, const R* b) { return std::fabs(Mt::dot(a, b)); }
  static V supportPoint(const OBB& box, const R* dir) {
    R sx = Mt::dot(dir, box.axis[0]) >= 0 ? 1 : -1;
    R sy = Mt::dot(dir, box.axis[1]) >= 0 ? 1 : -1;
    R sz = Mt::dot(dir, box.axis[2]) >= 0 ? 1 : -1;
    V p;
    Mt::addScaled3(p.v, box.center, box.axis[0], box.half[0] * sx);
    Mt::addScaled3(p.v, p.v, box.axis[1], box.half[1] * sy);
    Mt::addScaled3(p.v, p.v, box.axis[2], box.half[2] * sz);
    return p;
  }
  struct FaceAxes { const R* u; const R* v; R extentU, extentV; };
  static FaceAxes faceAxes(const OBB& box, int axisIndex) {
    if (axisIndex == 0) return {box.axis[1], box.axis[2], box.half[1], box.half[2]};
    if (axisIndex == 1) return {box.axis[0], box.axis[2], box.half[0], box.half[2]};
    return {box.axis[0], box.axis[1], box.half[0], box.half[1]};
  }
  static int chooseIncidentFaceAxis(const OBB& box, const R* refN) {
    int axis = 0;
    R best = -std::numeric_limits<R>::max();
    for (int i = 0; i < 3; i++) {
      R d = absDot(box.axis[i], refN);
      if (d > best) { best = d; axis = i; }
    }
    return axis;
  }
  static std::vector<V> clipPolygon(const std::vector<V>& in, const R* n, R off) {
    std::vector<V> out;
    if (in.empty()) return out;
    V a = in.back();
    R da = Mt::dot(n, a.v) - off;
    for (const V& b : in) {
      R db = Mt::dot(n, b.v) - off;
      bool aIn = da <= PLANE_EPS(), bIn = db <= PLANE_EPS();
      if (aIn != bIn) {
        R t = 0;
        R denom = da - db;
        if (std::fabs(denom) > SAT_EPS()) t = Mt::clamp(da / denom, 0, 1);
        if (int(out.size()) < MAX_POLY_VERTS) {
          V p, d;
          Mt::sub3(d.v, b.v, a.v);
          Mt::addScaled3(p.v, a.v, d.v, t);
          out.push_back(p);
        }
      }
      if (bIn && int(out.size()) < MAX_POLY_VERTS) out.push_back(b);
      a = b;
      da = db;
    }
    return out;
  }
  struct Builder {
    std::vector<Raw> contacts;
    std::vector<V> mids;
    const Body<R>& A;
    const Body<R>& B;
    Builder(const Body<R>& a, const Body<R>& b) : A(a), B(b) {}
    void add(const R* xA, const R* xB, uint32_t feature) {
      V mid;
      R s[3];
      Mt::add3(s, xA, xB);
      Mt::scale3(mid.v, s, R(0.5));
      for (const V& m : mids) {
        R d[3];
        Mt::sub3(d, mid.v, m.v);
        if (Mt::lengthSq(d) < MERGE_SQ()) return;
      }
      if (int(contacts.size()) >= MAX_CONTACTS) return;
      Raw c;
      c.feature = feature;
      R d[3];
      Mt::sub3(d, xA, A.pos);
      Mt::rotateInv(c.rA, A.q, d);
      Mt::sub3(d, xB, B.pos);
      Mt::rotateInv(c.rB, B.q, d);
      contacts.push_back(c);
      mids.push_back(mid);
    }
  };
  static bool testAxis(const OBB& A, const OBB& B, const R* delta, const R* axis, int type, int ia, int ib, SatAxis& best) {
    R lenSq = Mt::lengthSq(axis);
    if (lenSq < SAT_EPS()) return true;
    R invLen = 1 / std::sqrt(lenSq);
    R n[3];
    Mt::scale3(n, axis, invLen);
    if (Mt::dot(n, delta) < 0) Mt::neg3(n, n);
    R distance = std::fabs(Mt::dot(delta, n));
    R rA = A.half[0] * absDot(n, A.axis[0]) + A.half[1] * absDot(n, A.axis[1]) + A.half[2] * absDot(n, A.axis[2]);
    R rB = B.half[0] * absDot(n, B.axis[0]) + B.half[1] * absDot(n, B.axis[1]) + B.half[2] * absDot(n, B.axis[2]);
    R separation = distance - (rA + rB);
    if (separation > 0) return false;
    if (!best.valid || separation > best.separation) {
      best.valid = true;
      best.type = type;
      best.indexA = ia;
      best.indexB = ib;
      best.separation = separation;
      std::memcpy(best.normalAB, n, sizeof(n));
    }
    return true;
  }
  static void supportEdge(const OBB& box, int axisIndex, const R* dir, R* e0, R* e1) {
    int a1 = (axisIndex + 1) % 3, a2 = (axisIndex + 2) % 3;
    R s1 = Mt::dot(dir, box.axis[a1]) >= 0 ? 1 : -1;
    R s2 = Mt::dot(dir, box.axis[a2]) >= 0 ? 1 : -1;
    R c[3], e[3];
    Mt::addScaled3(c, box.center, box.axis[a1], box.half[a1] * s1);
    Mt::addScaled3(c, c, box.axis[a2], box.half[a2] * s2);
    Mt::scale3(e, box.axis[axisIndex], box.half[axisIndex]);
    Mt::sub3(e0, c, e);
    Mt::add3(e1, c, e);
  }
  static void closestPointsOnSegments(const R* p0, const R* p1, const R* q0, const R* q1, R* xA, R* xB) {
    R d1[3], d2[3], r[3];
    Mt::sub3(d1, p1, p0);
    Mt::sub3(d2, q1, q0);
    Mt::sub3(r, p0, q0);
    R a = Mt::dot(d1, d1), e = Mt::dot(d2, d2), f = Mt::dot(d2, r);
    R s = 0, t = 0;
    if (a <= SAT_EPS() && e <= SAT_EPS()) {
      std::memcpy(xA, p0, 3 * sizeof(R));
      std::memcpy(xB, q0, 3 * sizeof(R));
      return;
    }
    if (a <= SAT_EPS()) {
      t = Mt::clamp(f / e, 0, 1);
    } else {
      R c = Mt::dot(d1, r);
      if (e <= SAT_EPS()) {
        s = Mt::clamp(-c / a, 0, 1);
      } else {
        R b = Mt::dot(d1, d2);
        R denom = a * e - b * b;
        if (std::fabs(denom) > SAT_EPS()) s = Mt::clamp((b * f - c * e) / denom, 0, 1);
        t = (b * s + f) / e;
        if (t < 0) {
          t = 0;
          s = Mt::clamp(-c / a, 0, 1);
        } else if (t > 1) {
          t = 1;
          s = Mt::clamp((b - c) / a, 0, 1);
        }
      }
    }
    Mt::addScaled3(xA, p0, d1, s);
    Mt::addScaled3(xB, q0, d2, t);
  }
  static std::vector<Raw> faceManifold(const Body<R>& bA, const Body<R>& bB, const OBB& A, const OBB& B, bool refIsA, int refAxis, const R* nAB) {
    const OBB& refBox = refIsA ? A : B;
    const OBB& incBox = refIsA ? B : A;
    R refOut[3];
    if (refIsA) std::memcpy(refOut, nAB, sizeof(refOut));
    else Mt::neg3(refOut, nAB);
    // buildFaceFrame
    R sgn = Mt::dot(refOut, refBox.axis[refAxis]) >= 0 ? 1 : -1;
    R rn[3], rc[3];
    Mt::scale3(rn, refBox.axis[refAxis], sgn);
    Mt::addScaled3(rc, refBox.center, rn, refBox.half[refAxis]);
    FaceAxes rf = faceAxes(refBox, refAxis);
    int incAxis = chooseIncidentFaceAxis(incBox, rn);
    // buildIncidentFace
    R isg = Mt::dot(incBox.axis[incAxis], rn) > 0 ? -1 : 1;
    R fn[3], fc[3];
    Mt::scale3(fn, incBox.axis[incAxis], isg);
    Mt::addScaled3(fc, incBox.center, fn, incBox.half[incAxis]);
    FaceAxes inf = faceAxes(incBox, incAxis);
    auto vert = [&](R su, R sv) {
      V p;
      Mt::addScaled3(p.v, fc, inf.u, su * inf.extentU);
      Mt::addScaled3(p.v, p.v, inf.v, sv * inf.extentV);
      return p;
    };
    std::vector<V> poly = {vert(1, 1), vert(-1, 1), vert(-1, -1), vert(1, -1)};
    R nu[3], nv[3];
    Mt::neg3(nu, rf.u);
    Mt::neg3(nv, rf.v);
    const R* pn[4] = {rf.u, nu, rf.v, nv};
    R ext[4] = {rf.extentU, rf.extentU, rf.extentV, rf.extentV};
    for (int k = 0; k < 4; k++) {
      poly = clipPolygon(poly, pn[k], Mt::dot(pn[k], rc) + ext[k]);
      if (poly.empty()) return {};
    }
    Builder builder(bA, bB);
    uint32_t prefix = (uint32_t(refIsA ? AXIS_FACE_A : AXIS_FACE_B) << 24) | (uint32_t(refAxis & 0xff) << 16) | (uint32_t(incAxis & 0xff) << 8);
    for (int i = 0; i < int(poly.size()) && int(builder.contacts.size()) < MAX_CONTACTS; i++) {
      const R* pI = poly[i].v;
      R d[3];
      Mt::sub3(d, pI, rc);
      R distance = Mt::dot(d, rn);
      if (distance > PLANE_EPS()) continue;
      R pR[3];
      Mt::addScaled3(pR, pI, rn, -distance);
      const R* xA = refIsA ? pR : pI;
      const R* xB = refIsA ? pI : pR;
      builder.add(xA, xB, prefix | uint32_t(i & 0xff));
    }
    if (builder.contacts.empty()) {
      R mn[3];
      Mt::neg3(mn, nAB);
      V sa = supportPoint(A, nAB), sb = supportPoint(B, mn);
      builder.add(sa.v, sb.v, prefix);
    }
    return builder.contacts;
  }
  static std::vector<Raw> edgeContact(const Body<R>& bA, const Body<R>& bB, const OBB& A, const OBB& B, int axA, int axB, const R* nAB) {
    R a0[3], a1[3], b0[3], b1[3], mn[3], xA[3], xB[3];
    supportEdge(A, axA, nAB, a0, a1);
    Mt::neg3(mn, nAB);
    supportEdge(B, axB, mn, b0, b1);
    closestPointsOnSegments(a0, a1, b0, b1, xA, xB);
    Builder builder(bA, bB);
    uint32_t key = (uint32_t(AXIS_EDGE) << 24) | (uint32_t(axA & 0xff) << 8) | uint32_t(axB & 0xff);
    builder.add(xA, xB, key);
    if (builder.contacts.empty()) {
      V sa = supportPoint(A, nAB), sb = supportPoint(B, mn);
      builder.add(sa.v, sb.v, key);
    }
    return builder.contacts;
  }
  static std::vector<Raw> run(const Body<R>& bA, const Body<R>& bB, R* basis, bool faceBias) {
    OBB A = makeOBB(bA), B = makeOBB(bB);
    R delta[3];
    Mt::sub3(delta, B.center, A.center);
    R fmax = std::numeric_limits<float>::max();  // FLT_MAX as in collide.ts
    SatAxis bestFace{AXIS_FACE_A, 0, 0, -fmax, {0, 0, 0}, false};
    SatAxis bestEdge{AXIS_EDGE, 0, 0, -fmax, {0, 0, 0}, false};
    for (int i = 0; i < 3; i++) if (!testAxis(A, B, delta, A.axis[i], AXIS_FACE_A, i, -1, bestFace)) return {};
    for (int i = 0; i < 3; i++) if (!testAxis(A, B, delta, B.axis[i], AXIS_FACE_B, -1, i, bestFace)) return {};
    R axis[3];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        Mt::cross(axis, A.axis[i], B.axis[j]);
        if (!testAxis(A, B, delta, axis, AXIS_EDGE, i, j, bestEdge)) return {};
      }
    if (!bestFace.valid) return {};
    SatAxis best = bestFace;
    if (bestEdge.valid) {
      const R rel = R(0.95), absT = R(0.01);
      bool edgeWins = !faceBias ? rel * bestEdge.separation > bestFace.separation + absT
                                : bestEdge.separation > rel * bestFace.separation + absT;
      if (edgeWins) best = bestEdge;
    }
    R nn[3];
    Mt::neg3(nn, best.normalAB);
    Mt::orthonormal(basis, nn);
    if (best.type == AXIS_EDGE) return edgeContact(bA, bB, A, B, best.indexA, best.indexB, best.normalAB);
    if (best.type == AXIS_FACE_A) return faceManifold(bA, bB, A, B, true, best.indexA, best.normalAB);
    return faceManifold(bA, bB, A, B, false, best.indexB, best.normalAB);
  }
};

template <class R>
std::vector<typename Solver<R>::Raw> Solver<R>::collide(int ia, int ib, R* basis) const {
  return BoxCollide<R>::run(bodies[ia], bodies[ib], basis, app ? faceBias : false);
}

// ---------------------------------------------------------------- cpuContacts3D.js (spheres)
template <class R> struct Generic {
  using Mt = M<R>;
  using Raw = typename Solver<R>::Raw;
  struct V { R v[3]; };
  struct Face { V verts[4]; R normal[3]; };
  struct Geo {
    bool round = false;
    R radius = 0;
    V spine[2];
    V vertices[8];
    Face faces[6];
    int edges[12][2];  // vertex indices
    int nEdges = 0;
  };
  static R hyp(const R* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
  static void unit(R* o, const R* a) {
    R h = hyp(a);
    R s = R(1) / (h != 0 ? h : R(1));
    Mt::scale3(o, a, s);
  }
  static void world(R* o, const Body<R>& b, const R* p) {
    R t[3];
    Mt::rotate(t, b.q, p);
    Mt::add3(o, b.pos, t);
  }
  static Geo geometry(const Body<R>& b) {
    Geo g;
    if (b.shape == SHAPE_SPHERE || b.shape == SHAPE_CAPSULE) {  // cpuContacts3D.js:44-51
      g.round = true;
      g.radius = b.size[0] / 2;
      const R half = b.shape == SHAPE_CAPSULE ? std::max(R(0), b.size[1] / 2 - g.radius) : R(0);
      R p0[3] = {0, -half, 0}, p1[3] = {0, half, 0};
      world(g.spine[0].v, b, p0);
      world(g.spine[1].v, b, p1);
      return g;
    }
    for (int i = 0; i < 8; i++) {
      R local[3];
      for (int k = 0; k < 3; k++) local[k] = (b.size[k] / 2) * (((i >> k) & 1) ? R(1) : R(-1));
      world(g.vertices[i].v, b, local);
    }
    static const int boxFaces[6][4] = {{1, 3, 7, 5}, {0, 4, 6, 2}, {2, 6, 7, 3}, {0, 1, 5, 4}, {4, 5, 7, 6}, {0, 2, 3, 1}};
    static const R boxNormals[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (int f = 0; f < 6; f++) {
      for (int k = 0; k < 4; k++) g.faces[f].verts[k] = g.vertices[boxFaces[f][k]];
      Mt::rotate(g.faces[f].normal, b.q, boxNormals[f]);
    }
    bool seen[8][8] = {};
    for (int f = 0; f < 6; f++)
      for (int i = 0; i < 4; i++) {
        int ia = boxFaces[f][i], ib = boxFaces[f][(i + 1) % 4];
        int lo = std::min(ia, ib), hi = std::max(ia, ib);
        if (!seen[lo][hi]) {
          seen[lo][hi] = true;
          g.edges[g.nEdges][0] = ia;
          g.edges[g.nEdges][1] = ib;
          g.nEdges++;
        }
      }
    return g;
  }
  static V support(const Geo& g, const R* n) {
    if (g.round) {
      const V* p = &g.spine[0];
      for (int i = 0; i < 2; i++) if (Mt::dot(g.spine[i].v, n) > Mt::dot(p->v, n)) p = &g.spine[i];
      V o;
      Mt::addScaled3(o.v, p->v, n, g.radius);
      return o;
    }
    const V* p = &g.vertices[0];
    for (int i = 0; i < 8; i++) if (Mt::dot(g.vertices[i].v, n) > Mt::dot(p->v, n)) p = &g.vertices[i];
    return *p;
  }
  static void nearest(R* o, const R* a, const R* b, const R* p) {
    R e[3], ap[3];
    Mt::sub3(e, b, a);
    Mt::sub3(ap, p, a);
    R ee = Mt::dot(e, e);
    R t = Mt::dot(ap, e) / (ee != 0 ? ee : R(1));
    t = std::max(R(0), std::min(R(1), t));
    Mt::addScaled3(o, a, e, t);
  }
  static void closestSegments(const R* p, const R* q, const R* r, const R* s, R* oa, R* ob) {
    R d1[3], d2[3], w[3];
    Mt::sub3(d1, q, p);
    Mt::sub3(d2, s, r);
    Mt::sub3(w, p, r);
    R a = Mt::dot(d1, d1), e = Mt::dot(d2, d2), f = Mt::dot(d2, w);
    R u = 0, v = 0;
    auto cl = [](R x) { return std::max(R(0), std::min(R(1), x)); };
    if (a < R(1e-16)) v = e > R(1e-16) ? cl(f / e) : R(0);
    else {
      R c = Mt::dot(d1, w);
      if (e < R(1e-16)) u = cl(-c / a);
      else {
        R b = Mt::dot(d1, d2), den = a * e - b * b;
        u = den > R(1e-12) * a * e ? cl((b * f - c * e) / den) : R(0);
        v = (b * u + f) / e;
        if (v < 0) { v = 0; u = cl(-c / a); }
        else if (v > 1) { v = 1; u = cl((b - c) / a); }
      }
    }
    Mt::addScaled3(oa, p, d1, u);
    Mt::addScaled3(ob, r, d2, v);
  }
  static void closestTriangle(R* o, const R* p, const R* a, const R* b, const R* c) {
    R ab[3], ac[3], ap[3];
    Mt::sub3(ab, b, a); Mt::sub3(ac, c, a); Mt::sub3(ap, p, a);
    R d1 = Mt::dot(ab, ap), d2 = Mt::dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) { std::memcpy(o, a, 3 * sizeof(R)); return; }
    R bp[3];
    Mt::sub3(bp, p, b);
    R d3 = Mt::dot(ab, bp), d4 = Mt::dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { std::memcpy(o, b, 3 * sizeof(R)); return; }
    R vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { Mt::addScaled3(o, a, ab, d1 / (d1 - d3)); return; }
    R cp[3];
    Mt::sub3(cp, p, c);
    R d5 = Mt::dot(ab, cp), d6 = Mt::dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) { std::memcpy(o, c, 3 * sizeof(R)); return; }
    R vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) { Mt::addScaled3(o, a, ac, d2 / (d2 - d6)); return; }
    R va = d3 * d6 - d5 * d4;
    if (va <= 0 && d4 - d3 >= 0 && d5 - d6 >= 0) {
      R cb[3];
      Mt::sub3(cb, c, b);
      Mt::addScaled3(o, b, cb, (d4 - d3) / (d4 - d3 + d5 - d6));
      return;
    }
    R den = 1 / (va + vb + vc);
    R t1[3], t2[3], t3[3];
    Mt::scale3(t1, ab, vb * den);
    Mt::scale3(t2, ac, vc * den);
    Mt::add3(t3, t1, t2);
    Mt::add3(o, a, t3);
  }
  static void closestSurface(R* o, const Geo& g, const R* p) {
    R dist = std::numeric_limits<R>::infinity();
    for (int f = 0; f < 6; f++)
      for (int i = 1; i < 3; i++) {
        R q[3], d[3];
        closestTriangle(q, p, g.faces[f].verts[0].v, g.faces[f].verts[i].v, g.faces[f].verts[i + 1].v);
        Mt::sub3(d, p, q);
        R dd = Mt::dot(d, d);
        if (dd < dist) {
          std::memcpy(o, q, 3 * sizeof(R));
          dist = dd;
        }
      }
  }
  static std::vector<Raw> run(const Body<R>& a, const Body<R>& b, R* basis) {
    Geo ga = geometry(a), gb = geometry(b);
    R gap = -std::numeric_limits<R>::infinity();
    R n[3] = {0, 0, 1};
    int edgeA = -1, edgeB = -1;
    auto consider = [&](const R* axis, int ea, int eb) {
      if (hyp(axis) < R(1e-9)) return;
      R v[3], nv[3];
      unit(v, axis);
      Mt::scale3(nv, v, R(-1));
      V s1 = support(ga, nv), s2 = support(gb, v);
      R d[3];
      Mt::sub3(d, s1.v, s2.v);
      R g = Mt::dot(d, v);
      V s3 = support(gb, nv), s4 = support(ga, v);
      Mt::sub3(d, s3.v, s4.v);
      R rev = Mt::dot(d, v);
      if (rev > g) {
        g = rev;
        Mt::scale3(v, v, R(-1));
      }
      if (g > gap + R(1e-7)) {
        gap = g;
        std::memcpy(n, v, sizeof(n));
        edgeA = ea;
        edgeB = eb;
      }
    };
    for (const Geo* g : {&ga, &gb})
      if (!g->round)
        for (int f = 0; f < 6; f++) consider(g->faces[f].normal, -1, -1);
    if (!ga.round && !gb.round)
      for (int i = 0; i < ga.nEdges; i++)
        for (int j = 0; j < gb.nEdges; j++) {
          R e1[3], e2[3], c[3];
          Mt::sub3(e1, ga.vertices[ga.edges[i][1]].v, ga.vertices[ga.edges[i][0]].v);
          Mt::sub3(e2, gb.vertices[gb.edges[j][1]].v, gb.vertices[gb.edges[j][0]].v);
          Mt::cross(c, e1, e2);
          consider(c, i, j);
        }
    if (ga.round && gb.round) {
      R pa[3], pb[3], d[3];
      closestSegments(ga.spine[0].v, ga.spine[1].v, gb.spine[0].v, gb.spine[1].v, pa, pb);
      Mt::sub3(d, pa, pb);
      consider(d, -1, -1);
    }
    const Geo* rounds[2] = {&ga, &gb};
    const Geo* polys[2] = {&gb, &ga};
    for (int k = 0; k < 2; k++) {
      const Geo& round = *rounds[k];
      const Geo& poly = *polys[k];
      if (!round.round || poly.round) continue;
      for (int i = 0; i < 8; i++) {
        R q[3], d[3];
        nearest(q, round.spine[0].v, round.spine[1].v, poly.vertices[i].v);
        Mt::sub3(d, poly.vertices[i].v, q);
        consider(d, -1, -1);
      }
      for (int e = 0; e < poly.nEdges; e++) {
        R pa[3], pb[3], d[3];
        closestSegments(round.spine[0].v, round.spine[1].v, poly.vertices[poly.edges[e][0]].v, poly.vertices[poly.edges[e][1]].v, pa, pb);
        Mt::sub3(d, pa, pb);
        consider(d, -1, -1);
      }
    }
    const R ninf = -std::numeric_limits<R>::infinity();
    if (gap == ninf) {
      R d[3];
      Mt::sub3(d, a.pos, b.pos);
      consider(d, -1, -1);
    }
    if (gap > 0) return {};
    if (gap == ninf) {
      n[0] = 0; n[1] = 0; n[2] = 1;
    }
    R axisT[3] = {std::fabs(n[0]) < R(0.7) ? R(1) : R(0), std::fabs(n[0]) < R(0.7) ? R(0) : R(1), 0};
    R c[3], tangent[3], t2[3];
    Mt::cross(c, n, axisT);
    unit(tangent, c);
    Mt::cross(t2, n, tangent);
    for (int i = 0; i < 3; i++) { basis[i] = n[i]; basis[3 + i] = tangent[i]; basis[6 + i] = t2[i]; }
    std::vector<std::pair<V, V>> pairs;
    if (ga.round && gb.round) {
      R pa[3], pb[3];
      closestSegments(ga.spine[0].v, ga.spine[1].v, gb.spine[0].v, gb.spine[1].v, pa, pb);
      V A, B;
      Mt::addScaled3(A.v, pa, n, -ga.radius);
      Mt::addScaled3(B.v, pb, n, gb.radius);
      pairs.push_back({A, B});
    } else if (ga.round || gb.round) {
      const Geo& round = ga.round ? ga : gb;
      const Geo& poly = ga.round ? gb : ga;
      R dir[3];
      if (ga.round) Mt::scale3(dir, n, R(-1));
      else std::memcpy(dir, n, sizeof(dir));
      V pa = support(round, dir), pb;
      closestSurface(pb.v, poly, pa.v);
      if (ga.round) pairs.push_back({pa, pb});
      else pairs.push_back({pb, pa});
    } else if (edgeA >= 0) {
      V pa, pb;
      closestSegments(ga.vertices[ga.edges[edgeA][0]].v, ga.vertices[ga.edges[edgeA][1]].v, gb.vertices[gb.edges[edgeB][0]].v,
                      gb.vertices[gb.edges[edgeB][1]].v, pa.v, pb.v);
      pairs.push_back({pa, pb});
    }
    // (box-box never reaches this path: collideCpu3D sends it to collide())
    std::vector<Raw> out;
    for (int i = 0; i < int(pairs.size()) && i < 8; i++) {
      Raw r;
      r.feature = uint32_t(i + 1);
      R d[3];
      Mt::sub3(d, pairs[i].first.v, a.pos);
      Mt::rotateInv(r.rA, a.q, d);
      Mt::sub3(d, pairs[i].second.v, b.pos);
      Mt::rotateInv(r.rB, b.q, d);
      out.push_back(r);
    }
    return out;
  }
};

template <class R>
std::vector<typename Solver<R>::Raw> Solver<R>::collideGeneric(int ia, int ib, R* basis) const {
  return Generic<R>::run(bodies[ia], bodies[ib], basis);
}

}  // namespace avbd_oracle
