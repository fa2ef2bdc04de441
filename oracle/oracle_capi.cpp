// AVBD CPU ORACLE -- test infrastructure only (see avbd_oracle.hpp). C entry points for
// ctypes: build a world from flat arrays, step it in the reference's sequential order or in
// the GPU engine's colour order, read state back, import a full solver state (bodies, joints,
// manifolds with their warm-start contacts, colours) so one step can be compared with the
// CUDA engine from the same starting point, and run single narrowphase calls.
#include <omp.h>

#include <cstdio>

#include "avbd_oracle.hpp"

using namespace avbd_oracle;

// Constraint kinds, in the scene's creation order (the order matters: it is the order of the
// reference's force lists).
enum { K_JOINT = 0, K_SPRING = 1, K_IGNORE = 2, K_MOTOR = 3, K_LIMIT = 4 };

struct oracle_scene {
  int n_bodies;
  const double* pos;       // 3n
  const double* quat;      // 4n (x, y, z, w)
  const double* size;      // 3n full extents (spheres: 2r each)
  const double* vel;       // 3n
  const double* angvel;    // 3n
  const double* prev_vel;  // 3n
  const double* mass;      // n
  const double* moment;    // 3n
  const double* friction;  // n
  const double* radius;    // n
  const int32_t* shape;    // n: 0 box, 1 sphere
  const uint32_t* group;   // n
  const uint32_t* mask;    // n
  int n_cons;
  const int32_t* kind;  // n_cons
  const int32_t* ca;    // -1 = world
  const int32_t* cb;
  const double* ra;  // 3 n_cons
  const double* rb;  // 3 n_cons
  const double* p0;  // joint: linear stiffness; spring: stiffness
  const double* p1;  // joint: angular stiffness; spring: rest (-1: current distance)
  const double* p2;  // joint: fracture
  const double* restitution;  // n (null: 0)
  const int32_t* allow_sleep;  // n (null: 1)
  const double* p3;            // n_cons spring: breakStrain (null, <= 0 or inf: none); p2: breakForce
  const int32_t* is_trigger;   // n (null: 0)
};

struct oracle_params {
  double dt, gravity;
  double up[3];
  int iterations;
  double alpha, beta_lin, beta_ang, gamma;
  int app, mass_penalty, face_bias, colored, color_rounds;
  int sleeping;
  double sleep_speed, sleep_time;
};

struct OracleWorld {
  int fp64;
  Solver<double>* d = nullptr;
  Solver<float>* f = nullptr;
};

template <class R> static Solver<R>* build(const oracle_scene* s, const oracle_params* p) {
  auto* w = new Solver<R>();
  w->dt = R(p->dt);
  w->gravity = R(p->gravity);
  w->iterations = p->iterations;
  w->alpha = R(p->alpha);
  w->betaLin = R(p->beta_lin);
  w->betaAng = R(p->beta_ang);
  w->gamma = R(p->gamma);
  w->app = p->app != 0;
  w->massPenalty = p->mass_penalty != 0;
  w->faceBias = p->face_bias != 0;
  for (int i = 0; i < 3; i++) w->up[i] = R(p->up[i]);
  w->colored = p->colored != 0;
  w->colorRounds = p->color_rounds > 0 ? p->color_rounds : 64;
  w->sleepOn = p->sleeping != 0;
  w->sleepSpeed = R(p->sleep_speed);
  w->sleepDelay = R(p->sleep_time);
  for (int i = 0; i < s->n_bodies; i++) {
    Body<R> b;
    for (int k = 0; k < 3; k++) {
      b.pos[k] = R(s->pos[3 * i + k]);
      b.size[k] = R(s->size[3 * i + k]);
      b.v[k] = R(s->vel[3 * i + k]);
      b.w[k] = R(s->angvel[3 * i + k]);
      b.vprev[k] = R(s->prev_vel[3 * i + k]);
      b.moment[k] = R(s->moment[3 * i + k]);
    }
    for (int k = 0; k < 4; k++) b.q[k] = R(s->quat[4 * i + k]);
    b.mass = R(s->mass[i]);
    b.friction = R(s->friction[i]);
    b.radius = R(s->radius[i]);
    b.shape = s->shape[i];
    b.group = s->group ? s->group[i] : 0xffffffffu;
    b.mask = s->mask ? s->mask[i] : 0xffffffffu;
    b.restitution = s->restitution ? R(s->restitution[i]) : R(0);
    b.allowSleep = s->allow_sleep ? s->allow_sleep[i] != 0 : true;
    b.isTrigger = s->is_trigger ? s->is_trigger[i] != 0 : false;
    w->addBody(b);
  }
  for (int c = 0; c < s->n_cons; c++) {
    R ra[3], rb[3];
    for (int k = 0; k < 3; k++) { ra[k] = R(s->ra[3 * c + k]); rb[k] = R(s->rb[3 * c + k]); }
    if (s->kind[c] == K_JOINT) w->addJoint(s->ca[c], s->cb[c], ra, rb, R(s->p0[c]), R(s->p1[c]), R(s->p2[c]));
    else if (s->kind[c] == K_SPRING) {
      int id = w->addSpring(s->ca[c], s->cb[c], ra, rb, R(s->p0[c]), R(s->p1[c]));
      auto limit = [](double x) { return x > 0 && std::isfinite(float(x)) ? R(float(x)) : std::numeric_limits<R>::infinity(); };
      w->store[id]->breakForce = limit(s->p2[c]);
      w->store[id]->breakStrain = limit(s->p3 ? s->p3[c] : 0.0);
    }
    else if (s->kind[c] == K_MOTOR || s->kind[c] == K_LIMIT)
      w->addAngular(s->ca[c], s->cb[c], s->kind[c], ra, rb, R(s->p0[c]), R(s->p1[c]));
    else w->addIgnore(s->ca[c], s->cb[c]);
  }
  if (w->app) w->prepareApp();
  return w;
}

extern "C" void* oracle_world_create(int fp64, const oracle_scene* s, const oracle_params* p) {
  auto* w = new OracleWorld();
  w->fp64 = fp64;
  if (fp64) w->d = build<double>(s, p);
  else w->f = build<float>(s, p);
  return w;
}

extern "C" void oracle_world_destroy(void* h) {
  auto* w = static_cast<OracleWorld*>(h);
  delete w->d;
  delete w->f;
  delete w;
}

#define DISPATCH(h, ...)                              \
  do {                                                \
    auto* w_ = static_cast<OracleWorld*>(h);          \
    if (w_->fp64) { auto& S = *w_->d; __VA_ARGS__; }  \
    else { auto& S = *w_->f; __VA_ARGS__; }           \
  } while (0)

extern "C" void oracle_world_step(void* h, int steps) {
  DISPATCH(h, for (int i = 0; i < steps; i++) S.step());
}
extern "C" void oracle_world_step_collide(void* h) { DISPATCH(h, S.stepCollide()); }
extern "C" void oracle_world_step_solve(void* h) { DISPATCH(h, S.stepSolve()); }
extern "C" void oracle_world_set_colored(void* h, int colored) { DISPATCH(h, S.colored = colored != 0); }

// Sleep state per body: sleeping flag and accumulated quiet time (import for one-step parity).
extern "C" void oracle_world_set_sleep(void* h, const int32_t* asleep, const double* time) {
  DISPATCH(h, {
    const int n = int(S.bodies.size());
    S.sleepTime.assign(n, 0);
    for (int i = 0; i < n; i++) {
      S.bodies[i].sleeping = asleep[i] != 0;
      S.sleepTime[i] = decltype(S.dt)(time[i]);
    }
  });
}
extern "C" int oracle_world_sleep_state(void* h, int32_t* asleep, double* time) {
  int count = 0;
  DISPATCH(h, {
    const int n = int(S.bodies.size());
    for (int i = 0; i < n; i++) {
      asleep[i] = S.bodies[i].sleeping ? 1 : 0;
      time[i] = i < int(S.sleepTime.size()) ? double(S.sleepTime[i]) : 0.0;
      count += asleep[i];
    }
  });
  return count;
}
extern "C" void oracle_world_wake_all(void* h) { DISPATCH(h, S.wakeAll()); }
extern "C" void oracle_world_sleep_after(void* h) { DISPATCH(h, S.sleepAfter()); }

extern "C" int oracle_world_body_count(void* h) {
  int n = 0;
  DISPATCH(h, n = int(S.bodies.size()));
  return n;
}
extern "C" int oracle_world_force_count(void* h) {
  int n = 0;
  DISPATCH(h, n = S.forceCount());
  return n;
}
// Counts by kind of the live force list: out[0] manifolds, [1] joints, [2] springs, [3] ignores,
// [4] contacts, [5] colours used by the last coloured step, [6] colouring conflicts.
extern "C" void oracle_world_counts(void* h, int* out) {
  for (int i = 0; i < 7; i++) out[i] = 0;
  DISPATCH(h, {
    for (int id : S.forces) {
      const auto& f = *S.store[id];
      out[f.type]++;
      if (f.type == F_MANIFOLD) out[4] += int(f.contacts.size());
    }
    out[5] = S.lastNumColors;
    out[6] = S.lastConflicts;
  });
}

extern "C" void oracle_world_read_bodies(void* h, double* pos, double* quat, double* vel, double* angvel, double* prev_vel) {
  DISPATCH(h, {
    for (size_t i = 0; i < S.bodies.size(); i++) {
      const auto& b = S.bodies[i];
      for (int k = 0; k < 3; k++) {
        if (pos) pos[3 * i + k] = double(b.pos[k]);
        if (vel) vel[3 * i + k] = double(b.v[k]);
        if (angvel) angvel[3 * i + k] = double(b.w[k]);
        if (prev_vel) prev_vel[3 * i + k] = double(b.vprev[k]);
      }
      if (quat) for (int k = 0; k < 4; k++) quat[4 * i + k] = double(b.q[k]);
    }
  });
}

extern "C" void oracle_world_read_colors(void* h, int32_t* out) {
  DISPATCH(h, {
    for (size_t i = 0; i < S.bodies.size(); i++) out[i] = i < S.colors.size() ? S.colors[i] : -1;
  });
}

// Live manifolds as (hi, lo) pairs sorted ascending, with their contact counts.
extern "C" int oracle_world_manifolds(void* h, int32_t* pairs, int32_t* counts, int cap) {
  int n = 0;
  DISPATCH(h, {
    std::vector<std::tuple<int, int, int>> v;
    for (int id : S.forces) {
      const auto& f = *S.store[id];
      if (f.type == F_MANIFOLD) v.emplace_back(f.a, f.b, int(f.contacts.size()));
    }
    std::sort(v.begin(), v.end());
    n = int(v.size());
    for (int i = 0; i < n && i < cap; i++) {
      pairs[2 * i] = std::get<0>(v[i]);
      pairs[2 * i + 1] = std::get<1>(v[i]);
      counts[i] = std::get<2>(v[i]);
    }
  });
  return n;
}

// The app broadphase's pair predicate (cpuPhysics3D.js:319-343) evaluated on the current
// poses for every body pair, without creating manifolds: bounding spheres overlap, not both
// static, collision masks allow it, and no joint/spring/ignore links the two. Sorted (hi, lo).
extern "C" int oracle_world_candidate_pairs(void* h, int32_t* out, int cap) {
  int n = 0;
  DISPATCH(h, {
    using Rt = std::remove_reference_t<decltype(S.bodies[0].pos[0])>;
    const int nb = int(S.bodies.size());
    std::vector<std::pair<int, int>> linked;
    for (int id : S.forces) {
      const auto& f = *S.store[id];
      if (f.type == F_MANIFOLD || f.a < 0) continue;
      linked.emplace_back(std::max(f.a, f.b), std::min(f.a, f.b));
    }
    std::sort(linked.begin(), linked.end());
    std::vector<std::pair<int, int>> res;
    for (int hi = 0; hi < nb; hi++)
      for (int lo = 0; lo < hi; lo++) {
        const auto& A = S.bodies[hi];
        const auto& B = S.bodies[lo];
        if (A.mass <= 0 && B.mass <= 0) continue;
        if (!(A.group & B.mask) || !(B.group & A.mask)) continue;
        Rt r = A.radius + B.radius;
        Rt d[3] = {A.pos[0] - B.pos[0], A.pos[1] - B.pos[1], A.pos[2] - B.pos[2]};
        if (!(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] <= r * r)) continue;
        if (std::binary_search(linked.begin(), linked.end(), std::make_pair(hi, lo))) continue;
        res.emplace_back(hi, lo);
      }
    n = int(res.size());
    for (int i = 0; i < n && i < cap; i++) {
      out[2 * i] = res[i].first;
      out[2 * i + 1] = res[i].second;
    }
  });
  return n;
}

// One narrowphase call on two bodies of the world (hi = A, lo = B), on the current poses.
// Returns the contact count; basis9, features and local anchors (3 per contact) if non-null.
extern "C" int oracle_world_collide(void* h, int a, int b, double* basis9, uint32_t* features, double* ra, double* rb) {
  int n = 0;
  DISPATCH(h, {
    using Rt = std::remove_reference_t<decltype(S.bodies[0].pos[0])>;
    Rt basis[9] = {0};
    auto raw = S.narrowphase(a, b, basis);
    n = int(raw.size());
    if (basis9) for (int i = 0; i < 9; i++) basis9[i] = double(basis[i]);
    for (int i = 0; i < n; i++) {
      if (features) features[i] = raw[i].feature;
      for (int k = 0; k < 3; k++) {
        if (ra) ra[3 * i + k] = double(raw[i].rA[k]);
        if (rb) rb[3 * i + k] = double(raw[i].rB[k]);
      }
    }
  });
  return n;
}

// Replace the solver state: body kinematics, joint warm-start state, manifolds with their
// contacts (features, anchors, penalties, lambdas, stick flags) and colours. Manifolds are
// recreated after the joints in the given order; joints keep their creation order.
struct oracle_state {
  const double *pos, *quat, *vel, *angvel, *prev_vel;  // per body
  const double *jpen_lin, *jpen_ang, *jlam_lin, *jlam_ang;  // 3 per joint/spring (jid order)
  const int32_t* jbroken;
  int n_manifolds;
  const int32_t* mpairs;   // 2 per manifold (hi, lo)
  const int32_t* mcount;   // contacts per manifold
  const uint32_t* cfeature;  // flattened contacts
  const double *cra, *crb, *cpen, *clam;  // 3 per contact
  const int32_t* cstick;
  const int32_t* colors;  // per body (-1 none), or null
};

template <class R> static void import_state(Solver<R>& S, const oracle_state* st) {
  for (size_t i = 0; i < S.bodies.size(); i++) {
    auto& b = S.bodies[i];
    for (int k = 0; k < 3; k++) {
      b.pos[k] = R(st->pos[3 * i + k]);
      b.v[k] = R(st->vel[3 * i + k]);
      b.w[k] = R(st->angvel[3 * i + k]);
      b.vprev[k] = R(st->prev_vel[3 * i + k]);
    }
    for (int k = 0; k < 4; k++) b.q[k] = R(st->quat[4 * i + k]);
  }
  // drop manifolds, reset joints
  std::vector<int> kept;
  for (int id : S.forces) {
    auto& f = *S.store[id];
    if (f.type == F_MANIFOLD) { S.unlinkFromBodies(id); continue; }
    kept.push_back(id);
  }
  S.forces.swap(kept);
  for (auto& fp : S.store) {
    auto& f = *fp;
    if (f.jid < 0) continue;
    int j = f.jid;
    for (int k = 0; k < 3; k++) {
      f.penLin[k] = R(st->jpen_lin[3 * j + k]);
      f.penAng[k] = R(st->jpen_ang[3 * j + k]);
      f.lamLin[k] = R(st->jlam_lin[3 * j + k]);
      f.lamAng[k] = R(st->jlam_ang[3 * j + k]);
    }
    // the engine's flag: 1 gone; 2 broken in the last step (still in the bodies' lists until
    // the next initialize pass, after the broadphase)
    if (st->jbroken[j] != 0 && !f.broken) {
      f.broken = true;
      if (st->jbroken[j] == 1) {
        auto it = std::find(S.forces.begin(), S.forces.end(), int(&fp - &S.store[0]));
        if (it != S.forces.end()) { S.unlinkFromBodies(*it); S.forces.erase(it); }
      }
    }
  }
  int c = 0;
  for (int m = 0; m < st->n_manifolds; m++) {
    int id = S.newForce(F_MANIFOLD, st->mpairs[2 * m], st->mpairs[2 * m + 1]);
    auto& f = *S.store[id];
    for (int k = 0; k < st->mcount[m]; k++, c++) {
      Contact<R> ct;
      ct.feature = st->cfeature[c];
      for (int q = 0; q < 3; q++) {
        ct.rA[q] = R(st->cra[3 * c + q]);
        ct.rB[q] = R(st->crb[3 * c + q]);
        ct.pen[q] = R(st->cpen[3 * c + q]);
        ct.lam[q] = R(st->clam[3 * c + q]);
      }
      ct.stick = st->cstick[c] != 0;
      f.contacts.push_back(ct);
    }
  }
  if (st->colors) {
    S.colors.assign(S.bodies.size(), -1);
    for (size_t i = 0; i < S.bodies.size(); i++) S.colors[i] = st->colors[i];
  }
}

extern "C" void oracle_world_import(void* h, const oracle_state* st) { DISPATCH(h, import_state(S, st)); }

// src/native/cpu/world.js:229-300 flushEdits over n 12-word body command records
extern "C" int oracle_world_set_motor(void* h, int jid, int mask, double speed, double torque) {
  int ok = 0;
  DISPATCH(h, ok = S.setMotor(jid, mask, decltype(S.dt)(speed), decltype(S.dt)(torque)) ? 1 : 0);
  return ok;
}
extern "C" void oracle_world_release_joints(void* h, const int32_t* jids, int n) {
  DISPATCH(h, for (int k = 0; k < n; k++) S.releaseJoint(jids[k]));
}

extern "C" int oracle_world_set_spring_material(void* h, int jid, int mask, double strain, double force) {
  int ok = 0;
  DISPATCH(h, ok = S.setSpringMaterial(jid, mask, decltype(S.dt)(strain), decltype(S.dt)(force)) ? 1 : 0);
  return ok;
}
extern "C" int oracle_world_set_world_anchor(void* h, int jid, const double* point) {
  int ok = 0;
  DISPATCH(h, {
    decltype(S.dt) p[3] = {decltype(S.dt)(point[0]), decltype(S.dt)(point[1]), decltype(S.dt)(point[2])};
    ok = S.setWorldAnchor(jid, p) ? 1 : 0;
  });
  return ok;
}
extern "C" int oracle_world_capture_frame(void* h, int jid, int spring) {
  int ok = 0;
  DISPATCH(h, ok = S.captureFrame(jid, spring != 0) ? 1 : 0);
  return ok;
}

extern "C" void oracle_world_set_sensor(void* h, const int32_t* idx, int n, int enabled) {
  DISPATCH(h, for (int k = 0; k < n; k++) S.bodies[idx[k]].isTrigger = enabled != 0);
}

// The angular rows' atan2 restatement, elementwise (fp64 != 0: double, else float).
extern "C" void oracle_angle_atan2(int fp64, const double* y, const double* x, double* out, int n) {
  for (int i = 0; i < n; i++)
    out[i] = fp64 ? Solver<double>::angleAtan2(y[i], x[i]) : double(Solver<float>::angleAtan2(float(y[i]), float(x[i])));
}

extern "C" void oracle_world_edit(void* h, const uint32_t* records, int n) { DISPATCH(h, S.applyEdits(records, n)); }

// Step many independent worlds in parallel with OpenMP (the multi-world CPU baseline).
// Returns the thread count used.
extern "C" int oracle_worlds_step_parallel(void** hs, int n, int steps, int threads) {
  if (threads > 0) omp_set_num_threads(threads);
  int used = 1;
#pragma omp parallel
  {
#pragma omp single
    used = omp_get_num_threads();
#pragma omp for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) oracle_world_step(hs[i], steps);
  }
  return used;
}

