// The "gb300" backend of createSolverPipeline (src/native/pipeline.js:14-92) over the Node-API
// addon (avbd_addon.cc) and the engine's C ABI. A maintainer places this directory at
// src/native/gb300/ of the reference tree (the imports below are relative to that place), builds
// the addon with node-gyp, and lets pipeline.js accept backend "gb300":
//
//   if (backend === "gb300") return (await import("./gb300/index.js")).createGb300Pipeline(options);
//
// The world object offers the reference's native 3D world surface (src/native/scenes.d.ts:317-454);
// editBodies, advance, bodyIndex/body and the velocity setters come from the reference's own
// installNativeRuntime (src/native/runtime.js:324-410), which validates and stages exactly as the
// other backends do, and reach the engine through prepareBodyCommands / setVelocities here.
import { createRequire } from "node:module";
import { IgnoreCollision, Joint, Spring } from "../../../reference/three-avbd/src/avbd3d/ref/forces.ts";
import { isSphere } from "../../../reference/three-avbd/src/avbd3d/shapes.ts";
import { isCapsule } from "../../gpu/capsuleShape.js";
import { angularConstraintOptions, initialAngularConstraint } from "../../gpu/angularConstraints.js";
import { initialSpringMaterial, springMaterial } from "../../gpu/springMaterial.js";
import { installNativeRuntime } from "../runtime.js";

const require = createRequire(import.meta.url);
const addon = require("./build/Release/avbd_gb300.node");

const BROADPHASE = { grid: 0, hploc: 1, auto: 2 };
const INF = 3.4e38;

/** Body slots along a Z-order curve, 10 bits per axis (solver3D.ts:344-367), with static and
 * large bodies (radius above twice the median, at most 64) first in creation order: pairs are
 * enumerated by their higher-index body. */
export function spatialOrder(bodies) {
  const n = bodies.length;
  if (!n) return [];
  const radii = bodies.map((b) => b.radius).sort((a, b) => a - b);
  let thr = 2 * radii[Math.floor(n / 2)];
  if (radii.filter((r) => r > thr).length > 64) thr = radii[n - 65];
  const first = bodies.map((b) => !(b.mass > 0) || b.radius > thr);
  const rest = bodies.map((_, i) => i).filter((i) => !first[i]);
  const lo = [Infinity, Infinity, Infinity], hi = [-Infinity, -Infinity, -Infinity];
  for (const i of rest)
    for (let k = 0; k < 3; k++) {
      lo[k] = Math.min(lo[k], bodies[i].positionLin[k]);
      hi[k] = Math.max(hi[k], bodies[i].positionLin[k]);
    }
  const spread = (v) => {
    let x = v & 0x3ff;
    x = (x | (x << 16)) & 0x30000ff;
    x = (x | (x << 8)) & 0x300f00f;
    x = (x | (x << 4)) & 0x30c30c3;
    x = (x | (x << 2)) & 0x9249249;
    return x;
  };
  const code = new Map(rest.map((i) => {
    const q = [0, 1, 2].map((k) =>
      Math.min(1023, Math.floor(((bodies[i].positionLin[k] - lo[k]) / Math.max(hi[k] - lo[k], 1e-9)) * 1024)));
    return [i, (spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2)) >>> 0];
  }));
  rest.sort((a, b) => code.get(a) - code.get(b) || a - b);
  return bodies.map((_, i) => i).filter((i) => first[i]).concat(rest);
}

/** The scene as the structure of arrays of avbd_scene_desc, bodies in slot order. */
export function packScene(scene, options = {}) {
  const ref = scene.ref;
  const all = ref.bodies;
  const order = options.spatialSort === false ? all.map((_, i) => i) : spatialOrder(all);
  const slot = new Map(order.map((i, s) => [all[i], s]));
  const n = order.length;
  const a = {
    position: new Float32Array(3 * n), rotation: new Float32Array(4 * n), size: new Float32Array(3 * n),
    velocity: new Float32Array(3 * n), angularVelocity: new Float32Array(3 * n), prevVelocity: new Float32Array(3 * n),
    mass: new Float32Array(n), moment: new Float32Array(3 * n), friction: new Float32Array(n), radius: new Float32Array(n),
    shape: new Int32Array(n), group: new Uint32Array(n), collidesWith: new Uint32Array(n),
    restitution: new Float32Array(n), allowSleep: new Int32Array(n), isTrigger: new Int32Array(n),
  };
  order.forEach((i, s) => {
    const b = all[i];
    a.position.set(b.positionLin, 3 * s);
    a.rotation.set(b.positionAng, 4 * s);
    a.size.set(b.size, 3 * s);
    a.velocity.set(b.velocityLin, 3 * s);
    a.angularVelocity.set(b.velocityAng, 3 * s);
    a.prevVelocity.set(b.prevVelocityLin, 3 * s);
    a.moment.set(b.moment, 3 * s);
    a.mass[s] = b.mass;
    a.friction[s] = b.friction;
    a.radius[s] = b.radius;
    a.shape[s] = isSphere(b) ? 1 : isCapsule(b) ? 2 : 0;  // AVBD_SHAPE_BOX / SPHERE / CAPSULE
    a.group[s] = b.group ?? 0xffffffff;
    a.collidesWith[s] = b.collidesWith ?? 0xffffffff;
    a.restitution[s] = b.restitution ?? 0;
    a.allowSleep[s] = b.allowSleep === false ? 0 : 1;
    a.isTrigger[s] = b.isTrigger ? 1 : 0;
  });
  // joints, springs and ignore pairs in creation order (their order is the engine's joint id)
  const cons = ref.forces.filter((f) => f instanceof Joint || f instanceof Spring || f instanceof IgnoreCollision);
  const m = cons.length;
  Object.assign(a, {
    consKind: new Int32Array(m), consA: new Int32Array(m), consB: new Int32Array(m),
    consRA: new Float32Array(3 * m), consRB: new Float32Array(3 * m),
    consP0: new Float32Array(m), consP1: new Float32Array(m), consP2: new Float32Array(m),
    consP3: new Float32Array(m),
  });
  cons.forEach((f, c) => {
    a.consA[c] = f.bodyA ? slot.get(f.bodyA) : -1;
    a.consB[c] = slot.get(f.bodyB);
    const angular = f instanceof Joint ? initialAngularConstraint(f) : undefined;
    if (angular) {
      // addMotor / the limit row of addHinge (scenes.js:575-630): kinds 3 and 4 of the C ABI
      const motor = angular.type === "motor";
      a.consKind[c] = motor ? 3 : 4;
      a.consRA.set(angular.axisA, 3 * c);
      a.consRB.set(angular.axisB, 3 * c);
      a.consP0[c] = motor ? angular.speed : angular.minAngle;
      a.consP1[c] = motor ? angular.maxTorque : angular.maxAngle;
    } else if (f instanceof Joint) {
      a.consKind[c] = 0;
      a.consRA.set(f.rA, 3 * c);
      a.consRB.set(f.rB, 3 * c);
      a.consP0[c] = f.stiffnessLin;
      a.consP1[c] = f.stiffnessAng;
      a.consP2[c] = f.fracture;
    } else if (f instanceof Spring) {
      a.consKind[c] = 1;
      a.consRA.set(f.rA, 3 * c);
      a.consRB.set(f.rB, 3 * c);
      a.consP0[c] = f.stiffness;
      a.consP1[c] = f.rest;
      // tear limits (springMaterial.js; 0 = none): breakForce in p2, breakStrain in p3
      const material = initialSpringMaterial(f);
      a.consP2[c] = Number.isFinite(material?.breakForce) ? material.breakForce : 0;
      a.consP3[c] = Number.isFinite(material?.breakStrain) ? material.breakStrain : 0;
    } else {
      a.consKind[c] = 2;
    }
  });
  const sleeping = options.sleeping ?? (scene.sleepOptIn ? true : false);
  const params = {
    dt: ref.dt, gravity: ref.gravity, up: new Float32Array(scene.up), iterations: ref.iterations,
    alpha: ref.alpha, betaLin: ref.betaLin, betaAng: ref.betaAng, gamma: ref.gamma,
    massPenalty: 1, faceBias: 1, colorRounds: options.colorRounds ?? 64,
    broadphase: BROADPHASE[options.broadphase ?? "auto"], bvhRebuild: options.bvh?.rebuildInterval ?? 16,
    sleeping: sleeping ? 1 : 0, sleepSpeed: sleeping?.speedThreshold ?? 0.08, sleepTime: sleeping?.timeThreshold ?? 0.6,
  };
  if (params.broadphase === undefined) throw Error("broadphase must be 'grid', 'hploc' or 'auto'");
  return { arrays: a, params, order, jointCount: cons.filter((f) => !(f instanceof IgnoreCollision)).length };
}

class Gb300World {
  constructor(ctx, scene, options) {
    const packed = packScene(scene, options);
    this.ctx = ctx;
    this.handle = addon.createWorld(ctx, packed.arrays, packed.params);
    this.mass = packed.arrays.mass;  // per slot, for readBodyState(index)
    this.dimension = 3;
    this.bodyCount = packed.order.length;
    this.jointCount = packed.jointCount;
    this.params = { dt: packed.params.dt };
    this.timeAccumulator = 0;
    this.destroyed = false;
    this.slots = new Int32Array(this.bodyCount);
    packed.order.forEach((i, s) => (this.slots[i] = s));
    installNativeRuntime(this, { bodies: scene.ref.bodies }, 3, {
      setVelocities: this.setPackedVelocities,
      readSelectedBodies: this.readSelectedBodies,
    });
  }
  assertLive() {
    if (this.destroyed) throw Error("The solver has been destroyed");
  }
  liveIndex(index) {
    this.assertLive();
    if (!Number.isInteger(index) || index < 0 || index >= this.bodyCount) throw Error("A live body index is required");
  }
  gpuIndex(referenceIndex) {
    this.liveIndex(referenceIndex);
    return this.slots[referenceIndex];
  }
  step() {
    this.assertLive();
    addon.step(this.handle, 1);
    return this;
  }
  flushEdits() {
    this.assertLive();
    addon.flushEdits(this.handle);
    return this;
  }
  // the staged 12-word records of runtime.js editBodies
  prepareBodyCommands() {
    return { enqueueValidated: (commands) => addon.edit(this.handle, commands.u32.subarray(0, commands.count * 12)) };
  }
  // per-body commands of NativeBody handles (src/native/solver3D.js:140-190), staged by editBodies
  setLinearVelocity(index, v) {
    return this.editBodies([{ body: index, linearVelocity: v }]);
  }
  setAngularVelocity(index, v) {
    return this.editBodies([{ body: index, angularVelocity: v }]);
  }
  applyImpulse(index, v, point) {
    return this.editBodies([{ body: index, impulse: v, ...(point !== undefined ? { worldPoint: point } : {}) }]);
  }
  applyForce(index, v, point) {
    return this.editBodies([{ body: index, force: v, ...(point !== undefined ? { worldPoint: point } : {}) }]);
  }
  applyAngularImpulse(index, v) {
    return this.editBodies([{ body: index, angularImpulse: v }]);
  }
  applyTorque(index, v) {
    return this.editBodies([{ body: index, torque: v }]);
  }
  teleport(index, position, rotation) {
    return this.editBodies([{ body: index, position, ...(rotation !== undefined ? { rotation } : {}) }]);
  }
  setPoses(indices, positions, rotations) {
    this.assertLive();
    addon.setPoses(this.handle, Uint32Array.from(indices), Float32Array.from(positions),
      rotations ? Float32Array.from(rotations) : null);
    return this;
  }
  setPackedVelocities(indices, values) {
    if (values?.linear === undefined && values?.angular === undefined) throw Error("Provide linear or angular velocities");
    addon.setVelocities(this.handle, Uint32Array.from(indices),
      values.linear !== undefined ? Float32Array.from(values.linear) : null,
      values.angular !== undefined ? Float32Array.from(values.angular) : null);
    return this;
  }
  /** Resolves once the steps queued so far have run (a libuv worker waits, not the event loop);
   * the reads below await it, so the read itself finds the device idle. */
  deviceIdle() {
    return addon.fence(this.ctx);
  }
  async readSelectedBodies(indices, { posesOnly = false } = {}) {
    this.assertLive();
    await this.deviceIdle();
    return addon.readSelected(this.handle, Uint32Array.from(indices), posesOnly);
  }
  async readBodies() {
    return this.readSelectedBodies(Uint32Array.from({ length: this.bodyCount }, (_, i) => i));
  }
  /** readBodyState(index) (src/native/cpu/world.js:572-588): one body's state, from its 40-float
   * record (word 19 is its effective mass, 0 while it sleeps); without an index, every body. */
  async readBodyState(index) {
    this.assertLive();
    await this.deviceIdle();
    if (index === undefined) return addon.readState(this.handle, this.bodyCount);
    this.liveIndex(index);
    const r = addon.readSelected(this.handle, Uint32Array.of(index), false);
    const mass = this.mass[index];
    return {
      position: [r[0], r[1], r[2]], rotation: [r[4], r[5], r[6], r[7]],
      linearVelocity: [r[32], r[33], r[34]], angularVelocity: [r[36], r[37], r[38]],
      mass, effectiveMass: r[19], sleeping: mass > 0 && r[19] === 0,
    };
  }
  async readJoints() {
    this.assertLive();
    await this.deviceIdle();
    return addon.readJoints(this.handle, this.jointCount);
  }
  async readCounters() {
    this.assertLive();
    await this.deviceIdle();
    return addon.readCounters(this.handle);
  }
  setFilters(indices, groups, collidesWith) {
    this.assertLive();
    addon.setFilters(this.handle, Uint32Array.from(indices), Uint32Array.from(groups), Uint32Array.from(collidesWith));
  }
  setRestitution(index, value) {
    this.assertLive();
    addon.setRestitution(this.handle, Uint32Array.of(index), Float32Array.of(value));
  }
  /** setMotor(slot, { speed, maxTorque }) (appGpuSolver3D.js:547-562): slot is the joint slot. */
  setMotor(slot, options = {}) {
    this.assertLive();
    const o = angularConstraintOptions({ type: "motor", speed: options.speed ?? 0, maxTorque: options.maxTorque ?? 0 });
    addon.setMotor(this.handle, slot, options.speed === undefined ? undefined : o.speed,
      options.maxTorque === undefined ? undefined : o.maxTorque);
  }
  /** setSpringMaterial(slot, { breakStrain, breakForce }) (appGpuSolver3D.js:810-835). */
  setSpringMaterial(slot, options = {}) {
    this.assertLive();
    const m = springMaterial(options);
    addon.setSpringMaterial(this.handle, slot, options.breakStrain === undefined ? undefined : m.breakStrain,
      options.breakForce === undefined ? undefined : m.breakForce);
  }
  /** setWorldAnchor(slot, point) (appGpuSolver3D.js:928-941): move a world joint's anchor. */
  setWorldAnchor(slot, point) {
    this.assertLive();
    addon.setWorldAnchor(this.handle, slot, Float32Array.from(point));
  }
  /** captureConstraintFrames([{ slot, spring }]) (src/native/cpu/world.js:474-492). */
  captureConstraintFrames(entries) {
    this.assertLive();
    const list = Array.from(entries);
    addon.captureFrames(this.handle, Int32Array.from(list, (e) => e.slot), Int32Array.from(list, (e) => (e.spring ? 1 : 0)));
  }
  disableConstraint(slot) {
    this.releaseJoints([slot]);
  }
  /** releaseJoints(slots) (src/native/cpu/world.js:397-410). */
  releaseJoints(slots) {
    this.assertLive();
    addon.releaseJoints(this.handle, Int32Array.from(slots));
  }
  /** setSensor(index, enabled) (src/native/cpu/world.js:342-350). */
  setSensor(index, enabled) {
    this.liveIndex(index);
    if (typeof enabled !== "boolean") throw Error("isTrigger must be a boolean");
    addon.setSensor(this.handle, Uint32Array.of(index), enabled ? 1 : 0);
    return this;
  }
  setSleepEnabled(index, enabled) {
    this.liveIndex(index);
    addon.setSleepEnabled(this.handle, index, enabled);
    return this;
  }
  enableSleeping({ speedThreshold = 0.08, timeThreshold = 0.6 } = {}) {
    this.assertLive();
    addon.setSleeping(this.handle, true, speedThreshold, timeThreshold);
    return this;
  }
  disableSleeping() {
    this.assertLive();
    addon.setSleeping(this.handle, false, 0, 0);
    return this;
  }
  wakeAll() {
    this.assertLive();
    addon.wakeAll(this.handle);
    return this;
  }
  async readSleepStats() {
    this.assertLive();
    return { sleeping: addon.sleepStats(this.handle), wakeRequested: false };
  }
  watchContacts({ maxPairs = 8192, maxEvents = 4096, indices } = {}) {
    this.assertLive();
    addon.watchContacts(this.handle, indices === undefined ? null : Uint32Array.from(indices), maxPairs, maxEvents);
    return this;
  }
  async readContactEvents() {
    this.watchContacts();
    const { records, dropped, full } = addon.readContactEvents(this.handle);
    const f = new Float32Array(records.buffer, records.byteOffset, records.length);
    const events = [];
    for (let o = 0; o < records.length; o += 12)
      events.push({
        type: records[o] === 1 ? "begin" : "end", kind: records[o], a: records[o + 1], b: records[o + 2],
        step: records[o + 3], point: [f[o + 4], f[o + 5], f[o + 6]], impulse: f[o + 7],
        normal: [f[o + 8], f[o + 9], f[o + 10]], isTrigger: f[o + 11] !== 0,
      });
    return { events, dropped, full };
  }
  resetContactHistory(indices) {
    if (!(indices instanceof Uint32Array)) throw Error("Contact resets require Uint32 GPU slots");
    addon.resetContactHistory(this.handle, indices);
    return this;
  }
  async sphereCastAll(casts, options = {}) {
    this.assertLive();
    const q = new Float32Array(8 * casts.length);
    casts.forEach((c, i) => {
      const d = Array.from(c.direction), len = Math.hypot(...d);
      q.set([...c.origin, c.maxDistance ?? options.maxDistance ?? INF, ...d.map((x) => x / len), c.radius ?? 0], 8 * i);
    });
    const filter = {
      collidesWith: options.collidesWith ?? 0xffffffff,
      ...(options.membership !== undefined ? { membership: options.membership } : {}),
      ignore: Uint32Array.from(options.ignore ?? []),
    };
    const hits = casts.length ? addon.cast(this.handle, q, filter) : new Float32Array(0);
    const index = new Uint32Array(hits.buffer, hits.byteOffset, hits.length);
    return casts.map((c, i) => {
      const t = hits[8 * i + 3];
      if (t < 0) return null;
      const normal = [hits[8 * i], hits[8 * i + 1], hits[8 * i + 2]];
      const d = Array.from(c.direction), len = Math.hypot(...d);
      const center = c.origin.map((x, k) => x + (t * d[k]) / len);
      const r = c.radius ?? 0;
      return { index: index[8 * i + 4], distance: t, normal, center, point: center.map((x, k) => x - r * normal[k]) };
    });
  }
  async raycastAll(rays, options) {
    return this.sphereCastAll(rays.map((r) => ({ ...r, radius: 0 })), options);
  }
  async sphereCast(origin, radius, direction, options) {
    return (await this.sphereCastAll([{ origin, radius, direction }], options))[0];
  }
  async raycast(origin, direction, options) {
    return this.sphereCast(origin, 0, direction, options);
  }
  destroy() {
    if (this.destroyed) return;
    addon.destroyWorld(this.handle);
    this.destroyed = true;
  }
}

/** A request loop over the engine's world server (no counterpart in the reference, which creates
 * one solver per world). advance(id, steps) returns a promise of the world's poses after those
 * steps, 8 floats per body (position, friction, quaternion) in the scene's creation order.
 * Ticks are queued back to back, at most `depth` in flight on the device; each steps every world
 * with queued steps by up to `maxStepsPerTick` steps and captures the reply of every request it
 * completes. Admissions, edits and new requests made while ticks run join the next tick; nothing
 * here waits for the device on the event loop (the addon waits on a libuv worker). */
export class Gb300Server {
  constructor(ctx, { budgetBytes, initialBodies, initialWorlds, maxStepsPerTick = 16, depth = 2 } = {}) {
    this.ctx = ctx;
    this.handle = addon.createServer(ctx, budgetBytes, initialBodies, initialWorlds);
    this.maxSteps = maxStepsPerTick;
    this.depth = depth;
    this.orders = new Map();   // world id -> slot of each creation index
    this.waiting = new Map();  // ticket -> {id, resolve, reject}
    this.inFlight = 0;
    this.scheduled = false;
    this.destroyed = false;
  }
  assertLive() {
    if (this.destroyed) throw Error("The server has been destroyed");
  }
  /** Admit a scene (createSolver under the server's device-memory budget); returns the world id.
   * Throws when the world cannot fit even after evicting every idle world. */
  admit(scene, solverOptions = {}) {
    this.assertLive();
    const packed = packScene(scene, solverOptions);
    const id = addon.admit(this.handle, packed.arrays, packed.params);
    const slots = new Int32Array(packed.order.length);
    packed.order.forEach((i, s) => (slots[i] = s));
    this.orders.set(id, slots);
    scene.created = true;
    return id;
  }
  /** Queue `steps` steps of a world; resolves with its poses after them. */
  advance(id, steps) {
    this.assertLive();
    const ticket = addon.advance(this.handle, id, steps);
    if (steps === 0) return this.readPoses([id]);
    return new Promise((resolve, reject) => {
      this.waiting.set(ticket, { id, resolve, reject });
      this.schedule();
    });
  }
  /** Poses of the listed worlds once the ticks queued so far have run, world after world. */
  async readPoses(ids) {
    this.assertLive();
    const bodies = ids.reduce((n, id) => n + this.orders.get(id).length, 0);
    const poses = await addon.readPosesAsync(this.ctx, this.handle, Float64Array.from(ids), bodies);
    let at = 0;
    const out = new Float32Array(poses.length);
    for (const id of ids) {
      const slots = this.orders.get(id);
      out.set(this.creationOrder(poses.subarray(8 * at, 8 * (at + slots.length)), slots), 8 * at);
      at += slots.length;
    }
    return out;
  }
  creationOrder(poses, slots) {
    const out = new Float32Array(poses.length);
    for (let i = 0; i < slots.length; i++) out.set(poses.subarray(8 * slots[i], 8 * slots[i] + 8), 8 * i);
    return out;
  }
  edit(id, records) {
    this.assertLive();
    addon.serverEdit(this.handle, id, records);
  }
  evict(id) {
    this.assertLive();
    addon.evict(this.handle, id);
  }
  release(id) {
    this.assertLive();
    addon.release(this.handle, id);
    this.orders.delete(id);
  }
  stats() {
    return addon.serverStats(this.handle);
  }
  schedule() {
    if (this.scheduled || this.destroyed) return;
    this.scheduled = true;
    setImmediate(() => {
      this.scheduled = false;
      this.pump();
    });
  }
  pump() {
    while (!this.destroyed && this.inFlight < this.depth && addon.serverStats(this.handle).pendingWorlds > 0) {
      this.inFlight++;
      addon.tickAsync(this.ctx, this.handle, this.maxSteps).then(
        ({ replies }) => {
          this.inFlight--;
          for (const { ticket, poses } of replies ?? []) {
            const req = this.waiting.get(ticket);
            if (!req) continue;
            this.waiting.delete(ticket);
            req.resolve(this.creationOrder(poses, this.orders.get(req.id)));
          }
          this.schedule();
        },
        (err) => {
          this.inFlight--;
          for (const req of this.waiting.values()) req.reject(err);
          this.waiting.clear();
        },
      );
    }
  }
  destroy() {
    if (this.destroyed) return;
    this.destroyed = true;
    for (const req of this.waiting.values()) req.reject(Error("The server has been destroyed"));
    this.waiting.clear();
    addon.synchronize(this.ctx);
    addon.destroyServer(this.handle);
  }
}

/** createSolverPipeline({backend: "gb300", deviceIndex}) */
export function createGb300Pipeline(options = {}) {
  const ctx = addon.createContext(options.deviceIndex ?? 0);
  const worlds = new Set();
  const servers = new Set();
  return {
    backend: "gb300",
    createSolver(scene, solverOptions = {}) {
      const w = new Gb300World(ctx, scene, solverOptions);
      scene.created = true;
      worlds.add(w);
      return w;
    },
    createServer(serverOptions = {}) {
      const server = new Gb300Server(ctx, serverOptions);
      servers.add(server);
      return server;
    },
    destroy() {
      for (const w of worlds) w.destroy();
      worlds.clear();
      for (const s of servers) s.destroy();
      servers.clear();
      addon.destroyContext(ctx);
    },
  };
}
