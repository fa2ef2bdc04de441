// Ray and sphere casts against one world's current poses (raycast / sphereCast / raycastAll /
// sphereCastAll of src/native/solver3D.js:236-252 and src/native/cpu/world.js:824-856, computed
// as the GPU backend's shape queries, src/gpu/shapeQueries.wgsl).
//
// Per query and body: the query is moved into the body's frame; a sphere is hit as a sphere of
// radius r + R; a box with r = 0 by the slab test over its six face planes; a box with r > 0 as a
// rounded box: its six faces pushed out by r (a face hit counts where the touching point lies on
// the face) and its twelve edges as capsules of radius r. An origin inside the (rounded) shape
// hits at t = 0 with normal -d. Hits past the query's maximum distance are misses. The nearest hit
// wins; among equal distances the lowest body index. The normal is turned back to world space.
//
// GB300 arrangement: one launch over (body blocks) x (queries); each thread traces one body and
// the block reduces (distance bits << 32 | index), which orders as (distance, index) for
// distances >= 0, to one 64-bit atomicMin per block; a second launch re-traces each query's
// winner for its normal.
#include "engine.cuh"

namespace avbd {
namespace {

struct Hit {
  float t;
  V3 n;
};

__device__ __forceinline__ Hit miss() { return Hit{-1.f, V3{0.f, 0.f, 0.f}}; }

__device__ __forceinline__ V3 closest_on(V3 a, V3 b, V3 p) {
  const V3 e = b - a;
  const float s = clampr(dot(p - a, e) / fmaxf(dot(e, e), 1e-20f), 0.f, 1.f);
  return a + e * s;
}

__device__ Hit ray_sphere(V3 o, V3 d, V3 c, float r) {
  const V3 v = o - c;
  const float b = dot(v, d);
  const float disc = b * b - dot(v, v) + r * r;
  if (disc < 0.f) return miss();
  const float t = -b - sqrtf(disc);
  if (t < 0.f) return miss();
  const V3 p = o + d * t - c;
  const float len = sqrtf(dot(p, p));
  return Hit{t, len > 1e-10f ? vdiv(p, fmaxf(len, 1e-20f)) : -d};
}

__device__ Hit ray_capsule(V3 o, V3 d, V3 a, V3 b, float r) {
  const V3 ba = b - a, oa = o - a;
  const float bb = dot(ba, ba);
  if (bb < 1e-16f) return ray_sphere(o, d, a, r);
  const float bd = dot(ba, d), bo = dot(ba, oa), od = dot(oa, d);
  const float A = bb - bd * bd, B = bb * od - bo * bd, Cc = bb * dot(oa, oa) - bo * bo - r * r * bb;
  Hit hit = miss();
  const float disc = B * B - A * Cc;
  if (A > 1e-12f * bb && disc >= 0.f) {
    const float t = (-B - sqrtf(disc)) / A;
    const float y = bo + t * bd;
    if (t >= 0.f && y >= 0.f && y <= bb) {
      const V3 p = o + d * t;
      const V3 q = p - (a + vdiv(ba * y, bb));
      hit = Hit{t, vdiv(q, sqrtf(dot(q, q)))};
    }
  }
  for (int end = 0; end < 2; end++) {
    const Hit h = ray_sphere(o, d, end ? b : a, r);
    if (h.t >= 0.f && (hit.t < 0.f || h.t < hit.t)) hit = h;
  }
  return hit;
}

// Box corner v: bit k of v selects +h or -h on axis k.
__device__ __forceinline__ V3 corner(int v, V3 h) {
  return V3{(v & 1) ? h.x : -h.x, (v & 2) ? h.y : -h.y, (v & 4) ? h.z : -h.z};
}

// Face f = 2k + s: the plane of axis k with outward normal +e_k (s = 0) or -e_k (s = 1), offset
// h[k]; its corners in cyclic order around the face.
__device__ __forceinline__ V3 face_normal(int f) {
  const float s = (f & 1) ? -1.f : 1.f;
  const int k = f >> 1;
  return V3{k == 0 ? s : 0.f, k == 1 ? s : 0.f, k == 2 ? s : 0.f};
}
__device__ __forceinline__ int face_corner(int f, int j) {
  const int k = f >> 1, u = (k + 1) % 3, v = (k + 2) % 3;
  const int cu = (j == 1 || j == 2) ? 1 : 0, cv = (j >= 2) ? 1 : 0;
  return ((f & 1) ? 0 : (1 << k)) | (cu << u) | (cv << v);
}

// p on face f: inside every edge of the face polygon, with a 1e-6 tolerance
__device__ bool on_face(V3 p, int f, V3 h) {
  const V3 n = face_normal(f);
  V3 c{0.f, 0.f, 0.f};
  for (int j = 0; j < 4; j++) c = c + corner(face_corner(f, j), h);
  c = vdiv(c, 4.f);
  for (int j = 0; j < 4; j++) {
    const V3 a = corner(face_corner(f, j), h), b = corner(face_corner(f, (j + 1) & 3), h);
    const V3 side = cross(b - a, n);
    const float sg = dot(side, c - a) >= 0.f ? 1.f : -1.f;
    if (dot(side, p - a) * sg < -1e-6f) return false;
  }
  return true;
}

__device__ Hit ray_box(V3 o, V3 d, V3 h, float r) {
  if (r == 0.f) {
    float enter = -3.4e38f, exit = 3.4e38f;
    V3 normal = -d;
    for (int f = 0; f < 6; f++) {
      const V3 n = face_normal(f);
      const float w = comp(h, f >> 1);
      const float denom = dot(n, d), gap = w - dot(n, o);
      if (fabsf(denom) < 1e-12f) {
        if (gap < 0.f) return miss();
      } else {
        const float t = gap / denom;
        if (denom < 0.f) {
          if (t > enter) {
            enter = t;
            normal = n;
          }
        } else {
          exit = fminf(exit, t);
        }
      }
      if (enter > exit) return miss();
    }
    if (exit < 0.f) return miss();
    if (enter <= 0.f) return Hit{0.f, -d};
    return Hit{enter, normal};
  }
  bool inside = true;
  float distance = 3.4e38f;
  Hit hit = miss();
  for (int f = 0; f < 6; f++) {
    const V3 n = face_normal(f);
    const float w = comp(h, f >> 1);
    const float signed_ = dot(n, o) - w;
    if (signed_ > 0.f) inside = false;
    if (on_face(o - n * signed_, f, h)) distance = fminf(distance, signed_ * signed_);
    const float denom = dot(n, d);
    if (denom < -1e-12f) {
      const float t = (w + r - dot(n, o)) / denom;
      if (t >= 0.f && (hit.t < 0.f || t < hit.t) && on_face(o + d * t - n * r, f, h)) hit = Hit{t, n};
    }
  }
  for (int v = 0; v < 8; v++)
    for (int k = 0; k < 3; k++) {
      if (v & (1 << k)) continue;  // each edge once: from the corner with bit k clear
      const V3 a = corner(v, h), b = corner(v | (1 << k), h);
      const V3 q = o - closest_on(a, b, o);
      distance = fminf(distance, dot(q, q));
      const Hit c = ray_capsule(o, d, a, b, r);
      if (c.t >= 0.f && (hit.t < 0.f || c.t < hit.t)) hit = c;
    }
  if (inside || distance <= r * r) return Hit{0.f, -d};
  return hit;
}

__device__ Hit trace(const BodyPtrs& bd, int i, const CastQuery& q) {
  const float4 p4 = bd.pos(i), rq = bd.rot(i), sz = bd.size[i];
  const float4 inv = make_float4(-rq.x, -rq.y, -rq.z, rq.w);
  const V3 o = rotate(inv, v3(q.o) - v3(p4)), d = rotate(inv, v3(q.d));
  const float r = q.d.w;
  Hit hit;
  const int shape = bd.meta[i].y;
  if (shape == SHAPE_SPHERE) {
    const float radius = sz.x * 0.5f + r;
    hit = dot(o, o) <= radius * radius ? Hit{0.f, -d} : ray_sphere(o, d, V3{0.f, 0.f, 0.f}, radius);
  } else if (shape == SHAPE_CAPSULE) {  // its segment along local Y, radius + r (shapeQueries.wgsl trace)
    const float half = fmaxf(0.f, sz.y * 0.5f - sz.x * 0.5f);
    const V3 a{0.f, -half, 0.f}, b{0.f, half, 0.f};
    const float radius = sz.x * 0.5f + r;
    const V3 delta = o - closest_on(a, b, o);
    hit = dot(delta, delta) <= radius * radius ? Hit{0.f, -d} : ray_capsule(o, d, a, b, radius);
  } else {
    hit = ray_box(o, d, V3{sz.x * 0.5f, sz.y * 0.5f, sz.z * 0.5f}, r);
  }
  if (hit.t > q.o.w) return miss();
  hit.n = rotate(rq, hit.n);
  return hit;
}

__device__ __forceinline__ bool filtered(const BodyPtrs& bd, int i, int local, const CastFilter& f) {
  const int4 m = bd.meta[i];  // (world, shape, group, collidesWith)
  if ((uint32_t(m.z) & f.collidesWith) == 0u) return true;
  if (!f.includeTriggers && (bd.sleep[i] & BODY_TRIGGER)) return true;  // queries.js:229-233
  if (f.hasMembership && (f.membership == 0u || (uint32_t(m.w) & f.membership) == 0u)) return true;
  for (int k = 0; k < f.nIgnore; k++)
    if (int(f.ignore[k]) == local) return true;
  return false;
}

constexpr unsigned long long NO_HIT = ~0ull;

__global__ void k_cast_init(unsigned long long* best, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) best[k] = NO_HIT;
}

__global__ void k_cast_nearest(BodyPtrs bd, int off, int nb, const CastQuery* __restrict__ qs, CastFilter f,
                               unsigned long long* best) {
  __shared__ unsigned long long warpBest[8];
  const CastQuery q = qs[blockIdx.y];
  const int local = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long key = NO_HIT;
  if (local < nb && !filtered(bd, off + local, local, f)) {
    const Hit h = trace(bd, off + local, q);
    if (h.t >= 0.f) key = (unsigned long long)__float_as_uint(fmaxf(0.f, h.t)) << 32 | uint32_t(local);
  }
  for (int s = 16; s > 0; s >>= 1) {
    const unsigned long long o = __shfl_down_sync(0xffffffffu, key, s);
    key = o < key ? o : key;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) warpBest[warp] = key;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = warpBest[0];
    for (int k = 1; k < int(blockDim.x >> 5); k++) m = warpBest[k] < m ? warpBest[k] : m;
    if (m != NO_HIT) atomicMin(best + blockIdx.y, m);
  }
}

__global__ void k_cast_finish(BodyPtrs bd, int off, const CastQuery* __restrict__ qs, int n,
                              const unsigned long long* __restrict__ best, float4* out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const unsigned long long b = best[k];
    if (b == NO_HIT) {
      out[2 * k] = make_float4(0.f, 0.f, 0.f, -1.f);
      out[2 * k + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    const int local = int(b & 0xffffffffull);
    const Hit h = trace(bd, off + local, qs[k]);
    out[2 * k] = f4(h.n, fmaxf(0.f, h.t));
    out[2 * k + 1] = make_float4(__uint_as_float(uint32_t(local)), 0.f, 0.f, 0.f);
  }
}

}  // namespace

void launch_cast(const BodyPtrs& b, int off, int nb, const CastQuery* qs, int n, const CastFilter& f,
                 unsigned long long* best, float4* out, cudaStream_t s) {
  if (n <= 0) return;
  k_cast_init<<<grid_blocks(n, 256), 256, 0, s>>>(best, n);
  note_launches(1);
  if (nb > 0) {
    for (int q0 = 0; q0 < n; q0 += 65535) {
      const int m = n - q0 < 65535 ? n - q0 : 65535;
      const dim3 grid((unsigned)((nb + 255) / 256), (unsigned)m);
      k_cast_nearest<<<grid, 256, 0, s>>>(b, off, nb, qs + q0, f, best + q0);
      note_launches(1);
    }
  }
  k_cast_finish<<<grid_blocks(n, 256), 256, 0, s>>>(b, off, qs, n, best, out);
  note_launches(1);
}

}  // namespace avbd
