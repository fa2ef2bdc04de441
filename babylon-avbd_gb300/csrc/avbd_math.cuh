// Device vector, quaternion and 3x3 helpers for the AVBD kernels.
//
// The arithmetic follows reference/three-avbd/src/avbd3d/ref/math.ts operation for operation
// (left-to-right sums, separately rounded products where the translation unit is compiled
// with -fmad=false), so the contact generation reproduces the reference's float32 results
// bit for bit. Quaternions are float4 (x, y, z, w).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define AVBD_HD __host__ __device__ __forceinline__

struct V3 {
  float x, y, z;
};

AVBD_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
AVBD_HD V3 v3(float4 a) { return V3{a.x, a.y, a.z}; }
AVBD_HD float4 f4(V3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
AVBD_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
AVBD_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
AVBD_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
AVBD_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
AVBD_HD V3 vdiv(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
// a + b*s (math.ts addScaled3)
AVBD_HD V3 madd(V3 a, V3 b, float s) { return V3{a.x + b.x * s, a.y + b.y * s, a.z + b.z * s}; }
AVBD_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
AVBD_HD float len2(V3 a) { return dot(a, a); }
AVBD_HD V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
AVBD_HD float fminr(float a, float b) { return a < b ? a : b; }  // math.ts min
AVBD_HD float fmaxr(float a, float b) { return a > b ? a : b; }  // math.ts max
AVBD_HD float clampr(float x, float a, float b) { return fmaxr(a, fminr(b, x)); }
AVBD_HD V3 vabs(V3 a) { return V3{fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
AVBD_HD float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// quaternion (x, y, z, w)
AVBD_HD float4 qmul(float4 a, float4 b) {
  return make_float4(a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
                     a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z);
}
AVBD_HD float qlen2(float4 q) { return (q.x * q.x + q.y * q.y + q.z * q.z) + q.w * q.w; }
AVBD_HD float4 qinverse(float4 q) {
  float l = qlen2(q);
  return make_float4(-q.x / l, -q.y / l, -q.z / l, q.w / l);
}
AVBD_HD float4 qnormalize(float4 q) {
  float l = sqrtf(qlen2(q));
  return make_float4(q.x / l, q.y / l, q.z / l, q.w / l);
}
// rotation vector taking b to a (math.ts qsub)
// qsub(a, b) from b's inverse (qinverse(b)), for a b whose inverse is kept: the same bits
AVBD_HD V3 qsub_inv(float4 a, float4 bInv) {
  float4 t = qmul(a, bInv);
  return V3{t.x * 2, t.y * 2, t.z * 2};
}
AVBD_HD V3 qsub(float4 a, float4 b) { return qsub_inv(a, qinverse(b)); }
// integrate a rotation vector (math.ts qaddv)
AVBD_HD float4 qaddv(float4 a, V3 b) {
  float4 s = qmul(make_float4(b.x, b.y, b.z, 0.f), a);
  return qnormalize(make_float4(a.x + s.x * 0.5f, a.y + s.y * 0.5f, a.z + s.z * 0.5f, a.w + s.w * 0.5f));
}
AVBD_HD V3 rotate(float4 q, V3 v) {
  float ux = q.x, uy = q.y, uz = q.z, w = q.w;
  float tx = (uy * v.z - uz * v.y) * 2;
  float ty = (uz * v.x - ux * v.z) * 2;
  float tz = (ux * v.y - uy * v.x) * 2;
  return V3{v.x + tx * w + (uy * tz - uz * ty), v.y + ty * w + (uz * tx - ux * tz), v.z + tz * w + (ux * ty - uy * tx)};
}
AVBD_HD V3 rotateInv(float4 q, V3 v) { return rotate(make_float4(-q.x, -q.y, -q.z, q.w), v); }
// math.ts transform: rotate(q, v) + p
AVBD_HD V3 xform(V3 p, float4 q, V3 v) { return rotate(q, v) + p; }

// row-major 3x3 as three rows
struct M33 {
  V3 r0, r1, r2;
};
AVBD_HD V3 mulv(const M33& a, V3 v) { return V3{dot(a.r0, v), dot(a.r1, v), dot(a.r2, v)}; }
// math.ts orthonormal: rows (n, t1, t2)
AVBD_HD M33 orthonormal(V3 n) {
  V3 t1 = fabsf(n.x) > fabsf(n.z) ? V3{-n.y, n.x, 0.f} : V3{0.f, -n.z, n.y};
  float l = sqrtf(len2(t1));
  t1 = vdiv(t1, l);
  V3 t2 = cross(n, t1);
  return M33{n, t1, t2};
}

// Symmetric accumulation of the per-body 6x6 system: lower triangles of the linear and
// angular blocks, the full cross block (angular rows x linear columns), and both rhs halves.
struct Sys6 {
  float l00, l10, l11, l20, l21, l22;  // lin
  float a00, a10, a11, a20, a21, a22;  // ang
  float c[9];                          // cross, row-major (ang row, lin col)
  V3 bl, ba;
};
