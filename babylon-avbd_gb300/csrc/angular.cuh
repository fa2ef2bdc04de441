// Angular rows of hinge motors and angle limits (src/gpu/angularConstraints.js: angularFrame,
// angularAngle, angularRows, angularForce, addAngular, warmAngular, dualAngular; reference frames
// captured as src/gpu/angularFrames.wgsl).
//
// A record of kind KIND_MOTOR or KIND_LIMIT keeps, in the joint arrays:
//   rA.xyz   hinge axis in A's frame (world frame when A is the world); rA.w the kind
//   rB.xyz   hinge axis in B's frame
//   stiff.x  motor speed (rad/s) | lower angle     stiff.y  torque bound | upper angle
//   C0Lin    (reference tangent in A's frame, C0 of row 0)
//   C0Ang    (reference tangent in B's frame, C0 of row 1)
//   penLin.xy, lamLin.xy   penalty and lambda of the two rows (a motor uses row 0 only)
// The twist angle is the signed angle about the world axis from A's tangent to B's tangent.
#pragma once
#include "avbd_math.cuh"

constexpr float ANG_PI = 3.14159265358979f;
constexpr float ANG_HALF_PI = 1.57079632679490f;
constexpr float ANG_TWO_PI = 6.28318530717959f;
constexpr float ANGULAR_PENALTY0 = 1000.f;  // initial row penalty (appGpuSolver3D.js setAngularConstraint)

// atan2 built from the half-angle identity atan(t) = 2 atan(t / (1 + sqrt(1 + t^2))), applied
// twice so that |t| <= tan(pi/16), and the odd Taylor series of atan through t^9 there (the
// first omitted term is below 2e-9). It uses only +, -, *, / and sqrt, so the host restatement
// of the same steps gives the same bits.
AVBD_HD float angle_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float hi = fmaxr(ax, ay), lo = fminr(ax, ay);
  if (!(hi > 0.f)) return 0.f;
  const float t = lo / hi;
  const float u = t / (1.f + sqrtf(1.f + t * t));
  const float v = u / (1.f + sqrtf(1.f + u * u));
  const float w = v * v;
  const float s = v * (1.f + w * (-1.f / 3.f + w * (1.f / 5.f + w * (-1.f / 7.f + w * (1.f / 9.f)))));
  float a = 4.f * s;
  if (ay > ax) a = ANG_HALF_PI - a;
  if (x < 0.f) a = ANG_PI - a;
  return y < 0.f ? -a : a;
}

// The principal value of an angle difference in [-2 pi, 2 pi] (the reference's
// atan2(sin d, cos d)).
AVBD_HD float angle_wrap(float d) { return d > ANG_PI ? d - ANG_TWO_PI : (d < -ANG_PI ? d + ANG_TWO_PI : d); }

// A unit vector orthogonal to n (the tangent choice of angularFrames.wgsl).
AVBD_HD V3 angle_tangent(V3 n) {
  const V3 t = fabsf(n.x) > fabsf(n.z) ? V3{-n.y, n.x, 0.f} : V3{0.f, -n.z, n.y};
  return vdiv(t, sqrtf(len2(t)));
}

// Reference tangents from the poses at creation: A's tangent in A's frame, and its world image
// carried into B's frame and made orthogonal to B's axis.
AVBD_HD void angle_capture(float4 qa, float4 qb, V3 axisA, V3 axisB, V3& ta, V3& tb) {
  ta = angle_tangent(axisA);
  const V3 world = rotate(qa, ta);
  const V3 nb = vdiv(axisB, sqrtf(len2(axisB)));
  V3 t = rotateInv(qb, world);
  t = t - nb * dot(t, nb);
  if (sqrtf(len2(t)) < 1.0e-6f) t = fabsf(nb.x) > fabsf(nb.z) ? V3{-nb.y, nb.x, 0.f} : V3{0.f, -nb.z, nb.y};
  tb = vdiv(t, sqrtf(len2(t)));
}

// World axis and twist angle of the current poses.
AVBD_HD float angle_of(float4 qa, float4 qb, V3 axisA, V3 ta, V3 tb, V3& axis) {
  axis = rotate(qa, axisA);
  const V3 wa = rotate(qa, ta), wb = rotate(qb, tb);
  return angle_atan2(dot(axis, cross(wa, wb)), dot(wa, wb));
}

// Constraint values of the two rows: a motor's twist beyond C0 less its travel this step; a
// limit's distance past each stop less the alpha share of its step-start value.
AVBD_HD float2 angle_rows(bool motor, float angle, float p0, float p1, float c0, float c1, float alpha, float dt) {
  if (motor) return make_float2(angle_wrap(angle - c0) - p0 * dt, 0.f);
  return make_float2((angle - p0) - alpha * c0, (angle - p1) - alpha * c1);
}

// Row forces: a motor's clamped to the torque bound, a limit's one-sided.
AVBD_HD float2 angle_force(bool motor, float2 pen, float2 lam, float2 C, float bound) {
  const float fx = pen.x * C.x + lam.x, fy = pen.y * C.y + lam.y;
  if (motor) return make_float2(clampr(fx, -bound, bound), 0.f);
  return make_float2(fminr(0.f, fx), fmaxr(0.f, fy));
}
