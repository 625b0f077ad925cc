// AffineSpace.h -- TEST INFRASTRUCTURE ONLY: owl::common linear and affine
// spaces, restated for the reference pin harness (see owl-common.h).
#pragma once
#include "box.h"

namespace owl {
namespace common {

struct LinearSpace3f {
  vec3f vx, vy, vz;
  LinearSpace3f() = default;
  LinearSpace3f(const vec3f &x, const vec3f &y, const vec3f &z) : vx(x), vy(y), vz(z) {}
};
// Orthonormal frame around a unit normal N, as the reference's surface BSDFs
// call it (the Lambertian's scatter: xfmVector(frame(N), localDir)): dx the
// longer of (1,0,0) x N and (0,1,0) x N, normalized; dy = normalize(N x dx).
inline LinearSpace3f frame(const vec3f &N) {
  const vec3f dx0 = cross(vec3f(1.f, 0.f, 0.f), N), dx1 = cross(vec3f(0.f, 1.f, 0.f), N);
  const vec3f dx = normalize(dot(dx0, dx0) > dot(dx1, dx1) ? dx0 : dx1);
  const vec3f dy = normalize(cross(N, dx));
  return LinearSpace3f(dx, dy, N);
}
inline vec3f xfmVector(const LinearSpace3f &l, const vec3f &v) { return l.vx * v.x + l.vy * v.y + l.vz * v.z; }
struct AffineSpace3f {
  LinearSpace3f l;
  vec3f p;
};
// rcp of a linear space: its inverse, the transposed adjoint (cross products
// of the columns) times 1 / det
inline LinearSpace3f rcp(const LinearSpace3f &m) {
  const vec3f a = cross(m.vy, m.vz), b = cross(m.vz, m.vx), c = cross(m.vx, m.vy);
  const float r = 1.f / dot(m.vx, a);
  return LinearSpace3f(vec3f(a.x, b.x, c.x) * r, vec3f(a.y, b.y, c.y) * r, vec3f(a.z, b.z, c.z) * r);
}
typedef LinearSpace3f linear3f;
typedef AffineSpace3f affine3f;
inline vec3f xfmVector(const affine3f &a, const vec3f &v) { return xfmVector(a.l, v); }
inline vec3f xfmPoint(const affine3f &a, const vec3f &v) { return xfmVector(a.l, v) + a.p; }

}  // namespace common
}  // namespace owl
