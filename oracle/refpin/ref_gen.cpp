// ref_gen.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The reference pin's ray generation (see ref_harness.cpp for how the pin is
// built): the reference's own code, compiled unchanged from the reference
// tree --
//   barney/Camera.cu                  PerspectiveCamera::set3f, set1f, commit
//   barney/kernels/generateRays.cu    _generateRays
// -- exposed as C functions.  Restated here: only the objects the kernel
// receives -- the frame buffer's tile descriptors (32x32-pixel tiles in
// row-major order, TiledFB.cu:226-255), a ray queue, Renderer::DD's
// background colour, the per-thread ComputeInterface (one block per tile, one
// thread per pixel of the tile) -- and the API object base the camera
// derives from, which only names its context.
#include <cstring>
#include <vector>
#include "barney/Camera.cu"
#include "barney/kernels/generateRays.cu"

using namespace BARNEY_NS;

#pragma GCC visibility push(default)
extern "C" {

// The perspective camera a bnCamera "perspective" with these parameters
// commits: out = dir_00, dir_du, dir_dv, lens_00 (12 floats)
void ref_camera_commit(const float pos[3], const float dir[3], const float up[3], float fovy, float out[12]) {
  PerspectiveCamera cam(nullptr);
  cam.set3f("position", vec3f(pos[0], pos[1], pos[2]));
  cam.set3f("direction", vec3f(dir[0], dir[1], dir[2]));
  cam.set3f("up", vec3f(up[0], up[1], up[2]));
  cam.set1f("fovy", fovy);
  cam.commit();
  const Camera::DD &dd = cam.getDD();
  const vec3f v[4] = {dd.perspective.dir_00, dd.perspective.dir_du, dd.perspective.dir_dv, dd.perspective.lens_00};
  for (int i = 0; i < 4; i++) {
    out[3 * i + 0] = v[i].x;
    out[3 * i + 1] = v[i].y;
    out[3 * i + 2] = v[i].z;
  }
}

// _generateRays (generateRays.cu:44-243) for pass accumID of a W x H frame
// with that camera and background colour bg (w < 0: the gradient): per
// pixel, row-major, out = org[3], dir[3], tMax, missColor[4] (11 floats) and
// the ray's seed state; the path state's throughput must be 1 and its
// misWeight 0 (returned as the count of pixels where they are not).
int ref_generate(const float pos[3], const float dir[3], const float up[3], float fovy, int W, int H, int accumID,
                 const float bg[4], float *out, uint64_t *seeds) {
  PerspectiveCamera cam(nullptr);
  cam.set3f("position", vec3f(pos[0], pos[1], pos[2]));
  cam.set3f("direction", vec3f(dir[0], dir[1], dir[2]));
  cam.set3f("up", vec3f(up[0], up[1], up[2]));
  cam.set1f("fovy", fovy);
  cam.commit();
  Renderer::DD renderer;
  std::memset((void *)&renderer, 0, sizeof(renderer));
  renderer.bgColor = vec4f(bg[0], bg[1], bg[2], bg[3]);
  renderer.bgTexture = 0;
  renderer.cutPlane = vec4f(0.f, 0.f, 0.f, -1e30f);
  renderer.pathsPerPixel = 1;
  const int tilesX = (W + tileSize - 1) / tileSize, tilesY = (H + tileSize - 1) / tileSize;
  std::vector<TileDesc> tiles(tilesX * tilesY);
  for (int ty = 0; ty < tilesY; ty++)
    for (int tx = 0; tx < tilesX; tx++) tiles[tx + tilesX * ty].lower = vec2i(tx * tileSize, ty * tileSize);
  const int n = (int)tiles.size() * tileSize * tileSize;
  std::vector<render::Ray> rays(n);
  std::vector<render::PathState> states(n);
  std::vector<HitIDs> hitIDs(n);
  SingleQueue q;
  q.rays = rays.data();
  q.states = states.data();
  q.hitIDs = hitIDs.data();
  int count = 0;
  rtc::embree::ComputeInterface ci;
  std::memset((void *)&ci, 0, sizeof(ci));
  ci.blockDim = vec3ui(tileSize * tileSize, 1, 1);
  ci.gridDim = vec3ui((unsigned)tiles.size(), 1, 1);
  for (int t = 0; t < (int)tiles.size(); t++)
    for (int i = 0; i < tileSize * tileSize; i++) {
      ci.blockIdx = vec3ui(t, 0, 0);
      ci.threadIdx = vec3ui(i, 0, 0);
      render::_generateRays(ci, cam.getDD(), renderer, accumID, vec2i(W, H), &count, q, tiles.data(), false);
    }
  int bad = 0;
  for (int k = 0; k < count; k++) {
    const render::Ray &r = rays[k];
    const render::PathState &s = states[k];
    const int tile = s.pixelID / (tileSize * tileSize), local = s.pixelID % (tileSize * tileSize);
    const int ix = tiles[tile].lower.x + local % tileSize, iy = tiles[tile].lower.y + local / tileSize;
    if (ix >= W || iy >= H) continue;
    float *o = out + 11 * ((size_t)iy * W + ix);
    o[0] = r.org.x; o[1] = r.org.y; o[2] = r.org.z;
    o[3] = r.dir.x; o[4] = r.dir.y; o[5] = r.dir.z;
    o[6] = r.tMax;
    const vec4f &m = (const vec4f &)r.missColor;
    o[7] = m.x; o[8] = m.y; o[9] = m.z; o[10] = m.w;
    seeds[(size_t)iy * W + ix] = r.rngSeed.state;
    const uint16_t *tp = (const uint16_t *)&s.throughput;
    if (tp[0] != 0x3c00 || tp[1] != 0x3c00 || tp[2] != 0x3c00 || s.misWeight != 0.f) bad++;
  }
  return bad;
}

}  // extern "C"
#pragma GCC visibility pop
