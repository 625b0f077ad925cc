// barney_api.cpp -- the barney-compatible bn* surface (include/barney_gb300.h)
// over the gbv_* entry points.
//
// Object model after the reference's API layer (barney/api/barney.cu,
// barney/api/Context.h): opaque handles, string-keyed set/commit parameters,
// app reference counts; objects that reference others keep them alive.
// Rendering follows bnRender -> GlobalModel::render -> Context::renderTiles
// (barney/api/barney.cu:777-786, barney/Context.cpp:142-185) on one GPU.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/barney_gb300.h"
#include "../../include/gbvol.h"
#include "gbv_internal.h"

namespace bnimpl {

static thread_local std::string g_err;

static void fail(const std::string &msg) {
  g_err = msg;
  std::fprintf(stderr, "#bn: %s\n", msg.c_str());
}

// Device memory of one context.  Buffers come from a stream-ordered pool
// that keeps the blocks it is given back (release threshold: unlimited), so
// a scene rebuilt on the same context (new texel data, new field, new frame
// buffer) reuses the memory of the one it replaces instead of calling
// cudaMalloc and cudaFree (about a millisecond per GB each on GB300, and
// cudaFree waits for the device).  Every use of a buffer is on the
// context's stream, which also orders each reuse after the last use.  The
// pool's memory returns to the device when the context is destroyed.
struct DevPool {
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;  // null: plain cudaMalloc / cudaFree
};

template <typename T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  const DevPool *owner = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) {
      if (owner && owner->pool) cudaFreeAsync(p, owner->stream);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
  }
  bool alloc(size_t count, const DevPool &mem) {
    if (count == n && p) return true;
    release();
    if (count == 0) return true;
    owner = &mem;
    const cudaError_t e = mem.pool ? cudaMallocFromPoolAsync((void **)&p, count * sizeof(T), mem.pool, mem.stream)
                                   : cudaMalloc((void **)&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      fail("device allocation of " + std::to_string(count * sizeof(T)) + " bytes failed");
      return false;
    }
    n = count;
    return true;
  }
};

struct Context;

struct Object {
  Context *ctx = nullptr;
  std::string kind;
  int appRefs = 1;
  virtual ~Object() = default;
  virtual bool set1i(const std::string &, int) { return false; }
  virtual bool set1f(const std::string &, float) { return false; }
  virtual bool set2f(const std::string &, float, float) { return false; }
  virtual bool set3i(const std::string &, int, int, int) { return false; }
  virtual bool set3f(const std::string &, float, float, float) { return false; }
  virtual bool set4f(const std::string &, float, float, float, float) { return false; }
  virtual bool setObject(const std::string &, const std::shared_ptr<Object> &) { return false; }
  virtual bool setData(const std::string &, const std::shared_ptr<Object> &) { return false; }
  virtual bool setString(const std::string &, const std::string &) { return false; }
  virtual void commit() {}
};
using SP = std::shared_ptr<Object>;

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  DevPool mem;  // device buffers of this context's objects
  std::map<Object *, SP> handles;  // the app's references
  std::set<std::string> warned;
  SP find(void *h) {
    auto it = handles.find((Object *)h);
    return it == handles.end() ? SP() : it->second;
  }
  void warnOnce(const std::string &what) {
    if (warned.insert(what).second) std::fprintf(stderr, "#bn: warning: %s\n", what.c_str());
  }
};

static std::mutex g_mutex;
static std::set<Context *> g_contexts;

static SP lookup(void *h, Context **ctxOut = nullptr) {
  std::lock_guard<std::mutex> lock(g_mutex);
  for (Context *c : g_contexts) {
    SP o = c->find(h);
    if (o) {
      if (ctxOut) *ctxOut = c;
      return o;
    }
  }
  return SP();
}

template <typename T> static std::shared_ptr<T> as(const SP &o) { return std::dynamic_pointer_cast<T>(o); }

template <typename T> static T *track(Context *ctx, std::shared_ptr<T> obj, const char *kind) {
  obj->ctx = ctx;
  obj->kind = kind;
  std::lock_guard<std::mutex> lock(g_mutex);
  ctx->handles[obj.get()] = obj;
  return obj.get();
}

// ---------------------------------------------------------------- objects --

struct Data : Object {  // bnDataCreate: ObjectRefsData (BN_OBJECT) or PODData (BN_UINT8)
  int type = BN_OBJECT;
  std::vector<SP> objects;
  std::vector<unsigned char> bytes;
};

// Objects this path makes but does not render with: image texture data, 3D
// textures and samplers for material parameters (which the materials here
// refuse), kept so that callers holding them work unchanged.
struct Inert : Object {};

struct TextureData3D : Object {  // common/Texture.cpp, cudaCommon/TextureData.cu
  int dims[3] = {0, 0, 0};
  DevBuf<float> scalars;  // FP32 x-fastest on the device
};

struct Texture2D : Object {  // bnTexture2DCreate
  int W = 0, H = 0;
  int addr[2] = {GBV_ADDR_WRAP, GBV_ADDR_WRAP};
  DevBuf<float> texels;  // RGBA float
};

// A scalar field as the volume and the renderer see it (ScalarField,
// barney/volume/ScalarField.h): a macrocell range grid and the scene-record
// fields of its voxels.
struct Field : Object {
  int mcDims[3] = {0, 0, 0};
  DevBuf<float> ranges;
  virtual bool build(cudaStream_t s) = 0;
  virtual void fill(gbv_scene &s) const = 0;
};

struct StructuredField : Field {  // volume/StructuredData.{h,cu}
  std::shared_ptr<TextureData3D> td;
  int dims[3] = {0, 0, 0};
  float origin[3] = {0, 0, 0};
  float spacing[3] = {1, 1, 1};
  int cellsPerMC = 8;
  int voxelFormat = GBV_VOXEL_F32;
  int layout = GBV_LAYOUT_BRICK_CORNERS;
  int brickLog2[3] = {3, 3, 3};
  // built state
  bool built = false;
  DevBuf<unsigned char> bricks;
  DevBuf<float> scaleOffset;
  bool set3i(const std::string &m, int x, int y, int z) override {
    if (m == "dims") {
      dims[0] = x; dims[1] = y; dims[2] = z;
      built = false;
      return true;
    }
    if (m == "brickLog2") {  // brick shape of the brick-corner store (this library's knob)
      brickLog2[0] = x; brickLog2[1] = y; brickLog2[2] = z;
      built = false;
      return true;
    }
    return false;
  }
  bool set3f(const std::string &m, float x, float y, float z) override {
    if (m == "gridOrigin") { origin[0] = x; origin[1] = y; origin[2] = z; return true; }
    if (m == "gridSpacing") { spacing[0] = x; spacing[1] = y; spacing[2] = z; return true; }
    return false;
  }
  bool set1i(const std::string &m, int v) override {
    // storage knobs of this library (no counterpart in the reference)
    if (m == "cellsPerMacrocell") { cellsPerMC = v; built = false; return true; }
    if (m == "voxelFormat") { voxelFormat = v; built = false; return true; }
    if (m == "voxelLayout") { layout = v; built = false; return true; }
    return false;
  }
  bool setObject(const std::string &m, const SP &v) override {
    if (m == "textureData") {
      td = as<TextureData3D>(v);
      built = false;
      return td != nullptr;
    }
    return false;
  }
  void fill(gbv_scene &s) const override {
    s.layout = layout;
    s.format = voxelFormat;
    s.d_voxels = layout == GBV_LAYOUT_BRICK_CORNERS ? (const void *)bricks.p : (const void *)td->scalars.p;
    s.d_scale_offset = scaleOffset.p;
    s.cells_per_mc = cellsPerMC;
    for (int a = 0; a < 3; a++) {
      s.brick_log2[a] = brickLog2[a];
      s.dims[a] = dims[a];
      s.origin[a] = origin[a];
      s.spacing[a] = spacing[a];
    }
  }
  bool build(cudaStream_t s) override {
    if (built) return true;
    if (!td || !td->scalars.p) { fail("structured field has no textureData"); return false; }
    if (td->dims[0] != dims[0] || td->dims[1] != dims[1] || td->dims[2] != dims[2]) {
      fail("structured field dims do not match its textureData");
      return false;
    }
    if (gbv_mc_dims(dims, cellsPerMC, mcDims) != GBV_OK) { fail(gbv_last_error()); return false; }
    size_t nmc = (size_t)mcDims[0] * mcDims[1] * mcDims[2];
    if (!ranges.alloc(2 * std::max<size_t>(nmc, 1), ctx->mem)) return false;
    if (layout == GBV_LAYOUT_BRICK_CORNERS) {
      size_t vb = 0, sb = 0;
      if (gbv_brick_store_bytes_shaped(dims, voxelFormat, brickLog2, &vb, &sb) != GBV_OK) {
        fail(gbv_last_error());
        return false;
      }
      if (!bricks.alloc(vb, ctx->mem)) return false;
      if (sb && !scaleOffset.alloc(sb / sizeof(float), ctx->mem)) return false;
      if (gbv_build_brick_store_shaped(td->scalars.p, dims, voxelFormat, brickLog2, bricks.p,
                                       sb ? scaleOffset.p : nullptr, s) != GBV_OK) {
        fail(gbv_last_error());
        return false;
      }
    } else if (voxelFormat != GBV_VOXEL_F32) {
      fail("the linear voxel layout holds FP32 voxels only");
      return false;
    }
    // quantized stores: the ranges must bound the stored (rounded) values
    gbv_status rs = voxelFormat == GBV_VOXEL_F32
                        ? gbv_build_mc_ranges(td->scalars.p, dims, cellsPerMC, ranges.p, s)
                        : gbv_build_mc_ranges_from_store_shaped(bricks.p, scaleOffset.p, voxelFormat, dims,
                                                                brickLog2, cellsPerMC, ranges.p, s);
    if (rs != GBV_OK) {
      fail(gbv_last_error());
      return false;
    }
    built = true;
    return true;
  }
};

// volume/NanoVDB.{h,cu}: a NanoVDB float grid given as a BN_UINT8 data
// array ("data"), parsed and checked on commit, uploaded as is
struct NanoVDBField : Field {
  std::shared_ptr<Data> data;
  gbv_nanovdb_info info;
  DevBuf<unsigned char> grid;
  bool built = false, parsed = false;
  bool setData(const std::string &m, const SP &v) override {
    if (m == "data") {
      data = as<Data>(v);
      built = parsed = false;
      return data != nullptr;
    }
    return false;
  }
  void commit() override {
    parsed = false;
    if (!data || data->bytes.empty()) { fail("NanoVDB field has no data"); return; }
    if (gbv_nanovdb_parse(data->bytes.data(), data->bytes.size(), &info) != GBV_OK) {
      fail(gbv_last_error());
      return;
    }
    parsed = true;
  }
  void fill(gbv_scene &s) const override {
    s.layout = GBV_LAYOUT_NANOVDB;
    s.format = GBV_VOXEL_F32;
    s.d_voxels = grid.p;
    s.nanovdb = &info;
  }
  bool build(cudaStream_t s) override {
    if (built) return true;
    if (!parsed) { fail("NanoVDB field: no valid grid committed"); return false; }
    if (!grid.alloc(info.bytes, ctx->mem)) return false;
    if (cudaMemcpyAsync(grid.p, data->bytes.data(), info.bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) {
      fail("NanoVDB grid upload failed");
      return false;
    }
    for (int a = 0; a < 3; a++) mcDims[a] = info.mc_dims[a];
    const size_t nmc = (size_t)mcDims[0] * mcDims[1] * mcDims[2];
    if (!ranges.alloc(2 * nmc, ctx->mem)) return false;
    if (gbv_nanovdb_mc_ranges(grid.p, &info, ranges.p, s) != GBV_OK) {
      fail(gbv_last_error());
      return false;
    }
    // the host copy must live until the upload has run
    if (cudaStreamSynchronize(s) != cudaSuccess) { fail("NanoVDB grid upload failed"); return false; }
    built = true;
    return true;
  }
};

struct Volume : Object {  // volume/Volume.{h,cpp}, TransferFunction
  std::shared_ptr<Field> sf;
  std::vector<float> tfHost{1, 1, 1, 1, 1, 1, 1, 1};  // TransferFunction ctor default
  float domain[2] = {0.f, 1.f};
  float densityAt1 = 1.f;
  float anisotropy = 0.6f;        // Volume.h:158
  float scatteringAlbedo = 0.9f;  // Volume.h:159
  bool tfDirty = true;
  DevBuf<float> tf;
  DevBuf<float> majorants;
  int userID = 0;  // Volume::set1i("userID"): the object ID of its hits (BN_FB_OBJID)
  bool set1f(const std::string &m, float v) override {
    if (m == "anisotropy") { anisotropy = v; return true; }
    if (m == "scatteringAlbedo") { scatteringAlbedo = v; return true; }
    return false;
  }
  bool set1i(const std::string &m, int v) override {
    if (m == "userID") { userID = v; return true; }
    return false;
  }
  bool build(cudaStream_t s) {
    if (!sf || !sf->build(s)) return false;
    if (tfDirty || !majorants.p) {
      int n = (int)(tfHost.size() / 4);
      if (!tf.alloc(tfHost.size(), ctx->mem)) return false;
      if (cudaMemcpyAsync(tf.p, tfHost.data(), tfHost.size() * sizeof(float), cudaMemcpyHostToDevice, s) !=
          cudaSuccess) {
        fail("transfer function upload failed");
        return false;
      }
      size_t nmc = (size_t)sf->mcDims[0] * sf->mcDims[1] * sf->mcDims[2];
      if (!majorants.alloc(std::max<size_t>(nmc, 1), ctx->mem)) return false;
      if (gbv_map_majorants(sf->ranges.p, (int)nmc, tf.p, n, domain[0], domain[1], densityAt1, majorants.p, s) !=
          GBV_OK) {
        fail(gbv_last_error());
        return false;
      }
      // the host copy must outlive the async upload
      cudaStreamSynchronize(s);
      tfDirty = false;
    }
    return true;
  }
};

struct Light : Object {  // light/DirLight, light/EnvMap
  float direction[3] = {0.f, 0.f, -1.f};  // DirLight.h:36
  float color[3] = {1.f, 1.f, 1.f};
  float radiance = 1.f;
  float irradiance = NAN;
  // env map
  std::shared_ptr<Texture2D> texture;
  float envDir[3] = {1.f, 0.f, 0.f};  // EnvMap.h:82-84
  float envUp[3] = {0.f, 0.f, 1.f};
  float scale = 1.f;
  bool cdfDirty = true;
  DevBuf<float> cdfY, cdfX;
  bool set1f(const std::string &m, float v) override {
    if (m == "radiance") { radiance = v; return true; }
    if (m == "irradiance") { irradiance = v; return true; }
    if (m == "scale") { scale = v; return true; }
    return false;
  }
  bool set3f(const std::string &m, float x, float y, float z) override {
    if (m == "color") { color[0] = x; color[1] = y; color[2] = z; return true; }
    if (m == "direction") {
      if (kind == "envmap") { envDir[0] = x; envDir[1] = y; envDir[2] = z; }
      else { direction[0] = x; direction[1] = y; direction[2] = z; }
      return true;
    }
    if (m == "up") { envUp[0] = x; envUp[1] = y; envUp[2] = z; return true; }
    return false;
  }
  bool setObject(const std::string &m, const SP &v) override {
    if (m == "texture" && kind == "envmap") {
      texture = as<Texture2D>(v);
      cdfDirty = true;
      return texture != nullptr;
    }
    return false;
  }
  bool buildEnv(cudaStream_t s) {
    if (!texture || !texture->texels.p) { fail("envmap light without a texture"); return false; }
    if (!cdfDirty) return true;
    if (!cdfY.alloc(texture->H, ctx->mem) || !cdfX.alloc((size_t)texture->W * texture->H, ctx->mem)) return false;
    if (gbv_env_build_cdfs(texture->texels.p, texture->W, texture->H, texture->addr, cdfY.p, cdfX.p, s) != GBV_OK) {
      fail(gbv_last_error());
      return false;
    }
    cdfDirty = false;
    return true;
  }
};

// render/AnariMatte (barney/material/AnariMatte.{h,cpp}): constant color
// (default 0.8 grey, alpha 1) and opacity; parameters take effect on commit
// (HostMaterial::commit writes the device material).
struct Material : Object {
  struct P {
    float color[4] = {.8f, .8f, .8f, 1.f};
    float opacity = 1.f;
  } staged, live;
  bool committed = false;
  bool set1f(const std::string &m, float v) override {
    if (m == "opacity") { staged.opacity = v; return true; }
    return false;
  }
  bool set3f(const std::string &m, float x, float y, float z) override {
    if (m == "color") { staged.color[0] = x; staged.color[1] = y; staged.color[2] = z; staged.color[3] = 1.f; return true; }
    return false;
  }
  bool set4f(const std::string &m, float x, float y, float z, float w) override {
    if (m == "color") { staged.color[0] = x; staged.color[1] = y; staged.color[2] = z; staged.color[3] = w; return true; }
    return false;
  }
  bool setString(const std::string &m, const std::string &) override {
    if (m == "color" || m == "opacity") {
      fail("matte material: parameters mapped to geometry attributes are not supported (constant values only)");
      return true;
    }
    return false;
  }
  bool setObject(const std::string &m, const SP &) override {
    if (m == "color" || m == "opacity") {
      fail("matte material: parameters mapped to samplers are not supported (constant values only)");
      return true;
    }
    return false;
  }
  void commit() override {
    live = staged;
    committed = true;
  }
};

// geometry/IsoSurface (barney/geometry/IsoSurface.{h,cpp}): an iso-surface of
// a scalar field with a material
struct IsoSurfaceGeom : Object {
  std::shared_ptr<Field> sf;
  std::shared_ptr<Material> material;
  float isoValue = NAN;  // IsoSurface.h:79
  int userID = 0;        // the object ID of its hits (BN_FB_OBJID)
  bool set1f(const std::string &m, float v) override {
    if (m == "isoValue") { isoValue = v; return true; }
    return false;
  }
  bool set1i(const std::string &m, int v) override {
    if (m == "userID") { userID = v; return true; }
    return false;
  }
  bool setData(const std::string &m, const SP &) override {
    // "isoValues": kept by the reference but not read by its intersection
    // program, which tests isoValue alone (MCAccelerator.h:433-441)
    return m == "isoValues";
  }
  bool setObject(const std::string &m, const SP &v) override {
    if (m == "scalarField") {
      sf = as<Field>(v);
      if (!sf) fail("'scalarField' value set on 'iso_surface' is not a scalar field");
      return true;
    }
    if (m == "material") {
      material = as<Material>(v);
      if (v && !material) fail("'material' value set on 'iso_surface' is not a material");
      return true;
    }
    return false;
  }
};

struct Group : Object {
  std::vector<std::shared_ptr<IsoSurfaceGeom>> geoms;
  std::vector<std::shared_ptr<Volume>> volumes;
  std::shared_ptr<Data> lights;
  bool setData(const std::string &m, const SP &v) override {
    if (m == "lights") {
      lights = as<Data>(v);
      return lights != nullptr;
    }
    return false;
  }
};

struct Model : Object {
  std::vector<std::shared_ptr<Group>> groups;
  std::vector<BNTransform> xfms;
  std::map<std::string, SP> instanceAttributes;  // bnSetInstanceAttributes; not read by this path
};

struct Camera : Object {  // Camera.cu PerspectiveCamera
  float position[3] = {0, 0, 0};
  float direction[3] = {0, 0, 1};
  float up[3] = {0, 1, 0};
  float fovy = 60.f;
  bool set1f(const std::string &m, float v) override {
    if (m == "fovy") { fovy = v; return true; }
    if (m == "aspect" || m == "focusDistance") return true;
    if (m == "apertureRadius") {
      if (v > 0.f) { fail("apertureRadius > 0 (depth of field) is not supported"); return false; }
      return true;
    }
    return false;
  }
  bool set3f(const std::string &m, float x, float y, float z) override {
    if (m == "position") { position[0] = x; position[1] = y; position[2] = z; return true; }
    if (m == "direction") { direction[0] = x; direction[1] = y; direction[2] = z; return true; }
    if (m == "up") { up[0] = x; up[1] = y; up[2] = z; return true; }
    return false;
  }
};

struct Renderer : Object {  // render/Renderer.{h,cpp}; staged until commit
  struct P {
    float bg[4] = {0, 0, 0, 1};
    int spp = 1;
    float ambient = 1.f;
    int maxVolumeBounces = 0;
    int volumeMultiScatter = 0;
    int multiScatterBuild = 0;
    int frameStats = 0;  // this library's: count events for bnFrameBufferGetStats
  } staged, live;
  Renderer() {
    // The reference picks single or multiple scattering at compile time
    // (BARNEY_USE_MULTI_SCATTERING, CMakeLists.txt:219-221); here it is the
    // renderer parameter "multiScatter", defaulting to that variable's value
    // in the environment.
    const char *e = std::getenv("BARNEY_USE_MULTI_SCATTERING");
    staged.multiScatterBuild = live.multiScatterBuild = (e && std::atoi(e) != 0) ? 1 : 0;
  }
  bool set1i(const std::string &m, int v) override {
    if (m == "pathsPerPixel") { staged.spp = v; return true; }
    if (m == "crosshairs") return true;
    if (m == "maxVolumeBounces") { staged.maxVolumeBounces = v; return true; }
    if (m == "volumeMultiScatter") { staged.volumeMultiScatter = v; return true; }
    if (m == "multiScatter") { staged.multiScatterBuild = v ? 1 : 0; return true; }
    if (m == "frameStats") { staged.frameStats = v ? 1 : 0; return true; }
    return false;
  }
  bool set1f(const std::string &m, float v) override {
    if (m == "ambientRadiance") { staged.ambient = v; return true; }
    return false;
  }
  bool set4f(const std::string &m, float x, float y, float z, float w) override {
    if (m == "bgColor") { staged.bg[0] = x; staged.bg[1] = y; staged.bg[2] = z; staged.bg[3] = w; return true; }
    if (m == "cutPlane") {
      if (w > -1e28f) { fail("cutPlane is not supported"); return false; }
      return true;
    }
    return false;
  }
  void commit() override { live = staged; }
};

struct FrameBuffer : Object {  // fb/FrameBuffer, LocalFB
  int W = 0, H = 0;
  int colorFormat = BN_FLOAT4;
  int accumID = 0;
  uint32_t channels = BN_FB_COLOR;  // the resize's requiredChannels
  DevBuf<float> accum;
  DevBuf<unsigned char> color;
  // the aux channels (TiledFB's auxTiles, fb/TiledFB.cu:276-290), allocated
  // when the resize asks for them
  DevBuf<float> depth;
  DevBuf<int> primId, instId, objId;
  DevBuf<unsigned long long> counters;
  unsigned long long lastStats[4] = {0, 0, 0, 0};
};

static int fbFormat(int bnFormat) {
  switch (bnFormat) {
    case BN_FLOAT4: return GBV_FB_FLOAT4;
    case BN_UFIXED8_RGBA: return GBV_FB_RGBA8;
    case BN_UFIXED8_RGBA_SRGB: return GBV_FB_RGBA8_SRGB;
  }
  return -1;
}

static bool isIdentity(const BNTransform &x) {
  return x.l.vx.x == 1 && x.l.vx.y == 0 && x.l.vx.z == 0 && x.l.vy.x == 0 && x.l.vy.y == 1 && x.l.vy.z == 0 &&
         x.l.vz.x == 0 && x.l.vz.y == 0 && x.l.vz.z == 1 && x.p.x == 0 && x.p.y == 0 && x.p.z == 0;
}

}  // namespace bnimpl

using namespace bnimpl;

// ------------------------------------------------------------------ C ABI --
extern "C" {

const char *bnGetLastError(void) { return g_err.c_str(); }

BNContext bnContextCreate(const int *dataRanks, int numDataRanks, const int *gpuIDs, int numGPUs) {
  if (numDataRanks > 1 || (dataRanks && dataRanks[0] != 0)) {
    fail("only a single data slot is supported");
    return nullptr;
  }
  if (numGPUs > 1) {
    fail("only single-GPU contexts are supported");
    return nullptr;
  }
  if (gpuIDs && numGPUs == 1 && gpuIDs[0] < 0) {
    fail("the CPU backend (gpuIDs={-1}) is not part of this library");
    return nullptr;
  }
  auto *c = new Context();
  c->device = (gpuIDs && numGPUs == 1) ? gpuIDs[0] : 0;
  if (cudaSetDevice(c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) !=
                                                     cudaSuccess) {
    fail("cannot use CUDA device " + std::to_string(c->device));
    delete c;
    return nullptr;  // bnContextCreate returns 0 on failure (barney.cu:923-927)
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = c->device;
  c->mem.stream = c->stream;
  if (cudaMemPoolCreate(&c->mem.pool, &props) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(c->mem.pool, cudaMemPoolAttrReleaseThreshold, &keep);
  } else {
    c->mem.pool = nullptr;  // fall back to cudaMalloc / cudaFree
    cudaGetLastError();
  }
  g_err.clear();  // a new context starts with no recorded failure
  std::lock_guard<std::mutex> lock(g_mutex);
  g_contexts.insert(c);
  return (BNContext)c;
}

void bnContextDestroy(BNContext context) {
  Context *c = (Context *)context;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_contexts.erase(c)) return;
  }
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->handles.clear();  // the objects hand their buffers back to the pool
  cudaStreamSynchronize(c->stream);
  if (c->mem.pool) cudaMemPoolDestroy(c->mem.pool);
  cudaStreamDestroy(c->stream);
  delete c;
}

void bnRelease(BNObject object) {
  Context *c = nullptr;
  SP o = lookup(object, &c);
  if (!o) return;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (--o->appRefs <= 0) c->handles.erase(o.get());
}

void bnAddReference(BNObject object) {
  SP o = lookup(object);
  if (o) o->appRefs++;
}

BNCamera bnCameraCreate(BNContext context, const char *type) {
  Context *c = (Context *)context;
  std::string t = type ? type : "";
  if (t != "perspective" && t != "pinhole") {
    fail("camera type '" + t + "' is not supported");
    return nullptr;
  }
  return (BNCamera)track(c, std::make_shared<Camera>(), "camera");
}

BNFrameBuffer bnFrameBufferCreate(BNContext context, int) {
  return (BNFrameBuffer)track((Context *)context, std::make_shared<FrameBuffer>(), "frameBuffer");
}

BNModel bnModelCreate(BNContext ctx) { return (BNModel)track((Context *)ctx, std::make_shared<Model>(), "model"); }

BNRenderer bnRendererCreate(BNContext ctx, const char *) {
  return (BNRenderer)track((Context *)ctx, std::make_shared<Renderer>(), "renderer");
}

// the contents of a data array of d->type from numItems items
static bool fill_data(Context *c, Data *d, size_t numItems, const void *items) {
  if (d->type == BN_UINT8) {
    if (numItems && !items) {
      fail("bnDataCreate: null data");
      return false;
    }
    const unsigned char *b = (const unsigned char *)items;
    d->bytes.assign(b, b + numItems);
    return true;
  }
  std::vector<SP> objs;
  const BNObject *handles = (const BNObject *)items;
  for (size_t i = 0; i < numItems; i++) {
    SP o = c->find(handles[i]);
    if (!o) {
      fail("data array references an unknown object");
      return false;
    }
    objs.push_back(o);
  }
  d->objects = std::move(objs);
  return true;
}

void bnDataSet(BNData data, size_t numItems, const void *items) {
  Context *c = nullptr;
  auto d = as<Data>(lookup(data, &c));
  if (!d) return fail("bnDataSet: unknown data array");
  fill_data(c, d.get(), numItems, items);
}

BNTextureData bnTextureData2DCreate(BNContext context, int, BNDataType, int, int, const void *) {
  return (BNTextureData)track((Context *)context, std::make_shared<Inert>(), "textureData2D");
}

BNTexture3D bnTexture3DCreate(BNContext context, int, BNDataType, uint32_t, uint32_t, uint32_t, const void *,
                              BNTextureFilterMode, BNTextureAddressMode) {
  return (BNTexture3D)track((Context *)context, std::make_shared<Inert>(), "texture3D");
}

BNSampler bnSamplerCreate(BNContext context, int, const char *) {
  return (BNSampler)track((Context *)context, std::make_shared<Inert>(), "sampler");
}

BNData bnDataCreate(BNContext context, int, BNDataType dataType, size_t numItems, const void *items) {
  Context *c = (Context *)context;
  // BN_UINT8: a byte array (PODData), e.g. a NanoVDB grid; BN_OBJECT: object
  // references (ObjectRefsData)
  if (dataType != BN_UINT8 && dataType != BN_OBJECT) {
    fail("only BN_OBJECT and BN_UINT8 data arrays are used by this path");
    return nullptr;
  }
  auto d = std::make_shared<Data>();
  d->type = dataType;
  if (!fill_data(c, d.get(), numItems, items)) return nullptr;
  return (BNData)track(c, d, "data");
}

BNTextureData bnTextureData3DCreate(BNContext context, int, BNDataType texelFormat, int width, int height, int depth,
                                    const void *items) {
  Context *c = (Context *)context;
  if (width < 1 || height < 1 || depth < 1 || !items) {
    fail("bnTextureData3DCreate: empty texture");
    return nullptr;
  }
  size_t n = (size_t)width * height * depth;
  auto td = std::make_shared<TextureData3D>();
  td->dims[0] = width; td->dims[1] = height; td->dims[2] = depth;
  cudaSetDevice(c->device);
  if (!td->scalars.alloc(n, c->mem)) return nullptr;
  if (texelFormat == BN_FLOAT32) {
    // texels are copied at create time (rtcore/cudaCommon/TextureData.cu:59-75)
    if (cudaMemcpyAsync(td->scalars.p, items, n * sizeof(float), cudaMemcpyDefault, c->stream) != cudaSuccess) {
      fail("texel upload failed");
      return nullptr;
    }
    cudaStreamSynchronize(c->stream);
  } else if (texelFormat == BN_UFIXED8 || texelFormat == BN_UINT8 || texelFormat == BN_UFIXED16 ||
             texelFormat == BN_UINT16) {
    // normalised integer texels: upload the raw texels, normalise on the device
    const int bits = (texelFormat == BN_UFIXED8 || texelFormat == BN_UINT8) ? 8 : 16;
    DevBuf<unsigned char> raw;
    if (!raw.alloc(n * (bits / 8), c->mem)) return nullptr;
    if (cudaMemcpyAsync(raw.p, items, n * (bits / 8), cudaMemcpyDefault, c->stream) != cudaSuccess ||
        gbv_normalize_texels(raw.p, bits, (long long)n, td->scalars.p, c->stream) != GBV_OK ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
      fail("texel upload failed");
      return nullptr;
    }
  } else {
    fail("bnTextureData3DCreate: unsupported texel format " + std::to_string((int)texelFormat));
    return nullptr;
  }
  return (BNTextureData)track(c, td, "textureData3D");
}

BNTexture2D bnTexture2DCreate(BNContext context, int, BNDataType texelFormat, uint32_t sx, uint32_t sy,
                              const void *texels, BNTextureFilterMode filterMode, BNTextureAddressMode ax,
                              BNTextureAddressMode ay, BNTextureColorSpace) {
  Context *c = (Context *)context;
  if (texelFormat != BN_FLOAT4 || !texels || sx == 0 || sy == 0) {
    fail("bnTexture2DCreate: env maps need FLOAT4 texels");
    return nullptr;
  }
  if (filterMode != BN_TEXTURE_LINEAR) c->warnOnce("env-map textures are always sampled with the linear filter");
  auto t = std::make_shared<Texture2D>();
  t->W = (int)sx;
  t->H = (int)sy;
  t->addr[0] = (int)ax;
  t->addr[1] = (int)ay;
  cudaSetDevice(c->device);
  if (!t->texels.alloc((size_t)4 * sx * sy, c->mem)) return nullptr;
  if (cudaMemcpyAsync(t->texels.p, texels, (size_t)16 * sx * sy, cudaMemcpyDefault, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    fail("texture upload failed");
    return nullptr;
  }
  return (BNTexture2D)track(c, t, "texture2D");
}

BNLight bnLightCreate(BNContext context, int, const char *type) {
  std::string t = type ? type : "";
  if (t != "directional" && t != "envmap") {
    fail("light type '" + t + "' is not supported");
    return nullptr;
  }
  return (BNLight)track((Context *)context, std::make_shared<Light>(), t == "envmap" ? "envmap" : "directional");
}

BNGeom bnGeometryCreate(BNContext context, int, const char *type) {
  std::string t = type ? type : "";
  if (t != "iso_surface") {  // Geometry::create (barney/geometry/Geometry.cpp:26-43)
    fail("geometry type '" + t + "' is not supported (surface geometry other than iso_surface)");
    return nullptr;
  }
  return (BNGeom)track((Context *)context, std::make_shared<IsoSurfaceGeom>(), "iso_surface");
}

BNMaterial bnMaterialCreate(BNContext context, int, const char *type) {
  std::string t = type ? type : "";
  if (t != "matte" && t != "AnariMatte") {  // HostMaterial::create (barney/material/Material.cpp:83-98)
    fail("material type '" + t + "' is not supported (matte only)");
    return nullptr;
  }
  return (BNMaterial)track((Context *)context, std::make_shared<Material>(), "matte");
}

BNGroup bnGroupCreate(BNContext context, int, BNGeom *geoms, int numGeoms, BNVolume *volumes, int numVolumes) {
  Context *c = (Context *)context;
  auto g = std::make_shared<Group>();
  for (int i = 0; geoms && i < numGeoms; i++) {
    auto iso = as<IsoSurfaceGeom>(c->find(geoms[i]));
    if (!iso) {
      fail("bnGroupCreate: unknown geometry handle");
      return nullptr;
    }
    g->geoms.push_back(iso);
  }
  for (int i = 0; i < numVolumes; i++) {
    auto v = as<Volume>(c->find(volumes[i]));
    if (!v) {
      fail("bnGroupCreate: unknown volume handle");
      return nullptr;
    }
    g->volumes.push_back(v);
  }
  return (BNGroup)track(c, g, "group");
}

void bnGroupBuild(BNGroup group) {
  Context *c = nullptr;
  auto g = as<Group>(lookup(group, &c));
  if (!g) return fail("bnGroupBuild: unknown group");
  cudaSetDevice(c->device);
  for (auto &iso : g->geoms)
    if (iso->sf && !iso->sf->build(c->stream)) return;
  for (auto &v : g->volumes)
    if (!v->build(c->stream)) return;
}

BNScalarField bnScalarFieldCreate(BNContext context, int, const char *type) {
  std::string t = type ? type : "";
  if (t == "NanoVDB")  // ScalarFieldRegistry "NanoVDB" (barney/volume/ScalarField.cpp:56)
    return (BNScalarField)track((Context *)context, std::make_shared<NanoVDBField>(), "NanoVDB");
  if (t != "structured") {
    fail("scalar field type '" + t + "' is not supported");
    return nullptr;
  }
  return (BNScalarField)track((Context *)context, std::make_shared<StructuredField>(), "structured");
}

BNVolume bnVolumeCreate(BNContext context, int, BNScalarField sf) {
  Context *c = (Context *)context;
  auto f = as<Field>(c->find(sf));
  if (!f) {
    fail("bnVolumeCreate: unknown scalar field");
    return nullptr;
  }
  auto v = std::make_shared<Volume>();
  v->sf = f;
  return (BNVolume)track(c, v, "volume");
}

void bnVolumeSetXF(BNVolume volume, bn_float2 domain, const bn_float4 *colorMap, int n, float densityAt1) {
  auto v = as<Volume>(lookup(volume));
  if (!v) return fail("bnVolumeSetXF: unknown volume");
  if (n < 2 || !colorMap) return fail("bnVolumeSetXF: a transfer function needs at least 2 entries");
  v->tfHost.assign((const float *)colorMap, (const float *)colorMap + 4 * (size_t)n);
  v->domain[0] = domain.x;
  v->domain[1] = domain.y;
  v->densityAt1 = densityAt1;
  v->tfDirty = true;
}

void bnCommit(BNObject target) {
  SP o = lookup(target);
  if (o) o->commit();
}

#define BN_SETTER(call, ...)                                                                   \
  Context *c = nullptr;                                                                        \
  SP o = lookup(target, &c);                                                                   \
  if (!o) return fail(std::string("set '") + paramName + "' on an unknown object");           \
  if (!o->call) c->warnOnce(o->kind + " ignores parameter '" + paramName + "'");

void bnSetString(BNObject target, const char *paramName, const char *value) {
  Context *c = nullptr;
  SP o = lookup(target, &c);
  if (o && !o->setString(paramName, value ? value : ""))
    c->warnOnce(o->kind + " ignores string parameter '" + paramName + "'");
}
void bnSetData(BNObject target, const char *paramName, BNData value) {
  BN_SETTER(setData(paramName, c ? c->find(value) : SP()));
}
void bnSetObject(BNObject target, const char *paramName, const BNObject value) {
  BN_SETTER(setObject(paramName, c ? c->find(value) : SP()));
}
void bnSetLight(BNObject target, const char *paramName, BNLight value) {
  BN_SETTER(setObject(paramName, c ? c->find(value) : SP()));
}
void bnSet1i(BNObject target, const char *paramName, int v) { BN_SETTER(set1i(paramName, v)); }
void bnSet2i(BNObject target, const char *paramName, int, int) {
  Context *c = nullptr;
  SP o = lookup(target, &c);
  if (o) c->warnOnce(o->kind + " ignores int2 parameter '" + paramName + "'");
}
void bnSet3i(BNObject target, const char *paramName, int x, int y, int z) { BN_SETTER(set3i(paramName, x, y, z)); }
void bnSet4i(BNObject target, const char *paramName, int, int, int, int) {
  Context *c = nullptr;
  SP o = lookup(target, &c);
  if (o) c->warnOnce(o->kind + " ignores int4 parameter '" + paramName + "'");
}
void bnSet1f(BNObject target, const char *paramName, float v) { BN_SETTER(set1f(paramName, v)); }
void bnSet2f(BNObject target, const char *paramName, float x, float y) { BN_SETTER(set2f(paramName, x, y)); }
void bnSet3f(BNObject target, const char *paramName, float x, float y, float z) {
  BN_SETTER(set3f(paramName, x, y, z));
}
void bnSet4f(BNObject target, const char *paramName, float x, float y, float z, float w) {
  BN_SETTER(set4f(paramName, x, y, z, w));
}
void bnSet4x3fv(BNObject target, const char *paramName, const BNTransform *) {
  Context *c = nullptr;
  SP o = lookup(target, &c);
  if (o) c->warnOnce(o->kind + " ignores transform parameter '" + paramName + "'");
}
void bnSet4x4fv(BNObject target, const char *paramName, const bn_float4 *) {
  Context *c = nullptr;
  SP o = lookup(target, &c);
  if (o) c->warnOnce(o->kind + " ignores 4x4 matrix parameter '" + paramName + "'");
}

void bnSetInstances(BNModel model, int, BNGroup *groups, BNTransform *xfms, int n) {
  Context *c = nullptr;
  auto m = as<Model>(lookup(model, &c));
  if (!m) return fail("bnSetInstances: unknown model");
  m->groups.clear();
  m->xfms.clear();
  for (int i = 0; i < n; i++) {
    auto g = as<Group>(c->find(groups[i]));
    if (!g) return fail("bnSetInstances: unknown group");
    m->groups.push_back(g);
    BNTransform x{};
    if (xfms) x = xfms[i];
    else { x.l.vx.x = 1; x.l.vy.y = 1; x.l.vz.z = 1; }
    m->xfms.push_back(x);
  }
}

void bnUpdateInstanceTransforms(BNModel model, int, BNTransform *xfms, int n) {
  auto m = as<Model>(lookup(model));
  if (!m) return fail("bnUpdateInstanceTransforms: unknown model");
  if (n != (int)m->xfms.size() || (n > 0 && !xfms))
    return fail("bnUpdateInstanceTransforms: the count differs from the instances bnSetInstances set");
  for (int i = 0; i < n; i++) m->xfms[i] = xfms[i];
}

void bnSetInstanceAttributes(BNModel model, int, const char *attributeName, BNData data) {
  Context *c = nullptr;
  auto m = as<Model>(lookup(model, &c));
  if (!m) return fail("bnSetInstanceAttributes: unknown model");
  m->instanceAttributes[attributeName ? attributeName : ""] = data ? c->find(data) : SP();
}

void bnBuild(BNModel model, int) {
  Context *c = nullptr;
  auto m = as<Model>(lookup(model, &c));
  if (!m) return fail("bnBuild: unknown model");
  cudaSetDevice(c->device);
  for (size_t i = 0; i < m->groups.size(); i++) {
    if (!isIdentity(m->xfms[i])) return fail("instance transforms other than the identity are not supported");
    for (auto &iso : m->groups[i]->geoms)
      if (iso->sf && !iso->sf->build(c->stream)) return;
    for (auto &v : m->groups[i]->volumes)
      if (!v->build(c->stream)) return;
  }
}

void bnAccumReset(BNFrameBuffer fb) {
  auto f = as<FrameBuffer>(lookup(fb));
  if (f) f->accumID = 0;
}

void bnFrameBufferResize(BNFrameBuffer fb, BNDataType colorFormat, int sx, int sy, uint32_t requiredChannels) {
  auto f = as<FrameBuffer>(lookup(fb));
  if (!f) return fail("bnFrameBufferResize: unknown frame buffer");
  if (fbFormat(colorFormat) < 0) return fail("bnFrameBufferResize: unsupported color format");
  if (sx <= 0 || sy <= 0) return fail("bnFrameBufferResize: empty frame");
  f->W = sx;
  f->H = sy;
  f->colorFormat = colorFormat;
  f->accumID = 0;
  f->channels = requiredChannels | BN_FB_COLOR;
  cudaSetDevice(f->ctx->device);
  const size_t n = (size_t)sx * sy;
  if (!f->accum.alloc(4 * n, f->ctx->mem)) return;
  if (!f->color.alloc(16 * n, f->ctx->mem)) return;
  if ((f->channels & BN_FB_DEPTH) && !f->depth.alloc(n, f->ctx->mem)) return;
  if ((f->channels & BN_FB_PRIMID) && !f->primId.alloc(n, f->ctx->mem)) return;
  if ((f->channels & BN_FB_INSTID) && !f->instId.alloc(n, f->ctx->mem)) return;
  if ((f->channels & BN_FB_OBJID) && !f->objId.alloc(n, f->ctx->mem)) return;
}

void bnFrameBufferGetSize(BNFrameBuffer fb, int *sx, int *sy) {
  auto f = as<FrameBuffer>(lookup(fb));
  if (!f) return;
  if (sx) *sx = f->W;
  if (sy) *sy = f->H;
}

void bnFrameBufferGetStats(BNFrameBuffer fb, unsigned long long stats[4]) {
  auto f = as<FrameBuffer>(lookup(fb));
  for (int i = 0; i < 4; i++) stats[i] = f ? f->lastStats[i] : 0;
}

void bnRender(BNRenderer renderer, BNModel model, BNCamera camera, BNFrameBuffer fb) {
  Context *c = nullptr;
  auto r = as<Renderer>(lookup(renderer, &c));
  auto m = as<Model>(lookup(model));
  auto cam = as<Camera>(lookup(camera));
  auto f = as<FrameBuffer>(lookup(fb));
  if (!r || !m || !cam || !f) return fail("bnRender: unknown handle");
  if (!f->accum.p) return fail("bnRender: frame buffer was never resized");
  cudaSetDevice(c->device);
  // collect the world: one volume and/or one iso-surface, directional
  // lights, env map.  RTC instance indices follow
  // ModelSlot::flattenInstancesForDevice (barney/ModelSlot.cpp:129-155): per
  // group, its user-geometry group (the iso-surface), then one instance per
  // volume.
  std::shared_ptr<Volume> vol;
  std::shared_ptr<IsoSurfaceGeom> iso;
  int volInst = 0, isoInst = 0, nextInst = 0;
  std::vector<std::shared_ptr<Light>> dirs;
  std::shared_ptr<Light> env;
  for (size_t i = 0; i < m->groups.size(); i++) {
    if (!isIdentity(m->xfms[i])) return fail("instance transforms other than the identity are not supported");
    auto &g = m->groups[i];
    if (!g->geoms.empty()) {
      for (auto &gm : g->geoms) {
        if (iso && iso != gm) return fail("more than one iso-surface per model is not supported");
        iso = gm;
      }
      isoInst = nextInst++;
    }
    for (auto &v : g->volumes) {
      if (vol && vol != v) return fail("more than one volume per model is not supported");
      vol = v;
      volInst = nextInst++;
    }
    if (g->lights)
      for (auto &o : g->lights->objects) {
        auto l = as<Light>(o);
        if (!l) continue;
        if (l->kind == "envmap") env = l;
        else dirs.push_back(l);
      }
  }
  if (!vol && !iso) return fail("bnRender: the model holds no volume and no iso-surface");
  if (vol && !vol->build(c->stream)) return;
  gbv_iso_surface isoRec;
  if (iso) {
    // Geometry::getMaterial requires a committed material (Geometry.cpp:86-99)
    if (!iso->sf) return fail("bnRender: the iso-surface has no scalar field");
    if (!iso->material || !iso->material->committed)
      return fail("bnRender: the iso-surface has no committed material");
    if (vol && vol->sf != iso->sf)
      return fail("bnRender: an iso-surface and a volume over different scalar fields are not supported");
    if (!iso->sf->build(c->stream)) return;
    std::memset(&isoRec, 0, sizeof(isoRec));
    isoRec.iso_value = iso->isoValue;
    isoRec.d_ranges = iso->sf->ranges.p;
    for (int a = 0; a < 4; a++) isoRec.color[a] = iso->material->live.color[a];
    isoRec.opacity = iso->material->live.opacity;
    isoRec.instance = isoInst;
    isoRec.user_id = iso->userID;
  }
  if (env && !env->buildEnv(c->stream)) return;
  if (dirs.size() > 4) return fail("at most 4 directional lights are supported");
  gbv_scene s;
  std::memset(&s, 0, sizeof(s));
  (vol ? vol->sf : iso->sf)->fill(s);
  for (int a = 0; a < 3; a++) {
    s.cam_pos[a] = cam->position[a];
    s.cam_dir[a] = cam->direction[a];
    s.cam_up[a] = cam->up[a];
  }
  if (iso) s.iso = &isoRec;
  s.volume_instance = vol ? volInst : 0;
  s.volume_user_id = vol ? vol->userID : 0;
  // the aux channels the frame buffer holds
  if (f->channels & BN_FB_DEPTH) s.d_depth = f->depth.p;
  if (f->channels & BN_FB_PRIMID) s.d_prim_id = f->primId.p;
  if (f->channels & BN_FB_INSTID) s.d_inst_id = f->instId.p;
  if (f->channels & BN_FB_OBJID) s.d_obj_id = f->objId.p;
  if (vol) {
    s.d_majorants = vol->majorants.p;
    s.d_tf = vol->tf.p;
    s.tf_n = (int)(vol->tfHost.size() / 4);
    s.domain[0] = vol->domain[0];
    s.domain[1] = vol->domain[1];
    s.base_density = vol->densityAt1;
    s.anisotropy = vol->anisotropy;
    s.scattering_albedo = vol->scatteringAlbedo;
  }
  s.fovy = cam->fovy;
  s.num_dir_lights = (int)dirs.size();
  for (size_t i = 0; i < dirs.size(); i++) {
    for (int a = 0; a < 3; a++) {
      s.dir_light_dir[i][a] = dirs[i]->direction[a];
      s.dir_light_color[i][a] = dirs[i]->color[a];
    }
    // DirLight::getDD: irradiance takes precedence when set (DirLight.cu:15-18)
    s.dir_light_radiance[i] = std::isnan(dirs[i]->irradiance) ? dirs[i]->radiance : dirs[i]->irradiance;
  }
  if (env) {
    s.d_env_texels = env->texture->texels.p;
    s.d_env_cdf_y = env->cdfY.p;
    s.d_env_cdf_x = env->cdfX.p;
    s.env_dims[0] = env->texture->W;
    s.env_dims[1] = env->texture->H;
    s.env_addr[0] = env->texture->addr[0];
    s.env_addr[1] = env->texture->addr[1];
    for (int a = 0; a < 3; a++) {
      s.env_dir[a] = env->envDir[a];
      s.env_up[a] = env->envUp[a];
    }
    s.env_scale = env->scale;
  }
  const Renderer::P &rp = r->live;
  for (int a = 0; a < 4; a++) s.bg_color[a] = rp.bg[a];
  s.ambient_radiance = rp.ambient;
  s.multi_scatter = rp.multiScatterBuild;
  s.volume_multi_scatter = rp.volumeMultiScatter;
  s.max_volume_bounces = rp.maxVolumeBounces;
  // counters: [0..GBV_NUM_COUNTERS) event counts (renderer "frameStats" = 1),
  // else only a loop-cap flag, kept in the word after them (the counting
  // kernel is some 3% slower)
  if (!f->counters.alloc(GBV_NUM_COUNTERS + 1, c->mem)) return;
  cudaMemsetAsync(f->counters.p, 0, (GBV_NUM_COUNTERS + 1) * sizeof(unsigned long long), c->stream);
  int *capFlag = reinterpret_cast<int *>(f->counters.p + GBV_NUM_COUNTERS);
  const gbv_status rs = rp.frameStats
                            ? gbv_render(&s, f->accum.p, f->W, f->H, f->accumID, rp.spp, f->counters.p, c->stream)
                            : gbv::render_cap_flagged(&s, f->accum.p, f->W, f->H, f->accumID, rp.spp, capFlag,
                                                      c->stream);
  if (rs != GBV_OK) return fail(gbv_last_error());
  f->accumID += rp.spp;
  // FrameBuffer::finalizeFrame: linearize with accumScale = 1/accumID
  if (f->accumID > 0 &&
      gbv_tonemap(f->accum.p, f->W, f->H, f->accumID, fbFormat(f->colorFormat), f->color.p, c->stream) != GBV_OK)
    return fail(gbv_last_error());
  cudaMemcpyAsync(f->lastStats, f->counters.p, sizeof(f->lastStats), cudaMemcpyDeviceToHost, c->stream);
  unsigned long long capWord = 0;
  cudaMemcpyAsync(&capWord, f->counters.p + GBV_NUM_COUNTERS, sizeof(capWord), cudaMemcpyDeviceToHost, c->stream);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail("bnRender: CUDA error during the frame");
  if (capWord) f->lastStats[3] = 1;
  if (f->lastStats[3]) fail("bnRender: a device loop hit its iteration cap; the frame is partial");
}

void bnFrameBufferRead(BNFrameBuffer fb, BNFrameBufferChannel channel, void *dst, BNDataType requiredFormat) {
  Context *c = nullptr;
  auto f = as<FrameBuffer>(lookup(fb, &c));
  if (!f) return fail("bnFrameBufferRead: unknown frame buffer");
  if (f->accumID == 0) return fail("bnFrameBufferRead: nothing rendered since the last reset");
  const size_t n = (size_t)f->W * f->H;
  const void *src = nullptr;
  size_t bytes = 0;
  if (channel == BN_FB_COLOR) {
    if (requiredFormat != f->colorFormat) return fail("bnFrameBufferRead: format differs from the resize format");
    src = f->color.p;
    bytes = n * (f->colorFormat == BN_FLOAT4 ? 16 : 4);
  } else if (channel == BN_FB_DEPTH || channel == BN_FB_PRIMID || channel == BN_FB_INSTID ||
             channel == BN_FB_OBJID) {
    // FrameBuffer::read (fb/FrameBuffer.cu:310-360): depth as BN_FLOAT, the
    // IDs as 32-bit integers
    if (!(f->channels & channel)) return fail("bnFrameBufferRead: channel not requested at the resize");
    const bool isDepth = channel == BN_FB_DEPTH;
    if (isDepth ? requiredFormat != BN_FLOAT
                : (requiredFormat != BN_INT32 && requiredFormat != BN_UINT32))
      return fail("bnFrameBufferRead: depth reads as BN_FLOAT, IDs as BN_INT32 or BN_UINT32");
    src = isDepth ? (const void *)f->depth.p
          : channel == BN_FB_PRIMID ? (const void *)f->primId.p
          : channel == BN_FB_INSTID ? (const void *)f->instId.p
                                    : (const void *)f->objId.p;
    bytes = n * 4;
  } else {
    return fail("bnFrameBufferRead: the normal channel is not supported");
  }
  cudaSetDevice(c->device);
  if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    fail("bnFrameBufferRead: copy failed");
}

}  // extern "C"
