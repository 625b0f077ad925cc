// ref_nanovdb.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The reference pin for NanoVDB fields: the reference's NanoVDB field code
// (barney/volume/NanoVDB.h: NanoVDBDataSampler::DD::sample;
// barney/volume/NanoVDB.cu: NanoVDBData_computeMCs) compiled unchanged with
// the NanoVDB library the reference vendors (3rdParty/nanovdb, 32.7), and
// that library's grid builder (tools::build::Grid + tools::createNanoGrid)
// to make test grids.  The host code of NanoVDB.cu that needs the rest of
// the reference's object model is compiled too but left out of the library
// by the linker (section garbage collection: nothing here calls it).
#include "barney/common/barney-common.h"
#include "barney/common/math.h"
#include "barney/volume/NanoVDB.cu"
#include <nanovdb/tools/GridBuilder.h>
#include <nanovdb/tools/CreateNanoGrid.h>

#include <cstdlib>
#include <cstring>

using namespace BARNEY_NS;

namespace {
// An aligned host copy of a grid buffer
nanovdb::GridHandle<nanovdb::HostBuffer> load(const unsigned char *bytes, size_t n) {
  auto buf = nanovdb::HostBuffer::create(n);
  std::memcpy(buf.data(), bytes, n);
  return nanovdb::GridHandle<nanovdb::HostBuffer>(std::move(buf));
}
}  // namespace

#pragma GCC visibility push(default)
extern "C" {

// Byte offsets and sizes of the NanoVDB float-grid layout:
// [0] sizeof(GridData), [1] offsetof(GridData, mMap), [2] offsetof(GridData,
// mWorldBBox), [3] offsetof(GridData, mVoxelSize), [4] offsetof(GridData,
// mGridType), [5] offsetof(Map, mInvMatF), [6] offsetof(Map, mVecF),
// [7] sizeof(TreeData), [8] offsetof(TreeData, mNodeOffset[3]), [9] sizeof
// root data, [10] sizeof root tile, [11] offsetof(tile, child), [12]
// offsetof(tile, value), [13] offsetof(root, mTableSize), [14] offsetof(root,
// mBackground), [15] offsetof(upper, mChildMask), [16] offsetof(upper,
// mTable), [17] offsetof(lower, mChildMask), [18] offsetof(lower, mTable),
// [19] offsetof(leaf, mValues), [20] sizeof(upper), [21] sizeof(lower),
// [22] sizeof(leaf)
int ref_nanovdb_layout(long long *out) {
  using G = nanovdb::GridData;
  using Root = nanovdb::NanoRoot<float>::DataType;
  using Upper = nanovdb::NanoUpper<float>::DataType;
  using Lower = nanovdb::NanoLower<float>::DataType;
  using Leaf = nanovdb::NanoLeaf<float>::DataType;
  long long v[] = {(long long)sizeof(G),
                   (long long)offsetof(G, mMap),
                   (long long)offsetof(G, mWorldBBox),
                   (long long)offsetof(G, mVoxelSize),
                   (long long)offsetof(G, mGridType),
                   (long long)offsetof(nanovdb::Map, mInvMatF),
                   (long long)offsetof(nanovdb::Map, mVecF),
                   (long long)sizeof(nanovdb::TreeData),
                   (long long)offsetof(nanovdb::TreeData, mNodeOffset) + 3 * 8,
                   (long long)sizeof(Root),
                   (long long)sizeof(Root::Tile),
                   (long long)offsetof(Root::Tile, child),
                   (long long)offsetof(Root::Tile, value),
                   (long long)offsetof(Root, mTableSize),
                   (long long)offsetof(Root, mBackground),
                   (long long)offsetof(Upper, mChildMask),
                   (long long)offsetof(Upper, mTable),
                   (long long)offsetof(Lower, mChildMask),
                   (long long)offsetof(Lower, mTable),
                   (long long)offsetof(Leaf, mValues),
                   (long long)sizeof(Upper),
                   (long long)sizeof(Lower),
                   (long long)sizeof(Leaf)};
  const int n = (int)(sizeof(v) / sizeof(v[0]));
  for (int i = 0; i < n; i++) out[i] = v[i];
  return n;
}

// A NanoVDB float grid from a dense x-fastest array: voxel (i,j,k) of the
// array is index coordinate index_origin + (i,j,k); values equal to
// `background` stay unset (inactive); map: uniform scale voxel_size and the
// translation `translation`.  The grid's bytes go to a malloc'd buffer.
int ref_nanovdb_from_dense(const float *values, const int dims[3], const int index_origin[3], float background,
                           double voxel_size, const double translation[3], unsigned char **out, size_t *bytes) {
  nanovdb::tools::build::Grid<float> grid(background, "pin");
  grid.setTransform(voxel_size, nanovdb::Vec3d(translation[0], translation[1], translation[2]));
  auto acc = grid.getAccessor();
  for (int k = 0; k < dims[2]; k++)
    for (int j = 0; j < dims[1]; j++)
      for (int i = 0; i < dims[0]; i++) {
        const float v = values[i + (size_t)dims[0] * (j + (size_t)dims[1] * k)];
        if (v != background)
          acc.setValue(nanovdb::Coord(index_origin[0] + i, index_origin[1] + j, index_origin[2] + k), v);
      }
  auto handle = nanovdb::tools::createNanoGrid(grid);
  *bytes = handle.size();
  *out = (unsigned char *)std::malloc(*bytes);
  if (!*out) return 1;
  std::memcpy(*out, handle.data(), *bytes);
  return 0;
}

void ref_free(void *p) { std::free(p); }

// NanoVDBDataSampler<float>::DD::sample at n points
int ref_nanovdb_sample(const unsigned char *bytes, size_t n_bytes, const float *P, int n, float *out) {
  auto h = load(bytes, n_bytes);
  auto *grid = h.grid<float>();
  if (!grid) return 1;
  NanoVDBDataSampler<float>::DD dd;
  dd.nvdbGrid = grid;
  (nanovdb::CoordBBox &)dd.indexBounds = grid->indexBBox();
  for (int i = 0; i < n; i++) out[i] = dd.sample(vec3f(P[3 * i], P[3 * i + 1], P[3 * i + 2]));
  return 0;
}

// The field's macrocell grid as NanoVDBData::commit and ::buildMCs set it up
// (NanoVDB.cu:70-92, 193-232), and NanoVDBData_computeMCs (NanoVDB.cu:28-60)
// run for every macrocell.  mc_dims[3], world bounds (float, lower then
// upper) and the ranges (2 floats per macrocell) are returned.
int ref_nanovdb_mc_ranges(const unsigned char *bytes, size_t n_bytes, int mc_dims[3], float world[6],
                          float *ranges, long long max_mcs) {
  auto h = load(bytes, n_bytes);
  const nanovdb::GridMetaData *meta = h.gridMetaData();
  auto bmin = meta->worldBBox().min(), bmax = meta->worldBBox().max();
  const box3f worldBounds(vec3f(bmin[0], bmin[1], bmin[2]), vec3f(bmax[0], bmax[1], bmax[2]));
  NanoVDBData::DD dd;
  dd.worldBounds = worldBounds;
  (nanovdb::CoordBBox &)dd.indexBounds = meta->indexBBox();
  auto sz = meta->indexBBox().dim();
  dd.gridSize = vec3i(sz[0], sz[1], sz[2]);
  dd.gridType = meta->gridType();
  dd.gridData = h.data();
  const vec3i mcDims = divRoundUp(dd.gridSize, vec3i(16));
  const long long nmc = (long long)mcDims.x * mcDims.y * mcDims.z;
  mc_dims[0] = mcDims.x; mc_dims[1] = mcDims.y; mc_dims[2] = mcDims.z;
  world[0] = worldBounds.lower.x; world[1] = worldBounds.lower.y; world[2] = worldBounds.lower.z;
  world[3] = worldBounds.upper.x; world[4] = worldBounds.upper.y; world[5] = worldBounds.upper.z;
  if (nmc > max_mcs) return 1;
  std::vector<range1f> r((size_t)nmc);
  MCGrid::DD mc;
  mc.scalarRanges = r.data();
  mc.dims = mcDims;
  mc.gridOrigin = worldBounds.lower;
  mc.gridSpacing = vec3f(worldBounds.upper - worldBounds.lower) * rcp(vec3f(mcDims));
  rtc::embree::ComputeInterface ci;
  ci.threadIdx = vec3ui(0u);
  ci.blockDim = vec3ui(1u);
  ci.gridDim = vec3ui((uint32_t)nmc, 1u, 1u);
  for (long long t = 0; t < nmc; t++) {
    ci.blockIdx = vec3ui((uint32_t)t, 0u, 0u);
    NanoVDBData_computeMCs<float>(ci, mc, dd);
  }
  for (long long t = 0; t < nmc; t++) {
    ranges[2 * t] = r[(size_t)t].lower;
    ranges[2 * t + 1] = r[(size_t)t].upper;
  }
  return 0;
}

}  // extern "C"
#pragma GCC visibility pop
