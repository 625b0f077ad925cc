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

// The grid types the reference's NanoVDB field reads
// (BARNEY_NANOVDB_FLOAT_TYPES, barney/volume/NanoVDB.h:23-28): f(BuildType)
// for the grid's type; false for any other type.
template <typename F> bool with_build_type(nanovdb::GridType t, F &&f) {
  switch (t) {
  case nanovdb::GridType::Float: f(float()); return true;
  case nanovdb::GridType::Fp4: f(nanovdb::Fp4()); return true;
  case nanovdb::GridType::Fp8: f(nanovdb::Fp8()); return true;
  case nanovdb::GridType::Fp16: f(nanovdb::Fp16()); return true;
  case nanovdb::GridType::FpN: f(nanovdb::FpN()); return true;
  default: return false;
  }
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

// Byte offsets and sizes of the quantized leaves (LeafData<Fp4|Fp8|Fp16|FpN>,
// base LeafFnBase) and of the internal nodes above them:
// [0] offsetof(mFlags), [1] offsetof(mMinimum), [2] offsetof(mQuantum),
// [3] sizeof(LeafFnBase), [4..6] offsetof(mCode) of Fp4, Fp8, Fp16,
// [7..9] sizeof leaf of Fp4, Fp8, Fp16, [10] sizeof(LeafData<FpN>),
// [11] LeafData<FpN>::memUsage(8), [12..15] sizeof upper of Fp4, Fp8, Fp16,
// FpN, [16..19] sizeof lower of the same, [20..23] GridType Float, Fp4, Fp8,
// Fp16, [24] GridType FpN
int ref_nanovdb_fp_layout(long long *out) {
  using Base = nanovdb::LeafFnBase<nanovdb::Coord, nanovdb::Mask, 3>;
  using L4 = nanovdb::NanoLeaf<nanovdb::Fp4>::DataType;
  using L8 = nanovdb::NanoLeaf<nanovdb::Fp8>::DataType;
  using L16 = nanovdb::NanoLeaf<nanovdb::Fp16>::DataType;
  using LN = nanovdb::NanoLeaf<nanovdb::FpN>::DataType;
  long long v[] = {(long long)offsetof(Base, mFlags),
                   (long long)offsetof(Base, mMinimum),
                   (long long)offsetof(Base, mQuantum),
                   (long long)sizeof(Base),
                   (long long)offsetof(L4, mCode),
                   (long long)offsetof(L8, mCode),
                   (long long)offsetof(L16, mCode),
                   (long long)sizeof(L4),
                   (long long)sizeof(L8),
                   (long long)sizeof(L16),
                   (long long)sizeof(LN),
                   (long long)LN::memUsage(8u),
                   (long long)sizeof(nanovdb::NanoUpper<nanovdb::Fp4>::DataType),
                   (long long)sizeof(nanovdb::NanoUpper<nanovdb::Fp8>::DataType),
                   (long long)sizeof(nanovdb::NanoUpper<nanovdb::Fp16>::DataType),
                   (long long)sizeof(nanovdb::NanoUpper<nanovdb::FpN>::DataType),
                   (long long)sizeof(nanovdb::NanoLower<nanovdb::Fp4>::DataType),
                   (long long)sizeof(nanovdb::NanoLower<nanovdb::Fp8>::DataType),
                   (long long)sizeof(nanovdb::NanoLower<nanovdb::Fp16>::DataType),
                   (long long)sizeof(nanovdb::NanoLower<nanovdb::FpN>::DataType),
                   (long long)nanovdb::GridType::Float,
                   (long long)nanovdb::GridType::Fp4,
                   (long long)nanovdb::GridType::Fp8,
                   (long long)nanovdb::GridType::Fp16,
                   (long long)nanovdb::GridType::FpN};
  const int n = (int)(sizeof(v) / sizeof(v[0]));
  for (int i = 0; i < n; i++) out[i] = v[i];
  return n;
}

// A NanoVDB grid from a dense x-fastest array: voxel (i,j,k) of the array
// is index coordinate index_origin + (i,j,k); values equal to `background`
// stay unset (inactive); map: uniform scale voxel_size and the translation
// `translation`.  grid_type: a nanovdb::GridType the reference reads (Float,
// Fp4, Fp8, Fp16, FpN), made by the library's builder with dithering off;
// for FpN, `tolerance` >= 0 is the absolute error the bit width of each leaf
// is chosen for (tools::AbsDiff), else the builder's default for the grid
// class.  `fog`: mark the grid a fog volume (else its class is unknown).
// The grid's bytes go to a malloc'd buffer.
int ref_nanovdb_from_dense_typed(const float *values, const int dims[3], const int index_origin[3], float background,
                                 double voxel_size, const double translation[3], int grid_type, float tolerance,
                                 int fog, unsigned char **out, size_t *bytes) {
  nanovdb::tools::build::Grid<float> grid(background, "pin",
                                          fog ? nanovdb::GridClass::FogVolume : nanovdb::GridClass::Unknown);
  grid.setTransform(voxel_size, nanovdb::Vec3d(translation[0], translation[1], translation[2]));
  auto acc = grid.getAccessor();
  for (int k = 0; k < dims[2]; k++)
    for (int j = 0; j < dims[1]; j++)
      for (int i = 0; i < dims[0]; i++) {
        const float v = values[i + (size_t)dims[0] * (j + (size_t)dims[1] * k)];
        if (v != background)
          acc.setValue(nanovdb::Coord(index_origin[0] + i, index_origin[1] + j, index_origin[2] + k), v);
      }
  using SrcT = nanovdb::tools::build::Grid<float>;
  nanovdb::GridHandle<nanovdb::HostBuffer> handle;
  switch ((nanovdb::GridType)grid_type) {
  case nanovdb::GridType::Float: handle = nanovdb::tools::createNanoGrid(grid); break;
  case nanovdb::GridType::Fp4: handle = nanovdb::tools::createNanoGrid<SrcT, nanovdb::Fp4>(grid); break;
  case nanovdb::GridType::Fp8: handle = nanovdb::tools::createNanoGrid<SrcT, nanovdb::Fp8>(grid); break;
  case nanovdb::GridType::Fp16: handle = nanovdb::tools::createNanoGrid<SrcT, nanovdb::Fp16>(grid); break;
  case nanovdb::GridType::FpN:
    handle = nanovdb::tools::createNanoGrid<SrcT, nanovdb::FpN>(
        grid, nanovdb::tools::StatsMode::Default, nanovdb::CheckMode::Default, false, 0,
        nanovdb::tools::AbsDiff(tolerance));
    break;
  default: return 2;
  }
  *bytes = handle.size();
  *out = (unsigned char *)std::malloc(*bytes);
  if (!*out) return 1;
  std::memcpy(*out, handle.data(), *bytes);
  return 0;
}

int ref_nanovdb_from_dense(const float *values, const int dims[3], const int index_origin[3], float background,
                           double voxel_size, const double translation[3], unsigned char **out, size_t *bytes) {
  return ref_nanovdb_from_dense_typed(values, dims, index_origin, background, voxel_size, translation,
                                      (int)nanovdb::GridType::Float, -1.f, 0, out, bytes);
}

void ref_free(void *p) { std::free(p); }

// NanoVDBDataSampler<BuildType>::DD::sample at n points, BuildType the
// grid's type
int ref_nanovdb_sample(const unsigned char *bytes, size_t n_bytes, const float *P, int n, float *out) {
  auto h = load(bytes, n_bytes);
  const nanovdb::GridMetaData *meta = h.gridMetaData();
  int rc = 1;
  with_build_type(meta->gridType(), [&](auto tag) {
    using T = decltype(tag);
    auto *grid = h.template grid<T>();
    if (!grid) return;
    typename NanoVDBDataSampler<T>::DD dd;
    dd.nvdbGrid = grid;
    (nanovdb::CoordBBox &)dd.indexBounds = grid->indexBBox();
    for (int i = 0; i < n; i++) out[i] = dd.sample(vec3f(P[3 * i], P[3 * i + 1], P[3 * i + 2]));
    rc = 0;
  });
  return rc;
}

// The field's macrocell grid as NanoVDBData::commit and ::buildMCs set it up
// (NanoVDB.cu:70-92, 193-232), and NanoVDBData_computeMCs<BuildType>
// (NanoVDB.cu:28-60, BuildType the grid's type) run for every macrocell.  mc_dims[3], world bounds (float, lower then
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
  const bool known = with_build_type(dd.gridType, [&](auto tag) {
    using T = decltype(tag);
    for (long long t = 0; t < nmc; t++) {
      ci.blockIdx = vec3ui((uint32_t)t, 0u, 0u);
      NanoVDBData_computeMCs<T>(ci, mc, dd);
    }
  });
  if (!known) return 2;
  for (long long t = 0; t < nmc; t++) {
    ranges[2 * t] = r[(size_t)t].lower;
    ranges[2 * t + 1] = r[(size_t)t].upper;
  }
  return 0;
}

}  // extern "C"
#pragma GCC visibility pop
