// scene_gen.cpp -- seeded synthetic structured volumes (host).
//
// The reference's regression volumes are not available; these stand in for
// them.  A volume lives on the unit cube: voxel (i,j,k) sits at
// (i/(Nx-1), j/(Ny-1), k/(Nz-1)).  Its value is
//   clamp( sum_b a_b exp(-|x-c_b|^2 / (2 s_b^2)) + U[0,noise] + fBm(x), 0, 1 )
// with c_b ~ U[0,1]^3, s_b ~ U[0.05,0.2], a_b ~ U[0.2,1] drawn from a
// splitmix64 stream of `seed`.  Each Gaussian is separable, so a blob costs
// one multiply-add per voxel.  The fBm is value noise: octave k has
// 8*2^k lattice cells per axis, amplitude fbm_amplitude*2^-k, lattice values
// U[-1,1], smoothstep-weighted trilinear interpolation.
//
// Built into its own library (libgbv_scenegen.so), apart from the renderer:
// inputs are made by the same code for the GPU path, the CPU oracle and the
// timed CPU baseline, and loading them maps no renderer code.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>
#include "scene_gen.h"

namespace {

inline uint64_t splitmix64(uint64_t &s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
inline double u01(uint64_t &s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }
inline uint64_t hash64(uint64_t a, uint64_t b) {
  uint64_t s = a * 0x9e3779b97f4a7c15ull ^ (b + 0x632be59bd9b4e019ull);
  return splitmix64(s);
}

}  // namespace

extern "C" int sg_blob_volume(const int dims[3], int num_blobs, uint64_t seed, float noise_amplitude, int fbm_octaves,
                              float fbm_amplitude, int nthreads, float *out) {
  if (!dims || !out || dims[0] < 2 || dims[1] < 2 || dims[2] < 2 || num_blobs < 0 || fbm_octaves < 0)
    return 1;
  const int nx = dims[0], ny = dims[1], nz = dims[2];
  uint64_t s = seed;
  struct Blob { double c[3], sig, amp; };
  std::vector<Blob> blobs(num_blobs);
  for (auto &b : blobs) {
    for (int a = 0; a < 3; a++) b.c[a] = u01(s);
    b.sig = 0.05 + 0.15 * u01(s);
    b.amp = 0.2 + 0.8 * u01(s);
  }
  // per-axis Gaussian factors
  const int n[3] = {nx, ny, nz};
  std::vector<std::vector<double>> g(3);
  for (int a = 0; a < 3; a++) {
    g[a].resize((size_t)num_blobs * n[a]);
    for (int b = 0; b < num_blobs; b++)
      for (int i = 0; i < n[a]; i++) {
        double x = (double)i / (double)(n[a] - 1) - blobs[b].c[a];
        g[a][(size_t)b * n[a] + i] = std::exp(-x * x / (2.0 * blobs[b].sig * blobs[b].sig));
      }
  }
  // fBm lattices
  struct Lattice { int L; std::vector<float> v; double amp; };
  std::vector<Lattice> lat(fbm_octaves);
  for (int k = 0; k < fbm_octaves; k++) {
    lat[k].L = 8 << k;
    lat[k].amp = (double)fbm_amplitude * std::ldexp(1.0, -k);
    int L1 = lat[k].L + 1;
    lat[k].v.resize((size_t)L1 * L1 * L1);
    for (size_t i = 0; i < lat[k].v.size(); i++) {
      uint64_t h = hash64(seed ^ (0xf00dull + (uint64_t)k * 0x1000193ull), i);
      lat[k].v[i] = (float)(2.0 * ((double)(h >> 11) * (1.0 / 9007199254740992.0)) - 1.0);
    }
  }
  int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<int> next{0};
  auto work = [&]() {
    std::vector<double> row(nx), wyz(num_blobs);
    while (true) {
      int slice = next.fetch_add(1);
      if (slice >= ny * nz) break;
      int j = slice % ny, k = slice / ny;
      std::fill(row.begin(), row.end(), 0.0);
      for (int b = 0; b < num_blobs; b++) {
        double w = blobs[b].amp * g[1][(size_t)b * ny + j] * g[2][(size_t)b * nz + k];
        const double *gx = &g[0][(size_t)b * nx];
        for (int i = 0; i < nx; i++) row[i] += w * gx[i];
      }
      const double y = (double)j / (ny - 1), z = (double)k / (nz - 1);
      float *o = out + (size_t)nx * (j + (size_t)ny * k);
      for (int i = 0; i < nx; i++) {
        double v = row[i];
        if (noise_amplitude > 0.f) {
          uint64_t h = hash64(seed, (uint64_t)i + (uint64_t)nx * (j + (uint64_t)ny * k));
          v += (double)noise_amplitude * ((double)(h >> 11) * (1.0 / 9007199254740992.0));
        }
        const double x = (double)i / (nx - 1);
        for (const Lattice &L : lat) {
          double p[3] = {x * L.L, y * L.L, z * L.L};
          int c[3];
          double w[3];
          for (int a = 0; a < 3; a++) {
            c[a] = std::min((int)p[a], L.L - 1);
            double f = p[a] - c[a];
            w[a] = f * f * (3.0 - 2.0 * f);
          }
          const int L1 = L.L + 1;
          auto at = [&](int dx, int dy, int dz) {
            return (double)L.v[(size_t)(c[0] + dx) + (size_t)L1 * ((c[1] + dy) + (size_t)L1 * (c[2] + dz))];
          };
          double v00 = at(0, 0, 0) + w[0] * (at(1, 0, 0) - at(0, 0, 0));
          double v01 = at(0, 1, 0) + w[0] * (at(1, 1, 0) - at(0, 1, 0));
          double v10 = at(0, 0, 1) + w[0] * (at(1, 0, 1) - at(0, 0, 1));
          double v11 = at(0, 1, 1) + w[0] * (at(1, 1, 1) - at(0, 1, 1));
          double v0 = v00 + w[1] * (v01 - v00), v1 = v10 + w[1] * (v11 - v10);
          v += L.amp * (v0 + w[2] * (v1 - v0));
        }
        o[i] = (float)std::min(1.0, std::max(0.0, v));
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; t++) pool.emplace_back(work);
  for (auto &th : pool) th.join();
  return 0;
}
