// render_wavefront.cuh -- the frame render as a wavefront of two kernels per
// step, the alternative to the persistent megakernel of render_kernel.cuh
// (selected by gbv_render_config.mode = GBV_RENDER_WAVEFRONT).
//
// The reference's own structure (Context::renderTiles, barney/Context.cpp:
// 142-185): a trace launch over a queue of rays (traceRays.dev.cu:20-52 ->
// MCVolumeAccel::isProg), then a shade launch over the traced rays
// (shadeRays.cu:881-1041) that writes the next queue.  Here:
//
//  * one slot per pixel holds the pixel's path state in HBM for all of the
//    launch's passes: the main (camera or bounce) ray, the pending shadow
//    ray, the pass and generation numbers; the accumulation buffer itself
//    holds the pixel's running sum, so the pixel's fragments are added in
//    one fixed order with plain adds (no atomics) -- the order of the
//    persistent kernel, and the frames are bit-identical to its frames;
//  * wf_trace_kernel: a persistent grid whose warps take rays from the
//    step's queue and refill idle lanes as their rays finish; the traversal
//    code (box test, DDA, Woodcock, density sample) is the megakernel's, and
//    the kernel holds no shading code, so its instruction working set and
//    register budget are the traversal's alone;
//  * wf_shade_kernel: one thread per active slot: adds the shadow ray's
//    result, shades the main ray's hit or miss (bounce(), env lookups, light
//    sample, MIS), starts the next pass when a path ends, and appends the
//    slot's next rays to the next step's queue (warp-aggregated atomics).
//
// A pixel's next pass starts in the same step as its last shadow ray is
// traced (the two are independent: a primary ray's random numbers depend on
// the pixel and pass only); the shade step adds the shadow ray's fragment
// before the new pass's first one, so the accumulation order is unchanged.
#pragma once
#include "render_kernel.cuh"

namespace gbv {

// A PathRay in three 16-byte words (one vector load or store each).
struct WfRay {
  float4 a;  // org.xyz, tMax
  float4 b;  // dir.xyz, misWeight
  uint4 c;   // seed (lo, hi), tp.x | tp.y << 16, tp.z | numVolumeBounces << 16
};
__device__ __forceinline__ void wf_store(WfRay *r, const PathRay &p) {
  r->a = make_float4(p.org.x, p.org.y, p.org.z, p.tMax);
  r->b = make_float4(p.dir.x, p.dir.y, p.dir.z, p.misWeight);
  r->c = make_uint4((uint32_t)p.seed.state, (uint32_t)(p.seed.state >> 32), (uint32_t)p.tp.x | ((uint32_t)p.tp.y << 16),
                    (uint32_t)p.tp.z | ((uint32_t)p.numVolumeBounces << 16));
}
__device__ __forceinline__ PathRay wf_load(const WfRay *r) {
  const float4 a = r->a, b = r->b;
  const uint4 c = r->c;
  PathRay p;
  p.org = vec3(a.x, a.y, a.z);
  p.tMax = a.w;
  p.dir = vec3(b.x, b.y, b.z);
  p.misWeight = b.w;
  p.seed.state = (uint64_t)c.x | ((uint64_t)c.y << 32);
  p.tp = vec3h{(uint16_t)(c.z & 0xffffu), (uint16_t)(c.z >> 16), (uint16_t)(c.w & 0xffffu)};
  p.numVolumeBounces = (int)(c.w >> 16);
  return p;
}

// Per-slot bookkeeping
struct WfMeta {
  int pass;    // pass of the main ray (0-based within the launch)
  int gen;     // generation of the main ray within its pass
  int spass;   // pass of the pending shadow ray
  int flags;   // kWfMainQueued | kWfShadowQueued
};
constexpr int kWfMainQueued = 1, kWfShadowQueued = 2;

// Per-step counters (zeroed before the first step): queue length and the
// trace kernel's fetch head, number of active slots and its fetch head.
struct WfStep {
  int qlen, qhead, alen, ahead;
};

// Everything the steps share (device pointers; one allocation).
struct WfBuffers {
  WfRay *mainR, *shadowR;
  WfMeta *meta;
  float4 *hit;       // per (slot, kind): t (-inf on a miss) and rgb
  int *queue[2];     // entries slot * 2 + kind (0 main, 1 shadow)
  int *active[2];    // slots with rays in the step
  WfStep *steps;
};

// Slot s <-> pixel: warp tiles of 8x4 pixels, row-major tiles (as the
// persistent kernel hands them out), 32 slots per tile.
__device__ __forceinline__ void wf_pixel(const RenderParams &p, int slot, int &ix, int &iy) {
  const int tile = slot >> 5, k = slot & 31;
  const int tilesX = (int)(((long long)p.W + 7) >> 3);
  ix = (tile % tilesX) * 8 + (k & 7);
  iy = (tile / tilesX) * 4 + (k >> 3);
}

// Warp-aggregated append of `want` (0/1 per lane) entries to a list.
__device__ __forceinline__ int wf_append(int *counter, bool want) {
  const unsigned FULL = 0xffffffffu;
  const unsigned m = __ballot_sync(FULL, want);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (m) {
    const int leader = __ffs(m) - 1;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(FULL, base, leader);
  }
  return base + __popc(m & ((1u << lane) - 1u));
}

// First step: every pixel's first pass (the accumulation starts from the
// buffer's contents unless accum_id_start == 0).
static __global__ void __launch_bounds__(256) wf_init_kernel(const __grid_constant__ RenderParams p, WfBuffers B) {
  const long long nslots = warp_tile_count(p) * 32;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ((nslots + 31) & ~31ll);
       i += (long long)gridDim.x * blockDim.x) {
    const int slot = (int)i;
    int ix = 0, iy = 0;
    bool valid = i < nslots;
    if (valid) {
      wf_pixel(p, slot, ix, iy);
      valid = ix < p.W && iy < p.H;
    }
    if (valid) {
      PathRay ray;
      generate_primary(p, ix, iy, p.accumIdStart, ray);
      wf_store(B.mainR + slot, ray);
      B.meta[slot] = WfMeta{0, 0, 0, kWfMainQueued};
    }
    const int q = wf_append(&B.steps[0].qlen, valid);
    if (valid) B.queue[0][q] = slot * 2;
    const int a = wf_append(&B.steps[0].alen, valid);
    if (valid) B.active[0][a] = slot;
  }
}

// One trace step over the step's queue.  Each warp keeps up to 32 rays in
// flight and takes new ones from the queue when at least `refill` of its
// lanes are idle (or all of them).
template <class Store, bool Count>
__global__ void __launch_bounds__(256, 4) wf_trace_kernel(const __grid_constant__ RenderParams p, WfBuffers B, int step,
                                                       int refill) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  WfStep &S = B.steps[step];
  const int *queue = B.queue[step & 1];
  const int qlen = S.qlen;
  if (p.maskWords > 0) {
    // the bitmask of non-zero majorants in shared memory (as the persistent
    // kernel stages it)
    stage_majorant_mask(p);
    __syncthreads();
  }
  const Store store = make_store<Store>(p);
  Ctr<Count> cnt;
  bool busy = false, done = false;
  int entry = 0;
  Traversal T;
  Hit h;
  h.hit = false;
  while (true) {
    const unsigned idle = __ballot_sync(FULL, !busy);
    if (!done && idle != 0u && (__popc(idle) >= refill || idle == FULL)) {
      int base = 0;
      if (lane == 0) base = atomicAdd(&S.qhead, __popc(idle));
      base = __shfl_sync(FULL, base, 0);
      if (base >= qlen) {
        done = true;
      } else if (!busy) {
        const int r = base + __popc(idle & ((1u << lane) - 1u));
        if (r < qlen) {
          entry = queue[r];
          WfRay *R = (entry & 1) ? B.shadowR + (entry >> 1) : B.mainR + (entry >> 1);
          const float4 a = R->a, b = R->b;
          const uint4 c = R->c;
          RNGSeed seed;
          seed.state = (uint64_t)c.x | ((uint64_t)c.y << 32);
          h.hit = false;
          const bool active = trace_begin(p.F, p.G, p.rcpMc, vec3(a.x, a.y, a.z), vec3(b.x, b.y, b.z), a.w, seed, T,
                                          cnt);
          R->c = make_uint4((uint32_t)seed.state, (uint32_t)(seed.state >> 32), c.z, c.w);
          if (active) busy = true;
          else B.hit[entry] = make_float4(__int_as_float(0xff800000), 0.f, 0.f, 0.f);
        }
      }
    }
    if (done && __all_sync(FULL, !busy)) break;
    if (busy && T.inCell != 2 && trace_seek(p.G, T, cnt, p.skip, p.maskWords > 0, p.capFlag) == TR_MISS) {
      B.hit[entry] = make_float4(__int_as_float(0xff800000), 0.f, 0.f, 0.f);
      busy = false;
    }
    if (busy && T.inCell == 2 && trace_sample(p.F, store, p.xf, T, h, cnt) == TR_HIT) {
      B.hit[entry] = make_float4(h.t, h.rgb.x, h.rgb.y, h.rgb.z);
      busy = false;
    }
  }
  if (Count && p.counters) {
    unsigned long long v[5] = {cnt.samples, cnt.mcs, cnt.rays, cnt.caps, cnt.cells};
#pragma unroll
    for (int k = 0; k < 5; k++) {
      unsigned long long x = v[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(FULL, x, o);
      if (lane == 0 && x) atomicAdd(p.counters + k, x);
    }
  }
}

// One shade step over the step's active slots.
// Resident 256-thread blocks per SM the shade kernel's registers are capped
// for (2: 128 registers, no spills).
#ifndef GBV_WF_SHADE_BLOCKS
#define GBV_WF_SHADE_BLOCKS 2
#endif
template <class Store>
__global__ void __launch_bounds__(256, GBV_WF_SHADE_BLOCKS) wf_shade_kernel(const __grid_constant__ RenderParams p, WfBuffers B, int step) {
  if (p.rowOff >= 0) {
    for (int i = threadIdx.x; i < p.env.H; i += blockDim.x)
      reinterpret_cast<float2 *>(g_smem + p.rowOff)[i] = env_row_terms(p.env, i);
    __syncthreads();
  }
  const WfStep &S = B.steps[step];
  WfStep &N = B.steps[step + 1];
  const int *active = B.active[step & 1];
  int *nqueue = B.queue[(step + 1) & 1];
  int *nactive = B.active[(step + 1) & 1];
  const int alen = S.alen;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ((alen + 31) & ~31);
       i += (long long)gridDim.x * blockDim.x) {
    const bool valid = i < alen;
    int slot = 0, ix = 0, iy = 0;
    bool keep = false, qMain = false, qShadow = false;
    if (valid) {
      slot = active[i];
      wf_pixel(p, slot, ix, iy);
      WfMeta m = B.meta[slot];
      const size_t pix = (size_t)iy * p.W + ix;
      float4 acc = m.pass == 0 && m.gen == 0 && (m.flags & kWfMainQueued) && p.accumIdStart == 0
                       ? make_float4(0.f, 0.f, 0.f, 0.f)
                       : p.accum[pix];
      bool shadowPending = false;
      // the shadow ray first: it belongs to an earlier generation (or pass)
      if (m.flags & kWfShadowQueued) {
        const float4 hr = B.hit[2 * slot + 1];
        if (!(hr.x >= 0.f)) {
          const PathRay sray = wf_load(B.shadowR + slot);
          const float clampMax = 10.f * (float)(1 + p.accumIdStart + m.spass);
          accum_add(acc, vmin(sray.misWeight * from_half(sray.tp), vec3(clampMax)));
        }
      }
      bool mainAlive = false;
      if (m.flags & kWfMainQueued) {
        PathRay ray = wf_load(B.mainR + slot);
        const float4 hr = B.hit[2 * slot];
        Hit h;
        h.hit = hr.x >= 0.f;
        h.t = hr.x;
        h.rgb = vec3(hr.y, hr.z, hr.w);
        // the trace direction: zero components replaced by 1e-6 (as trace_begin does)
        vec3 tdir = ray.dir;
        if (tdir.x == 0.f) tdir.x = 1e-6f;
        if (tdir.y == 0.f) tdir.y = 1e-6f;
        if (tdir.z == 0.f) tdir.z = 1e-6f;
        Random rnd;
        EnvPick pick;
        float2 uv = make_float2(0.f, 0.f);
        bool needTex = false;
        if (h.hit) {
          rnd = Random::derive(ray.seed, (uint64_t)hit_hash(h.t));
          if (p.hasEnv) {
            pick = env_pick_coords(p, rnd);
            uv = make_float2(pick.sx, pick.sy);
            needTex = true;
          }
        } else if (p.hasEnv) {
          uv = env_miss_coords(p, ray.dir);
          needTex = true;
        }
        vec3 texel(0.f);
        if (needTex) {
          const float4 t = tex2D(p.env, uv.x, uv.y);
          texel = p.env.scale * vec3(t.x, t.y, t.z);
        }
        const int accumID = p.accumIdStart + m.pass;
        const float clampMax = 10.f * (float)(1 + accumID);
        vec3 frag(0.f);
        float alpha = 0.f;
        if (!h.hit) {
          const float4 miss = miss_color(p, iy);
          const vec3 env = p.hasEnv ? texel : (m.gen != 0 ? vec3(p.ambient) : vec3(0.f));
          if (m.gen == 0) {
            alpha = miss.w;
            frag = p.hasEnv ? env : vec3(miss.x, miss.y, miss.z);
          } else {
            frag = from_half(ray.tp) * env * ray.misWeight;
          }
          ray.tMax = -1.f;
        } else {
          if (m.gen == 0) alpha = 1.f;
          ShadeOut so;
          pick.radiance = texel;
          bounce_volume_hit(p, ray, h, ray.org + h.t * tdir, m.gen, rnd, pick, so);
          if (so.shadowValid && so.shadow.tMax > 0.f) {
            wf_store(B.shadowR + slot, so.shadow);
            shadowPending = true;
            m.spass = m.pass;
          }
        }
        frag = vmin(frag, vec3(clampMax));
        if (accumID == 0 && m.gen == 0) {
          acc = make_float4(frag.x, frag.y, frag.z, alpha);
        } else {
          if (m.gen == 0 && alpha > 0.f) acc.w += alpha;
          accum_add(acc, frag);
        }
        mainAlive = ray.tMax > 0.f;
        m.gen++;
        if (!mainAlive && m.pass + 1 < p.spp) {
          // the path ended: the pixel's next pass
          m.pass++;
          m.gen = 0;
          generate_primary(p, ix, iy, p.accumIdStart + m.pass, ray);
          mainAlive = true;
        }
        if (mainAlive) wf_store(B.mainR + slot, ray);
      }
      p.accum[pix] = acc;
      qMain = mainAlive;
      qShadow = shadowPending;
      keep = qMain || qShadow;
      m.flags = (qMain ? kWfMainQueued : 0) | (qShadow ? kWfShadowQueued : 0);
      B.meta[slot] = m;
    }
    const int q0 = wf_append(&N.qlen, qShadow);
    if (qShadow) nqueue[q0] = 2 * slot + 1;
    const int q1 = wf_append(&N.qlen, qMain);
    if (qMain) nqueue[q1] = 2 * slot;
    const int a = wf_append(&N.alen, keep);
    if (keep) nactive[a] = slot;
  }
}

// Host side: the steps until no slot is active.  Scratch in HBM: 2 x 48 B
// ray records, 16 B of bookkeeping, 32 B of trace results and 16 B of queue
// and active-list entries per pixel, plus the per-step counters; taken from
// the stream's memory pool and returned after the launch sequence.
template <class Store>
inline gbv_status launch_wavefront(RenderParams p, const Store &, cudaStream_t stream) {
  // the shade kernel stages the env map's row terms only (GBV_STAGE_ALL's
  // CDF tables are read from global memory)
  p.cdfYOff = p.pivOff = -1;
  p.pivPerRow = 0;
  int dev = 0, sms = 0, perSmTrace = 0, perSmShade = 0;
  gbv_status st = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (st == GBV_OK) st = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (st != GBV_OK) return st;
  const long long nslots = warp_tile_count(p) * 32;
  if (nslots > (1ll << 30)) return set_error(GBV_ERROR_INVALID_ARGUMENT, "wavefront render: frame above 2^30 pixels");
  // steps: at most (MAX_PATH_DEPTH + 1) main rays per pass and one step for
  // the last shadow ray
  const long long maxSteps = (long long)p.spp * 12 + 2;
  const size_t traceSmem = (size_t)p.maskWords * 4;
  const size_t shadeSmem = p.rowOff >= 0 ? (size_t)(p.rowOff + 2 * p.env.H) * 4 : 0;
  st = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSmTrace, wf_trace_kernel<Store, false>, 256,
                                                                traceSmem),
                  "wf_trace_kernel: occupancy");
  if (st == GBV_OK)
    st = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSmShade, wf_shade_kernel<Store>, 256, shadeSmem),
                    "wf_shade_kernel: occupancy");
  if (st != GBV_OK) return st;
  const size_t n = (size_t)nslots;
  const size_t bytes = n * (2 * sizeof(WfRay) + sizeof(WfMeta) + 2 * sizeof(float4) + 4 * 2 * sizeof(int) +
                            2 * sizeof(int)) +
                       (size_t)(maxSteps + 1) * sizeof(WfStep) + (size_t)p.maskWords * 4 + 4096;
  char *mem = nullptr;
  st = check_cuda(cudaMallocAsync((void **)&mem, bytes, stream), "cudaMallocAsync(wavefront state)");
  if (st != GBV_OK) return st;
  WfBuffers B;
  size_t off = 0;
  auto take = [&](size_t b) {
    char *q = mem + off;
    off += (b + 255) & ~(size_t)255;
    return q;
  };
  B.mainR = reinterpret_cast<WfRay *>(take(n * sizeof(WfRay)));
  B.shadowR = reinterpret_cast<WfRay *>(take(n * sizeof(WfRay)));
  B.meta = reinterpret_cast<WfMeta *>(take(n * sizeof(WfMeta)));
  B.hit = reinterpret_cast<float4 *>(take(2 * n * sizeof(float4)));
  B.queue[0] = reinterpret_cast<int *>(take(2 * n * sizeof(int)));
  B.queue[1] = reinterpret_cast<int *>(take(2 * n * sizeof(int)));
  B.active[0] = reinterpret_cast<int *>(take(n * sizeof(int)));
  B.active[1] = reinterpret_cast<int *>(take(n * sizeof(int)));
  B.steps = reinterpret_cast<WfStep *>(take((size_t)(maxSteps + 1) * sizeof(WfStep)));
  uint32_t *mask = reinterpret_cast<uint32_t *>(take((size_t)p.maskWords * 4 + 16));
  if (off > bytes) st = set_error(GBV_ERROR_INVALID_ARGUMENT, "wavefront render: scratch layout");
  if (st == GBV_OK)
    st = check_cuda(cudaMemsetAsync(B.steps, 0, (size_t)(maxSteps + 1) * sizeof(WfStep), stream),
                    "wavefront render: clearing the step counters");
  const unsigned gridTrace = (unsigned)(sms * (perSmTrace > 0 ? perSmTrace : 1));
  const unsigned gridShade = (unsigned)(sms * (perSmShade > 0 ? perSmShade : 1));
  if (st == GBV_OK && p.maskWords > 0 && p.maskMode == 0) {
    const int nmc = p.G.M[0] * p.G.M[1] * p.G.M[2];
    majorant_mask_kernel<<<(unsigned)((p.maskWords + 7) / 8), 256, 0, stream>>>(p.G.maj, nmc, p.maskWords, mask);
    st = check_launch("majorant_mask_kernel");
    p.maskSrc = mask;
  }
  if (st == GBV_OK) {
    wf_init_kernel<<<gridShade, 256, 0, stream>>>(p, B);
    st = check_launch("wf_init_kernel");
  }
  // the steps, in batches between reads of the active count; a warp of the
  // trace kernel refills once `refill` of its lanes are idle
  const int refill = p.threshold > 0 ? (p.threshold * 32 + 99) / 100 : 8;
  int alenHost = 1;
  long long k = 0;
  while (st == GBV_OK && k < maxSteps) {
    const long long batch = k < 8 ? 8 : 16;
    for (long long j = 0; j < batch && k < maxSteps && st == GBV_OK; j++, k++) {
      if (p.counters)
        wf_trace_kernel<Store, true><<<gridTrace, 256, traceSmem, stream>>>(p, B, (int)k, refill);
      else
        wf_trace_kernel<Store, false><<<gridTrace, 256, traceSmem, stream>>>(p, B, (int)k, refill);
      st = check_launch("wf_trace_kernel");
      if (st != GBV_OK) break;
      wf_shade_kernel<Store><<<gridShade, 256, shadeSmem, stream>>>(p, B, (int)k);
      st = check_launch("wf_shade_kernel");
    }
    if (st != GBV_OK) break;
    st = check_cuda(cudaMemcpyAsync(&alenHost, &B.steps[k].alen, sizeof(int), cudaMemcpyDeviceToHost, stream),
                    "wavefront render: reading the active count");
    if (st == GBV_OK) st = check_cuda(cudaStreamSynchronize(stream), "wavefront render: step sync");
    if (st == GBV_OK && alenHost == 0) break;
  }
  if (st == GBV_OK && k >= maxSteps && alenHost != 0)
    st = set_error(GBV_ERROR_LIMIT, "wavefront render: step limit reached");
  const gbv_status fst = check_cuda(cudaFreeAsync(mem, stream), "cudaFreeAsync(wavefront state)");
  return st != GBV_OK ? st : fst;
}

// The launchers of one voxel store, defined in render_store_*.cu: the
// persistent megakernel or, with gbv_render_config.mode =
// GBV_RENDER_WAVEFRONT, the trace/shade wavefront.
#define GBV_STORE_LAUNCHERS(NAME, STORE)                                                        \
  gbv_status render_launch_##NAME(const RenderParams &p, cudaStream_t s, const LaunchChoice &lc) { \
    if (lc.mode == GBV_RENDER_WAVEFRONT) {                                                      \
      RenderParams q = p;                                                                       \
      plan_staging(q, lc.stage);                                                                \
      return launch_wavefront(q, STORE{}, s);                                                   \
    }                                                                                           \
    return launch_render(p, STORE{}, s, lc);                                                    \
  }                                                                                             \
  gbv_status render_launch_noalloc_##NAME(const RenderParams &p, cudaStream_t s, int *pool) {   \
    return launch_render_noalloc(p, STORE{}, s, pool);                                          \
  }                                                                                             \
  gbv_status batch_launch_##NAME(const gbv_batch *b, const RenderParams &L, cudaStream_t s) {   \
    return batch_launch<STORE>(b, L, s);                                                        \
  }

}  // namespace gbv
