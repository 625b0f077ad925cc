"""Generates tests/golden/kernels.npz: known-answer vectors for the oracle.

The reference ships no golden vectors for the structured-volume path and
cannot be built here, so these vectors come from a second, independent
restatement of the reference's scalar kernels, written in plain Python with
numpy float32 scalars (IEEE single precision, no fused multiply-add):

* RNG streams        barney/common/barney-common.h:65-152
* fastLog            barney/volume/Volume.h:174-184
* half rounding      rtcore/embree/Float16.cpp (ties away from zero)
* trilinear sample   barney/volume/StructuredData.h:104-115,
                     rtcore/embree/Texture.cpp:324-411
* TF map / majorant  barney/volume/TransferFunction.h:66-116
* macrocell ranges   barney/volume/StructuredData.cu:29-61
* DDA + Woodcock     barney/volume/DDA.h:65-206, Volume.h:188-223,
                     MCAccelerator.h:569-708

Run:  python tests/golden/make_golden.py   (writes kernels.npz beside itself)
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

f32 = np.float32
M64 = (1 << 64) - 1
INF = f32(np.inf)


# ---------------------------------------------------------------- RNG ----
def rng_next(state: int):
    x = state
    count = x >> 61
    state = (x * 6364136223846793005) & M64
    x ^= x >> 22
    return state, (x >> (22 + count)) & 0xFFFFFFFF


def rng_seeded(a: int, b: int) -> int:
    st = 0xCAFEF00DD15EA5E5
    st ^= (2 * a + 1) & 0xFFFFFFFF
    st, _ = rng_next(st)
    st ^= (2 * b) & 0xFFFFFFFF
    st, _ = rng_next(st)
    return st


def rng_derive(seed_state: int, b: int):
    """Random2(RNGSeed &seed, b): returns (stream state, advanced seed state)."""
    st = seed_state
    seed_state, _ = rng_next(seed_state)
    st ^= ((b if b else 290374) << 1) & M64
    st, _ = rng_next(st)
    return st, seed_state


def rng_float(st: int):
    st, u = rng_next(st)
    return st, f32(u & 0xFFFFFF) * f32(1.0 / 16777216.0)


def fnv3(a, b, c):
    off, prime = 0xCBF29CE484222325, 0x100000001B3
    h = off ^ ((prime * a) & M64)
    h = ((h * prime) & M64) ^ b
    h = ((h * prime) & M64) ^ c
    return h


# ----------------------------------------------------------- fastLog ----
def fast_log(f):
    f = f32(f)
    f = (f - f32(1)) / (f + f32(1))
    f2 = f * f
    s = f
    f = f * f2
    s = s + f32(1.0 / 3.0) * f
    f = f * f2
    s = s + f32(1.0 / 5.0) * f
    return s + s


# --------------------------------------------------------------- half ----
def float_to_half(value) -> int:
    i = int(np.array(value, dtype=np.float32).view(np.int32))
    s = (i >> 16) & 0x8000
    e = ((i >> 23) & 0xFF) - (127 - 15)
    m = i & 0x7FFFFF
    if e <= 0:
        if e < -10:
            return s
        m = (m | 0x800000) >> (1 - e)
        if m & 0x1000:
            m += 0x2000
        return s | (m >> 13)
    if e == 0xFF - (127 - 15):
        if m == 0:
            return s | 0x7C00
        m >>= 13
        return s | 0x7C00 | m | (m == 0)
    if m & 0x1000:
        m += 0x2000
        if m & 0x800000:
            m = 0
            e += 1
    if e > 30:
        return s | 0x7C00
    return s | (e << 10) | (m >> 13)


# ------------------------------------------------------------ helpers ----
def mn(a, b):
    return b if b < a else a


def mx(a, b):
    return b if a < b else a


def lerp(f, a, b):
    return (f32(1) - f) * a + f * b


def lerp_coords(N, tc):
    if tc - f32(0.5) <= f32(0):
        return 0, 0, f32(0)
    if tc - f32(0.5) >= f32(N - 1):
        return N - 1, N - 1, f32(0)
    i0 = int(tc - f32(0.5))
    return i0, i0 + 1, (tc - f32(0.5)) - f32(i0)


class Field:
    def __init__(self, vol, origin, spacing):
        self.v = vol.astype(np.float32)
        nz, ny, nx = vol.shape
        self.N = (nx, ny, nz)
        self.C = (nx - 1, ny - 1, nz - 1)
        self.origin = [f32(x) for x in origin]
        self.rcp = [f32(1) / f32(x) for x in spacing]
        self.lo = self.origin
        self.hi = [self.origin[a] + f32(spacing[a]) * f32(self.C[a]) for a in range(3)]

    def sample(self, P):
        rel = [(f32(P[a]) - self.origin[a]) * self.rcp[a] for a in range(3)]
        if any(r < f32(0) for r in rel) or any(rel[a] >= f32(self.C[a]) for a in range(3)):
            return f32(np.nan)
        c = [lerp_coords(self.N[a], rel[a] + f32(0.5)) for a in range(3)]
        (x0, x1, fx), (y0, y1, fy), (z0, z1, fz) = c
        at = lambda i, j, k: self.v[k, j, i]
        v00 = lerp(fx, at(x0, y0, z0), at(x1, y0, z0))
        v01 = lerp(fx, at(x0, y1, z0), at(x1, y1, z0))
        v10 = lerp(fx, at(x0, y0, z1), at(x1, y0, z1))
        v11 = lerp(fx, at(x0, y1, z1), at(x1, y1, z1))
        return lerp(fz, lerp(fy, v00, v01), lerp(fy, v10, v11))


class TF:
    def __init__(self, values, lo, hi, bd):
        self.v = values.astype(np.float32)
        self.n = values.shape[0]
        self.lo, self.span, self.bd = f32(lo), f32(hi) - f32(lo), f32(bd)

    def map(self, s):
        f = (f32(s) - self.lo) / self.span
        f = mn(f32(1), mx(f32(0), f))
        f = f * f32(self.n - 1)
        idx = mn(self.n - 2, mx(0, int(f)))
        f = f - f32(idx)
        r = [lerp(f, self.v[idx, k], self.v[idx + 1, k]) for k in range(4)]
        r[3] = r[3] * self.bd
        return r

    def majorant(self, lower, upper):
        lower, upper = f32(lower), f32(upper)
        if lower > upper:
            return f32(0)
        fl = mn(f32(1), mx(f32(0), (lower - self.lo) / self.span)) * f32(self.n - 1)
        fh = mn(f32(1), mx(f32(0), (upper - self.lo) / self.span)) * f32(self.n - 1)
        il = mn(self.n - 2, mx(0, int(fl)))
        ih = mn(self.n - 2, mx(0, int(fh)))
        fl = fl - f32(il)
        fh = fh - f32(ih)
        m = f32(0)
        m = mx(m, lerp(fl, self.v[il, 3], self.v[il + 1, 3]))
        m = mx(m, lerp(fh, self.v[ih, 3], self.v[ih + 1, 3]))
        for i in range(il + 1, ih + 1):
            m = mx(m, self.v[i, 3])
        return m * self.bd


def mc_ranges(vol, cpm):
    nz, ny, nx = vol.shape
    M = [(n - 1 + cpm - 1) // cpm for n in (nx, ny, nz)]
    out = np.zeros((M[0] * M[1] * M[2], 2), np.float32)
    for cz in range(M[2]):
        for cy in range(M[1]):
            for cx in range(M[0]):
                blk = vol[cz * cpm:cz * cpm + cpm + 1, cy * cpm:cy * cpm + cpm + 1, cx * cpm:cx * cpm + cpm + 1]
                out[cx + M[0] * (cy + M[1] * cz)] = (blk.min(), blk.max())
    return M, out


def trace(field: Field, tf: TF, maj, M, cpm, spacing, org, dir_, tmax, seed_state):
    """One ray through the volume; returns (hit, t, rgb, seed_state)."""
    d = [f32(x) if f32(x) != f32(0) else f32(1e-6) for x in dir_]
    o = [f32(x) for x in org]
    t0, t1 = f32(0), f32(tmax)
    tn, tf_ = [], []
    for a in range(3):
        r = f32(1) / d[a]
        lo = (field.lo[a] - o[a]) * r
        hi = (field.hi[a] - o[a]) * r
        tn.append(mn(lo, hi))
        tf_.append(mx(lo, hi))
    t0 = mx(t0, mx(mx(tn[0], tn[1]), tn[2]))
    t1 = mn(t1, mn(mn(tf_[0], tf_[1]), tf_[2]))
    if not (t0 <= t1):
        return False, f32(0), [f32(0)] * 3, seed_state
    mcs = [f32(cpm) * f32(s) for s in spacing]
    rmc = [f32(1) / m for m in mcs]
    dorg = [(o[a] - field.lo[a]) * rmc[a] for a in range(3)]
    ddir = [d[a] * rmc[a] for a in range(3)]
    st, seed_state = rng_derive(seed_state, fnv3(0, 0, 0))
    tMax = t1
    fs = [f32(m) for m in M]
    rd = [f32(1) / x for x in ddir]
    tlo = [(f32(0) - dorg[a]) * rd[a] for a in range(3)]
    thi = [(fs[a] - dorg[a]) * rd[a] for a in range(3)]
    tnr = [mn(tlo[a], thi[a]) for a in range(3)]
    tfr = [mx(tlo[a], thi[a]) for a in range(3)]
    ray_t0 = mx(f32(0), mx(mx(tnr[0], tnr[1]), tnr[2]))
    ray_t1 = mn(tMax, mn(mn(tfr[0], tfr[1]), tfr[2]))
    if ray_t0 > ray_t1:
        return False, f32(0), [f32(0)] * 3, seed_state
    oiv = [dorg[a] + ray_t0 * ddir[a] for a in range(3)]
    fcell = [mx(f32(0), mn(fs[a] - f32(1), f32(np.floor(oiv[a])))) for a in range(3)]
    fend = [fcell[a] + f32(1) if ddir[a] > 0 else fcell[a] for a in range(3)]
    tstep = [f32(abs(rd[a])) for a in range(3)]
    tnext = [f32(abs(fend[a] - oiv[a])) * tstep[a] for a in range(3)]
    stop = [M[a] if ddir[a] > 0 else -1 for a in range(3)]
    delta = [1 if ddir[a] > 0 else -1 for a in range(3)]
    cell = [int(fcell[a]) for a in range(3)]
    ncb = f32(0)
    while True:
        tc = mn(mn(tnext[0], tnext[1]), tnext[2])
        ct0 = ray_t0 + ncb
        ct1 = ray_t0 + mn(tc, tMax)
        m = maj[cell[0] + M[0] * (cell[1] + M[1] * cell[2])]
        if m != f32(0):
            hi = mn(ct1, f32(tmax))
            t = ct0
            while True:
                st, r = rng_float(st)
                dt = -fast_log(f32(1) - r) / m
                t = t + dt
                if t >= hi:
                    break
                P = [o[a] + t * d[a] for a in range(3)]
                s = field.sample(P)
                smp = [f32(0)] * 4 if np.isnan(s) else tf.map(s)
                st, r2 = rng_float(st)
                if smp[3] >= r2 * m:
                    return True, t, smp[:3], seed_state
        ncb = tc
        for a in range(3):
            if tnext[a] == tc:
                tnext[a] = tnext[a] + tstep[a]
                cell[a] += delta[a]
                if cell[a] == stop[a]:
                    return False, f32(0), [f32(0)] * 3, seed_state


def main():
    rng = np.random.default_rng(1234)
    out = {}
    # RNG streams
    pairs = [(0, 0), (1, 2), (255, 17), (1920 * 63 + 5, 1080 * 63 + 7), (0xFFFFFFFF, 123456789)]
    seqs = []
    for a, b in pairs:
        st = rng_seeded(a, b)
        seq = []
        for _ in range(16):
            st, x = rng_float(st)
            seq.append(x)
        seqs.append(seq)
    out["rng_pairs"] = np.array(pairs, dtype=np.uint64)
    out["rng_seq"] = np.array(seqs, dtype=np.float32)
    # derive with the volume stream hash
    dseeds = [0xCAFEF00DD15EA5E5, 0x123456789ABCDEF0, rng_seeded(7, 9)]
    dseq, dnew = [], []
    for s0 in dseeds:
        st, s1 = rng_derive(s0, fnv3(0, 0, 0))
        seq = []
        for _ in range(8):
            st, x = rng_float(st)
            seq.append(x)
        dseq.append(seq)
        dnew.append(s1)
    out["derive_seed"] = np.array(dseeds, dtype=np.uint64)
    out["derive_seq"] = np.array(dseq, dtype=np.float32)
    out["derive_new_seed"] = np.array(dnew, dtype=np.uint64)
    # fastLog
    xs = np.concatenate([rng.uniform(2 ** -24, 1, 64), [2 ** -24, 0.5, 1.0, 0.999999]]).astype(np.float32)
    out["fastlog_x"] = xs
    out["fastlog_y"] = np.array([fast_log(x) for x in xs], dtype=np.float32)
    # half rounding, including exact ties
    hx = np.concatenate([rng.normal(0, 10, 64), [1 + 2 ** -11, 1 + 3 * 2 ** -11, 2 ** -15 * 1.5, 65520.0,
                                                 -0.0, 6e-8, 3e-8]]).astype(np.float32)
    out["half_x"] = hx
    out["half_y"] = np.array([float_to_half(x) for x in hx], dtype=np.uint16)
    # a small field, TF, samples, ranges, majorants and traced rays
    vol = rng.uniform(0, 1, (9, 8, 10)).astype(np.float32)
    vol[4, 3, 5] = 3.0
    origin, spacing = (-0.5, -0.4, -0.45), (0.11, 0.12, 0.1)
    field = Field(vol, origin, spacing)
    tfv = np.stack([np.linspace(0, 1, 16), np.linspace(1, 0, 16), np.full(16, 0.3), np.linspace(0, 0.9, 16) ** 2],
                   axis=1).astype(np.float32)
    tf = TF(tfv, 0.1, 0.9, 7.5)
    P = rng.uniform(-0.6, 0.6, (200, 3)).astype(np.float32)
    out["vol"] = vol
    out["origin"] = np.array(origin, np.float32)
    out["spacing"] = np.array(spacing, np.float32)
    out["tf"] = tfv
    out["tf_dom"] = np.array([0.1, 0.9, 7.5], np.float32)
    out["sample_P"] = P
    out["sample_v"] = np.array([field.sample(p) for p in P], dtype=np.float32)
    S = rng.uniform(-0.2, 1.2, 100).astype(np.float32)
    out["map_s"] = S
    out["map_rgba"] = np.array([tf.map(s) for s in S], dtype=np.float32)
    cpm = 2
    M, ranges = mc_ranges(vol, cpm)
    out["mc_cpm"] = np.array([cpm], np.int32)
    out["mc_dims"] = np.array(M, np.int32)
    out["mc_ranges"] = ranges
    maj = np.array([tf.majorant(a, b) for a, b in ranges], dtype=np.float32)
    out["mc_majorants"] = maj
    rays = []
    for k in range(48):
        org = rng.uniform(-1.5, 1.5, 3)
        tgt = rng.uniform(-0.3, 0.3, 3)
        d = tgt - org
        d = d / np.linalg.norm(d)
        if k % 8 == 0:
            d[k // 8 % 3] = 0.0  # zero direction components take the 1e-6 path
        seed = rng_seeded(k, 3 * k + 1)
        hit, t, rgb, nseed = trace(field, tf, maj, M, cpm, spacing, org.astype(np.float32), d.astype(np.float32),
                                   f32(1e30), seed)
        rays.append((org, d, seed, hit, t, rgb, nseed))
    out["ray_org"] = np.array([r[0] for r in rays], np.float32)
    out["ray_dir"] = np.array([r[1] for r in rays], np.float32)
    out["ray_seed"] = np.array([r[2] for r in rays], np.uint64)
    out["ray_hit"] = np.array([r[3] for r in rays], np.int32)
    out["ray_t"] = np.array([r[4] for r in rays], np.float32)
    out["ray_rgb"] = np.array([r[5] for r in rays], np.float32)
    out["ray_new_seed"] = np.array([r[6] for r in rays], np.uint64)
    path = Path(__file__).resolve().parent / "kernels.npz"
    np.savez_compressed(path, **out)
    print("wrote", path, "hits:", int(out["ray_hit"].sum()), "/", len(rays))


if __name__ == "__main__":
    main()
