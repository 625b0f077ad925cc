"""CPU oracle (TEST INFRASTRUCTURE ONLY) for the structured-volume path.

A restatement of the reference renderer's embree (CPU) backend for this path
(gbv_oracle.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg may use it, and only as the checker.

Pinned by the reference's own code where that compiles here (oracle.refpin,
tests/test_oracle_refpin.py); see gbv_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_f3 = C.c_float * 3


class OrcScene(C.Structure):
    _fields_ = [
        ("scalars", C.c_void_p), ("dims", C.c_int * 3), ("origin", _f3), ("spacing", _f3),
        ("cells_per_mc", C.c_int), ("majorants", C.c_void_p),
        ("tf", C.c_void_p), ("tf_n", C.c_int), ("domain", C.c_float * 2), ("base_density", C.c_float),
        ("anisotropy", C.c_float), ("scattering_albedo", C.c_float),
        ("cam_pos", _f3), ("cam_dir", _f3), ("cam_up", _f3), ("fovy", C.c_float),
        ("num_dir_lights", C.c_int), ("dir_light_dir", _f3 * 4), ("dir_light_color", _f3 * 4),
        ("dir_light_radiance", C.c_float * 4),
        ("env_texels", C.c_void_p), ("env_dims", C.c_int * 2), ("env_addr", C.c_int * 2),
        ("env_dir", _f3), ("env_up", _f3), ("env_scale", C.c_float),
        ("bg_color", C.c_float * 4), ("ambient_radiance", C.c_float),
        ("multi_scatter", C.c_int), ("volume_multi_scatter", C.c_int), ("max_volume_bounces", C.c_int),
        ("width", C.c_int), ("height", C.c_int), ("u8_scaled", C.c_int), ("bounded_math", C.c_int),
        ("nanovdb", C.c_void_p), ("nanovdb_bytes", C.c_ulonglong),
        ("iso_enabled", C.c_int), ("iso_value", C.c_float), ("iso_color", C.c_float * 4),
        ("iso_opacity", C.c_float), ("iso_instance", C.c_int), ("volume_instance", C.c_int),
        ("no_volume", C.c_int), ("volume_user_id", C.c_int), ("iso_user_id", C.c_int),
        ("aux_depth", C.c_void_p), ("aux_prim_id", C.c_void_p), ("aux_inst_id", C.c_void_p),
        ("aux_obj_id", C.c_void_p),
    ]


class OrcShadeWorld(C.Structure):
    """orc_shade_world: the world one shading step sees (DD-level values)."""
    _fields_ = [
        ("num_dir_lights", C.c_int), ("dir_light_dir", _f3 * 4), ("dir_light_color", _f3 * 4),
        ("dir_light_radiance", C.c_float * 4),
        ("env_texels", C.c_void_p), ("env_dims", C.c_int * 2), ("env_addr", C.c_int * 2),
        ("env_to_world", C.c_float * 9), ("env_to_local", C.c_float * 9), ("env_scale", C.c_float),
        ("env_cdf_y", C.c_void_p), ("env_cdf_x", C.c_void_p),
        ("ambient_radiance", C.c_float), ("volume_multi_scatter", C.c_int), ("max_volume_bounces", C.c_int),
    ]


class OrcShadePath(C.Structure):
    """orc_shade_path: a ray with its hit record and path state."""
    _fields_ = [
        ("org", _f3), ("dir", _f3), ("tmax", C.c_float), ("seed", C.c_uint64), ("hit", C.c_int),
        ("P", _f3), ("rgb", _f3), ("g", C.c_float), ("scattering_albedo", C.c_float), ("N", _f3),
        ("color", C.c_float * 4), ("opacity", C.c_float), ("shadow", C.c_int), ("tp", C.c_uint16 * 3),
        ("pad", C.c_uint16), ("mis", C.c_float), ("diffuse_bounces", C.c_int), ("volume_bounces", C.c_int),
        ("miss_color", C.c_float * 4),
    ]


class OrcStats(C.Structure):
    _fields_ = [("density_samples", C.c_uint64), ("mc_visits", C.c_uint64), ("rays", C.c_uint64)]


class OrcEAView(C.Structure):
    _fields_ = [("pos", _f3), ("dir", _f3), ("up", _f3), ("fovy", C.c_float),
                ("width", C.c_int), ("height", C.c_int)]


_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        sp = C.POINTER(OrcScene)
        sigs = {
            "orc_rng_sequence": (None, [C.c_uint32, C.c_uint32, i, vp]),
            "orc_rng_from_seed": (None, [C.c_uint64, C.c_uint64, i, i, vp, C.POINTER(C.c_uint64)]),
            "orc_rng_seed_state": (C.c_uint64, [C.c_uint32, C.c_uint32]),
            "orc_hash3": (C.c_uint64, [C.c_uint32, C.c_uint32, C.c_uint32]),
            "orc_fast_log": (f, [f]),
            "orc_float_to_half": (C.c_uint16, [f]),
            "orc_half_to_float": (f, [C.c_uint16]),
            "orc_sample_points": (None, [sp, vp, i, vp]),
            "orc_tf_map": (None, [sp, vp, i, vp]),
            "orc_mc_dims": (None, [vp, i, vp]),
            "orc_mc_ranges": (None, [vp, vp, i, vp]),
            "orc_scene_mc_ranges": (None, [sp, vp]),
            "orc_scene_mc_grid": (None, [sp, vp, vp]),
            "orc_majorants": (None, [vp, i, vp, i, f, f, f, vp]),
            "orc_trace_ray": (i, [sp, vp, vp, f, C.POINTER(C.c_uint64), C.POINTER(C.c_float), vp]),
            "orc_iso_intersect": (i, [sp, vp, f, vp, vp, f, vp]),
            "orc_iso_hit": (i, [sp, vp, f, vp, f, i, vp, vp, f, C.POINTER(C.c_uint64), C.POINTER(C.c_float),
                                vp, vp, vp]),
            "orc_lambertian": (None, [vp, vp, vp, vp, C.c_uint32, C.c_uint32, vp]),
            "orc_bounce": (None, [C.POINTER(OrcShadeWorld), i, i, C.POINTER(OrcShadePath), C.POINTER(OrcShadePath),
                                  vp]),
            "orc_camera_commit": (None, [vp, vp, vp, f, vp]),
            "orc_generate": (i, [vp, vp, vp, f, i, i, i, vp, vp, vp]),
            "orc_render": (None, [sp, vp, i, i, i, i, i, i, C.POINTER(OrcStats)]),
            "orc_tonemap": (None, [vp, i, i, i, i, vp]),
            "orc_env_cdfs": (None, [vp, vp, vp, vp, vp]),
            "orc_ea_render": (None, [sp, C.POINTER(OrcEAView), i, f, i, i, vp]),
            "orc_ea_backward": (None, [sp, C.POINTER(OrcEAView), i, f, vp, i, vp, vp]),
            "orc_bounded_sincos": (None, [vp, C.c_longlong, vp, vp]),
            "orc_bounded_angles": (None, [vp, vp, C.c_longlong, vp, vp]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)


def bounded_sincos(x: np.ndarray):
    """Sine and cosine of angles in [-pi/4, 2 pi + pi/4] by the oracle's
    bounded method (one of those orc_scene.bounded_math selects)."""
    x = np.ascontiguousarray(x, np.float32)
    sn, cs = np.empty_like(x), np.empty_like(x)
    lib().orc_bounded_sincos(_p(x), x.size, _p(sn), _p(cs))
    return sn, cs


def bounded_angles(y: np.ndarray, x: np.ndarray):
    """acos(x) and atan2(y, x) by the oracle's bounded methods."""
    y = np.ascontiguousarray(y, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    ac, at = np.empty_like(x), np.empty_like(x)
    lib().orc_bounded_angles(_p(y), _p(x), x.size, _p(ac), _p(at))
    return ac, at


class Oracle:
    """Oracle view of a barney_gb300.scenes.Scene (keeps its arrays alive)."""

    def __init__(self, scene, scalars=None, majorants=None, u8=False, bounded_math=False, nanovdb=None):
        """u8=True samples the field as the library's U8 brick store holds it
        (8-bit per 8^3-cell scale brick) and bounds macrocells by the
        dequantized corners -- float arithmetic only.  bounded_math=True
        takes the path's sines, cosines, arc cosines and arc tangents
        (scattering azimuth, env-map CDF rows, env sample and pdf angles,
        env lookups) by the device code's bounded methods instead of libm's."""
        self.s = scene
        self.u8 = bool(u8)
        self.scalars = np.ascontiguousarray(scene.scalars if scalars is None else scalars, dtype=np.float32)
        self.tf = np.ascontiguousarray(scene.tf, dtype=np.float32)
        self.majorants = None if majorants is None else np.ascontiguousarray(majorants, dtype=np.float32)
        self.env = None if scene.env is None else np.ascontiguousarray(scene.env.texels, dtype=np.float32)
        r = OrcScene()
        nz, ny, nx = self.scalars.shape
        r.scalars = self.scalars.ctypes.data
        r.dims[:] = [nx, ny, nz]
        origin, spacing = scene.geometry()
        r.origin[:] = list(origin)
        r.spacing[:] = list(spacing)
        r.cells_per_mc = scene.cells_per_mc
        r.majorants = None if self.majorants is None else self.majorants.ctypes.data
        r.tf = self.tf.ctypes.data
        r.tf_n = self.tf.shape[0]
        r.domain[:] = list(scene.domain)
        r.base_density = scene.base_density
        r.anisotropy, r.scattering_albedo = scene.anisotropy, scene.scattering_albedo
        r.cam_pos[:] = list(scene.cam_pos)
        r.cam_dir[:] = list(scene.cam_dir)
        r.cam_up[:] = list(scene.cam_up)
        r.fovy = scene.fovy
        r.num_dir_lights = len(scene.dir_lights)
        for i, (d, c, rad) in enumerate(scene.dir_lights[:4]):
            r.dir_light_dir[i][:] = list(d)
            r.dir_light_color[i][:] = list(c)
            r.dir_light_radiance[i] = rad
        if self.env is not None:
            e = scene.env
            H, W, _ = self.env.shape
            r.env_texels = self.env.ctypes.data
            r.env_dims[:] = [W, H]
            r.env_addr[:] = list(e.addr)
            r.env_dir[:] = list(e.direction)
            r.env_up[:] = list(e.up)
            r.env_scale = e.scale
        r.bg_color[:] = list(scene.bg_color)
        r.ambient_radiance = scene.ambient
        r.multi_scatter = scene.multi_scatter
        r.volume_multi_scatter = scene.volume_multi_scatter
        r.max_volume_bounces = scene.max_volume_bounces
        r.width, r.height = scene.width, scene.height
        r.u8_scaled = 1 if self.u8 else 0
        r.bounded_math = 1 if bounded_math else 0
        # nanovdb: the bytes of a NanoVDB float grid (the field instead of scalars)
        self.nanovdb = None if nanovdb is None else np.frombuffer(bytes(nanovdb), dtype=np.uint8).copy()
        if self.nanovdb is not None:
            r.nanovdb = self.nanovdb.ctypes.data
            r.nanovdb_bytes = self.nanovdb.size
        iso = getattr(scene, "iso", None)
        if iso is not None:
            r.iso_enabled = 1
            r.iso_value = iso.value
            r.iso_color[:] = [float(c) for c in iso.color]
            r.iso_opacity = iso.opacity
            r.iso_instance = iso.instance
            r.iso_user_id = getattr(iso, "user_id", 0)
            r.no_volume = 1 if scene.no_volume else 0
        r.volume_instance = getattr(scene, "volume_instance", 0)
        r.volume_user_id = getattr(scene, "volume_user_id", 0)
        self.rec = r

    # -- macrocells --
    def mc_dims(self):
        out = (C.c_int * 3)()
        lib().orc_mc_dims((C.c_int * 3)(*self.rec.dims), self.s.cells_per_mc, out)
        return tuple(out)

    def mc_grid(self):
        """(macrocell dims, world bounds lower+upper) of the scene's field."""
        m = (C.c_int * 3)()
        w = (C.c_float * 6)()
        lib().orc_scene_mc_grid(C.byref(self.rec), m, w)
        return tuple(m), tuple(w)

    def mc_ranges(self) -> np.ndarray:
        M = self.mc_grid()[0]
        out = np.empty((M[0] * M[1] * M[2], 2), dtype=np.float32)
        lib().orc_scene_mc_ranges(C.byref(self.rec), _p(out))
        return out

    def iso_intersect(self, rays: np.ndarray, iso: float, ranges=None) -> np.ndarray:
        """rays: (n, 8) float32 (org xyz, tmax, dir xyz, unused).  Returns (n, 8):
        t, P xyz, N xyz, hit (1/0) -- the layout of gbv_iso_intersect."""
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros((rays.shape[0], 8), np.float32)
        rp = None if ranges is None else _p(np.ascontiguousarray(ranges, np.float32))
        o7 = np.zeros(7, np.float32)
        for k in range(rays.shape[0]):
            h = lib().orc_iso_intersect(C.byref(self.rec), rp, iso, _p(rays[k, 0:3].copy()), _p(rays[k, 4:7].copy()),
                                        float(rays[k, 3]), _p(o7))
            if h:
                out[k, :7] = o7
                out[k, 7] = 1.0
        return out

    def iso_hit(self, org, dir, tmax, seed_state, iso, color=(0.8, 0.8, 0.8, 1.0), opacity=1.0, inst=0,
                ranges=None):
        """One ray against the iso-surface with a matte material (orc_iso_hit).
        Returns (hit, seed_state_out, t, P, N as 3 uint16 halfs, albedo+alpha)."""
        if ranges is None:
            ranges = self.mc_ranges()
        rg = np.ascontiguousarray(ranges, np.float32)
        seed = C.c_uint64(seed_state)
        t = C.c_float(0.0)
        P = np.zeros(3, np.float32)
        Nh = np.zeros(3, np.uint16)
        alb = np.zeros(4, np.float32)
        h = lib().orc_iso_hit(C.byref(self.rec), _p(rg), iso, _p(np.asarray(color, np.float32)), opacity, inst,
                              _p(np.asarray(org, np.float32)), _p(np.asarray(dir, np.float32)), tmax,
                              C.byref(seed), C.byref(t), _p(P), _p(Nh), _p(alb))
        return bool(h), seed.value, t.value, P, Nh, alb

    def majorants_of(self, ranges: np.ndarray) -> np.ndarray:
        out = np.empty(ranges.shape[0], dtype=np.float32)
        lib().orc_majorants(_p(np.ascontiguousarray(ranges, dtype=np.float32)), ranges.shape[0], _p(self.tf),
                            self.tf.shape[0], self.s.domain[0], self.s.domain[1], self.s.base_density, _p(out))
        return out

    # -- scalar kernels --
    def sample(self, P: np.ndarray) -> np.ndarray:
        P = np.ascontiguousarray(P, dtype=np.float32).reshape(-1, 3)
        out = np.empty(P.shape[0], dtype=np.float32)
        lib().orc_sample_points(C.byref(self.rec), _p(P), P.shape[0], _p(out))
        return out

    def tf_map(self, s: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(s, dtype=np.float32).reshape(-1)
        out = np.empty((s.shape[0], 4), dtype=np.float32)
        lib().orc_tf_map(C.byref(self.rec), _p(s), s.shape[0], _p(out))
        return out

    # -- render --
    def render(self, spp=None, accum=None, accum_id_start=0, use_double=False, nthreads=0, rows=None, aux=None):
        """aux: auxiliary channels to write, numpy arrays of (H, W) entries
        under "depth" (float32), "prim_id", "inst_id", "obj_id" (int32)."""
        W, H = self.s.width, self.s.height
        if use_double and self.u8:
            raise ValueError("the U8 storage form is sampled in float only")
        if accum is None:
            accum = np.zeros((H, W, 4), dtype=np.float32)
        st = OrcStats()
        r0, r1 = rows if rows is not None else (0, 0)
        aux = aux or {}
        for f, k, dt in (("aux_depth", "depth", np.float32), ("aux_prim_id", "prim_id", np.int32),
                         ("aux_inst_id", "inst_id", np.int32), ("aux_obj_id", "obj_id", np.int32)):
            a = aux.get(k)
            if a is not None:
                assert a.dtype == dt and a.flags.c_contiguous and a.size == W * H, k
            setattr(self.rec, f, a.ctypes.data if a is not None else None)
        lib().orc_render(C.byref(self.rec), _p(accum), accum_id_start, self.s.spp if spp is None else spp,
                         1 if use_double else 0, nthreads, r0, r1, C.byref(st))
        for f in ("aux_depth", "aux_prim_id", "aux_inst_id", "aux_obj_id"):
            setattr(self.rec, f, None)
        self.stats = dict(density_samples=st.density_samples, mc_visits=st.mc_visits, rays=st.rays)
        return accum

    def tonemap(self, accum: np.ndarray, accum_id: int, fmt: int = 0) -> np.ndarray:
        H, W, _ = accum.shape
        out = np.empty((H, W, 4), np.float32) if fmt == 0 else np.empty((H, W), np.uint32)
        lib().orc_tonemap(_p(np.ascontiguousarray(accum, np.float32)), W, H, accum_id, fmt, _p(out))
        return out

    def env_cdfs(self):
        H, W, _ = self.env.shape
        cy = np.empty(H, np.float32)
        cx = np.empty(H * W, np.float32)
        lib().orc_env_cdfs(_p(self.env), _p(np.array([W, H], np.int32)),
                           _p(np.array(list(self.s.env.addr), np.int32)), _p(cy), _p(cx))
        return cy, cx

    # -- emission-absorption --
    @staticmethod
    def _views(views):
        arr = (OrcEAView * len(views))()
        for a, v in zip(arr, views):
            a.pos[:] = list(v["pos"])
            a.dir[:] = list(v["dir"])
            a.up[:] = list(v["up"])
            a.fovy = v["fovy"]
            a.width, a.height = v["width"], v["height"]
        return arr

    def ea_render(self, views, step: float, use_double=False, nthreads=0) -> np.ndarray:
        if use_double and self.u8:
            raise ValueError("the U8 storage form is sampled in float only")
        npx = sum(v["width"] * v["height"] for v in views)
        out = np.empty((npx, 4), np.float32)
        lib().orc_ea_render(C.byref(self.rec), self._views(views), len(views), step, 1 if use_double else 0,
                            nthreads, _p(out))
        return out

    def ea_backward(self, views, step: float, d_images: np.ndarray, nthreads=0):
        if self.u8:
            raise ValueError("the adjoint is defined on the FP32 linear grid only")
        gv = np.zeros(self.scalars.size, np.float64)
        gt = np.zeros(self.tf.size, np.float64)
        lib().orc_ea_backward(C.byref(self.rec), self._views(views), len(views), step,
                              _p(np.ascontiguousarray(d_images, np.float32)), nthreads, _p(gv), _p(gt))
        return gv.reshape(self.scalars.shape), gt.reshape(self.tf.shape)


def lambertian(color, Ng, wo, wi, a: int, b: int) -> np.ndarray:
    """The AnariMatte Lambertian (orc_lambertian): eval value[3], eval pdf,
    pdf(wi), scatter dir[3], scatter pdf, f_r[3]."""
    out = np.zeros(12, np.float32)
    f4 = lambda v: _p(np.ascontiguousarray(v, np.float32))
    lib().orc_lambertian(f4(color), f4(Ng), f4(wo), f4(wi), a, b, _p(out))
    return out


def bounce(world: OrcShadeWorld, multi: bool, depth: int, path: OrcShadePath):
    """One shading step (orc_bounce) of the default or the multi-scatter
    build: (path afterwards, shadow ray, fragment); the inputs are copied."""
    io = OrcShadePath.from_buffer_copy(path)
    sh = OrcShadePath()
    frag = np.zeros(3, np.float32)
    lib().orc_bounce(C.byref(world), 1 if multi else 0, depth, C.byref(io), C.byref(sh), _p(frag))
    return io, sh, frag


def camera_commit(pos, direction, up, fovy) -> np.ndarray:
    """PerspectiveCamera::commit (orc_camera_commit): dir_00, dir_du, dir_dv,
    lens_00 as a (4, 3) array."""
    out = np.zeros(12, np.float32)
    f3 = lambda v: _p(np.ascontiguousarray(v, np.float32))
    lib().orc_camera_commit(f3(pos), f3(direction), f3(up), fovy, _p(out))
    return out.reshape(4, 3)


def generate(pos, direction, up, fovy, W, H, accum_id, bg):
    """_generateRays (orc_generate): (H, W, 11) float32 rays -- org, dir,
    tMax, missColor -- (H, W) seed states, and the count of pixels with a
    path state other than (throughput 1, misWeight 0)."""
    out = np.zeros((H, W, 11), np.float32)
    seeds = np.zeros((H, W), np.uint64)
    f = lambda v: _p(np.ascontiguousarray(v, np.float32))
    bad = lib().orc_generate(f(pos), f(direction), f(up), fovy, W, H, accum_id, f(bg), _p(out), _p(seeds))
    return out, seeds, bad


def env_cdfs(texels: np.ndarray, addr) -> tuple:
    """The env map's importance tables (orc_env_cdfs): cdf_y (H), cdf_x (H*W)."""
    texels = np.ascontiguousarray(texels, np.float32)
    H, W, _ = texels.shape
    cy, cx = np.empty(H, np.float32), np.empty(H * W, np.float32)
    lib().orc_env_cdfs(_p(texels), _p(np.array([W, H], np.int32)), _p(np.asarray(addr, np.int32)), _p(cy), _p(cx))
    return cy, cx


def rng_sequence(a: int, b: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float32)
    lib().orc_rng_sequence(a, b, n, _p(out))
    return out


def fast_log(f: float) -> float:
    return lib().orc_fast_log(f)


def float_to_half(f: float) -> int:
    return lib().orc_float_to_half(f)
