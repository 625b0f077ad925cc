"""Python binding of the barney-compatible bn* C API (include/barney_gb300.h).

Mirrors how an application drives the reference renderer through
barney/include/barney.h: create a context, a structured scalar field from a
3D texture, a volume with a transfer function, lights, a group, a model, a
camera, a renderer and a frame buffer, then bnRender and bnFrameBufferRead.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _native as N
from .scenes import Scene

BN_OBJECT = 2
BN_FLOAT32 = 180
BN_FLOAT4 = 183
BN_UINT8 = 110
BN_UINT16 = 130
BN_UFIXED8 = 300
BN_UFIXED8_RGBA = 301
BN_UFIXED8_RGBA_SRGB = 302
BN_UFIXED16 = 303
BN_FB_COLOR = 1
BN_FB_DEPTH, BN_FB_PRIMID, BN_FB_INSTID, BN_FB_OBJID = 2, 4, 8, 16
BN_INT32, BN_FLOAT = 140, 180
BN_TEXTURE_NEAREST, BN_TEXTURE_LINEAR = 0, 1

BN_SYMBOLS = [
    "bnContextCreate", "bnContextDestroy", "bnRelease", "bnAddReference", "bnCameraCreate",
    "bnFrameBufferCreate", "bnModelCreate", "bnRendererCreate", "bnDataCreate", "bnTextureData3DCreate",
    "bnTexture2DCreate", "bnLightCreate", "bnGroupCreate", "bnGroupBuild", "bnScalarFieldCreate",
    "bnVolumeCreate", "bnVolumeSetXF", "bnCommit", "bnSetString", "bnSetData", "bnSetObject", "bnSetLight",
    "bnSet1i", "bnSet2i", "bnSet3i", "bnSet4i", "bnSet1f", "bnSet2f", "bnSet3f", "bnSet4f", "bnSet4x3fv",
    "bnSetInstances", "bnBuild", "bnAccumReset", "bnFrameBufferResize", "bnFrameBufferRead",
    "bnFrameBufferGetSize", "bnRender", "bnGetLastError", "bnFrameBufferGetStats", "bnGeometryCreate",
    "bnMaterialCreate", "bnDataSet", "bnTextureData2DCreate", "bnTexture3DCreate", "bnSamplerCreate",
    "bnSet4x4fv", "bnUpdateInstanceTransforms", "bnSetInstanceAttributes",
]


class BnFloat2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


_ready = False


def lib() -> C.CDLL:
    global _ready
    L = N.lib()
    if not _ready:
        vp, i, f, cp = C.c_void_p, C.c_int, C.c_float, C.c_char_p
        sig = {
            "bnContextCreate": (vp, [vp, i, vp, i]),
            "bnContextDestroy": (None, [vp]),
            "bnRelease": (None, [vp]),
            "bnAddReference": (None, [vp]),
            "bnCameraCreate": (vp, [vp, cp]),
            "bnFrameBufferCreate": (vp, [vp, i]),
            "bnModelCreate": (vp, [vp]),
            "bnRendererCreate": (vp, [vp, cp]),
            "bnDataCreate": (vp, [vp, i, i, C.c_size_t, vp]),
            "bnTextureData3DCreate": (vp, [vp, i, i, i, i, i, vp]),
            "bnTexture2DCreate": (vp, [vp, i, i, C.c_uint32, C.c_uint32, vp, i, i, i, i]),
            "bnLightCreate": (vp, [vp, i, cp]),
            "bnGroupCreate": (vp, [vp, i, vp, i, vp, i]),
            "bnGroupBuild": (None, [vp]),
            "bnScalarFieldCreate": (vp, [vp, i, cp]),
            "bnVolumeCreate": (vp, [vp, i, vp]),
            "bnVolumeSetXF": (None, [vp, BnFloat2, vp, i, f]),
            "bnCommit": (None, [vp]),
            "bnSetData": (None, [vp, cp, vp]),
            "bnSetObject": (None, [vp, cp, vp]),
            "bnSet1i": (None, [vp, cp, i]),
            "bnSet3i": (None, [vp, cp, i, i, i]),
            "bnSet1f": (None, [vp, cp, f]),
            "bnSet3f": (None, [vp, cp, f, f, f]),
            "bnSet4f": (None, [vp, cp, f, f, f, f]),
            "bnSetInstances": (None, [vp, i, vp, vp, i]),
            "bnBuild": (None, [vp, i]),
            "bnAccumReset": (None, [vp]),
            "bnFrameBufferResize": (None, [vp, i, i, i, C.c_uint32]),
            "bnFrameBufferRead": (None, [vp, i, vp, i]),
            "bnFrameBufferGetSize": (None, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
            "bnRender": (None, [vp, vp, vp, vp]),
            "bnGetLastError": (cp, []),
            "bnFrameBufferGetStats": (None, [vp, C.POINTER(C.c_ulonglong)]),
            "bnGeometryCreate": (vp, [vp, i, cp]),
            "bnMaterialCreate": (vp, [vp, i, cp]),
            "bnSetString": (None, [vp, cp, cp]),
            "bnDataSet": (None, [vp, C.c_size_t, vp]),
            "bnTextureData2DCreate": (vp, [vp, i, i, i, i, vp]),
            "bnTexture3DCreate": (vp, [vp, i, i, C.c_uint32, C.c_uint32, C.c_uint32, vp, i, i]),
            "bnSamplerCreate": (vp, [vp, i, cp]),
            "bnSet4x4fv": (None, [vp, cp, vp]),
            "bnUpdateInstanceTransforms": (None, [vp, i, vp, i]),
            "bnSetInstanceAttributes": (None, [vp, i, cp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _ready = True
    return L


def last_error() -> str:
    return (lib().bnGetLastError() or b"").decode(errors="replace")


def _ok(h, what):
    if not h:
        raise N.GbvError(f"{what} failed: {last_error()}")
    return h


class BarneySession:
    """One context holding one structured-volume scene, driven through bn*.

    `scalars_host` may be any C-contiguous float32 host buffer pointer source
    (numpy array or pinned torch tensor); set_volume uploads it every call, as
    bnTextureData3DCreate copies texels at create time.
    """

    def __init__(self, gpu: int = 0):
        L = lib()
        ids = (C.c_int * 1)(gpu)
        self.ctx = _ok(L.bnContextCreate(None, 1, ids, 1), "bnContextCreate")
        self.L = L
        self.keep = []

    def close(self):
        if self.ctx:
            self.L.bnContextDestroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def build_scene(self, scene: Scene, scalars_ptr: int, voxel_format: int = N.GBV_VOXEL_F32,
                    layout: int = N.GBV_LAYOUT_BRICK_CORNERS, color_format: int = BN_FLOAT4, brick=None,
                    texel_format: int = BN_FLOAT32, frame_stats: bool = False, anari: Optional[str] = None,
                    nanovdb: Optional[bytes] = None, channels: int = BN_FB_COLOR):
        """anari: None (bn* calls as an app makes them), "vec4" or
        "vec3+opacity": the field and the transfer function made through the
        ANARI parameter translation (include/gbv_anari.h) from the
        structuredRegular data and a transferFunction1D whose colors are the
        scene TF's RGBA (or RGB with its alpha as the opacity array) and whose
        unitDistance is 1 / base density."""
        L, ctx, s = self.L, self.ctx, scene
        nx, ny, nz = s.dims
        origin, spacing = s.geometry()
        td = None
        if nanovdb is not None:
            # a "NanoVDB" field from a BN_UINT8 data array (anari/SpatialField.cpp:220-233)
            grid = np.frombuffer(bytes(nanovdb), np.uint8).copy()
            self.keep.append(grid)
            sf = _ok(L.bnScalarFieldCreate(ctx, 0, b"NanoVDB"), "bnScalarFieldCreate")
            bd = _ok(L.bnDataCreate(ctx, 0, BN_UINT8, grid.size, grid.ctypes.data_as(C.c_void_p)), "bnDataCreate")
            L.bnSetData(sf, b"data", bd)
            L.bnRelease(bd)
        elif anari is None:
            td = _ok(L.bnTextureData3DCreate(ctx, 0, texel_format, nx, ny, nz, C.c_void_p(scalars_ptr)),
                     "bnTextureData3DCreate")
            sf = _ok(L.bnScalarFieldCreate(ctx, 0, b"structured"), "bnScalarFieldCreate")
            L.bnSetObject(sf, b"textureData", td)
            L.bnSet3i(sf, b"dims", nx, ny, nz)
            L.bnSet3f(sf, b"gridOrigin", *origin)
            L.bnSet3f(sf, b"gridSpacing", *spacing)
        else:
            from . import anari as A
            A.lib()
            h = C.c_void_p(0)
            et = {BN_FLOAT32: A.GBV_ANARI_FLOAT32, BN_UFIXED8: A.GBV_ANARI_UFIXED8}[texel_format]
            N.check(L.gbv_anari_structured_regular(ctx, 0, et, C.c_void_p(scalars_ptr),
                                                   N.ivec(nx, ny, nz), (C.c_float * 3)(*origin),
                                                   (C.c_float * 3)(*spacing), C.byref(h)),
                    "gbv_anari_structured_regular")
            sf = h.value
        if nanovdb is None:
            L.bnSet1i(sf, b"cellsPerMacrocell", s.cells_per_mc)
            L.bnSet1i(sf, b"voxelFormat", voxel_format)
            L.bnSet1i(sf, b"voxelLayout", layout)
            if brick is not None:
                L.bnSet3i(sf, b"brickLog2", *brick)
        L.bnCommit(sf)
        geom = mat = None
        if s.iso is not None:
            # an iso_surface geometry with a matte material (IsoSurface, AnariMatte)
            mat = _ok(L.bnMaterialCreate(ctx, 0, b"matte"), "bnMaterialCreate")
            L.bnSet4f(mat, b"color", *[float(c) for c in s.iso.color])
            L.bnSet1f(mat, b"opacity", float(s.iso.opacity))
            L.bnCommit(mat)
            geom = _ok(L.bnGeometryCreate(ctx, 0, b"iso_surface"), "bnGeometryCreate")
            L.bnSetObject(geom, b"scalarField", sf)
            L.bnSet1f(geom, b"isoValue", float(s.iso.value))
            L.bnSet1i(geom, b"userID", int(s.iso.user_id))
            L.bnSetObject(geom, b"material", mat)
            L.bnCommit(geom)
        vol = _ok(L.bnVolumeCreate(ctx, 0, sf), "bnVolumeCreate")
        tf = np.ascontiguousarray(s.tf, np.float32)
        self.keep.append(tf)
        if anari is None:
            L.bnVolumeSetXF(vol, BnFloat2(*s.domain), tf.ctypes.data_as(C.c_void_p), tf.shape[0], s.base_density)
        else:
            from . import anari as A
            rng = np.asarray(s.domain, np.float32)
            if anari == "vec4":
                col, ch, op = tf, 4, None
            else:
                col, ch, op = np.ascontiguousarray(tf[:, :3]), 3, np.ascontiguousarray(tf[:, 3])
            self.keep += [col, op, rng]
            N.check(L.gbv_anari_transfer_function_1d(vol, A._p(col), ch, col.shape[0], A._p(op),
                                                     0 if op is None else op.shape[0], None, 1.0, A._p(rng),
                                                     float(np.float32(1.0) / np.float32(s.base_density)), 7),
                    "gbv_anari_transfer_function_1d")
        L.bnSet1f(vol, b"anisotropy", s.anisotropy)
        L.bnSet1f(vol, b"scatteringAlbedo", s.scattering_albedo)
        if anari is None:
            L.bnSet1i(vol, b"userID", int(getattr(s, "volume_user_id", 0)))
        L.bnCommit(vol)
        lights = []
        for d, c, rad in s.dir_lights:
            l = _ok(L.bnLightCreate(ctx, 0, b"directional"), "bnLightCreate")
            L.bnSet3f(l, b"direction", *d)
            L.bnSet3f(l, b"color", *c)
            L.bnSet1f(l, b"radiance", rad)
            L.bnCommit(l)
            lights.append(l)
        if s.env is not None:
            e = s.env
            H, W, _ = e.texels.shape
            tex = _ok(L.bnTexture2DCreate(ctx, 0, BN_FLOAT4, W, H, e.texels.ctypes.data_as(C.c_void_p),
                                          BN_TEXTURE_LINEAR, e.addr[0], e.addr[1], 0), "bnTexture2DCreate")
            l = _ok(L.bnLightCreate(ctx, 0, b"envmap"), "bnLightCreate")
            L.bnSetObject(l, b"texture", tex)
            L.bnSet3f(l, b"direction", *e.direction)
            L.bnSet3f(l, b"up", *e.up)
            L.bnSet1f(l, b"scale", e.scale)
            L.bnCommit(l)
            lights.append(l)
        # groups in instance order: the iso-surface shares the volume's group
        # when its instance index is the lower one (a group's user geometries
        # come before its volumes), else it has a group of its own after
        vols = (C.c_void_p * 1)(vol)
        geoms = (C.c_void_p * 1)(geom)
        grp2 = None
        if geom is None:
            grp = _ok(L.bnGroupCreate(ctx, 0, None, 0, vols, 1), "bnGroupCreate")
        elif s.no_volume:
            grp = _ok(L.bnGroupCreate(ctx, 0, geoms, 1, None, 0), "bnGroupCreate")
        elif (s.iso.instance, s.volume_instance) == (0, 1):
            grp = _ok(L.bnGroupCreate(ctx, 0, geoms, 1, vols, 1), "bnGroupCreate")
        elif (s.iso.instance, s.volume_instance) == (1, 0):
            grp = _ok(L.bnGroupCreate(ctx, 0, None, 0, vols, 1), "bnGroupCreate")
            grp2 = _ok(L.bnGroupCreate(ctx, 0, geoms, 1, None, 0), "bnGroupCreate")
        else:
            raise ValueError("iso-surface and volume instances must be (0, 1) or (1, 0)")
        if lights:
            arr = (C.c_void_p * len(lights))(*lights)
            data = _ok(L.bnDataCreate(ctx, 0, BN_OBJECT, len(lights), arr), "bnDataCreate")
            L.bnSetData(grp, b"lights", data)
        gl = [grp] if grp2 is None else [grp, grp2]
        for g in gl:
            L.bnCommit(g)
            L.bnGroupBuild(g)
        model = _ok(L.bnModelCreate(ctx), "bnModelCreate")
        groups = (C.c_void_p * len(gl))(*gl)
        L.bnSetInstances(model, 0, groups, None, len(gl))
        L.bnBuild(model, 0)
        cam = _ok(L.bnCameraCreate(ctx, b"perspective"), "bnCameraCreate")
        L.bnSet3f(cam, b"position", *s.cam_pos)
        L.bnSet3f(cam, b"direction", *s.cam_dir)
        L.bnSet3f(cam, b"up", *s.cam_up)
        L.bnSet1f(cam, b"fovy", s.fovy)
        L.bnCommit(cam)
        r = _ok(L.bnRendererCreate(ctx, b"default"), "bnRendererCreate")
        L.bnSet1i(r, b"pathsPerPixel", s.spp)
        if frame_stats:  # event counts for bnFrameBufferGetStats (a slower kernel)
            L.bnSet1i(r, b"frameStats", 1)
        L.bnSet1f(r, b"ambientRadiance", s.ambient)
        L.bnSet4f(r, b"bgColor", *s.bg_color)
        L.bnSet1i(r, b"multiScatter", s.multi_scatter)
        L.bnSet1i(r, b"volumeMultiScatter", s.volume_multi_scatter)
        L.bnSet1i(r, b"maxVolumeBounces", s.max_volume_bounces)
        L.bnCommit(r)
        fb = _ok(L.bnFrameBufferCreate(ctx, 0), "bnFrameBufferCreate")
        L.bnFrameBufferResize(fb, color_format, s.width, s.height, BN_FB_COLOR | channels)
        self.handles = dict(td=td, sf=sf, vol=vol, grp=grp, grp2=grp2, geom=geom, mat=mat, model=model, cam=cam,
                            renderer=r, fb=fb)
        self.handles = {k: v for k, v in self.handles.items() if v is not None}
        self.scene, self.color_format = s, color_format
        err = last_error()
        return err

    def render(self) -> None:
        h = self.handles
        self.L.bnRender(h["renderer"], h["model"], h["cam"], h["fb"])

    def read(self, out=None):
        s = self.scene
        if out is None:
            out = (np.empty((s.height, s.width, 4), np.float32) if self.color_format == BN_FLOAT4
                   else np.empty((s.height, s.width), np.uint32))
        ptr = out.ctypes.data if isinstance(out, np.ndarray) else out.data_ptr()
        self.L.bnFrameBufferRead(self.handles["fb"], BN_FB_COLOR, C.c_void_p(ptr), self.color_format)
        return out

    def read_channel(self, channel: int) -> np.ndarray:
        """An aux channel the frame buffer was resized with: BN_FB_DEPTH as
        float32, BN_FB_PRIMID/INSTID/OBJID as int32, (H, W)."""
        s = self.scene
        depth = channel == BN_FB_DEPTH
        out = np.empty((s.height, s.width), np.float32 if depth else np.int32)
        self.L.bnFrameBufferRead(self.handles["fb"], channel, C.c_void_p(out.ctypes.data),
                                 BN_FLOAT if depth else BN_INT32)
        return out

    def stats(self):
        st = (C.c_ulonglong * 4)()
        self.L.bnFrameBufferGetStats(self.handles["fb"], st)
        return list(st)

    def release_scene(self):
        for k in ("fb", "renderer", "cam", "model", "grp2", "grp", "geom", "mat", "vol", "sf", "td"):
            if k in self.handles:
                self.L.bnRelease(self.handles[k])
        self.handles = {}
