"""The native library without a GPU: it loads, exports every entry point its
headers declare, validates arguments before touching the device, and the
host-side generator is deterministic."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import bn, scenes

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"(?m)^inline .*$", "", text)  # header-only C++ overloads (bnSet)
        for m in re.finditer(r"\b((?:gbv|bn)[A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name.startswith("gbv_") or re.match(r"bn[A-Z]", name):
                names.add(name)
    return names


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = declared_functions()
    assert len(names) >= 50
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    assert set(bn.BN_SYMBOLS) <= names


def test_mc_dims():
    out = (C.c_int * 3)()
    assert N.lib().gbv_mc_dims(N.ivec(64, 64, 64), 8, out) == N.GBV_OK
    assert tuple(out) == (8, 8, 8)
    assert N.lib().gbv_mc_dims(N.ivec(512, 512, 512), 16, out) == N.GBV_OK
    assert tuple(out) == (32, 32, 32)
    assert N.lib().gbv_mc_dims(N.ivec(37, 20, 9), 8, out) == N.GBV_OK
    assert tuple(out) == (5, 3, 1)
    assert N.lib().gbv_mc_dims(N.ivec(1, 5, 5), 8, out) == N.GBV_OK
    assert out[0] == 0
    assert N.lib().gbv_mc_dims(N.ivec(8, 8, 8), 0, out) == 1


def test_brick_store_sizes():
    vb, sb = C.c_size_t(), C.c_size_t()
    L = N.lib()
    assert L.gbv_brick_store_bytes(N.ivec(512, 512, 512), N.GBV_VOXEL_F32, C.byref(vb), C.byref(sb)) == 0
    assert vb.value == 64 ** 3 * 512 * 8 * 4 and sb.value == 0
    assert L.gbv_brick_store_bytes(N.ivec(512, 512, 512), N.GBV_VOXEL_F16, C.byref(vb), C.byref(sb)) == 0
    assert vb.value == 64 ** 3 * 512 * 8 * 2
    assert L.gbv_brick_store_bytes(N.ivec(65, 9, 2), N.GBV_VOXEL_U8_SCALED, C.byref(vb), C.byref(sb)) == 0
    assert vb.value == 8 * 1 * 1 * 512 * 8 and sb.value == 8 * 8
    assert L.gbv_brick_store_bytes(N.ivec(8, 8, 8), 9, C.byref(vb), C.byref(sb)) == N.GBV_ERROR_UNSUPPORTED if hasattr(
        N, "GBV_ERROR_UNSUPPORTED") else 5


def test_arguments_checked_before_the_device():
    L = N.lib()
    rec = N.GbvScene()
    assert L.gbv_render(None, None, 4, 4, 0, 1, None, None) == 1
    assert L.gbv_render(C.byref(rec), C.c_void_p(16), 4, 4, 0, 1, None, None) == 1
    assert "lacks" in L.gbv_last_error().decode()
    assert L.gbv_build_mc_ranges(None, N.ivec(8, 8, 8), 8, None, None) == 1
    assert L.gbv_tonemap(C.c_void_p(16), 4, 4, 0, 0, C.c_void_p(16), None) == 1
    assert L.gbv_ea_render(C.byref(rec), None, 0, 0.1, None, None) == 1
    assert L.gbv_build_brick_store(C.c_void_p(16), N.ivec(1, 4, 4), 0, C.c_void_p(16), None, None) == 1


def test_generator_deterministic_and_in_range():
    a = scenes.blob_volume((33, 17, 20), 8, seed=7, noise=0.05, fbm_octaves=2, fbm_amplitude=0.1)
    b = scenes.blob_volume((33, 17, 20), 8, seed=7, noise=0.05, fbm_octaves=2, fbm_amplitude=0.1, nthreads=1)
    c = scenes.blob_volume((33, 17, 20), 8, seed=8, noise=0.05, fbm_octaves=2, fbm_amplitude=0.1)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    assert a.min() >= 0.0 and a.max() <= 1.0 and a.std() > 0.01
    with pytest.raises(ValueError):
        scenes.blob_volume((1, 4, 4), 1, seed=0)


def test_bn_context_rejects_cpu_backend_and_multi_gpu():
    L = bn.lib()
    ids = (C.c_int * 1)(-1)
    assert not L.bnContextCreate(None, 1, ids, 1)
    assert "CPU backend" in bn.last_error()
    ids2 = (C.c_int * 2)(0, 1)
    assert not L.bnContextCreate(None, 1, ids2, 2)
    slots = (C.c_int * 2)(0, 1)
    assert not L.bnContextCreate(slots, 2, None, -1)


def test_env_sky_map():
    e = scenes.env_sky(64, 32)
    assert e.texels.shape == (32, 64, 4)
    assert e.texels[..., :3].max() == 50.0  # the sun disk
    assert np.all(e.texels[..., 3] == 1.0)


def test_brick_store_bytes_for_shapes():
    L = N.lib()
    vb, sb = C.c_size_t(), C.c_size_t()
    # 99 x 59 x 32 cells in 16 x 8 x 4-cell bricks: 7 x 8 x 8 bricks of 512 cells
    assert L.gbv_brick_store_bytes_shaped(N.ivec(100, 60, 33), N.GBV_VOXEL_F32, N.ivec(4, 3, 2), C.byref(vb),
                                          C.byref(sb)) == N.GBV_OK
    assert vb.value == 7 * 8 * 8 * 512 * 32 and sb.value == 0
    # U8 keeps one (scale, offset) per 8^3 cells whatever the brick shape
    assert L.gbv_brick_store_bytes_shaped(N.ivec(100, 60, 33), N.GBV_VOXEL_U8_SCALED, N.ivec(4, 3, 2), C.byref(vb),
                                          C.byref(sb)) == N.GBV_OK
    assert vb.value == 7 * 8 * 8 * 512 * 8 and sb.value == 13 * 8 * 4 * 8
    # zeros and a null shape mean 8^3 bricks, as the unshaped call
    ref = C.c_size_t()
    assert L.gbv_brick_store_bytes(N.ivec(100, 60, 33), N.GBV_VOXEL_F16, C.byref(ref), None) == N.GBV_OK
    assert L.gbv_brick_store_bytes_shaped(N.ivec(100, 60, 33), N.GBV_VOXEL_F16, N.ivec(0, 0, 0), C.byref(vb),
                                          None) == N.GBV_OK
    assert vb.value == ref.value == 13 * 8 * 4 * 512 * 16
    assert L.gbv_brick_store_bytes_shaped(N.ivec(100, 60, 33), N.GBV_VOXEL_F16, None, C.byref(vb), None) == N.GBV_OK
    assert vb.value == ref.value


@pytest.mark.parametrize("shape", [(7, 3, 3), (-1, 3, 3), (6, 6, 6), (3, 3, 10)])
def test_brick_shape_out_of_range_is_rejected(shape):
    vb = C.c_size_t()
    st = N.lib().gbv_brick_store_bytes_shaped(N.ivec(64, 64, 64), N.GBV_VOXEL_F32, N.ivec(*shape), C.byref(vb), None)
    assert st == N.GBV_ERROR_INVALID_ARGUMENT
    assert "brick_log2" in N.lib().gbv_last_error().decode()


def _angle_sweep():
    # a dense sweep of [-pi/4, 2 pi + pi/4] plus every float within 2000 ulp
    # of each multiple of pi/2 in it (where sine or cosine crosses zero)
    x = np.linspace(-np.pi / 4, 2 * np.pi + np.pi / 4, 2_000_001, dtype=np.float64).astype(np.float32)
    near = []
    for k in range(5):
        c = np.float32(k * np.pi / 2)
        i = c.view(np.int32) if c != 0 else np.int32(0)
        ints = np.arange(max(int(i) - 2000, 0), int(i) + 2000, dtype=np.int32)
        near.append(ints.view(np.float32))
        if k == 0:
            near.append(-ints[1:].view(np.float32))
    return np.concatenate([x] + near)


def test_bounded_sincos_within_two_ulp():
    x = _angle_sweep()
    s = np.empty_like(x)
    c = np.empty_like(x)
    assert N.lib().gbv_selftest_sincos(x.ctypes.data, x.size, s.ctypes.data, c.ctypes.data, 0, None) == N.GBV_OK
    for got, ref in ((s, np.sin(x.astype(np.float64))), (c, np.cos(x.astype(np.float64)))):
        r32 = np.abs(ref).astype(np.float32)
        ulp = np.spacing(r32).astype(np.float64)
        ulp[r32 == 0] = np.float64(np.finfo(np.float32).smallest_subnormal)
        err = np.abs(got.astype(np.float64) - ref) / ulp
        assert err.max() <= 2.0, (err.max(), x[err.argmax()])


def test_bounded_acos_atan2_accuracy():
    """The renderer's arc cosine within 1.5 ulp and two-argument arc tangent
    within 2.5 ulp of float64, over [-1, 1] and directions of the sphere;
    atan2 keeps the sign conventions of signed zeros."""
    rng = np.random.default_rng(5)
    z = np.concatenate([rng.uniform(-1, 1, 400_000), np.linspace(-1, 1, 200_001)]).astype(np.float32)
    v = rng.normal(size=(z.size, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    y, x = v[:, 1].astype(np.float32), v[:, 0].astype(np.float32)
    ac, at = np.empty_like(z), np.empty_like(z)
    assert N.lib().gbv_selftest_angles(y.ctypes.data, z.ctypes.data, z.size, ac.ctypes.data, at.ctypes.data, 0,
                                       None) == N.GBV_OK
    ref = np.arccos(z.astype(np.float64))
    err = np.abs(ac.astype(np.float64) - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    assert err.max() <= 1.5, (err.max(), z[err.argmax()])
    assert N.lib().gbv_selftest_angles(y.ctypes.data, x.ctypes.data, x.size, ac.ctypes.data, at.ctypes.data, 0,
                                       None) == N.GBV_OK
    ref = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    r32 = np.abs(ref).astype(np.float32)
    ulp = np.spacing(r32).astype(np.float64)
    err = np.abs(at.astype(np.float64) - ref) / ulp
    assert err.max() <= 2.5, (err.max(), y[err.argmax()], x[err.argmax()])
    yy = np.array([0.0, -0.0, 0.0, -0.0], np.float32)
    xx = np.array([0.0, 0.0, -0.0, -0.0], np.float32)
    a2, t2 = np.empty_like(xx), np.empty_like(xx)
    assert N.lib().gbv_selftest_angles(yy.ctypes.data, xx.ctypes.data, 4, a2.ctypes.data, t2.ctypes.data, 0,
                                       None) == N.GBV_OK
    np.testing.assert_array_equal(t2, np.arctan2(yy, xx))
    np.testing.assert_array_equal(np.signbit(t2), np.signbit(np.arctan2(yy, xx)))


def test_ea_step_cap_rejected_before_the_device():
    """A step so small that one ray could take more than 2^24 steps is an
    error returned before any launch (the march's loop is bounded)."""
    L = N.lib()
    rec = N.GbvScene()
    rec.d_voxels = 16
    rec.d_tf = 16
    rec.tf_n = 4
    rec.format, rec.layout = N.GBV_VOXEL_F32, N.GBV_LAYOUT_LINEAR
    rec.dims[:] = (8, 8, 8)
    rec.origin[:] = (-.5, -.5, -.5)
    rec.spacing[:] = (1 / 7, 1 / 7, 1 / 7)
    rec.domain[:] = (0.0, 1.0)
    view = N.GbvEAView()
    view.width = view.height = 4
    img = C.c_void_p(16)
    for step in (1e-30, 1e-8, float("nan"), 0.0, -1.0):
        assert L.gbv_ea_render(C.byref(rec), C.byref(view), 1, step, img, None) == N.GBV_ERROR_INVALID_ARGUMENT
        assert L.gbv_ea_render_f64(C.byref(rec), C.byref(view), 1, step, img, None) == N.GBV_ERROR_INVALID_ARGUMENT
        assert L.gbv_ea_backward(C.byref(rec), C.byref(view), 1, step, img, img, img, img,
                                 None) == N.GBV_ERROR_INVALID_ARGUMENT
    L.gbv_ea_render(C.byref(rec), C.byref(view), 1, 1e-30, img, None)
    assert "2^24" in L.gbv_last_error().decode()


def test_tile_counts_of_very_wide_frames():
    """Tile counts are formed in 64-bit arithmetic: a frame 2^31-1 pixels wide
    has ceil((2^31-1)/32) = 2^26 tiles of 32x32 per row (no int overflow)."""
    L = N.lib()
    n = C.c_int()
    assert L.gbv_tile_partition(2 ** 31 - 1, 1, 0, 1, C.byref(n), None) == N.GBV_OK
    assert n.value == 2 ** 26
    assert L.gbv_tile_partition(2 ** 31 - 1, 1, 3, 4, C.byref(n), None) == N.GBV_OK
    assert n.value == 2 ** 24
    assert L.gbv_tile_partition(2 ** 31 - 1, 33, 0, 2 ** 26 + 1, C.byref(n), None) == N.GBV_OK
    assert n.value == 2
    buf = (C.c_int * (2 * n.value))()
    assert L.gbv_tile_partition(2 ** 31 - 1, 33, 0, 2 ** 26 + 1, C.byref(n), buf) == N.GBV_OK
    # rank 0 of 2^26+1 owns tiles 0 and 2^26+1: (0, 0) and the second tile of
    # the second row of a 2^26-tile-wide grid
    assert list(buf) == [0, 0, 32, 32]


def test_render_config_checked_before_the_device():
    """gbv_render_ex rejects out-of-range launch settings before any CUDA
    call; a zero config is the default launch (spp = 0: nothing to do)."""
    L = N.lib()
    rec = N.GbvScene()
    rec.d_voxels = rec.d_majorants = rec.d_tf = 16
    rec.tf_n, rec.cells_per_mc = 4, 8
    rec.dims[:] = (8, 8, 8)
    acc = C.c_void_p(16)
    bad = [dict(blocks_per_sm=3), dict(blocks_per_sm=7), dict(threshold_pct=101), dict(threshold_pct=-1),
           dict(skip_cells=1025), dict(stage=4), dict(profile=2), dict(mode=2)]
    for kw in bad:
        cfg = N.render_config(**kw)
        assert L.gbv_render_ex(C.byref(rec), acc, 4, 4, 0, 0, None, C.byref(cfg), None) == 1, kw
        assert "launch config" in L.gbv_last_error().decode()
    cfg = N.render_config()
    cfg.reserved[1] = 1
    assert L.gbv_render_ex(C.byref(rec), acc, 4, 4, 0, 0, None, C.byref(cfg), None) == 1
    assert L.gbv_render_ex(C.byref(rec), acc, 4, 4, 0, 0, None, C.byref(N.render_config()), None) == 0
    assert L.gbv_render_ex(C.byref(rec), acc, 4, 4, 0, 0, None, None, None) == 0
    good = N.render_config(blocks_per_sm=6, threshold_pct=100, skip_cells=1024, stage=N.GBV_STAGE_ALL, profile=1)
    assert L.gbv_render_ex(C.byref(rec), acc, 4, 4, 0, 0, None, C.byref(good), None) == 0


def test_nanovdb_parse():
    """gbv_nanovdb_parse on the pinned grid (tests/golden/nanovdb_pin.npz):
    header fields, index and world bboxes, macrocell grid; and the checks
    that keep malformed buffers off the device."""
    from barney_gb300 import nanovdb
    z = np.load(ROOT / "tests" / "golden" / "nanovdb_pin.npz")
    grid = z["grid"].tobytes()
    info = nanovdb.parse(grid)
    assert info.bytes == len(grid)
    assert list(info.mc_dims) == z["mc_dims"].tolist()
    assert np.array_equal(np.array(list(info.world_lo) + list(info.world_hi), np.float32), z["world"])
    assert all(info.index_hi[i] >= info.index_lo[i] for i in range(3))
    assert info.background == 0.0 and info.root_tiles >= 1
    L = nanovdb.lib()
    out = nanovdb.GbvNanovdbInfo()

    def parse(b):
        a = np.frombuffer(b, np.uint8).copy()
        return L.gbv_nanovdb_parse(a.ctypes.data_as(C.c_void_p), a.size, C.byref(out))

    assert parse(grid) == N.GBV_OK
    assert parse(b"X" + grid[1:]) == N.GBV_ERROR_INVALID_ARGUMENT        # magic number
    assert parse(grid[:1000]) == N.GBV_ERROR_INVALID_ARGUMENT            # truncated
    bad = bytearray(grid)
    bad[636:640] = (2).to_bytes(4, "little")                             # value type Double
    assert parse(bytes(bad)) == N.GBV_ERROR_UNSUPPORTED
    # a root tile whose child offset points past the end of the buffer
    root = 672 + int.from_bytes(grid[672 + 24:672 + 32], "little", signed=True)
    bad = bytearray(grid)
    bad[root + 64 + 8:root + 64 + 16] = (len(grid)).to_bytes(8, "little", signed=True)
    assert parse(bytes(bad)) == N.GBV_ERROR_INVALID_ARGUMENT


# every function barney/include/barney.h declares (its C++-only inline bnSet
# overloads aside, which this library's header defines the same way)
BARNEY_H_FUNCTIONS = [
    "bnAccumReset", "bnAddReference", "bnBuild", "bnCameraCreate", "bnCommit", "bnContextCreate",
    "bnContextDestroy", "bnDataCreate", "bnDataSet", "bnFrameBufferCreate", "bnFrameBufferGetSize",
    "bnFrameBufferRead", "bnFrameBufferResize", "bnGeometryCreate", "bnGroupBuild", "bnGroupCreate",
    "bnLightCreate", "bnMaterialCreate", "bnModelCreate", "bnRelease", "bnRender", "bnRendererCreate",
    "bnSamplerCreate", "bnScalarFieldCreate", "bnSet1f", "bnSet1i", "bnSet2f", "bnSet2i", "bnSet3f", "bnSet3i",
    "bnSet4f", "bnSet4i", "bnSet4x3fv", "bnSet4x4fv", "bnSetData", "bnSetInstanceAttributes", "bnSetInstances",
    "bnSetLight", "bnSetObject", "bnSetString", "bnTexture2DCreate", "bnTexture3DCreate", "bnTextureData2DCreate",
    "bnTextureData3DCreate", "bnUpdateInstanceTransforms", "bnVolumeCreate", "bnVolumeSetXF"]


def test_every_barney_h_function_is_declared_and_exported():
    """An application or ANARI device written against barney.h links
    against this library: every one of its functions is declared in
    include/barney_gb300.h and exported (those outside the volume path make
    inert objects or record a message)."""
    L = N.lib()
    names = declared_functions()
    assert not [n for n in BARNEY_H_FUNCTIONS if n not in names]
    assert not [n for n in BARNEY_H_FUNCTIONS if not hasattr(L, n)]
