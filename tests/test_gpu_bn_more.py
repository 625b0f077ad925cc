"""The rest of barney.h's entry points through a live context: data arrays
refilled in place (bnDataSet), instance transforms updated and instance
attributes set on a built model, and the image-texture and sampler objects
this volume path makes but does not render with."""
import ctypes as C

import numpy as np
import pytest

from barney_gb300 import bn, scenes

pytestmark = pytest.mark.gpu


def _identity(n):
    xf = (C.c_float * (12 * n))()
    for k in range(n):
        xf[12 * k + 0] = xf[12 * k + 4] = xf[12 * k + 8] = 1.0
    return xf


def test_instance_updates_attributes_and_inert_objects(cuda):
    s = scenes.small_scene(dims=24, spp=1, width=32, height=24)
    vol = np.ascontiguousarray(s.scalars)
    with bn.BarneySession() as ses:
        assert ses.build_scene(s, vol.ctypes.data) == ""
        L, h = ses.L, ses.handles
        ses.render()
        before = ses.read().copy()
        # identity transforms for the one instance: the same frame
        L.bnUpdateInstanceTransforms(h["model"], 0, _identity(1), 1)
        L.bnAccumReset(h["fb"])
        ses.render()
        assert bn.last_error() == ""
        assert np.array_equal(ses.read(), before)
        # a count other than the instances'
        L.bnUpdateInstanceTransforms(h["model"], 0, _identity(2), 2)
        assert "count differs" in bn.last_error()
        # a translated instance is refused at render time
        xf = _identity(1)
        xf[9] = 0.5
        L.bnUpdateInstanceTransforms(h["model"], 0, xf, 1)
        ses.render()
        assert "identity" in bn.last_error()
        L.bnUpdateInstanceTransforms(h["model"], 0, _identity(1), 1)
        # instance attributes are kept, rendering is unchanged
        ids = np.array([h["grp"]], np.uint64)
        d = L.bnDataCreate(ses.ctx, 0, bn.BN_OBJECT, 1, C.c_void_p(ids.ctypes.data))
        L.bnSetInstanceAttributes(h["model"], 0, b"attribute0", d)
        L.bnAccumReset(h["fb"])
        ses.render()
        assert np.array_equal(ses.read(), before)
        # inert objects: made, released
        td = L.bnTextureData2DCreate(ses.ctx, 0, bn.BN_FLOAT4, 2, 2, None)
        t3 = L.bnTexture3DCreate(ses.ctx, 0, bn.BN_FLOAT32, 2, 2, 2, None, 1, 1)
        smp = L.bnSamplerCreate(ses.ctx, 0, b"texture2D")
        assert td and t3 and smp
        L.bnSet4x4fv(smp, b"inTransform", None)
        for o in (td, t3, smp, d):
            L.bnRelease(o)


def test_data_set_refills_a_byte_array(cuda):
    """bnDataSet on a BN_UINT8 array (as a NanoVDB field's "data" holds):
    the field committed afterwards reads the new bytes -- a valid grid
    commits, the same array refilled with bytes that are no grid is
    refused."""
    a = scenes.nanovdb_grid(np.ones((10, 10, 10), np.float32), (0, 0, 0), 0.1, (-0.5, -0.5, -0.5))
    with bn.BarneySession() as ses:
        L = ses.L
        ga = np.frombuffer(a, np.uint8).copy()
        d = L.bnDataCreate(ses.ctx, 0, bn.BN_UINT8, ga.size, C.c_void_p(ga.ctypes.data))
        sf = L.bnScalarFieldCreate(ses.ctx, 0, b"NanoVDB")
        L.bnSetData(sf, b"data", d)
        L.bnCommit(sf)
        assert bn.last_error() == ""
        junk = np.zeros(4096, np.uint8)
        L.bnDataSet(d, junk.size, C.c_void_p(junk.ctypes.data))
        L.bnSetData(sf, b"data", d)
        L.bnCommit(sf)
        assert "NanoVDB" in bn.last_error()
        for o in (sf, d):
            L.bnRelease(o)
