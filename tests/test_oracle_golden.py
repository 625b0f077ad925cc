"""The CPU oracle against the golden vectors of tests/golden/kernels.npz.

The vectors come from an independent pure-Python restatement of the
reference's scalar kernels (tests/golden/make_golden.py); every comparison is
bit-exact.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import oracle
from barney_gb300.scenes import Scene

G = np.load(Path(__file__).resolve().parent / "golden" / "kernels.npz")


def golden_scene():
    dom = G["tf_dom"]
    return Scene(scalars=G["vol"], tf=G["tf"], domain=(float(dom[0]), float(dom[1])), base_density=float(dom[2]),
                 cells_per_mc=int(G["mc_cpm"][0]), origin=tuple(G["origin"].tolist()),
                 spacing=tuple(G["spacing"].tolist()))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def test_rng_streams():
    for (a, b), seq in zip(G["rng_pairs"], G["rng_seq"]):
        np.testing.assert_array_equal(bits(oracle.rng_sequence(int(a), int(b), 16)), bits(seq))


def test_rng_derive():
    L = oracle.lib()
    h = ((0xCBF29CE484222325 * 0x100000001B3) & (2 ** 64 - 1)) * 0x100000001B3 & (2 ** 64 - 1)
    for s0, seq, s1 in zip(G["derive_seed"], G["derive_seq"], G["derive_new_seed"]):
        out = np.empty(8, np.float32)
        ns = C.c_uint64()
        L.orc_rng_from_seed(int(s0), h, 1, 8, out.ctypes.data_as(C.c_void_p), C.byref(ns))
        np.testing.assert_array_equal(bits(out), bits(seq))
        assert ns.value == int(s1)


def test_fast_log():
    got = np.array([oracle.fast_log(float(x)) for x in G["fastlog_x"]], np.float32)
    np.testing.assert_array_equal(bits(got), bits(G["fastlog_y"]))


def test_half_rounding_ties_away():
    got = np.array([oracle.float_to_half(float(x)) for x in G["half_x"]], np.uint16)
    np.testing.assert_array_equal(got, G["half_y"])
    # 1 + 2^-11 is an exact tie: rounds away (RNE would give 1.0)
    assert oracle.float_to_half(1 + 2 ** -11) == 0x3C01
    assert np.float16(1 + 2 ** -11).view(np.uint16) == 0x3C00


def test_trilinear_samples():
    o = oracle.Oracle(golden_scene())
    got = o.sample(G["sample_P"])
    np.testing.assert_array_equal(np.isnan(got), np.isnan(G["sample_v"]))
    m = ~np.isnan(got)
    np.testing.assert_array_equal(bits(got[m]), bits(G["sample_v"][m]))
    assert m.sum() > 50 and (~m).sum() > 10


def test_tf_map():
    o = oracle.Oracle(golden_scene())
    np.testing.assert_array_equal(bits(o.tf_map(G["map_s"])), bits(G["map_rgba"]))


def test_macrocell_ranges_and_majorants():
    o = oracle.Oracle(golden_scene())
    assert o.mc_dims() == tuple(G["mc_dims"].tolist())
    r = o.mc_ranges()
    np.testing.assert_array_equal(r, G["mc_ranges"])
    np.testing.assert_array_equal(bits(o.majorants_of(r)), bits(G["mc_majorants"]))


def test_traced_rays():
    o = oracle.Oracle(golden_scene())
    L = oracle.lib()
    for k in range(len(G["ray_hit"])):
        org = np.ascontiguousarray(G["ray_org"][k], np.float32)
        d = np.ascontiguousarray(G["ray_dir"][k], np.float32)
        seed = C.c_uint64(int(G["ray_seed"][k]))
        t = C.c_float(0)
        rgb = np.zeros(3, np.float32)
        hit = L.orc_trace_ray(C.byref(o.rec), org.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                              np.float32(1e30), C.byref(seed), C.byref(t), rgb.ctypes.data_as(C.c_void_p))
        assert hit == G["ray_hit"][k], k
        assert seed.value == int(G["ray_new_seed"][k]), k
        if hit:
            assert np.float32(t.value).view(np.uint32) == G["ray_t"][k].view(np.uint32), k
            np.testing.assert_array_equal(bits(rgb), bits(G["ray_rgb"][k]))
