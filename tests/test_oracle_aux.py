"""The oracle's auxiliary frame channels (host code, no GPU): depth and hit
IDs of each pixel's primary ray with the reference's rules -- pass 0 writes
the depth and the IDs, later passes keep the smaller depth and the first
pass's IDs; a miss has depth 1e30 (the generated tMax) and IDs -1."""
import numpy as np

from barney_gb300 import scenes
import oracle


def _aux(W, H):
    return {"depth": np.zeros((H, W), np.float32), "prim_id": np.zeros((H, W), np.int32),
            "inst_id": np.zeros((H, W), np.int32), "obj_id": np.zeros((H, W), np.int32)}


def test_depth_is_the_minimum_over_passes_and_ids_come_from_pass_0():
    s = scenes.small_scene(dims=24, spp=1, width=20, height=16)
    s.volume_user_id = 4
    o = oracle.Oracle(s)
    first, every = _aux(20, 16), []
    o.render(spp=1, accum_id_start=0, aux=first)
    for k in range(1, 5):
        a = _aux(20, 16)
        a["depth"][:] = np.float32(1e30)
        o.render(spp=1, accum_id_start=k, aux=a)
        every.append(a["depth"].copy())
    acc = _aux(20, 16)
    o.render(spp=5, accum_id_start=0, aux=acc)
    np.testing.assert_array_equal(acc["depth"], np.minimum(first["depth"], np.min(every, axis=0)))
    for k in ("prim_id", "inst_id", "obj_id"):
        np.testing.assert_array_equal(acc[k], first[k])
    miss = first["prim_id"] == -1
    assert miss.any() and (~miss).any()
    assert np.all(first["depth"][miss] == np.float32(1e30))
    assert np.all(first["obj_id"][~miss] == 4) and np.all(first["inst_id"][~miss] == 0)
