"""The C-ABI from plain C programs (tests/c/*.c): both headers compile as
C99 with -pedantic -Werror and as C++, the programs link against the
library, host-only entry points give the expected answers, and (GPU) a frame
rendered through bn* from C equals the same frame rendered through the
Python binding, bit for bit."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from barney_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent
LIBDIR = ROOT / "barney_gb300" / "_lib"


def _compile(src: str, out: Path, lang: str = "c"):
    N.lib()  # the library must exist
    cmd = (["gcc", "-std=c99", "-pedantic"] if lang == "c" else ["g++", "-std=c++17", "-x", "c++"])
    cmd += ["-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(ROOT / "tests" / "c" / src),
            "-L", str(LIBDIR), "-lbarney_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_host_entry_points_from_c(tmp_path, lang):
    exe = tmp_path / "abi_check"
    _compile("abi_check.c", exe, lang)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.splitlines() == [
        "mc_dims 13 8 4",
        f"store_bytes {7 * 8 * 8 * 512 * 8} {13 * 8 * 4 * 8}",
        "tiles 4 32,0 0,32 96,32 64,64",
        "tile_bytes 6144",
        'error "gbv_mc_dims: bad argument"',
        "version 1",
    ]


@pytest.mark.gpu
def test_bn_frame_from_c_equals_python_binding(cuda, tmp_path):
    from barney_gb300 import bn, scenes
    exe = tmp_path / "bn_frame"
    _compile("bn_frame.c", exe)
    out = tmp_path / "frame.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    got = np.fromfile(out, np.float32).reshape(48, 64, 4)
    n = 33
    # x-fastest texels: index i + n (j + n k); numpy arrays are (z, y, x)
    kk, jj, ii = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    vol = (((ii * 7 + jj * 13 + kk * 29) % 97).astype(np.float32) / np.float32(96)).astype(np.float32)
    q = np.arange(16, dtype=np.float32) / np.float32(15)
    tf = np.stack([q, np.full(16, 0.5, np.float32), np.float32(1) - q, q * np.float32(0.8)], 1).astype(np.float32)
    s = scenes.Scene(scalars=np.ascontiguousarray(vol), tf=tf, domain=(0.0, 1.0), base_density=10.0, cells_per_mc=8,
                     cam_pos=(0.5, 0.625, 2.25), cam_dir=(-0.5, -0.625, -2.25), cam_up=(0.0, 1.0, 0.0), fovy=40.0,
                     dir_lights=[((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), 2.0)], ambient=0.25,
                     bg_color=(0.0, 0.0, 0.0, 1.0), width=64, height=48, spp=4)
    with bn.BarneySession() as ses:
        assert ses.build_scene(s, s.scalars.ctypes.data) == ""
        ses.render()
        ref = ses.read()
    assert np.abs(ref[..., :3]).max() > 0
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
