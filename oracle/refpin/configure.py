"""TEST INFRASTRUCTURE ONLY: the configure step of the reference pin harness.

The reference's public header barney/include/barney.h and its
barney/common/barneyConfig.h.in are CMake templates (#cmakedefine01,
@VAR@).  This step does what the reference build's configure_file does for
an embree-only (CPU backend), single-process build with NanoVDB (its
headers are vendored in the reference, 3rdParty/nanovdb) and without MPI
or denoisers, and writes the configured headers to <out dir>/barney/ (build
output, never committed): the default build, or with --multi-scatter the
build with the BARNEY_USE_MULTI_SCATTERING option on (CMakeLists.txt:219-226).

  python oracle/refpin/configure.py <reference root> <out dir> [--multi-scatter]
"""
import re
import sys
from pathlib import Path

VALUES = {
    "BARNEY_VERSION_MAJOR": "1", "BARNEY_VERSION_MINOR": "1", "BARNEY_VERSION_PATCH": "8",
    "BARNEY_BACKEND_OPTIX": "0", "BARNEY_BACKEND_CUDA": "0", "BARNEY_BACKEND_EMBREE": "1",
    "BARNEY_BACKEND_HIPRT": "0", "BARNEY_HAVE_MPI": "0", "BARNEY_HAVE_NANOVDB": "1",
    "BARNEY_HAVE_CUDA": "0", "BARNEY_OIDN_CPU": "0", "BARNEY_OIDN_GPU": "0",
    "BARNEY_DISABLE_DENOISING": "1", "BARNEY_USE_MULTI_SCATTERING": "0", "BARNEY_CUBQL_BVH_WIDTH": "4",
}


def configure(text: str) -> str:
    def cm01(m):
        name = m.group(1)
        return f"#define {name} {VALUES.get(name, '0')}"
    text = re.sub(r"^#cmakedefine01\s+(\w+)\s*$", cm01, text, flags=re.M)
    text = re.sub(r"^#cmakedefine\s+(\w+).*$", lambda m: f"/* #undef {m.group(1)} */", text, flags=re.M)
    text = re.sub(r"@(\w+)@", lambda m: VALUES.get(m.group(1), "0"), text)
    text = re.sub(r"\$\{(\w+)\}", lambda m: VALUES.get(m.group(1), "0"), text)
    return text


def main(ref: str, out: str, multi_scatter: bool = False) -> None:
    VALUES["BARNEY_USE_MULTI_SCATTERING"] = "1" if multi_scatter else "0"
    ref_root, out_dir = Path(ref), Path(out) / "barney"
    out_dir.mkdir(parents=True, exist_ok=True)
    (out_dir / "barney.h").write_text(configure((ref_root / "barney/include/barney.h").read_text()))
    (out_dir / "barneyConfig.h").write_text(configure((ref_root / "barney/common/barneyConfig.h.in").read_text()))


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2], "--multi-scatter" in sys.argv[3:])
