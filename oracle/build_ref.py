"""TEST INFRASTRUCTURE ONLY: build the CPU emulation of the reference's CUDA
kernels into ``oracle/_ref/libref_emu.so`` (git-ignored).

The reference's kernels live in header files that also hold host launchers
written with CUDA's triple-chevron launch syntax, which g++ cannot parse.  The
recipe therefore copies, at build time and only into the git-ignored
``oracle/_ref/src``, the line ranges that hold the kernels and device functions
(each prefixed by a #line directive naming the original file and line), and
compiles them with ``oracle/ref_emu/ref_driver.cpp`` against the shim headers
in ``oracle/ref_emu/shim``.  The reference's common.h, data_spec.h, kernels.h,
shencoder.h and helper_math.h are included unmodified from the reference's
gs/src/include.  Nothing from the reference is committed.

The reference checkout is taken from $GSX_REFERENCE_DIR (default
/root/reference, where the build container mounts it); where it is absent
``reference_available()`` is False and nothing is built.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
from pathlib import Path

# the reference checkout: $GSX_REFERENCE_DIR, else where this build's
# container mounts it
REF = Path(os.environ.get("GSX_REFERENCE_DIR", "/root/reference"))
INC = REF / "gs" / "src" / "include"
HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC_OUT = OUT / "src"
LIB = OUT / "libref_emu.so"

# (file within the reference, first line, last line), inclusive
SECTIONS = {
    "ref_vol_render_helpers.inc": [("gs/src/include/vol_render.h", 10, 85)],
    "ref_vol_render_sh.inc": [("gs/src/include/vol_render_sh.h", 11, 248),
                              ("gs/src/include/vol_render_sh.h", 268, 455)],
    "ref_aabb_culling.inc": [("gs/src/include/aabb_culling.h", 11, 41),
                             ("gs/src/include/aabb_culling.h", 70, 103)],
    "ref_culling.inc": [("gs/src/include/culling.h", 11, 20)],
}


def reference_available() -> bool:
    return (INC / "vol_render_sh.h").exists()


def extract() -> None:
    SRC_OUT.mkdir(parents=True, exist_ok=True)
    for name, parts in SECTIONS.items():
        chunks = []
        for rel, a, b in parts:
            lines = (REF / rel).read_text().splitlines()
            chunks.append(f'#line {a} "{REF / rel}"')
            chunks.extend(lines[a - 1:b])
        (SRC_OUT / name).write_text("\n".join(chunks) + "\n")


def build(force: bool = False) -> Path:
    if not reference_available():
        raise FileNotFoundError("reference sources not present")
    extract()
    driver = HERE / "ref_emu" / "ref_driver.cpp"
    shim = HERE / "ref_emu" / "shim"
    h = hashlib.sha256()
    for p in sorted(list(SRC_OUT.glob("*.inc")) + [driver] + list(shim.rglob("*.h*"))):
        h.update(p.read_bytes())
    for p in sorted(INC.glob("*.h")):
        h.update(p.read_bytes())
    stamp = OUT / "libref_emu.sha256"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == h.hexdigest():
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-w",
           "-D__CUDACC__", "-I", str(shim), "-I", str(SRC_OUT), "-I", str(INC), str(driver), "-o",
           str(LIB) + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference emulation build failed:\n{' '.join(cmd)}\n{r.stderr[-4000:]}")
    os.replace(str(LIB) + ".tmp", LIB)
    stamp.write_text(h.hexdigest())
    return LIB


if __name__ == "__main__":
    print(build(force=True))
