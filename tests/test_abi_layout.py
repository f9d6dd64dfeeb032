"""The ctypes mirrors of the C-ABI structs have exactly the C layout: a small
C program built against include/gsx.h prints every field offset and size."""
import ctypes
import subprocess
from pathlib import Path

import pytest

from gaussian_splatting_3d_gb300._lib import GsxCamera, GsxRasterParams
from gaussian_splatting_3d_gb300.batch import GsxBatchView

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def c_layout(struct_name, fields, tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gsx.h"', "int main(void) {",
             f'  printf("size %zu\\n", sizeof({struct_name}));']
    for f in fields:
        lines.append(f'  printf("{f} %zu\\n", offsetof({struct_name}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / f"{struct_name}.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / struct_name
    subprocess.run(["gcc", "-I", str(INCLUDE), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}


@pytest.mark.parametrize("cls,name", [(GsxCamera, "gsx_camera"), (GsxRasterParams, "gsx_raster_params"),
                                      (GsxBatchView, "gsx_batch_view")])
def test_struct_layout_matches_header(cls, name, tmp_path):
    fields = [f[0] for f in cls._fields_]
    got = c_layout(name, fields, tmp_path)
    assert got["size"] == ctypes.sizeof(cls)
    for f in fields:
        assert got[f] == getattr(cls, f).offset, f
