"""The ctypes mirrors of the C ABI's structs have the C layout: the size and
every field offset of pfdd_request (include/pfdd_serve.h, mirrored in
pfdd_gb300/serve.py) and of pfdd_diag_params (include/pfdd_gpu.h, mirrored in
pfdd_gb300/native.py), as the C compiler lays them out, equal the ctypes ones
(a mismatch would hand the library shifted pointers and values)."""
import ctypes as C
import subprocess
from pathlib import Path

import pytest

from pfdd_gb300 import native, serve

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("ctype,cname,header", [(serve._Request, "pfdd_request", "pfdd_serve.h"),
                                                (native.DiagParams, "pfdd_diag_params", "pfdd_gpu.h")])
def test_struct_layout_matches_the_header(tmp_path, ctype, cname, header):
    fields = [f for f, _ in ctype._fields_]
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{header}"', "int main(void) {",
             f'  printf("size %zu\\n", sizeof({cname}));']
    lines += [f'  printf("{f} %zu\\n", offsetof({cname}, {f}));' for f in fields]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    out = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True,
                                                    check=True).stdout.splitlines())
    assert int(out["size"]) == C.sizeof(ctype)
    for f in fields:
        assert int(out[f]) == getattr(ctype, f).offset, f
