"""The ctypes mirror of the C structs matches the header: sizes and field offsets of
frg_config, frg_stats and frg_system_desc as the C compiler lays them out (CPU only)."""
import ctypes
import os
import shutil
import subprocess

import pytest

import finite_root_generation_gb300 as frg

ROOT = os.path.join(os.path.dirname(__file__), "..")


def _c_layout(tmp_path, struct, fields):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = [f'printf("size %zu\\n", sizeof({struct}));']
    lines += [f'printf("{f} %zu\\n", offsetof({struct}, {f}));' for f in fields]
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "frg_gb300.h"\nint main(void) {\n'
                   + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (ln.split() for ln in out.strip().splitlines())}


@pytest.mark.parametrize("struct,cls", [("frg_config", frg.FrgConfig), ("frg_stats", frg.FrgStats),
                                        ("frg_system_desc", frg.FrgSystemDesc)])
def test_struct_layout_matches_header(tmp_path, struct, cls):
    names = [f for f, _ in cls._fields_]
    c = _c_layout(tmp_path, struct, names)
    assert c["size"] == ctypes.sizeof(cls)
    for f in names:
        assert c[f] == getattr(cls, f).offset, f
