"""Every C struct that the ctypes bindings mirror has, field for field, the
offset and the total size the C compiler gives it: a field added on one side
only would otherwise shift the rest or let the library write past the
Python-owned buffer. A small C program built against include/ prints
sizeof / offsetof; no GPU and no library call."""
import ctypes
import os
import shutil
import subprocess

import pytest

from gpi_project_gb300 import _native as N
from gpi_project_gb300 import host as H
from gpi_project_gb300 import serve as S

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (C type, header, ctypes class)
STRUCTS = [
    ("sofi_config", "sofigpu.h", N.SofiConfig),
    ("sofi_tti_stress_args", "sofigpu.h", N.TtiStressArgs),
    ("sofih_par", "sofihost.h", H.SofihPar),
    ("sofi_request", "sofiserve.h", S.SofiRequest),
    ("sofi_request_info", "sofiserve.h", S.SofiRequestInfo),
    ("sofi_server_stats", "sofiserve.h", S.SofiServerStats),
    ("sofi_server_options", "sofiserve.h", S.SofiServerOptions),
]


def _c_name(name):
    return name[:-1] if name.endswith("_") else name  # del_ mirrors the C field del (a Python keyword)


def _c_layout(tmp_path):
    lines = ["#include <stddef.h>", "#include <stdio.h>"]
    lines += sorted({f'#include "{h}"' for _, h, _ in STRUCTS})
    lines.append("int main(void) {")
    for ctype, _, cls in STRUCTS:
        lines.append(f'printf("{ctype} size %zu\\n", sizeof({ctype}));')
        for name, *_ in cls._fields_:
            lines.append(f'printf("{ctype} {name} %zu\\n", offsetof({ctype}, {_c_name(name)}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(REPO, "include"), "-o", str(exe), str(src)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {tuple(ln.split()[:2]): int(ln.split()[2]) for ln in out.splitlines()}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_structs_match_the_c_headers(tmp_path):
    c = _c_layout(tmp_path)
    for ctype, _, cls in STRUCTS:
        assert ctypes.sizeof(cls) == c[(ctype, "size")], ctype
        for name, *_ in cls._fields_:
            assert getattr(cls, name).offset == c[(ctype, name)], (ctype, name)
