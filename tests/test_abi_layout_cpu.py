"""The Python mirrors of the C ABI's structures (ctypes) have the layout that
include/sph_c.h gives them: for every public structure, a C program compiled
against the header reports sizeof and the offset of each field, which must
equal the ctypes structure's.  Also the documented 128-byte snapshot header.
Host only: gcc and the header, no device and no library call."""
import ctypes as C
import json
import os
import shutil
import subprocess

import pytest

from libfluid_gb300._capi import SphExec, SphParams
from libfluid_gb300._capi_batch import SphLattice
from libfluid_gb300.server import Request, ServerConfig, ServerStats

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "sph_params": SphParams,
    "sph_exec_config": SphExec,
    "sph_lattice": SphLattice,
    "sph_server_config": ServerConfig,
    "sph_request": Request,
    "sph_server_stats": ServerStats,
}


def _c_layout(tmp_path):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "sph_c.h"', 'int main(void) {',
             '    printf("{");']
    first = True
    for cname, py in list(MIRRORS.items()) + [("sph_snapshot_header", None)]:
        fields = [f[0] for f in py._fields_] if py is not None else []
        parts = ['\\"size\\": %zu']
        args = [f"sizeof({cname})"]
        for f in fields:
            parts.append(f'\\"{f}\\": %zu')
            args.append(f"offsetof({cname}, {f})")
        sep = "" if first else ", "
        first = False
        lines.append(f'    printf("{sep}\\"{cname}\\": {{{", ".join(parts)}}}", {", ".join(args)});')
    lines += ['    printf("}\\n");', '    return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_mirrors_match_the_header(tmp_path):
    layout = _c_layout(tmp_path)
    for cname, py in MIRRORS.items():
        c = layout[cname]
        assert C.sizeof(py) == c["size"], cname
        for f in py._fields_:
            assert getattr(py, f[0]).offset == c[f[0]], (cname, f[0])
    assert layout["sph_snapshot_header"]["size"] == 128
