"""The C ABI is usable from plain C: the header compiles as C99 and a C program that calls
every entry point links against the built library (no GPU needed; nothing is run)."""
import os
import re
import shutil
import subprocess

import pytest

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import build

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "gpuvoxels_gb300.h")


def test_header_is_c99_and_links(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    build.build()
    names = re.findall(r"\b(vx3_[a-z0-9_]+)\s*\(", open(HEADER).read())
    names = sorted(set(n for n in names if n in g.EXPORTS))
    assert set(names) == set(g.EXPORTS)
    src = tmp_path / "use.c"
    body = "\n".join(f"    p[{i}] = (void*)&{n};" for i, n in enumerate(names))
    src.write_text('#include "gpuvoxels_gb300.h"\n#include <stdio.h>\n'
                   f"int main(void) {{\n    void* p[{len(names)}];\n{body}\n"
                   "    printf(\"%p\\n\", p[0]);\n    return 0;\n}\n")
    exe = tmp_path / "use"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe),
                        "-L", build.OUT_DIR, "-lgpuvoxels_gb300", "-Wl,-rpath," + build.OUT_DIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
