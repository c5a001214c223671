"""The C ABI is usable from plain C: the header compiles as C99 and a C program that calls
every entry point links against the built library (no GPU needed; nothing is run); on a GPU,
a C program loads two creatures from a VXA file, steps them and reads their results and poses,
and gets exactly what the Python binding of the same library gets."""
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


C_STEPPER = r"""
#include "gpuvoxels_gb300.h"
#include <stdio.h>
#include <stdlib.h>

static char* slurp(const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    char* s = (char*)malloc((size_t)n + 1);
    if (fread(s, 1, (size_t)n, f) != (size_t)n) { fclose(f); free(s); return NULL; }
    s[n] = 0;
    fclose(f);
    return s;
}

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    char* a = slurp(argv[1]);
    char* b = slurp(argv[2]);
    long steps = atol(argv[3]);
    if (!a || !b) return 3;
    vx3_ctx* c = vx3_create(0, (size_t)1 << 30);
    if (!c) { fprintf(stderr, "vx3_create failed\n"); return 4; }
    const char* docs[2] = {a, b};
    const char* names[2] = {"a", "b"};
    vx3_sim_id ids[2];
    int st[2];
    if (vx3_load_vxa_many(c, NULL, docs, names, 2, ids, st) != VX3_OK) { fprintf(stderr, "%s\n", vx3_last_error(c)); return 5; }
    if (vx3_step(c, ids, 2, VX3_BATCHED, steps) != VX3_OK) { fprintf(stderr, "%s\n", vx3_last_error(c)); return 6; }
    for (int k = 0; k < 2; k++) {
        vx3_result r;
        vx3_sim_info info;
        if (vx3_get_result(c, ids[k], &r) != VX3_OK || vx3_sim_info_get(c, ids[k], &info) != VX3_OK) return 7;
        printf("result %d %lld %.17g %.17g %.17g %.17g\n", r.status, (long long)r.steps, r.current_time,
               r.current_center_of_mass[0], r.current_center_of_mass[1], r.current_center_of_mass[2]);
        int32_t nv = info.num_voxel;
        double* pos = (double*)malloc(sizeof(double) * 3 * (size_t)nv);
        double* q = (double*)malloc(sizeof(double) * 4 * (size_t)nv);
        uint8_t* fl = (uint8_t*)malloc((size_t)nv);
        if (vx3_get_state(c, ids[k], pos, q, fl) != VX3_OK) return 8;
        printf("pose %d %.17g %.17g %.17g %.17g\n", nv, pos[0], pos[3 * nv - 1], q[0], q[4 * nv - 1]);
        free(pos); free(q); free(fl);
    }
    vx3_destroy(c);
    free(a); free(b);
    return 0;
}
"""


@pytest.mark.gpu
def test_c_program_steps_creatures_like_python(tmp_path):
    import numpy as np
    from gpuvoxels_gb300 import synth
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    build.build()
    src = tmp_path / "step.c"
    src.write_text(C_STEPPER)
    exe = tmp_path / "step"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe),
                        "-L", build.OUT_DIR, "-lgpuvoxels_gb300", "-Wl,-rpath," + build.OUT_DIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    creatures = [synth.config0_creature(3), synth.config0_creature(4)]
    files = []
    for i, c in enumerate(creatures):
        f = tmp_path / f"c{i}.vxa"
        f.write_text(c.vxa)
        files.append(str(f))
    steps = 300
    r = subprocess.run([str(exe)] + files + [str(steps)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    results = [l.split()[1:] for l in lines if l.startswith("result ")]
    poses = [l.split()[1:] for l in lines if l.startswith("pose ")]
    assert len(results) == 2 and len(poses) == 2
    ctx = g.Context(0, 1 << 30)
    try:
        ids = [ctx.load_vxa(c.vxa, name=str(i)) for i, c in enumerate(creatures)]
        ctx.step(ids, steps, g.BATCHED)
        for k, sim in enumerate(ids):
            res = ctx.result(sim)
            pos, q, _ = ctx.get_state(sim)
            got = results[k]
            assert int(got[0]) == res.status and int(got[1]) == res.steps == steps
            assert float(got[2]) == res.current_time
            assert [float(x) for x in got[3:6]] == list(res.current_center_of_mass)
            nv = int(poses[k][0])
            assert nv == pos.shape[0]
            pos = pos.reshape(-1)
            q = q.reshape(-1)
            assert [float(x) for x in poses[k][1:]] == [pos[0], pos[-1], q[0], q[-1]]
            assert np.isfinite(pos).all()
    finally:
        ctx.close()
