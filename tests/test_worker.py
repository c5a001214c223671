"""The vx3_node_worker executable: the reference worker's process contract
(Voxelyze3/src/Executables/vx3_node_worker.cu:32-141) over the engine.

CPU tests cover the argument and input checks (exit status 1 with the reference's
messages).  The GPU test runs a generation of three VXD files and compares the report
with the results of the same files run through the Python API, and checks the
SavePositionOfAllVoxels fields (init_pos, pos, mats)."""
import os
import re
import subprocess
import xml.etree.ElementTree as ET

import pytest

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import build, synth


@pytest.fixture(scope="module")
def worker():
    build.build()
    return build.WORKER


def _run(worker, *args):
    return subprocess.run([worker, *args], capture_output=True, text=True, timeout=600)


def test_usage_without_arguments(worker):
    r = _run(worker)
    assert r.returncode == 1 and "Usage" in r.stdout


def test_missing_input(worker, tmp_path):
    r = _run(worker, "-i", str(tmp_path / "none.vxt"), "-o", str(tmp_path / "out.vxr"))
    assert r.returncode == 1 and "Error: input file not found." in r.stdout


def test_existing_output_needs_force(worker, tmp_path):
    (tmp_path / "out.vxr").write_text("x")
    (tmp_path / "job.vxt").write_text("<vxa>a</vxa>")
    r = _run(worker, "-i", str(tmp_path / "job.vxt"), "-o", str(tmp_path / "out.vxr"))
    assert r.returncode == 1 and "Error: output file exists." in r.stdout


def test_vxt_without_input_dir_is_rejected(worker, tmp_path):
    (tmp_path / "job.vxt").write_text('<?xml version="1.0" encoding="utf-8"?>\n<vxa>base.vxa</vxa>')
    r = _run(worker, "--input", str(tmp_path / "job.vxt"), "--output=" + str(tmp_path / "out.vxr"))
    assert r.returncode == 1 and "needs <vxa> and <input_dir>" in r.stderr


def _structure_vxd(seed):
    c = synth.random_creature(seed, (5, 5, 5), 0.7)
    s = re.search(r"<Structure.*</Structure>", c.vxa, re.S).group(0)
    s = s.replace("<Structure", '<Structure replace="VXA.VXC.Structure"', 1)
    return f"<VXD>{s}</VXD>"


@pytest.mark.gpu
def test_simulation_manager_python_mirror(tmp_path):
    """SimulationManager(sub_batches, base, input_dir).start() (the VX3_SimulationManager
    mirror) runs the files as one batch; h_results are sorted by fitness and equal the
    per-file results of the C ABI; write_report gives the worker's keys."""
    base = synth.config0_creature(0, stop_time=0.01).vxa
    (tmp_path / "base.vxa").write_text(base)
    gen = tmp_path / "gen"
    gen.mkdir()
    names = [f"bot_{i:04d}.vxd" for i in range(3)]
    for i, n in enumerate(names):
        (gen / n).write_text(_structure_vxd(60 + i))
    sm = g.SimulationManager([names[:2], names[2:]], base=str(tmp_path / "base.vxa"), input_dir=str(gen))
    res = sm.start()
    assert sorted(r.vxa_filename for r in res) == names
    fits = [r.fitness_score for r in res]
    assert fits == sorted(fits, reverse=True)
    with g.Context(0, 1 << 30) as ctx:
        for n in names:
            sid = ctx.load_vxa(base, (gen / n).read_text(), name=n)
            ctx.run([sid])
            r = ctx.result(sid)
            mine = [x for x in res if x.vxa_filename == n][0]
            assert mine.fitness_score == r.fitness_score and mine.currentTime == r.current_time
    sm.write_report(str(tmp_path / "report.xml"))
    rep = ET.parse(tmp_path / "report.xml").getroot()
    assert rep.find("bestfit/filename").text == res[0].vxa_filename


@pytest.mark.gpu
def test_worker_generation_report(worker, tmp_path):
    base = synth.config0_creature(0, stop_time=0.01).vxa
    base = base.replace("<Simulator>", "<Simulator><SavePositionOfAllVoxels>1</SavePositionOfAllVoxels>", 1)
    gen = tmp_path / "generation_0001"
    gen.mkdir()
    (tmp_path / "base.vxa").write_text(base)
    names = [f"bot_{i:04d}.vxd" for i in range(3)]
    vxds = [_structure_vxd(40 + i) for i in range(3)]
    for n, v in zip(names, vxds):
        (gen / n).write_text(v)
    # the layout Voxelyze3.cpp:101-112 writes: elements side by side, no single root
    (tmp_path / "job.vxt").write_text('<?xml version="1.0" encoding="utf-8"?>\n<vxa>' + str(tmp_path / "base.vxa") +
                                      "</vxa><input_dir>" + str(gen) + "</input_dir><vxd>" +
                                      "".join(f"<f>{n}</f>" for n in names) + "</vxd>")
    out = tmp_path / "report.vxr"
    r = _run(worker, "-i", str(tmp_path / "job.vxt"), "-o", str(out))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "GPU found." in r.stdout
    rep = ET.parse(out).getroot()
    assert rep.find("inputdir").text == "generation_0001"
    # the same files through the Python API
    with g.Context(0, 1 << 30) as ctx:
        ids = [ctx.load_vxa(base, v, name=n) for n, v in zip(names, vxds)]
        ctx.run(ids)
        res = {n: ctx.result(i) for n, i in zip(names, ids)}
        nvox = {n: ctx.info(i).num_voxel for n, i in zip(names, ids)}
    best = max(res, key=lambda n: res[n].fitness_score)
    assert rep.find("bestfit/filename").text == best
    for n in names:
        d = rep.find("detail/" + n.split(".")[0])
        assert float(d.find("fitness_score").text) == res[n].fitness_score
        assert float(d.find("currentTime").text) == res[n].current_time
        assert int(d.find("num_voxel").text) == nvox[n]
        pos = [p for p in d.find("pos").text.split(";") if p]
        init = [p for p in d.find("init_pos").text.split(";") if p]
        mats = [m for m in d.find("mats").text.split(";") if m]
        assert len(pos) == len(init) == len(mats) == nvox[n]
        assert all(m in ("1", "2") for m in mats)
        assert all(len(p.split(",")) == 3 for p in pos)
