"""The .history recorder (vx3_record_history): the stream the reference prints from its
simulation loop when the VXA sets RecordHistory (Voxelyze3/src/VX3/VX3_SimulationManager.cu:40-114).

The GPU test records a creature for 300 steps and checks the header lines, the record step
labels (every int(RecordStepSize/(10000*recommendedTimeStep*DtFrac))+1 loop steps), and every
number of every record against the CPU oracle stepped alongside: positions, rotation angle,
orientation, deformed corner offsets (CVX_Voxel::cornerOffset from the link strains, as
VX3_Voxel.cu:147-159 forms it) and material ids, within half a unit of the printed digit."""
import math
import re

import numpy as np
import pytest

from oracle.oracle import OracleSim, desc_from_vxa

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth


def _with_history(vxa, step_size, link=1):
    rec = (f"<RecordHistory><RecordStepSize>{step_size}</RecordStepSize><RecordVoxel>1</RecordVoxel>"
           f"<RecordLink>{link}</RecordLink></RecordHistory>")
    return vxa.replace("<Simulator>", "<Simulator>" + rec, 1)


def _expected_record(o, info):
    """Numbers of one voxel record from the oracle's state (the reference's formulas)."""
    vs, ls = o.voxel_state(), o.link_state()
    vox, links = info["voxels"], info["links"]
    vm, nom = info["voxmat"], info["nom"]
    E = vm[:, 0]
    nv = len(vox)
    # links per voxel and direction (X+, X-, Y+, Y-, Z+, Z-)
    dirs = -np.ones((nv, 6), np.int64)
    for l, (ng, pv, ax) in enumerate(zip(links[:, 0], links[:, 1], links[:, 2])):
        dirs[ng, 2 * ax] = l
        dirs[pv, 2 * ax + 1] = l
    rows = []
    for v in range(nv):
        if (dirs[v] >= 0).all():
            continue
        p = vs["pos"][v] * 1000.0
        w, x, y, z = vs["orient"][v]
        ang = 2.0 * math.acos(min(w, 1.0)) * 57.29577951308232
        mi = int(vox[v, 3])
        half = 0.5 * (nom[mi] * float(np.float32(1) + np.float32(vs["temp"][v]) * np.float32(vm[mi, 3])))
        nnn, ppp = [], []
        for i in range(3):
            for pos_link in (False, True):
                l = dirs[v, 2 * i + (0 if pos_link else 1)]
                st = 1.0 if pos_link else -1.0
                if l >= 0:
                    s = np.float32(ls["strain"][l])
                    ratio = np.float32(E[vox[links[l, 1], 3]]) / np.float32(E[vox[links[l, 0], 3]])
                    ax = (np.float32(2) * s * ratio / (np.float32(1) + ratio)) if pos_link else (np.float32(2) * s / (np.float32(1) + ratio))
                    st = (1 + float(ax)) * (1 if pos_link else -1)
                (ppp if pos_link else nnn).append(float(np.float32(half * st)) * 1000.0)
        rows.append([*p, ang, x, y, z, *nnn, *ppp, mi + 1, 0.0])
    return np.array(rows)


@pytest.mark.gpu
def test_history_stream_matches_oracle(ctx, tmp_path):
    c = synth.config0_creature(3)
    vxa = _with_history(c.vxa, 20)
    info = g.inspect_vxa(vxa)
    sim = ctx.load_vxa(vxa, name="hist")
    path = tmp_path / "run.history"
    with pytest.raises(g.VX3Error):
        other = ctx.load_vxa(c.vxa, name="nohist")
        try:
            ctx.record_history(other, str(tmp_path / "x.history"))
        finally:
            ctx.free(other)
    ctx.record_history(sim, str(path))
    o = OracleSim(desc_from_vxa(vxa))
    total = 300
    try:
        ctx.step(sim, total)
        ctx.record_history(sim, None)       # closes the file
        text = path.read_text()
        lines = text.split("\n")
        assert lines[1] == "{{{setting}}}<rescale>0.001</rescale>"
        assert sum(1 for ln in lines if ln.startswith("{{{setting}}}<matcolor>")) == len(info["voxmat"])
        assert "{{{setting}}}<voxel_size>0.010000</voxel_size>" in lines
        m = [re.match(r"real_stepsize: (\d+) ; recommendedTimeStep ([0-9.]+); d_v3->DtFrac ([0-9.]+) \. $", ln) for ln in lines]
        m = [x for x in m if x]
        assert len(m) == 1
        rs = int(m[0].group(1))
        opt = o.scalars()["optimal_dt"] if o.scalars()["optimal_dt"] else None
        recs = [ln for ln in lines if ln.startswith("<<<Step")]
        want_j = list(range(0, total, rs))
        assert [int(re.match(r"<<<Step(\d+) ", r).group(1)) for r in recs] == want_j
        done = 0
        for r in recs:
            j = int(re.match(r"<<<Step(\d+) ", r).group(1))
            o.step(j + 1 - done)
            done = j + 1
            if opt is None:
                opt = o.scalars()["optimal_dt"]
                assert rs == int(20 / (10000 * opt * info["env"]["dt_frac"])) + 1
            t = float(re.match(r"<<<Step\d+ Time:([0-9.]+)>>>", r).group(1))
            assert abs(t - o.scalars()["t"]) < 1e-6
            body = r[r.index(">>>") + 3:r.index("<<<>>>")]
            got = np.array([[float(x) for x in item.split(",")[:-1]] for item in body.split(";") if item])
            exp = _expected_record(o, info)
            assert got.shape == exp.shape
            tol = np.array([0.051] * 4 + [0.0051] * 3 + [0.051] * 6 + [0, 0])
            assert (np.abs(got - exp) <= tol + 1e-9).all(), np.abs(got - exp).max(axis=0)
            links = r[r.index("|[[[") :]
            assert links.startswith(f"|[[[{j}]]]") and links.endswith("[[[]]]")
            assert links.count(";") == len(info["links"])
    finally:
        ctx.free(sim)
