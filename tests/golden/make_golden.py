"""Generates the golden fixtures under tests/golden/ from the reference itself.

Each fixture is a small VXA world (seeded, built by gpuvoxels_gb300.synth or
below), run through the reference's own CPU Voxelyze compiled from the
reference sources (oracle/_ref, see oracle/Makefile) with the VX3 step-driver
semantics of oracle/ref_harness.cpp.  The .npz files keep the VXA text, the
externals, and the reference's topology, material constants (as float bit
patterns) and state snapshots.

    make -C oracle ref && python tests/golden/make_golden.py

Only needed where the reference sources exist; the committed .npz files are
what the tests read.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from gpuvoxels_gb300 import synth  # noqa: E402
from oracle.oracle import RefSim, desc_from_vxa, merge_vxd  # noqa: E402


def grid_world(cells, materials, **kw):
    """cells: (Z, Y, X) material ids (0 = empty)."""
    cells = np.asarray(cells, np.int32)
    phase = np.zeros(cells.shape)
    return synth.vxa_document(cells, phase, materials, **kw)


SOFT = dict(E=1e5, rho=1000.0, nu=0.35, cte=0.0, mus=1.0, muk=0.5)
STIFF = dict(E=1e6, rho=1000.0, nu=0.35, cte=0.0, mus=0.8, muk=0.4)


def worlds():
    w = {}
    w["c0_seed0"] = dict(vxa=synth.config0_creature(0).vxa, ext=[], snaps=[1, 100, 300])
    c1 = synth.random_creature(11, (8, 8, 8), 0.7,
                               [dict(E=2.1e5, rho=1000.0, nu=0.35, cte=0.01, mus=1.0, muk=0.5),
                                dict(E=3.7e6, rho=1000.0, nu=0.35, cte=0.0, mus=1.0, muk=0.5),
                                dict(E=9.0e5, rho=1000.0, nu=0.35, cte=0.01, mus=1.0, muk=0.5),
                                dict(E=6.3e6, rho=1000.0, nu=0.35, cte=0.0, mus=1.0, muk=0.5)])
    w["c1_poisson"] = dict(vxa=c1.vxa, ext=[], snaps=[1, 150, 300])
    # two blocks: the upper one falls onto the lower one (self-collision between unlinked voxels)
    blocks = np.zeros((5, 3, 3), np.int32)
    blocks[0:2] = 1
    blocks[3:5] = 1
    w["falling_blocks"] = dict(vxa=grid_world(blocks, [SOFT], collision=True, expansion=False, vary_temp=False,
                                              damping=(1.0, 0.8, 0.01)), ext=[], snaps=[600, 1400, 2000])
    # bilinear cantilever: root fixed, tip pulled and pushed down (plasticity path, no gravity/floor)
    bil = dict(E=1e6, rho=1000.0, nu=0.0, cte=0.0, mus=0.0, muk=0.0)
    beam = np.ones((1, 1, 6), np.int32)
    vxa = grid_world(beam, [bil], gravity=0.0, floor=False, vary_temp=False, volume_effects=False)
    vxa = vxa.replace("<MatModel>0</MatModel><Elastic_Mod>1000000.0</Elastic_Mod><Fail_Stress>0</Fail_Stress>",
                      "<MatModel>2</MatModel><Elastic_Mod>1000000.0</Elastic_Mod><Plastic_Mod>200000.0</Plastic_Mod>"
                      "<Yield_Stress>10000.0</Yield_Stress><Fail_Stress>40000.0</Fail_Stress>")
    w["bilinear_cantilever"] = dict(vxa=vxa, ext=[dict(voxel=0, dof_fixed=0x3F), dict(voxel=5, force=(2.0, 0.0, -0.3))],
                                    snaps=[1, 200, 500])
    # large-angle bending: a tip moment rotates the end voxels past the small-angle threshold
    beam3 = np.ones((1, 1, 4), np.int32)
    vxa = grid_world(beam3, [STIFF], gravity=0.0, floor=False, vary_temp=False)
    w["large_angle"] = dict(vxa=vxa, ext=[dict(voxel=0, dof_fixed=0x3F), dict(voxel=3, moment=(0.0, 0.02, 0.05))],
                            snaps=[1, 300, 800])
    # partial fixes: translations of two corners, two rotation axes of another, moment in the middle
    plate = np.ones((1, 3, 3), np.int32)
    vxa = grid_world(plate, [STIFF], vary_temp=False)
    w["partial_fix"] = dict(vxa=vxa, ext=[dict(voxel=0, dof_fixed=0x07), dict(voxel=8, dof_fixed=0x07, translate=(0.0, 0.0, 0.001)),
                                          dict(voxel=2, dof_fixed=0x18), dict(voxel=4, moment=(0.01, 0.0, 0.0), force=(0.0, 0.5, 0.0))],
                            snaps=[1, 200, 400])
    # boundary-condition regions in the VXA: a fixed box, a forced/torqued sphere, a displaced cylinder
    bc = ("<Boundary_Conditions><NumBCs>3</NumBCs>"
          "<FRegion><PrimType>0</PrimType><X>0</X><Y>0</Y><Z>0</Z><dX>0.3</dX><dY>1</dY><dZ>1</dZ><DofFixed>63</DofFixed></FRegion>"
          "<FRegion><PrimType>2</PrimType><X>0.8</X><Y>0.5</Y><Z>0.5</Z><Radius>0.25</Radius><DofFixed>0</DofFixed>"
          "<ForceX>0.3</ForceX><ForceZ>-0.7</ForceZ><TorqueY>0.001</TorqueY></FRegion>"
          "<FRegion><PrimType>1</PrimType><X>0.5</X><Y>0.5</Y><Z>0</Z><dZ>1</dZ><Radius>0.2</Radius><DofFixed>5</DofFixed>"
          "<DisplaceZ>0.002</DisplaceZ><ForceY>0.1</ForceY></FRegion></Boundary_Conditions>")
    vxa = synth.config0_creature(0).vxa.replace("<Boundary_Conditions><NumBCs>0</NumBCs></Boundary_Conditions>", bc)
    w["bc_regions"] = dict(vxa=vxa, ext=[], snaps=[1, 300, 1000])
    # the smallest worlds: one voxel (no link: the time step from the voxel's own frequency),
    # dropped on the floor and pushed sideways (contact, static then kinetic friction)
    one = np.ones((1, 1, 1), np.int32)
    vxa = grid_world(one, [STIFF], vary_temp=False)
    w["single_voxel"] = dict(vxa=vxa, ext=[dict(voxel=0, force=(0.009, 0.002, 0.0))], snaps=[1, 400, 1500])
    # two voxels and one link, actuated (a thermal material beside a passive one)
    pair = np.array([[[1, 2]]], np.int32)
    vxa = grid_world(pair, [dict(SOFT, cte=0.01), STIFF])
    w["one_link"] = dict(vxa=vxa, ext=[], snaps=[1, 400, 1500])
    # a small creature of the collision configuration's materials (soft E=1e5 among E=1e6,
    # contraction-only actuation, self-collision on): it folds onto itself, so its watch lists
    # regenerate many times over the run
    mats = [dict(E=1e5, rho=1000.0, nu=0.35, cte=0.01, mus=1.0, muk=0.5),
            dict(E=1e6, rho=1000.0, nu=0.35, cte=0.01, mus=1.0, muk=0.5),
            dict(E=1e6, rho=1000.0, nu=0.35, cte=0.0, mus=1.0, muk=0.5)]
    cr = synth.random_creature(77, (12, 12, 12), 0.5, mats, collision=True, expansion=False)
    w["collide_creature"] = dict(vxa=cr.vxa, ext=[], snaps=[1, 800, 2000])
    return w


# The reference's own sample worlds (read from its source tree; the merged VXA text is stored in the fixture).
REF = os.environ.get("VX_REFERENCE", "")   # the reference's project root (required to regenerate the fixtures)
SAMPLES = {
    "ref_zoo_basic": ("zoo/basic/base.vxa", "zoo/basic/robot.vxd", [1, 300, 1000]),
    "ref_example": ("doc/misc/example.vxa", None, [1, 300, 1000]),
    "ref_signaling": ("Experiments/xenobot/c.signaling/data1/base.vxa", "Experiments/xenobot/c.signaling/data1/rob.vxd",
                      [1, 300, 1000]),
    "ref_memleaking": ("Experiments/xenobot/d.memleaking/data/base.vxa", "Experiments/xenobot/d.memleaking/data/rob.vxd",
                       [1, 300, 1000]),
    "ref_circle_push": ("Experiments/xenobot/e.circle_push/data1/base.vxa",
                        "Experiments/xenobot/e.circle_push/data1/bot_0017.vxd", [1, 300, 1000]),
    "ref_target_only": ("Experiments/xenobot/h.target_only/data1/base.vxa",
                        "Experiments/xenobot/h.target_only/data1/bot_0000.vxd", [1, 300]),
}
DAMPING_DEFAULTS = ("<Damping><BondDampingZ>0.1</BondDampingZ><ColDampingZ>1</ColDampingZ>"
                    "<SlowDampingZ>1</SlowDampingZ></Damping>")


def sample_worlds():
    """The reference's sample worlds, VXD merged into the base.  A world without
    <Damping> leaves the reference's damping members unset (VXA/VX_Sim.cpp:197-212
    only assigns them inside that element), so the fixture states the documented
    defaults 0.1/1.0/1.0 explicitly; nothing else is changed."""
    w = {}
    for name, (base, vxd, snaps) in SAMPLES.items():
        with open(os.path.join(REF, base), encoding="latin-1") as f:
            xml = f.read()
        if vxd:
            with open(os.path.join(REF, vxd), encoding="latin-1") as f:
                xml = merge_vxd(xml, f.read())
        if "<Damping>" not in xml:
            i = xml.index("<Simulator>") + len("<Simulator>")
            xml = xml[:i] + DAMPING_DEFAULTS + xml[i:]
        # cilia, run-time attachment and detachment are VX3-only behaviour the reference's CPU path
        # does not have: switched off so that the reference's output is the expected one (they are
        # tested on their own)
        for key in ("EnableCilia", "EnableAttach", "EnableDetach"):
            xml = re.sub(r"(<%s(?:\s[^>]*)?>)\s*1\s*(</%s>)" % (key, key), r"\g<1>0\g<2>", xml)
        w[name] = dict(vxa=xml, ext=[], snaps=snaps)
    return w


def run(name, spec):
    d = desc_from_vxa(spec["vxa"])
    r = RefSim(spec["vxa"], d)
    for e in spec["ext"]:
        r.set_external(e["voxel"], e.get("dof_fixed", 0), e.get("force", (0, 0, 0)), e.get("moment", (0, 0, 0)),
                       e.get("translate", (0, 0, 0)), e.get("rotate", (0, 0, 0)))
    topo = r.topology()
    mats = r.materials()
    exts = r.externals()
    out = dict(vxa=np.array(spec["vxa"]), ext=np.array(repr(spec["ext"])), snaps=np.array(spec["snaps"], np.int64),
               voxels=topo["voxels"], links=topo["links"], phase=topo["phase"],
               ext_dof=exts["dof"], ext_vals=exts["vals"],
               voxmat_bits=mats["voxmat"].view(np.uint32), nom=mats["nom"],
               linkmat_idx=mats["linkmat_idx"], linkmat_bits=mats["linkmat"].view(np.uint32))
    done = 0
    for k, s in enumerate(spec["snaps"]):
        r.step(s - done)
        done = s
        vs, ls, sc = r.voxel_state(), r.link_state(), r.scalars()
        out[f"s{k}_pos"] = vs["pos"]; out[f"s{k}_orient"] = vs["orient"]
        out[f"s{k}_linMom"] = vs["linMom"]; out[f"s{k}_angMom"] = vs["angMom"]
        out[f"s{k}_temp"] = vs["temp"]; out[f"s{k}_pStrain"] = vs["pStrain"]; out[f"s{k}_flags"] = vs["flags"]
        out[f"s{k}_strain"] = ls["strain"]; out[f"s{k}_maxStrain"] = ls["maxStrain"]; out[f"s{k}_smallAngle"] = ls["smallAngle"]
        out[f"s{k}_scalars"] = np.array([sc["t"], sc["optimal_dt"], sc["dt"], sc["diverged"], sc["steps"]])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: {r.nvox} voxels, {r.nlink} links, steps {spec['snaps']}")


if __name__ == "__main__":
    if not RefSim.available():
        sys.exit("oracle/_ref/libvxref.so missing: run `make -C oracle ref` where the reference sources exist")
    todo = dict(worlds())
    if os.path.isdir(REF):
        todo.update(sample_worlds())
    only = sys.argv[1:]
    for name, spec in todo.items():
        if not only or name in only:
            run(name, spec)
