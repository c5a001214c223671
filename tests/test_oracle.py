"""The CPU oracle (oracle/vx_oracle.c) pinned against the reference: the golden
fixtures made from the reference's own CPU Voxelyze (tests/golden/make_golden.py),
and, where the reference sources are present, the reference itself."""
import numpy as np
import pytest

from conftest import GOLDEN_WORLDS, load_golden
from oracle.oracle import OracleSim, RefSim, desc_from_vxa, merge_vxd

from gpuvoxels_gb300 import synth


def _oracle_for(vxa, ext):
    d = desc_from_vxa(vxa)
    d["externals"] = d["externals"] + list(ext)    # boundary-condition regions of the VXA, then the API externals
    return OracleSim(d)


def _u(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


@pytest.mark.parametrize("name", GOLDEN_WORLDS)
def test_oracle_matches_golden_bitwise(name):
    z, vxa, ext = load_golden(name)
    o = _oracle_for(vxa, ext)
    topo, mats = o.topology(), o.materials()
    assert np.array_equal(topo["voxels"], z["voxels"])
    assert np.array_equal(topo["links"], z["links"])
    assert np.array_equal(_u(mats["voxmat"]), z["voxmat_bits"])
    assert np.array_equal(_u(mats["linkmat"]), z["linkmat_bits"])
    done = 0
    for k, s in enumerate(z["snaps"]):
        o.step(int(s) - done)
        done = int(s)
        vs, ls, sc = o.voxel_state(), o.link_state(), o.scalars()
        for key in ("pos", "orient", "linMom", "angMom"):
            assert np.array_equal(_u(vs[key]), _u(z[f"s{k}_{key}"])), (name, s, key)
        assert np.array_equal(_u(vs["temp"]), _u(z[f"s{k}_temp"]))
        assert np.array_equal(_u(vs["pStrain"]), _u(z[f"s{k}_pStrain"]))
        assert np.array_equal(vs["flags"], z[f"s{k}_flags"])
        assert np.array_equal(_u(ls["strain"]), _u(z[f"s{k}_strain"]))
        assert np.array_equal(ls["smallAngle"], z[f"s{k}_smallAngle"])
        assert sc["dt"] == z[f"s{k}_scalars"][2] and sc["t"] == z[f"s{k}_scalars"][0]


def test_golden_worlds_exercise_the_hard_paths():
    """The fixtures cover large-angle links, plastic yield, static friction and contact."""
    z, _, _ = load_golden("large_angle")
    assert z["s1_smallAngle"].min() == 0
    z, _, _ = load_golden("bilinear_cantilever")
    assert z["s2_maxStrain"].max() > 10000.0 / 1e6          # past the yield strain
    z, _, _ = load_golden("c0_seed0")
    assert (z["s2_flags"] & 8).any()                       # some voxel in static friction
    z, _, _ = load_golden("falling_blocks")
    top_before, top_after = z["s0_pos"][18:, 2].min(), z["s2_pos"][18:, 2].min()
    assert top_after < top_before and top_after < 0.0225  # top block rests on the bottom one: contact


@pytest.mark.skipif(not RefSim.available(), reason="reference sources not compiled here (oracle/_ref)")
@pytest.mark.parametrize("seed", [3, 4])
def test_oracle_matches_reference_on_random_creatures(seed):
    c = synth.random_creature(seed, (7, 6, 5), 0.65,
                              [synth.PASSIVE, synth.ACTIVE, dict(E=3e5, rho=800.0, nu=0.3, cte=0.02, mus=0.6, muk=0.3)],
                              collision=True, expansion=(seed % 2 == 0))
    d = desc_from_vxa(c.vxa)
    r, o = RefSim(c.vxa, d), OracleSim(d)
    for n in (1, 99, 400):
        r.step(n)
        o.step(n)
        a, b = r.voxel_state(), o.voxel_state()
        assert np.array_equal(_u(a["pos"]), _u(b["pos"]))
        assert np.array_equal(_u(a["orient"]), _u(b["orient"]))
        assert np.array_equal(a["flags"], b["flags"])


def test_vxd_merge_replaces_subtrees():
    base = "<VXA><Simulator><Integration><DtFrac>0.5</DtFrac></Integration></Simulator><VXC><Structure>A</Structure></VXC></VXA>"
    vxd = "<VXD><Structure replace=\"VXA.VXC.Structure\">B</Structure><X replace=\"VXA.Simulator.New\">7</X><Y>ignored</Y></VXD>"
    m = merge_vxd(base, vxd)
    assert "<Structure replace=\"VXA.VXC.Structure\">B</Structure>" in m
    assert "<New replace=\"VXA.Simulator.New\">7</New>" in m
    assert "ignored" not in m and ">A<" not in m
