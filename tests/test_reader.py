"""Host side of the product, no GPU: the library loads and exports every declared
entry point; the VXA/VXD reader, material derivation and topology builder agree
bit for bit with the reference (golden fixtures); formula evaluation; errors."""
import math
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_WORLDS, ROOT, load_golden

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth


def _declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(vx3_\w+)\s*\(", txt, re.M))
    return names


def test_library_exports_every_declared_symbol():
    L = g.library()
    declared = _declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    assert declared == set(g.EXPORTS)


@pytest.mark.parametrize("name", GOLDEN_WORLDS)
def test_reader_matches_reference(name):
    z, vxa, _ = load_golden(name)
    p = g.inspect_vxa(vxa)
    assert np.array_equal(p["voxels"], z["voxels"])
    assert np.array_equal(p["links"], z["links"])
    assert np.array_equal(p["phase"], z["phase"])
    assert np.array_equal(p["voxmat"].view(np.uint32), z["voxmat_bits"])
    assert np.array_equal(p["linkmat"].view(np.uint32), z["linkmat_bits"])
    assert np.array_equal(p["linkmat_idx"], z["linkmat_idx"])
    # externals from the VXA's boundary-condition regions (none where the fixture sets them by API)
    if not load_golden(name)[2]:
        x = g.inspect_externals(vxa)
        assert np.array_equal(x["dof"], z["ext_dof"])
        fm = np.concatenate([x["force"], x["moment"]], 1)
        assert np.array_equal(fm.view(np.uint32), z["ext_vals"][:, :6].astype(np.float32).view(np.uint32))
        assert np.array_equal(np.concatenate([x["translate"], x["rotate"]], 1), z["ext_vals"][:, 6:])


def test_bc_regions_cover_every_primitive():
    z, vxa, _ = load_golden("bc_regions")
    dof = z["ext_dof"]
    assert (dof == 0x3F).sum() > 0 and (dof == 0x05).sum() > 0            # fixed box, displaced cylinder
    assert (np.abs(z["ext_vals"][:, 0]) > 0).sum() > 0                      # forced sphere
    assert (z["ext_vals"][:, 8] == 0.002).sum() > 0                        # prescribed z translation
    assert ((z["ext_vals"][:, 8] == 0.002) <= ((dof & 0x04) != 0)).all()    # only where z is fixed


def test_reader_counts_and_environment():
    c = synth.config0_creature(0)
    p = g.inspect_vxa(c.vxa)
    assert p["counts"]["voxels"] == c.num_voxel
    e = p["env"]
    assert e["vox_size"] == 0.01 and e["dt_frac"] == 0.95
    assert e["vary_temp"] == 1 and e["temp_amplitude"] == 39.0 and e["temp_period"] == 0.2 and e["enable_expansion"] == 1
    assert e["collisions"] == 0
    assert abs(e["gravity_mult"] - 9.81 / 9.80665) < 1e-6
    # every link joins lattice neighbours, negative end at the lower index along its axis
    v = p["voxels"]
    for neg, pos, axis, _ in p["links"]:
        d = v[pos, :3] - v[neg, :3]
        assert d[axis] == 1 and abs(d).sum() == 1


def test_volume_effects_off_zeroes_poisson_ratio():
    c = synth.config0_creature(0, volume_effects=False)
    p = g.inspect_vxa(c.vxa)
    assert (p["voxmat"][:, 1] == 0).all() and (p["linkmat"][:, 1] == 0).all()


def test_vxd_overrides_structure():
    base = synth.config0_creature(0).vxa
    vxd = ("<VXD><Structure replace=\"VXA.VXC.Structure\" Compression=\"ASCII_READABLE\"><X_Voxels>2</X_Voxels>"
           "<Y_Voxels>1</Y_Voxels><Z_Voxels>1</Z_Voxels><Data><Layer><![CDATA[12]]></Layer></Data></Structure></VXD>")
    p = g.inspect_vxa(base, vxd)
    assert p["counts"]["voxels"] == 2 and p["counts"]["links"] == 1
    assert p["voxels"][:, 3].tolist() == [0, 1]


def test_entity_references_and_cdata_are_read():
    """Character and entity references in text and attributes are replaced (tinyxml's reading),
    CDATA is taken as it stands."""
    base = synth.config0_creature(0).vxa
    vxd = ("<VXD><Structure replace=\"VXA.VXC.Structure\" Compression=\"ASCII_READABL&#69;\"><X_Voxels>&#50;</X_Voxels>"
           "<Y_Voxels>1</Y_Voxels><Z_Voxels>1</Z_Voxels><Data><Layer><![CDATA[12]]></Layer></Data></Structure>"
           "<Lattice replace=\"VXA.VXC.Lattice\"><Lattice_Dim>0.0&#x32;</Lattice_Dim></Lattice>"
           "<DtFrac replace=\"VXA.Simulator.Integration.DtFrac\">0.&#55;5</DtFrac></VXD>")
    p = g.inspect_vxa(base, vxd)
    assert p["counts"]["voxels"] == 2 and p["counts"]["links"] == 1
    assert p["env"]["vox_size"] == 0.02 and p["env"]["dt_frac"] == 0.75


def test_formula_evaluation():
    vxa = synth.config0_creature(0, stop_time=0.25).vxa
    vars9 = [0.1, 0.2, 0.3, 0, 0.3, 0, 0, 0, 100]
    assert g.eval_formula(vxa, "stop", vars9) == pytest.approx(0.3 - 0.25)
    assert g.eval_formula(vxa, "fitness", vars9) == 0.1
    tree = ("<FitnessFunction><mtADD><mtMUL><mtVAR>x</mtVAR><mtVAR>y</mtVAR></mtMUL><mtDIV><mtVAR>z</mtVAR>"
            "<mtCONST>2</mtCONST></mtDIV></mtADD></FitnessFunction>")
    vxa2 = vxa.replace("<FitnessFunction><mtVAR>x</mtVAR></FitnessFunction>", tree)
    assert g.eval_formula(vxa2, "fitness", vars9) == pytest.approx(0.1 * 0.2 + 0.3 / 2)


@pytest.mark.parametrize("bad", [
    "<VXA><VXC><Structure>",                                   # truncated XML
    "<NOTVXA/>",
    "<VXA><VXC><Palette/><Structure Compression=\"ASCII_READABLE\"><X_Voxels>2</X_Voxels><Y_Voxels>1</Y_Voxels>"
    "<Z_Voxels>1</Z_Voxels><Data><Layer><![CDATA[1]]></Layer></Data></Structure></VXC></VXA>",   # short layer
    "<VXA><VXC><Palette/><Structure Compression=\"ASCII_READABLE\"><X_Voxels>1</X_Voxels><Y_Voxels>1</Y_Voxels>"
    "<Z_Voxels>1</Z_Voxels><Data><Layer><![CDATA[3]]></Layer></Data></Structure></VXC></VXA>",   # missing material
    "<VXA><VXC><Palette><Material><Mechanical><Elastic_Mod>1e6</Elastic_Mod></Mechanical></Material></Palette>"
    "<Structure Compression=\"ASCII_READABLE\"><X_Voxels>2</X_Voxels><Y_Voxels>1</Y_Voxels><Z_Voxels>1</Z_Voxels>"
    "<Data><Layer><![CDATA[00]]></Layer></Data></Structure></VXC></VXA>",   # no voxels (the reference aborts such a simulation)
    "<VXA><Environment><Boundary_Conditions><NumBCs>1</NumBCs><FRegion><PrimType>3</PrimType></FRegion></Boundary_Conditions>"
    "</Environment><VXC><Palette><Material><Mechanical><Elastic_Mod>1e6</Elastic_Mod></Mechanical></Material></Palette>"
    "<Structure Compression=\"ASCII_READABLE\"><X_Voxels>1</X_Voxels><Y_Voxels>1</Y_Voxels><Z_Voxels>1</Z_Voxels>"
    "<Data><Layer><![CDATA[1]]></Layer></Data></Structure></VXC></VXA>",   # mesh boundary-condition region
    "<VXA><Environment><Boundary_Conditions><NumBCs>2</NumBCs><FRegion><PrimType>0</PrimType></FRegion></Boundary_Conditions>"
    "</Environment><VXC><Palette><Material><Mechanical><Elastic_Mod>1e6</Elastic_Mod></Mechanical></Material></Palette>"
    "<Structure Compression=\"ASCII_READABLE\"><X_Voxels>1</X_Voxels><Y_Voxels>1</Y_Voxels><Z_Voxels>1</Z_Voxels>"
    "<Data><Layer><![CDATA[1]]></Layer></Data></Structure></VXC></VXA>",   # fewer regions than NumBCs
])
def test_reader_rejects_malformed_worlds(bad):
    with pytest.raises(g.VX3Error, match="VX3_E_PARSE"):
        g.inspect_vxa(bad)


def test_reach_exclusion_matches_lattice_hops():
    """The collision exclusion rule (within 5 links) for a bent chain: two voxels that are
    lattice-adjacent but 6 links apart along the chain must not be excluded."""
    from oracle.oracle import desc_from_vxa  # noqa: F401  (import check only)
    # U-shaped chain of 8 voxels in the x-y plane: the ends are 1 apart in the lattice, 7 links along the chain
    cells = np.zeros((1, 3, 4), np.int32)
    for x, y in [(0, 0), (1, 0), (2, 0), (3, 0), (3, 1), (3, 2), (2, 2), (1, 2)]:
        cells[0, y, x] = 1
    vxa = synth.vxa_document(cells, np.zeros(cells.shape), [synth.PASSIVE], collision=True)
    p = g.inspect_vxa(vxa)
    assert p["counts"]["links"] == 7 and p["counts"]["surface"] == 8
