"""VX3 extras on the GPU: the force field (VXA Simulator/ForceField formulas,
VX3_Voxel.cu:178-184), cilia (EnableCilia, material Cilia and its start time,
per-voxel BaseCiliaForce; VX3_VoxelyzeKernel.cu:846-859, VX3_Voxel.cu:376) and the
delayed thermal actuation (TurnOnThermalExpansionAfterThisManySeconds,
VX3_VoxelyzeKernel.cu:625-650).  The reference's CPU path has none of these, so the
expectations are formed from the VX3 formulas on single voxels where every other
force is zero: after one step from rest the momentum is exactly dt times the force."""
import numpy as np
import pytest

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

pytestmark = pytest.mark.gpu


def _single_voxel(extra_sim="", extra_mech="", structure_extra="", cells=((1,),)):
    grid = np.array([list(cells)], np.int32)   # (Z=1, Y, X)
    mat = dict(E=1e6, rho=1000.0, nu=0.0, cte=0.0, mus=1.0, muk=0.5)
    vxa = synth.vxa_document(grid, np.zeros(grid.shape), [mat], gravity=0.0, floor=False, vary_temp=False,
                             damping=(0.0, 0.0, 0.0), volume_effects=False)
    vxa = vxa.replace("<Simulator>", "<Simulator>" + extra_sim, 1)
    vxa = vxa.replace("<Mechanical>", "<Mechanical>" + extra_mech, 1)
    vxa = vxa.replace("</Data>", "</Data>" + structure_extra, 1)
    return vxa


def _step1(ctx, vxa):
    sim = ctx.load_vxa(vxa)
    try:
        ctx.step(sim, 1)
        st = ctx.voxel_state(sim)
        return st, ctx.info(sim).dt
    finally:
        ctx.free(sim)


def test_force_field_formula_of_position(ctx):
    # x force = -3 * x, z force = 0.25 (constant), y absent (0)
    ff = ("<ForceField><x_forcefield><mtMUL><mtCONST>-3</mtCONST><mtVAR>x</mtVAR></mtMUL></x_forcefield>"
          "<z_forcefield><mtCONST>0.25</mtCONST></z_forcefield></ForceField>")
    vxa = _single_voxel(ff, cells=((0, 0, 1),))           # the voxel sits at x = 2 voxel sizes
    st, dt = _step1(ctx, vxa)
    x0 = 2 * 0.01
    dtd = float(np.float32(dt))
    assert st["linMom"][0, 0] == dtd * (-3.0 * x0)
    assert st["linMom"][0, 1] == 0.0
    assert st["linMom"][0, 2] == dtd * 0.25


def test_force_field_absent_or_zero_changes_nothing(ctx):
    base = _single_voxel()
    zero = _single_voxel("<ForceField><x_forcefield><mtCONST>0</mtCONST></x_forcefield></ForceField>")
    a, _ = _step1(ctx, base)
    b, _ = _step1(ctx, zero)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["linMom"], b["linMom"])


def test_cilia_force_and_start_time(ctx):
    cilia = "<BaseCiliaForce><Layer><![CDATA[0.5,-0.25,1.0]]></Layer></BaseCiliaForce>"
    on = _single_voxel("<EnableCilia>1</EnableCilia>", "<Cilia>2</Cilia>", cilia)
    st, dt = _step1(ctx, on)
    dtd = float(np.float32(dt))
    np.testing.assert_array_equal(st["linMom"][0], [dtd * (0.5 * 2.0), dtd * (-0.25 * 2.0), dtd * (1.0 * 2.0)])
    later = _single_voxel("<EnableCilia>1</EnableCilia>", "<Cilia>2</Cilia><TurnOnCiliaAfterThisManySeconds>1</TurnOnCiliaAfterThisManySeconds>",
                          cilia)
    st, _ = _step1(ctx, later)
    assert not st["linMom"].any()
    off = _single_voxel("", "<Cilia>2</Cilia>", cilia)        # EnableCilia absent: no cilia
    st, _ = _step1(ctx, off)
    assert not st["linMom"].any()


def test_cilia_only_on_surface_voxels(ctx):
    # a 3x3x3 block: the centre voxel is interior and gets no cilia force
    grid = np.ones((3, 3, 3), np.int32)
    mat = dict(E=1e6, rho=1000.0, nu=0.0, cte=0.0, mus=1.0, muk=0.5)
    vxa = synth.vxa_document(grid, np.zeros(grid.shape), [mat], gravity=0.0, floor=False, vary_temp=False,
                             damping=(0.0, 0.0, 0.0), volume_effects=False)
    layer = ",".join(["0,0,1"] * 9)
    vxa = vxa.replace("<Simulator>", "<Simulator><EnableCilia>1</EnableCilia>", 1)
    vxa = vxa.replace("<Mechanical>", "<Mechanical><Cilia>1</Cilia>", 1)
    vxa = vxa.replace("</Data>", "</Data><BaseCiliaForce>" + "".join(f"<Layer><![CDATA[{layer}]]></Layer>" for _ in range(3)) +
                      "</BaseCiliaForce>", 1)
    st, dt = _step1(ctx, vxa)
    dtd = float(np.float32(dt))
    mz = st["linMom"][:, 2]
    assert mz[13] == 0.0                                      # centre voxel (index 13 in x-fastest order)
    assert (np.delete(mz, 13) == dtd * 1.0).all()


def test_thermal_expansion_start_time(ctx):
    c = synth.config0_creature(1)
    delayed = c.vxa.replace("<Mechanical>", "<Mechanical><TurnOnThermalExpansionAfterThisManySeconds>0.01"
                                            "</TurnOnThermalExpansionAfterThisManySeconds>", 1)
    sim = ctx.load_vxa(delayed)
    try:
        info = g.inspect_vxa(delayed)
        e = info["env"]
        mats = info["voxels"][:, 3]
        delayed_mat = 0                                        # the first palette material carries the delay
        ctx.step(sim, 20)
        t = ctx.info(sim).current_time
        assert t < 0.01
        temp = ctx.voxel_state(sim)["temp"]
        assert (temp[mats == delayed_mat] == e["initial_temp"]).all()
        two_pi = float(np.float32(2 * np.float32(3.1415926)))
        want = e["temp_amplitude"] * np.sin(two_pi * (t / e["temp_period"] + info["phase"]))
        if not e["enable_expansion"]:
            want = np.minimum(want, 0)
        want = want.astype(np.float32)
        np.testing.assert_allclose(temp[mats != delayed_mat], want[mats != delayed_mat], rtol=0, atol=1e-4)
        assert (temp[mats != delayed_mat] != e["initial_temp"]).any()
    finally:
        ctx.free(sim)
