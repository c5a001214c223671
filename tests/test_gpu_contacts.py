"""Voxel-voxel contacts with no per-voxel limit (the reference keeps every pair of
surface voxels more than 5 links apart in an unbounded list,
Voxelyze3/src/old/Voxelyze.cpp:671-751, old/VX_Collision.cpp:42-56).

* A dense pile — a soft 10^3 block dropped onto another one, collision radius
  0.75 — matches the CPU oracle within 1e-6 voxel sizes, with bit-exact
  static-friction flags, and never stops with an error.
* Keeping a single contact in each voxel's own slots sends every further contact
  through the spill pool: the run is bit-identical to the default one.
* A collision-heavy creature (40^3 at fill 0.5, a soft E=1e5 material among
  three, self-collision, contraction at 5 Hz) runs 20,000 steps without an error.
"""
import concurrent.futures as cf

import numpy as np
import pytest

from oracle.oracle import OracleSim, desc_from_vxa

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

pytestmark = pytest.mark.gpu

POS_TOL = 1e-6      # voxel sizes
SOFT = dict(E=1e5, rho=1000.0, nu=0.35, cte=0.0, mus=1.0, muk=0.5)


def dense_pile():
    """Two soft 10^3 blocks: the upper one starts one voxel above the lower one, shifted by
    three voxels along x, and falls onto it."""
    cells = np.zeros((21, 10, 13), np.int32)
    cells[0:10, :, 0:10] = 1
    cells[11:21, :, 3:13] = 1
    return synth.vxa_document(cells, np.zeros(cells.shape), [SOFT], collision=True, expansion=False, vary_temp=False,
                              bounding_radius=0.75, damping=(1.0, 0.8, 0.01))


def _state(ctx, sim):
    st = ctx.voxel_state(sim)
    return st["pos"], st["orient"], (st["flags"] >> 6) & 1


def test_dense_pile_matches_oracle(ctx):
    vxa = dense_pile()
    snaps = (700, 1100, 1500)
    o = OracleSim(desc_from_vxa(vxa))
    sim = ctx.load_vxa(vxa, name="pile")
    try:
        done = 0
        for s in snaps:
            ctx.step(sim, s - done)
            o.step(s - done)
            done = s
            pos, q, stat = _state(ctx, sim)
            b = o.voxel_state()
            assert ctx.info(sim).status == g.SIM_IDLE
            assert np.abs(pos - b["pos"]).max() / 0.01 <= POS_TOL, s
            assert np.abs(q - b["orient"]).max() <= POS_TOL, s
            assert np.array_equal(stat, (b["flags"] >> 3) & 1), s
        # the blocks touched: the upper block came to rest on the lower one
        assert pos[:, 2].max() < 0.20
    finally:
        ctx.free(sim)


def test_contact_spill_is_bit_identical():
    vxa = dense_pile()
    out = []
    for slots in (16, 1):
        with g.Context(0, 1 << 30) as c:
            c.set_contact_slots(slots)
            sim = c.load_vxa(vxa, name=f"pile{slots}")
            c.step(sim, 1500)
            assert c.info(sim).status == g.SIM_IDLE
            out.append(_state(c, sim))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))


def test_collision_heavy_creature_long_run(ctx):
    c = synth.config2_batch(1, seed=12)[0]
    sim = ctx.load_vxa(c.vxa, name="c2long")
    try:
        ctx.step(sim, 20000)
        info = ctx.info(sim)
        assert info.steps == 20000
        assert info.status == g.SIM_IDLE, info.status
        pos = ctx.voxel_state(sim)["pos"]
        assert np.isfinite(pos).all()
    finally:
        ctx.free(sim)


def test_watch_lists_across_step_calls_are_bit_identical():
    """Collision creatures stepped in many short calls (each call stops them at its target and
    starts them again, some of them right before a watch-list regeneration) end exactly where
    one long call takes them."""
    cs = synth.config2_batch(3, seed=31)
    out = []
    for calls in ([600], [37] * 16 + [8]):
        with g.Context(0, 4 << 30) as c:
            ids = [c.load_vxa(cr.vxa, name=f"w{i}") for i, cr in enumerate(cs)]
            for n in calls:
                c.step(ids, n, g.BATCHED)
            for i in ids:
                info = c.info(i)
                assert info.steps == 600 and info.status == g.SIM_IDLE, (info.steps, info.status)
            out.append([_state(c, i) for i in ids])
    for a, b in zip(out[0], out[1]):
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))


def test_contact_slots_argument_checked(ctx):
    for bad in (0, 17):
        with pytest.raises(g.VX3Error):
            ctx.set_contact_slots(bad)
    ctx.set_contact_slots(16)
