"""GPU parity on the shapes of the benchmark configurations, against the CPU oracle.

* Collision-heavy creature: 40^3 at fill 0.5, three materials including a soft
  one (E=1e5), self-collision with collision radius 0.75, contraction-only
  actuation at 5 Hz; 1,000 steps.
* Single large body, reduced: a solid 40x40x20 slab of one actuated material
  with per-voxel phase; 1,000 steps.
  Both: positions and orientations within 1e-6 voxel sizes, static-friction
  flags bit-exact (the bar of the specification).
* Full horizons: three plain creatures (10^3, fill 0.6) over their 10,000
  steps, and four creatures of the batched configuration (side U{6..20}, four
  materials with E log-uniform in [1e5, 1e7]) run to their stop condition at
  0.5 s simulated (35,000-56,000 steps): centre-of-mass displacement within
  1e-4 relative.

The oracle runs on host threads (its C calls release the GIL) while the GPU
works.
"""
import concurrent.futures as cf

import numpy as np
import pytest

from oracle.oracle import OracleSim, desc_from_vxa

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

pytestmark = pytest.mark.gpu

POS_TOL = 1e-6      # voxel sizes
COM_RTOL = 1e-4


def _oracle_run(vxa, steps):
    o = OracleSim(desc_from_vxa(vxa))
    o.step(steps)
    return o


def _oracle_state(vxa, steps):
    o = _oracle_run(vxa, steps)
    return o.voxel_state()


@pytest.fixture(scope="module")
def pool():
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        yield ex


@pytest.mark.parametrize("shape", ["collide_40cube", "slab_40x40x20"])
def test_config_shapes_match_oracle_1000_steps(ctx, pool, shape):
    if shape == "collide_40cube":
        c = synth.config2_batch(1, seed=12)[0]
    else:
        c = synth.slab(40, 40, 20, seed=5)
    fut = pool.submit(_oracle_state, c.vxa, 1000)
    sim = ctx.load_vxa(c.vxa, name=shape)
    try:
        ctx.step(sim, 1000)
        assert ctx.info(sim).status == g.SIM_IDLE
        st = ctx.voxel_state(sim)
    finally:
        ctx.free(sim)
    b = fut.result()
    assert np.abs(st["pos"] - b["pos"]).max() / 0.01 <= POS_TOL
    assert np.abs(st["orient"] - b["orient"]).max() <= POS_TOL
    assert np.array_equal((st["flags"] >> 6) & 1, (b["flags"] >> 3) & 1)


def _com_displacements(ctx, pool, creatures, steps=None):
    """Runs the creatures together on the GPU (to their stop condition, or `steps` steps) and
    each on the oracle for the GPU's step count; returns (gpu, oracle) displacements."""
    sims = [ctx.load_vxa(c.vxa, name=f"h{i}") for i, c in enumerate(creatures)]
    try:
        if steps is None:
            ctx.run(sims, g.BATCHED)
            rs = [ctx.result(s) for s in sims]
            for r in rs:
                assert r.status == g.SIM_DONE
        else:
            ctx.step(sims, steps, g.BATCHED)
            rs = [ctx.result(s) for s in sims]
            for r in rs:
                assert r.steps == steps
        futs = [pool.submit(_oracle_run, c.vxa, r.steps) for c, r in zip(creatures, rs)]
        out = []
        for r, f in zip(rs, futs):
            o = f.result()
            assert abs(o.scalars()["t"] - r.current_time) < 1e-12
            init = np.array(r.initial_center_of_mass)
            out.append((np.array(r.current_center_of_mass) - init, o.center_of_mass() - init))
        return out
    finally:
        for s in sims:
            ctx.free(s)


def test_config0_center_of_mass_full_horizon(ctx, pool):
    creatures = [synth.config0_creature(seed) for seed in (0, 1, 2)]
    for dg, do in _com_displacements(ctx, pool, creatures, steps=10000):
        assert np.linalg.norm(dg - do) <= COM_RTOL * max(np.linalg.norm(do), 1e-12)


def test_config1_center_of_mass_full_horizon(ctx, pool):
    cs = synth.config1_batch(40, seed=21, sim_time=0.5)
    creatures = [c for c in cs if 200 <= c.num_voxel <= 400][:4]
    assert len(creatures) == 4
    for dg, do in _com_displacements(ctx, pool, creatures):
        assert np.linalg.norm(dg - do) <= COM_RTOL * max(np.linalg.norm(do), 1e-12)
