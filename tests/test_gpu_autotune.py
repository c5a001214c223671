"""The project autotuner (vx3_autotune) and the launch-shape knobs it searches.

* It picks a shape from its search space: threads per block 128 or 256 (links
  and voxels alike), elements per link and per voxel work item 256, 512 or
  1024, elements a warp claims from the link and voxel queues 32, 64 or 128.
* It leaves the simulations' state as it found it: tuned and untuned runs of
  the same steps are bit-identical, and so are the steps after tuning.
* Claim sizes and block sizes never change results (the step kernels' work is
  per element and the force gather has a fixed order).
"""
import numpy as np
import pytest

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

pytestmark = pytest.mark.gpu

BLOCKS = {128, 256}
ITEMS = {256, 512, 1024}
CLAIMS = {32, 64, 128}


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def _run(creatures, steps, tune=False, claims=None, block=None):
    with g.Context(0, 2 << 30) as ctx:
        if claims:
            ctx.set_claim_sizes(*claims)
        if block:
            ctx.set_tuning(block_links=block, block_voxels=block)
        ids = [ctx.load_vxa(c.vxa, name=f"a{i}") for i, c in enumerate(creatures)]
        ctx.step(ids, 3, g.BATCHED)
        before = ctx.get_states(ids)
        if tune:
            ctx.autotune(ids)
            after = ctx.get_states(ids)
            for a, b in zip(before[:3], after[:3]):
                assert np.array_equal(_bits(a), _bits(b))      # tuning put the state back
        shape = ctx.tuning()
        ctx.step(ids, steps, g.BATCHED)
        pos, q, fl, _ = ctx.get_states(ids)
        return shape, pos, q, fl


def test_autotune_shape_and_state():
    cs = synth.config1_batch(24, seed=31, sim_time=0.5)
    shape, pos, q, fl = _run(cs, 150, tune=True)
    assert shape["block_links"] in BLOCKS and shape["block_voxels"] == shape["block_links"]
    assert shape["items_links"] in ITEMS and shape["items_voxels"] in ITEMS
    assert shape["claim_links"] in CLAIMS and shape["claim_voxels"] in CLAIMS
    _, pos0, q0, fl0 = _run(cs, 150)
    assert np.array_equal(_bits(pos), _bits(pos0))
    assert np.array_equal(_bits(q), _bits(q0))
    assert np.array_equal(fl, fl0)


@pytest.mark.parametrize("claims,block", [((64, 64), None), ((128, 32), 128), ((32, 128), None)])
def test_launch_shapes_do_not_change_results(claims, block):
    cs = synth.config1_batch(12, seed=32, sim_time=0.5)
    shape, pos, q, fl = _run(cs, 120, claims=claims, block=block)
    assert (shape["claim_links"], shape["claim_voxels"]) == claims
    _, pos0, q0, fl0 = _run(cs, 120)
    assert np.array_equal(_bits(pos), _bits(pos0))
    assert np.array_equal(_bits(q), _bits(q0))
    assert np.array_equal(fl, fl0)
