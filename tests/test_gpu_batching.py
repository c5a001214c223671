"""Batching and serving semantics on the GPU: the batched form, the plain
one-simulation-per-launch form, and a simulation served in a mix of others all
produce identical results; divergence retires one simulation without touching
the rest; the HBM budget gates admission."""
import numpy as np
import pytest

from oracle.oracle import OracleSim, desc_from_vxa

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def test_load_many_matches_one_by_one(ctx):
    """vx3_load_vxa_many (host threads) loads exactly what vx3_load_vxa loads, in both its
    forms (whole VXAs; base + VXDs), and rejects a malformed VXD without dropping the rest."""
    cs = synth.config1_batch(5, seed=21)
    a = [ctx.load_vxa(c.vxa, name=f"a{i}") for i, c in enumerate(cs)]
    b = ctx.load_many([c.vxa for c in cs], names=[f"b{i}" for i in range(len(cs))])
    base = cs[0].vxa
    vxd = ("<VXD><Structure replace=\"VXA.VXC.Structure\" Compression=\"ASCII_READABLE\"><X_Voxels>2</X_Voxels>"
           "<Y_Voxels>1</Y_Voxels><Z_Voxels>1</Z_Voxels><Data><Layer><![CDATA[12]]></Layer></Data></Structure></VXD>")
    c = ctx.load_many([vxd, vxd], base=base)
    with pytest.raises(g.VX3Error):
        ctx.load_many([vxd, "<VXD><Structure"], base=base)
    try:
        assert [ctx.info(i).num_voxel for i in c] == [2, 2]
        ctx.step(a + b, 100, g.BATCHED)
        for x, y in zip(a, b):
            assert np.array_equal(_bits(ctx.voxel_state(x)["pos"]), _bits(ctx.voxel_state(y)["pos"]))
    finally:
        for s in a + b + c:
            ctx.free(s)


def test_get_states_equals_per_simulation_readback(ctx):
    """vx3_get_states (one gather kernel, one copy) returns exactly what vx3_get_state
    returns for each simulation, in id order, including for a simulation never stepped."""
    cs = synth.config1_batch(4, seed=31)
    ids = [ctx.load_vxa(c.vxa, name=f"g{i}") for i, c in enumerate(cs)]
    try:
        ctx.step(ids[:3], 60, g.BATCHED)
        order = [ids[2], ids[0], ids[3], ids[1]]
        pos, q, fl, off = ctx.get_states(order)
        for k, i in enumerate(order):
            p1, q1, f1 = ctx.get_state(i)
            assert np.array_equal(_bits(pos[off[k]:off[k + 1]]), _bits(p1))
            assert np.array_equal(_bits(q[off[k]:off[k + 1]]), _bits(q1))
            assert np.array_equal(fl[off[k]:off[k + 1]], f1)
        nv, nl = ctx.sizes(order)                  # host-side counts, no device read
        assert list(nv) == [ctx.info(i).num_voxel for i in order]
        assert list(nl) == [ctx.info(i).num_link for i in order]
    finally:
        for s in ids:
            ctx.free(s)


def test_plain_and_batched_are_bit_identical(ctx):
    cs = synth.config1_batch(4, seed=9)
    a = [ctx.load_vxa(c.vxa, name=f"p{i}") for i, c in enumerate(cs)]
    b = [ctx.load_vxa(c.vxa, name=f"q{i}") for i, c in enumerate(cs)]
    try:
        for s in a:
            ctx.step(s, 200, g.PLAIN)
        ctx.step(b, 200, g.BATCHED)
        for x, y in zip(a, b):
            assert np.array_equal(_bits(ctx.voxel_state(x)["pos"]), _bits(ctx.voxel_state(y)["pos"]))
            assert np.array_equal(_bits(ctx.voxel_state(x)["orient"]), _bits(ctx.voxel_state(y)["orient"]))
    finally:
        for s in a + b:
            ctx.free(s)


def test_served_alone_and_in_mix_are_identical():
    c_probe = synth.config0_creature(21, stop_time=0.02)
    others = synth.config1_batch(5, seed=13, sim_time=0.01)
    with g.Context(0, 2 << 30) as c1:
        s = c1.load_vxa(c_probe.vxa, name="alone")
        c1.submit(s, 0)
        res = []
        while c1.pending():
            res += c1.poll(chunk_steps=32)
        r_alone = [r for r in res if r.id == s][0]
    with g.Context(0, 2 << 30) as c2:
        ids = [c2.load_vxa(o.vxa, name=f"o{i}") for i, o in enumerate(others[:2])]
        for i in ids:
            c2.submit(i, 0)
        c2.poll(chunk_steps=7)                        # the probe arrives while others run
        s2 = c2.load_vxa(c_probe.vxa, name="mix")
        c2.submit(s2, 0)
        for o in others[2:]:
            c2.submit(c2.load_vxa(o.vxa, name="late"), 0)
        res2 = []
        while c2.pending():
            res2 += c2.poll(chunk_steps=32)
        r_mix = [r for r in res2 if r.id == s2][0]
    assert r_alone.steps == r_mix.steps
    assert r_alone.current_time == r_mix.current_time
    assert list(r_alone.current_center_of_mass) == list(r_mix.current_center_of_mass)
    assert r_alone.fitness_score == r_mix.fitness_score
    assert r_alone.total_distance_of_all_voxels == r_mix.total_distance_of_all_voxels


def test_divergence_retires_only_that_simulation(ctx):
    ok = synth.config0_creature(2)
    # a DtFrac far beyond the stable step makes the link strains explode
    bad = synth.config0_creature(3, dt_frac=40.0)
    s_ok, s_bad = ctx.load_vxa(ok.vxa, name="ok"), ctx.load_vxa(bad.vxa, name="bad")
    try:
        ctx.step([s_ok, s_bad], 300, g.BATCHED)
        assert ctx.info(s_bad).status == g.SIM_DIVERGED
        o = OracleSim(desc_from_vxa(bad.vxa))
        o.step(300)
        assert o.scalars()["diverged"] == 1 and ctx.info(s_bad).steps == o.scalars()["steps"]
        assert ctx.info(s_ok).steps == 300 and ctx.info(s_ok).status != g.SIM_DIVERGED
        ref = OracleSim(desc_from_vxa(ok.vxa))
        ref.step(300)
        assert np.abs(ctx.voxel_state(s_ok)["pos"] - ref.voxel_state()["pos"]).max() / 0.01 <= 1e-6
    finally:
        ctx.free(s_ok)
        ctx.free(s_bad)


def test_hbm_budget_admission():
    big = synth.config0_creature(4)
    with g.Context(0, 64 << 10) as c:         # 64 KiB budget: too small for one creature
        s = c.load_vxa(big.vxa)
        with pytest.raises(g.VX3Error, match="OOM_BUDGET"):
            c.step(s, 1)
    cs = synth.config1_batch(12, seed=17, sim_time=0.005)
    with g.Context(0, 24 << 20) as c:         # room for a few at a time: the rest wait in the queue
        ids = [c.load_vxa(x.vxa) for x in cs]
        for i in ids:
            c.submit(i, 0)
        peak, done = 0, []
        while c.pending():
            done += c.poll(chunk_steps=64)
            peak = max(peak, c.bytes_in_use())
        assert len(done) == len(ids) and peak <= 24 << 20
        assert all(r.status == g.SIM_DONE for r in done)


def test_report_matches_worker_format(ctx, tmp_path):
    cs = [synth.config0_creature(30 + i, stop_time=0.01) for i in range(3)]
    ids = [ctx.load_vxa(c.vxa, name=f"bot_{i:04d}.vxd") for i, c in enumerate(cs)]
    try:
        ctx.run(ids)
        p = tmp_path / "report.xml"
        ctx.write_report(ids, str(p), "/data/generation_0001")
        txt = p.read_text()
        assert "<inputdir>generation_0001</inputdir>" in txt
        fits = sorted([ctx.result(i).fitness_score for i in ids], reverse=True)
        best = [i for i in ids if ctx.result(i).fitness_score == fits[0]][0]
        assert f"<filename>bot_{ids.index(best):04d}.vxd</filename>" in txt
        for i in range(3):
            assert f"<bot_{i:04d}><currentTime>" in txt
    finally:
        for i in ids:
            ctx.free(i)


def _serve_all(order, cap, creatures, horizons, chunk=32):
    with g.Context(0, 2 << 30) as c:
        c.set_serving(order, cap)
        ids = [c.load_vxa(cr.vxa, name=f"s{i}") for i, cr in enumerate(creatures)]
        for i, h in zip(ids, horizons):
            c.submit(i, h)
        finished = []
        while c.pending():
            finished += c.poll(chunk_steps=chunk)
        by_sim = {ids.index(r.id): r for r in finished}
        order_done = [ids.index(r.id) for r in finished]
        return by_sim, order_done


def test_serving_policies_change_order_not_results():
    """Least-work-first admission under a voxel cap finishes the small jobs first; with the lane
    for the longest, the request with the most work starts first; every simulation's result is
    bit-identical to first-come-first-served admission."""
    cs = sorted(synth.config1_batch(6, seed=41, sim_time=10.0), key=lambda c: c.num_voxel)[::-1]
    horizons = [600, 500, 400, 300, 200, 100]    # the larger creatures run longer: work order = arrival order reversed
    cap = max(c.num_voxel for c in cs) + min(c.num_voxel for c in cs)   # about two at a time
    fcfs, _ = _serve_all(g.SERVE_FCFS, 0, cs, horizons)
    lw, done = _serve_all(g.SERVE_LEAST_WORK, cap, cs, horizons)
    work = [c.num_voxel * h for c, h in zip(cs, horizons)]
    assert done[0] == int(np.argmin(work))
    lane, done_lane = _serve_all(g.SERVE_LONG_LANE, cap, cs, horizons)
    big = int(np.argmax(work))
    assert all(lane[big].start_time_s <= lane[k].start_time_s for k in range(len(cs)))
    assert done_lane[0] == int(np.argmin(work))
    for k in range(len(cs)):
        a, b, c = fcfs[k], lw[k], lane[k]
        assert a.steps == b.steps == c.steps == horizons[k]
        assert list(a.current_center_of_mass) == list(b.current_center_of_mass) == list(c.current_center_of_mass)
        assert a.total_distance_of_all_voxels == b.total_distance_of_all_voxels == c.total_distance_of_all_voxels
    with g.Context(0, 1 << 30) as c:
        with pytest.raises(g.VX3Error):
            c.set_serving(3, 0)
