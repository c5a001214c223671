"""VX3 extras with state of their own, on the GPU: voxel signals (EnableSignals,
pacemaker materials, relayed signals, the signal-scaled cilia term), target measures
(targetCloseness, numClosePairs, target contacts), link detachment on failure
(AttachDetach/EnableDetach), the secondary experiment (material removal, initial
position reset) and Fixed materials.

The reference's CPU path has none of these and its GPU code does not build here, so
the checks are against the restatement in oracle/vx3_extras.py (signals, closeness),
against the VX3 formulas on single voxels, and against the invariants the VX3 code
keeps (a detached or removed link is gone from both voxels' link lists, removed voxels
stay where they were)."""
import numpy as np
import pytest

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth
from oracle.vx3_extras import SignalNet, target_closeness

pytestmark = pytest.mark.gpu

SOFT = dict(E=1e4, rho=1000.0, nu=0.0, cte=0.0, mus=1.0, muk=0.5)


def _mat(**kw):
    m = dict(SOFT)
    m.update(kw)
    return m


def _sig_mech(pacemaker=False, period=0.0, decay=0.9, delay=0.03, inactive=0.03, extra=""):
    return (f"<isPaceMaker>{1 if pacemaker else 0}</isPaceMaker><PaceMakerPeriod>{period!r}</PaceMakerPeriod>"
            f"<signalValueDecay>{decay!r}</signalValueDecay><signalTimeDelay>{delay!r}</signalTimeDelay>"
            f"<inactivePeriod>{inactive!r}</inactivePeriod>{extra}")


def _world(grid, mats, sim_extra="", detach=False, **kw):
    grid = np.asarray(grid, np.int32)
    opts = dict(gravity=0.0, floor=False, vary_temp=False, damping=(0.1, 1.0, 0.0), volume_effects=False)
    opts.update(kw)
    vxa = synth.vxa_document(grid, np.zeros(grid.shape), mats, **opts)
    if detach:
        vxa = vxa.replace("<AttachDetach>", "<AttachDetach><EnableDetach>1</EnableDetach>", 1)
    return vxa.replace("<Simulator>", "<Simulator>" + sim_extra, 1)


def _neighbours(vxa):
    top = g.inspect_vxa(vxa)
    nv = top["counts"]["voxels"]
    nbrs = [[-1] * 6 for _ in range(nv)]
    for n, p, axis, _ in top["links"]:
        nbrs[n][2 * axis] = p
        nbrs[p][2 * axis + 1] = n
    return nbrs, top["voxels"][:, 3]


def _oracle_net(vxa, sig_mats):
    nbrs, mat_of = _neighbours(vxa)
    return SignalNet(nbrs, sig_mats, mat_of)


def _sig(pacemaker=False, period=0.0, decay=0.9, delay=0.03, inactive=0.03):
    return dict(pacemaker=pacemaker, period=period, decay=decay, delay=delay, inactive=inactive)


def _run_against_oracle(ctx, vxa, net, steps, chunk=1):
    sim = ctx.load_vxa(vxa)
    try:
        t = 0.0
        done = 0
        while done < steps:
            k = min(chunk, steps - done)
            ctx.step(sim, k)
            dt = ctx.info(sim).dt
            for _ in range(k):
                net.step(t)
                t = t + dt
            done += k
        ex = ctx.extras(sim)
        got = np.stack([ex["localSignal"], ex["localSignalDt"], ex["inactiveUntil"], ex["signalValue"], ex["signalTime"],
                        ex["pacemakerNextPulse"]], axis=1)
        assert ctx.info(sim).current_time == t
        return got, np.array(net.state())
    finally:
        ctx.free(sim)


def test_pacemaker_signal_travels_along_a_bar(ctx):
    # 1 x 1 x 12 bar; voxel 0 is a pacemaker (pulse every 0.05 s); relay delay 0.01 s
    grid = [[[2] + [1] * 11]]
    mats = [_mat(mech=_sig_mech(delay=0.01, inactive=0.02)), _mat(mech=_sig_mech(True, 0.05, delay=0.01, inactive=0.02))]
    vxa = _world(grid, mats, "<EnableSignals>1</EnableSignals>")
    net = _oracle_net(vxa, [_sig(delay=0.01, inactive=0.02), _sig(True, 0.05, delay=0.01, inactive=0.02)])
    got, want = _run_against_oracle(ctx, vxa, net, 600, chunk=100)
    np.testing.assert_array_equal(got, want)
    assert (got[:, 0] > 0).sum() >= 3          # the signal reached several voxels


def test_signals_in_a_block_with_several_pacemakers(ctx):
    # 4 x 4 x 3 block, pacemakers at two corners with different periods, decay 0.8
    grid = np.ones((3, 4, 4), np.int32)
    grid[0, 0, 0] = 2
    grid[2, 3, 3] = 3
    sigs = [_sig(decay=0.8, delay=0.004, inactive=0.01), _sig(True, 0.03, decay=0.8, delay=0.004, inactive=0.01),
            _sig(True, 0.045, decay=0.8, delay=0.004, inactive=0.01)]
    mats = [_mat(mech=_sig_mech(s["pacemaker"], s["period"], s["decay"], s["delay"], s["inactive"])) for s in sigs]
    vxa = _world(grid, mats, "<EnableSignals>1</EnableSignals>")
    net = _oracle_net(vxa, sigs)
    got, want = _run_against_oracle(ctx, vxa, net, 800, chunk=50)
    np.testing.assert_array_equal(got, want)
    assert (got[:, 0] > 0).sum() >= 10


def test_signals_off_leave_no_state(ctx):
    grid = [[[2, 1, 1]]]
    mats = [_mat(mech=_sig_mech()), _mat(mech=_sig_mech(True, 0.05))]
    sim = ctx.load_vxa(_world(grid, mats))
    try:
        ctx.step(sim, 50)
        assert not ctx.extras(sim)["localSignal"].any()
    finally:
        ctx.free(sim)


def test_cilia_shift_scales_with_the_local_signal(ctx):
    # one pacemaker voxel with cilia: step 1 uses the base force (local signal 0); its own
    # signal step at t = 0 pulses (100) and decays it once (90), which step 2 uses
    mats = [_mat(mech=_sig_mech(True, 1.0) + "<Cilia>2</Cilia>")]
    vxa = _world([[[1]]], mats, "<EnableSignals>1</EnableSignals><EnableCilia>1</EnableCilia>", damping=(0.0, 0.0, 0.0))
    vxa = vxa.replace("</Data>", "</Data><BaseCiliaForce><Layer><![CDATA[0.5,-0.25,1.0]]></Layer></BaseCiliaForce>"
                      "<ShiftCiliaForce><Layer><![CDATA[0.01,0.02,-0.03]]></Layer></ShiftCiliaForce>", 1)
    sim = ctx.load_vxa(vxa)
    try:
        ctx.step(sim, 1)
        dtd = float(np.float32(ctx.info(sim).dt))
        m1 = ctx.voxel_state(sim)["linMom"][0].copy()
        np.testing.assert_array_equal(m1, [dtd * (0.5 * 2.0), dtd * (-0.25 * 2.0), dtd * (1.0 * 2.0)])
        assert ctx.extras(sim)["localSignal"][0] == 90.0
        ctx.step(sim, 1)
        m2 = ctx.voxel_state(sim)["linMom"][0]
        base = np.array([0.5, -0.25, 1.0]) + 90.0 * np.array([0.01, 0.02, -0.03])
        np.testing.assert_allclose(m2, m1 + dtd * (base * 2.0), rtol=1e-14, atol=0)
    finally:
        ctx.free(sim)


def _two_bodies(target_top=True, signals=False, max_dist=0.0):
    # a 3 x 3 x 2 target slab falling onto a 3 x 3 x 2 slab, two voxel layers apart
    grid = np.zeros((6, 3, 3), np.int32)
    grid[0:2] = 1
    grid[4:6] = 2 if target_top else 1
    mats = [_mat(E=1e5, mech=_sig_mech()), _mat(E=1e5, mech=_sig_mech(extra="<isTarget>1</isTarget>"))]
    extra = f"<MaxDistInVoxelLengthsToCountAsPair>{max_dist!r}</MaxDistInVoxelLengthsToCountAsPair>"
    if signals:
        extra += "<EnableSignals>1</EnableSignals>"
    return _world(grid, mats, extra, gravity=-9.81, floor=True, collision=True, damping=(0.1, 1.0, 0.0))


def _touching_pairs(st, nom, targets):
    """Touching target/non-target pairs before a step, with the engine's contact test
    (CVX_Collision::updateContactForce, VX_Collision.cpp:42-56): the float distance against
    (float)((baseSizeAverage1 + baseSizeAverage2) * 0.625), no thermal expansion here."""
    pos = st["pos"]
    n = len(pos)
    b = nom * 1.0
    bsa = (b + b + b) / 3.0
    nom_dist = np.float32((bsa + bsa) * float(np.float32(0.625)))
    out = []
    for a in range(n):
        for c in range(a + 1, n):
            if targets[a] == targets[c]:
                continue
            o = [np.float32(pos[c][k] - pos[a][k]) for k in range(3)]
            ln = np.sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2], dtype=np.float32)
            if np.float32(nom_dist - ln) > 0:
                out.append((a, c))
    return out


def test_target_contacts_count_and_hand_over_signals(ctx):
    vxa = _two_bodies(target_top=True, signals=True)
    top = g.inspect_vxa(vxa)
    targets = top["voxels"][:, 3] == 1
    sigs = [_sig(), _sig()]
    nbrs, mat_of = _neighbours(vxa)
    net = SignalNet(nbrs, sigs, mat_of)
    sim = ctx.load_vxa(vxa)
    try:
        count = 0
        t = 0.0
        for k in range(900):
            st = ctx.voxel_state(sim)
            pairs = _touching_pairs(st, 0.01, targets)
            count += len(pairs)
            hits = sorted({a if not targets[a] else b for a, b in pairs})
            ctx.step(sim, 1)
            net.step(t, hits)
            t = t + ctx.info(sim).dt
        ex = ctx.extras(sim)
        assert count > 0
        assert ex["collisionCount"] == count
        got = np.stack([ex["localSignal"], ex["localSignalDt"], ex["inactiveUntil"], ex["signalValue"], ex["signalTime"],
                        ex["pacemakerNextPulse"]], axis=1)
        np.testing.assert_array_equal(got, np.array(net.state()))
        assert ex["localSignal"][~targets].max() > 0   # the touched slab got signals
    finally:
        ctx.free(sim)


def test_target_closeness_at_the_sampling_steps(ctx):
    # three falling target voxels and one non-target voxel, apart; closeness at every CoM sample
    grid = np.zeros((3, 1, 7), np.int32)
    grid[0, 0, 0] = 2
    grid[1, 0, 3] = 2
    grid[2, 0, 6] = 2
    grid[0, 0, 5] = 1
    mats = [_mat(), _mat(mech="<isTarget>1</isTarget>")]
    vxa = _world(grid, mats, "<MaxDistInVoxelLengthsToCountAsPair>3.5</MaxDistInVoxelLengthsToCountAsPair>",
                 gravity=-9.81, floor=True, temp_period=0.05)
    top = g.inspect_vxa(vxa)
    targets = [i for i in range(top["counts"]["voxels"]) if top["voxels"][i, 3] == 1]
    sim = ctx.load_vxa(vxa)
    try:
        ctx.step(sim, 1)
        cycle = int(0.05 / ctx.info(sim).dt)             # int(TempPeriod / dt), VX3_VoxelyzeKernel.cu:312
        for _ in range(3):
            ctx.step(sim, cycle - (ctx.info(sim).steps % cycle))
            pos = ctx.voxel_state(sim)["pos"]
            ret, pairs = target_closeness(pos, targets, 3.5, 0.01)
            ex = ctx.extras(sim)
            assert ex["targetCloseness"] == ret
            assert ex["numClosePairs"] == pairs
        assert ex["numClosePairs"] >= 1
    finally:
        ctx.free(sim)


def _bar_with_fragile_middle(detach):
    # a 1 x 1 x 6 bar whose middle link joins two voxels of a weak material; the end voxel is
    # pulled, the first is fixed: the weak link fails
    grid = [[[1, 1, 2, 2, 1, 1]]]
    strong = _mat(E=1e6)
    weak = _mat(E=1e6, mech="<MatModel>1</MatModel><Fail_Stress>2000</Fail_Stress>")
    return _world(grid, [strong, weak], detach=detach, damping=(1.0, 1.0, 0.0))


def test_failed_links_detach_from_both_voxels(ctx):
    vxa = _bar_with_fragile_middle(True)
    top = g.inspect_vxa(vxa)
    nv = top["counts"]["voxels"]
    sim = ctx.load_vxa(vxa)
    try:
        ctx.set_external(sim, 0, dof_fixed=0x3F)
        ctx.set_external(sim, nv - 1, force=(2.0, 0.0, 0.0))
        ctx.step(sim, 3000)
        ls = ctx.link_state(sim)
        vs = ctx.voxel_state(sim)
        gone = (ls["flags"] & 32) != 0
        assert gone.any(), "no link failed"
        for l, (n, p, axis, _) in enumerate(top["links"]):
            has_n = (vs["flags"][n] >> (2 * axis)) & 1
            has_p = (vs["flags"][p] >> (2 * axis + 1)) & 1
            assert has_n == has_p == (0 if gone[l] else 1)
        # the detached part flies away with the pulled end
        assert vs["pos"][nv - 1, 0] > (nv - 1) * 0.01 + 0.02
    finally:
        ctx.free(sim)


def test_without_detach_failed_links_stay(ctx):
    vxa = _bar_with_fragile_middle(False)
    nv = g.inspect_vxa(vxa)["counts"]["voxels"]
    sim = ctx.load_vxa(vxa)
    try:
        ctx.set_external(sim, 0, dof_fixed=0x3F)
        ctx.set_external(sim, nv - 1, force=(2.0, 0.0, 0.0))
        ctx.step(sim, 3000)
        ls = ctx.link_state(sim)
        assert not (ls["flags"] & 32).any()
        assert (ls["maxStrain"] > 0).any()
    finally:
        ctx.free(sim)


def test_secondary_experiment_removes_a_material(ctx):
    # a 2 x 2 x 4 block falling under gravity whose top layer (material 2) leaves at t = 0.02 s
    grid = np.ones((4, 2, 2), np.int32)
    grid[3] = 2
    mats = [_mat(E=1e5), _mat(E=1e5, mech="<RemoveFromSimulationAfterThisManySeconds>0.02</RemoveFromSimulationAfterThisManySeconds>")]
    vxa = _world(grid, mats, "<SecondaryExperiment>1</SecondaryExperiment>"
                 "<ReinitializeInitialPositionAfterThisManySeconds>1000</ReinitializeInitialPositionAfterThisManySeconds>",
                 gravity=-9.81, floor=True)
    top = g.inspect_vxa(vxa)
    removed = top["voxels"][:, 3] == 1
    sim = ctx.load_vxa(vxa)
    try:
        ctx.step(sim, 1)
        dt = ctx.info(sim).dt
        n_before = int(0.02 / dt) - 2
        ctx.step(sim, n_before)
        assert not (ctx.voxel_state(sim)["flags"] & (1 << 11)).any()
        ctx.step(sim, 10)
        vs = ctx.voxel_state(sim)
        fl = vs["flags"]
        assert ((fl & (1 << 11)) != 0).tolist() == removed.tolist()
        assert not (fl[removed] & 0x3F).any()                       # no links left on removed voxels
        for n, p, axis, _ in top["links"]:                           # nor on their neighbours
            if removed[n] or removed[p]:
                assert not (fl[n] >> (2 * axis)) & 1 and not (fl[p] >> (2 * axis + 1)) & 1
        frozen = vs["pos"][removed].copy()
        ctx.step(sim, 200)
        vs2 = ctx.voxel_state(sim)
        np.testing.assert_array_equal(vs2["pos"][removed], frozen)    # removed voxels stay put
        assert not np.array_equal(vs2["pos"][~removed], vs["pos"][~removed])
        assert (ctx.link_state(sim)["flags"][[removed[n] or removed[p] for n, p, _, _ in top["links"]]] & 96 == 96).all()
    finally:
        ctx.free(sim)


def test_secondary_experiment_resets_initial_positions(ctx):
    # the reset time 0 passes at the second step: the initial centre of mass becomes the
    # last sampled one (still the initial one) and the initial positions those after step 2
    grid = np.ones((2, 2, 2), np.int32)
    vxa = _world(grid, [_mat(E=1e5)], "<SecondaryExperiment>1</SecondaryExperiment>", gravity=-9.81, floor=True)
    sim = ctx.load_vxa(vxa)
    try:
        ctx.step(sim, 2)
        p2 = ctx.voxel_state(sim)["pos"].copy()
        ctx.step(sim, 500)
        pf = ctx.voxel_state(sim)["pos"]
        r = ctx.result(sim)
        want = sum(float(np.sqrt(((pf[i] - p2[i]) ** 2).sum())) for i in range(len(pf)))
        np.testing.assert_allclose(r.total_distance_of_all_voxels, want, rtol=1e-12)
    finally:
        ctx.free(sim)


def test_fixed_material_voxels_never_move(ctx):
    # a 1 x 1 x 4 bar whose first voxel is of a Fixed material, under gravity
    grid = [[[2, 1, 1, 1]]]
    mats = [_mat(E=1e4), _mat(E=1e4, mech="<Fixed>1</Fixed>")]
    vxa = _world(grid, mats, gravity=-9.81, floor=False)
    sim = ctx.load_vxa(vxa)
    try:
        p0 = ctx.voxel_state(sim)["pos"].copy()
        ctx.step(sim, 500)
        vs = ctx.voxel_state(sim)
        np.testing.assert_array_equal(vs["pos"][0], p0[0])
        np.testing.assert_array_equal(vs["orient"][0], [1, 0, 0, 0])
        assert vs["pos"][3, 2] < p0[3, 2] - 1e-5                    # the free end sags
    finally:
        ctx.free(sim)


def _sticky_blocks(attach=True, cond="", same_material=True, sticky=True):
    # a 3 x 3 x 2 block falling onto another, two voxel layers apart, one sticky material
    grid = np.zeros((6, 3, 3), np.int32)
    grid[0:2] = 1
    grid[4:6] = 1 if same_material else 2
    mech = "<Sticky>1</Sticky>" if sticky else ""
    mats = [_mat(E=1e5, mech=mech), _mat(E=1e5, mech=mech)]
    vxa = _world(grid, mats, gravity=-9.81, floor=True, collision=True, damping=(0.1, 1.0, 0.0))
    ad = f"<EnableAttach>{1 if attach else 0}</EnableAttach><SafetyGuard>50</SafetyGuard>"
    if cond:
        ad += f"<AttachCondition><Condition_0>{cond}</Condition_0></AttachCondition>"
    return vxa.replace("<EnableAttach>0</EnableAttach>", ad, 1)


def _touch_set(st):
    pos = st["pos"]
    n = len(pos)
    b = 0.01 * 1.0
    bsa = (b + b + b) / 3.0
    nom_dist = np.float32((bsa + bsa) * float(np.float32(0.625)))
    out = set()
    for a in range(n):
        for c in range(a + 1, n):
            o = [np.float32(pos[c][k] - pos[a][k]) for k in range(3)]
            ln = np.sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2], dtype=np.float32)
            if np.float32(nom_dist - ln) > 0:
                out.add((a, c))
    return out


def test_attachment_joins_touching_sticky_voxels(ctx):
    from oracle.vx3_extras import attach_links
    vxa = _sticky_blocks()
    top = g.inspect_vxa(vxa)
    nv, nl0 = top["counts"]["voxels"], top["counts"]["links"]
    lower = top["voxels"][:, 2] < 3
    sim = ctx.load_vxa(vxa)
    try:
        made_total = 0
        for k in range(1500):
            st = ctx.voxel_state(sim)
            links = ctx.links(sim)
            touch = _touch_set(st)
            # pairs within 5 links of the loaded topology (same block) never reach the contact set
            cands = [(a, b) for (a, b) in touch if lower[a] != lower[b]]
            cur = [(n, p, ax) for n, p, ax, fl in links if not fl & 32]
            want = attach_links(st["pos"], st["orient"], cur, cands, nv)
            ctx.step(sim, 1)
            after = ctx.links(sim)
            got = [tuple(int(x) for x in r[:3]) for r in after[len(links):]]
            assert got == want, f"step {k}"
            made_total += len(got)
            if made_total and k > 600:
                break
        assert made_total > 0
        after = ctx.links(sim)
        fl = ctx.voxel_state(sim)["flags"]
        for n, p, ax, lf in after[nl0:]:
            assert lower[n] != lower[p]                       # new links join the two blocks
            assert (fl[n] >> (2 * ax)) & 1 and (fl[p] >> (2 * ax + 1)) & 1
    finally:
        ctx.free(sim)


@pytest.mark.parametrize("case", ["off", "condition_false", "not_sticky", "other_material"])
def test_attachment_needs_every_condition(ctx, case):
    kw = dict(off=dict(attach=False), condition_false=dict(cond="<mtCONST>-1</mtCONST>"),
              not_sticky=dict(sticky=False), other_material=dict(same_material=False))[case]
    vxa = _sticky_blocks(**kw)
    nl0 = g.inspect_vxa(vxa)["counts"]["links"]
    sim = ctx.load_vxa(vxa)
    try:
        ctx.step(sim, 1500)
        assert len(ctx.links(sim)) == nl0
    finally:
        ctx.free(sim)


def test_attachment_is_deterministic(ctx):
    vxa = _sticky_blocks()
    res = []
    for _ in range(2):
        sim = ctx.load_vxa(vxa)
        try:
            ctx.step(sim, 1200)
            res.append((ctx.links(sim).copy(), ctx.voxel_state(sim)["pos"].copy()))
        finally:
            ctx.free(sim)
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    assert len(res[0][0]) > g.inspect_vxa(vxa)["counts"]["links"]
