"""Known-answer tests restated from the reference's own unit tests
(VoxCAD/src/VX2/test/tVoxelyze.h:61-243, `test2Vox` with the cases of
`singleBondFixedFree` and `singleBondFreeFree`).

Two 1 mm voxels of a 1 MPa, 1000 kg/m^3 material (internal damping 1.0,
global damping 0.2) joined by one link; voxel 1 is fixed (or loaded with the
opposite force/moment), voxel 2 gets a force or moment with all other DOFs
fixed.  The displacement (or rotation) of voxel 2 must settle on the expected
value — within 1e-5 relative for 10 consecutive steps — in fewer steps than the
reference's limit.  Each case runs on the CPU oracle (no GPU) and on the GPU
engine through the C ABI."""
import math

import numpy as np
import pytest

from oracle.oracle import OracleSim, desc_from_vxa

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

TX, TY, TZ, RX, RY, RZ = range(6)
F = 1e-3
M = 1e-9
DIRS = {"X_POS": (1, 0, 0), "X_NEG": (-1, 0, 0), "Y_POS": (0, 1, 0), "Y_NEG": (0, -1, 0), "Z_POS": (0, 0, 1), "Z_NEG": (0, 0, -1)}


def dof(tx, ty, tz, rx, ry, rz):
    return sum(int(b) << i for i, b in enumerate((tx, ty, tz, rx, ry, rz)))


def vec(axis, s):
    v = [0.0, 0.0, 0.0]
    v[axis] = s
    return tuple(v)


# (v1 fixed, direction, force, moment, dof, step limit, expected, readout)  tVoxelyze.h:142-199, :205-243
FIXED_FREE = [
    (True, "X_POS", vec(0, F), None, dof(0, 1, 1, 1, 1, 1), 150, 1e-6, TX),
    (True, "X_POS", vec(0, -F), None, dof(0, 1, 1, 1, 1, 1), 150, -1e-6, TX),
    (True, "X_POS", vec(1, F), None, dof(1, 0, 1, 1, 1, 1), 150, 1e-6, TY),
    (True, "X_POS", vec(2, -F), None, dof(1, 1, 0, 1, 1, 1), 150, -1e-6, TZ),
    (True, "X_NEG", vec(0, F), None, dof(0, 1, 1, 1, 1, 1), 150, 1e-6, TX),
    (True, "Y_POS", vec(1, F), None, dof(1, 0, 1, 1, 1, 1), 150, 1e-6, TY),
    (True, "Y_NEG", vec(0, F), None, dof(0, 1, 1, 1, 1, 1), 150, 1e-6, TX),
    (True, "Z_POS", vec(2, F), None, dof(1, 1, 0, 1, 1, 1), 150, 1e-6, TZ),
    (True, "Z_NEG", vec(0, F), None, dof(0, 1, 1, 1, 1, 1), 150, 1e-6, TX),
    (True, "X_POS", None, vec(0, M), dof(1, 1, 1, 0, 1, 1), 200, 1.2e-5, RX),
    (True, "X_POS", None, vec(1, -M), dof(1, 1, 1, 1, 0, 1), 200, -3e-6, RY),
    (True, "X_POS", None, vec(2, M), dof(1, 1, 1, 1, 1, 0), 200, 3e-6, RZ),
    (True, "Y_POS", None, vec(1, M), dof(1, 1, 1, 1, 0, 1), 200, 1.2e-5, RY),
    (True, "Z_NEG", None, vec(2, M), dof(1, 1, 1, 1, 1, 0), 200, 1.2e-5, RZ),
    (True, "X_POS", None, vec(1, M), dof(1, 1, 0, 1, 0, 1), 300, -6e-9, TZ),
    (True, "X_POS", None, vec(2, -M), dof(1, 0, 1, 1, 1, 0), 300, -6e-9, TY),
    (True, "X_POS", vec(1, F), None, dof(1, 0, 1, 1, 1, 0), 300, 6e-3, RZ),
    (True, "X_POS", vec(2, F), None, dof(1, 1, 0, 1, 0, 1), 300, -6e-3, RY),
    (True, "X_POS", None, vec(0, M), dof(0, 1, 1, 0, 1, 1), 10, 0.0, TX),
    (True, "X_POS", vec(0, F), None, dof(0, 1, 1, 0, 1, 1), 10, 0.0, RX),
]
FREE_FREE = [
    (False, "X_POS", vec(0, F), None, dof(0, 1, 1, 1, 1, 1), 100, 5e-7, TX),
    (False, "X_POS", vec(1, -F), None, dof(1, 0, 1, 1, 1, 1), 100, -5e-7, TY),
    (False, "Y_NEG", vec(1, F), None, dof(1, 0, 1, 1, 1, 1), 100, 5e-7, TY),
    (False, "Z_POS", vec(2, F), None, dof(1, 1, 0, 1, 1, 1), 100, 5e-7, TZ),
    (False, "X_POS", None, vec(0, M), dof(1, 1, 1, 0, 1, 1), 150, 6e-6, RX),
    (False, "X_POS", None, vec(2, -M), dof(1, 1, 1, 1, 1, 0), 150, -6e-6, RZ),
    (False, "Y_POS", None, vec(0, M), dof(1, 1, 1, 0, 1, 1), 150, 6e-6, RX),
    (False, "Z_NEG", None, vec(0, M), dof(1, 1, 1, 0, 1, 1), 150, 6e-6, RX),
]
CASES = FIXED_FREE + FREE_FREE


def kat_world(direction):
    """Two voxels along `direction` (shifted to non-negative lattice indices); returns
    (vxa, index of voxel 1, index of voxel 2)."""
    d = DIRS[direction]
    p1 = np.array([0, 0, 0]) - np.minimum(d, 0)
    p2 = p1 + np.array(d)
    shape = (max(p1[2], p2[2]) + 1, max(p1[1], p2[1]) + 1, max(p1[0], p2[0]) + 1)
    cells = np.zeros(shape, np.int32)
    cells[p1[2], p1[1], p1[0]] = 1
    cells[p2[2], p2[1], p2[0]] = 1
    mat = dict(E=1e6, rho=1e3, nu=0.0, cte=0.0, mus=0.0, muk=0.0)
    vxa = synth.vxa_document(cells, np.zeros(shape), [mat], vox_size=0.001, gravity=0.0, floor=False, collision=False,
                             vary_temp=False, dt_frac=1.0, damping=(1.0, 0.0, 0.2), volume_effects=False)
    lin = lambda p: int(p[0] + shape[2] * (p[1] + shape[1] * p[2]))
    order = sorted([lin(p1), lin(p2)])
    return vxa, order.index(lin(p1)), order.index(lin(p2))


def externals(case, i1, i2):
    fixed1, _, force, moment, dofs, *_ = case
    f = np.array(force or (0, 0, 0), np.float32)
    m = np.array(moment or (0, 0, 0), np.float32)
    e1 = dict(voxel=i1, dof_fixed=0x3F) if fixed1 else dict(voxel=i1, dof_fixed=dofs, force=tuple(-f), moment=tuple(-m))
    e2 = dict(voxel=i2, dof_fixed=dofs, force=tuple(f), moment=tuple(m))
    return [e1, e2]


def rotvec(q):
    """Quat3D::ToRotationVector (Voxelyze3/src/old/Quat3D.h:121-126)."""
    w, x, y, z = q
    if w >= 1.0 or w <= -1.0:
        return np.zeros(3)
    sl = 1.0 - w * w
    if sl < 2.4e-3:
        return np.array([x, y, z]) * 2.0 * math.sqrt((2 - 2 * w) / sl)
    return np.array([x, y, z]) * 2.0 * math.acos(w) / math.sqrt(sl)


def readout(pos, q, nominal, what):
    return (pos - nominal)[what] if what < 3 else rotvec(q)[what - 3]


def converge_steps(step_and_read, limit, expected):
    """tVoxelyze.h:92-104: first step after which 10 consecutive values match."""
    run = 0
    for k in range(1000):
        v = step_and_read()
        if abs(v - expected) < abs(expected) * 1e-5 or np.float32(v) == np.float32(expected):
            run += 1
        else:
            run = 0
        if run == 10:
            return k
    return 1000


def _case_id(c):
    return f"{'fixed' if c[0] else 'free'}-{c[1]}-{['TX', 'TY', 'TZ', 'RX', 'RY', 'RZ'][c[7]]}-{c[6]:g}"


@pytest.mark.parametrize("case", CASES, ids=[_case_id(c) for c in CASES])
def test_kat_oracle(case):
    vxa, i1, i2 = kat_world(case[1])
    d = desc_from_vxa(vxa)
    d["externals"] = externals(case, i1, i2)
    o = OracleSim(d)
    nominal = o.topology()["voxels"][i2, :3] * 0.001

    def step():
        o.step(1)
        st = o.voxel_state()
        return readout(st["pos"][i2], st["orient"][i2], nominal, case[7])

    assert converge_steps(step, case[5], case[6]) < case[5]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[_case_id(c) for c in CASES])
def test_kat_gpu(ctx, case):
    vxa, i1, i2 = kat_world(case[1])
    sim = ctx.load_vxa(vxa, name="kat")
    for e in externals(case, i1, i2):
        ctx.set_external(sim, e["voxel"], e["dof_fixed"], e.get("force", (0, 0, 0)), e.get("moment", (0, 0, 0)))
    nominal = g.inspect_vxa(vxa)["voxels"][i2, :3] * 0.001
    try:
        def step():
            ctx.step(sim, 1, g.PLAIN)
            st = ctx.voxel_state(sim)
            return readout(st["pos"][i2], st["orient"][i2], nominal, case[7])

        assert converge_steps(step, case[5], case[6]) < case[5]
    finally:
        ctx.free(sim)
