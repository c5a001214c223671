"""CPU restatement of the VX3 extras that have no counterpart in the reference's CPU
path: voxel signals, target closeness and run-time attachment of touching voxels.
TEST INFRASTRUCTURE: only the tests use it, as the checker of the engine's results.

Signals follow VX3_Voxel's signal routines (Voxelyze3/src/VX3/VX3_Voxel.cu:271-347).
The reference runs them inside the parallel voxel kernel and writes into the
neighbours' signal state from the sending thread while those neighbours run their
own step, so its outcome depends on thread timing.  The engine (and this restatement)
fixes one order: every voxel first does its own signal work of the step (relay a
due signal, pacemaker pulse, local decay, in the reference's order), then each voxel
takes the signals its linked neighbours relayed, in link-direction order X+, X-, Y+,
Y-, Z+, Z-.  A forced signal from touching a target voxel is taken before the step.

Attachment is likewise racy in the reference (many threads create links at once);
the engine and this restatement create them one pair at a time in increasing pair
order.

Pinning: the reference's GPU code does not build with this toolchain and its CPU path
has neither feature, so this restatement is pinned to VX3's source text, not to outputs.
"""
import math

# per-voxel fields, in the engine's read-back order (vx3_get_extras signals6)
LOCAL, LOCAL_DT, INACTIVE, VALUE, ACTIVE, PULSE = range(6)


class SignalNet:
    """Signal state of one simulation.

    nbrs[v][d]: neighbour voxel across direction d (X+, X-, Y+, Y-, Z+, Z-) or -1.
    mats: list of dicts with keys pacemaker (bool), period, decay, delay, inactive.
    mat_of[v]: material index of voxel v.  frozen[v]: the voxel runs no own signal
    step (fixed in every degree of freedom, of a Fixed material, or removed)."""

    def __init__(self, nbrs, mats, mat_of, frozen=None):
        self.nbrs = [list(n) for n in nbrs]
        self.mats = mats
        self.mat_of = list(mat_of)
        n = len(self.mat_of)
        self.frozen = list(frozen) if frozen is not None else [False] * n
        self.s = [[0.0] * 6 for _ in range(n)]
        self.out = [0.0] * n
        self.out_t = [0.0] * n

    # VX3_Voxel::receiveSignal, VX3_Voxel.cu:301-322
    def receive(self, v, value, active, force):
        s = self.s[v]
        m = self.mats[self.mat_of[v]]
        if not force and s[INACTIVE] > active:
            return
        if value < 0.1:
            return
        s[INACTIVE] = active + m["inactive"]
        s[LOCAL] = value
        relay = value * m["decay"]
        if relay < 0.1:
            relay = 0.0
        s[VALUE] = relay
        s[ACTIVE] = active

    # VX3_Voxel::timeStep's signal part, VX3_Voxel.cu:271-276
    def own_step(self, v, t):
        s = self.s[v]
        m = self.mats[self.mat_of[v]]
        out = out_t = 0.0
        # propagateSignal, VX3_Voxel.cu:323-347 (the sending half)
        if not (s[ACTIVE] > t) and not (s[VALUE] < 0.1):
            out = s[VALUE]
            out_t = t + m["delay"]
            s[VALUE] = 0.0
            s[ACTIVE] = 0.0
            s[INACTIVE] = t + 2 * m["delay"] + m["inactive"]
        self.out[v] = out
        self.out_t[v] = out_t
        # packMaker, VX3_Voxel.cu:291-299
        if m["pacemaker"] and not (s[PULSE] > t):
            self.receive(v, 100.0, t, True)
            s[PULSE] = t + m["period"]
        # localSignalDecay, VX3_Voxel.cu:279-289
        if not (s[LOCAL_DT] > t):
            if s[LOCAL] < 0.1:
                s[LOCAL] = 0.0
            else:
                s[LOCAL] = s[LOCAL] * 0.9
                s[LOCAL_DT] = t + 0.01

    def step(self, t, hits=()):
        """One time step that starts at time t; hits: non-target voxels touching a target."""
        for v in hits:
            self.receive(v, 100.0, t, True)
        for v in range(len(self.s)):
            if self.frozen[v]:
                self.out[v] = 0.0
            else:
                self.own_step(v, t)
        for v in range(len(self.s)):
            for d in range(6):
                u = self.nbrs[v][d]
                if u >= 0 and self.out[u] > 0:
                    self.receive(v, self.out[u], self.out_t[u], False)

    def state(self):
        return [list(x) for x in self.s]


def target_closeness(pos, targets, max_dist_voxels, vox_size):
    """VX3_VoxelyzeKernel::computeTargetCloseness (VX3_VoxelyzeKernel.cu:545-563): pairs of
    target voxels closer than MaxDistInVoxelLengthsToCountAsPair voxel sizes, and the sum of
    their inverse distances, in index order."""
    if max_dist_voxels == 0:
        return 0.0, 0
    R = max_dist_voxels * vox_size
    ret = 0.0
    pairs = 0
    for i in range(len(targets)):
        a = pos[targets[i]]
        for j in range(i + 1, len(targets)):
            b = pos[targets[j]]
            dx, dy, dz = float(b[0]) - float(a[0]), float(b[1]) - float(a[1]), float(b[2]) - float(a[2])
            dist = math.sqrt(dx * dx + dy * dy + dz * dz)
            if dist < R:
                pairs += 1
            ret += 1 / dist
    return ret, pairs


def _qrotinv(q, f):
    """Quat3D::RotateVec3DInv (Voxelyze3/src/old/Quat3D.h:192-199); q = (w, x, y, z)."""
    w, x, y, z = (float(c) for c in q)
    fx, fy, fz = (float(c) for c in f)
    tw = x * fx + y * fy + z * fz
    tx = w * fx - y * fz + z * fy
    ty = w * fy + x * fz - z * fx
    tz = w * fz - x * fy + y * fx
    return (tw * x + tx * w + ty * z - tz * y, tw * y - tx * z + ty * w + tz * x, tw * z + tx * y - ty * x + tz * w)


def attach_links(pos, orient, links, pairs, n_voxels):
    """New links VX3 attachment makes in one step (handle_collision_attachment,
    Voxelyze3/src/VX3/VX3_VoxelyzeKernel.cu:729-827), in the engine's deterministic order.

    links: current links as (neg, pos, axis) rows (gone links left out); pairs: candidate
    pairs (a < b) that touch and pass the material tests.  Returns the new links as
    (neg, pos, axis) in creation order; `links` is not modified."""
    slot = [[-1] * 6 for _ in range(n_voxels)]
    lk = [list(map(int, l)) for l in links]
    for i, (n, p, ax) in enumerate(lk):
        slot[n][2 * ax] = i
        slot[p][2 * ax + 1] = i

    def within(a, b, depth):
        # is_neighbor (VX3_VoxelyzeKernel.cu:651-680)
        def rec(v, incoming, d):
            if v == b:
                return True
            if d <= 0:
                return False
            for k in range(6):
                l = slot[v][k]
                if l >= 0 and l != incoming:
                    n, p, _ = lk[l]
                    if rec(p if n == v else n, l, d - 1):
                        return True
            return False
        return rec(a, -1, depth)

    made = []
    for a, b in sorted(pairs):
        v1, v2 = b, a                                   # voxel1: the later voxel of the pair
        if within(v1, v2, 5):
            continue
        e = [float(pos[v1][k]) - float(pos[v2][k]) for k in range(3)]
        ea = _qrotinv(orient[v1], (-e[0], -e[1], -e[2]))
        f = [abs(c) for c in ea]
        if f[0] >= f[1] and f[0] >= f[2]:
            axis = 0
        elif f[1] >= f[0] and f[1] >= f[2]:
            axis = 1
        else:
            axis = 2
        reverse = ea[axis] < 0
        vneg, vpos = (v2, v1) if reverse else (v1, v2)
        if slot[vneg][2 * axis] >= 0 or slot[vpos][2 * axis + 1] >= 0:
            continue
        lk.append([vneg, vpos, axis])
        slot[vneg][2 * axis] = len(lk) - 1
        slot[vpos][2 * axis + 1] = len(lk) - 1
        made.append((vneg, vpos, axis))
    return made
