"""Seeded synthetic creatures as VXA documents.

No public dataset is involved: the workloads are lattices filled at random
from a seed, reduced to their largest 6-connected component (as the
reference's experiment helper does with scipy.ndimage.label's default
structure, Experiments/framework/voxelyze/helper.py:1-17), with per-voxel
actuation phases written as VXA ``PhaseOffset`` layers in cycles
(Voxelyze3/src/VX3/VX3_VoxelyzeKernel.cu:638-639).
"""
from __future__ import annotations

import math
from collections import deque
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

PASSIVE = dict(E=1e6, rho=1000.0, nu=0.35, cte=0.0, mus=1.0, muk=0.5)
ACTIVE = dict(E=1e6, rho=1000.0, nu=0.35, cte=0.01, mus=1.0, muk=0.5)


def largest_component(cells: np.ndarray) -> np.ndarray:
    """Keeps the largest 6-connected component of a boolean (Z, Y, X) array (the first one in
    raster order among equals): scipy.ndimage.label with its default structure where scipy is
    installed, else a breadth-first search with the same result."""
    try:
        from scipy import ndimage
    except ImportError:
        ndimage = None
    if ndimage is not None:
        lab, n = ndimage.label(cells)
        if n == 0:
            return cells.copy()
        cnt = np.bincount(lab.ravel())
        cnt[0] = 0
        return lab == int(cnt.argmax())
    filled = np.argwhere(cells)
    if len(filled) == 0:
        return cells.copy()
    label = -np.ones(cells.shape, np.int64)
    best, best_n, cur = -1, 0, 0
    Z, Y, X = cells.shape
    for z, y, x in filled:
        if label[z, y, x] >= 0:
            continue
        q = deque([(z, y, x)])
        label[z, y, x] = cur
        n = 0
        while q:
            a, b, c = q.popleft()
            n += 1
            for da, db, dc in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
                na, nb, nc = a + da, b + db, c + dc
                if 0 <= na < Z and 0 <= nb < Y and 0 <= nc < X and cells[na, nb, nc] and label[na, nb, nc] < 0:
                    label[na, nb, nc] = cur
                    q.append((na, nb, nc))
        if n > best_n:
            best, best_n = cur, n
        cur += 1
    return label == best


def _mat_xml(i: int, m: dict) -> str:
    """One palette material; m['mech'] (optional) is extra XML inside <Mechanical> (model, VX3 keys)."""
    mech = m.get("mech", "")
    model = "" if "<MatModel>" in mech else "<MatModel>0</MatModel><Fail_Stress>0</Fail_Stress>"
    return (f"<Material ID=\"{i}\"><MatType>0</MatType><Name>m{i}</Name>"
            f"<Display><Red>0.5</Red><Green>0.5</Green><Blue>0.5</Blue><Alpha>1</Alpha></Display>"
            f"<Mechanical>{model}<Elastic_Mod>{m['E']!r}</Elastic_Mod>"
            f"<Density>{m['rho']!r}</Density><Poissons_Ratio>{m['nu']!r}</Poissons_Ratio><CTE>{m['cte']!r}</CTE>"
            f"<MaterialTempPhase>0</MaterialTempPhase><uStatic>{m['mus']!r}</uStatic><uDynamic>{m['muk']!r}</uDynamic>"
            f"{mech}</Mechanical></Material>")


def _formula_t_gt(t_end: float) -> str:
    return f"<mtSUB><mtVAR>t</mtVAR><mtCONST>{t_end!r}</mtCONST></mtSUB>"


def vxa_document(mat_grid: np.ndarray, phase_grid: np.ndarray, materials: Sequence[dict], *, vox_size=0.01,
                 temp_amplitude=39.0, temp_period=0.2, vary_temp=True, expansion=True, gravity=-9.81, floor=True,
                 collision=False, bounding_radius=0.75, dt_frac=0.95, damping=(1.0, 0.8, 0.01), volume_effects=True,
                 stop_time: Optional[float] = None) -> str:
    """mat_grid: (Z, Y, X) ints, 0 empty, k = materials[k-1]; phase_grid: cycles per cell."""
    Z, Y, X = mat_grid.shape
    if len(materials) > 9:
        raise ValueError("ASCII structure data holds at most 9 materials")
    layers = []
    phases = []
    for z in range(Z):
        layers.append("".join(chr(48 + int(v)) for v in mat_grid[z].reshape(-1)))
        phases.append(",".join(repr(float(p)) for p in phase_grid[z].reshape(-1)))
    stop = f"<StopCondition><StopConditionFormula>{_formula_t_gt(stop_time)}</StopConditionFormula></StopCondition>" if stop_time else ""
    bond, col, slow = damping
    return (
        "<?xml version=\"1.0\" encoding=\"ISO-8859-1\"?>\n<VXA Version=\"1.1\">"
        "<Simulator>"
        f"<EnableExpansion>{1 if expansion else 0}</EnableExpansion>"
        f"<AttachDetach><EnableCollision>{1 if collision else 0}</EnableCollision><EnableAttach>0</EnableAttach>"
        f"<boundingRadius>{bounding_radius!r}</boundingRadius><watchDistance>1</watchDistance></AttachDetach>"
        f"<FitnessFunction><mtVAR>x</mtVAR></FitnessFunction>"
        f"<Integration><Integrator>0</Integrator><DtFrac>{dt_frac!r}</DtFrac></Integration>"
        f"<Damping><BondDampingZ>{bond!r}</BondDampingZ><ColDampingZ>{col!r}</ColDampingZ><SlowDampingZ>{slow!r}</SlowDampingZ></Damping>"
        f"<Collisions><SelfColEnabled>{1 if collision else 0}</SelfColEnabled></Collisions>"
        f"<Features><VolumeEffectsEnabled>{1 if volume_effects else 0}</VolumeEffectsEnabled></Features>"
        f"{stop}"
        "</Simulator>"
        "<Environment><Boundary_Conditions><NumBCs>0</NumBCs></Boundary_Conditions>"
        f"<Gravity><GravEnabled>1</GravEnabled><GravAcc>{gravity!r}</GravAcc><FloorEnabled>{1 if floor else 0}</FloorEnabled></Gravity>"
        f"<Thermal><TempEnabled>1</TempEnabled><TempAmplitude>{temp_amplitude!r}</TempAmplitude><TempBase>25</TempBase>"
        f"<VaryTempEnabled>{1 if vary_temp else 0}</VaryTempEnabled><TempPeriod>{temp_period!r}</TempPeriod></Thermal>"
        "</Environment>"
        f"<VXC Version=\"0.94\"><Lattice><Lattice_Dim>{vox_size!r}</Lattice_Dim></Lattice>"
        "<Palette>" + "".join(_mat_xml(i + 1, m) for i, m in enumerate(materials)) + "</Palette>"
        f"<Structure Compression=\"ASCII_READABLE\"><X_Voxels>{X}</X_Voxels><Y_Voxels>{Y}</Y_Voxels><Z_Voxels>{Z}</Z_Voxels>"
        "<Data>" + "".join(f"<Layer><![CDATA[{l}]]></Layer>" for l in layers) + "</Data>"
        "<PhaseOffset>" + "".join(f"<Layer><![CDATA[{p}]]></Layer>" for p in phases) + "</PhaseOffset>"
        "</Structure></VXC></VXA>\n")


@dataclass
class Creature:
    vxa: str
    num_voxel: int
    shape: Tuple[int, int, int]
    seed: int
    meta: dict = field(default_factory=dict)


def random_creature(seed: int, side: Sequence[int] = (10, 10, 10), fill: float = 0.6,
                    materials: Sequence[dict] = (PASSIVE, ACTIVE), material_p: Optional[Sequence[float]] = None,
                    keep_largest: bool = True, **kw) -> Creature:
    """A seeded random creature (std of the reference experiments: fill, keep the largest component)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = side
    cells = rng.random((Z, Y, X)) < fill
    if keep_largest:
        cells = largest_component(cells)
    mats = rng.choice(len(materials), size=(Z, Y, X), p=material_p) + 1
    grid = np.where(cells, mats, 0).astype(np.int32)
    phase = rng.random((Z, Y, X)) * 2 * math.pi / (2 * math.pi)   # phi in [0, 2pi) written in cycles
    return Creature(vxa_document(grid, phase, materials, **kw), int(cells.sum()), (X, Y, Z), seed,
                    dict(fill=fill, materials=list(materials)))


def config0_creature(seed: int = 0, **kw) -> Creature:
    """Plain single creature: 10x10x10, fill 0.6, passive + active material, 0.01 m voxels."""
    return random_creature(seed, (10, 10, 10), 0.6, (PASSIVE, ACTIVE), **kw)


def config1_batch(n: int = 512, seed: int = 1, sim_time: float = 0.5, **kw) -> List[Creature]:
    """Batched plain physics: side U{6..20}, fill U(0.3, 0.9), four materials with E log-uniform in
    [1e5, 1e7] (one or two actuated), rho=1000, nu=0.35."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        s = int(rng.integers(6, 21))
        fill = float(rng.uniform(0.3, 0.9))
        mats = config1_materials(rng)
        out.append(random_creature(int(rng.integers(1 << 31)), (s, s, s), fill, mats, stop_time=sim_time, **kw))
    return out


def config2_batch(n: int = 64, seed: int = 2, **kw) -> List[Creature]:
    """Collision-heavy: 40^3 at fill 0.5, three materials including a soft one (E=1e5), self-collision on."""
    rng = np.random.default_rng(seed)
    mats = [dict(E=1e5, rho=1000.0, nu=0.35, cte=0.01, mus=1.0, muk=0.5),
            dict(E=1e6, rho=1000.0, nu=0.35, cte=0.01, mus=1.0, muk=0.5),
            dict(E=1e6, rho=1000.0, nu=0.35, cte=0.0, mus=1.0, muk=0.5)]
    kw.setdefault("expansion", False)
    return [random_creature(int(rng.integers(1 << 31)), (40, 40, 40), 0.5, mats, collision=True, **kw) for _ in range(n)]


def config1_materials(rng) -> List[dict]:
    """Four materials with E log-uniform in [1e5, 1e7] Pa, rho=1000, nu=0.35; the first one or
    two actuated (CTE 0.01), as in the batched configuration."""
    Es = 10 ** rng.uniform(5, 7, size=4)
    n_act = int(rng.integers(1, 3))
    return [dict(E=float(E), rho=1000.0, nu=0.35, cte=(0.01 if k < n_act else 0.0), mus=1.0, muk=0.5) for k, E in enumerate(Es)]


def serving_requests(n: int = 64, seed: int = 4, v_range=(100, 100000), horizon_range=(1000, 50000),
                     collide_frac: float = 0.2, fill_range=(0.5, 0.9)) -> List[tuple]:
    """Serving requests: (creature, horizon_steps).  The target voxel count is log-uniform in
    v_range and sets a cubic lattice's side from the fill; materials as in the batched
    configuration; the horizon is uniform in horizon_range; a fraction has self-collision on
    (with contraction-only actuation).  The fill is drawn from U(0.5, 0.9) rather than the batch's
    U(0.3, 0.9): below the cubic lattice's percolation threshold (about 0.31) the largest
    component holds a vanishing share of the cells and the voxel count could not follow its draw."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        v = math.exp(rng.uniform(math.log(v_range[0]), math.log(v_range[1])))
        fill = float(rng.uniform(*fill_range))
        s = max(2, int(round((v / fill) ** (1.0 / 3.0))))
        collide = bool(rng.random() < collide_frac)
        kw = dict(collision=True, expansion=False) if collide else {}
        mats = config1_materials(rng)
        c = random_creature(int(rng.integers(1 << 31)), (s, s, s), fill, mats, **kw)
        c.meta["collide"] = collide
        out.append((c, int(rng.integers(horizon_range[0], horizon_range[1] + 1))))
    return out


def slab(X: int = 200, Y: int = 200, Z: int = 100, seed: int = 3, **kw) -> Creature:
    """Single large body: a solid X x Y x Z slab of one actuated material (E=1e6), random phases."""
    rng = np.random.default_rng(seed)
    grid = np.ones((Z, Y, X), np.int32)
    phase = rng.random((Z, Y, X))
    mat = dict(E=1e6, rho=1000.0, nu=0.35, cte=0.01, mus=1.0, muk=0.5)
    return Creature(vxa_document(grid, phase, [mat], **kw), X * Y * Z, (X, Y, Z), seed)
