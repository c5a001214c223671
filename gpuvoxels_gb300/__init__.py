"""gpuvoxels_gb300: GB300-native Voxelyze3 soft-body step engine.

Python mirror of the reference's simulation interface over the C ABI
(include/gpuvoxels_gb300.h):

* ``SimulationManager`` mirrors ``VX3_SimulationManager`` (Voxelyze3/src/VX3/
  VX3_SimulationManager.cuh:15-46): a base VXA plus VXD files in, ``start()``
  runs them all and fills ``h_results`` sorted by fitness (NaN last).
* ``Context`` exposes every entry point: load, step/run (plain or batched),
  the serving pair submit/poll, state readout, the report writer.

The compute path is the CUDA library built by ``gpuvoxels_gb300.build``; there
is no CPU fallback.  Loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Iterable, List, Optional, Sequence

import numpy as np

from . import build as _build

PLAIN, BATCHED = 0, 1
SERVE_FCFS, SERVE_LEAST_WORK, SERVE_LONG_LANE = 0, 1, 2
EXACT, FMA = 0, 1
SIM_IDLE, SIM_RUNNING, SIM_DONE, SIM_DIVERGED, SIM_ERROR = range(5)
ERRORS = {-1: "VX3_E_PARSE", -2: "VX3_E_OOM_BUDGET", -3: "VX3_E_DIVERGED", -4: "VX3_E_TIMEOUT", -5: "VX3_E_CUDA",
          -6: "VX3_E_ARG", -7: "VX3_E_STATE"}

# Every symbol include/gpuvoxels_gb300.h declares.
EXPORTS = ["vx3_create", "vx3_destroy", "vx3_last_error", "vx3_load_vxa", "vx3_set_external", "vx3_run", "vx3_step",
           "vx3_submit", "vx3_poll", "vx3_pending", "vx3_get_result", "vx3_sim_info_get", "vx3_sim_sizes", "vx3_get_state",
           "vx3_get_voxel_state", "vx3_get_link_state", "vx3_write_report", "vx3_free_sim", "vx3_last_timing",
           "vx3_set_tuning", "vx3_autotune", "vx3_set_profiling", "vx3_set_precision", "vx3_sim_bytes", "vx3_bytes_in_use",
           "vx3_inspect_vxa", "vx3_inspect_topology", "vx3_inspect_formula", "vx3_center_of_mass_noalloc",
           "vx3_write_report_multi", "vx3_load_vxa_many", "vx3_record_history", "vx3_inspect_externals", "vx3_get_states",
           "vx3_get_extras", "vx3_get_links", "vx3_transfer_bytes", "vx3_set_claim_sizes", "vx3_get_tuning",
           "vx3_set_contact_slots", "vx3_eval_formula", "vx3_set_serving"]
NOALLOC_MAX_POINTS = 4194304
E_LIMIT = -8


class VX3Error(RuntimeError):
    pass


class Result(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("status", ctypes.c_int32), ("num_voxel", ctypes.c_int32),
                ("num_measured_voxel", ctypes.c_int32), ("num_close_pairs", ctypes.c_int32), ("steps", ctypes.c_int64),
                ("current_time", ctypes.c_double), ("fitness_score", ctypes.c_double), ("vox_size", ctypes.c_double),
                ("initial_center_of_mass", ctypes.c_double * 3), ("current_center_of_mass", ctypes.c_double * 3),
                ("total_distance_of_all_voxels", ctypes.c_double), ("submit_time_s", ctypes.c_double),
                ("start_time_s", ctypes.c_double), ("finish_time_s", ctypes.c_double)]


class SimInfo(ctypes.Structure):
    _fields_ = [("num_voxel", ctypes.c_int32), ("num_link", ctypes.c_int32), ("status", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("dt", ctypes.c_double), ("current_time", ctypes.c_double),
                ("steps", ctypes.c_int64)]


_LIB = None


def library(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads (building first if needed) the in-tree CUDA library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing and (not os.path.exists(path) or _build.needs_build()):
        _build.build()
    if not os.path.exists(path):
        raise VX3Error(f"CUDA engine library not built: {path}")
    L = ctypes.CDLL(path)
    P, I, I64, D, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_char_p
    sig = {
        "vx3_create": (P, [I, ctypes.c_size_t]), "vx3_destroy": (None, [P]), "vx3_last_error": (S, [P]),
        "vx3_load_vxa": (I, [P, S, S, S, ctypes.POINTER(I64)]),
        "vx3_set_external": (I, [P, I64, I, I, P, P, P, P]),
        "vx3_run": (I, [P, P, I, I, I64]), "vx3_step": (I, [P, P, I, I, I64]),
        "vx3_submit": (I, [P, I64, I64]), "vx3_poll": (I, [P, P, I, I]), "vx3_pending": (I, [P]),
        "vx3_get_result": (I, [P, I64, ctypes.POINTER(Result)]), "vx3_sim_info_get": (I, [P, I64, ctypes.POINTER(SimInfo)]),
        "vx3_sim_sizes": (I, [P, P, I, P, P]),
        "vx3_get_state": (I, [P, I64, P, P, P]), "vx3_get_voxel_state": (I, [P, I64, P, P, P]),
        "vx3_get_link_state": (I, [P, I64, P, P, P]), "vx3_write_report": (I, [P, P, I, S, S]),
        "vx3_free_sim": (I, [P, I64]), "vx3_last_timing": (I, [P, P]), "vx3_set_tuning": (I, [P, I, I, I, I, I]),
        "vx3_autotune": (I, [P, P, I]), "vx3_set_claim_sizes": (I, [P, I, I]), "vx3_get_tuning": (I, [P, P]),
        "vx3_set_contact_slots": (I, [P, I]), "vx3_set_serving": (I, [P, I, I64]), "vx3_eval_formula": (I, [P, S, S, I, P, I, P]), "vx3_set_profiling": (I, [P, I]), "vx3_set_precision": (I, [P, I]), "vx3_sim_bytes": (I64, [P, I64]),
        "vx3_bytes_in_use": (ctypes.c_size_t, [P]),
        "vx3_inspect_vxa": (I, [S, S, P, P, ctypes.c_char_p, I]),
        "vx3_inspect_topology": (I, [S, S, P, P, P, P, P, P, P]),
        "vx3_inspect_formula": (I, [S, S, I, P, P]),
        "vx3_center_of_mass_noalloc": (I, [P, P, P, P, I64, P, P]),
        "vx3_write_report_multi": (I, [P, P, P, I, S, S]),
        "vx3_load_vxa_many": (I, [P, S, P, P, I, P, P]),
        "vx3_record_history": (I, [P, I64, S]),
        "vx3_inspect_externals": (I, [S, S, P, P, P]),
        "vx3_get_states": (I, [P, P, I, P, P, P]),
        "vx3_get_extras": (I, [P, I64, P, P]),
        "vx3_get_links": (I, [P, I64, P, P, I]),
        "vx3_transfer_bytes": (I, [P, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _b(s: Optional[str]):
    return None if s is None else s.encode()


def inspect_vxa(base_xml: str, vxd_xml: Optional[str] = None) -> dict:
    """Host-only: what the engine would simulate for this VXA/VXD (no GPU needed)."""
    L = library()
    counts = np.zeros(6, np.int32)
    env = np.zeros(12)
    err = ctypes.create_string_buffer(512)
    rc = L.vx3_inspect_vxa(_b(base_xml), _b(vxd_xml), _p(counts), _p(env), err, 512)
    if rc:
        raise VX3Error(f"{ERRORS.get(rc, rc)}: {err.value.decode()}")
    nv, nl, nvm, nlm = (int(x) for x in counts[:4])
    vox = np.zeros((nv, 4), np.int32); lnk = np.zeros((max(nl, 1), 4), np.int32); ph = np.zeros(nv)
    vm = np.zeros((nvm, 18), np.float32); vnom = np.zeros(nvm); lidx = np.zeros((max(nlm, 1), 2), np.int32)
    lm = np.zeros((max(nlm, 1), 20), np.float32)
    L.vx3_inspect_topology(_b(base_xml), _b(vxd_xml), _p(vox), _p(lnk), _p(ph), _p(vm), _p(vnom), _p(lidx), _p(lm))
    keys = ["vox_size", "dt_frac", "gravity_mult", "floor", "collisions", "vary_temp", "temp_amplitude", "temp_period",
            "enable_expansion", "initial_temp", "bounding_radius", "watch_distance"]
    return dict(counts=dict(voxels=nv, links=nl, voxel_materials=nvm, link_materials=nlm, surface=int(counts[4]),
                            externals=int(counts[5])),
                env=dict(zip(keys, env.tolist())), voxels=vox, links=lnk[:nl], phase=ph, voxmat=vm, nom=vnom,
                linkmat_idx=lidx[:nlm], linkmat=lm[:nlm])


def inspect_externals(base_xml: str, vxd_xml: Optional[str] = None) -> dict:
    """Host-only: per-voxel externals from the VXA's boundary-condition regions."""
    L = library()
    nv = inspect_vxa(base_xml, vxd_xml)["counts"]["voxels"]
    dof = np.zeros(nv, np.int32); fm = np.zeros((nv, 6), np.float32); tr = np.zeros((nv, 6))
    rc = L.vx3_inspect_externals(_b(base_xml), _b(vxd_xml), _p(dof), _p(fm), _p(tr))
    if rc:
        raise VX3Error(ERRORS.get(rc, str(rc)))
    return dict(dof=dof, force=fm[:, :3], moment=fm[:, 3:], translate=tr[:, :3], rotate=tr[:, 3:])


def eval_formula(base_xml: str, which: str, vars9: Sequence[float], vxd_xml: Optional[str] = None) -> float:
    L = library()
    v = np.asarray(vars9, np.float64)
    out = np.zeros(1)
    rc = L.vx3_inspect_formula(_b(base_xml), _b(vxd_xml), 0 if which == "stop" else 1, _p(v), _p(out))
    if rc:
        raise VX3Error(ERRORS.get(rc, str(rc)))
    return float(out[0])


class Context:
    """One device context: an HBM budget, a stream, and the simulations loaded into it."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.L = library()
        self.h = self.L.vx3_create(device, hbm_budget_bytes)
        if not self.h:
            raise VX3Error("vx3_create failed (no CUDA device, or the budget could not be reserved)")
        self.names = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.vx3_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc < 0:
            raise VX3Error(f"{ERRORS.get(rc, rc)}: {self.L.vx3_last_error(self.h).decode()}")
        return rc

    def load_vxa(self, base_xml: str, vxd_xml: Optional[str] = None, name: str = "") -> int:
        out = ctypes.c_int64()
        self._check(self.L.vx3_load_vxa(self.h, _b(base_xml), _b(vxd_xml), name.encode(), ctypes.byref(out)))
        self.names[out.value] = name
        return out.value

    def load_many(self, docs: Sequence, base: Optional[str] = None, names: Optional[Sequence[str]] = None) -> List[int]:
        """Loads many simulations, parsed and built on host threads: each of `docs` (str, or the
        file's bytes as read) is a VXD merged into `base`, or a whole VXA when `base` is None."""
        n = len(docs)
        names = list(names) if names is not None else [""] * n
        enc = [d if isinstance(d, bytes) else d.encode() for d in docs]
        cdocs = (ctypes.c_char_p * n)(*enc)
        cnames = (ctypes.c_char_p * n)(*[s.encode() for s in names])
        ids = np.full(n, -1, np.int64)
        st = np.zeros(n, np.int32)
        self._check(self.L.vx3_load_vxa_many(self.h, _b(base), ctypes.cast(cdocs, ctypes.c_void_p),
                                             ctypes.cast(cnames, ctypes.c_void_p), n, _p(ids), _p(st)))
        out = [int(i) for i in ids]
        for i, nm in zip(out, names):
            self.names[i] = nm
        return out

    def record_history(self, sim: int, path: Optional[str]):
        """Writes the simulation's .history stream to `path` during later step/run calls (None stops)."""
        self._check(self.L.vx3_record_history(self.h, sim, _b(path)))

    def set_external(self, sim: int, voxel: int, dof_fixed: int = 0, force=(0, 0, 0), moment=(0, 0, 0),
                     translate=(0, 0, 0), rotate=(0, 0, 0)):
        f = np.asarray(force, np.float32); m = np.asarray(moment, np.float32)
        t = np.asarray(translate, np.float64); r = np.asarray(rotate, np.float64)
        self._check(self.L.vx3_set_external(self.h, sim, voxel, dof_fixed, _p(f), _p(m), _p(t), _p(r)))

    def _ids(self, ids):
        a = np.ascontiguousarray(np.atleast_1d(np.asarray(ids, np.int64)))
        return a

    def step(self, ids, steps: int, mode: int = BATCHED):
        a = self._ids(ids)
        self._check(self.L.vx3_step(self.h, _p(a), len(a), mode, steps))

    def run(self, ids, mode: int = BATCHED, max_steps: int = 0):
        a = self._ids(ids)
        self._check(self.L.vx3_run(self.h, _p(a), len(a), mode, max_steps))

    def submit(self, sim: int, horizon_steps: int):
        self._check(self.L.vx3_submit(self.h, sim, horizon_steps))

    def poll(self, chunk_steps: int = 64, max_results: int = 4096) -> List[Result]:
        buf = (Result * max_results)()
        n = self._check(self.L.vx3_poll(self.h, buf, max_results, chunk_steps))
        return [buf[i] for i in range(n)]

    def pending(self) -> int:
        return self.L.vx3_pending(self.h)

    def result(self, sim: int) -> Result:
        r = Result()
        self._check(self.L.vx3_get_result(self.h, sim, ctypes.byref(r)))
        return r

    def sizes(self, ids):
        """(voxel counts, link counts) of many simulations, without reading the device."""
        a = self._ids(ids)
        nv = np.zeros(len(a), np.int32); nl = np.zeros(len(a), np.int32)
        self._check(self.L.vx3_sim_sizes(self.h, _p(a), len(a), _p(nv), _p(nl)))
        return nv, nl

    def info(self, sim: int) -> SimInfo:
        r = SimInfo()
        self._check(self.L.vx3_sim_info_get(self.h, sim, ctypes.byref(r)))
        return r

    def voxel_state(self, sim: int) -> dict:
        nv = self.info(sim).num_voxel
        d = np.zeros((nv, 13)); f = np.zeros((nv, 4), np.float32); fl = np.zeros(nv, np.int32)
        self._check(self.L.vx3_get_voxel_state(self.h, sim, _p(d), _p(f), _p(fl)))
        return dict(pos=d[:, 0:3], linMom=d[:, 3:6], orient=d[:, 6:10], angMom=d[:, 10:13], temp=f[:, 0],
                    pStrain=f[:, 1:4], flags=fl)

    def link_state(self, sim: int) -> dict:
        nl = self.info(sim).num_link
        d = np.zeros((nl, 9)); f = np.zeros((nl, 3), np.float32); fl = np.zeros(nl, np.int32)
        self._check(self.L.vx3_get_link_state(self.h, sim, _p(d), _p(f), _p(fl)))
        return dict(pos2=d[:, 0:3], angle1v=d[:, 3:6], angle2v=d[:, 6:9], strain=f[:, 0], maxStrain=f[:, 1],
                    strainOffset=f[:, 2], smallAngle=fl & 1, flags=fl)

    def extras(self, sim: int) -> dict:
        """VX3 extras: targetCloseness, numClosePairs, collisionCount, recentAngle and the per-voxel
        signal state (localSignal, localSignaldt, inactiveUntil, pending value and time, next pulse)."""
        nv = self.info(sim).num_voxel
        m = np.zeros(4); g = np.zeros((nv, 6))
        self._check(self.L.vx3_get_extras(self.h, sim, _p(m), _p(g)))
        return dict(targetCloseness=m[0], numClosePairs=int(m[1]), collisionCount=int(m[2]), recentAngle=m[3],
                    localSignal=g[:, 0], localSignalDt=g[:, 1], inactiveUntil=g[:, 2], signalValue=g[:, 3],
                    signalTime=g[:, 4], pacemakerNextPulse=g[:, 5])

    def links(self, sim: int) -> np.ndarray:
        """Every link in use (loaded, then made by VX3 attachment): rows of negative end,
        positive end, axis, flags."""
        n = np.zeros(1, np.int32)
        self._check(self.L.vx3_get_links(self.h, sim, _p(n), None, 0))
        out = np.zeros((max(int(n[0]), 1), 4), np.int32)
        self._check(self.L.vx3_get_links(self.h, sim, _p(n), _p(out), int(n[0])))
        return out[:int(n[0])]

    def get_state(self, sim: int):
        nv = self.info(sim).num_voxel
        pos = np.zeros((nv, 3)); q = np.zeros((nv, 4)); fl = np.zeros(nv, np.uint8)
        self._check(self.L.vx3_get_state(self.h, sim, _p(pos), _p(q), _p(fl)))
        return pos, q, fl

    def get_states(self, ids):
        """Poses of many simulations in one device pass: (pos, orient, flags, offsets) with the
        simulations' voxels one after another; simulation k owns rows offsets[k]:offsets[k+1]."""
        a = self._ids(ids)
        counts = self.sizes(a)[0]
        offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        tot = int(offsets[-1])
        pos = np.zeros((tot, 3)); q = np.zeros((tot, 4)); fl = np.zeros(tot, np.uint8)
        self._check(self.L.vx3_get_states(self.h, _p(a), len(a), _p(pos), _p(q), _p(fl)))
        return pos, q, fl, offsets

    def write_report(self, ids, path: str, input_dir: str = ""):
        a = self._ids(ids)
        self._check(self.L.vx3_write_report(self.h, _p(a), len(a), input_dir.encode(), path.encode()))

    def free(self, sim: int):
        self._check(self.L.vx3_free_sim(self.h, sim))

    def timing(self) -> dict:
        o = np.zeros(7)
        self.L.vx3_last_timing(self.h, _p(o))
        return dict(device_ms=o[0], wall_ms=o[1], voxel_steps=int(o[2]), launches=int(o[3]), link_ms=o[4],
                    contact_ms=o[5], voxel_ms=o[6])

    def transfer_bytes(self):
        """(host->device, device->host) bytes this context has copied so far."""
        h = np.zeros(1, np.int64); d = np.zeros(1, np.int64)
        self._check(self.L.vx3_transfer_bytes(self.h, _p(h), _p(d)))
        return int(h[0]), int(d[0])

    def set_tuning(self, block_links=0, block_voxels=0, items_links=0, items_voxels=0, graph_steps=0):
        self.L.vx3_set_tuning(self.h, block_links, block_voxels, items_links, items_voxels, graph_steps)

    def set_serving(self, order: int = 0, max_active_voxels: int = 0):
        """Admission policy of poll(): order 0 first come first served, 1 least voxels x horizon first,
        2 least work first beside one lane that takes the queued request with the most work whenever
        it is free; max_active_voxels caps the running batch (0 = the HBM budget decides; the lane's
        request is not counted)."""
        self._check(self.L.vx3_set_serving(self.h, order, max_active_voxels))

    def set_claim_sizes(self, claim_links=0, claim_voxels=0):
        self._check(self.L.vx3_set_claim_sizes(self.h, claim_links, claim_voxels))

    def set_contact_slots(self, slots):
        """Contacts kept in each voxel's own slots for simulations uploaded afterwards (1..16)."""
        self._check(self.L.vx3_set_contact_slots(self.h, slots))

    def tuning(self):
        """The launch shape in use (vx3_get_tuning)."""
        out = np.zeros(8, np.int32)
        self._check(self.L.vx3_get_tuning(self.h, _p(out)))
        keys = ("block_links", "block_voxels", "items_links", "items_voxels", "graph_steps", "claim_links", "claim_voxels",
                "contact_slots")
        return {k: int(v) for k, v in zip(keys, out)}

    def eval_formula(self, base_xml: str, which: str, vars9, vxd_xml: Optional[str] = None) -> np.ndarray:
        """A formula of the VXA evaluated on the device for each row of vars9 (n x 9):
        which = 'stop', 'fitness', 'force_x', 'force_y' or 'force_z'."""
        w = {"stop": 0, "fitness": 1, "force_x": 2, "force_y": 3, "force_z": 4}[which]
        v = np.ascontiguousarray(vars9, np.float64).reshape(-1, 9)
        out = np.zeros(len(v))
        self._check(self.L.vx3_eval_formula(self.h, _b(base_xml), _b(vxd_xml), w, _p(v), len(v), _p(out)))
        return out

    def autotune(self, ids):
        a = self._ids(ids)
        self._check(self.L.vx3_autotune(self.h, _p(a), len(a)))

    def set_profiling(self, on: bool):
        self.L.vx3_set_profiling(self.h, int(on))

    def set_precision(self, mode: int):
        """EXACT (default, the reference's rounding) or FMA (contracted multiply-adds)."""
        self._check(self.L.vx3_set_precision(self.h, mode))

    def sim_bytes(self, sim: int) -> int:
        return self._check(self.L.vx3_sim_bytes(self.h, sim))

    def bytes_in_use(self) -> int:
        return int(self.L.vx3_bytes_in_use(self.h))


@dataclass
class SimulationResult:
    """VX3_SimulationResult (Voxelyze3/src/VX3/VX3_SimulationResult.h:4-33)."""
    vxa_filename: str
    fitness_score: float
    currentTime: float
    num_voxel: int
    num_measured_voxel: int
    voxSize: float
    numClosePairs: int
    initialCenterOfMass: tuple
    currentCenterOfMass: tuple
    total_distance_of_all_voxels: float
    status: int


class SimulationManager:
    """Mirror of VX3_SimulationManager(sub_batches, base, input_dir, nDevices).start()
    (Voxelyze3/src/VX3/VX3_SimulationManager.cu:123-155, 416-460) on one GB300."""

    def __init__(self, sub_batches: Sequence[Sequence[str]], base: str, input_dir: str, num_of_devices: int = 1,
                 mode: int = BATCHED, hbm_budget_bytes: int = 0):
        self.files = [f for batch in sub_batches for f in batch]
        self.base = base
        self.input_dir = input_dir
        self.mode = mode
        self.budget = hbm_budget_bytes
        self.h_results: List[SimulationResult] = []
        self.ctx: Optional[Context] = None
        self.ids: List[int] = []

    def start(self):
        base_xml = open(self.base).read()
        self.ctx = Context(0, self.budget)
        vxds = []
        for f in self.files:
            with open(os.path.join(self.input_dir, f)) as fh:
                vxds.append(fh.read())
        self.ids = self.ctx.load_many(vxds, base=base_xml, names=[os.path.basename(f) for f in self.files])
        self.ctx.run(self.ids, self.mode)
        res = []
        for f, i in zip(self.files, self.ids):
            r = self.ctx.result(i)
            res.append(SimulationResult(os.path.basename(f), r.fitness_score, r.current_time, r.num_voxel,
                                        r.num_measured_voxel, r.vox_size, r.num_close_pairs,
                                        tuple(r.initial_center_of_mass), tuple(r.current_center_of_mass),
                                        r.total_distance_of_all_voxels, r.status))
        nan = [r for r in res if r.fitness_score != r.fitness_score]
        ok = sorted([r for r in res if r.fitness_score == r.fitness_score], key=lambda r: -r.fitness_score)
        self.h_results = ok + nan
        return self.h_results

    def write_report(self, path: str):
        self.ctx.write_report(self.ids, path, self.input_dir)
