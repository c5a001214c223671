"""CPU oracle bindings: TEST INFRASTRUCTURE ONLY.

* ``desc_from_vxa`` restates, in Python, how the reference turns a merged VXA
  document into a simulation (Voxelyze3/src/VXA/VX_Sim.cpp:59-153, 185-258,
  368-420; Voxelyze3/src/old/VX_Environment.cpp:101-175;
  Voxelyze3/src/VXA/VX_Object.cpp:446-500, 1373-1460, 1760-1860) and the VX3
  keys read by Voxelyze3/src/VX3/VX3_SimulationManager.cu:326-367.
* ``merge_vxd`` restates the VXD override rule of Voxelyze3/src/Utils/ctool.h:49-57.
* ``OracleSim`` drives the C restatement (oracle/vx_oracle.c).
* ``RefSim`` drives the reference's own CPU Voxelyze (oracle/_ref), which only
  exists where the reference sources were available to compile.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module; the product never does.
"""
from __future__ import annotations

import copy
import ctypes
import math
import os
import subprocess
import xml.etree.ElementTree as ET

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libvxref.so")

_MAXD = 16


class _Mat(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("E", ctypes.c_float), ("plastic_mod", ctypes.c_float),
                ("yield_stress", ctypes.c_float), ("fail_stress", ctypes.c_float), ("ndata", ctypes.c_int),
                ("strain_data", ctypes.c_float * _MAXD), ("stress_data", ctypes.c_float * _MAXD),
                ("rho", ctypes.c_float), ("nu", ctypes.c_float), ("cte", ctypes.c_float),
                ("mu_static", ctypes.c_float), ("mu_kinetic", ctypes.c_float),
                ("zeta_internal", ctypes.c_float), ("zeta_global", ctypes.c_float),
                ("zeta_collision", ctypes.c_float), ("is_measured", ctypes.c_int)]


class _Env(ctypes.Structure):
    _fields_ = [("vox_size", ctypes.c_double), ("dt_frac", ctypes.c_double), ("gravity_mult", ctypes.c_float),
                ("floor_enabled", ctypes.c_int), ("collisions_enabled", ctypes.c_int),
                ("bounding_radius", ctypes.c_float), ("watch_distance", ctypes.c_float),
                ("vary_temp", ctypes.c_int), ("temp_amplitude", ctypes.c_double), ("temp_period", ctypes.c_double),
                ("enable_expansion", ctypes.c_int), ("initial_temp", ctypes.c_float)]


class _Ext(ctypes.Structure):
    _fields_ = [("voxel", ctypes.c_int), ("dof_fixed", ctypes.c_int), ("force", ctypes.c_float * 3),
                ("moment", ctypes.c_float * 3), ("translate", ctypes.c_double * 3), ("rotate", ctypes.c_double * 3)]


def build_port(force: bool = False) -> str:
    """Compile oracle/vx_oracle.c (make -C oracle port)."""
    if force or not os.path.exists(PORT_SO) or os.path.getmtime(PORT_SO) < os.path.getmtime(os.path.join(HERE, "vx_oracle.c")):
        subprocess.check_call(["make", "-s", "-C", HERE, "port"])
    return PORT_SO


# ----------------------------------------------------------------------------
# VXA text -> description


def _f32(x) -> float:
    return float(np.float32(x))


def _atof(s) -> float:
    """C atof: longest numeric prefix, 0.0 when none."""
    s = (s or "").strip()
    best = 0.0
    for end in range(len(s), 0, -1):
        try:
            best = float(s[:end])
            break
        except ValueError:
            continue
    return best


def _atoi(s) -> int:
    s = (s or "").strip()
    sign, i, v = 1, 0, 0
    if s[:1] in "+-":
        sign = -1 if s[0] == "-" else 1
        i = 1
    while i < len(s) and s[i].isdigit():
        v = v * 10 + int(s[i])
        i += 1
    return sign * v


def _child(el, tag):
    if el is None:
        return None
    for c in el:
        if c.tag == tag:
            return c
    return None


def _text(el, tag):
    c = _child(el, tag)
    return None if c is None else (c.text or "")


def _load_double(el, tag, default):
    t = _text(el, tag)
    return default if t is None else _atof(t)


def _load_float(el, tag, default):
    t = _text(el, tag)
    return _f32(default) if t is None else _f32(_atof(t))


def _load_int(el, tag, default):
    t = _text(el, tag)
    return default if t is None else _atoi(t)


def _load_bool(el, tag, default):
    t = _text(el, tag)
    return default if t is None else (_atoi(t) != 0)


def _ptree_path(root, path):
    node = root
    parts = path.split(".")
    if parts[0] != node.tag:
        return None
    for p in parts[1:]:
        node = _child(node, p)
        if node is None:
            return None
    return node


def _ptree_bool(root, path, default):
    n = _ptree_path(root, path)
    if n is None:
        return default
    t = (n.text or "").strip().lower()
    if t in ("true", "1"):
        return True
    if t in ("false", "0"):
        return False
    return default


def _ptree_num(root, path, default):
    n = _ptree_path(root, path)
    if n is None:
        return default
    try:
        return float((n.text or "").strip())
    except ValueError:
        return default


def merge_vxd(base_xml, vxd_xml):
    """Apply VXD overrides: every child of <VXD> carrying replace="VXA.a.b" replaces
    (or creates) the subtree at that path (Voxelyze3/src/Utils/ctool.h:49-57)."""
    root = ET.fromstring(base_xml.encode() if isinstance(base_xml, str) else base_xml)
    if vxd_xml:
        vxd = ET.fromstring(vxd_xml.encode() if isinstance(vxd_xml, str) else vxd_xml)
        src = vxd if vxd.tag == "VXD" else _child(vxd, "VXD")
        for c in list(src if src is not None else []):
            rep = c.get("replace", "")
            if not rep:
                continue
            parts = rep.split(".")
            node = root
            if parts[0] != root.tag:
                continue
            for p in parts[1:-1]:
                nxt = _child(node, p)
                if nxt is None:
                    nxt = ET.SubElement(node, p)
                node = nxt
            new = copy.deepcopy(c)
            new.tag = parts[-1]
            old = _child(node, parts[-1])
            if old is not None:
                idx = list(node).index(old)
                node.remove(old)
                node.insert(idx, new)
            else:
                node.append(new)
    return ET.tostring(root, encoding="unicode")


def desc_from_vxa(xml_text):
    """Merged VXA document -> dict(env, mats, voxels, phase, externals)."""
    root = ET.fromstring(xml_text.encode() if isinstance(xml_text, str) else xml_text)
    sim = _child(root, "Simulator")
    dt_frac = 0.9
    bond, colz, slow = 0.1, 1.0, 1.0
    volume = False
    if sim is not None:
        integ = _child(sim, "Integration")
        if integ is not None:
            dt_frac = _load_double(integ, "DtFrac", 0.9)
        damp = _child(sim, "Damping")
        if damp is not None:
            bond = _load_float(damp, "BondDampingZ", 0.1)
            colz = _load_float(damp, "ColDampingZ", 1.0)
            slow = _load_float(damp, "SlowDampingZ", 1.0)
        feat = _child(sim, "Features")
        if feat is not None:
            volume = _load_bool(feat, "VolumeEffectsEnabled", False)
    env_el = _child(root, "Environment")
    grav_acc, floor = -9.81, True
    temp_enabled, vary, temp_base, temp_amp, temp_period = True, False, 25.0, 0.0, 0.1
    if env_el is not None:
        g = _child(env_el, "Gravity")
        if g is not None:
            grav_acc = _load_double(g, "GravAcc", -9.81)
            floor = _load_bool(g, "FloorEnabled", False)
        th = _child(env_el, "Thermal")
        if th is not None:
            temp_enabled = _load_bool(th, "TempEnabled", False)
            temp_base = _load_double(th, "TempBase", 25.0)
            if _text(th, "TempAmplitude") is not None:
                temp_amp = _load_double(th, "TempAmplitude", 0.0)
            elif _text(th, "TempAmp") is not None:
                temp_amp = _load_double(th, "TempAmp", 0.0) - temp_base
            else:
                temp_amp = 0.0
            vary = _load_bool(th, "VaryTempEnabled", False)
            temp_period = _load_double(th, "TempPeriod", 0.1)
    vxc = _child(root, "VXC")
    lat = _child(vxc, "Lattice")
    vox_size = _load_double(lat, "Lattice_Dim", 0.001) * _load_double(lat, "X_Dim_Adj", 1.0) if lat is not None else 0.001
    mats = []
    pal = _child(vxc, "Palette")
    for m in (pal if pal is not None else []):
        if m.tag != "Material":
            continue
        mech = _child(m, "Mechanical")
        d = dict(model=_load_int(mech, "MatModel", 0), E=_load_double(mech, "Elastic_Mod", 0.0),
                 plastic_mod=_load_double(mech, "Plastic_Mod", 0.0), yield_stress=_load_double(mech, "Yield_Stress", 0.0),
                 fail_stress=_load_double(mech, "Fail_Stress", 0.0), rho=_load_double(mech, "Density", 0.0),
                 nu=_load_double(mech, "Poissons_Ratio", 0.0), cte=_load_double(mech, "CTE", 0.0),
                 mu_static=_load_double(mech, "uStatic", 0.0), mu_kinetic=_load_double(mech, "uDynamic", 0.0),
                 is_measured=_load_int(mech, "isMeasured", 1), strain_data=[], stress_data=[])
        ss = _child(mech, "SSData")
        if ss is not None:
            se, st = _child(ss, "StrainData"), _child(ss, "StressData")
            d["strain_data"] = [_atof(c.text) for c in (se if se is not None else []) if c.tag == "Strain"]
            d["stress_data"] = [_atof(c.text) for c in (st if st is not None else []) if c.tag == "Stress"]
        mats.append(d)
    st = _child(vxc, "Structure")
    X, Y, Z = _load_int(st, "X_Voxels", 1), _load_int(st, "Y_Voxels", 1), _load_int(st, "Z_Voxels", 1)
    comp = st.get("Compression", "")
    data = _child(st, "Data")
    layers = [c for c in data if c.tag == "Layer"] if data is not None else []
    cells = np.zeros(X * Y * Z, np.int32)
    for k in range(Z):
        raw = (layers[k].text or "") if k < len(layers) else ""
        if comp == "ASCII_READABLE":
            vals = [ord(ch) - 48 for ch in raw]
        else:
            import base64
            vals = list(base64.b64decode(raw))
        if len(vals) != X * Y:
            raise ValueError("voxel layer data does not match X_Voxels*Y_Voxels")
        cells[k * X * Y:(k + 1) * X * Y] = vals
    po = _child(st, "PhaseOffset")
    phases_per_voxel = None
    if po is not None:
        player = [c for c in po if c.tag == "Layer"]
        phases_per_voxel = []
        for k in range(Z):
            arr = [a for a in (player[k].text or "").split(",")] if k < len(player) else []
            for j in range(X * Y):
                if cells[k * X * Y + j] > 0:
                    phases_per_voxel.append(_atof(arr[j]) if j < len(arr) else 0.0)
    voxels, phase = [], []
    n = 0
    for i in range(X * Y * Z):
        mi = int(cells[i]) - 1
        if mi < 0:
            continue
        if mi >= len(mats):
            raise ValueError("voxel references a missing material")
        voxels.append((i % X, (i // X) % Y, i // (X * Y), mi))
        phase.append(phases_per_voxel[n] if phases_per_voxel is not None else 0.0)
        n += 1
    if not volume:
        for m in mats:
            m["nu"] = 0.0
    grav = _f32(_f32(-_f32(grav_acc)) / 9.80665)
    if temp_enabled:
        if vary:
            init = _f32(_f32(temp_base) - temp_base) if temp_period != 0 else _f32(0.0 - temp_base)
        else:
            init = _f32(_f32(temp_base + temp_amp) - temp_base)
    else:
        init = 0.0
    env = dict(vox_size=vox_size, dt_frac=dt_frac, gravity_mult=grav, floor_enabled=int(floor),
               collisions_enabled=int(_ptree_bool(root, "VXA.Simulator.AttachDetach.EnableCollision", True)),
               bounding_radius=_ptree_num(root, "VXA.Simulator.AttachDetach.boundingRadius", 0.75),
               watch_distance=_ptree_num(root, "VXA.Simulator.AttachDetach.watchDistance", 1.0),
               vary_temp=int(vary), temp_amplitude=temp_amp, temp_period=temp_period,
               enable_expansion=int(_ptree_num(root, "VXA.Simulator.EnableExpansion", 0)), initial_temp=init,
               zeta_internal=bond, zeta_global=slow, zeta_collision=colz)
    voxels = np.array(voxels, np.int32).reshape(-1, 4)
    externals = _boundary_conditions(env_el, lat, X, Y, Z, cells, voxels, vox_size)
    return dict(env=env, mats=mats, voxels=voxels, phase=np.array(phase, np.float64), externals=externals)


def _read_region(fr):
    """CVX_FRegion::ReadXML (Voxelyze3/src/old/VX_FRegion.cpp:165-216)."""
    prim = _load_int(fr, "PrimType", -1)
    if prim not in (0, 1, 2):
        raise ValueError("unsupported boundary-condition PrimType %d" % prim)
    r = dict(prim=prim, X=_load_double(fr, "X", 0.0), Y=_load_double(fr, "Y", 0.0), Z=_load_double(fr, "Z", 0.0),
             dX=_load_double(fr, "dX", 0.0), dY=_load_double(fr, "dY", 0.0), dZ=_load_double(fr, "dZ", 0.0),
             radius=_load_double(fr, "Radius", 0.0))
    if _text(fr, "DofFixed") is not None:
        r["dof"] = _load_int(fr, "DofFixed", 0) & 0xFF
        if r["dof"] >= 0x80:
            r["dof"] -= 0x100                      # (char) cast
    else:
        r["dof"] = 0x3F if _load_bool(fr, "Fixed", False) else 0
    r["force"] = [_load_double(fr, t, 0.0) for t in ("ForceX", "ForceY", "ForceZ")]
    r["torque"] = [_load_double(fr, t, 0.0) for t in ("TorqueX", "TorqueY", "TorqueZ")]
    r["disp"] = [_load_double(fr, t, 0.0) for t in ("DisplaceX", "DisplaceY", "DisplaceZ")]
    r["ang"] = [_load_double(fr, t, 0.0) for t in ("AngDisplaceX", "AngDisplaceY", "AngDisplaceZ")]
    return r


def _touching(r, P, D, E):
    """CPrimitive::IsTouching(P, Dist, Envelope) for box, cylinder, sphere (VX_FRegion.cpp:420-429, 495-534, 591-604)."""
    if r["prim"] == 0:
        ps = [P[k] / E[k] for k in range(3)]
        ds = [D[k] / E[k] for k in range(3)]
        lo, dd = (r["X"], r["Y"], r["Z"]), (r["dX"], r["dY"], r["dZ"])
        return all(ps[k] + ds[k] > lo[k] and ps[k] - ds[k] < lo[k] + dd[k] for k in range(3))
    pos = [r["X"] * E[0], r["Y"] * E[1], r["Z"] * E[2]]
    size = [r["dX"] * E[0], r["dY"] * E[1], r["dZ"] * E[2]]
    rad = r["radius"] * max(E)
    if r["prim"] == 1:
        for a, (b, c) in ((0, (1, 2)), (1, (0, 2)), (2, (0, 1))):
            if (r["dX"], r["dY"], r["dZ"])[a] != 0:
                return (P[a] > pos[a] and P[a] < pos[a] + size[a] and
                        math.sqrt((P[b] - pos[b]) * (P[b] - pos[b]) + (P[c] - pos[c]) * (P[c] - pos[c])) < rad)
        return False
    dist = math.sqrt(D[0] * D[0] + D[1] * D[1] + D[2] * D[2])
    return math.sqrt((P[0] - pos[0]) * (P[0] - pos[0]) + (P[1] - pos[1]) * (P[1] - pos[1]) +
                     (P[2] - pos[2]) * (P[2] - pos[2])) < rad + dist


def _boundary_conditions(env_el, lat, NX, NY, NZ, cells, voxels, vox_size):
    """Externals from <Environment> boundary-condition regions as CVX_Sim::Import applies them
    (VXA/VX_Sim.cpp:109-144; regions read by CVX_Environment::ReadXML, VX_Environment.cpp:101-146;
    counts by CVX_Environment::GetNumTouching, VX_Environment.cpp:215-232 on CVX_Object::GetXYZ
    cell points, VXA/VX_Object.cpp:525-558)."""
    regions = []
    if env_el is not None:
        lists = []
        bc = _child(env_el, "Boundary_Conditions")
        if bc is not None:
            lists.append((bc, "NumBCs"))
        else:
            for tag, cnt in (("Fixed_Regions", "NumFixed"), ("Forced_Regions", "NumForced")):
                el = _child(env_el, tag)
                if el is not None:
                    lists.append((el, cnt))
        for el, cnt in lists:
            n = _load_int(el, cnt, 0)
            frs = [c for c in el if c.tag == "FRegion"]
            if n > len(frs):
                raise ValueError("fewer FRegion elements than " + cnt)
            regions += [_read_region(fr) for fr in frs[:n]]
    if not regions:
        return []
    ld = _load_double(lat, "Lattice_Dim", 0.001)
    adj = [_load_double(lat, t, 1.0) for t in ("X_Dim_Adj", "Y_Dim_Adj", "Z_Dim_Adj")]
    latenv = [ld * a for a in adj]
    ws = [ld * adj[0] * NX, ld * adj[1] * NY, ld * adj[2] * NZ]
    half = [x / 2.0 for x in latenv]
    eps = 0.000001
    offx = eps - int(eps / adj[0]) * adj[0]
    offy = eps - int(eps / adj[1]) * adj[1]
    touching = [0] * len(regions)
    for i in range(NX * NY * NZ):
        if cells[i] == 0:
            continue
        ix, iy, iz = i % NX, (i // NX) % NY, i // (NX * NY)
        p = [ld * (adj[0] * (0.5 + ix) + offx), ld * (adj[1] * (0.5 + iy) + offy), ld * adj[2] * (0.5 + iz)]
        for j, r in enumerate(regions):
            if _touching(r, p, half, ws):
                touching[j] += 1
    ext = {}
    for v, (ix, iy, iz, _) in enumerate(voxels):
        p = [ix * vox_size + latenv[0] / 2, iy * vox_size + latenv[1] / 2, iz * vox_size + latenv[2] / 2]
        for j, r in enumerate(regions):
            if not _touching(r, p, half, ws):
                continue
            e = ext.setdefault(v, dict(voxel=v, dof_fixed=0, force=np.zeros(3, np.float32), moment=np.zeros(3, np.float32),
                                       translate=[0.0, 0.0, 0.0], rotate=[0.0, 0.0, 0.0]))
            vals = r["disp"] + r["ang"]
            for k in range(6):
                if r["dof"] & (1 << k):
                    e["dof_fixed"] |= 1 << k
                    if vals[k] != 0.0:
                        (e["translate"] if k < 3 else e["rotate"])[k % 3] = vals[k]
            with np.errstate(divide="ignore", invalid="ignore"):
                for k in range(3):
                    f_add = np.float32(float(e["force"][k]) + np.float64(r["force"][k]) / np.float64(touching[j]))
                    m_add = np.float32(float(e["moment"][k]) + np.float64(r["torque"][k]) / np.float64(touching[j]))
                    e["force"][k] = np.float32(e["force"][k] + f_add)
                    e["moment"][k] = np.float32(e["moment"][k] + m_add)
    return [dict(x, force=tuple(float(f) for f in x["force"]), moment=tuple(float(m) for m in x["moment"]))
            for _, x in sorted(ext.items())]


# ----------------------------------------------------------------------------
def _lib(path):
    lib = ctypes.CDLL(path)
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleSim:
    """The C restatement (oracle/vx_oracle.c) of one simulation."""

    _lib = None

    def __init__(self, desc):
        if OracleSim._lib is None:
            lib = _lib(build_port())
            lib.vxo_create.restype = ctypes.c_void_p
            lib.vxo_create.argtypes = [ctypes.POINTER(_Env), ctypes.POINTER(_Mat), ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_Ext), ctypes.c_int]
            for fn in ("vxo_free", "vxo_step", "vxo_counts", "vxo_scalars", "vxo_voxel_state", "vxo_link_state",
                       "vxo_topology", "vxo_voxmats", "vxo_linkmats", "vxo_center_of_mass"):
                getattr(lib, fn).restype = ctypes.c_int if fn == "vxo_step" else None
            OracleSim._lib = lib
        L = OracleSim._lib
        e = desc["env"]
        env = _Env(e["vox_size"], e["dt_frac"], e["gravity_mult"], e["floor_enabled"], e["collisions_enabled"],
                   e["bounding_radius"], e["watch_distance"], e["vary_temp"], e["temp_amplitude"], e["temp_period"],
                   e["enable_expansion"], e["initial_temp"])
        mats = (_Mat * max(1, len(desc["mats"])))()
        model_map = {0: 0, 1: 1, 2: 2, 3: 3}
        for i, m in enumerate(desc["mats"]):
            mm = mats[i]
            mm.model = model_map.get(m["model"], 0)
            mm.E, mm.plastic_mod, mm.yield_stress, mm.fail_stress = m["E"], m["plastic_mod"], m["yield_stress"], m["fail_stress"]
            nd = min(len(m["strain_data"]), _MAXD)
            mm.ndata = nd
            for k in range(nd):
                mm.strain_data[k] = m["strain_data"][k]
                mm.stress_data[k] = m["stress_data"][k]
            mm.rho, mm.nu, mm.cte = m["rho"], m["nu"], m["cte"]
            mm.mu_static, mm.mu_kinetic = m["mu_static"], m["mu_kinetic"]
            mm.zeta_internal, mm.zeta_global, mm.zeta_collision = e["zeta_internal"], e["zeta_global"], e["zeta_collision"]
            mm.is_measured = m.get("is_measured", 1)
        vox = np.ascontiguousarray(desc["voxels"], np.int32)
        ph = np.ascontiguousarray(desc["phase"], np.float64)
        exts = desc.get("externals", [])
        ext = (_Ext * max(1, len(exts)))()
        for i, x in enumerate(exts):
            ext[i].voxel, ext[i].dof_fixed = x["voxel"], x.get("dof_fixed", 0)
            for k in range(3):
                ext[i].force[k] = x.get("force", (0, 0, 0))[k]
                ext[i].moment[k] = x.get("moment", (0, 0, 0))[k]
                ext[i].translate[k] = x.get("translate", (0, 0, 0))[k]
                ext[i].rotate[k] = x.get("rotate", (0, 0, 0))[k]
        self._keep = (mats, vox, ph, ext)
        self.h = ctypes.c_void_p(L.vxo_create(ctypes.byref(env), mats, len(desc["mats"]), _p(vox), _p(ph), len(vox), ext, len(exts)))
        c = np.zeros(4, np.int32)
        L.vxo_counts(self.h, _p(c))
        self.nvox, self.nlink, self.nvmat, self.nlmat = (int(x) for x in c)

    def __del__(self):
        if getattr(self, "h", None) and OracleSim._lib is not None:
            OracleSim._lib.vxo_free(self.h)
            self.h = None

    def step(self, n):
        return OracleSim._lib.vxo_step(self.h, int(n))

    def scalars(self):
        o = np.zeros(5)
        OracleSim._lib.vxo_scalars(self.h, _p(o))
        return dict(t=o[0], optimal_dt=o[1], dt=o[2], diverged=int(o[3]), steps=int(o[4]))

    def voxel_state(self):
        d = np.zeros((self.nvox, 13)); f = np.zeros((self.nvox, 4), np.float32); fl = np.zeros(self.nvox, np.int32)
        OracleSim._lib.vxo_voxel_state(self.h, _p(d), _p(f), _p(fl))
        return dict(pos=d[:, 0:3], linMom=d[:, 3:6], orient=d[:, 6:10], angMom=d[:, 10:13], temp=f[:, 0],
                    pStrain=f[:, 1:4], flags=fl)

    def link_state(self):
        d = np.zeros((self.nlink, 22)); f = np.zeros((self.nlink, 6), np.float32); i2 = np.zeros((self.nlink, 2), np.int32)
        OracleSim._lib.vxo_link_state(self.h, _p(d), _p(f), _p(i2))
        return dict(pos2=d[:, 0:3], angle1v=d[:, 3:6], angle2v=d[:, 6:9], forceNeg=d[:, 9:12], forcePos=d[:, 12:15],
                    momentNeg=d[:, 15:18], momentPos=d[:, 18:21], restLength=d[:, 21], strain=f[:, 0],
                    maxStrain=f[:, 1], strainOffset=f[:, 2], stress=f[:, 3], area=f[:, 4], tss=f[:, 5],
                    smallAngle=i2[:, 0], flags=i2[:, 1])

    def topology(self):
        v = np.zeros((self.nvox, 4), np.int32); l = np.zeros((self.nlink, 4), np.int32)
        OracleSim._lib.vxo_topology(self.h, _p(v), _p(l))
        return dict(voxels=v, links=l)

    def materials(self):
        f = np.zeros((self.nvmat, 18), np.float32); nom = np.zeros(self.nvmat)
        OracleSim._lib.vxo_voxmats(self.h, _p(f), _p(nom))
        idx = np.zeros((self.nlmat, 2), np.int32); lf = np.zeros((self.nlmat, 20), np.float32)
        OracleSim._lib.vxo_linkmats(self.h, _p(idx), _p(lf))
        return dict(voxmat=f, nom=nom, linkmat_idx=idx, linkmat=lf)

    def center_of_mass(self):
        o = np.zeros(3)
        OracleSim._lib.vxo_center_of_mass(self.h, _p(o))
        return o


class RefSim:
    """The reference's own CPU Voxelyze (oracle/_ref/libvxref.so) on one merged VXA."""

    _lib = None

    @staticmethod
    def available():
        return os.path.exists(REF_SO)

    def __init__(self, merged_xml, desc=None):
        if RefSim._lib is None:
            lib = _lib(REF_SO)
            lib.vxref_load.restype = ctypes.c_void_p
            lib.vxref_load.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float]
            lib.vxref_step.restype = ctypes.c_int
            RefSim._lib = lib
        L = RefSim._lib
        desc = desc or desc_from_vxa(merged_xml)
        e = desc["env"]
        self.h = ctypes.c_void_p(L.vxref_load(merged_xml.encode(), int(e["collisions_enabled"]), int(e["enable_expansion"]),
                                              float(e["bounding_radius"]), float(e["watch_distance"])))
        c = np.zeros(4, np.int32)
        L.vxref_counts(self.h, _p(c))
        self.nvox, self.nlink, self.nvmat, self.nlmat = (int(x) for x in c)

    def __del__(self):
        if getattr(self, "h", None) and RefSim._lib is not None:
            RefSim._lib.vxref_free(self.h)
            self.h = None

    def set_external(self, voxel, dof_fixed=0, force=(0, 0, 0), moment=(0, 0, 0), translate=(0, 0, 0), rotate=(0, 0, 0)):
        f = np.asarray(force, np.float32); m = np.asarray(moment, np.float32)
        t = np.asarray(translate, np.float64); r = np.asarray(rotate, np.float64)
        RefSim._lib.vxref_set_external(self.h, int(voxel), int(dof_fixed), _p(f), _p(m), _p(t), _p(r))

    def step(self, n):
        return RefSim._lib.vxref_step(self.h, int(n))

    def scalars(self):
        o = np.zeros(5)
        RefSim._lib.vxref_scalars(self.h, _p(o))
        return dict(t=o[0], optimal_dt=o[1], dt=o[2], diverged=int(o[3]), steps=int(o[4]))

    def env(self):
        o = np.zeros(9)
        RefSim._lib.vxref_env(self.h, _p(o))
        return o

    def voxel_state(self):
        d = np.zeros((self.nvox, 13)); f = np.zeros((self.nvox, 4), np.float32); fl = np.zeros(self.nvox, np.int32)
        RefSim._lib.vxref_voxel_state(self.h, _p(d), _p(f), _p(fl))
        return dict(pos=d[:, 0:3], linMom=d[:, 3:6], orient=d[:, 6:10], angMom=d[:, 10:13], temp=f[:, 0],
                    pStrain=f[:, 1:4], flags=fl)

    def link_state(self):
        d = np.zeros((self.nlink, 22)); f = np.zeros((self.nlink, 6), np.float32); i2 = np.zeros((self.nlink, 2), np.int32)
        RefSim._lib.vxref_link_state(self.h, _p(d), _p(f), _p(i2))
        return dict(pos2=d[:, 0:3], angle1v=d[:, 3:6], angle2v=d[:, 6:9], forceNeg=d[:, 9:12], forcePos=d[:, 12:15],
                    momentNeg=d[:, 15:18], momentPos=d[:, 18:21], restLength=d[:, 21], strain=f[:, 0],
                    maxStrain=f[:, 1], strainOffset=f[:, 2], stress=f[:, 3], area=f[:, 4], tss=f[:, 5],
                    smallAngle=i2[:, 0], flags=i2[:, 1])

    def topology(self):
        v = np.zeros((self.nvox, 4), np.int32); l = np.zeros((self.nlink, 4), np.int32); ph = np.zeros(self.nvox)
        RefSim._lib.vxref_topology(self.h, _p(v), _p(l), _p(ph))
        return dict(voxels=v, links=l, phase=ph)

    def externals(self):
        """Per voxel: fixed-DOF bits and force3, moment3, translation3, rotation3 (zeros without an external)."""
        dof = np.zeros(self.nvox, np.int32); vals = np.zeros((self.nvox, 12))
        RefSim._lib.vxref_externals(self.h, _p(dof), _p(vals))
        return dict(dof=dof, vals=vals)

    def materials(self):
        f = np.zeros((self.nvmat, 18), np.float32); nom = np.zeros(self.nvmat)
        RefSim._lib.vxref_voxmats(self.h, _p(f), _p(nom))
        idx = np.zeros((self.nlmat, 2), np.int32); lf = np.zeros((self.nlmat, 20), np.float32)
        RefSim._lib.vxref_linkmats(self.h, _p(idx), _p(lf))
        return dict(voxmat=f, nom=nom, linkmat_idx=idx, linkmat=lf)
