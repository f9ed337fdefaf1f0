"""Backend-independent description of one FDTD job.

A ``JobSpec`` records the same calls a reference ``program.f90`` makes during
set-up (grid, materials in update order, PML, sources, monitors, probes) and
is replayed onto a backend: the GB300 library (``fdtd_gpu.Job``) or the CPU
oracle used by the tests.  Cell indices are 0-based; reference index i is i-1.
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

from . import abi

Box = Tuple[Tuple[int, int, int], Tuple[int, int, int]]


@dataclass
class Material:
    kind: str                      # "dielectric" | "gold" | "graphene" | "lorentz" | "graphene_cp" | "conductive"
    #                                  | "graphene_nk"
    region: dict                   # {"kind": "box", "lo":..., "hi":...} | spheres | mask
    eps: float = 1.0
    params: Optional[dict] = None


@dataclass
class Monitor:
    lo: Tuple[int, int, int]
    hi: Tuple[int, int, int]
    comps: Tuple[int, ...]
    omega: np.ndarray
    n_first: int = 1
    n_last: int = 2 ** 31 - 1
    mean: bool = False  # transform the box mean of each component


@dataclass
class Probe:
    cell: Tuple[int, int, int]
    comps: Tuple[int, ...]
    n_first: int = 1
    n_last: int = 2 ** 31 - 1


@dataclass
class JobSpec:
    layout: int
    n: Tuple[int, int, int]
    ku: float
    dt: float
    ds: float
    periodic: Tuple[int, int, int] = (0, 0, 0)
    main_lo: Tuple[int, int, int] = (0, 0, 0)
    main_hi: Optional[Tuple[int, int, int]] = None
    precision: int = abi.F64
    materials: List[Material] = field(default_factory=list)
    pml: Optional[dict] = None
    sources: List[dict] = field(default_factory=list)
    monitors: List[Monitor] = field(default_factory=list)
    probes: List[Probe] = field(default_factory=list)
    tfsf: Optional[dict] = None        # 1D line: {"boundary", "eps_lo", "eps_hi"}
    tfsf_box: Optional[dict] = None    # 2D/3D: {"lo", "hi", "eps_line"}
    name: str = ""

    # -- builders ---------------------------------------------------------
    def add_dielectric(self, region, eps):
        self.materials.append(Material("dielectric", region, eps=eps))
        return len(self.materials)

    def add_gold(self, region, params):
        self.materials.append(Material("gold", region, params=dict(params)))
        return len(self.materials)

    def add_graphene(self, region, params):
        self.materials.append(Material("graphene", region, params=dict(params)))
        return len(self.materials)

    def add_lorentz(self, region, params):
        """params: {"form": abi.LORENTZ_JP | abi.LORENTZ_S, "eps_inf",
        "delta_eps": [...], "omega": [...], "gamma": [...]} (rad/s)."""
        self.materials.append(Material("lorentz", region, params=dict(params)))
        return len(self.materials)

    def add_conductive(self, region, params):
        """A conductive dielectric (SiL800): params {"eps_inf", "sigma" [S/m]}."""
        self.materials.append(Material("conductive", region, params=dict(params)))
        return len(self.materials)

    def add_graphene_nk(self, region, params):
        """The reference's 1D graphene at 633 nm (graphene633): params {"n",
        "k", "wavelength", "scale", "chi3", "alpha", "w_nl", "gamma_nl"}."""
        self.materials.append(Material("graphene_nk", region, params=dict(params)))
        return len(self.materials)

    def add_graphene_cp(self, region, params):
        """The reference's Graphene (Drude + 4 critical points + Raman):
        params {"eps_inf", "drude_omega", "drude_gamma", "amp", "phi", "omega",
        "gamma" (4 each), "width", "chi3", "w_nl", "gamma_nl", "raman_form",
        "normal_axis"}."""
        self.materials.append(Material("graphene_cp", region, params=dict(params)))
        return len(self.materials)

    def add_monitor(self, lo, hi, comps, omega, n_first=1, n_last=2 ** 31 - 1, mean=False):
        self.monitors.append(Monitor(tuple(lo), tuple(hi), tuple(comps),
                                     np.ascontiguousarray(omega, dtype=np.float64),
                                     int(n_first), int(n_last), bool(mean)))
        return len(self.monitors) - 1

    def add_probe(self, cell, comps, n_first=1, n_last=2 ** 31 - 1):
        self.probes.append(Probe(tuple(cell), tuple(comps), int(n_first), int(n_last)))
        return len(self.probes) - 1

    def cells(self):
        return int(self.n[0]) * int(self.n[1]) * int(self.n[2])

    def with_precision(self, precision):
        import copy
        s = copy.copy(self)
        s.precision = precision
        return s

    # -- C descriptors ------------------------------------------------------
    def grid_desc(self):
        hi = self.main_hi if self.main_hi is not None else tuple(max(0, x - 1) for x in self.n)
        return abi.GridDesc(self.layout, self.precision, abi.I3(*self.n), abi.I3(*self.periodic),
                            abi.I3(*self.main_lo), abi.I3(*hi), self.ku, self.dt, self.ds)


def box(lo, hi):
    return {"kind": "box", "lo": tuple(lo), "hi": tuple(hi)}


def spheres(rows):
    """rows: iterable of (cx, cy, cz, r) in cell units (2D: cz ignored)."""
    return {"kind": "spheres", "rows": np.ascontiguousarray(np.asarray(rows, dtype=np.float64).reshape(-1, 4))}


def mask(arr):
    return {"kind": "mask", "mask": np.ascontiguousarray(arr, dtype=np.uint8)}


def region_struct(reg, keep):
    """Return an abi.Region for a region dict; arrays it points to are
    appended to ``keep`` so they outlive the call."""
    r = abi.Region()
    if reg["kind"] == "box":
        r.kind = abi.REGION_BOX
        r.lo = abi.I3(*reg["lo"])
        r.hi = abi.I3(*reg["hi"])
    elif reg["kind"] == "spheres":
        rows = reg["rows"]
        keep.append(rows)
        r.kind = abi.REGION_SPHERES
        r.count = rows.shape[0]
        r.centers_radii = rows.ctypes.data_as(C.POINTER(C.c_double))
    elif reg["kind"] == "mask":
        m = reg["mask"].ravel(order="F") if reg["mask"].ndim > 1 else reg["mask"]
        m = np.ascontiguousarray(m)
        keep.append(m)
        r.kind = abi.REGION_MASK
        r.mask = m.ctypes.data_as(C.POINTER(C.c_uint8))
    else:
        raise ValueError(reg["kind"])
    return r


def drude2cp_struct(p):
    d = abi.Drude2CP()
    d.eps_inf = p["eps_inf"]
    d.omega_d = p["omega_d"]
    d.gamma_d = p["gamma_d"]
    for q in range(2):
        d.amp[q] = p["amp"][q]
        d.phi[q] = p["phi"][q]
        d.omega[q] = p["omega"][q]
        d.gamma[q] = p["gamma"][q]
    return d


def graphene_struct(p):
    return abi.GrapheneDesc(p["fermi_ev"], p["tau"], p["temperature"], p["chi3"], p["raman_frac"],
                            p["raman_freq"], p["raman_tau"], p["thickness"], p.get("e_scale", 1.0))


def lorentz_struct(p):
    d = abi.LorentzDesc()
    d.form = int(p.get("form", abi.LORENTZ_JP))
    d.npoles = len(p["delta_eps"])
    d.eps_inf = p["eps_inf"]
    for q in range(d.npoles):
        d.delta_eps[q] = p["delta_eps"][q]
        d.omega[q] = p["omega"][q]
        d.gamma[q] = p["gamma"][q]
    d.sheet = int(p.get("sheet", 0))
    d.ez_uses_x_current = int(p.get("ez_uses_x_current", 0))
    d.chi3 = p.get("chi3", 0.0)
    d.w_nl = p.get("w_nl", 0.0)
    d.gamma_nl = p.get("gamma_nl", 0.0)
    d.e_scale = p.get("e_scale", 1.0)
    return d


def graphene_nk_struct(p):
    return abi.GrapheneNkDesc(p["n"], p["k"], p["wavelength"], p["scale"], p.get("chi3", 0.0), p.get("alpha", 0.0),
                              p.get("w_nl", 0.0), p.get("gamma_nl", 0.0))


def graphene_cp_struct(p):
    d = abi.GrapheneCpDesc()
    d.eps_inf = p["eps_inf"]
    d.drude_omega = p["drude_omega"]
    d.drude_gamma = p["drude_gamma"]
    for q in range(4):
        d.amp[q] = p["amp"][q]
        d.phi[q] = p["phi"][q]
        d.omega[q] = p["omega"][q]
        d.gamma[q] = p["gamma"][q]
    d.width = p["width"]
    d.chi3 = p.get("chi3", 0.0)
    d.w_nl = p.get("w_nl", 0.0)
    d.gamma_nl = p.get("gamma_nl", 0.0)
    d.raman_form = int(p.get("raman_form", abi.RAMAN_EXACT))
    d.normal_axis = int(p.get("normal_axis", 1))
    return d


def pml_struct(p):
    d = abi.PmlDesc()
    d.mode = p["mode"]
    for a in range(3):
        for s in range(2):
            d.npml[a][s] = p["npml"][a][s]
    d.eps_lo = p["eps_lo"]
    d.eps_hi = p.get("eps_hi", p["eps_lo"])
    d.sigma_max = p["sigma_max"]
    d.order = p["order"]
    return d


def source_struct(s):
    return abi.SourceDesc(s["component"], abi.I3(*s["lo"]), abi.I3(*s["hi"]), s["amp"],
                          s["t0"], s["st"], s["w0"])


def comp_mask(comps):
    m = 0
    for c in comps:
        m |= 1 << int(c)
    return m


def monitor_struct(m, keep):
    keep.append(m.omega)
    return abi.MonitorDesc(abi.I3(*m.lo), abi.I3(*m.hi), comp_mask(m.comps), m.n_first, m.n_last,
                           len(m.omega), m.omega.ctypes.data_as(C.POINTER(C.c_double)),
                           abi.MONITOR_MEAN if m.mean else abi.MONITOR_CELLS)


def probe_struct(p):
    return abi.ProbeDesc(abi.I3(*p.cell), comp_mask(p.comps), p.n_first, p.n_last)


def tfsf_box_struct(t):
    return abi.TfsfDesc(abi.I3(*t["lo"]), abi.I3(*t["hi"]), float(t.get("eps_line", 1.0)))


def field_count(spec, comp):
    """Values fdtd_get_field returns for ``comp``: the grid, or the ny
    cells of a 2D/3D box's incident line."""
    if spec.tfsf_box is not None and comp >= abi.E_INC:
        return int(spec.n[1])
    return spec.cells()


def tfsf_struct(t):
    return abi.Tfsf1dDesc(t["boundary"], t["eps_lo"], t["eps_hi"])


def monitor_shape(m):
    ncell = 1
    for a in range(3):
        ncell *= 1 if m.mean else m.hi[a] - m.lo[a] + 1
    return len(sorted(set(m.comps))), len(m.omega), ncell
