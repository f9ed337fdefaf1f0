"""TEST INFRASTRUCTURE ONLY: ctypes binding of the FP64 CPU oracle.

Replays a ``fdtd_gpu.spec.JobSpec`` onto oracle/_build/libfdtd_oracle.so
(built by ``make -C oracle``).  Used by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg only, as the checker.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libfdtd_oracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = C.CDLL(_LIB)
        vp = C.c_void_p
        L.ora_create.restype = vp
        L.ora_create.argtypes = [vp]
        L.ora_destroy.argtypes = [vp]
        L.ora_error.restype = C.c_char_p
        for name in ("ora_add_dielectric",):
            getattr(L, name).argtypes = [vp, vp, C.c_double]
        L.ora_add_conductive.argtypes = [vp, vp, C.c_double, C.c_double]
        for name in ("ora_add_gold", "ora_add_graphene", "ora_add_lorentz", "ora_add_graphene_cp", "ora_add_graphene_nk",
                     "ora_add_pml", "ora_add_tfsf_1d", "ora_add_tfsf",
                     "ora_add_source", "ora_add_monitor", "ora_add_probe"):
            getattr(L, name).argtypes = [vp, vp] if name in ("ora_add_pml", "ora_add_tfsf_1d", "ora_add_tfsf", "ora_add_source",
                                                              "ora_add_monitor", "ora_add_probe") else [vp, vp, vp]
        L.ora_commit.argtypes = [vp]
        L.ora_step.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.ora_get_field.argtypes = [vp, C.c_int, vp]
        L.ora_set_field.argtypes = [vp, C.c_int, vp]
        L.ora_get_monitor.argtypes = [vp, C.c_int, vp, vp]
        L.ora_monitor_size.argtypes = [vp, C.c_int, vp, vp, vp]
        L.ora_get_probe.argtypes = [vp, C.c_int, vp, vp]
        _lib = L
    return _lib


class OracleJob:
    """The oracle twin of fdtd_gpu.Job (same method names)."""

    def __init__(self, spec, nthreads=1):
        from fdtd_gpu import spec as S
        self.spec = spec
        self.nthreads = int(nthreads)
        L = lib()
        g = spec.grid_desc()
        self.h = L.ora_create(C.byref(g))
        if not self.h:
            raise RuntimeError(L.ora_error().decode())
        keep = []
        for m in spec.materials:
            r = S.region_struct(m.region, keep)
            if m.kind == "dielectric":
                rc = L.ora_add_dielectric(self.h, C.byref(r), m.eps)
            elif m.kind == "gold":
                p = S.drude2cp_struct(m.params)
                rc = L.ora_add_gold(self.h, C.byref(r), C.byref(p))
            elif m.kind == "lorentz":
                p = S.lorentz_struct(m.params)
                rc = L.ora_add_lorentz(self.h, C.byref(r), C.byref(p))
            elif m.kind == "graphene_nk":
                p = S.graphene_nk_struct(m.params)
                rc = L.ora_add_graphene_nk(self.h, C.byref(r), C.byref(p))
            elif m.kind == "conductive":
                rc = L.ora_add_conductive(self.h, C.byref(r), m.params["eps_inf"], m.params["sigma"])
            elif m.kind == "graphene_cp":
                p = S.graphene_cp_struct(m.params)
                rc = L.ora_add_graphene_cp(self.h, C.byref(r), C.byref(p))
            else:
                p = S.graphene_struct(m.params)
                rc = L.ora_add_graphene(self.h, C.byref(r), C.byref(p))
            self._check(rc)
        if spec.pml:
            p = S.pml_struct(spec.pml)
            self._check(L.ora_add_pml(self.h, C.byref(p)))
        if spec.tfsf:
            t = S.tfsf_struct(spec.tfsf)
            self._check(L.ora_add_tfsf_1d(self.h, C.byref(t)))
        if spec.tfsf_box:
            t = S.tfsf_box_struct(spec.tfsf_box)
            self._check(L.ora_add_tfsf(self.h, C.byref(t)))
        for s in spec.sources:
            d = S.source_struct(s)
            self._check(L.ora_add_source(self.h, C.byref(d)))
        for m in spec.monitors:
            d = S.monitor_struct(m, keep)
            self._check(L.ora_add_monitor(self.h, C.byref(d)))
        for p in spec.probes:
            d = S.probe_struct(p)
            self._check(L.ora_add_probe(self.h, C.byref(d)))
        self._check(L.ora_commit(self.h))
        self.n_done = 0

    def _check(self, rc):
        if rc < 0:
            raise RuntimeError("oracle: " + lib().ora_error().decode())
        return rc

    def step(self, n_first, n_steps):
        self._check(lib().ora_step(self.h, int(n_first), int(n_steps), self.nthreads))
        self.n_done = n_first + n_steps - 1

    def run(self, n_steps):
        self.step(self.n_done + 1, n_steps)

    def get_field(self, comp):
        from fdtd_gpu import spec as S
        n = self.spec.n
        cnt = S.field_count(self.spec, comp)
        out = np.empty(cnt)
        self._check(lib().ora_get_field(self.h, int(comp), out.ctypes.data))
        return out if cnt != self.spec.cells() else out.reshape(n[2], n[1], n[0])

    def set_field(self, comp, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        self._check(lib().ora_set_field(self.h, int(comp), a.ctypes.data))

    def get_monitor(self, mid):
        nc, nf, ncell = C.c_int(), C.c_int(), C.c_int()
        self._check(lib().ora_monitor_size(self.h, mid, C.byref(nc), C.byref(nf), C.byref(ncell)))
        re = np.empty(nc.value * nf.value * ncell.value)
        im = np.empty_like(re)
        self._check(lib().ora_get_monitor(self.h, mid, re.ctypes.data, im.ctypes.data))
        shape = (nc.value, nf.value, ncell.value)
        return re.reshape(shape), im.reshape(shape)

    def get_probe(self, pid):
        cnt = C.c_int()
        self._check(lib().ora_get_probe(self.h, pid, None, C.byref(cnt)))
        ncomp = len(set(self.spec.probes[pid].comps))
        out = np.empty(max(1, cnt.value * ncomp))
        self._check(lib().ora_get_probe(self.h, pid, out.ctypes.data, C.byref(cnt)))
        return out[: cnt.value * ncomp].reshape(cnt.value, ncomp)

    def close(self):
        if self.h:
            lib().ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
