"""ctypes binding of libfdtd_gb300.so: ``Job`` replays a JobSpec onto the GPU.

The library is loaded from fortran-mpi-fdtd_gb300/lib/ (built in-tree by
fdtd_gpu.build).  There is no fallback: if the library or an sm_103a device
is missing, creating a Job raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi, spec as S

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "lib", "libfdtd_gb300.so")
_lib = None

# every entry point declared in include/fdtd_gb300.h
EXPORTS = [
    "fdtd_create", "fdtd_destroy", "fdtd_last_error", "fdtd_device_count",
    "fdtd_add_dielectric", "fdtd_add_gold", "fdtd_add_graphene", "fdtd_add_lorentz", "fdtd_add_graphene_cp", "fdtd_add_conductive", "fdtd_add_graphene_nk",
    "fdtd_add_pml",
    "fdtd_add_tfsf_1d", "fdtd_add_tfsf", "fdtd_add_source", "fdtd_add_monitor", "fdtd_add_probe", "fdtd_commit",
    "fdtd_step", "fdtd_update_DE", "fdtd_pml_update_E", "fdtd_interchange", "fdtd_update_H",
    "fdtd_pml_update_H", "fdtd_sample", "fdtd_sync", "fdtd_get_field", "fdtd_set_field",
    "fdtd_get_monitor", "fdtd_get_probe", "fdtd_device_bytes", "fdtd_estimate_bytes", "fdtd_profile",
    "fdtd_kernel_time", "fdtd_kernel_cells", "fdtd_set_tile", "fdtd_get_tile", "fdtd_launch_count", "fdtd_set_stream", "fdtd_transfer_bytes",
    "fdtd_dft_sample_noalloc", "fdtd_state_bytes", "fdtd_save_state", "fdtd_load_state",
    "fdtd_check_finite", "fdtd_debug_fail_alloc", "fdtd_debug_wait_limit",
    "fdtd_server_create", "fdtd_server_submit", "fdtd_server_wait", "fdtd_server_job", "fdtd_server_times",
    "fdtd_server_release", "fdtd_server_stats", "fdtd_server_destroy",
]


class FdtdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fdtd error {code}: {msg}")
        self.code = code


def lib(path=None):
    global _lib
    if _lib is None or path:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise FdtdError(abi.FDTD_ENODEV, f"{p} is not built (run fdtd_gpu.build.build())")
        L = C.CDLL(p)
        vp, i32, dbl = C.c_void_p, C.c_int32, C.c_double
        sig = {
            "fdtd_create": [vp, C.POINTER(vp)], "fdtd_destroy": [vp],
            "fdtd_last_error": [C.c_char_p, C.c_size_t], "fdtd_device_count": [C.POINTER(i32)],
            "fdtd_add_dielectric": [vp, vp, dbl, C.POINTER(i32)],
            "fdtd_add_gold": [vp, vp, vp, C.POINTER(i32)], "fdtd_add_graphene": [vp, vp, vp, C.POINTER(i32)],
            "fdtd_add_lorentz": [vp, vp, vp, C.POINTER(i32)], "fdtd_add_graphene_cp": [vp, vp, vp, C.POINTER(i32)],
            "fdtd_add_conductive": [vp, vp, dbl, dbl, C.POINTER(i32)],
            "fdtd_add_graphene_nk": [vp, vp, vp, C.POINTER(i32)],
            "fdtd_state_bytes": [vp, C.POINTER(C.c_uint64)], "fdtd_save_state": [vp, vp, C.c_uint64],
            "fdtd_load_state": [vp, vp, C.c_uint64],
            "fdtd_check_finite": [vp, C.POINTER(C.c_int64)], "fdtd_debug_fail_alloc": [i32],
            "fdtd_debug_wait_limit": [vp, i32],
            "fdtd_add_pml": [vp, vp], "fdtd_add_tfsf_1d": [vp, vp], "fdtd_add_tfsf": [vp, vp],
            "fdtd_add_source": [vp, vp, C.POINTER(i32)], "fdtd_add_monitor": [vp, vp, C.POINTER(i32)],
            "fdtd_add_probe": [vp, vp, C.POINTER(i32)], "fdtd_commit": [vp],
            "fdtd_step": [vp, i32, i32], "fdtd_update_DE": [vp, i32], "fdtd_pml_update_E": [vp, i32],
            "fdtd_interchange": [vp, i32], "fdtd_update_H": [vp, i32], "fdtd_pml_update_H": [vp, i32],
            "fdtd_sample": [vp, i32], "fdtd_sync": [vp],
            "fdtd_get_field": [vp, i32, vp], "fdtd_set_field": [vp, i32, vp],
            "fdtd_get_monitor": [vp, i32, vp, vp], "fdtd_get_probe": [vp, i32, vp, C.POINTER(i32)],
            "fdtd_device_bytes": [vp, C.POINTER(C.c_uint64)], "fdtd_profile": [vp, i32],
            "fdtd_estimate_bytes": [vp, C.POINTER(C.c_uint64)],
            "fdtd_kernel_time": [vp, i32, C.POINTER(C.c_int64), C.POINTER(dbl)],
            "fdtd_kernel_cells": [vp, i32, C.POINTER(C.c_int64)],
            "fdtd_set_tile": [vp, i32], "fdtd_get_tile": [vp, C.POINTER(i32)],
            "fdtd_launch_count": [vp, C.POINTER(C.c_int64)],
            "fdtd_set_stream": [vp, vp],
            "fdtd_transfer_bytes": [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)],
            "fdtd_dft_sample_noalloc": [vp, i32, i32, i32, i32, C.POINTER(i32), C.POINTER(i32), i32, i32, i32,
                                        dbl, vp, i32, vp, vp, i32, vp],
            "fdtd_server_create": [vp, C.POINTER(vp)], "fdtd_server_submit": [vp, vp, i32, C.POINTER(C.c_int64)],
            "fdtd_server_wait": [vp, C.c_int64, i32, C.POINTER(i32)],
            "fdtd_server_job": [vp, C.c_int64, C.POINTER(vp)],
            "fdtd_server_times": [vp, C.c_int64, C.POINTER(dbl), C.POINTER(dbl), C.POINTER(dbl)],
            "fdtd_server_release": [vp, C.c_int64], "fdtd_server_stats": [vp, vp],
            "fdtd_server_destroy": [vp],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = L
    return _lib


def dft_sample_noalloc(field_ptr, precision, shape_xyz, lo, hi, n, n_first, n_last, dt, omega_ptr, nfreq,
                       acc_re_ptr, acc_im_ptr, flush=False, stream=None):
    """fdtd_dft_sample_noalloc on caller-owned device memory (all *_ptr are
    device addresses); the library allocates nothing on this call."""
    lo3 = (C.c_int32 * 3)(*lo)
    hi3 = (C.c_int32 * 3)(*hi)
    nx, ny, nz = shape_xyz
    check(lib().fdtd_dft_sample_noalloc(field_ptr, int(precision), int(nx), int(ny), int(nz), lo3, hi3, int(n),
                                        int(n_first), int(n_last), float(dt), omega_ptr, int(nfreq), acc_re_ptr,
                                        acc_im_ptr, 1 if flush else 0, stream))


def last_error():
    buf = C.create_string_buffer(512)
    lib().fdtd_last_error(buf, 512)
    return buf.value.decode()


def check(rc):
    if rc != abi.FDTD_OK:
        raise FdtdError(rc, last_error())
    return rc


def fail_alloc_after(n):
    """fdtd_debug_fail_alloc: the device allocation after ``n`` more
    successful ones fails with FDTD_ENOMEM (-1: none)."""
    check(lib().fdtd_debug_fail_alloc(int(n)))


def device_count():
    n = C.c_int32(0)
    check(lib().fdtd_device_count(C.byref(n)))
    return n.value


class Job:
    """One simulation on the GPU, built from a ``JobSpec``."""

    def __init__(self, spec, commit=True, tile=0):
        """Builds the job on the device.  With commit=False the set-up calls
        are made but nothing is allocated: the handle can then be handed to
        a Server (``detach``), which commits it when it admits the job."""
        self.spec = spec
        L = lib()
        g = spec.grid_desc()
        h = C.c_void_p()
        check(L.fdtd_create(C.byref(g), C.byref(h)))
        self.h = h
        keep = []
        mid = C.c_int32()
        try:
            for m in spec.materials:
                r = S.region_struct(m.region, keep)
                if m.kind == "dielectric":
                    check(L.fdtd_add_dielectric(self.h, C.byref(r), m.eps, C.byref(mid)))
                elif m.kind == "gold":
                    p = S.drude2cp_struct(m.params)
                    check(L.fdtd_add_gold(self.h, C.byref(r), C.byref(p), C.byref(mid)))
                elif m.kind == "lorentz":
                    p = S.lorentz_struct(m.params)
                    check(L.fdtd_add_lorentz(self.h, C.byref(r), C.byref(p), C.byref(mid)))
                elif m.kind == "graphene_nk":
                    p = S.graphene_nk_struct(m.params)
                    check(L.fdtd_add_graphene_nk(self.h, C.byref(r), C.byref(p), C.byref(mid)))
                elif m.kind == "conductive":
                    check(L.fdtd_add_conductive(self.h, C.byref(r), m.params["eps_inf"], m.params["sigma"],
                                                C.byref(mid)))
                elif m.kind == "graphene_cp":
                    p = S.graphene_cp_struct(m.params)
                    check(L.fdtd_add_graphene_cp(self.h, C.byref(r), C.byref(p), C.byref(mid)))
                else:
                    p = S.graphene_struct(m.params)
                    check(L.fdtd_add_graphene(self.h, C.byref(r), C.byref(p), C.byref(mid)))
            if spec.pml:
                p = S.pml_struct(spec.pml)
                check(L.fdtd_add_pml(self.h, C.byref(p)))
            if spec.tfsf:
                t = S.tfsf_struct(spec.tfsf)
                check(L.fdtd_add_tfsf_1d(self.h, C.byref(t)))
            if spec.tfsf_box:
                t = S.tfsf_box_struct(spec.tfsf_box)
                check(L.fdtd_add_tfsf(self.h, C.byref(t)))
            for s in spec.sources:
                d = S.source_struct(s)
                check(L.fdtd_add_source(self.h, C.byref(d), C.byref(mid)))
            for m in spec.monitors:
                d = S.monitor_struct(m, keep)
                check(L.fdtd_add_monitor(self.h, C.byref(d), C.byref(mid)))
            for p in spec.probes:
                d = S.probe_struct(p)
                check(L.fdtd_add_probe(self.h, C.byref(d), C.byref(mid)))
            if tile:
                check(L.fdtd_set_tile(self.h, int(tile)))
            if commit:
                check(L.fdtd_commit(self.h))
        except Exception:
            self.close()
            raise
        self.n_done = 0
        self.owned = True

    @classmethod
    def view(cls, handle, spec):
        """A non-owning wrapper of a job handle held elsewhere (a Server)."""
        j = cls.__new__(cls)
        j.spec, j.h, j.n_done, j.owned = spec, C.c_void_p(handle), 0, False
        return j

    def detach(self):
        """Gives up ownership of the handle (to a Server) and returns it."""
        h, self.h = self.h, None
        return h

    # -- the time loop ---------------------------------------------------
    def step(self, n_first, n_steps):
        check(lib().fdtd_step(self.h, int(n_first), int(n_steps)))
        self.n_done = n_first + n_steps - 1

    def run(self, n_steps):
        self.step(self.n_done + 1, n_steps)

    def step_procedures(self, n):
        """One step through the per-procedure entry points, in the order of
        the reference's loop body (3D/.../program.f90:389-540)."""
        L = lib()
        check(L.fdtd_update_DE(self.h, n))
        check(L.fdtd_pml_update_E(self.h, n))
        check(L.fdtd_interchange(self.h, 0))
        check(L.fdtd_update_H(self.h, n))
        check(L.fdtd_pml_update_H(self.h, n))
        check(L.fdtd_interchange(self.h, 1))
        check(L.fdtd_sample(self.h, n))
        self.n_done = n

    def sync(self):
        check(lib().fdtd_sync(self.h))

    # -- results ---------------------------------------------------------
    def get_field(self, comp):
        n = self.spec.n
        cnt = S.field_count(self.spec, comp)
        out = np.empty(cnt)
        check(lib().fdtd_get_field(self.h, int(comp), out.ctypes.data))
        return out if cnt != self.spec.cells() else out.reshape(n[2], n[1], n[0])

    def set_field(self, comp, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        check(lib().fdtd_set_field(self.h, int(comp), a.ctypes.data))

    def get_monitor(self, mid, out=None):
        """The monitor's running sums (re, im), each [comp][freq][cell].
        ``out``: an (re, im) pair of contiguous float64 arrays of that size
        (e.g. views of pinned host memory) to download into, else new arrays."""
        nc, nf, ncell = S.monitor_shape(self.spec.monitors[mid])
        if out is None:
            re = np.empty(nc * nf * ncell)
            im = np.empty_like(re)
        else:
            re, im = out
            for a in (re, im):
                if a.dtype != np.float64 or a.size != nc * nf * ncell or not a.flags.c_contiguous:
                    raise ValueError(f"monitor {mid} needs contiguous float64 arrays of {nc * nf * ncell}")
        check(lib().fdtd_get_monitor(self.h, int(mid), re.ctypes.data, im.ctypes.data))
        return re.reshape(nc, nf, ncell), im.reshape(nc, nf, ncell)

    def get_probe(self, pid):
        cnt = C.c_int32()
        check(lib().fdtd_get_probe(self.h, int(pid), None, C.byref(cnt)))
        ncomp = len(set(self.spec.probes[pid].comps))
        out = np.empty(max(1, cnt.value * ncomp))
        check(lib().fdtd_get_probe(self.h, int(pid), out.ctypes.data, C.byref(cnt)))
        return out[: cnt.value * ncomp].reshape(cnt.value, ncomp)

    def debug_wait_limit(self, rounds):
        """fdtd_debug_wait_limit: polls of a TMA core's mbarrier before its
        wait gives up (-1: the default)."""
        check(lib().fdtd_debug_wait_limit(self.h, int(rounds)))

    def count_nonfinite(self):
        """NaN and infinite values in the job's evolving state."""
        n = C.c_int64()
        check(lib().fdtd_check_finite(self.h, C.byref(n)))
        return n.value

    def save_state(self):
        """The job's evolving state at this step boundary (fdtd_save_state)."""
        n = C.c_uint64()
        check(lib().fdtd_state_bytes(self.h, C.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        check(lib().fdtd_save_state(self.h, buf.ctypes.data, n.value))
        return buf

    def load_state(self, buf):
        """Restore a state saved from a job of the same description."""
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        check(lib().fdtd_load_state(self.h, buf.ctypes.data, buf.size))

    def device_bytes(self):
        b = C.c_uint64()
        check(lib().fdtd_device_bytes(self.h, C.byref(b)))
        return b.value

    def estimate_bytes(self):
        b = C.c_uint64()
        check(lib().fdtd_estimate_bytes(self.h, C.byref(b)))
        return b.value

    def profile(self, enable=True):
        check(lib().fdtd_profile(self.h, 1 if enable else 0))

    def kernel_time(self, kind):
        n, ms = C.c_int64(), C.c_double()
        check(lib().fdtd_kernel_time(self.h, int(kind), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def tile(self):
        t = C.c_int32()
        check(lib().fdtd_get_tile(self.h, C.byref(t)))
        return t.value

    def kernel_cells(self, kind):
        c = C.c_int64()
        check(lib().fdtd_kernel_cells(self.h, int(kind), C.byref(c)))
        return c.value

    def launch_count(self):
        n = C.c_int64()
        check(lib().fdtd_launch_count(self.h, C.byref(n)))
        return n.value

    def set_stream(self, cuda_stream):
        """Queue the job's work on a caller-owned CUDA stream (an int handle)."""
        check(lib().fdtd_set_stream(self.h, C.c_void_p(cuda_stream)))

    def transfer_bytes(self):
        h, d = C.c_uint64(), C.c_uint64()
        check(lib().fdtd_transfer_bytes(self.h, C.byref(h), C.byref(d)))
        return h.value, d.value

    def close(self):
        if getattr(self, "h", None) and getattr(self, "owned", True):
            lib().fdtd_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
