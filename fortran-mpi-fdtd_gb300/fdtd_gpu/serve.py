"""Serving: many FDTD jobs continuously batched on one GPU.

``Server`` wraps the library's server (fdtd_server_*): jobs are submitted
as ``JobSpec``s; the server admits them by HBM footprint, advances every
admitted job on its own stream in chunks of whole 32-step rings, and keeps a
finished job's results until it is released.  ``poisson_mix`` draws the
serving workload: seeded Poisson arrivals of 2D TMz cylinder jobs and 3D
gold-sphere jobs.
"""
import ctypes as C
import math
import time

import numpy as np

from . import abi, problems
from .job import Job, check, lib


class Server:
    def __init__(self, hbm_budget=0, max_active=16, chunk_steps=256, pack_cells=0):
        """pack_cells: 2D jobs of at most this many cells share launches
        (0: the library's default, 2^20 cells; < 0: every job runs alone)."""
        d = abi.ServerDesc(hbm_budget=int(hbm_budget), max_active=int(max_active), chunk_steps=int(chunk_steps),
                           pack_cells=int(pack_cells))
        h = C.c_void_p()
        check(lib().fdtd_server_create(C.byref(d), C.byref(h)))
        self.h = h
        self.specs = {}

    def submit(self, spec, n_steps):
        """Queues a job; returns its ticket.  The server owns the job."""
        j = Job(spec, commit=False)
        t = C.c_int64()
        try:
            check(lib().fdtd_server_submit(self.h, j.h, int(n_steps), C.byref(t)))
        except Exception:
            j.close()
            raise
        j.detach()
        self.specs[t.value] = spec
        return t.value

    def wait(self, ticket, timeout_ms=-1):
        st = C.c_int32()
        check(lib().fdtd_server_wait(self.h, C.c_int64(ticket), int(timeout_ms), C.byref(st)))
        return st.value

    def job(self, ticket):
        """The finished job (non-owning view) for reading its results."""
        h = C.c_void_p()
        check(lib().fdtd_server_job(self.h, C.c_int64(ticket), C.byref(h)))
        return Job.view(h.value, self.specs[ticket])

    def times(self, ticket):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        check(lib().fdtd_server_times(self.h, C.c_int64(ticket), C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def release(self, ticket):
        check(lib().fdtd_server_release(self.h, C.c_int64(ticket)))
        self.specs.pop(ticket, None)

    def stats(self):
        s = abi.ServerStatus()
        check(lib().fdtd_server_stats(self.h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in abi.ServerStatus._fields_}

    def close(self):
        if getattr(self, "h", None):
            lib().fdtd_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_mix(count, rate_hz, seed=1, frac_2d=0.8, sizes_2d=(256, 512, 1024), sizes_3d=(128, 192, 256),
                steps=(2000, 8000), freqs=(32, 128), precision=abi.F32):
    """Seeded serving workload: (arrival time s, spec, n_steps) per job.

    80% 2D TMz jobs (N x N, N from sizes_2d, 1-20 gold cylinders) and 20% 3D
    gold spheres (N^3, N from sizes_3d); 2000-8000 steps and 32-128 DFT
    frequencies each, uniformly drawn; exponential inter-arrival times."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for q in range(count):
        t += rng.exponential(1.0 / rate_hz)
        nst = int(rng.integers(steps[0], steps[1] + 1))
        nf = int(rng.integers(freqs[0], freqs[1] + 1))
        if rng.random() < frac_2d:
            n = int(rng.choice(sizes_2d))
            ncyl = int(rng.integers(1, 21))
            npml = 16 if n <= 512 else 32
            spec, _ = problems.config_2d_tmz(precision=precision, n=n, steps=nst, ncyl=ncyl, nfreq=nf, npml=npml,
                                             seed=int(rng.integers(1 << 30)))
        else:
            n = int(rng.choice(sizes_3d))
            spec, _ = problems.config_3d_sphere(precision=precision, n=n, steps=nst, nfreq=nf, npml=12)
        out.append((t, spec, nst))
    return out


def percentile(xs, p):
    """Nearest-rank percentile (p in 0..100) of a non-empty list."""
    s = sorted(xs)
    k = max(1, math.ceil(p / 100.0 * len(s)))
    return s[k - 1]


def run_mix(server, mix, time_scale=1.0, on_done=None):
    """Submits the jobs of ``mix`` at their arrival times (scaled), waits for
    all, and returns per-job latencies (done - submit, seconds) and the
    wall time from the first submission to the last completion."""
    t0 = time.perf_counter()
    tickets = []
    for (ta, spec, nst) in mix:
        delay = ta * time_scale - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        tickets.append(server.submit(spec, nst))
    lat = []
    for tk in tickets:
        server.wait(tk)
        if on_done is not None:
            on_done(tk, server.job(tk))
        ts, _, td = server.times(tk)
        lat.append(td - ts)
        server.release(tk)
    wall = time.perf_counter() - t0
    return lat, wall
