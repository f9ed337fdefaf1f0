"""The C ABI from C: tests/c_driver/fdtd_driver.c builds a 2D TMz job (gold
cylinder, split PML, line source, line monitor, probe) through the plain C
interface, as a C or Fortran host would.  Without a device it must get
FDTD_ENODEV from fdtd_create; on a GB300 its results must equal those of the
same job built through the Python binding, bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from fdtd_gpu import abi, build, problems
from fdtd_gpu.spec import JobSpec, box, spheres

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    build.build()
    lib_dir = os.path.dirname(build.LIB)
    exe = str(tmp_path_factory.mktemp("c_driver") / "fdtd_driver")
    src = os.path.join(ROOT, "tests", "c_driver", "fdtd_driver.c")
    # -ffp-contract=off: the driver's sums round like the Python twin's (no fused multiply-add)
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), src, "-L", lib_dir,
                    "-lfdtd_gb300", "-Wl,-rpath," + lib_dir, "-lm", "-o", exe], check=True)
    return exe


def run(exe, prec, steps):
    out = subprocess.run([exe, str(prec), str(steps)], capture_output=True, text=True, check=True).stdout.split()
    if out == ["ENODEV"]:
        return None
    return {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}


def test_c_driver_runs(driver):
    res = run(driver, abi.F64, 50)
    if res is not None:  # a device is present: the job ran
        assert res["probe_count"] == 50 and np.isfinite(res["ez2"])


def python_twin(prec, steps):
    """The driver's job, built with the Python binding from the same numbers."""
    from fdtd_gpu import job
    n, npml, ds, ku = 96, 10, 1e-9, 0.5
    c0, pi = problems.C0, problems.PI
    spec = JobSpec(layout=abi.LAYOUT_2D_TM, n=(n, n, 1), ku=ku, dt=ku * ds / c0, ds=ds, precision=prec,
                   main_lo=(0, 0, 0), main_hi=(n - 1, n - 1, 0))
    spec.add_dielectric(box((0, 0, 0), (n - 1, n - 1, 0)), 1.0)
    spec.add_gold(spheres([(48.0, 52.0, 0.0, 8.0)]), problems.GOLD_REFERENCE)
    spec.pml = dict(mode=abi.PML_SPLIT, npml=((npml, npml), (npml, npml), (0, 0)), eps_lo=1.0, eps_hi=1.0,
                    sigma_max=4.0 * c0 * 16.0 / (2.0 * npml * ds), order=3.0)
    f0 = c0 / 600e-9
    st = 1.0 / f0
    spec.sources.append(dict(component=abi.EZ, lo=(npml, 20, 0), hi=(n - 1 - npml, 20, 0), amp=1.0, t0=4.0 * st,
                             st=st, w0=2.0 * pi * f0))
    omega = [2.0 * pi * c0 / (400e-9 + 50e-9 * m) for m in range(8)]
    spec.add_monitor((npml, 70, 0), (n - 1 - npml, 70, 0), (abi.EZ,), omega, 1, 1 << 30)
    spec.add_probe((48, 70, 0), (abi.EZ,), 1, 1 << 30)
    J = job.Job(spec)
    J.step(1, steps)
    ez = J.get_field(abi.EZ).ravel()
    re, im = (a.ravel() for a in J.get_monitor(0))
    pr = J.get_probe(0)[:, 0]
    J.close()
    s = sr = si = 0.0
    for v in ez:  # the driver's sums, in its order
        s += float(v) * float(v)
    for a, b in zip(re, im):
        sr += float(a)
        si += float(b)
    return {"ez2": s, "re": sr, "im": si, "probe_count": float(len(pr)), "probe_last": float(pr[-1])}


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
def test_c_driver_equals_python_binding(driver, prec):
    got = run(driver, prec, 300)
    assert got is not None, "no device"
    want = python_twin(prec, 300)
    assert got["ez2"] > 0
    assert got == want
