"""One small run of a configuration, for a profiler to capture.

    PYTHONPATH=fortran-mpi-fdtd_gb300 python -m fdtd_gpu.profcase 3d_sphere --n 256 --tile 5 --steps 40

The job's core block shape is pinned (``--tile``, see fdtd_set_tile) so that a
capture does not depend on the commit-time tuner's timing.  The steps run
eagerly with per-launch event timing; the kernels' times and cell counts are
printed as one JSON line.
"""
import argparse
import json

from . import abi, job, problems


def spec_for(case, n, precision):
    if case == "3d_sphere":
        return problems.config_3d_sphere(precision=precision, n=n, nfreq=64, npml=16)[0]
    if case == "2d_tmz":
        return problems.config_2d_tmz(precision=precision, n=n, steps=200)[0]
    if case == "3d_graphene":
        return problems.config_3d_graphene(precision=precision, nxy=n, nz=384)[0]
    raise ValueError(case)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["3d_sphere", "2d_tmz", "3d_graphene"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--tile", type=int, default=2)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--f64", action="store_true")
    a = ap.parse_args(argv)
    spec = spec_for(a.case, a.n, abi.F64 if a.f64 else abi.F32)
    J = job.Job(spec, tile=a.tile)
    J.profile(True)
    J.step(1, a.steps)
    J.sync()
    kinds = {"E": abi.KERNEL_E, "H": abi.KERNEL_H, "EDGE": abi.KERNEL_EDGE, "ADE": abi.KERNEL_ADE,
             "STEP": abi.KERNEL_STEP, "DFT": abi.KERNEL_DFT}
    out = {k: dict(zip(("launches", "ms"), J.kernel_time(v))) for k, v in kinds.items()}
    print(json.dumps(dict(case=a.case, n=a.n, tile=J.tile(), core_cells=J.kernel_cells(abi.KERNEL_E),
                          edge_cells=J.kernel_cells(abi.KERNEL_EDGE), step_cells=J.kernel_cells(abi.KERNEL_STEP),
                          kernels=out)))
    J.close()


if __name__ == "__main__":
    main()
