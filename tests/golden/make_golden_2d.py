"""Extract the 2D golden fixtures from the reference's shipped run outputs.

The reference ships the outputs of its 2D run (125 x 1266 cells, 13696 steps,
3 MPI ranks of 422 rows each):

  FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate/transforms/*.dat
  FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate/timesLiney/r{0,1,2}E_time{1..20}.dat
  FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate/timesGnuplotmap/r{0,1,2}E_time{k}.dat

They are written by program.f90:376-378 (r0infld), :397-399 (r0rfld),
:417-419 (r2tfld), :446-451 (timesLiney), :459-467 (timesGnuplotmap),
:477-530 (Sy spectra and tf_r).  This script parses them (Fortran
list-directed and fixed-format text) and stores them as one compressed
float64 archive, ``golden_2d_ref.npz``, that the tests read.  It runs only
where the reference checkout exists; the archive it writes is committed.

Usage:  python tests/golden/make_golden_2d.py /path/to/reference
"""
import os
import re
import sys

import numpy as np

P2 = "FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate"
NRANK, NY_RANK, NX = 3, 422, 125
MAP_FRAMES = (1, 20)

# Fortran drops the 'E' for three-digit exponents (1.0-100); restore it.
_EXP3 = re.compile(r"(\d)([+-]\d{3})(?!\d)")


def load_table(path):
    rows = []
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if not line:
                continue
            line = _EXP3.sub(r"\1E\2", line)
            rows.append([float(tok) for tok in line.split()])
    return np.asarray(rows, dtype=np.float64)


def main(ref_root):
    base = os.path.join(ref_root, P2)
    out = {}
    tr = os.path.join(base, "transforms")
    out["syin"] = load_table(os.path.join(tr, "r0Syin.dat"))
    out["syr"] = load_table(os.path.join(tr, "r0Syr.dat"))
    out["syt"] = load_table(os.path.join(tr, "r2Syt.dat"))
    out["rta"] = load_table(os.path.join(tr, "RTA_2Dfdtd.data"))
    out["infld"] = load_table(os.path.join(tr, "r0infld.dat"))
    out["rfld"] = load_table(os.path.join(tr, "r0rfld.dat"))
    out["tfld"] = load_table(os.path.join(tr, "r2tfld.dat"))
    out["tf_r"] = load_table(os.path.join(tr, "r0tf_r.dat"))

    # timesLiney: y[nm], Ex(ic,j), Hz(ic,j) for the rank's 422 rows; stitch
    # the three ranks into the global 1266-row line per frame.
    liney = np.zeros((20, NRANK * NY_RANK, 2))
    for f in range(1, 21):
        parts = [load_table(os.path.join(base, "timesLiney", f"r{r}E_time{f}.dat"))
                 for r in range(NRANK)]
        stitched = np.concatenate(parts, axis=0)
        assert stitched.shape == (NRANK * NY_RANK, 3), stitched.shape
        liney[f - 1] = stitched[:, 1:]
    out["liney"] = liney

    # timesGnuplotmap: x, y (global 1-based indices), Hz for every cell of
    # the rank; keep two full frames as (frame, y, x) arrays.
    maps = np.zeros((len(MAP_FRAMES), NRANK * NY_RANK, NX))
    for q, f in enumerate(MAP_FRAMES):
        for r in range(NRANK):
            t = load_table(os.path.join(base, "timesGnuplotmap", f"r{r}E_time{f}.dat"))
            assert t.shape == (NY_RANK * NX, 3), t.shape
            ix = t[:, 0].astype(int) - 1
            iy = t[:, 1].astype(int) - 1
            maps[q, iy, ix] = t[:, 2]
    out["map_frames"] = np.asarray(MAP_FRAMES, dtype=np.int64)
    out["maps"] = maps

    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_2d_ref.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")
    for k, v in out.items():
        print(f"  {k}: {v.shape}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden_2d.py <root of the reference project>")
    main(sys.argv[1])
