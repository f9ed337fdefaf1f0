"""The reference 2D program's output files, written from a run of the engine.

The reference's post-processing -- transforms/calR_Sy.f90, which reads the
Sy spectra and writes RTA_2Dfdtd.data, and the gnuplot scripts that read the
frame files -- reads per-rank text files named after the MPI rank that held
each line or point (2D/.../program.f90:296-320, 370-470, 477-530).  The
engine runs the whole domain at once; ``write_reference_2d`` splits its
results by the reference's row decomposition and writes the same files, in
the same record layout, so those tools run unchanged:

  transforms/r<k>infld.dat, r<k>rfld.dat, r<k>tfld.dat   per-step probes
  transforms/r<k>Syin.dat, r<k>Syr.dat, r<k>Syt.dat       Sy per wavelength
  transforms/r<k>tf_r.dat                                 per-x products
  timesLiney/r<k>E_time<f>.dat                            Ex, Hz along x=ic
  timesGnuplotmap/r<k>E_time<f>.dat                       Hz maps

``cal_r_sy`` then does what transforms/calR_Sy.f90 does with those files:
R = -Syr/Syin, T = Syt/Syin, A = 1 - R - T per wavelength, written to
RTA_2Dfdtd.data (3D/.../transforms/calR_Sy.f90:16-35).

Free-format records use a full-precision exponent form that Fortran
list-directed input reads; the fixed-format records follow the reference's
edit descriptors (E30.19, F30.19, F15.5, E20.10).

``write_reference_3d`` does the same for the 3D program
(3D/.../program.f90:355-378, 436-690; fileid_tracks.txt): per-step records of
all six components at the incident, reflected and transmitted points
(7E30.19), the Sy spectra, the tf_r products of the row k = kc
(2F15.5,4E20.10) and the timesLiney frames along y at (ic, kc) (7F10.5),
over its six y-ranks.  The program's maps and VTK frames are switched off
(printTimesMap, printTimesVTK = .false., program.f90:13-15) and so are not
written.
"""
import math
import os

import numpy as np

from . import problems

NANO = 1e-9


def fortran_e(x, w, d):
    """Fortran Ew.d: 0.<d digits>E+xx (three-digit exponents drop the E)."""
    if x == 0.0 or not math.isfinite(x):
        body, exp = "0." + "0" * d, 0
    else:
        s = f"{abs(x):.{d - 1}e}"           # d significant digits, rounded once
        mant, e = s.split("e")
        body = "0." + mant.replace(".", "")
        exp = int(e) + 1
    ex = f"E{exp:+03d}" if abs(exp) < 100 else f"{exp:+04d}"
    s = ("-" if x < 0 else "") + body + ex
    return s.rjust(w)


def fortran_f(x, w, d):
    """Fortran Fw.d."""
    return f"{x:{w}.{d}f}"


def free(*vals):
    """One list-directed record: every value with 17 significant digits."""
    return " ".join(f"{v: .17E}" for v in vals)


def rank_rows(ny, nranks):
    """Global 0-based row ranges [a, b) of each rank (rows split evenly, the
    remainder to the first ranks, as the reference's set_index does)."""
    base, extra = divmod(ny, nranks)
    out, a = [], 0
    for r in range(nranks):
        b = a + base + (1 if r < extra else 0)
        out.append((a, b))
        a = b
    return out


def owner(rows, j):
    return next(r for r, (a, b) in enumerate(rows) if a <= j < b)


def write_reference_2d(outdir, meta, monitors, probes, frames, nranks=3):
    """Writes the reference 2D program's files under ``outdir``.

    meta      the meta dict of ``problems.reference_2d()``
    monitors  [(re, im)] of its three monitors (incident, reflected,
              transmitted), each of shape (2, nfreq, nx) for (Ex, Hz)
    probes    [samples] of its three probes, each (steps, 2) for (Ex, Hz),
              starting at the probe's first step
    frames    {frame: (ex, hz)} full 2D fields (ny, nx) at step frame*dn
    """
    ds, dt = meta["ds"], meta["dt"]
    ny, nx = meta["ny"], meta["nx"]
    rows = rank_rows(ny, nranks)
    tr = os.path.join(outdir, "transforms")
    os.makedirs(tr, exist_ok=True)
    os.makedirs(os.path.join(outdir, "timesLiney"), exist_ok=True)
    os.makedirs(os.path.join(outdir, "timesGnuplotmap"), exist_ok=True)
    pts = meta["probe_cells"]  # [(i, j)] 0-based: incident, reflected, transmitted
    firsts = meta["probe_first"]

    # ---- per-step probes (program.f90:376-378, 397-399, 417-419) ----
    for q, name in enumerate(("infld", "rfld", "tfld")):
        i, j = pts[q]
        k = owner(rows, j)
        with open(os.path.join(tr, f"r{k}{name}.dat"), "w") as fh:
            for s, (e, h) in enumerate(probes[q]):
                n = firsts[q] + s
                if name == "infld":
                    fh.write(free(n * dt, e, h) + "\n")
                else:  # '(E30.19,4F30.19)'
                    fh.write(fortran_e(n * dt, 30, 19) + fortran_f(e, 30, 19) + fortran_f(h, 30, 19) + "\n")

    # ---- spectra (program.f90:477-530) ----
    lam = 2.0 * math.pi * problems.C0 / np.asarray(meta["arg"]) / NANO
    sy = [problems.poynting_2d_te(re, im, ds) for re, im in monitors]
    for q, name in enumerate(("Syin", "Syr", "Syt")):
        k = owner(rows, pts[q][1])
        with open(os.path.join(tr, f"r{k}{name}.dat"), "w") as fh:
            for m in range(len(lam)):
                fh.write(free(lam[m], sy[q][m]) + "\n")
    k = owner(rows, pts[1][1])
    re, im = monitors[1]
    with open(os.path.join(tr, f"r{k}tf_r.dat"), "w") as fh:  # '(2F15.5,2E20.10)' per x, blank per m
        for m in range(len(lam)):
            for i in range(nx):
                fh.write(fortran_f(lam[m], 15, 5) + fortran_f((i + 1) * ds / NANO, 15, 5) +
                         fortran_e(re[0, m, i] * re[1, m, i], 20, 10) + fortran_e(im[1, m, i] * im[0, m, i], 20, 10) + "\n")
            fh.write("\n")

    # ---- frames (program.f90:436-469) ----
    ic = meta["ic"] - 1
    for f, (ex, hz) in frames.items():
        for k, (a, b) in enumerate(rows):
            with open(os.path.join(outdir, "timesLiney", f"r{k}E_time{f}.dat"), "w") as fh:
                for j in range(a, b):
                    fh.write(free((j + 1) * ds / NANO, ex[j, ic], hz[j, ic]) + "\n")
            with open(os.path.join(outdir, "timesGnuplotmap", f"r{k}E_time{f}.dat"), "w") as fh:
                for j in range(a, b):
                    for i in range(nx):
                        fh.write(free(float(i + 1), float(j + 1), hz[j, i]) + "\n")
                    fh.write("\n")


def read_free(path):
    """Rows of a list-directed text file (blank lines skipped)."""
    rows = []
    with open(path) as fh:
        for line in fh:
            f = line.replace("D", "E").replace("d", "e").split()
            if f:
                rows.append([float(x) for x in f])
    return np.asarray(rows, dtype=np.float64)


def rta(syin, syr, syt):
    """r = -y1/y0, t = y2/y0, a = 1 - r - t (calR_Sy.f90:27-35)."""
    syin, syr, syt = (np.asarray(x, dtype=np.float64) for x in (syin, syr, syt))
    r = -syr / syin
    t = syt / syin
    return r, t, 1.0 - r - t


def cal_r_sy(transforms_dir, inc=0, ref=0, tras=2, out_name="RTA_2Dfdtd.data"):
    """calR_Sy on the per-rank spectra under ``transforms_dir``: the ranks
    that hold the incident, reflected and transmitted planes are the
    reference's config.xml entries <inc>, <ref>, <tras>.  Writes
    ``out_name`` (x0, r, t, a per line) beside them and returns its rows."""
    y0 = read_free(os.path.join(transforms_dir, f"r{inc}Syin.dat"))
    y1 = read_free(os.path.join(transforms_dir, f"r{ref}Syr.dat"))
    y2 = read_free(os.path.join(transforms_dir, f"r{tras}Syt.dat"))
    n = min(len(y0), len(y1), len(y2))
    r, t, a = rta(y0[:n, 1], y1[:n, 1], y2[:n, 1])
    rows = np.stack([y0[:n, 0], r, t, a], 1)
    with open(os.path.join(transforms_dir, out_name), "w") as fh:
        for row in rows:
            fh.write(free(*row) + "\n")
    return rows


def poynting_3d_ordered(re, im, ds):
    """Sy per frequency in the program's summation order (k outer, i inner;
    program.f90:613-685); re/im: (4, nfreq, ncell) with (Ex, Ez, Hx, Hz)."""
    ex, ez, hx, hz = 0, 1, 2, 3
    nf, nc = re.shape[1], re.shape[2]
    out = np.zeros(nf)
    for m in range(nf):
        s = 0.0
        for c in range(nc):
            s = s + ((re[hx, m, c] * re[ez, m, c]) + (im[hx, m, c] * im[ez, m, c]) -
                     (re[hz, m, c] * re[ex, m, c]) - (im[hz, m, c] * im[ex, m, c])) * ds
        out[m] = s
    return out


def write_reference_3d(outdir, meta, monitors, probes, lines, nranks=6):
    """Writes the reference 3D program's files under ``outdir``.

    meta      the meta dict of ``problems.reference_3d()``
    monitors  [(re, im)] of its three plane monitors (incident, reflected,
              transmitted), each (4, nfreq, nx*nz) for (Ex, Ez, Hx, Hz)
    probes    [samples] of its three probes (infld, tfld, rfld), each
              (steps, 6) for (Ex, Ey, Ez, Hx, Hy, Hz), from the probe's first
              step (meta["probe_first"])
    lines     {frame: (6, ny)} the six components along y at (ic, kc) at
              step frame*dn
    """
    ds, dt = meta["ds"], meta["dt"]
    nx, ny, nz = meta["nx"], meta["ny"], meta["nz"]
    rows = rank_rows(ny, nranks)
    tr = os.path.join(outdir, "transforms")
    os.makedirs(tr, exist_ok=True)
    os.makedirs(os.path.join(outdir, "timesLiney"), exist_ok=True)
    firsts = meta["probe_first"]
    ptiny, ptty, kc = meta["ptiny"] - 1, meta["ptty"] - 1, meta["kc"] - 1

    # ---- per-step records: write(2|3|4,'(7E30.19)') n*dt, ex..hz (:445-520) ----
    for q, (name, j) in enumerate((("infld", ptiny), ("tfld", ptty), ("rfld", ptiny))):
        k = owner(rows, j)
        with open(os.path.join(tr, f"r{k}{name}.dat"), "w") as fh:
            for s, vals in enumerate(probes[q]):
                n = firsts[q] + s
                fh.write(fortran_e(n * dt, 30, 19) + "".join(fortran_e(v, 30, 19) for v in vals) + "\n")

    # ---- spectra and tf_r (:613-685) ----
    lam = 2.0 * math.pi * problems.C0 / np.asarray(meta["arg"]) / NANO
    sy = [poynting_3d_ordered(re, im, ds) for re, im in monitors]
    for q, (name, j) in enumerate((("Syin", ptiny), ("Syr", ptiny), ("Syt", ptty))):
        with open(os.path.join(tr, f"r{owner(rows, j)}{name}.dat"), "w") as fh:
            for m in range(len(lam)):
                fh.write(free(lam[m], sy[q][m]) + "\n")
    re, im = monitors[1]
    ex, ez, hx, hz = 0, 1, 2, 3
    with open(os.path.join(tr, f"r{owner(rows, ptiny)}tf_r.dat"), "w") as fh:
        for m in range(len(lam)):
            for i in range(nx):
                c = i + nx * kc
                fh.write(fortran_f(lam[m], 15, 5) + fortran_f((i + 1) * ds / NANO, 15, 5) +
                         fortran_e(re[hx, m, c] * re[ez, m, c], 20, 10) + fortran_e(im[hx, m, c] * im[ez, m, c], 20, 10) +
                         fortran_e(re[hz, m, c] * re[ex, m, c], 20, 10) + fortran_e(im[hz, m, c] * im[ex, m, c], 20, 10) +
                         "\n")
            fh.write("\n")

    # ---- frames along y at (ic, kc): write(400+frame,'(7F10.5)') (:563-583) ----
    for f, line in lines.items():
        for k, (a, b) in enumerate(rows):
            with open(os.path.join(outdir, "timesLiney", f"r{k}E_time{f}.dat"), "w") as fh:
                for j in range(a, b):
                    fh.write(fortran_f((j + 1) * ds / NANO, 10, 5) +
                             "".join(fortran_f(line[u][j], 10, 5) for u in range(6)) + "\n")
