"""The writer of the reference program's output files (fdtd_gpu.outputs) on
CPU: Fortran edit descriptors, the per-rank split, and a write / read round
trip through the parser that reads the reference's own files."""
import os
import sys

import numpy as np

from fdtd_gpu import outputs, problems

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden_2d import load_table  # noqa: E402


def test_fortran_edit_descriptors():
    assert outputs.fortran_e(0.375, 30, 19) == "0.3750000000000000000E+00".rjust(30)
    assert outputs.fortran_e(2.0 ** -60, 30, 19) == "0.8673617379884035472E-18".rjust(30)
    assert outputs.fortran_e(-2.0, 20, 10) == "-0.2000000000E+01".rjust(20)
    assert outputs.fortran_e(0.0, 20, 10) == "0.0000000000E+00".rjust(20)
    assert outputs.fortran_e(3.0e-120, 20, 10) == "0.3000000000-119".rjust(20)  # no E for 3-digit exponents
    assert outputs.fortran_f(0.25, 15, 5) == "        0.25000"
    assert len(outputs.fortran_f(-1.0e-6, 30, 19)) == 30


def test_rank_split_matches_the_reference_decomposition():
    assert outputs.rank_rows(1266, 3) == [(0, 422), (422, 844), (844, 1266)]
    assert outputs.rank_rows(10, 3) == [(0, 4), (4, 7), (7, 10)]


def test_write_read_round_trip(tmp_path):
    spec, meta = problems.reference_2d()
    rng = np.random.default_rng(0)
    nf, nx, ny = len(meta["arg"]), meta["nx"], meta["ny"]
    mons = [(rng.standard_normal((2, nf, nx)), rng.standard_normal((2, nf, nx))) for _ in range(3)]
    probes = [rng.standard_normal((5, 2)) for _ in range(3)]
    frames = {3: (rng.standard_normal((ny, nx)), rng.standard_normal((ny, nx)))}
    outputs.write_reference_2d(str(tmp_path), meta, mons, probes, frames)
    tr = tmp_path / "transforms"
    t = load_table(str(tr / "r0Syin.dat"))
    np.testing.assert_array_equal(t[:, 1], problems.poynting_2d_te(*mons[0], meta["ds"]))
    inf = load_table(str(tr / "r0infld.dat"))
    np.testing.assert_array_equal(inf[:, 1:], probes[0])
    np.testing.assert_allclose(inf[:, 0], np.arange(1, 6) * meta["dt"], rtol=1e-15)
    rf = load_table(str(tr / "r0rfld.dat"))     # F30.19: 19 decimals
    np.testing.assert_allclose(rf[:, 1:], probes[1], atol=1e-19)
    assert (tr / "r2tfld.dat").exists() and (tr / "r2Syt.dat").exists() and (tr / "r0tf_r.dat").exists()
    line = np.concatenate([load_table(str(tmp_path / "timesLiney" / f"r{k}E_time3.dat")) for k in range(3)])
    np.testing.assert_array_equal(line[:, 1], frames[3][0][:, meta["ic"] - 1])
    m = load_table(str(tmp_path / "timesGnuplotmap" / "r1E_time3.dat"))
    assert m.shape == (422 * nx, 3) and m[0, 0] == 1.0 and m[0, 1] == 423.0
    np.testing.assert_array_equal(m[:, 2], frames[3][1][422:844].ravel())


def test_cal_r_sy_on_written_spectra(tmp_path):
    """calR_Sy restated: the RTA rows computed from the written per-rank Sy
    files equal R, T, A of the in-memory spectra bit for bit (the files keep
    17 significant digits), and the file it writes reads back the same."""
    spec, meta = problems.reference_2d()
    rng = np.random.default_rng(1)
    nf, nx, ny = len(meta["arg"]), meta["nx"], meta["ny"]
    mons = [(rng.standard_normal((2, nf, nx)), rng.standard_normal((2, nf, nx))) for _ in range(3)]
    probes = [rng.standard_normal((2, 2)) for _ in range(3)]
    outputs.write_reference_2d(str(tmp_path), meta, mons, probes, {})
    rows = outputs.cal_r_sy(str(tmp_path / "transforms"))
    sy = [problems.poynting_2d_te(*m, meta["ds"]) for m in mons]
    r, t, a = outputs.rta(*sy)
    np.testing.assert_array_equal(rows[:, 1:], np.stack([r, t, a], 1))
    back = load_table(str(tmp_path / "transforms" / "RTA_2Dfdtd.data"))
    np.testing.assert_array_equal(back, rows)


def test_write_read_round_trip_3d(tmp_path):
    """The 3D program's files: per-step records (7E30.19, exact for doubles),
    Sy spectra in the program's summation order, tf_r at k = kc, the y-line
    frames (7F10.5) split over the six y-ranks, and calR_Sy's RTA on them."""
    spec, meta = problems.reference_3d()
    rng = np.random.default_rng(2)
    nf, nx, ny, nz = len(meta["arg"]), meta["nx"], meta["ny"], meta["nz"]
    mons = [(rng.standard_normal((4, nf, nx * nz)), rng.standard_normal((4, nf, nx * nz))) for _ in range(3)]
    probes = [rng.standard_normal((n, 6)) for n in (5, 7, 3)]
    lines = {2: rng.uniform(-1, 1, (6, ny))}
    outputs.write_reference_3d(str(tmp_path), meta, mons, probes, lines)
    tr = tmp_path / "transforms"
    assert outputs.rank_rows(ny, 6)[0] == (0, 211)
    for name, q, k in (("infld", 0, 0), ("tfld", 1, 5), ("rfld", 2, 0)):
        t = load_table(str(tr / f"r{k}{name}.dat"))
        np.testing.assert_array_equal(t[:, 1:], probes[q])
        first = meta["probe_first"][q]
        np.testing.assert_allclose(t[:, 0], np.arange(first, first + len(probes[q])) * meta["dt"], rtol=1e-15)
    for name, q, k in (("Syin", 0, 0), ("Syr", 1, 0), ("Syt", 2, 5)):
        t = load_table(str(tr / f"r{k}{name}.dat"))
        np.testing.assert_array_equal(t[:, 1], outputs.poynting_3d_ordered(*mons[q], meta["ds"]))
    np.testing.assert_allclose(outputs.poynting_3d_ordered(*mons[0], meta["ds"]),
                               problems.poynting_3d_y(*mons[0], meta["ds"]), rtol=1e-12)
    tf = load_table(str(tr / "r0tf_r.dat"))
    assert tf.shape == (nf * nx, 6)
    re, im = mons[1]
    c = np.arange(nx) + nx * (meta["kc"] - 1)
    np.testing.assert_allclose(tf[:nx, 2], re[2, 0, c] * re[1, 0, c], rtol=5.01e-10)
    np.testing.assert_allclose(tf[:nx, 5], im[3, 0, c] * im[0, 0, c], rtol=5.01e-10)
    line = np.concatenate([load_table(str(tmp_path / "timesLiney" / f"r{k}E_time2.dat")) for k in range(6)])
    assert line.shape == (ny, 7)
    np.testing.assert_allclose(line[:, 1:].T, lines[2], atol=5.01e-6)
    rows = outputs.cal_r_sy(str(tr), inc=0, ref=0, tras=5, out_name="RTA_3Dfdtd.data")
    sy = [outputs.poynting_3d_ordered(*m, meta["ds"]) for m in mons]
    np.testing.assert_array_equal(rows[:, 1:], np.stack(outputs.rta(*sy), 1))
