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
