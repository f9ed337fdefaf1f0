"""Pins the FP64 oracle against the reference's own shipped 2D outputs.

The reference ships the outputs of FDTDsimulations/2D/air-nanoAntennas_
Si02-Sisubstrate/program.f90 (transforms/, timesLiney/, timesGnuplotmap/);
tests/golden/make_golden_2d.py converted them into golden_2d_ref.npz.  The
oracle replays the same program on one domain and must reproduce them to
the precision the files were printed with.
"""
import numpy as np
import pytest

from fdtd_gpu import abi, problems

GOLDEN = None


def golden():
    global GOLDEN
    if GOLDEN is None:
        import os
        GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_2d_ref.npz"))
    return GOLDEN


@pytest.fixture(scope="module")
def run2d(oracle_lib):
    spec, meta = problems.reference_2d()
    job = oracle_lib.OracleJob(spec, nthreads=1)
    ic = meta["ic"] - 1
    liney = np.zeros((20, meta["ny"], 2))
    maps = {}
    n = 0
    for f in range(1, 21):
        target = f * meta["dn"]
        job.step(n + 1, target - n)
        n = target
        ex = job.get_field(abi.EX)[0]
        hz = job.get_field(abi.HZ)[0]
        liney[f - 1, :, 0] = ex[:, ic]
        liney[f - 1, :, 1] = hz[:, ic]
        if f in (1, 20):
            maps[f] = hz.copy()
    job.step(n + 1, meta["Nt"] - n)
    out = dict(meta=meta, liney=liney, maps=maps)
    out["mon"] = [job.get_monitor(q) for q in range(3)]
    out["probe"] = [job.get_probe(q) for q in range(3)]
    return out


def test_run_parameters_match_reference_log():
    # values printed by the reference run (P2/out.out:7-36)
    spec, meta = problems.reference_2d()
    assert repr(meta["sigmam"]) == "2.398939398849712e+17"
    assert repr(meta["dt"]) == "6.669614083487051e-18"
    assert repr(meta["ds"]) == "3.999000000000001e-09"
    assert (meta["Nt"], meta["dn"], meta["tfinStop"], meta["ptty"]) == (13696, 684, 3424, 1170)
    assert meta["au"] == {"x": (50, 74), "y": (1008, 1012)}
    assert meta["si"]["y"] == (1084, 1256) and meta["sio2"]["y"] == (1013, 1083)


def test_poynting_spectra_bit_exact(run2d):
    g = golden()
    ds = run2d["meta"]["ds"]
    for q, key in enumerate(("syin", "syr", "syt")):
        re, im = run2d["mon"][q]
        sy = problems.poynting_2d_te(re, im, ds)
        np.testing.assert_array_equal(sy, g[key][:, 1])
    lam = 2.0 * problems.PI * problems.C0 / run2d["meta"]["arg"] / problems.NANO
    np.testing.assert_allclose(lam, g["syin"][:, 0], rtol=1e-15)


def test_rta(run2d):
    g = golden()
    ds = run2d["meta"]["ds"]
    sy = [problems.poynting_2d_te(*run2d["mon"][q], ds) for q in range(3)]
    r = -sy[1] / sy[0]
    t = sy[2] / sy[0]
    a = 1.0 - r - t
    np.testing.assert_array_equal(np.stack([r, t, a], 1), g["rta"][:, 1:])


def test_tf_r_products(run2d):
    # r0tf_r.dat: ReEx*ReHz and ImHz*ImEx per x at the reflection line (E20.10)
    g = golden()["tf_r"]
    re, im = run2d["mon"][1]
    prod = np.stack([re[0] * re[1], im[1] * im[0]], -1).reshape(-1, 2)
    np.testing.assert_allclose(prod, g[:, 2:], rtol=5.01e-10, atol=1e-45)  # 10 significant digits


def test_time_series(run2d):
    g = golden()
    # r0infld.dat is list-directed (17 digits); r0rfld/r2tfld are F30.19
    np.testing.assert_array_equal(run2d["probe"][0], g["infld"][:, 1:])
    np.testing.assert_allclose(run2d["probe"][1], g["rfld"][:, 1:], rtol=0, atol=1e-19)
    np.testing.assert_allclose(run2d["probe"][2], g["tfld"][:, 1:], rtol=0, atol=1e-19)


def test_field_snapshots(run2d):
    g = golden()
    np.testing.assert_array_equal(run2d["liney"], g["liney"])
    for q, f in enumerate(g["map_frames"]):
        np.testing.assert_array_equal(run2d["maps"][int(f)], g["maps"][q])
