"""GPU parity: the CUDA path through the C ABI against the FP64 oracle and
against the reference's own shipped 2D outputs.

FP64 plain path: relative L2 <= 1e-10 on fields, DFT sums and spectra.
FP32 path: DFT spectra relative L2 <= 1e-4 against the FP64 oracle.
"""
import math
import os

import numpy as np
import pytest

from fdtd_gpu import abi, problems

pytestmark = pytest.mark.gpu

NTH = os.cpu_count() or 1
TOL64 = 1e-10
TOL32_DFT = 1e-4


def rel_l2(a, b):
    """Relative L2 error of a against b.  A reference that is all zeros
    passes only a value that is all zeros too (a monitor gated off in both):
    any nonzero value against it is an infinite error, not a small one."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    if nb == 0:
        return 0.0 if not np.any(a) else float("inf")
    return np.linalg.norm(a - b) / nb


def check_state(J, O, comps, tol=TOL64, per_comp=1e-8):
    """A field snapshot is the whole state vector (all components): its
    relative L2 must be <= tol.  Each component on its own must be within
    per_comp (a component far smaller than the others, e.g. Hx under x
    polarisation, carries rounding noise of the dominant ones: per_comp=None
    checks the whole state only)."""
    a = [J.get_field(c) for c in comps]
    b = [O.get_field(c) for c in comps]
    assert any(np.any(x) for x in b), "the oracle's state is all zeros: nothing was driven"
    tot = rel_l2(np.concatenate([x.ravel() for x in a]), np.concatenate([x.ravel() for x in b]))
    assert tot <= tol, f"state rel L2 {tot:.3e}"
    for c, x, y in zip(comps, a, b):
        if per_comp is None:
            break
        e = rel_l2(x, y)
        assert e <= per_comp, f"component {c}: rel L2 {e:.3e}"


@pytest.fixture(scope="module")
def gpu():
    from fdtd_gpu import build, job
    build.build()
    if job.device_count() < 1:
        pytest.skip("no sm_103a device")
    return job


def golden():
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_2d_ref.npz"))


# ---------------------------------------------------------------------------
# 2D reference program: full 13696-step run against the shipped outputs
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def run2d_gpu(gpu):
    spec, meta = problems.reference_2d()
    J = gpu.Job(spec)
    ic = meta["ic"] - 1
    liney = np.zeros((20, meta["ny"], 2))
    maps, frames = {}, {}
    n = 0
    for f in range(1, 21):
        target = f * meta["dn"]
        J.step(n + 1, target - n)
        n = target
        ex = J.get_field(abi.EX)[0]
        hz = J.get_field(abi.HZ)[0]
        liney[f - 1, :, 0] = ex[:, ic]
        liney[f - 1, :, 1] = hz[:, ic]
        frames[f] = (ex.copy(), hz.copy())
        if f in (1, 20):
            maps[f] = hz.copy()
    J.step(n + 1, meta["Nt"] - n)
    out = dict(meta=meta, liney=liney, maps=maps, frames=frames, job=J)
    out["mon"] = [J.get_monitor(q) for q in range(3)]
    out["probe"] = [J.get_probe(q) for q in range(3)]
    return out


def test_2d_reference_spectra_match_shipped_outputs(run2d_gpu):
    g = golden()
    ds = run2d_gpu["meta"]["ds"]
    for q, key in enumerate(("syin", "syr", "syt")):
        sy = problems.poynting_2d_te(*run2d_gpu["mon"][q], ds)
        assert rel_l2(sy, g[key][:, 1]) <= TOL64, key
    sy = [problems.poynting_2d_te(*run2d_gpu["mon"][q], ds) for q in range(3)]
    rta = np.stack([-sy[1] / sy[0], sy[2] / sy[0]], 1)
    assert np.max(np.abs(rta - g["rta"][:, 1:3])) <= 1e-10


def test_2d_reference_fields_match_shipped_outputs(run2d_gpu):
    g = golden()
    for f in range(20):
        assert rel_l2(run2d_gpu["liney"][f], g["liney"][f]) <= TOL64, f
    for q, f in enumerate(g["map_frames"]):
        assert rel_l2(run2d_gpu["maps"][int(f)], g["maps"][q]) <= TOL64
    assert rel_l2(run2d_gpu["probe"][0], g["infld"][:, 1:]) <= TOL64
    assert rel_l2(run2d_gpu["probe"][2], g["tfld"][:, 1:]) <= TOL64
    assert rel_l2(run2d_gpu["probe"][1], g["rfld"][:, 1:]) <= 1e-9  # F30.19 print precision


def test_2d_reference_output_files_match_shipped_files(run2d_gpu, tmp_path):
    """The reference program's per-rank output files, written from the GPU
    run by fdtd_gpu.outputs and read back with the same parser that read the
    reference's shipped files, hold the shipped values."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden_2d import load_table
    from fdtd_gpu import outputs
    r = run2d_gpu
    probes = [p[:, :2] for p in r["probe"]]
    outputs.write_reference_2d(str(tmp_path), r["meta"], r["mon"], probes, r["frames"])
    g = golden()
    tr = tmp_path / "transforms"
    for key, fn in (("syin", "r0Syin.dat"), ("syr", "r0Syr.dat"), ("syt", "r2Syt.dat")):
        t = load_table(str(tr / fn))
        assert rel_l2(t[:, 1], g[key][:, 1]) <= TOL64, key
        np.testing.assert_allclose(t[:, 0], g[key][:, 0], rtol=1e-12)
    assert rel_l2(load_table(str(tr / "r0infld.dat")), g["infld"]) <= TOL64
    assert rel_l2(load_table(str(tr / "r2tfld.dat")), g["tfld"]) <= TOL64
    assert rel_l2(load_table(str(tr / "r0rfld.dat")), g["rfld"]) <= 1e-9
    np.testing.assert_allclose(load_table(str(tr / "r0tf_r.dat")), g["tf_r"], rtol=5.01e-10, atol=1e-30)
    rows = outputs.cal_r_sy(str(tr))          # transforms/calR_Sy.f90 on the written files
    assert rel_l2(rows[:, 1:], g["rta"][:, 1:]) <= TOL64
    for f in (1, 7, 20):
        parts = [load_table(str(tmp_path / "timesLiney" / f"r{k}E_time{f}.dat")) for k in range(3)]
        assert rel_l2(np.concatenate(parts)[:, 1:], g["liney"][f - 1]) <= TOL64
    for q, f in enumerate(g["map_frames"]):
        m = np.zeros_like(g["maps"][q])
        for k in range(3):
            t = load_table(str(tmp_path / "timesGnuplotmap" / f"r{k}E_time{int(f)}.dat"))
            m[t[:, 1].astype(int) - 1, t[:, 0].astype(int) - 1] = t[:, 2]
        assert rel_l2(m, g["maps"][q]) <= TOL64


def test_2d_per_procedure_path_equals_fused(gpu):
    spec, meta = problems.reference_2d()
    a, b = gpu.Job(spec), gpu.Job(spec)
    a.step(1, 700)
    for n in range(1, 701):
        b.step_procedures(n)
    for c in (abi.EX, abi.EY, abi.HZ):
        np.testing.assert_array_equal(a.get_field(c), b.get_field(c))
    for q in range(3):
        for x, y in zip(a.get_monitor(q), b.get_monitor(q)):
            np.testing.assert_array_equal(x, y)


def test_2d_reference_deterministic(gpu):
    spec, _ = problems.reference_2d()
    a, b = gpu.Job(spec), gpu.Job(spec)
    a.step(1, 1500)
    b.step(1, 1500)
    np.testing.assert_array_equal(a.get_field(abi.HZ), b.get_field(abi.HZ))
    np.testing.assert_array_equal(a.get_monitor(0)[0], b.get_monitor(0)[0])


# ---------------------------------------------------------------------------
# 3D and 1D reference programs against the oracle
# ---------------------------------------------------------------------------
def test_3d_reference_vs_oracle(gpu, oracle_lib):
    """The 3D reference program for its whole Nt = 13696 steps.

    By step 4500 the pulse has crossed the gold strip, the SiO2 layer and the
    Si substrate and has driven the high-y PML slab (setboundayEyb/Hyb,
    eps_hi = Si): there the whole state, slabs included, must match the
    oracle to 1e-10.  At Nt every monitor and probe, and every field outside
    the two PML slabs, must still match to 1e-10.  Inside the slabs the
    difference grows after the pulse has gone, about 7x per 2000 steps, in a
    build without fused multiply-adds as in this one: the reference's slab
    coupling (only Exy/Ezy are copied back to the main grid,
    3D/BERpmly_mod.f90:200-278) amplifies the last-bit differences that the
    E-form dielectric and gold updates make by design.  The slab rows are
    held to 1e-7 of the state's norm at Nt (and each driven component to
    1e-7 of its own)."""
    spec, meta = problems.reference_3d()
    assert meta["Nt"] == 13696
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec, nthreads=NTH)
    comps = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    mid = 4500
    J.step(1, mid)
    O.step(1, mid)
    # the strip is uniform along z and the source is Ex: the fields are Ex,
    # Ey and Hz, each held to 1e-8 on its own; Ez, Hx and Hy carry only the
    # rounding noise of those, far below them, which the whole-state
    # tolerance holds
    check_state(J, O, comps, per_comp=None)  # whole state <= 1e-10
    check_state(J, O, (abi.EX, abi.EY, abi.HZ))
    npml, ny = 10, meta["ny"]
    si_lo = spec.materials[3].region["lo"][1]  # first row of the Si substrate (0-based)
    for c in (abi.EX, abi.EY, abi.HZ):
        f = O.get_field(c)                    # [z][y][x]
        assert np.any(f[:, si_lo:ny - npml, :]), f"component {c}: Si substrate not driven"
    for c in (abi.EX, abi.HZ):  # the high slab's coupling row takes Exy / Hzy (setboundayEyb/Hyb)
        assert np.any(O.get_field(c)[:, ny - npml, :]), f"component {c}: high-y PML slab not driven"
    J.step(mid + 1, meta["Nt"] - mid)
    O.step(mid + 1, meta["Nt"] - mid)
    a = np.concatenate([J.get_field(c)[:, npml:ny - npml, :].ravel() for c in comps])
    b = np.concatenate([O.get_field(c)[:, npml:ny - npml, :].ravel() for c in comps])
    assert rel_l2(a, b) <= TOL64
    # the slab rows: the state's difference there to 1e-7 of the state's
    # norm, and each driven component's to 1e-7 of its own norm
    fj = {c: J.get_field(c) for c in comps}
    fo = {c: O.get_field(c) for c in comps}
    state = math.sqrt(sum(float(np.sum(fo[c] ** 2)) for c in comps))
    for rows in (slice(0, npml), slice(ny - npml, ny)):
        d = math.sqrt(sum(float(np.sum((fj[c] - fo[c])[:, rows, :] ** 2)) for c in comps))
        assert d <= 1e-7 * state, (rows, d, state)
        for c in (abi.EX, abi.EY, abi.HZ):
            assert np.linalg.norm((fj[c] - fo[c])[:, rows, :]) <= 1e-7 * np.linalg.norm(fo[c]), (c, rows)
    assert _dft_err(J, O, 3, live=(0, 1, 2)) <= TOL64
    for q in range(3):
        p = O.get_probe(q)
        assert np.any(p), f"probe {q} of the oracle is zero"
        assert rel_l2(J.get_probe(q), p) <= TOL64


def test_1d_reference_vs_oracle(gpu, oracle_lib):
    spec, meta = problems.reference_1d()
    steps = 12000
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec)
    J.step(1, steps)
    O.step(1, steps)
    check_state(J, O, (abi.EX, abi.HZ, abi.EX_INC, abi.HZ_INC))
    for q in range(2):
        for x, y in zip(J.get_monitor(q), O.get_monitor(q)):
            assert rel_l2(x, y) <= TOL64
        assert rel_l2(J.get_probe(q), O.get_probe(q)) <= TOL64


# ---------------------------------------------------------------------------
# benchmark workloads at reduced size: FP64 plain and FP32 against the oracle
# ---------------------------------------------------------------------------
def _dft_err(J, O, nmon, live=None):
    """Largest relative L2 error of the monitors' sums.  At least one monitor
    of the oracle must hold nonzero sums; the monitors listed in `live` must
    each hold them (a monitor gated off for the whole run may stay zero, and
    then the GPU's must be zero too)."""
    errs, norms = [], []
    for q in range(nmon):
        (jr, ji), (orr, oi) = J.get_monitor(q), O.get_monitor(q)
        ref = np.concatenate([orr.ravel(), oi.ravel()])
        norms.append(np.linalg.norm(ref))
        errs.append(rel_l2(np.concatenate([jr.ravel(), ji.ravel()]), ref))
    assert max(norms) > 0, "every monitor of the oracle is zero"
    for q in live or ():
        assert norms[q] > 0, f"monitor {q} of the oracle is zero"
    return max(errs)


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
def test_2d_tmz_cylinders_vs_oracle(gpu, oracle_lib, prec):
    spec, meta = problems.config_2d_tmz(precision=prec, n=384, ncyl=8, nfreq=24)
    steps = 2500
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64))
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, 3)
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, (abi.EZ, abi.HX, abi.HY))
    else:
        assert err <= TOL32_DFT
        check_state(J, O, (abi.EZ, abi.HX, abi.HY), tol=TOL32_DFT, per_comp=None)


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
def test_3d_sphere_vs_oracle(gpu, oracle_lib, prec):
    spec, meta = problems.config_3d_sphere(precision=prec, n=96, nfreq=8, npml=8, radius=40.0, half=20)
    steps = 600
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, 6)
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ))
    else:
        assert err <= TOL32_DFT
        # the FP32 fields themselves, PML shell included (where FP32 splits a
        # component only across a PML axis), against the FP64 oracle's
        check_state(J, O, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ), tol=TOL32_DFT, per_comp=None)


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
def test_1d_gold_slab_vs_oracle(gpu, oracle_lib, prec):
    spec, meta = problems.config_1d_gold(precision=prec)
    steps = 20000
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64))
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, 3)
    assert err <= (TOL64 if prec == abi.F64 else TOL32_DFT)


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
def test_3d_graphene_sheet_vs_oracle(gpu, oracle_lib, prec):
    """The graphene configuration (Drude sheet from E_F, Kerr and Raman) on a
    laterally periodic 8 x 8 column of the 384-cell stack: the same physics
    per cell as the full 256 x 256 plane, which the problem's lateral
    periodicity makes uniform."""
    spec, meta = problems.config_3d_graphene(precision=prec, nxy=8, nz=384, nfreq=32)
    steps = 3000
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64))
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, 1)
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ))
    else:
        assert err <= TOL32_DFT


@pytest.mark.parametrize("dim", [2, 3])
def test_core_block_shapes_give_identical_results(gpu, dim):
    """Every candidate block shape of the interior kernels (pinned with
    fdtd_set_tile) gives the same fields bit for bit; the commit-time tuner
    picks one of them."""
    if dim == 2:
        spec, _ = problems.config_2d_tmz(precision=abi.F32, n=384, ncyl=8, nfreq=8)
        comps, steps = (abi.EZ, abi.HX, abi.HY), 400
    else:
        spec, _ = problems.config_3d_sphere(precision=abi.F32, n=96, nfreq=4, npml=8, radius=40.0, half=20)
        comps, steps = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ), 200
    ref = None
    # 3D 4..6: z-marching kernels; 7: the TMA-staged E core (FP32, core box inside the grid)
    # 3D 8: the TMA-staged E and H cores; 9: the fused step kernel (ping-pong field sets)
    # 2D 4: the fused step kernel (ping-pong field sets, the whole grid in one launch)
    for tile in ((1, 2, 3, 4) if dim == 2 else (1, 2, 3, 4, 5, 6, 7, 8, 9)):
        J = gpu.Job(spec, tile=tile)
        assert J.tile() == tile
        J.step(1, steps)
        got = [J.get_field(c) for c in comps]
        if ref is None:
            ref = got
            assert any(np.abs(g).max() > 0 for g in got)
        else:
            for a, b in zip(ref, got):
                np.testing.assert_array_equal(a, b)
        J.close()
    J = gpu.Job(spec)
    assert J.tile() in ((1, 2, 3, 4) if dim == 2 else range(1, 10))
    J.close()


def test_tma_cores_across_tile_seams(gpu, oracle_lib):
    """The TMA-staged 3D cores on a grid of several tiles: a 300^3 sphere
    with a 7-cell PML has a core box of 284 x 286 x 286 cells, so its x-range
    spans three 128-cell tiles (the last one 28 cells wide) and its y- and
    z-ranges are not multiples of the 8-row, 8-plane tiles.  The wave
    crosses the sphere, so the fields vary along every axis at every seam.
    Each TMA core shape gives the plain shape's fields bit for bit, and the
    plain shape's spectra match the FP64 oracle to the FP32 tolerance."""
    spec, _ = problems.config_3d_sphere(precision=abi.F32, n=300, nfreq=4, npml=7, radius=40.0, half=70)
    comps, steps = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ), 300
    ref = None
    for tile in (2, 7, 8, 9):
        J = gpu.Job(spec, tile=tile)
        assert J.tile() == tile
        J.step(1, steps)
        got = [J.get_field(c) for c in comps]
        if ref is None:
            ref = got
            O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
            O.step(1, steps)
            assert _dft_err(J, O, 6) <= TOL32_DFT
            for c, g in zip(comps, got):
                assert np.any(g), f"component {c} is zero"
        else:
            for c, a, b in zip(comps, ref, got):
                np.testing.assert_array_equal(a, b, err_msg=f"tile {tile}, component {c}")
        J.close()


def test_fused_step_across_calls_rings_and_procedures(gpu):
    """The fused step kernel alternates two sets of field buffers.  Calls of
    any length -- an odd number of eager steps before and after graph rings,
    steps one at a time, the per-procedure entry points (which keep the
    split kernels) in between -- must leave the fields where the other entry
    points find them: the run equals the split kernels' single call bit for
    bit, for the fields, the spectra and a probe."""
    spec, _ = problems.config_3d_sphere(precision=abi.F32, n=96, nfreq=4, npml=8, radius=40.0, half=20)
    spec.add_probe((48, 48, 48), (abi.EX, abi.HY))
    comps = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    ref = gpu.Job(spec, tile=2)
    ref.step(1, 240)
    J = gpu.Job(spec, tile=9)
    assert J.tile() == 9
    n = 1
    for k in (45, 1, 1, 77, 3):
        J.step(n, k)
        n += k
    for n in range(n, n + 3):
        J.step_procedures(n)
    n += 1
    J.step(n, 241 - n)
    for c in comps:
        np.testing.assert_array_equal(J.get_field(c), ref.get_field(c), err_msg=f"component {c}")
    for q in range(len(spec.monitors)):
        for x, y in zip(J.get_monitor(q), ref.get_monitor(q)):
            np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(J.get_probe(0), ref.get_probe(0))


def test_fused_2d_step_across_calls_and_procedures(gpu):
    """The fused 2D step kernel alternates two sets of fields (and of the
    stored PML part).  Calls of any length -- odd numbers of eager steps
    around graph rings, single steps, the per-procedure entry points (which
    keep the split kernels) in between -- must leave the state where the
    other entry points find it: the run equals the split kernels' single
    call bit for bit, for the fields, the spectra and a probe.  The grid has
    gold cylinders (the dispersive-cell kernel beside the fused one), the
    split PML on all faces, a source row and monitor rows, and its 384-cell
    rows end in a partly filled strip of the kernel's 124-cell strips."""
    spec, _ = problems.config_2d_tmz(precision=abi.F32, n=384, ncyl=8, nfreq=8)
    spec.add_probe((200, 150, 0), (abi.EZ, abi.HX, abi.HY))
    comps = (abi.EZ, abi.HX, abi.HY)
    ref = gpu.Job(spec, tile=2)
    ref.step(1, 400)
    J = gpu.Job(spec, tile=4)
    assert J.tile() == 4
    n = 1
    for k in (45, 1, 77, 3, 101):
        J.step(n, k)
        n += k
    for n in range(n, n + 3):
        J.step_procedures(n)
    n += 1
    J.step(n, 401 - n)
    for c in comps:
        g = J.get_field(c)
        assert np.any(g), f"component {c} is zero"
        np.testing.assert_array_equal(g, ref.get_field(c), err_msg=f"component {c}")
    for q in range(len(spec.monitors)):
        for x, y in zip(J.get_monitor(q), ref.get_monitor(q)):
            np.testing.assert_array_equal(x, y)
    p = J.get_probe(0)
    assert np.any(p)
    np.testing.assert_array_equal(p, ref.get_probe(0))


def test_fused_2d_without_dispersive_cells_equals_split(gpu):
    """The fused 2D step kernel on a grid with no dispersive cells: no
    dispersive-cell kernel runs before it, so the kernel waits for the
    previous step itself.  Against the split path, bit for bit, over three
    graph rings and an eager tail."""
    spec, _ = problems.config_2d_tmz(precision=abi.F32, n=256, ncyl=0, nfreq=8, npml=16)
    a, b = gpu.Job(spec, tile=4), gpu.Job(spec, tile=2)
    a.step(1, 101)
    b.step(1, 101)
    for c in (abi.EZ, abi.HX, abi.HY):
        x = a.get_field(c)
        assert np.any(x), f"component {c} is zero"
        np.testing.assert_array_equal(x, b.get_field(c), err_msg=f"component {c}")
    for q in range(len(spec.monitors)):
        for x, y in zip(a.get_monitor(q), b.get_monitor(q)):
            np.testing.assert_array_equal(x, y)


def test_fused_2d_large_grid_equals_split(gpu):
    """The fused 2D step kernel where the tuner picks it: a 4096^2 grid of
    the bench's workload (34 strips of 124 cells, the last partly filled, 512 marches of 8 rows per
    strip, every dispersive cell of 40 cylinders), 96 steps -- three graph
    rings -- against the split path, bit for bit."""
    spec, _ = problems.config_2d_tmz(precision=abi.F32, n=4096, nfreq=8)
    a, b = gpu.Job(spec, tile=4), gpu.Job(spec, tile=2)
    a.step(1, 96)
    b.step(1, 96)
    for c in (abi.EZ, abi.HX, abi.HY):
        x = a.get_field(c)
        assert np.any(x), f"component {c} is zero"
        np.testing.assert_array_equal(x, b.get_field(c), err_msg=f"component {c}")
    for q in range(len(spec.monitors)):
        for x, y in zip(a.get_monitor(q), b.get_monitor(q)):
            np.testing.assert_array_equal(x, y)


@pytest.fixture(scope="module")
def bench2d_oracle(oracle_lib):
    """The FP64 oracle on the bench's whole 2D workload: 2048^2 cells, 40
    cylinders, 10000 steps."""
    spec, meta = problems.config_2d_tmz(precision=abi.F64)
    O = oracle_lib.OracleJob(spec, nthreads=NTH)
    O.step(1, meta["Nt"])
    return O, meta


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
def test_2d_bench_workload_full_size_vs_oracle(gpu, bench2d_oracle, prec):
    """The bench's 2D workload at its full size and length against the FP64
    oracle: FP64 plain, fields and spectra <= 1e-10; FP32, spectra <= 1e-4
    (the metric's tolerance)."""
    O, meta = bench2d_oracle
    spec, _ = problems.config_2d_tmz(precision=prec)
    J = gpu.Job(spec)
    J.step(1, meta["Nt"])
    err = _dft_err(J, O, 3, live=(0, 1, 2))
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, (abi.EZ, abi.HX, abi.HY))
    else:
        assert err <= TOL32_DFT


@pytest.mark.parametrize("dim", [1, 3])
def test_per_procedure_path_equals_fused(gpu, dim):
    """The reference's loop body through the per-procedure entry points
    (update_DE, pml_update_E, interchange, update_H, pml_update_H, sample)
    gives the fused fdtd_step's fields and spectra bit for bit: in 3D the
    core and general launches split by role, in 1D the line kernel runs one
    stage per call."""
    if dim == 3:
        spec, _ = problems.config_3d_sphere(precision=abi.F64, n=64, nfreq=4, npml=8, radius=40.0, half=12)
        comps, steps = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ), 120
    else:
        spec, _ = problems.config_1d_gold(precision=abi.F64)
        comps, steps = (abi.EX, abi.HZ), 400
    a, b = gpu.Job(spec), gpu.Job(spec)
    a.step(1, steps)
    for n in range(1, steps + 1):
        b.step_procedures(n)
    for c in comps:
        np.testing.assert_array_equal(a.get_field(c), b.get_field(c))
    for q in range(len(spec.monitors)):
        for x, y in zip(a.get_monitor(q), b.get_monitor(q)):
            np.testing.assert_array_equal(x, y)


def test_footprint_estimate_bounds_the_commit(gpu):
    """fdtd_estimate_bytes, which the server admits jobs by, is an upper
    bound of what commit allocates."""
    cases = [problems.config_2d_tmz(precision=abi.F32, n=384, ncyl=8, nfreq=24)[0],
             problems.config_2d_tmz(precision=abi.F64, n=256, ncyl=4, nfreq=8, npml=16)[0],
             problems.config_3d_sphere(precision=abi.F32, n=96, nfreq=8, npml=8, radius=40.0, half=20)[0],
             problems.config_3d_sphere(precision=abi.F64, n=64, nfreq=4, npml=8, radius=40.0, half=12)[0],
             problems.config_3d_graphene(precision=abi.F32, nxy=8, nz=384, nfreq=32)[0],
             problems.config_1d_gold(precision=abi.F64)[0],
             problems.reference_2d()[0]]
    for spec in cases:
        j = gpu.Job(spec, commit=False)
        est = j.estimate_bytes()
        j.close()
        J = gpu.Job(spec)
        held = J.device_bytes()
        J.close()
        assert held <= est, (spec.name, held, est)
        assert est <= 4 * held + (4 << 20), (spec.name, held, est)


@pytest.mark.parametrize("dim", [2, 3])
def test_mean_monitor_is_the_mean_of_the_cell_spectra(gpu, dim):
    """A FDTD_MONITOR_MEAN monitor transforms the box mean of each
    component; by linearity its spectrum equals the mean over the box of a
    per-cell monitor's spectra on the same box (FP64)."""
    if dim == 2:
        spec, meta = problems.config_2d_tmz(precision=abi.F64, n=256, ncyl=4, nfreq=8, npml=16)
        mon = spec.monitors[2]
        steps = 600
    else:
        spec, meta = problems.config_3d_sphere(precision=abi.F64, n=64, nfreq=4, npml=8, radius=40.0, half=12)
        mon = spec.monitors[5]
        steps = 200
    spec.add_monitor(mon.lo, mon.hi, mon.comps, mon.omega, mon.n_first, mon.n_last, mean=True)
    J = gpu.Job(spec)
    J.step(1, steps)
    cre, cim = J.get_monitor(spec.monitors.index(mon))
    mre, mim = J.get_monitor(len(spec.monitors) - 1)
    assert mre.shape == (cre.shape[0], cre.shape[1], 1)
    assert np.linalg.norm(cre) > 0
    for a, b in ((mre[..., 0], cre.mean(axis=2)), (mim[..., 0], cim.mean(axis=2))):
        assert rel_l2(a, b) <= 1e-12


# ---------------------------------------------------------------------------
# Lorentz-pole materials (the *LorentzJp modules and si_mod) against the
# oracle's literal restatement of each reference coding
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("name", ["SI_S", "GOLD_JP"])
def test_lorentz_1d_slab_vs_oracle(gpu, oracle_lib, prec, name):
    spec, meta = problems.config_1d_slab(getattr(problems, name), precision=prec)
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64))
    J.step(1, meta["Nt"])
    O.step(1, meta["Nt"])
    err = _dft_err(J, O, 3)
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, (abi.EX, abi.HZ))
    else:
        assert err <= TOL32_DFT


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("case", ["tm_gold_jp", "te_gold_jp", "te_gold", "te_si_s"])
def test_2d_cylinders_other_materials_vs_oracle(gpu, oracle_lib, prec, case):
    """The cylinder workload with Lorentz gold or Si in place of Drude+2CP
    gold, in TMz and in the reference's own TE layout (Hz, Ex, Ey)."""
    spec, meta = problems.config_2d_tmz(precision=prec, n=384, ncyl=8, nfreq=24)
    mat = {"gold_jp": problems.GOLD_JP, "si_s": problems.SI_S}.get(case.split("_", 1)[1])
    if mat is not None:
        spec = problems.swap_gold(spec, mat)
    if case.startswith("te"):
        spec = problems.as_te(spec)
    steps = 2500
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64))
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, 3)
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, (abi.EX, abi.EY, abi.HZ) if case.startswith("te") else (abi.EZ, abi.HX, abi.HY))
    else:
        assert err <= TOL32_DFT


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
def test_lorentz_3d_sphere_vs_oracle(gpu, oracle_lib, prec):
    spec, meta = problems.config_3d_sphere(precision=prec, n=96, nfreq=8, npml=8, radius=40.0, half=20)
    spec = problems.swap_gold(spec, problems.GOLD_JP)
    steps = 600
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, 6)
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ))
    else:
        assert err <= TOL32_DFT
        # the FP32 fields themselves, PML shell included (where FP32 splits a
        # component only across a PML axis), against the FP64 oracle's
        check_state(J, O, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ), tol=TOL32_DFT, per_comp=None)


# ---------------------------------------------------------------------------
# 2D/3D total-field/scattered-field box
# ---------------------------------------------------------------------------
def _tfsf_masks(spec, meta, shape, npml=10):
    lo, hi = meta["box"]
    inside = np.zeros(shape, bool)
    inside[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = True
    core = np.zeros(shape, bool)
    px = 0 if spec.periodic[0] else npml
    zs = slice(npml, shape[0] - npml) if spec.layout == abi.LAYOUT_3D else slice(None)
    core[zs, npml:shape[1] - npml, px:shape[2] - px] = True
    return inside, core & ~inside


TFSF_CASES = [(abi.LAYOUT_2D_TM, False, 128, 1200), (abi.LAYOUT_2D_TE, True, 128, 1200),
              (abi.LAYOUT_2D_TE, False, 128, 1200), (abi.LAYOUT_3D, False, 64, 500)]


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("layout,periodic_x,n,steps", TFSF_CASES)
def test_tfsf_plane_wave_fills_the_box_only(gpu, prec, layout, periodic_x, n, steps):
    """In vacuum the box holds exactly the incident line's wave and the
    scattered region stays empty: to rounding in FP64, to FP32 rounding of
    the incident amplitude in FP32."""
    spec, meta = problems.config_tfsf(layout=layout, periodic_x=periodic_x, n=n, precision=prec)
    J = gpu.Job(spec)
    J.step(1, steps // 2)
    ce = abi.EX if layout == abi.LAYOUT_2D_TE else abi.EZ
    e, le = J.get_field(ce), J.get_field(abi.E_INC)
    inside, outside = _tfsf_masks(spec, meta, e.shape)
    peak = np.abs(e[inside]).max()
    tol = 1e-12 if prec == abi.F64 else 1e-5
    assert peak > 0
    assert np.abs(e[inside] - np.broadcast_to(le[None, :, None], e.shape)[inside]).max() <= tol * peak
    assert np.abs(e[outside]).max() <= tol * peak


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("layout,periodic_x,n,steps", TFSF_CASES)
def test_tfsf_scatterer_vs_oracle(gpu, oracle_lib, prec, layout, periodic_x, n, steps):
    """A gold cylinder (2D) or sphere (3D) in the box: the scattered field
    leaves the box through the faces."""
    spec, meta = problems.config_tfsf(layout=layout, periodic_x=periodic_x, n=n, precision=prec,
                                      scatterer="gold", radius=8.0)
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, 3)
    if prec == abi.F64:
        assert err <= TOL64
        comps = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ) if layout == abi.LAYOUT_3D else \
            (abi.EX, abi.EY, abi.HZ) if layout == abi.LAYOUT_2D_TE else (abi.EZ, abi.HX, abi.HY)
        check_state(J, O, comps)
        assert rel_l2(J.get_field(abi.E_INC), O.get_field(abi.E_INC)) <= TOL64
        assert rel_l2(J.get_field(abi.H_INC), O.get_field(abi.H_INC)) <= TOL64
    else:
        assert err <= TOL32_DFT


def test_3d_reference_output_files(gpu, tmp_path):
    """The 3D program run on the GPU and written as its per-rank files: the
    records hold the run's values, the record counts follow the program's
    gates, and calR_Sy on the files gives finite R, T, A within [-0.05, 1.05]."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden_2d import load_table
    from fdtd_gpu import outputs
    spec, meta = problems.reference_3d()
    six = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    J = gpu.Job(spec)
    ic, kc = meta["ic"] - 1, meta["kc"] - 1
    lines, n = {}, 0
    for f in range(1, 21):
        target = f * meta["dn"]
        J.step(n + 1, target - n)
        n = target
        lines[f] = np.stack([J.get_field(c)[kc, :, ic] for c in six])
    J.step(n + 1, meta["Nt"] - n)
    mons = [J.get_monitor(q) for q in range(3)]
    probes = [J.get_probe(q) for q in range(3)]
    assert [len(p) for p in probes] == [meta["tfinStop"] - 1, meta["Nt"], meta["Nt"] - meta["tfinStop"]]
    outputs.write_reference_3d(str(tmp_path), meta, mons, probes, lines)
    tr = tmp_path / "transforms"
    np.testing.assert_array_equal(load_table(str(tr / "r5tfld.dat"))[:, 1:], probes[1])
    rows = outputs.cal_r_sy(str(tr), inc=0, ref=0, tras=5, out_name="RTA_3Dfdtd.data")
    assert np.all(np.isfinite(rows))
    assert rows[:, 1:].min() > -0.05 and rows[:, 1:3].max() < 1.05
    line = np.concatenate([load_table(str(tmp_path / "timesLiney" / f"r{k}E_time20.dat")) for k in range(6)])
    np.testing.assert_allclose(line[:, 1:].T, lines[20], atol=5.01e-6)


@pytest.mark.parametrize("dim", [2, 3])
def test_chained_branches_equal_serialised_run(gpu, dim):
    """The replayed step -- core kernels with programmatic dependencies, side
    kernels released by the previous core kernel's programmatic event -- gives
    the fields of the same job run with profiling on, where every kernel runs
    on its own after the previous one has finished.  Bit for bit: a side
    kernel that read a field before its writer finished would show here."""
    if dim == 2:
        spec, _ = problems.config_2d_tmz(precision=abi.F32, n=512, ncyl=6, nfreq=8)
        comps, steps = (abi.EZ, abi.HX, abi.HY), 640
    else:
        spec, _ = problems.config_3d_sphere(precision=abi.F32, n=96, nfreq=4, npml=8, radius=40.0, half=20)
        comps, steps = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ), 320
    runs = []
    for serial in (False, True):
        J = gpu.Job(spec, tile=1)
        if serial:
            J.profile(True)
        J.step(1, steps)
        runs.append(([J.get_field(c) for c in comps], [J.get_monitor(q) for q in range(len(spec.monitors))]))
        J.close()
    (fa, ma), (fb, mb) = runs
    assert any(np.abs(x).max() > 0 for x in fa)
    for x, y in zip(fa, fb):
        np.testing.assert_array_equal(x, y)
    for (ra, ia), (rb, ib) in zip(ma, mb):
        np.testing.assert_array_equal(ra, rb)
        np.testing.assert_array_equal(ia, ib)


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("case", ["3d", "2d_te", "2d_tm"])
def test_lorentz_sheet_vs_oracle(gpu, oracle_lib, prec, case):
    """The Lorentz-Jp graphene sheet (SLG_3LJp1nm) with its Kerr term: in 3D
    the graphene configuration's column with this sheet in place of the Drude
    one; in 2D a sheet across the cylinder workload (TE: Ex in-plane and Ey
    the vacuum normal component; TM: Ez in-plane)."""
    from fdtd_gpu.spec import box
    if case == "3d":
        spec, _ = problems.config_3d_graphene(precision=prec, nxy=8, nz=384, nfreq=32)
        spec = problems.swap_graphene(spec, dict(problems.GRAPHENE_3LJP, chi3=1e-12, e_scale=1.0))
        steps, nmon = 3000, 1
    else:
        spec, _ = problems.config_2d_tmz(precision=prec, n=384, ncyl=4, nfreq=16)
        if case == "2d_te":
            spec = problems.as_te(spec)
        spec.add_lorentz(box((24, 150, 0), (359, 150, 0)), dict(problems.GRAPHENE_3LJP, chi3=1e-2, e_scale=1.0))
        steps, nmon = 2500, 3
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, nmon)
    assert err <= (TOL64 if prec == abi.F64 else TOL32_DFT)


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("case", ["1d", "2d_te", "2d_tm", "3d", "3d_first_init"])
def test_graphene_cp_vs_oracle(gpu, oracle_lib, prec, case):
    """The reference's Graphene (Drude + 4 critical points + Raman):
    1D: a 50 nm slab, every component updated, no Raman (the 1D module);
    2D TE: a sheet along x with the 3D module's exact Raman coefficients (Ex
    in-plane, Ey = Dy), crossing the all-face PML shell at both ends;
    2D TM: the same sheet with the 2D module's central Raman coefficients;
    3D: the graphene configuration's column with this sheet in place of the
    Drude one (normal z), and the same with the 3D module's first-initialised
    coefficients (no critical points)."""
    from fdtd_gpu.spec import box
    raman = dict(w_nl=2 * np.pi * 47.4e12, gamma_nl=1e12)
    if case == "1d":
        spec, meta = problems.config_1d_slab(dict(problems.GRAPHENE_4CP, normal_axis=-1), precision=prec)
        steps, nmon, comps = meta["Nt"], 3, (abi.EX, abi.HZ)
    elif case.startswith("3d"):
        mat = dict(problems.GRAPHENE_4CP, chi3=1e-18, normal_axis=2, raman_form=abi.RAMAN_EXACT, **raman)
        if case == "3d_first_init":
            mat = problems.as_first_initialised_3d(mat)
        spec, _ = problems.config_3d_graphene(precision=prec, nxy=8, nz=384, nfreq=32)
        spec = problems.swap_graphene_cp(spec, mat)
        steps, nmon, comps = 3000, 1, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    else:
        spec, _ = problems.config_2d_tmz(precision=prec, n=384, ncyl=4, nfreq=16)
        form = abi.RAMAN_EXACT if case == "2d_te" else abi.RAMAN_CENTRAL
        comps = (abi.EZ, abi.HX, abi.HY)
        if case == "2d_te":
            spec = problems.as_te(spec)
            comps = (abi.EX, abi.EY, abi.HZ)
        spec.add_graphene_cp(box((24, 150, 0), (359, 150, 0)),
                             dict(problems.GRAPHENE_4CP, chi3=1e-2, raman_form=form, **raman))
        steps, nmon = 2500, 3
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, nmon)
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, comps)
    else:
        assert err <= TOL32_DFT


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("case", ["1d", "2d_te", "3d"])
def test_conductive_vs_oracle(gpu, oracle_lib, prec, case):
    """SiL800's conductive dielectric (sigma 2e5 S/m, so that the conduction
    current matters) in place of the gold of the 1D slab, the 2D cylinders
    (TE) and the 3D sphere.  The state is compared while the pulse is in the
    material: once it has gone, the conductor keeps a static charge, D and I
    stay large and nearly equal, and the oracle's E = (D - I)/ga carries the
    rounding of that difference (~1e-16 |D|), far above the small E left."""
    mat = dict(problems.SI_L800, sigma=2e5)
    if case == "1d":
        spec, meta = problems.config_1d_slab(mat, precision=prec)
        steps, nmon, comps = meta["Nt"], 3, (abi.EX, abi.HZ)
    elif case == "2d_te":
        spec, _ = problems.config_2d_tmz(precision=prec, n=384, ncyl=8, nfreq=24)
        spec = problems.as_te(problems.swap_gold(spec, mat, kind="conductive"))
        steps, nmon, comps = 2500, 3, (abi.EX, abi.EY, abi.HZ)
    else:
        spec, _ = problems.config_3d_sphere(precision=prec, n=96, nfreq=4, npml=8, radius=120.0, half=30)
        spec = problems.swap_gold(spec, mat, kind="conductive")
        steps, nmon, comps = 400, 6, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    mid = 3000 if case == "1d" else steps // 2
    J.step(1, mid)
    O.step(1, mid)
    if prec == abi.F64:
        check_state(J, O, comps)
    J.step(mid + 1, steps - mid)
    O.step(mid + 1, steps - mid)
    err = _dft_err(J, O, nmon)
    assert err <= (TOL64 if prec == abi.F64 else TOL32_DFT)


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("case", ["4ljp_column", "4ljp_ez_quirk", "nd_column"])
def test_lorentz_sheet_variants_vs_oracle(gpu, oracle_lib, prec, case):
    """The other Lorentz-Jp graphene sheets: SLG_LJp's four poles with the
    Kerr term on the graphene column (normal z); SLG_LJp with its Ez line
    taking the x current, on a sheet normal to y across a 3D box; SLG_ndJp
    (zero pole weights) with its Kerr term on the column."""
    from fdtd_gpu.spec import box
    if case == "4ljp_ez_quirk":
        spec, _ = problems.config_3d_sphere(precision=prec, n=48, nfreq=4, npml=6, radius=120.0, half=200)
        spec.add_lorentz(box((8, 24, 8), (39, 24, 39)),
                         dict(problems.GRAPHENE_4LJP, chi3=1e-2, e_scale=1.0, ez_uses_x_current=1))
        steps, nmon, comps = 400, 6, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    else:
        mat = problems.GRAPHENE_ND_3LJP if case == "nd_column" else dict(problems.GRAPHENE_4LJP, ez_uses_x_current=0)
        spec, _ = problems.config_3d_graphene(precision=prec, nxy=8, nz=384, nfreq=32)
        spec = problems.swap_graphene(spec, dict(mat, chi3=1e-12, e_scale=1.0))
        steps, nmon, comps = 3000, 1, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    J.step(1, steps)
    O.step(1, steps)
    err = _dft_err(J, O, nmon)
    if prec == abi.F64:
        assert err <= TOL64
        check_state(J, O, comps)
    else:
        assert err <= TOL32_DFT


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("name", ["gold", "gold_jp", "si_s", "graphene_cp", "conductive", "graphene_633"])
def test_cell_response_vs_oracle(gpu, oracle_lib, prec, name):
    """Each dispersive update on its own (problems.config_cell: a uniformly
    driven periodic 8 x 8 grid, so curl H = 0): the GPU's E(n) series against
    the oracle's (FP64), and the permittivity it implies (FP32)."""
    params = {"gold": ("gold", problems.GOLD_CONFIG), "gold_jp": ("lorentz", problems.GOLD_JP),
              "si_s": ("lorentz", problems.SI_S),
              "graphene_cp": ("graphene_cp", dict(problems.GRAPHENE_4CP, normal_axis=-1)),
              "conductive": ("conductive", dict(problems.SI_L800, sigma=2e5)),
              "graphene_633": ("graphene_nk", problems.GRAPHENE_633)}[name]
    spec, meta = problems.config_cell(*params, precision=prec, steps=20000)
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64))
    J.step(1, meta["Nt"])
    O.step(1, meta["Nt"])
    ej, eo = J.get_probe(0)[:, 0], O.get_probe(0)[:, 0]
    if prec == abi.F64:
        assert rel_l2(ej, eo) <= TOL64
    else:
        w = problems.dft_omegas(400e-9, 900e-9, 50)
        ej_eps, eo_eps = problems.cell_eps(ej, meta, w), problems.cell_eps(eo, meta, w)  # complex
        assert np.linalg.norm(ej_eps - eo_eps) / np.linalg.norm(eo_eps) <= 1e-4


@pytest.mark.parametrize("case", ["2d_tmz", "2d_ref", "3d_ref", "1d_ref", "tfsf_3d"])
def test_checkpoint_resume_is_bitwise(gpu, case):
    """A job saved at a step boundary inside a DFT ring and loaded into a new
    job of the same description continues bit for bit as the uninterrupted
    run: fields, DFT sums and probes.  The cases cover the gold ADE, the
    all-face and the reference PML, the 1D TFSF line and the 2D/3D box."""
    if case == "2d_tmz":
        spec, _ = problems.config_2d_tmz(precision=abi.F32, n=256, ncyl=4, nfreq=8)
        comps, n1, n2 = (abi.EZ, abi.HX, abi.HY), 333, 700
    elif case == "2d_ref":
        spec, _ = problems.reference_2d()
        comps, n1, n2 = (abi.EX, abi.EY, abi.HZ), 1001, 2000
    elif case == "3d_ref":
        spec, _ = problems.reference_3d()
        comps, n1, n2 = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ), 150, 300
    elif case == "1d_ref":
        spec, _ = problems.reference_1d()
        comps, n1, n2 = (abi.EX, abi.HZ, abi.EX_INC, abi.HZ_INC), 2501, 5000
    else:
        spec, _ = problems.config_tfsf(layout=abi.LAYOUT_3D, precision=abi.F64, n=64, scatterer="gold", radius=8.0)
        comps, n1, n2 = (abi.EX, abi.EY, abi.EZ, abi.E_INC, abi.H_INC), 101, 260
    whole = gpu.Job(spec)
    whole.step(1, n2)
    first = gpu.Job(spec)
    first.step(1, n1)
    state = first.save_state()
    first.close()
    resumed = gpu.Job(spec)
    resumed.load_state(state)
    resumed.step(n1 + 1, n2 - n1)
    for c in comps:
        np.testing.assert_array_equal(resumed.get_field(c), whole.get_field(c))
    for q in range(len(spec.monitors)):
        for x, y in zip(resumed.get_monitor(q), whole.get_monitor(q)):
            np.testing.assert_array_equal(x, y)
    for q in range(len(spec.probes)):
        np.testing.assert_array_equal(resumed.get_probe(q), whole.get_probe(q))
    whole.close()
    resumed.close()


def test_checkpoint_from_another_job_is_refused(gpu):
    a, _ = problems.config_2d_tmz(precision=abi.F32, n=256, ncyl=4, nfreq=8)
    b, _ = problems.config_2d_tmz(precision=abi.F32, n=512, ncyl=4, nfreq=8)
    ja, jb = gpu.Job(a), gpu.Job(b)
    ja.step(1, 10)
    state = ja.save_state()
    with pytest.raises(gpu.FdtdError) as e:
        jb.load_state(state)
    assert e.value.code == abi.FDTD_EINVAL
    state[:8] = 0
    with pytest.raises(gpu.FdtdError):
        ja.load_state(state)
    ja.close()
    jb.close()
    # damaged checkpoints whose header total agrees with their length: cut
    # short, or with a probe record that claims more samples than it holds
    a.add_probe((128, 128, 0), (abi.EZ,))
    ja = gpu.Job(a)
    ja.step(1, 10)
    good = ja.save_state()
    nbuf = int(good[32:36].view(np.uint32)[0])
    short = good[:-8].copy()
    short[56:64] = np.frombuffer(np.uint64(short.size).tobytes(), np.uint8)
    rec = 64 + 8 * nbuf                       # the probe's (samples, components) record
    more = good.copy()
    more[rec:rec + 4] = np.frombuffer(np.int32(good[rec:rec + 4].view(np.int32)[0] + 1).tobytes(), np.uint8)
    for bad in (short, more):
        with pytest.raises(gpu.FdtdError) as e:
            ja.load_state(bad)
        assert e.value.code == abi.FDTD_EINVAL
    ja.load_state(good)
    ja.close()


@pytest.mark.parametrize("tile", [8, 9])
def test_tma_wait_give_up_is_reported_and_recovered(gpu, tile):
    """The bounded waits of the TMA-staged kernels (tile 8: the E and H
    cores; tile 9: the fused step kernel), made to run out at once (a wait
    limit of 0 polls) while every copy still lands: the kernels set the
    job's flag, let their copies land and return; fdtd_sync reports
    FDTD_ECUDA once, the context stays usable, and with the default limit
    the job then steps without error, and a fresh job gives the plain
    cores' fields."""
    spec, _ = problems.config_3d_sphere(precision=abi.F32, n=96, nfreq=4, npml=8, radius=40.0, half=20)
    J = gpu.Job(spec, tile=tile)
    J.debug_wait_limit(0)
    J.step(1, 3)
    with pytest.raises(gpu.FdtdError) as e:
        J.sync()
    assert e.value.code == abi.FDTD_ECUDA
    J.sync()                                # reported once
    J.debug_wait_limit(-1)
    J.step(4, 40)
    J.sync()
    J.close()
    a, b = gpu.Job(spec, tile=tile), gpu.Job(spec, tile=2)
    a.step(1, 40)
    b.step(1, 40)
    for c in (abi.EX, abi.HY):
        np.testing.assert_array_equal(a.get_field(c), b.get_field(c))


def test_nonfinite_values_are_counted(gpu):
    """A NaN written into one cell on the host spreads through the update,
    and fdtd_check_finite sees it; a clean run counts none."""
    spec, _ = problems.config_2d_tmz(precision=abi.F32, n=256, ncyl=4, nfreq=8)
    J = gpu.Job(spec)
    J.step(1, 100)
    assert J.count_nonfinite() == 0
    ez = J.get_field(abi.EZ)
    ez[0, 128, 128] = np.nan
    J.set_field(abi.EZ, ez)
    assert J.count_nonfinite() == 1
    J.step(101, 40)
    assert J.count_nonfinite() > 100
    J.close()


def test_allocation_failures_are_reported_and_recovered(gpu):
    """Every device allocation of set-up and stepping fails once in turn
    (fdtd_debug_fail_alloc): each failure comes back as FDTD_ENOMEM with the
    job still usable, and a job whose step failed runs correctly when
    stepped again."""
    spec, _ = problems.config_2d_tmz(precision=abi.F32, n=256, ncyl=4, nfreq=8)
    spec.add_probe((128, 128, 0), (abi.EZ,))
    ref = gpu.Job(spec)
    ref.step(1, 100)
    want = [ref.get_field(c) for c in (abi.EZ, abi.HX, abi.HY)], ref.get_probe(0)
    ref.close()
    failed_setup = failed_step = 0
    try:
        for k in range(400):
            gpu.fail_alloc_after(k)
            try:
                J = gpu.Job(spec)
            except gpu.FdtdError as e:
                assert e.code == abi.FDTD_ENOMEM, str(e)
                failed_setup += 1
                continue
            try:
                J.step(1, 100)
                done = True
            except gpu.FdtdError as e:
                assert e.code == abi.FDTD_ENOMEM, str(e)
                failed_step += 1
                done = False
            gpu.fail_alloc_after(-1)
            if not done:
                J.step(1, 100)  # a failed step ran nothing: the same call again
            got = [J.get_field(c) for c in (abi.EZ, abi.HX, abi.HY)], J.get_probe(0)
            J.close()
            for x, y in zip(got[0], want[0]):
                np.testing.assert_array_equal(x, y)
            np.testing.assert_array_equal(got[1], want[1])
            if done:
                break
    finally:
        gpu.fail_alloc_after(-1)
    assert failed_setup >= 10 and failed_step >= 2


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
@pytest.mark.parametrize("case", ["1d", "2d_te", "3d"])
def test_graphene_nk_vs_oracle(gpu, oracle_lib, prec, case):
    """The reference's 1D graphene at 633 nm (graphene633), Kerr and Raman on:
    a 10-cell layer of the 1D line; a 3-row layer across the 2D TE cylinder
    workload; the graphene column of the 3D configuration (fields in V/m)."""
    from fdtd_gpu.spec import Material, box
    raman = dict(alpha=0.7, w_nl=2 * np.pi * 47.4e12, gamma_nl=1e12)
    if case == "1d":
        spec, meta = problems.config_1d_slab(dict(problems.GRAPHENE_633, chi3=1.0, **raman), thickness=10,
                                             precision=prec)
        steps, nmon, comps = meta["Nt"], 3, (abi.EX, abi.HZ)
    elif case == "2d_te":
        spec, _ = problems.config_2d_tmz(precision=prec, n=384, ncyl=4, nfreq=16)
        spec = problems.as_te(spec)
        spec.add_graphene_nk(box((40, 150, 0), (343, 152, 0)), dict(problems.GRAPHENE_633, chi3=1e-2, **raman))
        steps, nmon, comps = 2500, 3, (abi.EX, abi.EY, abi.HZ)
    else:
        spec, _ = problems.config_3d_graphene(precision=prec, nxy=8, nz=384, nfreq=32)
        mat = dict(problems.GRAPHENE_633, scale=0.17, chi3=1e-18, **raman)
        spec.materials = [Material("graphene_nk", m.region, params=dict(mat)) if m.kind == "graphene" else m
                          for m in spec.materials]
        steps, nmon, comps = 3000, 1, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    # the state is compared mid-run: afterwards the conducting layer keeps a
    # static charge, and the oracle's (D - I) carries rounding of ~1e-16 |D|
    # far above the small E left (as in test_conductive_vs_oracle)
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    mid = 3000 if case == "1d" else steps // 2
    J.step(1, mid)
    O.step(1, mid)
    if prec == abi.F64:
        check_state(J, O, comps)
    J.step(mid + 1, steps - mid)
    O.step(mid + 1, steps - mid)
    err = _dft_err(J, O, nmon)
    assert err <= (TOL64 if prec == abi.F64 else TOL32_DFT)


def test_tma_core_only_where_the_core_box_lies_inside(gpu):
    """Tile 7 (the TMA-staged E core) needs every neighbour of the core box
    inside the grid: the laterally periodic graphene column refuses it at
    commit, and its tuner picks among the other shapes."""
    spec, _ = problems.config_3d_graphene(precision=abi.F32, nxy=8, nz=384, nfreq=8)
    with pytest.raises(gpu.FdtdError) as e:
        gpu.Job(spec, tile=7)
    assert e.value.code == abi.FDTD_EINVAL
    J = gpu.Job(spec)
    assert J.tile() in range(1, 7)
    J.close()


@pytest.mark.parametrize("prec", [abi.F64, abi.F32])
def test_odd_grid_with_several_dispersive_kinds_vs_oracle(gpu, oracle_lib, prec):
    """A 203 x 203 TE grid (one cell per vector in both precisions) holding
    Lorentz-Jp gold cylinders, a 4-critical-point graphene sheet and a
    conductive block at once: the core and edge kernels' one-cell path beside
    three kinds of dispersive update in one launch."""
    from fdtd_gpu.spec import box
    spec, _ = problems.config_2d_tmz(precision=prec, n=203, ncyl=4, nfreq=8, npml=16)
    spec = problems.as_te(problems.swap_gold(spec, problems.GOLD_JP))
    spec.add_graphene_cp(box((20, 120, 0), (182, 120, 0)), dict(problems.GRAPHENE_4CP, chi3=1e-2, w_nl=2 * np.pi * 47.4e12,
                                                                gamma_nl=1e12))
    spec.add_conductive(box((60, 150, 0), (90, 160, 0)), dict(problems.SI_L800, sigma=2e5))
    J = gpu.Job(spec)
    O = oracle_lib.OracleJob(spec.with_precision(abi.F64), nthreads=NTH)
    J.step(1, 700)
    O.step(1, 700)
    if prec == abi.F64:
        check_state(J, O, (abi.EX, abi.EY, abi.HZ))
    J.step(701, 800)
    O.step(701, 800)
    err = _dft_err(J, O, len(spec.monitors))
    assert err <= (TOL64 if prec == abi.F64 else TOL32_DFT)
