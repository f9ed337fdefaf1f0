"""The oracle's 2D/3D total-field/scattered-field box, checked on the CPU.

A plane wave along +y in vacuum: inside the box the grid must carry exactly
the incident line's wave, and outside it nothing.  Both hold to rounding only
if every face term has the right cell, sign and incident value, so the test
pins the face terms of each layout (Ez/Hx for 3D and 2D TM, as the
reference's incEzHx helper writes them; Ex/Hz for 2D TE), with and without x
faces (an x-periodic box spanning the grid has none).
"""
import numpy as np
import pytest

from fdtd_gpu import abi, problems

CASES = [(abi.LAYOUT_2D_TM, False, 96, 400), (abi.LAYOUT_2D_TM, True, 96, 400),
         (abi.LAYOUT_2D_TE, False, 96, 400), (abi.LAYOUT_2D_TE, True, 96, 400),
         (abi.LAYOUT_3D, False, 48, 200), (abi.LAYOUT_3D, True, 48, 200)]


def box_masks(spec, meta, shape, npml=10):
    lo, hi = meta["box"]
    inside = np.zeros(shape, bool)
    inside[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = True
    core = np.zeros(shape, bool)
    px = 0 if spec.periodic[0] else npml
    zs = slice(npml, shape[0] - npml) if spec.layout == abi.LAYOUT_3D else slice(None)
    core[zs, npml:shape[1] - npml, px:shape[2] - px] = True
    return inside, core & ~inside


def tf_components(layout):
    return (abi.EX, abi.HZ) if layout == abi.LAYOUT_2D_TE else (abi.EZ, abi.HX)


def check_plane_wave(job, spec, meta):
    ce, _ = tf_components(spec.layout)
    e = job.get_field(ce)
    le = job.get_field(abi.E_INC)
    inside, outside = box_masks(spec, meta, e.shape)
    peak = np.abs(e[inside]).max()
    assert peak > 1e-3 * np.abs(le).max() > 0
    line = np.broadcast_to(le[None, :, None], e.shape)
    assert np.abs(e[inside] - line[inside]).max() <= 1e-12 * peak
    assert np.abs(e[outside]).max() <= 1e-12 * peak


@pytest.mark.parametrize("layout,periodic_x,n,steps", CASES)
def test_plane_wave_fills_the_box_and_nothing_else(oracle_lib, layout, periodic_x, n, steps):
    spec, meta = problems.config_tfsf(layout=layout, periodic_x=periodic_x, n=n)
    O = oracle_lib.OracleJob(spec, nthreads=4)
    O.step(1, steps)
    check_plane_wave(O, spec, meta)
    O.close()


def test_box_rows_must_leave_room_for_the_line(oracle_lib):
    spec, meta = problems.config_tfsf(layout=abi.LAYOUT_2D_TM, n=64)
    spec.tfsf_box = dict(lo=(20, 0, 0), hi=(40, 40, 0), eps_line=1.0)
    with pytest.raises(RuntimeError):
        oracle_lib.OracleJob(spec)
