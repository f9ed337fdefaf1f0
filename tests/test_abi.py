"""CPU tests of the C ABI library: it loads, exports every declared entry
point, and reports errors (no device here) without crashing."""
import ctypes as C
import os
import re

import pytest

from fdtd_gpu import abi, build, job, problems
from fdtd_gpu import spec as spec_mod

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def built():
    return build.build()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "fdtd_gb300.h")).read()
    return sorted(set(re.findall(r"^int\s+(fdtd_\w+)\s*\(", text, re.M)))


def test_header_matches_binding_list():
    assert declared_functions() == sorted(job.EXPORTS)


def test_library_exports_every_declared_symbol(built):
    L = C.CDLL(built)
    for name in declared_functions():
        assert hasattr(L, name), name


def test_struct_sizes_match_header(built, tmp_path):
    # compile a tiny C program that prints sizeof/offsetof of the descriptors
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "fdtd_gb300.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n",'
                   'sizeof(fdtd_grid_desc),sizeof(fdtd_region),sizeof(fdtd_drude2cp),'
                   'sizeof(fdtd_graphene_desc),sizeof(fdtd_pml_desc),sizeof(fdtd_source_desc),'
                   'sizeof(fdtd_monitor_desc),sizeof(fdtd_probe_desc),sizeof(fdtd_tfsf1d_desc),'
                   'sizeof(fdtd_lorentz_desc));printf("%zu %zu %zu\\n",sizeof(fdtd_tfsf_desc),'
                   'sizeof(fdtd_graphene_cp_desc),sizeof(fdtd_graphene_nk_desc));return 0;}\n')
    exe = tmp_path / "sz"
    import subprocess
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    got = [C.sizeof(t) for t in (abi.GridDesc, abi.Region, abi.Drude2CP, abi.GrapheneDesc, abi.PmlDesc,
                                 abi.SourceDesc, abi.MonitorDesc, abi.ProbeDesc, abi.Tfsf1dDesc, abi.LorentzDesc,
                                 abi.TfsfDesc, abi.GrapheneCpDesc, abi.GrapheneNkDesc)]
    assert [int(x) for x in out] == got


def test_no_device_is_reported_not_faked(built):
    if job.device_count() > 0:
        pytest.skip("a GPU is present")
    spec, _ = problems.reference_2d()
    with pytest.raises(job.FdtdError) as e:
        job.Job(spec)
    assert e.value.code == abi.FDTD_ENODEV
    assert "device" in str(e.value)


def test_bad_arguments_are_rejected(built):
    L = job.lib()
    h = C.c_void_p()
    g = abi.GridDesc()
    g.layout = 99
    assert L.fdtd_create(C.byref(g), C.byref(h)) == abi.FDTD_EINVAL
    assert "layout" in job.last_error()
    assert L.fdtd_create(None, C.byref(h)) == abi.FDTD_EINVAL
    assert L.fdtd_step(None, 1, 1) == abi.FDTD_EINVAL
    d = abi.LorentzDesc()
    d.form, d.npoles, d.eps_inf = abi.LORENTZ_JP, abi.LORENTZ_MAX_POLES + 1, 1.0
    assert L.fdtd_add_lorentz(None, None, C.byref(d), None) == abi.FDTD_EINVAL
    assert "npoles" in job.last_error()
    d.npoles, d.form = 1, 7
    assert L.fdtd_add_lorentz(None, None, C.byref(d), None) == abi.FDTD_EINVAL
    assert "form" in job.last_error()
    gp = spec_mod.graphene_cp_struct(dict(problems.GRAPHENE_4CP, width=0.0))
    assert L.fdtd_add_graphene_cp(None, None, C.byref(gp), None) == abi.FDTD_EINVAL
    assert "width" in job.last_error()
    gp = spec_mod.graphene_cp_struct(dict(problems.GRAPHENE_4CP, normal_axis=3))
    assert L.fdtd_add_graphene_cp(None, None, C.byref(gp), None) == abi.FDTD_EINVAL
    assert "normal_axis" in job.last_error()
    gp = spec_mod.graphene_cp_struct(dict(problems.GRAPHENE_4CP, chi3=1.0, w_nl=1e12, gamma_nl=4e12))
    assert L.fdtd_add_graphene_cp(None, None, C.byref(gp), None) == abi.FDTD_EINVAL
    assert "w_nl" in job.last_error()


def test_new_entry_points_reject_bad_arguments(built):
    """Checkpoint, health and graphene entry points answer a null job or bad
    parameters with an error code, without a device."""
    L = job.lib()
    n = C.c_uint64()
    assert L.fdtd_state_bytes(None, C.byref(n)) == abi.FDTD_EINVAL
    buf = (C.c_uint8 * 64)()
    assert L.fdtd_save_state(None, buf, 64) == abi.FDTD_EINVAL
    assert L.fdtd_load_state(None, buf, 64) == abi.FDTD_EINVAL
    cnt = C.c_int64()
    assert L.fdtd_check_finite(None, C.byref(cnt)) == abi.FDTD_EINVAL
    assert L.fdtd_debug_fail_alloc(-1) == abi.FDTD_OK
    p = spec_mod.graphene_nk_struct(dict(problems.GRAPHENE_633, wavelength=0.0))
    assert L.fdtd_add_graphene_nk(None, None, C.byref(p), None) == abi.FDTD_EINVAL
    assert "wavelength" in job.last_error()
    p = spec_mod.graphene_nk_struct(dict(problems.GRAPHENE_633, chi3=1.0, w_nl=1e12, gamma_nl=2e12))
    assert L.fdtd_add_graphene_nk(None, None, C.byref(p), None) == abi.FDTD_EINVAL
    assert "Raman" in job.last_error()
    assert L.fdtd_add_conductive(None, None, 1.0, -1.0, None) == abi.FDTD_EINVAL
