"""Serving: continuous batching of jobs on one GPU (fdtd_server_*).

Each job's results must be the same alone and in the mix: a served job runs
the same kernels in the same order as fdtd_step(job, 1, n) on its own (its
chunks are whole 32-step rings from step 1), so the tolerance is zero --
the spectra are compared bit for bit.
"""
import numpy as np
import pytest

from fdtd_gpu import abi, problems, serve

gpu = pytest.mark.gpu


def small_mix():
    """2D TMz and 3D sphere jobs of different sizes, step counts (not all
    multiples of the 32-step ring) and frequency counts."""
    jobs = []
    for q, (n, ncyl, nst, nf) in enumerate(((128, 3, 700, 16), (192, 6, 613, 24), (160, 1, 900, 8),
                                             (128, 5, 450, 32), (256, 10, 777, 12))):
        spec, _ = problems.config_2d_tmz(precision=abi.F32, n=n, steps=nst, ncyl=ncyl, nfreq=nf, npml=16, seed=q)
        jobs.append((spec, nst))
    for n, nst in ((48, 300), (64, 257)):
        spec, _ = problems.config_3d_sphere(precision=abi.F32, n=n, steps=nst, nfreq=8, npml=8)
        jobs.append((spec, nst))
    return jobs


def spectra(job, spec):
    return [job.get_monitor(q) for q in range(len(spec.monitors))]


@pytest.fixture(scope="module")
def gpu_lib():
    from fdtd_gpu import build, job
    build.build()
    if job.device_count() < 1:
        pytest.skip("no sm_103a device")
    return job


@gpu
@pytest.mark.parametrize("pack_cells", [0, -1])
def test_mixed_results_equal_alone(gpu_lib, pack_cells):
    """pack_cells 0: the small 2D jobs share launches (packs); -1: every job
    runs on its own stream."""
    jobs = small_mix()
    alone = []
    for spec, nst in jobs:
        J = gpu_lib.Job(spec)
        J.step(1, nst)
        alone.append(spectra(J, spec))
        J.close()
    S = serve.Server(max_active=8, chunk_steps=64, pack_cells=pack_cells)
    tickets = [S.submit(spec, nst) for spec, nst in jobs]
    for q, tk in enumerate(tickets):
        assert S.wait(tk) == abi.REQ_DONE
        got = spectra(S.job(tk), jobs[q][0])
        # gated monitors (the reflected-wave window) may still be empty
        assert any(np.linalg.norm(ra) > 0 for ra, _ in alone[q])
        for (ra, ia), (rb, ib) in zip(alone[q], got):
            np.testing.assert_array_equal(ra, rb)
            np.testing.assert_array_equal(ia, ib)
        S.release(tk)
    st = S.stats()
    assert st["finished"] == len(jobs) and st["active"] == 0 and st["queued"] == 0
    assert st["held_bytes"] == 0
    assert (st["packed_rings"] > 0) == (pack_cells == 0)
    S.close()


@gpu
def test_admission_by_footprint_is_fifo_and_within_budget(gpu_lib):
    jobs = small_mix()[:5]
    est = []
    for spec, _ in jobs:
        j = gpu_lib.Job(spec, commit=False)
        est.append(j.estimate_bytes())
        j.close()
    budget = int(2.2 * max(est))  # about two jobs at a time
    S = serve.Server(hbm_budget=budget, max_active=8, chunk_steps=32)
    tickets = [S.submit(spec, nst) for spec, nst in jobs]
    admits = []
    for tk in tickets:
        assert S.wait(tk) == abi.REQ_DONE
        _, ta, td = S.times(tk)
        admits.append(ta)
        assert td >= ta >= 0
        S.release(tk)
    assert admits == sorted(admits)  # first come, first admitted
    st = S.stats()
    assert 0 < st["held_bytes_max"] <= budget
    S.close()


@gpu
def test_job_larger_than_budget_fails_and_others_run(gpu_lib):
    big, _ = problems.config_2d_tmz(precision=abi.F32, n=512, steps=100, ncyl=2, nfreq=8, npml=16)
    small, _ = problems.config_2d_tmz(precision=abi.F32, n=96, steps=100, ncyl=1, nfreq=4, npml=8)
    j = gpu_lib.Job(small, commit=False)
    budget = 3 * j.estimate_bytes()
    j.close()
    S = serve.Server(hbm_budget=budget, max_active=4, chunk_steps=32)
    tb = S.submit(big, 100)
    ts = S.submit(small, 100)
    with pytest.raises(gpu_lib.FdtdError) as e:
        S.wait(tb)
    assert e.value.code == abi.FDTD_ENOMEM
    assert S.wait(ts) == abi.REQ_DONE
    S.release(tb)
    S.release(ts)
    S.close()


def test_server_without_device_reports_enodev():
    from fdtd_gpu import build, job
    build.build()
    if job.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(job.FdtdError) as e:
        serve.Server()
    assert e.value.code == abi.FDTD_ENODEV


def test_poisson_mix_is_seeded_and_shaped():
    a = serve.poisson_mix(50, 10.0, seed=3)
    b = serve.poisson_mix(50, 10.0, seed=3)
    assert [(t, s.n, n) for t, s, n in a] == [(t, s.n, n) for t, s, n in b]
    times = [t for t, _, _ in a]
    assert times == sorted(times)
    for _, spec, nst in a:
        assert 2000 <= nst <= 8000
        assert spec.n[0] in (256, 512, 1024, 128, 192, 256)
        assert 32 <= len(spec.monitors[0].omega) <= 128
    n3d = sum(1 for _, s, _ in a if s.layout == abi.LAYOUT_3D)
    assert 2 <= n3d <= 20  # about 20% of 50


def test_percentile_nearest_rank():
    xs = list(range(1, 101))
    assert serve.percentile(xs, 50) == 50
    assert serve.percentile(xs, 99) == 99
    assert serve.percentile([7.0], 99) == 7.0
