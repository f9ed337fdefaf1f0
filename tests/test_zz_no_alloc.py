"""fdtd_dft_sample_noalloc: the allocation-free DFT of a caller-owned field.

A job with one Ez line monitor runs the 2D TMz cylinders problem at 128^2;
the test copies Ez to its own device buffer after every step of the
monitor's window and feeds it to the allocation-free entry point, whose
stage ring is a static device array.  Its sums must match the job's monitor
(fdtd_get_monitor) to the FP64 tolerance of the parity tests, on two
sequences of calls in a row (the second also flushes in mid-ring), which
shows that nothing from the first sequence leaks into the second.
"""
import numpy as np
import pytest

from fdtd_gpu import abi, problems

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
N1, N2 = 4501, 4700          # window: starts in mid-ring (slot 4), ends at slot 27


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    from fdtd_gpu import build, job
    build.build()
    if job.device_count() < 1:
        pytest.skip("no sm_103a device")
    spec, meta = problems.config_2d_tmz(precision=abi.F64, n=128, ncyl=2, nfreq=16, npml=16)
    yin = spec.monitors[0].lo[1]
    spec.monitors = []
    spec.add_monitor((0, yin, 0), (127, yin, 0), (abi.EZ,), meta["arg"], N1, N2)
    J = job.Job(spec)
    J.step(1, N1 - 20)
    frames = {}
    for n in range(N1 - 19, N2 + 21):   # a few steps either side of the window
        J.step(n, 1)
        frames[n] = J.get_field(abi.EZ)[0].copy()
    re, im = J.get_monitor(0)
    return torch, job, spec, meta, yin, frames, re[0], im[0]


def run_sequence(torch, job, meta, yin, frames, precision, flush_at=(), steps=None, acc=None):
    """Feed the recorded Ez frames of `steps` (default: all) to the entry
    point, into the accumulators `acc` (default: new zeroed ones)."""
    dev = torch.device("cuda", 0)
    dtype = torch.float64 if precision == abi.F64 else torch.float32
    field = torch.zeros((128, 128), dtype=dtype, device=dev)
    omega = torch.tensor(np.asarray(meta["arg"], np.float64), device=dev)
    nf, ncell = len(meta["arg"]), 128
    if acc is None:
        acc = (torch.zeros(nf * ncell, dtype=torch.float64, device=dev),
               torch.zeros(nf * ncell, dtype=torch.float64, device=dev))
    acc_re, acc_im = acc
    stream = torch.cuda.current_stream(dev).cuda_stream
    for n in sorted(frames) if steps is None else steps:
        field.copy_(torch.from_numpy(frames[n]).to(dtype))
        job.dft_sample_noalloc(field.data_ptr(), precision, (128, 128, 1), (0, yin, 0), (127, yin, 0), n, N1, N2,
                               meta["dt"], omega.data_ptr(), nf, acc_re.data_ptr(), acc_im.data_ptr(),
                               flush=n in flush_at, stream=stream)
    torch.cuda.synchronize(dev)
    return acc_re.cpu().numpy().reshape(nf, ncell), acc_im.cpu().numpy().reshape(nf, ncell)


def test_noalloc_sequence_resumed_mid_window(setup):
    """A run that stops inside the window (flushing its last ring) and later
    resumes mid-ring, after another sequence has filled the shared stage
    array, still sums to the job's monitor: the slots before the resumed
    step are cleared, not folded with the other sequence's samples."""
    torch, job, spec, meta, yin, frames, jre, jim = setup
    dev = torch.device("cuda", 0)
    nf, ncell = len(meta["arg"]), 128
    acc = (torch.zeros(nf * ncell, dtype=torch.float64, device=dev),
           torch.zeros(nf * ncell, dtype=torch.float64, device=dev))
    stop = N1 + 39                      # the run stops mid-ring; the resumed step N1 + 40 lies at slot 28
    assert (stop - 1) % 32 != 31 and stop % 32 == 28
    run_sequence(torch, job, meta, yin, frames, abi.F64, flush_at=(stop,), steps=range(N1, stop + 1), acc=acc)
    run_sequence(torch, job, meta, yin, frames, abi.F64)          # another sequence fills the ring
    re, im = run_sequence(torch, job, meta, yin, frames, abi.F64, steps=range(stop + 1, N2 + 1), acc=acc)
    assert rel_l2(re, jre) <= TOL64
    assert rel_l2(im, jim) <= TOL64


def test_noalloc_matches_job_monitor_two_sequences(setup):
    torch, job, spec, meta, yin, frames, jre, jim = setup
    assert np.linalg.norm(jre) > 0
    a_re, a_im = run_sequence(torch, job, meta, yin, frames, abi.F64)
    b_re, b_im = run_sequence(torch, job, meta, yin, frames, abi.F64, flush_at=(N1 + 40, N1 + 41, 4650))
    for re, im in ((a_re, a_im), (b_re, b_im)):
        assert rel_l2(re, jre) <= TOL64
        assert rel_l2(im, jim) <= TOL64


def test_noalloc_f32_field(setup):
    torch, job, spec, meta, yin, frames, jre, jim = setup
    re, im = run_sequence(torch, job, meta, yin, frames, abi.F32)
    assert rel_l2(re, jre) <= 1e-6
    assert rel_l2(im, jim) <= 1e-6


def test_noalloc_rejects_box_over_limit(setup):
    torch, job, spec, meta, yin, frames, jre, jim = setup
    from fdtd_gpu.job import FdtdError
    # 1024 x 512 cells > FDTD_NOALLOC_MAX_CELLS; rejected before any device work
    with pytest.raises(FdtdError) as e:
        job.dft_sample_noalloc(1, abi.F64, (1024, 512, 1), (0, 0, 0), (1023, 511, 0), 1, 1, 10, 1e-18, 1, 4, 1, 1)
    assert e.value.code == abi.FDTD_ERANGE
    assert "exceeds" in str(e.value)
