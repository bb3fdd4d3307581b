"""GPU tests of the ragged batch (one persistent launch over many transforms
of uneven lengths and mixed modes) against an FP64 FFT per transform and
against the one-launch-per-transform comparator."""
import numpy as np
import pytest
import torch

from util import rel_l2

pytestmark = pytest.mark.gpu


def ref_segment(x, mode):
    x = x.astype(np.complex128)
    if mode == -1:
        return np.fft.fft(x)
    y = np.fft.ifft(x)
    return y * len(x) if mode == 1 else y


def check_segments(lengths, modes, offsets, x, y, tol=4e-6, sample=None):
    idx = range(len(lengths)) if sample is None else sample
    for i in idx:
        n, o = int(lengths[i]), int(offsets[i])
        if n == 0:
            continue
        e = rel_l2(y[o:o + n], ref_segment(x[o:o + n], int(modes[i])))
        assert e < tol, (i, n, int(modes[i]), e)


def test_ragged_small_mixed(gbfft_lib):
    g = gbfft_lib
    from gbfft import synth
    lengths, modes = synth.ragged_lengths(300, seed=11, hi=20000)
    extra = np.array([1, 2, 3, 5, 7, 16, 17, 97, 4096, 4097, 8192, 8191, 12289, 65536, 65521], np.int64)
    lengths = np.concatenate([lengths, extra])
    modes = np.concatenate([modes, np.array([-1, 1, 2] * 5, np.int32)])
    rng = np.random.default_rng(0)
    total = int(lengths.sum())
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    plan = g.RaggedPlan(lengths, modes)
    xt = torch.from_numpy(x).cuda()
    y = plan(xt)
    torch.cuda.synchronize()
    assert plan.status() == 0
    yn = y.cpu().numpy()
    check_segments(lengths, modes, plan.offsets, x, yn)
    # relaunch with fresh buffers (graph parameter update) and the comparator
    y2 = torch.empty_like(xt)
    plan(xt, out=y2)
    y3 = plan(xt, per_transform=True)
    torch.cuda.synchronize()
    assert torch.equal(y2, y)
    assert rel_l2(y3.cpu().numpy(), yn) < 4e-6
    assert torch.equal(xt.cpu(), torch.from_numpy(x))


def test_ragged_dependency_wait_times_out(gbfft_lib, monkeypatch):
    """A device-side wait that runs out: GBFFT_FAULT_INJECT=ragged_dep makes the
    plan's first task wait on a counter that no task ever signals, with a
    short bound.  The launch must end by itself, report GBFFT_ERR_TIMEOUT
    through gbfft_ragged_status, and leave the GPU usable: a normal plan
    afterwards is correct and reports OK."""
    import time
    g = gbfft_lib
    from gbfft import _lib as L
    lengths = np.array([16, 1000, 1009, 4096, 8192, 65521, 300, 7], np.int64)
    modes = np.array([-1, 1, 2, -1, 2, -1, 1, 2], np.int32)
    rng = np.random.default_rng(5)
    total = int(lengths.sum())
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    xt = torch.from_numpy(x).cuda()
    monkeypatch.setenv("GBFFT_FAULT_INJECT", "ragged_dep")
    bad = g.RaggedPlan(lengths, modes)
    monkeypatch.delenv("GBFFT_FAULT_INJECT")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bad(xt)
    st = bad.status()  # synchronises the stream
    dt = time.perf_counter() - t0
    assert st == L.ERR_TIMEOUT
    assert dt < 5.0, dt
    assert bad.status() == L.OK  # the status word was cleared by the read
    bad.close()
    good = g.RaggedPlan(lengths, modes)
    y = good(xt)
    torch.cuda.synchronize()
    assert good.status() == L.OK
    check_segments(lengths, modes, good.offsets, x, y.cpu().numpy())
    good.close()


def test_ragged_offsets_with_gaps_and_double(gbfft_lib):
    # (1024 and 4096 in Complex Double: lengths the plans run on kernels of
    # their own, which the ragged executor replaces by its tiles)
    g = gbfft_lib
    lengths = np.array([16, 1000, 1009, 5, 8192, 3, 1024, 4096], np.int64)
    modes = np.array([-1, 2, 1, -1, 2, 1, 2, -1], np.int32)
    offsets = np.array([0, 40, 1100, 3000, 3020, 12000, 12010, 13100], np.int64)
    total = 17200
    rng = np.random.default_rng(1)
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex128)
    plan = g.RaggedPlan(lengths, modes, offsets=offsets, dtype=torch.complex128)
    y = plan(torch.from_numpy(x).cuda()).cpu().numpy()
    check_segments(lengths, modes, offsets, x, y, tol=1e-12)
    # gaps are left untouched (zeros from zeros_like)
    assert np.all(y[20:40] == 0)


def test_ragged_config4_full_size(gbfft_lib):
    # 20,000 transforms, lengths 16..65536 (70% 7-smooth, 30% prime), mixed modes
    g = gbfft_lib
    from gbfft import synth
    lengths, modes = synth.ragged_lengths(20000, seed=4)
    total = int(lengths.sum())
    gen = torch.Generator().manual_seed(4)
    x = torch.complex(torch.randn(total, generator=gen), torch.randn(total, generator=gen))
    plan = g.RaggedPlan(lengths, modes)
    xt = x.cuda()
    y = plan(xt)
    yp = plan(xt, per_transform=True)
    torch.cuda.synchronize()
    assert plan.status() == 0
    yn = y.cpu().numpy()
    assert rel_l2(yn, yp.cpu().numpy()) < 4e-6
    rng = np.random.default_rng(4)
    sample = rng.choice(len(lengths), 300, replace=False)
    check_segments(lengths, modes, plan.offsets, x.numpy(), yn, sample=sample)


def test_ragged_edge_cases(gbfft_lib):
    """Zero-length and length-1 transforms inside a batch, a batch of only
    length-1 transforms, and an empty batch."""
    g = gbfft_lib
    rng = np.random.default_rng(21)
    lengths = np.array([0, 1, 0, 7, 1, 0, 4099, 2, 0], np.int64)
    modes = np.array([-1, 1, 2, 2, -1, 1, 1, -1, 2], np.int32)
    total = int(lengths.sum())
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    plan = g.RaggedPlan(lengths, modes)
    y = plan(torch.from_numpy(x).cuda())
    torch.cuda.synchronize()
    assert plan.status() == 0
    check_segments(lengths, modes, plan.offsets, x, y.cpu().numpy())
    plan.close()
    ones = np.ones(50, np.int64)
    plan = g.RaggedPlan(ones, np.array([-1, 1] * 25, np.int32))
    x1 = torch.from_numpy((rng.standard_normal(50) + 1j * rng.standard_normal(50)).astype(np.complex64)).cuda()
    y1 = plan(x1)
    torch.cuda.synchronize()
    assert torch.equal(y1, x1)  # the DFT of length 1 is the identity in every mode
    plan.close()
    plan = g.RaggedPlan(np.zeros(0, np.int64), np.zeros(0, np.int32))
    plan.close()
