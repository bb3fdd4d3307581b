"""GPU tests of the autotuner (gbfft_autotune, GBFFT_AUTOTUNE, GBFFT_TUNE_FILE):
the search runs, the chosen plan is used by later plan creations and stays
correct against FP64, and the choice persists through the JSON-lines file."""
import numpy as np
import pytest
import torch

from util import rel_l2, uniform_complex

pytestmark = pytest.mark.gpu


@pytest.fixture
def clean_tuner(gbfft_lib):
    from gbfft import _lib as L
    L.lib().gbfft_tune_clear()
    L.lib().gbfft_cache_clear()
    yield L.lib()
    L.lib().gbfft_tune_clear()
    L.lib().gbfft_cache_clear()


def check_plan(g, shape, kind, rng):
    x = uniform_complex(rng, shape, np.complex64)
    plan = g.Plan(shape, kind=kind, dtype=torch.complex64)
    y = plan("forward", torch.from_numpy(x).cuda()).cpu().numpy()
    ref = np.fft.fftn(x.astype(np.complex128)) if kind == "full" else \
        np.fft.fft(x.astype(np.complex128), axis=-1)
    assert rel_l2(y, ref) < 2e-6, plan.describe()
    desc = plan.describe()
    plan.close()
    return desc


@pytest.mark.parametrize("shape,kind", [((4096, 512), "full"), ((4, 65536), "many"),
                                        ((64, 256, 128), "full")])
def test_autotune_search_and_persistence(clean_tuner, monkeypatch, tmp_path, shape, kind):
    g = __import__("gbfft")
    lib = clean_tuner
    path = tmp_path / "tune.jsonl"
    monkeypatch.setenv("GBFFT_TUNE_FILE", str(path))
    lib.gbfft_tune_clear()
    report = g.autotune(shape, kind=kind)
    lines = [ln for ln in report.splitlines() if ln.strip()]
    assert len(lines) >= 3 and lines[-1].startswith("best:"), report
    assert lib.gbfft_tune_count() == 1
    rng = np.random.default_rng(31)
    assert "tuned(" in check_plan(g, shape, kind, rng)
    # the file holds the choice; a cleared cache reloads it
    text = path.read_text()
    assert text.count("\n") == 1 and '"key": "' in text
    lib.gbfft_tune_clear()
    assert "tuned(" in check_plan(g, shape, kind, rng)
    assert lib.gbfft_tune_count() == 1


def test_autotune_on_plan_creation(clean_tuner, monkeypatch):
    g = __import__("gbfft")
    monkeypatch.delenv("GBFFT_TUNE_FILE", raising=False)
    monkeypatch.setenv("GBFFT_AUTOTUNE", "1")
    rng = np.random.default_rng(32)
    assert "tuned(" in check_plan(g, (512, 4096), "full", rng)
    assert clean_tuner.gbfft_tune_count() == 1


def test_ragged_autotune(gbfft_lib):
    """The ragged search runs, caches a choice that the next plan of the same
    batch uses, and the tuned plan stays correct against FP64."""
    g = gbfft_lib
    from gbfft import synth
    lengths, modes = synth.ragged_lengths(300, seed=11)
    report = g.ragged_autotune(lengths, modes)
    lines = [ln for ln in report.splitlines() if ln.strip()]
    assert len(lines) >= 4 and lines[-1].startswith("best:"), report
    plan = g.RaggedPlan(lengths, modes)
    total = int(lengths.sum())
    rng = np.random.default_rng(12)
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    xt = torch.from_numpy(x).cuda()
    y = torch.empty_like(xt)
    plan.exec_ptr(xt.data_ptr(), y.data_ptr())
    torch.cuda.synchronize()
    assert plan.status() == 0
    yy = y.cpu().numpy()
    for i in range(0, len(lengths), 7):
        n, o = int(lengths[i]), int(plan.offsets[i])
        r = np.fft.fft(x[o:o + n].astype(np.complex128)) if modes[i] == -1 else \
            np.fft.ifft(x[o:o + n].astype(np.complex128))
        assert rel_l2(yy[o:o + n], r) < 4e-6, (i, n)
    plan.close()
