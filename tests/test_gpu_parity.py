"""GPU parity: libgbfft (through its C ABI) against the oracle.

Every result is compared (a) with an FP64 FFT of the same input (numpy's
pocketfft; the oracle's FP64 restatement for the golden cases) and (b) with
the oracle's restatement of the reference's own transform in the same
precision (oracle/adhoc.cpp: Adhoc.hs + FFT.hs).

Tolerances (relative L2):
  complex64 vs FP64:  2e-6 (radix 2/3/4/5/7/8/16 stages, four-step), 4e-6
                      (Bluestein, whose filter and chirp add two roundings)
  complex128 vs FP64: 1e-12
  vs the same-precision restatement: within the restatement's own FP64 error
  plus the tolerance above (the reference's Float Bluestein forms its chirp
  angle in single precision, Adhoc.hs:264-265, so it is itself ~1e-4 off).
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import lib as O
from util import dim1, dim2, dim3, np_reference, rel_l2, uniform_complex

pytestmark = pytest.mark.gpu

MODES = ("forward", "reverse", "inverse")
MODE_IDX = {"forward": 0, "reverse": 1, "inverse": 2}


def fast(n):
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def tol_fp64(dtype, shape):
    if dtype == np.complex128:
        return 1e-12
    return 2e-6 if all(fast(s) for s in shape) else 4e-6


def run_gpu(g, kind, mode, x):
    t = torch.from_numpy(x).cuda()
    f = {"fft": g.fft, "fft1D": g.fft1D, "fft2D": g.fft2D, "fft3D": g.fft3D}[kind]
    y = f(mode, t)
    torch.cuda.synchronize()
    assert torch.equal(t.cpu(), torch.from_numpy(x)), "input must be preserved"
    return y.cpu().numpy()


def check(g, kind, mode, x, same_precision=True):
    y = run_gpu(g, kind, mode, x)
    ref64 = np_reference(kind, MODE_IDX[mode], x)
    e64 = rel_l2(y, ref64)
    tol = tol_fp64(x.dtype.type, x.shape if kind != "fft" else x.shape[-1:])
    assert e64 < tol, (kind, mode, x.shape, x.dtype, e64)
    if same_precision:
        r = O.run(kind, MODE_IDX[mode], x)
        e_or = rel_l2(r, ref64)
        assert rel_l2(y, r) <= 1.5 * e_or + 2 * tol, (kind, mode, x.shape, rel_l2(y, r), e_or)
    return e64


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_fft1d_small_lengths_all_modes(gbfft_lib, dtype):
    rng = np.random.default_rng(10)
    for n in range(1, 130):
        x = uniform_complex(rng, (n,), dtype)
        for mode in MODES:
            check(gbfft_lib, "fft1D", mode, x)


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_fft1d_reference_generator_lengths(gbfft_lib, dtype):
    rng = np.random.default_rng(11)
    for _ in range(40):
        (n,) = dim1(rng)
        x = uniform_complex(rng, (n,), dtype)
        check(gbfft_lib, "fft1D", MODES[int(rng.integers(0, 3))], x)


@pytest.mark.parametrize("n", [1000, 1009, 1024, 2048, 2025, 4096, 4097, 8192, 16384, 65536,
                               65521, 5003, 100000, 3 * 5 * 7 * 11 * 13])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_fft1d_paths(gbfft_lib, n, dtype):
    # covers single-CTA radix, four-step (n > CTA capacity), single-kernel and
    # four-pass Bluestein (prime n, padded length above the CTA capacity)
    rng = np.random.default_rng(n)
    x = uniform_complex(rng, (n,), dtype)
    for mode in MODES:
        check(gbfft_lib, "fft1D", mode, x, same_precision=(n <= 16384))


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_many_innermost_generator_shapes(gbfft_lib, dtype):
    rng = np.random.default_rng(12)
    for _ in range(12):
        for gen in (dim2, dim3):
            x = uniform_complex(rng, gen(rng), dtype)
            check(gbfft_lib, "fft", MODES[int(rng.integers(0, 3))], x)


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_fft2d_fft3d_generator_shapes(gbfft_lib, dtype):
    rng = np.random.default_rng(13)
    for _ in range(12):
        x = uniform_complex(rng, dim2(rng), dtype)
        check(gbfft_lib, "fft2D", MODES[int(rng.integers(0, 3))], x)
        x = uniform_complex(rng, dim3(rng), dtype)
        check(gbfft_lib, "fft3D", MODES[int(rng.integers(0, 3))], x)


@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (7, 1), (3, 8192), (8192, 3), (2, 16384),
                                   (16384, 2), (600, 1009), (1009, 24), (12, 10007)])
def test_fft2d_edge_shapes(gbfft_lib, shape):
    rng = np.random.default_rng(sum(shape))
    x = uniform_complex(rng, shape, np.complex64)
    for mode in MODES:
        check(gbfft_lib, "fft2D", mode, x, same_precision=max(shape) <= 8192)


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 3, 5), (16, 32, 64), (64, 1, 1), (1, 1, 300),
                                   (5, 9000, 2), (9000, 2, 3), (7, 11, 13)])
def test_fft3d_edge_shapes(gbfft_lib, shape):
    rng = np.random.default_rng(sum(shape))
    x = uniform_complex(rng, shape, np.complex64)
    for mode in MODES:
        check(gbfft_lib, "fft3D", mode, x, same_precision=max(shape) <= 8192)


def test_config1_fft1d_c64_roundtrip(gbfft_lib):
    # fft1D Forward then Inverse on one Complex Double vector, N = 1024, U[-1, 1]
    g = gbfft_lib
    rng = np.random.default_rng(1024)
    x = uniform_complex(rng, (1024,), np.complex128)
    t = torch.from_numpy(x).cuda()
    X = g.fft1D("forward", t)
    xr = g.fft1D("inverse", X).cpu().numpy()
    naive = O.dft_naive(-1, x)
    assert rel_l2(X.cpu().numpy(), naive) < 1e-13
    assert rel_l2(X.cpu().numpy(), O.fft1D(0, x)) < 1e-13
    assert rel_l2(xr, x) < 1e-14


@pytest.mark.parametrize("rows", [1, 3, 16, 17])
def test_c64_1024_vectors_cluster_path(gbfft_lib, rows):
    """A few Complex Double vectors of 1024 run one per 8-CTA cluster
    (vec1024_kernel, up to 16 vectors); 17 go to the throughput kernels.
    Every mode against FP64, the fused shift (of the single-vector full plan)
    bit-identical to shifting the plain result, and an input that the
    transform may not modify."""
    g = gbfft_lib
    rng = np.random.default_rng(1000 + rows)
    shape = (rows, 1024) if rows > 1 else (1024,)
    x = uniform_complex(rng, shape, np.complex128)
    t = torch.from_numpy(x).cuda()
    plan = g.Plan(shape, kind="many" if rows > 1 else "full", dtype=torch.complex128)
    assert ("vec1024_kernel" in plan.pass_kernels()) == (rows <= 16), plan.describe()
    for mode in MODES:
        y = plan(mode, t).cpu().numpy()
        assert rel_l2(y, np_reference("fft", MODE_IDX[mode], x)) < 1e-14, (rows, mode)
        if rows == 1:  # fused shifts are offered on full plans
            assert np.array_equal(plan(mode, t, shift_out="shift").cpu().numpy(), O.shift(y)), mode
            assert np.array_equal(plan(mode, t, shift_out="ishift").cpu().numpy(), O.shift(y, inverse=True)), mode
    assert np.array_equal(t.cpu().numpy(), x)
    from gbfft import _lib as L
    assert L.lib().gbfft_exec_status(plan.handle, None) == 0
    plan.close()


@pytest.mark.parametrize("shape,dt,split", [((8192, 64), np.complex64, True), ((8192, 24), np.complex64, True),
                                            ((3, 8192, 16), np.complex64, True), ((6144, 16), np.complex64, True),
                                            ((3000, 16), np.complex64, False)])
def test_long_strided_axes_four_step(gbfft_lib, shape, dt, split):
    """Strided axes longer than 2048 without a strided kernel of their own
    run as two four-step passes when a half of the split has a strided
    kernel (8192 = 64 x 128, 6144 = 64 x 96) and as one generic pass
    otherwise (3000 = 50 x 60); every mode against FP64."""
    g = gbfft_lib
    rng = np.random.default_rng(sum(shape))
    x = uniform_complex(rng, shape, dt)
    plan = g.Plan(shape, kind="full", dtype=torch.complex64 if dt == np.complex64 else torch.complex128)
    assert ("four-step" in plan.describe()) == split, plan.describe()
    xt = torch.from_numpy(x).cuda()
    fam = {2: "fft2D", 3: "fft3D"}[len(shape)]
    for mode in MODES:
        y = plan(mode, xt).cpu().numpy()
        assert rel_l2(y, np_reference(fam, MODE_IDX[mode], x)) < tol_fp64(dt, shape), (shape, mode)
    from gbfft import _lib as L
    assert L.lib().gbfft_exec_status(plan.handle, None) == 0
    plan.close()


# ---- reference properties (test/Test/FFT.hs:112-236) on the GPU -------------
def _rev(x):
    n = x.shape[-1]
    return x[..., (-np.arange(n)) % n]


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("gen,full", [(dim1, "fft1D"), (dim2, "fft2D"), (dim3, "fft3D")])
def test_reference_properties_gpu(gbfft_lib, dtype, gen, full):
    g = gbfft_lib
    rng = np.random.default_rng(hash((full, str(dtype))) % 2**32)
    tol = 1e-12 if dtype == np.complex128 else 1e-5
    F = lambda m, a: run_gpu(g, full, m, a)
    G = lambda m, a: run_gpu(g, "fft" if full != "fft1D" else "fft1D", m, a)
    for _ in range(6):
        sh = gen(rng)
        mode = MODES[int(rng.integers(0, 3))]
        x = uniform_complex(rng, sh, dtype)
        y = uniform_complex(rng, sh, dtype)
        a = uniform_complex(rng, (), dtype)
        assert rel_l2(F(mode, (a * x).astype(dtype)), a * F(mode, x)) < tol           # homogeneity
        assert rel_l2(F(mode, (x + y).astype(dtype)), F(mode, x) + F(mode, y)) < tol   # additivity
        assert rel_l2(F("inverse", F("forward", x)), x) < tol                           # inverse
        assert rel_l2(_rev(G(mode, x)), G(mode, _rev(x).copy())) < tol                  # reverse
        assert rel_l2(np.conj(G(mode, x)), G(mode, np.conj(_rev(x)).astype(dtype))) < tol  # conjugate
        m2 = MODES[int(rng.integers(0, 2))]
        n = sh[-1]
        fx, fy = G(m2, x).astype(np.complex128), G(m2, y).astype(np.complex128)
        x64, y64 = x.astype(np.complex128), y.astype(np.complex128)
        assert rel_l2(np.linalg.norm(fx, axis=-1), np.sqrt(n) * np.linalg.norm(x64, axis=-1)) < tol  # isometry
        assert rel_l2(np.sum(fx * np.conj(fy), axis=-1), n * np.sum(x64 * np.conj(y64), axis=-1)) < 10 * tol  # unitarity


# ---- full-size configurations through size-independent properties ---------
def test_config2_fft2d_4096_full(gbfft_lib):
    g = gbfft_lib
    rng = np.random.default_rng(2)
    x = (rng.standard_normal((4096, 4096)) + 1j * rng.standard_normal((4096, 4096))).astype(np.complex64)
    t = torch.from_numpy(x).cuda()
    y = g.fft2D("forward", t)
    ref = np.fft.fft2(x.astype(np.complex128))
    assert rel_l2(y.cpu().numpy(), ref) < 2e-6
    back = g.fft2D("inverse", y)
    assert rel_l2(back.cpu().numpy(), x) < 2e-6
    # linearity at full size
    s = g.fft2D("forward", 2.5 * t) - 2.5 * y
    assert float(s.abs().max()) < 1e-3 * float(y.abs().max())


def test_config3_many_full_sizes(gbfft_lib):
    g = gbfft_lib
    rng = np.random.default_rng(3)
    for rows, n in ((65536, 1000), (4096, 1009)):
        x = torch.complex(torch.randn(rows, n, generator=torch.Generator().manual_seed(n)),
                          torch.randn(rows, n, generator=torch.Generator().manual_seed(n + 1)))
        t = x.cuda()
        y = g.fft("forward", t)
        idx = rng.choice(rows, 64, replace=False)
        sub = x.numpy()[idx].astype(np.complex128)
        assert rel_l2(y.cpu().numpy()[idx], O.dft_naive(-1, sub)) < 4e-6
        back = g.fft("inverse", y)
        assert rel_l2(back.cpu().numpy(), x.numpy()) < 4e-6
        # Parseval per row
        ny = torch.linalg.vector_norm(y, dim=-1).double()
        nx = torch.linalg.vector_norm(t, dim=-1).double() * np.sqrt(n)
        assert float(((ny - nx).abs() / nx).max()) < 1e-5


def test_config5_shape_3d_roundtrip(gbfft_lib):
    g = gbfft_lib
    t = torch.complex(torch.randn(256, 256, 256), torch.randn(256, 256, 256)).cuda()
    y = g.fft3D("forward", t)
    ref = torch.fft.fftn(t.to(torch.complex128))
    err = float(torch.linalg.vector_norm(y.to(torch.complex128) - ref) / torch.linalg.vector_norm(ref))
    assert err < 2e-6
    back = g.fft3D("inverse", y)
    assert float(torch.linalg.vector_norm(back - t) / torch.linalg.vector_norm(t)) < 2e-6


@pytest.mark.parametrize("shape", [(256, 256), (5, 256, 256), (1, 256, 256)])
def test_plane_pass_256(gbfft_lib, shape, monkeypatch):
    """With GBFFT_ENABLE=plane, fft2D of 256 x 256 and fft3D of d x 256 x 256
    run the x and y axes as one cluster pass per plane; every mode against
    FP64 and the output shift (its fallback pass) against shifting the
    result."""
    monkeypatch.setenv("GBFFT_ENABLE", "plane")
    g = gbfft_lib
    rng = np.random.default_rng(len(shape))
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    plan = g.Plan(shape, kind="full", dtype=torch.complex64)
    assert plan.pass_kernels()[0] == "plane256_kernel", plan.pass_kernels()
    xt = torch.from_numpy(x).cuda()
    fam = {2: "fft2D", 3: "fft3D"}[len(shape)]
    for mode in MODES:
        y = plan(mode, xt).cpu().numpy()
        assert rel_l2(y, np_reference(fam, MODE_IDX[mode], x)) < 2e-6, mode
    assert np.array_equal(plan("forward", xt, shift_out="shift").cpu().numpy(),
                          O.shift(plan("forward", xt).cpu().numpy()))
    assert torch.equal(xt.cpu(), torch.from_numpy(x))


# ---- edge cases and error behaviour -----------------------------------------
def test_empty_and_unit_arrays(gbfft_lib):
    g = gbfft_lib
    for shape in ((0,), (0, 5), (5, 0), (3, 0, 2)):
        t = torch.zeros(shape, dtype=torch.complex64, device="cuda")
        assert g.fft("forward", t).shape == t.shape
    t = torch.tensor([1.5 - 2j], dtype=torch.complex64, device="cuda")
    for mode in MODES:
        assert torch.equal(g.fft1D(mode, t), t)


def test_error_codes(gbfft_lib):
    import ctypes
    from gbfft import _lib as L
    lib = L.lib()
    h = ctypes.c_void_p()
    dims = (ctypes.c_int64 * 2)(4, 4)
    assert lib.gbfft_plan_create(ctypes.byref(h), 0, dims, 1, 0, 0) == L.ERR_INVALID_ARG
    assert lib.gbfft_plan_create(ctypes.byref(h), 6, dims, 0, 0, 0) == L.ERR_INVALID_ARG
    dims4 = (ctypes.c_int64 * 4)(2, 2, 4, 4)
    assert lib.gbfft_plan_create(ctypes.byref(h), 4, dims4, 1, 0, 0) == L.ERR_UNSUPPORTED  # no full 4D
    assert lib.gbfft_plan_create(ctypes.byref(h), 2, dims, 7, 0, 0) == L.ERR_INVALID_ARG
    assert lib.gbfft_plan_create(ctypes.byref(h), 2, dims, 1, 3, 0) == L.ERR_INVALID_ARG
    neg = (ctypes.c_int64 * 2)(4, -1)
    assert lib.gbfft_plan_create(ctypes.byref(h), 2, neg, 1, 0, 0) == L.ERR_INVALID_ARG
    assert lib.gbfft_exec(None, -1, None, None, None) == L.ERR_NULL_PLAN
    assert lib.gbfft_plan_create(ctypes.byref(h), 2, dims, 1, 0, 0) == L.OK
    a = torch.zeros(16, dtype=torch.complex64, device="cuda")
    b = torch.zeros(16, dtype=torch.complex64, device="cuda")
    assert lib.gbfft_exec(h, 5, a.data_ptr(), b.data_ptr(), None) == L.ERR_INVALID_ARG
    assert lib.gbfft_exec(h, -1, a.data_ptr(), a.data_ptr(), None) == L.ERR_INVALID_ARG
    assert lib.gbfft_exec(h, -1, None, b.data_ptr(), None) == L.ERR_INVALID_ARG
    assert lib.gbfft_exec(h, -1, a.data_ptr() + 4, b.data_ptr(), None) == L.ERR_INVALID_ARG
    assert lib.gbfft_exec(h, -1, a.data_ptr(), b.data_ptr(), None) == L.OK
    assert lib.gbfft_plan_destroy(h) == L.OK
    with pytest.raises(TypeError):
        g = gbfft_lib
        g.fft("forward", torch.zeros(4, device="cuda"))


def test_plan_cache_and_concurrent_streams(gbfft_lib):
    g = gbfft_lib
    rng = np.random.default_rng(7)
    x = uniform_complex(rng, (64, 1000), np.complex64)
    t = torch.from_numpy(x).cuda()
    ref = np_reference("fft", 0, x)
    streams = [torch.cuda.Stream() for _ in range(4)]
    outs = []
    for s in streams:
        with torch.cuda.stream(s):
            outs.append(g.fft("forward", t, stream=s))
    torch.cuda.synchronize()
    for o in outs:
        assert rel_l2(o.cpu().numpy(), ref) < 2e-6


@pytest.mark.parametrize("shape,kind", [((6, 40009), "many"), ((16, 10007), "many")])
def test_scratch_plan_on_concurrent_streams(gbfft_lib, shape, kind):
    """A plan with scratch (multi-pass Bluestein) run on several streams at
    once, each stream with its own input: the executions are ordered on the
    shared scratch."""
    g = gbfft_lib
    rng = np.random.default_rng(8)
    plan = g.Plan(shape, kind=kind, dtype=torch.complex64)
    assert plan.info["workspace_bytes"] > 0
    xs = [uniform_complex(rng, shape, np.complex64) for _ in range(4)]
    ts = [torch.from_numpy(x).cuda() for x in xs]
    torch.cuda.synchronize()
    streams = [torch.cuda.Stream() for _ in range(4)]
    outs = []
    for rep in range(3):
        for t, s in zip(ts, streams):
            with torch.cuda.stream(s):
                outs.append(plan("forward", t, stream=s))
    torch.cuda.synchronize()
    for i, o in enumerate(outs):
        x = xs[i % 4]
        ref = np.fft.fft(x.astype(np.complex128), axis=-1) if kind == "many" else \
            np.fft.fftn(x.astype(np.complex128))
        assert rel_l2(o.cpu().numpy(), ref) < 4e-6, (i, plan.describe())
    plan.close()


def test_fault_injection_alloc(gbfft_lib, monkeypatch):
    import ctypes
    from gbfft import _lib as L
    monkeypatch.setenv("GBFFT_FAULT_INJECT", "alloc")
    h = ctypes.c_void_p()
    dims = (ctypes.c_int64 * 1)(1024)
    assert L.lib().gbfft_plan_create(ctypes.byref(h), 1, dims, 1, 0, 0) == L.ERR_ALLOC
    assert not h.value


# ---- kernel variants: TMA-fed rows, register rows, cluster columns, generic --
@pytest.mark.parametrize("disable,rowv,colv", [("", "1", "2"), ("", "0", "0"), ("tma", "0", "1"),
                                               ("", "1", "3"), ("", "1", "4"), ("", "1", "5"),
                                               ("", "1", "6"), ("", "1", "7"), ("", "1", "8"),
                                               ("", "1", "9"), ("", "1", "10"), ("", "1", "11"),
                                               ("", "1", "12"), ("", "1", "13"), ("", "1", "14"),
                                               ("", "1", "15"), ("", "1", "16"), ("", "1", "17"),
                                               ("", "1", "18"), ("", "1", "19"), ("tma", "1", "14"), ("strided", "1", "9"),
                                               ("row", "1", "2"),
                                               ("cluster", "1", "2"), ("tma,row,cluster", "0", "0")])
def test_kernel_variants_agree(gbfft_lib, monkeypatch, disable, rowv, colv):
    g = gbfft_lib
    from gbfft import _lib as L
    monkeypatch.setenv("GBFFT_DISABLE", disable)
    monkeypatch.setenv("GBFFT_ROW_VARIANT", rowv)
    monkeypatch.setenv("GBFFT_ROW_TMA", "1" if rowv == "0" else "0")  # bulk-copy-fed rows
    monkeypatch.setenv("GBFFT_COL_VARIANT", colv)
    rng = np.random.default_rng(99)
    cases = [((4096, 4096), "full", np.complex64), ((300, 1024), "many", np.complex64),
             ((64, 1000), "many", np.complex64), ((67, 1000), "many", np.complex64),
             ((5, 8192), "many", np.complex64),
             ((41, 256), "many", np.complex64), ((3, 2048), "full", np.complex64),
             ((7, 512), "many", np.complex64), ((33, 4096), "many", np.complex128),
             ((2, 4096, 32), "full", np.complex64), ((256, 48), "full", np.complex64),
             ((1024, 64), "full", np.complex64), ((3, 256, 32), "full", np.complex64),
             ((128, 16, 64), "full", np.complex64), ((512, 16), "full", np.complex128),
             ((64, 64, 16), "full", np.complex64), ((33, 1009), "many", np.complex64),
             ((5, 4001), "many", np.complex64), ((210, 243), "full", np.complex64)]
    for shape, kind, dt in cases:
        x = uniform_complex(rng, shape, dt)
        plan = g.Plan(shape, kind=kind, dtype=torch.complex64 if dt == np.complex64 else torch.complex128)
        for mode in MODES:
            y = plan(mode, torch.from_numpy(x).cuda()).cpu().numpy()
            ref = np_reference("fft2D" if kind == "full" else "fft", MODE_IDX[mode], x) if len(shape) == 2 \
                else np_reference("fft3D" if kind == "full" else "fft", MODE_IDX[mode], x)
            assert rel_l2(y, ref) < tol_fp64(dt, shape), (shape, kind, mode, disable, plan.describe())
        assert L.lib().gbfft_exec_status(plan.handle, None) == 0
        plan.close()


def test_row_kernel_input_not_16_byte_aligned(gbfft_lib):
    # an 8-byte-aligned view: the TMA bulk copy needs 16 bytes, the planner
    # falls back to direct loads
    g = gbfft_lib
    rng = np.random.default_rng(5)
    rows, n = 64, 4096
    base = torch.from_numpy(uniform_complex(rng, (rows * n + 1,), np.complex64)).cuda()
    view = base[1:].view(rows, n)
    assert view.data_ptr() % 16 == 8
    plan = g.Plan((rows, n), kind="many", dtype=torch.complex64)
    out = torch.empty((rows, n), dtype=torch.complex64, device="cuda")
    plan.exec_ptr("forward", view.data_ptr(), out.data_ptr())
    ref = np.fft.fft(view.cpu().numpy().astype(np.complex128), axis=-1)
    assert rel_l2(out.cpu().numpy(), ref) < 2e-6


# ---- split-FP16 tensor-core radix-16 stages ---------------------------------
TC_KERNELS = ("rowfft_tc_kernel", "tcdft_mma_kernel", "tcdft8_kernel")


def test_split_fp16_without_tensor_core_pass_is_refused(gbfft_lib):
    # a split-FP16 request that no tensor-core kernel serves is refused, not
    # silently run in FP32
    g = gbfft_lib
    from gbfft import _lib as L
    with pytest.raises(L.GbfftError) as ei:
        g.Plan((4, 3000), kind="many", dtype=torch.complex64, precision="split_fp16")
    assert ei.value.status == L.ERR_UNSUPPORTED


@pytest.mark.parametrize("shape,kind", [((4096, 4096), "full"), ((300, 4096), "many"), ((100, 1024), "many"),
                                        ((64, 256), "many"), ((8, 8192), "many"), ((17, 2048), "many"),
                                        ((5, 512), "many"), ((3, 256, 256), "full"),
                                        # dense tensor-core rows (tcdft): Bluestein-class and other lengths
                                        ((4096, 1009), "many"), ((130, 1009), "many"), ((1009,), "full"),
                                        ((3, 7, 97), "many"), ((257, 3), "many"), ((9, 4), "many"),
                                        ((6, 1000), "many"), ((40, 2047), "many"), ((5, 2048 - 2), "many"),
                                        ((20, 1009), "full"),
                                        # fused radix-8 + dense odd stage (tcdft8): n = 8 * odd
                                        ((8192, 1000), "many"), ((33, 1000), "many"), ((17, 24), "many"),
                                        ((5, 3, 40), "many"), ((100, 1016), "many"), ((31, 504), "many")])
def test_split_fp16_accuracy(gbfft_lib, shape, kind):
    # the specification's bar: <= 2e-6 relative L2 against FP64
    g = gbfft_lib
    rng = np.random.default_rng(sum(shape))
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    plan = g.Plan(shape, kind=kind, dtype=torch.complex64, precision="split_fp16")
    # a split-FP16 plan runs at least one pass on the tensor cores
    assert any(k in TC_KERNELS for k in plan.pass_kernels()), (shape, plan.pass_kernels())
    xt = torch.from_numpy(x).cuda()
    fam = {1: "fft1D", 2: "fft2D", 3: "fft3D"}[len(shape)] if kind == "full" else "fft"
    for mode in MODES:
        y = plan(mode, xt).cpu().numpy()
        e = rel_l2(y, np_reference(fam, MODE_IDX[mode], x))
        assert e < 2e-6, (shape, kind, mode, e, plan.describe())
    from gbfft import _lib as L
    assert L.lib().gbfft_exec_status(plan.handle, None) == 0
    # zero input stays zero, large and tiny magnitudes keep relative accuracy
    for scale in (0.0, 1e-20, 1e20):
        xs = (x * np.float32(scale)).astype(np.complex64)
        y = plan("forward", torch.from_numpy(xs).cuda()).cpu().numpy()
        ref = np_reference(fam, 0, xs)
        if scale == 0.0:
            assert np.all(y == 0)
        else:
            assert rel_l2(y, ref) < 2e-6, scale


# ---- strided passes: tensor-copy-fed persistent kernel vs direct loads ------
TMA_CASES = [((256, 48), "full", np.complex64), ((3, 256, 32), "full", np.complex64),
             ((2, 65536, 16), "full", np.complex64), ((256, 256, 16), "full", np.complex128),
             ((4, 65536), "many", np.complex64), ((8, 65521), "many", np.complex64),
             ((64, 256, 64), "full", np.complex64)]


@pytest.mark.parametrize("shape,kind,dt", TMA_CASES)
def test_strided_tensor_copy_kernel(gbfft_lib, monkeypatch, shape, kind, dt):
    """Each layout runs once with the tensor-copy kernel (at least one pass
    must use it) and once with it disabled; both must match FP64 and agree."""
    g = gbfft_lib
    from gbfft import _lib as L
    rng = np.random.default_rng(2024)
    x = uniform_complex(rng, shape, dt)
    tdt = torch.complex64 if dt == np.complex64 else torch.complex128
    name = ("fft3D" if len(shape) == 3 else "fft2D") if kind == "full" else "fft"
    outs = {}
    for disable in ("", "tma"):
        monkeypatch.setenv("GBFFT_DISABLE", disable)
        plan = g.Plan(shape, kind=kind, dtype=tdt)
        kernels = plan.pass_kernels()
        if disable == "":
            assert "strfft_tma_kernel" in kernels, (shape, kernels, plan.describe())
        else:
            assert "strfft_tma_kernel" not in kernels
        for mode in MODES:
            y = plan(mode, torch.from_numpy(x).cuda()).cpu().numpy()
            ref = np_reference(name, MODE_IDX[mode], x)
            assert rel_l2(y, ref) < tol_fp64(dt, shape if kind == "full" else shape[-1:]), \
                (shape, mode, disable, plan.describe())
            outs[(disable, mode)] = y
        assert L.lib().gbfft_exec_status(plan.handle, None) == 0
        plan.close()
    for mode in MODES:
        assert rel_l2(outs[("", mode)], outs[("tma", mode)]) < 2 * tol_fp64(dt, shape if kind == "full"
                                                                            else shape[-1:])


@pytest.mark.parametrize("shape,kind", [((65536, 16), "full"), ((4, 65536), "many")])
def test_strided_input_not_16_byte_aligned(gbfft_lib, shape, kind):
    # the first pass of these plans is a strided four-step half reading the
    # caller's input; an 8-byte-aligned view cannot be described by a tensor
    # map (16-byte base), so that launch falls back to direct loads
    g = gbfft_lib
    rng = np.random.default_rng(6)
    n = int(np.prod(shape))
    base = torch.from_numpy(uniform_complex(rng, (n + 1,), np.complex64)).cuda()
    view = base[1:].view(*shape)
    assert view.data_ptr() % 16 == 8
    plan = g.Plan(shape, kind=kind, dtype=torch.complex64)
    assert plan.pass_kernels()[0] == "strfft_tma_kernel", plan.describe()
    out = torch.empty(shape, dtype=torch.complex64, device="cuda")
    plan.exec_ptr("forward", view.data_ptr(), out.data_ptr())
    xv = view.cpu().numpy().astype(np.complex128)
    ref = np.fft.fft2(xv) if kind == "full" else np.fft.fft(xv, axis=-1)
    assert rel_l2(out.cpu().numpy(), ref) < 2e-6


@pytest.mark.parametrize("shape", [(2, 3, 4, 5, 96), (3, 2, 2, 1009), (2, 2, 3, 4096)])
def test_fft_rank4_and_5(gbfft_lib, shape):
    """The innermost-axis transform of rank-4 and rank-5 arrays runs on the
    GPU (the reference's PTX path stops at rank 3), in every mode."""
    g = gbfft_lib
    from gbfft import _lib as L
    rng = np.random.default_rng(40)
    x = uniform_complex(rng, shape, np.complex64)
    for mode in MODES:
        check(g, "fft", mode, x, same_precision=False)
    # the C ABI takes the rank directly; a full 4D transform is not offered
    dims = (ctypes.c_int64 * len(shape))(*shape)
    h = ctypes.c_void_p()
    assert L.lib().gbfft_plan_create(ctypes.byref(h), len(shape), dims, L.KIND_MANY, L.C32, L.PLAIN) == L.OK
    L.lib().gbfft_plan_destroy(h)
    assert L.lib().gbfft_plan_create(ctypes.byref(h), len(shape), dims, L.KIND_FULL, L.C32,
                                     L.PLAIN) == L.ERR_UNSUPPORTED


def test_probe_tile_copy(gbfft_lib):
    """The bandwidth probe of the passes' access patterns copies the array
    exactly at every tile width (powers of two, whole rows of 1000, runs of a
    24000-column row), and refuses widths that do not tile."""
    from gbfft import _lib as L
    import ctypes
    x = torch.randn(300, 256, dtype=torch.complex64, device="cuda")
    for w in (2, 16, 64, 256):
        y = torch.zeros_like(x)
        assert L.lib().gbfft_probe_tile_copy(300, 256, w, ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(y.data_ptr()), None) == 0
        torch.cuda.synchronize()
        assert torch.equal(x, y), w
    big = torch.randn(4, 16384, dtype=torch.complex64, device="cuda")
    y = torch.zeros_like(big)
    assert L.lib().gbfft_probe_tile_copy(4, 16384, 16384, ctypes.c_void_p(big.data_ptr()),
                                         ctypes.c_void_p(y.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(big, y)
    rows = torch.randn(64, 1000, dtype=torch.complex64, device="cuda")
    y = torch.zeros_like(rows)
    assert L.lib().gbfft_probe_tile_copy(64, 1000, 1000, ctypes.c_void_p(rows.data_ptr()),
                                         ctypes.c_void_p(y.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(rows, y)
    wide = torch.randn(3, 2 * 12000, dtype=torch.complex64, device="cuda")
    y = torch.zeros_like(wide)
    assert L.lib().gbfft_probe_tile_copy(3, 24000, 24000, ctypes.c_void_p(wide.data_ptr()),
                                         ctypes.c_void_p(y.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(wide, y)
    y = torch.zeros_like(x)
    for bad in (24, 3, 0):
        assert L.lib().gbfft_probe_tile_copy(300, 256, bad, ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(y.data_ptr()), None) == L.ERR_INVALID_ARG
