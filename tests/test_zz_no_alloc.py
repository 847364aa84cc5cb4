"""dmtz_extract_noalloc: the allocation-free entry point for callers that
cannot call cudaMalloc (applications whose device memory belongs to their own
pool allocator, or pipelines that cannot afford the device synchronisation a
cudaMalloc/cudaFree brings).  It must give exactly what dmtz_extract gives,
on consecutive calls that share its fixed scratch array, and refuse grids
larger than that array.  Runs last (file name) so a failure here cannot hide
the other tests' results; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    import dmtz_gb300 as dm

    L = dm.load_library()
    fn = L.dmtz_extract_noalloc
    fn.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 6
    fn.restype = ctypes.c_int
    return fn


def test_extract_noalloc_matches_extract():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import dmtz_gb300 as dm
    from dmtz_gb300 import synth

    fn = _noalloc_fn()
    ctx = dm.Context(0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    # two consecutive calls on different fields and sizes: the second reuses
    # the scratch the first left behind
    for dims, seed in (((40, 36, 30), 31), ((24, 20, 28), 32), ((64, 64, 64), 33)):
        f = synth.power_law(dims, seed).reshape(-1)
        want = ctx.extract(f, dims)
        V, E, F, T = dm.cell_counts(dims)
        d = torch.from_numpy(f).cuda()
        outs = [torch.full((n,), -7, dtype=torch.int32, device="cuda") for n in (V, E, F, T)]
        rc = fn(*dims, d.data_ptr(), *[o.data_ptr() for o in outs], stream.cuda_stream)
        assert rc == 0
        torch.cuda.synchronize()
        for got, ref, name in zip(outs, want, ("PV", "PE", "PF", "PT")):
            assert np.array_equal(got.cpu().numpy(), ref), name
    ctx.close()


def test_extract_noalloc_side_stream_and_thin_grids():
    """On a stream the caller created (synchronised on that stream alone),
    including grids with an extent of 2, where every anchor lies on the
    surface and takes the bounds-checked code."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import dmtz_gb300 as dm
    from dmtz_gb300 import synth

    fn = _noalloc_fn()
    ctx = dm.Context(0)
    torch.cuda.set_device(0)
    side = torch.cuda.Stream()
    for dims, seed in (((64, 2, 48), 41), ((2, 37, 5), 42), ((33, 31, 29), 43)):
        f = synth.power_law(dims, seed).reshape(-1)
        want = ctx.extract(f, dims)
        V, E, F, T = dm.cell_counts(dims)
        with torch.cuda.stream(side):
            d = torch.from_numpy(f).pin_memory().to("cuda", non_blocking=True)
            outs = [torch.full((n,), -7, dtype=torch.int32, device="cuda") for n in (V, E, F, T)]
        rc = fn(*dims, d.data_ptr(), *[o.data_ptr() for o in outs], side.cuda_stream)
        assert rc == 0
        side.synchronize()
        for got, ref, name in zip(outs, want, ("PV", "PE", "PF", "PT")):
            assert np.array_equal(got.cpu().numpy(), ref), (dims, name)
    ctx.close()


def test_extract_noalloc_rejects_large_grids():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fn = _noalloc_fn()
    d = torch.zeros(65 * 64 * 64, dtype=torch.float64, device="cuda")
    o = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = fn(65, 64, 64, d.data_ptr(), o.data_ptr(), o.data_ptr(), o.data_ptr(), o.data_ptr(), None)
    assert rc == 9  # DMTZ_ERR_TOO_LARGE, before anything is launched
