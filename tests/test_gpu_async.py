"""The reference entry points on a caller's stream in asynchronous mode (mitos_set_stream): the same
grids as the synchronous calls, and capturable into the caller's CUDA graph (the *_async form of
fft_r2c_dg / fft_apply_kernel_dg / fft_c2r_dg, src/fft.c:219-302, and of generate_complex_grf,
src/grf.c:26-69)."""
import numpy as np
import pytest

import mitos_gb300.lib as ml

pytestmark = pytest.mark.gpu


def _chain(g):
    ml.fft_r2c_dg(g)
    assert ml.fft_apply_kernel_dg(g, g, "inv_poisson") == 0
    ml.fft_c2r_dg(g)


@pytest.mark.parametrize("prec", [ml.FP32, ml.FP64])
def test_async_chain_in_a_captured_graph(prec):
    torch = pytest.importorskip("torch")
    N, L = 64, 100.0
    g = ml.alloc_local_grid(N, L, prec)
    try:
        dt = np.float32 if prec == ml.FP32 else np.float64
        real = np.random.default_rng(9).standard_normal((N, N, N + 2)).astype(dt)
        ml.set_box(g, real)
        _chain(g)  # synchronous, on the library stream: the reference result and the warm-up
        ref = ml.get_box(g)[..., :N].copy()
        ml.set_box(g, real)
        s = torch.cuda.Stream()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=s):
            ml.set_stream(s.cuda_stream, True)
            try:
                _chain(g)
            finally:
                ml.set_stream(0)
        assert np.array_equal(ml.get_box(g)[..., :N], real[..., :N])  # captured, not run
        for _ in range(2):
            ml.set_box(g, real)
            graph.replay()
            torch.cuda.synchronize()
            assert np.array_equal(ml.get_box(g)[..., :N], ref)
    finally:
        ml.set_stream(0)
        ml.free_local_grid(g)


def test_async_noise_on_a_caller_stream():
    """generate_complex_grf enqueued on a torch stream without synchronising: the same noise"""
    torch = pytest.importorskip("torch")
    N, L = 32, 64.0
    g = ml.alloc_local_grid(N, L, ml.FP64)
    try:
        ml.generate_complex_grf(g, ml.rng_init(3))
        ref = ml.get_fbox(g).copy()
        s = torch.cuda.Stream()
        ml.set_stream(s.cuda_stream, True)
        try:
            ml.generate_complex_grf(g, ml.rng_init(3))
        finally:
            ml.set_stream(0)
        s.synchronize()
        assert np.array_equal(ml.get_fbox(g), ref)
    finally:
        ml.free_local_grid(g)
