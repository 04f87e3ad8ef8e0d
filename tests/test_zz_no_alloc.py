"""The no-allocation render pass (bling_render_pass_noalloc).

Some callers cannot let the library call cudaMalloc while they render: a
render server that reserved its device memory up front for resident scenes and
films, or a host sharing the GPU with another caching allocator, where an
allocation mid-frame could fail and cudaMalloc/cudaFree would stall the
device.  This entry point renders into the caller's device film and keeps its
path state in a static device array of the library (at most 65536 path
samples per call).

Checked here through the C ABI: two calls in a row agree with the allocating
entry point (bling_render_pass) on the same film-sized job, within the render
tests' tolerance, and with the CPU oracle within the parity bar of the render
tests; a pass over the limit and a film that is host memory are refused with a
clear error before anything runs on the device.
This file is collected last, so a run that stops at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from bling_gb300 import abi
from bling_gb300 import scene as S
from bling_gb300.api import lib
from oracle.oracle import OracleScene

pytestmark = pytest.mark.gpu


def _bind():
    L = lib()
    L.bling_render_pass_noalloc.argtypes = [C.c_void_p, C.POINTER(abi.RenderParams), C.c_uint64,
                                            C.c_void_p]
    L.bling_render_pass_noalloc.restype = C.c_int
    return L


def test_noalloc_pass_matches_render_pass_twice(gpu_ctx):
    L = _bind()
    w = h = 48  # 50 x 50 sample extent x 16 strata = 40000 path samples per pass
    sc = S.cornell_room(w, h)
    params = S.cornell_params(w, h, spp_side=4)
    g = gpu_ctx.scene(sc)
    film_ref = gpu_ctx.film(w, h)
    d_film = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for k in range(2):
        g.render_pass(film_ref, params, k)
        rc = L.bling_render_pass_noalloc(g.h, C.byref(params), k, C.c_void_p(d_film.data_ptr()))
        assert rc == 0, L.bling_last_error(gpu_ctx.h).decode()
        torch.cuda.synchronize()
        ref = film_ref.read()
        out = d_film.cpu().numpy()
        # box filter: weights are sums of 1.0 and must agree exactly
        assert np.array_equal(out[..., 0], ref[..., 0])
        # same kernels, same random numbers: only the order of atomic adds differs
        assert np.allclose(out[..., 1:], ref[..., 1:], rtol=1e-5, atol=1e-6)
        assert out[..., 2].mean() > 0
    # the two passes against the oracle's: weights exact (box filter), XYZ
    # within 1e-3 relative for >= 97% of pixels, image means within 0.5%
    o = OracleScene(sc)
    fo, _ = o.render_pass(params, 0)
    fo, _ = o.render_pass(params, 1, fo)
    out = d_film.cpu().numpy()
    assert np.array_equal(out[..., 0], fo[..., 0])
    scale = np.abs(fo[..., 1:]).mean() + 1e-12
    err = np.abs(out[..., 1:] - fo[..., 1:]) / (np.abs(fo[..., 1:]) + 1e-3 * scale)
    assert (err <= 1e-3).all(-1).mean() >= 0.97
    m_g, m_o = out[..., 1:].mean(axis=(0, 1)), fo[..., 1:].mean(axis=(0, 1))
    assert np.all(np.abs(m_g - m_o) <= 5e-3 * np.abs(m_o))


def test_noalloc_pass_refuses_a_host_film(gpu_ctx):
    """A film in host memory is refused on the host (the pointer's memory
    type is checked before any launch), so no kernel ever sees it."""
    L = _bind()
    w = h = 16
    sc = S.cornell_room(w, h)
    params = S.cornell_params(w, h, spp_side=1)
    g = gpu_ctx.scene(sc)
    host = np.zeros((h, w, 4), np.float32)
    rc = L.bling_render_pass_noalloc(g.h, C.byref(params), 0, C.c_void_p(host.ctypes.data))
    assert rc == abi.BLING_ERR_INVALID_ARG
    assert "device memory" in L.bling_last_error(gpu_ctx.h).decode()
    assert not host.any()


def test_noalloc_pass_refuses_oversized_passes(gpu_ctx):
    L = _bind()
    w = h = 96  # 98 x 98 x 16 = 153664 path samples: over the 65536 limit
    sc = S.cornell_room(w, h)
    params = S.cornell_params(w, h, spp_side=4)
    g = gpu_ctx.scene(sc)
    d_film = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = L.bling_render_pass_noalloc(g.h, C.byref(params), 0, C.c_void_p(d_film.data_ptr()))
    assert rc == abi.BLING_ERR_BOUNDS
    msg = L.bling_last_error(gpu_ctx.h).decode()
    assert "153664" in msg and "65536" in msg
    assert float(d_film.abs().sum()) == 0.0
