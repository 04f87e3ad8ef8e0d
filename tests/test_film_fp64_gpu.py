"""Compensated film accumulation (BLING_FILM_FP64) on the GPU.

Every pass is summed in FP32 by the kernels and then added into FP64 totals,
so FP32 rounding never spans more than one pass.  After 1536 samples per
pixel (96 passes of 16) the FP64 film must equal the float64 sum of the
passes' own films within 1e-6 relative (the FP32 sums of one pass differ
between runs only in the order of their additions), and its box-filter
weights must be the exact sample counts."""
import numpy as np
import pytest

from bling_gb300 import scene as S

pytestmark = pytest.mark.gpu


def test_fp64_film_equals_the_float64_sum_of_its_passes(gpu_ctx):
    sc = S.cornell_room(16, 16)
    g = gpu_ctx.scene(sc)
    p = S.cornell_params(16, 16, spp_side=4)
    passes = 96
    f64 = gpu_ctx.film(16, 16, fp64=True)
    f32 = gpu_ctx.film(16, 16)
    one = gpu_ctx.film(16, 16)
    ref = np.zeros((16, 16, 4), np.float64)
    for k in range(passes):
        g.render_pass(f64, p, k)
        g.render_pass(f32, p, k)
        one.clear()
        g.render_pass(one, p, k)
        ref += one.read().astype(np.float64)
    acc = f64.read_f64()
    assert np.array_equal(acc[..., 0], ref[..., 0])
    assert np.array_equal(acc[..., 0], np.full((16, 16), passes * 16.0))
    scale = np.abs(ref[..., 1:]).max()
    err64 = np.abs(acc[..., 1:] - ref[..., 1:]).max() / scale
    assert err64 <= 1e-6, err64
    # read() hands out the totals rounded once to float
    assert np.array_equal(f64.read(), acc.astype(np.float32))
    err32 = np.abs(f32.read()[..., 1:].astype(np.float64) - ref[..., 1:]).max() / scale
    print(f"relative error after {passes * 16} spp: fp64 film {err64:.2e}, fp32 film {err32:.2e}")


def test_fold_after_batched_jobs(gpu_ctx):
    from bling_gb300.api import Batch
    sc = S.cornell_room(16, 16)
    g = gpu_ctx.scene(sc)
    p = S.cornell_params(16, 16, spp_side=2)
    f64 = gpu_ctx.film(16, 16, fp64=True)
    ref = gpu_ctx.film(16, 16)
    b = Batch(gpu_ctx, slots=2048)
    for k in range(4):
        b.submit(g, f64, p, k)
        b.run()
        f64.fold()
        g.render_pass(ref, p, k)
    b.close()
    r = ref.read().astype(np.float64)
    a = f64.read_f64()
    assert np.array_equal(a[..., 0], r[..., 0])
    assert np.allclose(a[..., 1:], r[..., 1:], rtol=1e-5, atol=1e-6 * np.abs(r[..., 1:]).max())
