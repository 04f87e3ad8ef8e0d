"""Known answers and convergence of the GPU path integrator.

* White furnace: a Lambertian sphere of albedo rho under a uniform
  environment reflects exactly rho of it, at every depth limit >= 0 (direct
  light only: reflected rays of a convex object escape, and a diffuse bounce
  adds no environment radiance afterwards).  The GPU's sphere/background
  ratio must be within 0.3% of rho at 1024 spp.
* Convergence: a 4096-spp GPU render of the Cornell room (FP64-compensated
  film) against a 16384-spp render of the CPU oracle with the same seedless
  scene but independent random streams, summed in float64 over its passes.
  Relative RMSE (over pixels and X, Y, Z, divided by the reference's mean)
  must be within 1%, the bar for converged images; the measured value is
  printed.
"""
import numpy as np
import pytest

from bling_gb300 import scene as S
from oracle.oracle import OracleScene

pytestmark = pytest.mark.gpu


def _furnace_ratio(film):
    w = film[..., 0]
    y = film[..., 2] / np.where(w > 0, w, 1)
    h, wd = y.shape
    yy, xx = np.mgrid[0:h, 0:wd]
    r = np.hypot(xx + 0.5 - wd / 2, yy + 0.5 - h / 2)
    return y[r < 0.25 * wd].mean() / y[r > 0.48 * wd].mean()


@pytest.mark.parametrize("rho,depth", [(0.5, 0), (0.5, 5), (0.8, 3)])
def test_white_furnace(gpu_ctx, rho, depth):
    sc = S.furnace_scene(rho, 32, 32)
    g = gpu_ctx.scene(sc)
    f = gpu_ctx.film(32, 32, fp64=True)
    p = S.render_params(32, 32, (8, 8), max_depth=depth, sample_depth=3, rr_depth=7)
    for k in range(16):
        g.render_pass(f, p, k)
    ratio = _furnace_ratio(f.read_f64())
    assert abs(ratio - rho) < 0.003 * rho, ratio


def test_4096spp_converges_to_the_16k_oracle_render(gpu_ctx):
    sc = S.cornell_room(24, 24)
    g = gpu_ctx.scene(sc)
    f = gpu_ctx.film(24, 24, fp64=True)
    p = S.cornell_params(24, 24, spp_side=16, seed=5)  # 256 spp per pass
    for k in range(16):
        g.render_pass(f, p, k)
    a = f.read_f64()
    o = OracleScene(sc)
    po = S.cornell_params(24, 24, spp_side=32, seed=99)  # 1024 spp per pass
    ref = np.zeros((24, 24, 4), np.float64)
    for k in range(16):
        fo, _ = o.render_pass(po, k)
        ref += fo.astype(np.float64)
    xa = a[..., 1:] / a[..., :1]
    xr = ref[..., 1:] / ref[..., :1]
    rmse = float(np.sqrt(np.mean((xa - xr) ** 2)) / np.mean(xr))
    print(f"relative RMSE, 4096-spp GPU vs 16384-spp oracle: {rmse:.4%}")
    assert rmse <= 0.01, rmse
