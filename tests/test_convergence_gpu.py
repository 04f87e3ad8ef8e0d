"""Known answers and convergence of the GPU path integrator.

* White furnace: a Lambertian sphere of albedo rho under a uniform
  environment reflects exactly rho of it, at every depth limit >= 1 (direct
  light only: reflected rays of a convex object escape, and a diffuse bounce
  adds no environment radiance afterwards).  The GPU's sphere/background
  ratio must be within 0.3% of rho at 1024 spp.  At depth limit 0 the
  reference returns the path's radiance so far at the first hit
  (`depth == md = return l`, Integrator/Path.hs:51), so the sphere is
  black and the background (a miss on the camera ray) still sees the
  environment.
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


@pytest.mark.parametrize("rho,depth", [(0.5, 1), (0.5, 5), (0.8, 3)])
def test_white_furnace(gpu_ctx, rho, depth):
    sc = S.furnace_scene(rho, 32, 32)
    g = gpu_ctx.scene(sc)
    f = gpu_ctx.film(32, 32, fp64=True)
    p = S.render_params(32, 32, (8, 8), max_depth=depth, sample_depth=3, rr_depth=7)
    for k in range(16):
        g.render_pass(f, p, k)
    ratio = _furnace_ratio(f.read_f64())
    assert abs(ratio - rho) < 0.003 * rho, ratio


def test_furnace_depth_limit_zero_is_black(gpu_ctx):
    sc = S.furnace_scene(0.5, 32, 32)
    g = gpu_ctx.scene(sc)
    f = gpu_ctx.film(32, 32, fp64=True)
    g.render_pass(f, S.render_params(32, 32, (2, 2), max_depth=0, sample_depth=3, rr_depth=7), 0)
    film = f.read_f64()
    assert _furnace_ratio(film) == 0.0
    w = film[..., 0]
    bg = film[..., 2] / np.where(w > 0, w, 1)
    assert bg[0, 0] > 0


def _pass_estimates(films):
    """per-pass pixel estimates (X, Y, Z) / w of a list of per-pass films"""
    return np.stack([f[..., 1:] / np.where(f[..., :1] > 0, f[..., :1], 1) for f in films])


def test_4096spp_converges_to_the_16k_oracle_render(gpu_ctx):
    """GPU: 32 passes of 128 spp (4096 spp, FP64 film).  Oracle: 32 passes of
    512 spp (16384 spp) with another seed, so the two share no random
    numbers.  Per pixel and channel, z = (mean_gpu - mean_ref) /
    sqrt(var_gpu + var_ref), the variances of the means estimated from the
    spread of the pass estimates (31 degrees of freedom each).

    * per-pixel means agree within 3 sigma: at most 2% of the values have
      |z| > 3 (0.5% expected for 31 degrees of freedom), and the mean of z^2
      is within [0.8, 1.35] (1.07 expected);
    * the image RMSE beyond noise is within 1%: the measured squared error
      minus the expected noise (the mean of var_gpu + var_ref), square-rooted
      and divided by the reference's mean, is at most 1%.  The raw relative
      RMSE (noise included) is printed next to it.
    """
    n_pass = 32
    sc = S.cornell_room(24, 24)
    g = gpu_ctx.scene(sc)
    f = gpu_ctx.film(24, 24, fp64=True)
    p = S.cornell_params(24, 24)  # depth 5, Russian roulette after bounce 3
    p2 = S.render_params(24, 24, (16, 8), max_depth=p.max_depth, sample_depth=p.sample_depth,
                         rr_depth=p.rr_depth, seed=5)  # 128 spp per pass
    prev = np.zeros((24, 24, 4), np.float64)
    gpu_films = []
    for k in range(n_pass):
        g.render_pass(f, p2, k)
        cur = f.read_f64()
        gpu_films.append(cur - prev)
        prev = cur
    o = OracleScene(sc)
    po = S.render_params(24, 24, (32, 16), max_depth=p.max_depth, sample_depth=p.sample_depth,
                         rr_depth=p.rr_depth, seed=99)  # 512 spp per pass
    ref_films = [o.render_pass(po, k)[0].astype(np.float64) for k in range(n_pass)]
    eg, er = _pass_estimates(gpu_films), _pass_estimates(ref_films)
    mg, mr = eg.mean(0), er.mean(0)
    vg, vr = eg.var(0, ddof=1) / n_pass, er.var(0, ddof=1) / n_pass
    z = (mg - mr) / np.sqrt(vg + vr)
    frac3 = float(np.mean(np.abs(z) > 3))
    z2 = float(np.mean(z ** 2))
    mse = float(np.mean((mg - mr) ** 2))
    noise = float(np.mean(vg + vr))
    scale = float(np.mean(mr))
    raw = np.sqrt(mse) / scale
    excess = np.sqrt(max(0.0, mse - noise)) / scale
    print(f"4096-spp GPU vs 16384-spp oracle: relative RMSE {raw:.4%} (noise floor "
          f"{np.sqrt(noise) / scale:.4%}, beyond noise {excess:.4%}); |z|>3: {frac3:.3%}; "
          f"mean z^2 {z2:.3f}")
    assert frac3 <= 0.02, frac3
    assert 0.8 <= z2 <= 1.35, z2
    assert excess <= 0.01, excess
