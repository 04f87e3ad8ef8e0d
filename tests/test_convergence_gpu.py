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
* Convergence: a 4096-spp GPU render of the 256 x 256 Cornell room
  (FP64-compensated film) against the oracle's 16384-spp render of the same
  scene into float64 films, with independent random streams (the committed
  fixture tests/golden/cornell256_oracle_16k.npz, made by
  make_cornell_reference.py).  The linear relative RMSE, noise included, is
  within 1% (measured 0.82%, of which 0.78% is the two renders' Monte Carlo
  noise); per-pixel means agree within 3 sigma; the RMSE beyond the noise is
  within 1%; and the output image (gamma 2.2, clamped, 8 bit) is within 1%
  RMSE of the reference's.
* The large-mesh geometry: the full 8.4M-triangle heightfield and 4096
  spheres at a small image size, GPU against oracle with independent random
  streams, per-pixel means within 3 sigma.
"""
from pathlib import Path

import numpy as np
import pytest

from bling_gb300 import image
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


GOLDEN = Path(__file__).resolve().parent / "golden"


def test_4096spp_converges_to_the_16k_fp64_oracle_render(gpu_ctx):
    """GPU: 32 passes of 128 spp (4096 spp, FP64 film), seed 5.  Reference:
    the oracle's 32 passes of 512 spp (16384 spp, float64 films), seed 99,
    as per-pixel means and variances of the mean.  Per pixel and channel,
    z = (mean_gpu - mean_ref) / sqrt(var_gpu + var_ref).

    * the linear relative RMSE (over pixels and X, Y, Z, divided by the
      reference's mean), noise included, is at most 1%;
    * at most 2% of the values have |z| > 3 (0.5% expected for 31 degrees
      of freedom) and the mean of z^2 is within [0.8, 1.35] (1.07 expected);
      values without variance on either side (the light seen directly) are
      equal instead;
    * linear relative RMSE beyond noise (the squared error minus the
      expected noise, square-rooted, over the reference's mean) <= 1%;
    * display RMSE: both images resolved to RGB (xyzToRgb), gamma 2.2,
      clamped and quantised to 8 bits as the reference writes them; the RMSE
      over pixels and channels, in units of full scale, <= 1%.
    """
    ref = np.load(GOLDEN / "cornell256_oracle_16k.npz")
    mr, vr = ref["mean"].astype(np.float64), ref["var_mean"].astype(np.float64)
    assert int(ref["spp"]) == 16384
    n_pass, size = 32, mr.shape[0]
    sc = S.cornell_room(size, size)
    g = gpu_ctx.scene(sc)
    f = gpu_ctx.film(size, size, fp64=True)
    base = S.cornell_params(size, size)  # depth 5, Russian roulette after bounce 3
    p = S.render_params(size, size, (16, 8), max_depth=base.max_depth,
                        sample_depth=base.sample_depth, rr_depth=base.rr_depth,
                        filter_kind=base.filter_kind, seed=5)  # 128 spp per pass
    prev = np.zeros((size, size, 4), np.float64)
    gpu_films = []
    for k in range(n_pass):
        g.render_pass(f, p, k)
        cur = f.read_f64()
        gpu_films.append(cur - prev)
        prev = cur
    eg = _pass_estimates(gpu_films)
    mg, vg = eg.mean(0), eg.var(0, ddof=1) / n_pass
    var = vg + vr
    flat = var == 0
    assert np.allclose(mg[flat], mr[flat], rtol=1e-6, atol=0)
    z = (mg - mr)[~flat] / np.sqrt(var[~flat])
    frac3 = float(np.mean(np.abs(z) > 3))
    z2 = float(np.mean(z ** 2))
    mse = float(np.mean((mg - mr) ** 2))
    noise = float(np.mean(vg + vr))
    scale = float(np.mean(mr))
    raw = np.sqrt(mse) / scale
    excess = np.sqrt(max(0.0, mse - noise)) / scale
    # the output images: the full film's own estimate (all 4096 spp)
    full = prev[..., 1:] / prev[..., :1]
    rgb_g = image.to_rgb8(_xyz_to_rgb(full)).astype(np.float64)
    rgb_r = image.to_rgb8(_xyz_to_rgb(mr)).astype(np.float64)
    disp = float(np.sqrt(np.mean((rgb_g - rgb_r) ** 2)) / 255.0)
    print(f"4096-spp GPU vs 16384-spp FP64 oracle, {size}x{size}: linear relative RMSE "
          f"{raw:.4%} (noise floor {np.sqrt(noise) / scale:.4%}, beyond noise {excess:.4%}); "
          f"display RMSE {disp:.4%} of full scale; |z|>3: {frac3:.3%}; mean z^2 {z2:.3f}")
    assert raw <= 0.01, raw
    assert frac3 <= 0.02, frac3
    assert 0.8 <= z2 <= 1.35, z2
    assert excess <= 0.01, excess
    assert disp <= 0.01, disp


def _xyz_to_rgb(xyz):
    """xyzToRgb (Spectrum.hs:162-168) in float32, per pixel"""
    x, y, z = (xyz[..., i].astype(np.float32) for i in range(3))
    F = np.float32
    r = F(3.240479) * x - F(1.537150) * y - F(0.498535) * z
    g = F(-0.969256) * x + F(1.875991) * y + F(0.041556) * z
    b = F(0.055648) * x - F(0.204043) * y + F(1.057311) * z
    return np.stack([r, g, b], -1)


def test_heightfield_full_geometry_independent_streams(gpu_ctx):
    """the full large-mesh geometry (8.4M triangles, 4096 spheres, sky and
    sun) at 40 x 24: 24 passes of 4 spp on each side with independent seeds;
    per-pixel luminance means within 3 sigma for all but 2% of pixels and no
    bias in the mean z"""
    w, h, passes = 40, 24, 24
    sc = S.heightfield_scene(ns=2048, n_spheres=4096, width=w, height=h, env_size=(256, 128))
    g = gpu_ctx.scene(sc)
    o = OracleScene(sc)
    film = gpu_ctx.film(w, h)
    yg, yo = [], []
    for k in range(passes):
        film.clear()
        g.render_pass(film, S.heightfield_params(w, h, spp_side=2, seed=21), k)
        fg = film.read()
        yg.append(fg[..., 2] / fg[..., 0])
        fo, _ = o.render_pass(S.heightfield_params(w, h, spp_side=2, seed=4242), k)
        yo.append(fo[..., 2] / fo[..., 0])
    yg, yo = np.asarray(yg, np.float64), np.asarray(yo, np.float64)
    se = np.sqrt(yg.var(0, ddof=1) / passes + yo.var(0, ddof=1) / passes)
    ok = se > 0
    z = (yg.mean(0) - yo.mean(0))[ok] / se[ok]
    # pixels with zero variance on both sides (pure sky) must agree exactly
    assert np.allclose(yg.mean(0)[~ok], yo.mean(0)[~ok], rtol=1e-5)
    print(f"heightfield 8.4M tris, 40x24, 96 spp each side: |z|>3 {np.mean(np.abs(z) > 3):.3%}, "
          f"mean z {np.mean(z):.3f}, mean z^2 {np.mean(z ** 2):.3f}")
    assert np.mean(np.abs(z) > 3) <= 0.02
    assert abs(np.mean(z)) < 0.15
