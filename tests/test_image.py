"""Image output (bling_gb300/image.py): getPixel/xyzToRgb resolve, the
8-bit mapping of rgbPixels (gamma 2.2, clamp, round half to even), and PNG
and Radiance RGBE files read back."""
import numpy as np
import pytest

from bling_gb300 import image as I
from bling_gb300 import scene as S
from bling_gb300.spectrum import xyz_to_rgb
from oracle.oracle import OracleScene, resolve as oracle_resolve

F = np.float32


def test_resolve_matches_the_oracle_and_handles_empty_pixels():
    sc = S.cornell_room(16, 16)
    film, _ = OracleScene(sc).render_pass(S.cornell_params(16, 16, spp_side=2), 0)
    assert np.array_equal(I.resolve(film), oracle_resolve(film))
    film[0, 0] = 0  # no samples: getPixel gives xyzToRgb (0, 0, 0)
    assert np.array_equal(I.resolve(film)[0, 0], np.zeros(3, F))


def test_resolve_divides_by_the_weight_first():
    film = np.array([[[2.0, 1.0, 0.5, 0.25]]], F)
    r, g, b = xyz_to_rgb(F(1.0) * F(0.5), F(0.5) * F(0.5), F(0.25) * F(0.5))
    assert np.array_equal(I.resolve(film)[0, 0], np.array([r, g, b], F))


def test_rgb8_gamma_clamp_and_rounding():
    v = np.array([[[0.0, 1.0, 2.0], [-1.0, np.nan, 0.5]]], F)
    out = I.to_rgb8(v)
    assert out[0, 0].tolist() == [0, 255, 255]
    assert out[0, 1, 0] == 0 and out[0, 1, 1] == 0
    assert out[0, 1, 2] == int(np.rint(F(np.power(F(0.5), F(1) / F(2.2))) * F(255)))
    # round half to even at an exact .5: 0.5 * 255 = 127.5 -> 128, 1.5 -> 2
    assert np.rint(np.float32(127.5)) == 128 and np.rint(np.float32(2.5)) == 2


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (13, 7, 3)).astype(np.uint8)
    p = tmp_path / "x.png"
    I.write_png(p, img)
    assert p.read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"
    assert np.array_equal(I.read_png(p), img)


def test_rgbe_round_trip_within_the_mantissa_step(tmp_path):
    rng = np.random.default_rng(2)
    rgb = (rng.uniform(0, 1, (9, 11, 3)) * rng.choice([1e-3, 1.0, 40.0], (9, 11, 1))).astype(F)
    rgb[0, 0] = 0
    p = tmp_path / "x.hdr"
    I.write_rgbe(p, rgb)
    assert p.read_bytes().startswith(b"#?RADIANCE\n")
    back = I.read_rgbe(p)
    assert back.shape == rgb.shape and np.all(back[0, 0] == 0)
    m = rgb.max(-1, keepdims=True)
    # one mantissa step is 2^(e-8) <= m/128: the midpoint decode is within half of it
    assert np.all(np.abs(back - rgb) <= m / 256 + 1e-30)


def test_png_rejects_bad_shapes(tmp_path):
    with pytest.raises(ValueError):
        I.write_png(tmp_path / "y.png", np.zeros((4, 4), np.uint8))
