"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares; host-only helpers agree with the oracle bit for bit."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from bling_gb300 import build as gbuild
from bling_gb300.spectrum import rgb_to_spectrum
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def so():
    return C.CDLL(str(gbuild.build()))


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        src = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(bling_\w+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for required in ("bling_ctx_create", "bling_scene_create", "bling_trace_closest",
                     "bling_trace_any", "bling_render_pass", "bling_film_read", "bling_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(so):
    missing = [n for n in declared_functions() if not hasattr(so, n)]
    assert not missing, missing


def test_abi_version(so):
    from bling_gb300 import abi
    so.bling_abi_version.restype = C.c_int
    assert so.bling_abi_version() == abi.ABI_VERSION == 5
    hdr = (ROOT / "include" / "bling_gpu.h").read_text()
    assert f"#define BLING_ABI_VERSION {abi.ABI_VERSION}" in hdr
    # bling_render_params: 8 int32, 4 float, uint64 seed, int32 sampler_kind, int32 reserved
    assert C.sizeof(abi.RenderParams) == 64
    # bling_camera_desc: c2w, c2w_inv, r2c, r2c_inv, lens radius, focal distance, w2r,
    # pixel area, reserved
    assert C.sizeof(abi.CameraDesc) == 4 * (16 * 5 + 4)


def test_host_spectrum_helpers_match_oracle(so):
    so.bling_rgb_to_spectrum.argtypes = [C.c_int32, C.c_float, C.c_float, C.c_float,
                                         C.POINTER(C.c_float)]
    so.bling_spectrum_to_xyz.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float)]
    for rgb in [(0.75, 0.75, 0.75), (0.63, 0.065, 0.05), (0.14, 0.45, 0.09), (15, 15, 15)]:
        for illum in (0, 1):
            a = np.zeros(16, np.float32)
            so.bling_rgb_to_spectrum(illum, *map(float, rgb), O.fp(a))
            assert np.array_equal(a.view(np.uint32), rgb_to_spectrum(rgb, bool(illum)).view(np.uint32))
            x1, x2 = np.zeros(3, np.float32), np.zeros(3, np.float32)
            so.bling_spectrum_to_xyz(O.fp(a), O.fp(x1))
            O.lib().orc_spectrum_to_xyz(O.fp(a), O.fp(x2))
            assert np.array_equal(x1.view(np.uint32), x2.view(np.uint32))


def test_context_without_gpu_fails_cleanly(so):
    """No CPU fallback: without a usable device the context reports an error."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from bling_gb300.api import BlingUnavailable, Context
    with pytest.raises(BlingUnavailable):
        Context()
