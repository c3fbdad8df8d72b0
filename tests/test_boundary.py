"""The C-ABI library loads and exports every entry point include/kpt.h
declares; the host-side API behaves without a GPU."""

import ctypes as C
import os
import re

import pytest

from kittlespt_gb300 import _lib as K

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "kpt.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kpt_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(K.LIB_PATH):
        from kittlespt_gb300 import build
        build.build()
    return K.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    assert set(declared()) <= set(K.SIGNATURES)


def test_defaults_match_reference_values(lib):
    e = K.Environment()
    lib.kpt_environment_default(C.byref(e))
    assert abs(e.sun_phi - 4.18879) < 1e-6 and abs(e.rayleigh_height - 7994.0) < 1e-6
    assert [round(x * 1e6, 3) for x in e.rayleigh] == [3.8, 13.5, 33.1]
    s = K.Settings()
    lib.kpt_settings_default(C.byref(s))
    assert s.max_depth == 3 and abs(s.bloom_internal_blend - 0.65) < 1e-7
    x = K.Exposure()
    lib.kpt_exposure_default(C.byref(x))
    assert x.aperture == 11.0 and x.white_ev == 6.5 and x.black_ev == -10.0


def test_errors_without_context(lib):
    assert lib.kpt_resize(None, 4, 4) == -1
    assert lib.kpt_last_error()
    assert lib.kpt_render_frame(None, 1, 16.0) == -1
    assert lib.kpt_get_level_counts(None, 4, None, None) == -1
    assert lib.kpt_destroy(None) == 0
