"""The C-ABI library builds, loads without a GPU, exports every symbol that
include/awe.h declares, and rejects bad descriptors with a status code."""
import ctypes as C
import os
import re

import pytest

import wavefield_imaging_gb300 as awe
from wavefield_imaging_gb300 import build as awe_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    awe_build.build()
    return awe.lib()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "awe.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(awe_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("awe_plan_create", "awe_set_model", "awe_set_geometry", "awe_forward", "awe_forward_device",
              "awe_plan_destroy"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_status_strings(lib):
    assert b"sm_103a" in lib.awe_version()
    assert lib.awe_status_string(1) == b"invalid argument"


@pytest.mark.parametrize("field,value", [("ndim", 4), ("nt", 0), ("fdorder", 3), ("scheme", 7)])
def test_bad_descriptor_is_rejected(lib, field, value):
    d = awe.make_desc(2, (10, 12), (5.0, 5.0), (0.0, 0.0), 10, 0.005, fdorder=4)
    setattr(d, field, value)
    h = C.c_void_p()
    st = lib.awe_plan_create(C.byref(d), 0, C.byref(h))
    assert st == 1 and not h.value
    assert lib.awe_last_error()


def test_spherical_cpu_scheme_unsupported(lib):
    d = awe.make_desc(2, (10, 12), (5.0, 5.0), (0.0, 0.0), 10, 0.005, coords=awe.SPHER, scheme=awe.SCHEME_CPU)
    h = C.c_void_p()
    assert lib.awe_plan_create(C.byref(d), 0, C.byref(h)) == 4


def test_null_arguments(lib):
    assert lib.awe_plan_create(None, 0, None) == 1
    assert lib.awe_set_model(None, None, None, None) == 1
    assert lib.awe_forward(None, None, 1, None, None) == 1
    assert lib.awe_plan_destroy(None) == 0
