"""Host-side checks of liblagrbf.so that need no GPU: the library loads, exports every symbol that
include/lagrbf.h declares, registers like the reference's ctypes layer, keeps the options store the
way PETSc's options database behaves for the keys lagrbf_create() reads, and fails cleanly (NULL /
error code + message, no abort) where a GPU would be needed."""
import ctypes
import os
import re

import numpy as np
import pytest

import lagrbf_gb300 as L
from lagrbf_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lagrbf.h")

REFERENCE_SYMBOLS = [  # register_cfunc.py:50-191
    "lagrbf_create", "lagrbf_destroy", "lagrbf_fill_swarm", "lagrbf_interpolation", "lagrbf_output",
    "lagrbf_reset_coefficients", "lagrbf_avect_analytical", "lagrbf_advect_interpolate",
    "lagrbf_advection_function", "lagrbf_advection_function_batch", "lagrbf_interpolate_driver",
]


def header_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"LAGRBF_EXPORT[^;{]*?\b(lagrbf_\w+)\s*\(", text, flags=re.S)))


@pytest.fixture(scope="module")
def lib():
    return _lib.load_shared_lib()


def test_header_declares_reference_surface():
    syms = header_symbols()
    for s in REFERENCE_SYMBOLS:
        assert s in syms
    assert len(syms) >= 29


def test_library_exports_every_header_symbol(lib):
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_ctypes_registration_matches_reference_keys():
    cf = L.load_cfuncs()
    for s in REFERENCE_SYMBOLS:
        key = "lagrbf_avect_interpolate" if s == "lagrbf_advect_interpolate" else s
        assert key in cf, key


def test_options_store_roundtrip(lib):
    lib.lagrbf_options_clear()
    assert lib.lagrbf_options_set_value(b"-pu_mesh_n", b"8,8,8") == 0
    assert lib.lagrbf_options_set_value(b"kernel_type", b"2") == 0
    buf = ctypes.create_string_buffer(64)
    assert lib.lagrbf_options_get_value(b"pu_mesh_n", buf, 64) == 1 and buf.value == b"8,8,8"
    assert lib.lagrbf_options_get_value(b"--kernel_type", buf, 64) == 1 and buf.value == b"2"
    assert lib.lagrbf_options_set_value(b"kernel_type", b"6") == 0  # overwrite
    assert lib.lagrbf_options_get_value(b"kernel_type", buf, 64) == 1 and buf.value == b"6"
    assert lib.lagrbf_options_get_value(b"not_set", buf, 64) == 0
    lib.lagrbf_options_clear()
    assert lib.lagrbf_options_get_value(b"pu_mesh_n", buf, 64) == 0


def test_options_file_petsc_syntax(lib, tmp_path):
    p = tmp_path / "opts"
    p.write_text("# comment line\n-pu_mesh_dim 2   -pu_mesh_n 5,7 # trailing comment\n"
                 "-advection\n-dt -1e-3\n-pu_mesh_O -0.5,-0.25 -log_view\n")
    lib.lagrbf_options_clear()
    assert lib.lagrbf_options_insert_file(str(p).encode()) == 0
    buf = ctypes.create_string_buffer(64)
    expect = {b"pu_mesh_dim": b"2", b"pu_mesh_n": b"5,7", b"advection": b"true", b"dt": b"-1e-3",
              b"pu_mesh_O": b"-0.5,-0.25", b"log_view": b"true"}
    for k, v in expect.items():
        assert lib.lagrbf_options_get_value(k, buf, 64) == 1, k
        assert buf.value == v, (k, buf.value)
    assert lib.lagrbf_options_insert_file(b"/nonexistent/opts") == 62
    lib.lagrbf_options_clear()


def test_python_options_mapping():
    """LagRBFCtx keyword defaults (context.py:113-201) land in the store as the reference's keys."""
    o = L.Options({})
    o["pu_mesh_n"] = np.array([4, 5, 6], dtype=np.int32)
    o["pu_mesh_O"] = np.zeros(3)
    o["advection"] = True
    o.push()
    lib = _lib.load_shared_lib()
    buf = ctypes.create_string_buffer(128)
    assert lib.lagrbf_options_get_value(b"pu_mesh_n", buf, 128) == 1 and buf.value == b"4,5,6"
    assert lib.lagrbf_options_get_value(b"advection", buf, 128) == 1 and buf.value in (b"true", b"1")
    lib.lagrbf_options_clear()


def test_create_without_gpu_fails_cleanly(lib):
    lib.lagrbf_create.restype = ctypes.c_void_p
    lib.lagrbf_gpu_last_error.restype = ctypes.c_char_p
    lib.lagrbf_options_clear()
    lib.lagrbf_options_set_value(b"pu_mesh_dim", b"2")
    lib.lagrbf_options_set_value(b"pu_mesh_n", b"4,4")
    ctx = lib.lagrbf_create()
    lib.lagrbf_options_clear()
    if ctx:
        lib.lagrbf_destroy(ctypes.c_void_p(ctx))
        pytest.skip("a GPU is present")
    assert b"CUDA" in lib.lagrbf_gpu_last_error()
    lib.lagrbf_gpu_fp32_peak_tflops.restype = ctypes.c_double
    assert lib.lagrbf_gpu_fp32_peak_tflops() < 0
    lib.lagrbf_gpu_fp64_peak_tflops.restype = ctypes.c_double
    assert lib.lagrbf_gpu_fp64_peak_tflops() < 0


def test_create_rejects_bad_options(lib):
    """Option validation happens before any device work (errors as in PUSetFromOptions)."""
    lib.lagrbf_create.restype = ctypes.c_void_p
    lib.lagrbf_gpu_last_error.restype = ctypes.c_char_p
    for opts, msg in (({}, b"pu_mesh_dim"), ({b"pu_mesh_dim": b"4", b"pu_mesh_n": b"4,4"}, b"2 or 3"),
                      ({b"pu_mesh_dim": b"2", b"pu_mesh_n": b"4"}, b"expected 2")):
        lib.lagrbf_options_clear()
        for k, v in opts.items():
            lib.lagrbf_options_set_value(k, v)
        assert not lib.lagrbf_create()
        assert msg in lib.lagrbf_gpu_last_error(), lib.lagrbf_gpu_last_error()
    lib.lagrbf_options_clear()


def test_null_context_is_an_error_not_a_crash(lib):
    assert lib.lagrbf_interpolation(None) == 85
    assert lib.lagrbf_reset_coefficients(None) == 85
    lib.lagrbf_advect_interpolate.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
    assert lib.lagrbf_advect_interpolate(None, 0.0, 1.0) == 85
    lib.lagrbf_destroy(None)


def test_python_surface_mirrors_lagrbfpy():
    """Every class of lagrbfpy's context, interpolation and advection modules exists in the mirror
    with every method it defines (inherited ones count); parsed from the LagRBF source tree, skipped
    without it."""
    import ast
    if not os.environ.get("LAGRBF_REFERENCE"):
        pytest.skip("LAGRBF_REFERENCE (a LagRBF checkout) not set")
    ref = os.path.join(os.environ["LAGRBF_REFERENCE"], "python_api", "lagrbfpy")
    if not os.path.isdir(ref):
        pytest.skip("LagRBF source tree not present")
    deprecated = {"_LagRBFCtx__deprecated_set_advection_function"}  # name-mangled, deprecated in lagrbfpy
    for rf in ("interface/context.py", "interpolation.py", "advection.py"):
        with open(os.path.join(ref, rf)) as f:
            tree = ast.parse(f.read())
        for cls in [n for n in tree.body if isinstance(n, ast.ClassDef)]:
            assert hasattr(L, cls.name), cls.name
            ours = getattr(L, cls.name)
            for fn in [n for n in cls.body if isinstance(n, ast.FunctionDef)]:
                name = fn.name
                if name.startswith("__") and not name.endswith("__"):
                    name = "_%s%s" % (cls.name, name)
                if name in deprecated:
                    continue
                assert hasattr(ours, name), (cls.name, fn.name)


def test_record_loop_probe_compiles(tmp_path):
    """The compute-only probe of the evaluation's record loop (lagrbf_gb300/probe_eval.py) builds for
    sm_103a (it runs only on a GPU)."""
    import subprocess
    from lagrbf_gb300 import build
    try:
        cuda = build._cuda_home()
    except RuntimeError:
        pytest.skip("nvcc not available")
    src = os.path.join(os.path.dirname(build.__file__), "csrc", "probe_record_loop.cu")
    out = tmp_path / "probe.o"
    r = subprocess.run([os.path.join(cuda, "bin", "nvcc"), "-std=c++17", *build.ARCH, "-c", src, "-o", str(out)],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    assert out.exists()
