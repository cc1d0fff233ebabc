"""CPU tests of the C-ABI library: it builds for sm_103a, loads, and exports
every function include/gpucpm.h declares.  No compute call is made."""
import ctypes
import pathlib
import re

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "gpucpm.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cpm_\w+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("cpm_create", "cpm_destroy", "cpm_push", "cpm_pull", "cpm_run",
                     "cpm_synchronize", "cpm_add_cell", "cpm_set_adhesion",
                     "cpm_set_area", "cpm_set_perimeter", "cpm_get_centroids",
                     "cpm_host_lattice", "cpm_last_error", "cpm_create_batch"):
        assert required in names


def test_library_exports_every_declared_symbol(engine_lib):
    missing = [n for n in declared_functions() if not hasattr(engine_lib, n)]
    assert not missing, missing


def test_create_failure_reports_message_without_gpu(engine_lib):
    import torch
    if torch.cuda.is_available():
        return  # covered by the GPU tests
    h = ctypes.c_void_p()
    rc = engine_lib.cpm_create(64, 2, 10, 10.0, 0, ctypes.byref(h))
    assert rc != 0 and not h.value
    assert engine_lib.cpm_last_error(None)


def test_invalid_arguments_rejected_before_touching_cuda(engine_lib):
    h = ctypes.c_void_p()
    assert engine_lib.cpm_create(64, 4, 10, 10.0, 0, ctypes.byref(h)) == 1
    assert b"dimensionality" in engine_lib.cpm_last_error(None)
    assert engine_lib.cpm_create(64, 2, 10, 10.0, 4, ctypes.byref(h)) == 6  # unknown flag
    assert engine_lib.cpm_create(2, 2, 10, 10.0, 0, ctypes.byref(h)) == 1


def test_static_sweep_refuses_handle_only_terms_before_touching_cuda(engine_lib):
    """cpm_sweep_static models adhesion, area, perimeter, stickiness and fixed
    types; a record with a chemotaxis, act or persistence lambda is refused
    (CPM_ERR_UNSUPPORTED) before any CUDA call, and bad sizes are refused
    with CPM_ERR_INVALID."""
    import sys
    sys.path.insert(0, str(ROOT / "gpu-cpm_gb300"))
    from gpucpm import StaticParams
    f = engine_lib.cpm_sweep_static
    f.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p] * 4 + [
        ctypes.c_int, ctypes.POINTER(StaticParams), ctypes.c_uint64, ctypes.c_uint32,
        ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    buf = (ctypes.c_uint32 * 64)()  # never dereferenced: the calls fail first
    ptr = ctypes.addressof(buf)
    for field in ("chemotaxis", "act_lambda", "persistence_lambda"):
        p = StaticParams()
        getattr(p, field)[1] = 1.0
        rc = f(2, 8, 8, 1, 4, ptr, ptr, ptr, ptr, 0, ctypes.byref(p), 0, 0, 0, 1, None, None)
        assert rc == 6, field  # CPM_ERR_UNSUPPORTED
        assert b"handle engine" in engine_lib.cpm_last_error(None)
    p = StaticParams()
    assert f(2, 2, 8, 1, 4, ptr, ptr, ptr, ptr, 0, ctypes.byref(p), 0, 0, 0, 1, None,
             None) == 1  # a side below 3
    # non-finite energies are refused as the handle setters refuse them
    for field, idx in (("temperature", None), ("lambda_area", 1), ("lambda_perimeter", 2),
                       ("J", 5), ("stickiness", 7)):
        for bad in (float("nan"), float("inf")):
            p = StaticParams()
            p.temperature = 5.0
            if idx is None:
                p.temperature = bad
            else:
                getattr(p, field)[idx] = bad
            rc = f(2, 8, 8, 1, 4, ptr, ptr, ptr, ptr, 0, ctypes.byref(p), 0, 0, 0, 1, None,
                   None)
            assert rc == 1, (field, bad)  # CPM_ERR_INVALID
            assert b"finite" in engine_lib.cpm_last_error(None)


def test_c_example_compiles_and_links(engine_lib, tmp_path):
    """tests/capi/example2d.c, a C caller of include/gpucpm.h only, builds
    with the system C compiler and links against the library (it runs in
    tests/test_gpu_api.py)."""
    import shutil
    import subprocess
    cc = shutil.which("cc") or shutil.which("gcc")
    if cc is None:
        return
    lib_dir = ROOT / "gpu-cpm_gb300"
    out = tmp_path / "example2d"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                        str(ROOT / "tests" / "capi" / "example2d.c"), "-L", str(lib_dir),
                        "-lgpucpm_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert out.exists()
