"""The C ABI library builds for sm_103a, loads, and exports every entry point
include/flowlab_gb300.h declares. No GPU needed (nothing is computed)."""
import ctypes
import os
import re

import pytest

from flowlab_gb300 import build, native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "flowlab_gb300.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fl_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_the_header():
    bound = {n for n, _, _ in native.SIGNATURES}
    assert set(declared()) == bound


def test_abi_version_and_defaults(lib):
    assert lib.fl_abi_version() == native.ABI_VERSION == 3
    p = native.default_params()
    # simulation.ts:223-234 and pressureMultigrid.ts:47-67
    assert p.cfl_target == 2.0 and abs(p.dt_max - 1 / 30) < 1e-15 and p.tol == 5e-3
    assert (p.mg_pre, p.mg_post, p.mg_coarse_sweeps, p.mg_coarsest, p.mg_max_cycles) == (2, 2, 8, 4, 3)
    assert p.residual_every == 1  # simulation.ts:233
    assert ctypes.sizeof(native.Params) == 160
    assert p.mg_tail_side == 0  # the engine's default first tail level (32)
    assert native.Params.mg_tail_side.offset == 140 and native.Params.residual_every.offset == 144
    assert native.Params.reserved.offset == 148
    assert ctypes.sizeof(native.Stats) == 96 and native.Stats.initial_rel_residual.offset == 88


def test_python_defaults_equal_the_library_defaults(lib):
    # default_params() builds fl_params without the library (the CPU
    # reference arm of the bench must not load it); the library's own
    # fl_default_params (host code only) is the authority
    ours = native.default_params()
    theirs = native.Params()
    lib.fl_default_params(ctypes.byref(theirs))
    assert bytes(ours) == bytes(theirs)


def test_create_fails_loudly_without_a_device(lib):
    h = ctypes.c_void_p()
    st = lib.fl_create(8, 8, 0.125, 1, None, 0, ctypes.byref(h))
    if st == native.FL_OK:  # a GPU is present: nothing to check here
        lib.fl_destroy(h)
        pytest.skip("a CUDA device is present")
    assert st == native.FL_EDEVICE
    assert b"CUDA" in lib.fl_last_error(None)


def test_null_engine_is_rejected(lib):
    assert lib.fl_synchronize(None) == native.FL_EINVAL


def test_profile_phases_match_the_header():
    src = open(HEADER).read()
    n = int(re.search(r"#define FL_PHASES (\d+)", src).group(1))
    enum = re.search(r"enum fl_phase \{(.*?)\};", src, flags=re.S).group(1)
    names = re.findall(r"FL_PH_([A-Z0-9_]+) = (\d+)", enum)
    assert [int(k) for _, k in names] == list(range(n))
    assert [nm.lower() for nm, _ in names] == native.PHASES
    assert ctypes.sizeof(native.Profile) == n * 24


def test_plain_c_caller_links_and_fails_loudly_without_a_device(lib, tmp_path):
    """tests/c_abi_step.c binds the ABI from plain C (gcc, the header and the
    shared library, nothing else). Without a GPU it must stop at fl_create
    with FL_EDEVICE and the CUDA message; with one, it takes a step."""
    import shutil
    import subprocess

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not found")
    here = os.path.dirname(os.path.abspath(__file__))
    libdir = os.path.dirname(build.LIB)
    exe = str(tmp_path / "c_abi_step")
    subprocess.run([cc, "-std=c11", "-O1", "-Wall", "-Werror", "-I" + os.path.dirname(HEADER),
                    os.path.join(here, "c_abi_step.c"), "-o", exe, "-L" + libdir, "-lflowlab_gb300",
                    "-Wl,-rpath," + libdir, "-lm"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    if r.returncode == 0:
        assert "stepped:" in r.stdout
    else:
        assert r.returncode == 2, r.stdout + r.stderr
        assert "no device" in r.stdout and "CUDA" in r.stdout
