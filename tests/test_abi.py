"""CPU: the C-ABI library loads and exports every entry point include/dogm_gb300.h declares;
layouts match the reference's structs; host-side argument checks run without a GPU.
Nothing here launches a kernel."""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "dogm_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dogm_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_and_library_exports_everything(dogm):
    names = declared_functions()
    assert len(names) >= 35
    lib = dogm.load()
    for n in names:
        assert hasattr(lib, n), "libdogm_gb300.so does not export %s" % n
    assert sorted(dogm.ABI_SYMBOLS) == names


def test_exports_with_nm(dogm):
    nm = shutil.which("nm")
    if not nm:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--defined-only", dogm.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (dogm_\w+)", out))
    assert set(declared_functions()) <= exported


def test_layouts(dogm):
    assert dogm.GRID_CELL_DTYPE.itemsize == 64
    assert dogm.MEAS_DTYPE.itemsize == 16
    assert ctypes.sizeof(dogm.Params) == 44
    assert dogm.load().dogm_abi_version() == 1


def test_host_argument_checks_without_gpu(dogm):
    lib = dogm.load()
    h = ctypes.c_void_p()
    bad = dogm.make_params(size=0.0)
    assert lib.dogm_create(ctypes.byref(bad), None, ctypes.byref(h)) == 1
    huge = dogm.make_params(size=1000.0, resolution=0.1)  # 10000^2 cells > 2^22
    assert lib.dogm_create(ctypes.byref(huge), None, ctypes.byref(h)) == 6
    assert b"2048" in lib.dogm_last_error()
    assert lib.dogm_create(None, None, ctypes.byref(h)) == 1
    assert lib.dogm_status_string(4) == b"device wait timed out"
    opt = dogm.Options()
    assert lib.dogm_default_options(ctypes.byref(opt)) == 0
    assert opt.seed == 123456 and opt.sync_each_update == 1
    # state bytes for the large workload: particles + cells, well under the HBM budget
    p = dogm.make_params(size=120.0, resolution=0.1, particle_count=2_000_000, new_born_particle_count=200_000)
    b = dogm.state_bytes(p)
    assert 150e6 < b < 600e6


def test_cpp_dropin_compiles_and_links(dogm, tmp_path):
    """The header-only dogm::DOGM drop-in compiles against the C ABI and links."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    src = os.path.join(REPO, "tests", "cpp", "dogm_spec.cpp")
    exe = str(tmp_path / "dogm_spec")
    lib_dir = os.path.dirname(dogm.LIB_PATH)
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"), src, "-o", exe,
                        "-L" + lib_dir, "-ldogm_gb300", "-Wl,-rpath," + lib_dir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_server_argument_checks_without_gpu(dogm):
    """Serving-loop configuration and stream checks that return before any device call."""
    lib = dogm.load()
    cfg = dogm.ServerConfig()
    assert lib.dogm_server_default_config(ctypes.byref(cfg)) == 0
    assert cfg.hbm_budget_bytes == 150 * 10**9 and cfg.mode == dogm.SERVE_BATCHED
    assert cfg.max_batch == 64 and cfg.max_inflight == 2 and cfg.queue_admission == 1
    s = ctypes.c_void_p()
    for field, value in (("max_batch", 0), ("max_batch", 257), ("max_inflight", 5), ("mode", 7),
                         ("hbm_budget_bytes", 0)):
        bad = dogm.ServerConfig()
        lib.dogm_server_default_config(ctypes.byref(bad))
        setattr(bad, field, value)
        assert lib.dogm_server_create(ctypes.byref(bad), ctypes.byref(s)) == 1, field
    assert lib.dogm_server_create(None, ctypes.byref(s)) == 1
    sid = ctypes.c_int(0)
    assert lib.dogm_server_open_stream(None, None, None, ctypes.byref(sid)) == 1
    assert lib.dogm_server_submit(None, 0, None, 0, 0.0, 0.0, 0.0, 0.1, None, 0) == 1
    assert lib.dogm_server_stream_state(None, 0) == -1
    n = ctypes.c_int(5)
    assert lib.dogm_server_poll(None, None, 0, 0, ctypes.byref(n)) == 1
    t0 = lib.dogm_server_now_ns()
    assert lib.dogm_server_now_ns() >= t0 > 0
    assert ctypes.sizeof(dogm.ServerResult) == 48 and ctypes.sizeof(dogm.ServerStats) == 56
