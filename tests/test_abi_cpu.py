"""C-ABI library checks that need no GPU: it loads, exports every symbol the
public header declares, reads catalogs exactly like the reference, and fails
loudly (no CPU fallback) when no device is present."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import refformat as rf
import tpcf
import oracle

HEADER = os.path.join(rf.ROOT, "include", "tpcf.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:tpcf_status|const char\*|int32_t)\s+(tpcf_\w+)\s*\(", text, re.M)))


def test_header_symbols_match_binding_list():
    assert declared_symbols() == sorted(tpcf.ABI_SYMBOLS)


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(tpcf.LIB_PATH)
    for name in declared_symbols():
        assert hasattr(L, name), name
    assert L.tpcf_abi_version() == 3


def _has_gpu():
    ctx = ctypes.c_void_p()
    st = tpcf.lib().tpcf_create(ctypes.byref(ctx), 0)
    if st == 0:
        tpcf.lib().tpcf_destroy(ctx)
        return True
    return False


def test_no_device_fails_loudly():
    if _has_gpu():
        pytest.skip("a GPU is present")
    with pytest.raises(tpcf.EngineError) as e:
        tpcf.Engine(0)
    assert e.value.status == -3  # TPCF_ERR_NO_DEVICE


@pytest.mark.parametrize("name", ["h_blobs", "h_lattice", "c_blobs", "c_lattice", "c_pairs_d"])
def test_reader_matches_reference_fscanf(name):
    path = os.path.join(rf.GOLDEN, "ref", name + ".dat")
    fmt = 0 if name.startswith("h_") else 1
    got = tpcf.read_catalog(path, fmt)
    want = oracle.read_header(path) if fmt == 0 else oracle.read_7col(path)
    assert got.shape == want.shape
    assert got.tobytes() == want.tobytes()


def test_reader_scale_factor_matches_reference():
    path = os.path.join(rf.GOLDEN, "ref", "h_unif.dat")
    got = tpcf.read_catalog(path, 0, 3437.74677)
    want = oracle.read_header(path, 3437.74677)
    assert got.tobytes() == want.tobytes()


def test_reader_sandbox_catalog(tmp_path):
    p = rf.gunzip_to(os.path.join(rf.GOLDEN, "sandbox", "MICE_LRGs_10degx10deg.dat.gz"), str(tmp_path / "l.dat"))
    got = tpcf.read_catalog(p, 1)
    assert len(got) == 1316
    assert got.tobytes() == oracle.read_7col(p).tobytes()


def test_reader_row_limit(tmp_path):
    p = tmp_path / "big.dat"
    with open(p, "w") as f:
        f.write("1 0 0 0 1 2 3\n" * 1000001)
    with pytest.raises(tpcf.EngineError):
        tpcf.read_catalog(str(p), 1)


def test_hist_len():
    assert tpcf.hist_len(tpcf.make_spec(tpcf.THREE_SIDE, 0, [(16, 0, 40)])) == 4096
    assert tpcf.hist_len(tpcf.make_spec(tpcf.TRIANGLE, 1, [(8, 2, 10), (8, 1, 3), (16, 0, 1)])) == 1024
    assert tpcf.hist_len(tpcf.make_spec(tpcf.PAIR, 1, [(700, 0, 70)])) == 700


@pytest.mark.parametrize("prog,nargs", [("tpcf_3side", 2), ("tpcf_tp", 2), ("tpcf_2pcf", 1)])
def test_cli_too_few_arguments(prog, nargs):
    exe = os.path.join(tpcf.BIN_DIR, prog)
    r = subprocess.run([exe] + ["x"] * (nargs - 1), capture_output=True, text=True)
    assert r.returncode == 1
    assert "Must pass in at least" in r.stdout


def test_cli_without_gpu_fails_loudly(tmp_path):
    if _has_gpu():
        pytest.skip("a GPU is present")
    cat = os.path.join(rf.GOLDEN, "ref", "c_blobs.dat")
    r = subprocess.run([os.path.join(tpcf.BIN_DIR, "tpcf_tp"), cat, cat, cat, "-o", str(tmp_path / "o.dat")],
                       capture_output=True, text=True)
    assert r.returncode == 2
    assert "no CUDA device" in r.stderr
    assert not (tmp_path / "o.dat").exists()


def test_x86_acos_fixture_matches_this_host():
    """The committed x86-64 glibc acosf table equals an exhaustive scan of this
    machine's libm when this machine is x86-64 with glibc 2.39."""
    import platform
    libc = ctypes.CDLL("libc.so.6")
    libc.gnu_get_libc_version.restype = ctypes.c_char_p
    if platform.machine() != "x86_64" or libc.gnu_get_libc_version().decode() != "2.39":
        pytest.skip("fixture is for x86-64 glibc 2.39")
    L = tpcf.lib()
    n = ctypes.c_uint64()
    L.tpcf_debug_acos_exceptions(None, None, ctypes.c_uint64(0), ctypes.byref(n))
    keys = np.zeros(n.value, dtype=np.uint32)
    dirs = np.zeros(n.value, dtype=np.int8)
    L.tpcf_debug_acos_exceptions(keys.ctypes.data_as(ctypes.c_void_p), dirs.ctypes.data_as(ctypes.c_void_p),
                                 ctypes.c_uint64(n.value), ctypes.byref(n))
    fk, fu = rf.x86_acos_exceptions()
    assert np.array_equal(keys, fk)
    assert np.array_equal(dirs > 0, fu)
    assert np.all(np.abs(dirs) == 1)


def test_sum_voxels_tool_matches_reference_script(tmp_path):
    """tpcf_sum_voxels on the reference's own eight DDD_voxel2 chunk files
    against the restatement of examples/sum_voxels.py, byte for byte."""
    import glob
    import subprocess
    import refformat as rf
    import sum_voxels_ref
    exe = os.path.join(rf.ROOT, "3pcf_gb300", "bin", "tpcf_sum_voxels")
    files = []
    for src in sorted(glob.glob(os.path.join(rf.GOLDEN, "sandbox", "DDD_voxel2_*_1k.dat.gz"))):
        dst = str(tmp_path / os.path.basename(src)[:-3])
        rf.gunzip_to(src, dst)
        files.append(dst)
    assert len(files) == 8
    got = subprocess.run([exe] + files, capture_output=True, check=True).stdout.decode()
    assert got == sum_voxels_ref.sum_voxels(files)
    assert got.endswith("\n\n")
    bad = subprocess.run([exe, files[0], str(tmp_path / "missing.dat")], capture_output=True)
    assert bad.returncode == 1
