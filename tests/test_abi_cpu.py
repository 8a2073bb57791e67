"""CPU-side checks of the C ABI library and the b200 target programs.

No kernel is launched here: the library must load and export every symbol
include/kg_b200.h declares, reject bad arguments before touching the GPU,
and the b200 programs must reproduce the reference's host-side lines
(coefficients, initial mean) before they reach the device.
"""
import ctypes
import json
import os
import re
import subprocess

import pytest

import kgb200

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "kernelgen-perf-tests_gb300", "build", "bin")
SUMS = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_checksums.json")))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(kgb200.LIB_PATH) or not os.path.exists(os.path.join(BIN, "laplacian_b200")):
        kgb200.build()
    return kgb200.load()


def header_symbols():
    src = open(kgb200.HEADER).read()
    return sorted(set(re.findall(r"^(?:kg_status|int|const char\*)\s+(kg_\w+)\s*\(", src, re.M)))


def test_header_symbols_exported(lib):
    syms = header_symbols()
    assert len(syms) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", kgb200.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(kg_\w+)$", out, re.M))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    assert sorted(syms) == sorted(kgb200.EXPORTS)


def test_metadata(lib):
    assert [lib.kg_stencil_narrays(i) for i in range(11)] == [2, 4, 4, 6, 3, 5, 5, 2, 2, 2, 2]
    assert [lib.kg_stencil_ncoefs(i) for i in range(11)] == [2, 3, 3, 2, 3, 0, 0, 3, 4, 6, 0]
    assert [lib.kg_stencil_is2d(i) for i in range(11)] == [0, 0, 0, 0, 0, 0, 0, 1, 0, 1, 1]
    assert lib.kg_stencil_outputs(2) == 0xE and lib.kg_stencil_outputs(1) == 0x1
    assert lib.kg_stencil_narrays(11) == -1
    assert lib.kg_version().startswith(b"kg_b200")
    assert lib.kg_status_string(4) == b"KG_ETIMEOUT"


def test_bad_arguments_rejected_before_launch(lib):
    a = ctypes.create_string_buffer(8 * 512)
    b = ctypes.create_string_buffer(8 * 512)
    pa, pb = ctypes.addressof(a), ctypes.addressof(b)
    # unknown stencil
    p = kgb200.problem(42, kgb200.KG_F64, (8, 8, 8), [], [pa, pb])
    assert lib.kg_sweep(ctypes.byref(p), None) == 1
    assert b"unknown stencil" in lib.kg_last_error()
    # negative size
    assert lib.kg_laplacian(kgb200.KG_F64, -1, 8, 8, 1.0, 1.0, pa, pb, None) == 1
    # aliasing output
    assert lib.kg_laplacian(kgb200.KG_F64, 8, 8, 8, 1.0, 1.0, pa, pa, None) == 1
    assert b"overlaps" in lib.kg_last_error()
    # null array
    assert lib.kg_laplacian(kgb200.KG_F64, 8, 8, 8, 1.0, 1.0, pa, None, None) == 1
    # byte cells for a real-valued stencil
    assert lib.kg_laplacian(kgb200.KG_U8, 8, 8, 8, 1.0, 1.0, pa, pb, None) == 5
    # bad plan arguments
    h = ctypes.c_void_p()
    assert lib.kg_plan_create(ctypes.byref(h), None, 3) == 1
    # engines: unknown id, not built for the type, TMA on rows that are not
    # a multiple of 16 bytes or on unaligned arrays
    p = kgb200.problem("laplacian", kgb200.KG_F64, (8, 8, 8), [1.0, 1.0], [pa, pb], engine=7)
    assert lib.kg_sweep(ctypes.byref(p), None) == 1 and b"unknown engine" in lib.kg_last_error()
    p = kgb200.problem("laplacian", kgb200.KG_F64, (8, 8, 8), [1.0, 1.0], [pa, pb], engine="staged")
    assert lib.kg_sweep(ctypes.byref(p), None) == 5
    p = kgb200.problem("laplacian", kgb200.KG_U8, (8, 8, 8), [1.0, 1.0], [pa, pb], engine="tma")
    assert lib.kg_sweep(ctypes.byref(p), None) == 5
    p = kgb200.problem("laplacian", kgb200.KG_F32, (6, 8, 8), [1.0, 1.0], [pa, pb], engine="tma")
    assert lib.kg_sweep(ctypes.byref(p), None) == 1 and b"16-byte" in lib.kg_last_error()
    p = kgb200.problem("laplacian", kgb200.KG_F32, (8, 8, 8), [1.0, 1.0], [pa + 4, pb], engine="tma")
    assert lib.kg_sweep(ctypes.byref(p), None) == 1 and b"16-byte" in lib.kg_last_error()


def test_device_check_without_gpu(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert lib.kg_device_check() == 6


SMALL = [(t, r) for t in SUMS["runs"] for r in SUMS["runs"][t] if not r.get("readme_config")][::3]


@pytest.mark.parametrize("name,run", SMALL, ids=["%s-%s" % (t, "x".join(map(str, r["args"]))) for t, r in SMALL])
def test_driver_host_lines(lib, name, run):
    """Before the device phases, the b200 program prints the reference's
    coefficient and initial-mean lines (its rand() draw order)."""
    env = {k: v for k, v in os.environ.items() if k != "NO_TIMING"}
    out = subprocess.run([os.path.join(BIN, name + "_b200")] + [str(a) for a in run["args"]],
                         capture_output=True, text=True, env=env, timeout=120)
    lines = [ln.rstrip() for ln in out.stdout.splitlines()]
    want = [ln.rstrip() for ln in run["lines"] if not ln.startswith("final mean")]
    for w in want:
        assert w in lines
    if out.returncode != 0:  # no GPU here: it must stop, loudly, at the device
        assert "Error" in out.stderr


def test_driver_usage_and_bad_args(lib):
    out = subprocess.run([os.path.join(BIN, "laplacian_b200"), "1", "2"], capture_output=True, text=True)
    assert out.returncode == 1 and out.stdout.startswith("Usage:")
    out = subprocess.run([os.path.join(BIN, "gameoflife_b200"), "8", "-3", "2"], capture_output=True, text=True)
    assert out.returncode == 1 and "Value for ny is invalid: -3" in out.stdout
