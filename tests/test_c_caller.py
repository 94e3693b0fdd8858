"""A plain C translation unit against the C ABI (tests/c_caller.c).

The header promises that C code can include the reference's own headers
first (mtgp32-fast.h, mtgp64-fast.h: their structs, mtgp32-fast.h:47-88) and
then mtgp_gpu.h, and pass the reference's parameter tables to the library
unchanged.  These tests compile and link such callers with gcc against
libmtgp_gb300.so: with the reference's headers and table (CPU, where the
reference tree is present), with the header's own definitions (CPU), and one
that generates on the GPU and is compared with the oracle.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("MTGP_REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference"))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path, with_ref):
    from mtgp_gb300 import build as b
    lib = b.build()
    exe = str(tmp_path / ("c_caller_ref" if with_ref else "c_caller"))
    cmd = ["gcc", "-std=gnu99", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_caller.c")]
    if with_ref:
        cmd += ["-DWITH_REF", "-I", REF, os.path.join(REF, "mtgp32-param-fast.c")]
    libdir = os.path.dirname(lib)
    cmd += ["-L", libdir, "-lmtgp_gb300", "-Wl,-rpath," + libdir,
            "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64"),
            "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _params_file(tmp_path):
    from mtgp_gb300.params import load_table
    p = load_table("mtgp32_fast_11213")[0]
    pf = tmp_path / "params.bin"
    pf.write_bytes(bytes(p))
    return p, str(pf)


def test_c_caller_with_own_types(tmp_path):
    exe = _build(tmp_path, False)
    _, pf = _params_file(tmp_path)
    r = subprocess.run([exe, "abi", pf], capture_output=True, text=True)
    assert r.returncode == 0 and "abi ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "mtgp32-fast.h")),
                    reason="reference tree not present")
def test_c_caller_with_reference_headers_and_table(tmp_path):
    exe = _build(tmp_path, True)
    r = subprocess.run([exe, "abi"], capture_output=True, text=True)
    assert r.returncode == 0 and "abi ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
def test_c_caller_generates_on_the_gpu(gpu, orc, tmp_path):
    p, pf = _params_file(tmp_path)
    exe = _build(tmp_path, False)
    r = subprocess.run([exe, "gen", pf], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.array([int(x, 16) for x in r.stdout.split()], dtype=np.uint32)
    o = orc.gen(p, seed=1234)
    ref = np.concatenate([o.fill(0, 1000).view(np.uint32), o.fill(2, 1000).view(np.uint32)])
    assert np.array_equal(got, ref)
