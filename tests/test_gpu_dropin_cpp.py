"""GPU: a C++ caller of the reference's entry points, linked to the library.

``tests/dropin/driver_dropin.cpp`` calls ``RBRP`` (gpu/rbrp.hpp:6-8) and
``RandAdapLUPP`` (gpu/rid.hpp:5-7) as the reference's driver does
(gpu/driver.cpp:177), through ``include/rbrp_gb300.hpp``.  The test compiles it
with the host C++ compiler, links ``librbrp_gb300.so`` and the CUDA runtime,
runs it on the GPU and compares its output with the oracle: the RBRP trace
(cumulative ranks exactly, squared residuals to rtol 1e-6) on a 150 x 170
matrix, and RandAdapLUPP's rank, skeleton (bit for bit) and ID error (within
1.05x of the oracle's) on the seeded 1000 x 1000 workload (b = 40, squared
tol 1e-12).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import id_error, interp_sid, rbrp_column_id  # noqa: E402
from robust_blockwise_random_pivoting_gb300 import _lib  # noqa: E402
from robust_blockwise_random_pivoting_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver(rbrp_lib, tmp_path_factory):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    cuda = os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"))
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("dropin") / "driver_dropin")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.dirname(_lib.HEADER), "-I", os.path.join(cuda, "include"),
           os.path.join(HERE, "dropin", "driver_dropin.cpp"), "-o", exe, "-L", libdir, "-lrbrp_gb300",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{libdir}:{os.path.join(cuda, 'lib64')}"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    return exe


def _run(exe, A, blk, tol, tmp_path):
    mat, res = tmp_path / "A.bin", tmp_path / "out.bin"
    m, n = A.shape
    with open(mat, "wb") as f:
        np.array([m, n], np.int32).tofile(f)
        np.asfortranarray(A, dtype=np.float64).ravel(order="F").tofile(f)
    p = subprocess.run([exe, str(mat), str(blk), repr(float(tol)), str(res)], capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, (p.returncode, p.stderr)
    lines = p.stdout.strip().splitlines()
    nb = int(lines[0].split()[1])
    trace = np.array([[float(x) for x in ln.split()] for ln in lines[1:1 + nb]])
    raw = open(res, "rb").read()
    k = int(np.frombuffer(raw[:4], np.int32)[0])
    ints = np.frombuffer(raw[4:4 + 4 * n], np.int32)
    T = np.frombuffer(raw[4 + 4 * n:], np.float64).reshape(n - k, k).T if 0 < k < n else np.zeros((k, n - k))
    return trace, k, ints[:k], ints[k:], T


def test_cpp_rbrp_trace_matches_oracle(driver, tmp_path):
    A = W.gaussian_exp(150, 170, decay=10.0, seed=7)
    trace, _, _, _, _ = _run(driver, A, 20, 1e-10, tmp_path)
    o = rbrp_column_id(A, 20, tol=None, seed=0)
    assert np.array_equal(trace[:, 0].astype(int), o["ranks"])
    np.testing.assert_allclose(trace[:, 1], o["residuals"], rtol=1e-6, atol=1e-14)


def test_cpp_rand_adap_lupp_matches_oracle_on_cfg0(driver, tmp_path):
    A = W.gaussian_exp()                       # 1000 x 1000, s_i = exp(-i/20), Philox seed 0
    _, k, sk, rd, T = _run(driver, A, 40, 1e-12, tmp_path)
    o = rbrp_column_id(A, 40, tol=1e-12, seed=0)
    assert k == o["k"]
    assert np.array_equal(sk, o["perm"][:k]) and np.array_equal(rd, o["perm"][k:])
    perm = np.concatenate([sk, rd])
    e_ref = id_error(A, o["perm"], interp_sid(A, o["perm"], k))
    assert np.sqrt(id_error(A, perm, T)) <= 1.05 * np.sqrt(e_ref)
