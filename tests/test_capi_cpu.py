"""CPU: the C-ABI library loads and exports every symbol the header declares."""
import ctypes
import subprocess

import pytest

from robust_blockwise_random_pivoting_gb300 import _lib


def test_header_symbols_exported(rbrp_lib):
    names = _lib.header_symbols()
    assert "rbrp_id_f64" in names and "rbrp_RBRP" in names and "rbrp_RandAdapRBRP" in names
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(rbrp_lib, n)


def test_ctypes_struct_layout_matches_header(rbrp_lib):
    assert ctypes.sizeof(_lib.Params) == 48
    p = _lib.Params()
    rbrp_lib.rbrp_params_default(ctypes.byref(p))
    assert p.b == 64 and p.tol == 1e-12 and p.sampler == 0 and p.compute_T == 1 and p.kmax == 0
    assert rbrp_lib.rbrp_abi_version() == 1


def test_status_strings(rbrp_lib):
    for code, text in _lib.STATUS.items():
        assert rbrp_lib.rbrp_status_string(code).decode() == text


def test_null_arguments_rejected_without_gpu(rbrp_lib):
    # argument checks run before any CUDA call
    assert rbrp_lib.rbrp_create(None, 0) == 1
    assert rbrp_lib.rbrp_destroy(None) == 1
    r = _lib.Result()
    assert rbrp_lib.rbrp_id_f64(None, 4, 4, None, 4, None, None, ctypes.byref(r)) == 1
    assert rbrp_lib.rbrp_copy_T(None, None, 0) == 1
    assert rbrp_lib.rbrp_copy_L(None, None, 0) == 1


def test_create_without_gpu_fails_cleanly(rbrp_lib):
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert rbrp_lib.rbrp_create(ctypes.byref(h), 0) == 2   # RBRP_ERR_CUDA, no crash


def test_cpp_dropin_header_compiles(tmp_path):
    """include/rbrp_gb300.hpp (the gpu/rbrp.hpp and gpu/rid.hpp shims) is valid C++."""
    import os
    inc = os.path.dirname(_lib.HEADER)
    src = tmp_path / "use.cpp"
    src.write_text('#include "rbrp_gb300.hpp"\n'
                   'int f(double* A) { std::vector<int> r; std::vector<double> e, t; double tt, fl;\n'
                   '  return (int)rbrp_gb300::RBRP(4, 4, A, 2, r, e, t, tt, fl); }\n')
    out = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", inc, str(src)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr


def test_struct_sizes_match_c(tmp_path):
    """ctypes mirrors of the ABI structs have the C compiler's sizes and field offsets."""
    import os
    inc = os.path.dirname(_lib.HEADER)
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "rbrp_gb300.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(rbrp_params), '
                   'sizeof(rbrp_result), sizeof(rbrp_batch_problem), sizeof(rbrp_batch_result), '
                   'sizeof(rbrp_batch_info), offsetof(rbrp_batch_problem, T_cap), '
                   'offsetof(rbrp_batch_result, alg_flops)); return 0; }\n')
    exe = tmp_path / "sz"
    out = subprocess.run(["gcc", "-I", inc, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert sizes == [ctypes.sizeof(_lib.Params), ctypes.sizeof(_lib.Result), ctypes.sizeof(_lib.BatchProblem),
                     ctypes.sizeof(_lib.BatchResult), ctypes.sizeof(_lib.BatchInfo),
                     _lib.BatchProblem.T_cap.offset, _lib.BatchResult.alg_flops.offset]


def test_batch_entry_points_reject_bad_arguments_without_gpu(rbrp_lib):
    assert rbrp_lib.rbrp_batch_plan(None, 1, None, None) == 1
    assert rbrp_lib.rbrp_batch_run(None) == 1
    assert rbrp_lib.rbrp_batch_results(None, None, 0) == 1
    info = _lib.BatchInfo()
    assert rbrp_lib.rbrp_batch_get_info(None, ctypes.byref(info)) == 1
    assert rbrp_lib.rbrp_batch_set_profiling(None, 1) == 1
    assert rbrp_lib.rbrp_batch_set_order(None, None, 0) == 1


def test_sketch_lu_and_fixed_skeleton_entry_points_reject_null_handle(rbrp_lib):
    """The comparison-ID and differentiable entry points check arguments before any CUDA call."""
    r = _lib.Result()
    loss = ctypes.c_double()
    assert rbrp_lib.rbrp_sketch_gaussian_f32(None, 4, 8, 8, None, 8, 0, ctypes.c_float(1.0), None, 4) == 1
    assert rbrp_lib.rbrp_lupp_pivots_f64(None, 2, 8, None, 2, None, None) == 1
    assert rbrp_lib.rbrp_fixed_id_f64(None, 8, 8, None, 8, None, 2, 2, None, ctypes.byref(r)) == 1
    assert rbrp_lib.rbrp_fixed_id_f32(None, 8, 8, None, 8, None, 2, 2, None, ctypes.byref(r)) == 1
    assert rbrp_lib.rbrp_fixed_id_adjoint_f32(None, 8, 8, None, 8, None, ctypes.c_float(1.0), None, 8,
                                              ctypes.byref(loss)) == 1
    p, fl = ctypes.c_void_p(), ctypes.c_double()
    assert rbrp_lib.rbrp_RandLUPP_OS(None, 8, 8, 2, ctypes.byref(p), ctypes.byref(p), ctypes.byref(p),
                                     ctypes.byref(fl), 0) == 1
    assert rbrp_lib.rbrp_RandCPQR_OS(None, 8, 8, 2, None, None, ctypes.byref(p), ctypes.byref(fl), 0) == 1
    assert rbrp_lib.rbrp_CPQR(8, 8, None, None, 0, None, None, None, None) == 1
