"""The C++ adaptor include/qed3_linop.h compiles inside the reference's own
operator and solver headers and links against libqed3 (tests/c_abi/
reference_shim.cu instantiates the reference's MatPoly::solve over Qed3Op).
Needs the reference tree ($QED3_REFERENCE, or `reference` beside the
repository); skipped where it is absent.  Build only: no GPU call."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _reference():
    for c in (os.environ.get("QED3_REFERENCE"), os.path.join(os.path.dirname(ROOT), "reference")):
        if c and os.path.isdir(os.path.join(c, "src", "both_3d")):
            return c
    return None


def test_linop_shim_compiles_against_reference_headers(tmp_path):
    ref = _reference()
    if ref is None:
        pytest.skip("reference tree absent")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc absent")
    import qed3_gb300 as Q
    lib = Q.lib()._name
    b3 = os.path.join(ref, "src", "both_3d")
    exe = str(tmp_path / "shim")
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
           f"-I{os.path.join(ROOT, 'include')}",
           f"-DREF_GPU_HEADER_H=\"{os.path.join(b3, 'gpu_header.h')}\"",
           f"-DREF_SPARSE_MATRIX_H=\"{os.path.join(b3, 'sparse_matrix.h')}\"",
           f"-DREF_MATPOLY_H=\"{os.path.join(b3, 'matpoly.h')}\"",
           os.path.join(HERE, "c_abi", "reference_shim.cu"), "-o", exe,
           lib, "-lcublas", f"-Xlinker=-rpath={os.path.dirname(lib)}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(exe)
