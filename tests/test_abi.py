"""The C-ABI library loads and exports every symbol include/*.h declares (CPU)."""
import re

import pytest
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"#define[^\n]*(\\\n[^\n]*)*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name in {"if", "for", "while", "return", "sizeof", "COSMA_GPU_PXGEMM_ARGS"}:
                continue
            # function declarations end with ');' after the parameter list
            tail = text[m.end():]
            depth, i = 1, 0
            while depth and i < len(tail):
                depth += {"(": 1, ")": -1}.get(tail[i], 0)
                i += 1
            if tail[i:].lstrip().startswith(";"):
                names.add(name)
    return names


def test_header_declares_the_drop_in_surface():
    names = declared_symbols()
    for must in ["pdgemm_", "pzgemm_", "psgemm", "PDGEMM_", "cosma_pdgemm", "COSMA_PZGEMM_",
                 "cosma_gpu_tmm_gemm_d", "cosma_gpu_tmm_make_context", "cosma_gpu_local_multiply_d",
                 "cosma_gpu_dgemm_ozaki_device", "cosma_gpu_zgemm_ozaki_device", "costa_gpu_pack", "costa_gpu_unpack_d"]:
        assert must in names, must


def test_library_exports_every_declared_symbol(native_lib):
    names = declared_symbols()
    assert len(names) >= 60
    missing = [n for n in sorted(names) if not hasattr(native_lib, n)]
    assert not missing, missing


def test_build_targets_sm_103a_only():
    from cosma_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_version_string_without_gpu(native_lib):
    assert b"sm_103a" in native_lib.cosma_gpu_version()


def test_python_bindings_cover_the_header():
    from cosma_gb300 import _native
    assert declared_symbols() <= set(_native.SIGNATURES)


def test_cpp_shims_compile_link_and_throw_without_a_gpu(native_lib, tmp_path):
    """include/cosma_gb300.hpp (gpu::make_context / gpu::gemm / local_multiply
    with the reference's call shapes) compiles, links against the library and,
    on a machine without a usable GPU, reports the failure as the reference
    does: by throwing std::runtime_error with the library's message."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        import pytest
        pytest.skip("g++ not available")
    from cosma_gb300._native import LIB_PATH
    src = tmp_path / "shim.cpp"
    src.write_text(r'''
#include "cosma_gb300.hpp"
#include <cstdio>
#include <vector>
int main() {
    using namespace cosma_gb300;
    std::vector<double> a(4, 1.0), b(4, 1.0), c(4, 0.0);
    try {
        auto ctx = gpu::make_context<double>(2, 0, 0, 0);
        gpu::gemm(*ctx, 'N', 'N', 2, 2, 2, 1.0, a.data(), 2, b.data(), 2, 0.0, c.data(), 2);
        local_multiply(ctx.get(), a.data(), b.data(), c.data(), 2, 2, 2, 1.0, 0.0);
        std::printf("ran %g\n", c[0]);
    } catch (const std::runtime_error& e) {
        std::printf("threw %s\n", e.what());
    }
    return 0;
}
''')
    exe = tmp_path / "shim"
    cmd = ["g++", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe), f"-L{LIB_PATH.parent}",
           "-lcosma_gb300", f"-Wl,-rpath,{LIB_PATH.parent}"]
    subprocess.run(cmd, check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120).stdout
    assert out.startswith("ran 2") or out.startswith("threw cosma_gb300: "), out


_FAKE_SCALAPACK = r'''
#include <stdio.h>
/* stands in for the real ScaLAPACK linked after the drop-in: marks C */
void pdgemm_(const char* ta, const char* tb, const int* m, const int* n, const int* k, const double* alpha,
             const double* a, const int* ia, const int* ja, const int* desca, const double* b, const int* ib,
             const int* jb, const int* descb, const double* beta, double* c, const int* ic, const int* jc,
             const int* descc) { c[0] = 42.0; }
void pzgemm_(const char* ta, const char* tb, const int* m, const int* n, const int* k, const double* alpha,
             const double* a, const int* ia, const int* ja, const int* desca, const double* b, const int* ib,
             const int* jb, const int* descb, const double* beta, double* c, const int* ic, const int* jc,
             const int* descc) { c[0] = 43.0; }
'''

_THRESHOLD_MAIN = r'''
#include "cosma_gb300.h"
#include <stdio.h>
int main(int argc, char** argv) {
    int nn = 4, one = 1;
    int desc[9] = {1, 0, 4, 4, 2, 2, 0, 0, 4};
    double a[32], b[32], c[32], alpha[2] = {1.0, 0.0}, beta[2] = {0.0, 0.0};
    for (int i = 0; i < 32; ++i) { a[i] = 1.0; b[i] = 1.0; c[i] = 0.0; }
    pdgemm_("N", "N", &nn, &nn, &nn, alpha, a, &one, &one, desc, b, &one, &one, desc, beta, c, &one, &one, desc);
    printf("pdgemm_ %g\n", c[0]);
    c[0] = -1.0;
    cosma_pdgemm("N", "N", &nn, &nn, &nn, alpha, a, &one, &one, desc, b, &one, &one, desc, beta, c, &one, &one, desc);
    printf("cosma_pdgemm %g\n", c[0]);
    c[0] = -1.0;
    c[1] = -1.0;
    /* complex view: every entry of A and B is 1 + 1i, so C = 4 (1 + 1i)^2 = 8i */
    PZGEMM("N", "N", &nn, &nn, &nn, alpha, a, &one, &one, desc, b, &one, &one, desc, beta, c, &one, &one, desc);
    printf("PZGEMM %g %g\n", c[0], c[1]);
    return 0;
}
'''


def _build_threshold_case(tmp_path):
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        import pytest
        pytest.skip("gcc not available")
    from cosma_gb300._native import LIB_PATH
    (tmp_path / "fake.c").write_text(_FAKE_SCALAPACK)
    (tmp_path / "main.c").write_text(_THRESHOLD_MAIN)
    subprocess.run(["gcc", "-shared", "-fPIC", str(tmp_path / "fake.c"), "-o", str(tmp_path / "libfakescalapack.so")],
                   check=True, capture_output=True)
    exe = tmp_path / "main"
    # the drop-in first, the "real" ScaLAPACK after it, as the reference's README links them
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(tmp_path / "main.c"), "-o", str(exe),
                    f"-L{LIB_PATH.parent}", "-lcosma_gb300", "-Wl,--no-as-needed", f"-L{tmp_path}", "-lfakescalapack",
                    f"-Wl,-rpath,{LIB_PATH.parent}:{tmp_path}"], check=True, capture_output=True)
    return exe


def test_dim_threshold_falls_through_to_the_next_pxgemm(native_lib, tmp_path):
    """COSMA_DIM_THRESHOLD: problems with min(m, n, k) below it go to the
    next p?gemm_ definition (the real ScaLAPACK), for every spelling of the
    entry point (src/cosma/pxgemm.cpp, cosma_pxgemm.cpp:652-655).  The fake
    next library marks C; the drop-in's own path is never entered."""
    import os
    import subprocess
    exe = _build_threshold_case(tmp_path)
    env = dict(os.environ, COSMA_DIM_THRESHOLD="5")
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120, env=env).stdout
    assert out.split("\n")[:3] == ["pdgemm_ 42", "cosma_pdgemm 42", "PZGEMM 43 -1"], out


@pytest.mark.gpu
def test_dim_threshold_keeps_larger_problems(native_lib, tmp_path):
    """At or above the threshold the drop-in computes C itself (4 = 1 x 1
    summed over k = 4; complex 8i), never the next library's marker."""
    import os
    import subprocess
    exe = _build_threshold_case(tmp_path)
    env = dict(os.environ, COSMA_DIM_THRESHOLD="4")
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300, env=env).stdout
    assert out.split("\n")[:3] == ["pdgemm_ 4", "cosma_pdgemm 4", "PZGEMM 0 8"], out
