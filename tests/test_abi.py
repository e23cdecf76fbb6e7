"""The C-ABI library loads and exports every symbol include/*.h declares (CPU)."""
import re
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
