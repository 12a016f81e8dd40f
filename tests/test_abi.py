"""The C-ABI libraries build, load without a GPU and export every entry point
their headers declare.  No compute calls (this suite runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header: str) -> list[str]:
    with open(os.path.join(ROOT, "include", header)) as f:
        text = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "for", "return", "sizeof")))


def exported(lib: str) -> set[str]:
    out = subprocess.run(["nm", "-D", "--defined-only", lib], check=True, stdout=subprocess.PIPE, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.split()}


@pytest.fixture(scope="module")
def built():
    from thirring2d_gb300 import build
    return build.build()


def test_gpu_library_exports(built):
    names = declared("thirring_gpu.h")
    assert len(names) >= 25
    missing = [n for n in names if n not in exported(built["libthirring_gpu"])]
    assert not missing, missing


def test_python_binding_covers_header(built):
    from thirring2d_gb300 import native
    assert set(declared("thirring_gpu.h")) == set(native.SIGNATURES)


def test_library_loads_without_gpu(built):
    lib = ctypes.CDLL(built["libthirring_gpu"])
    lib.tg_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.tg_version()



def test_compat_library_exports_reference_names(built):
    """libthirring_hmc.so exports every hmc.c / mersenne.h name of include/thirring_hmc.h
    (functions and the globals m, g, mu, A, eta, tup, tdn, xup, xdn, mersenne_i, mersenne_array)."""
    names = set(declared("thirring_hmc.h"))
    assert {"fm_mul", "fm_conjugate_mul", "fmdm_invert_cg", "update_gauge", "momentum_step",
            "seed_mersenne", "mersenne_generate"} <= names
    globals_ = {"m", "g", "mu", "A", "eta", "tup", "tdn", "xup", "xdn", "mersenne_i", "mersenne_array"}
    missing = sorted((names | globals_) - exported(built["libthirring_hmc"]))
    assert not missing, missing


def test_hmc_program_built(built):
    assert os.access(built["hmc"], os.X_OK)


def test_integration_example_compiles_as_c(built, tmp_path):
    """The native-ABI example of INTEGRATION.md, wrapped in main(), compiles as
    plain C99 against include/thirring_gpu.h and links against
    libthirring_gpu.so (it is not run: no GPU here)."""
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        doc = f.read()
    m = re.search(r"```c\n(#include \"thirring_gpu.h\"\n.*?)```", doc, flags=re.S)
    assert m, "native-ABI example not found"
    include, body = m.group(1).split("\n", 1)
    src = tmp_path / "example.c"
    src.write_text("#include <stdio.h>\n#include <stdlib.h>\n" + include + "\n"
                   "static double A[1024 * 1024 * 2];\n"
                   "int main(void) {\n" + body + "  return rc == TG_OK ? 0 : 1;\n}\n")
    lib_dir = os.path.dirname(built["libthirring_gpu"])
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", f"-I{os.path.join(ROOT, 'include')}",
                        str(src), "-o", str(tmp_path / "example"), f"-L{lib_dir}", "-lthirring_gpu",
                        f"-Wl,-rpath,{lib_dir}"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout


def test_noalloc_path_calls_no_allocator():
    """tg_cg_noalloc (csrc/tg_noalloc.cu) and the explicit-grid launchers it
    calls (the *_fixed functions and resident_grid_nocache of tg_kernels.cu)
    name no allocating routine: no cudaMalloc* / cudaFree*, no cudaHostAlloc,
    no library allocator (dmalloc), no torch."""
    csrc = os.path.join(ROOT, "thirring2d_gb300", "csrc")

    def code(text):
        return re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", text, flags=re.S))

    with open(os.path.join(csrc, "tg_noalloc.cu")) as f:
        bodies = [code(f.read())]
    with open(os.path.join(csrc, "tg_kernels.cu")) as f:
        kern = code(f.read())
    for name in ("resident_grid_nocache", "link_phase_fixed", "cg64_init_fixed", "cg64_iter_fixed"):
        m = re.search(r"\n[^\n]*\b" + name + r"\([^;{]*\)\s*\{", kern)
        assert m, name
        depth, i = 0, m.end() - 1
        while True:  # the function body, by brace matching
            depth += {"{": 1, "}": -1}.get(kern[i], 0)
            i += 1
            if depth == 0:
                break
        bodies.append(kern[m.start():i])
    banned = re.compile(r"\b(cudaMalloc\w*|cudaFree\w*|cudaHostAlloc|cudaMallocHost|cuMem\w*Alloc\w*|dmalloc|"
                        r"malloc|calloc|realloc|new\s|torch)\b")
    for body in bodies:
        hits = banned.findall(body)
        assert not hits, hits
