"""Recipe: build the reference hmc.c, with its adjoint corrected, into oracle/_ref/.

TEST INFRASTRUCTURE ONLY (the oracle side of the parity tests and the
reference arm of bench.py).  Nothing in the product imports this.

The reference (rantahar/Thirring2D) has no library form: hmc.c fixes NT/NX with
unconditional #defines (hmc.c:14-15), defines main() (hmc.c:847) and needs
<lapacke.h> for a determinant that main never calls (hmc.c:6, 314-336).  Its
fm_conjugate_mul (hmc.c:188-249) is a verbatim copy of fm_mul, so its CG on
"M^dagger M" diverges and calls exit(1) (hmc.c:383-386) on every lattice tried.

This script writes ONE generated source, oracle/_ref/src/hmc_patched.c, from the
reference's own hmc.c with these textual edits and nothing else:

  * ``#define NT 32`` / ``#define NX 32``  ->  ``#define NT REF_NT`` / ``REF_NX``
    (sizes chosen per build with -D);
  * ``int main(void)`` -> ``int hmc_reference_main(void)`` (the driver has its own
    set-up and never calls it);
  * ``#define CG_MAX_ITER 100000`` -> ``REF_CG_MAX_ITER`` (100000 in every build
    except the "sample" variant, whose CG stops silently after 20 iterations as
    hmc.c:364 does at its cap -- the bounded CPU-baseline sample of bench.py);
  * inside fm_conjugate_mul only: every ``v += `` / ``v -= `` of a hop term is
    multiplied by ``REF_ADJ_SIGN`` and ``exp(mu)``/``exp(-mu)`` by
    ``REF_ADJ_MUSIGN``.  With -DREF_ADJ_SIGN=-1 -DREF_ADJ_MUSIGN=-1 the function
    applies the true adjoint M^dagger = m - D(-mu) ("REF-FIXED"); with +1/+1 it is
    the shipped code ("REF-EXACT");
  * every ``x2 > x`` test (the x-boundary branches of fm_mul, fm_conjugate_mul,
    fermion_matrix and momentum_step) becomes ``(x2 > x || REF_PERIODIC_X)``
    after ``x2 = xup[x]`` and ``(x2 > x && !REF_PERIODIC_X)`` after
    ``x2 = xdn[x]``, so -DREF_PERIODIC_X=1 gives a periodic x direction and 0
    the shipped antiperiodic one.

Each edit asserts how many places it changed, so a different hmc.c fails loudly.
mersenne_inline.c / mersenne.h are copied unchanged.  oracle/ref_driver.c (own
code) #includes the generated file and exposes flat-array entry points; one
shared library is built per (NT, NX, variant) into oracle/_ref/.

The reference tree (THIRRING2D_REF, default /root/reference) is read only
here, at generation time.  The generated sources
stay in oracle/_ref/src (git-ignored); where the reference tree is absent (the
GPU host) the libraries are rebuilt from those generated sources if present.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout; THIRRING2D_REF overrides the default location
REF_ROOT = os.environ.get("THIRRING2D_REF", "/root/reference")
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")

# (nt, nx) sizes the tests, fixtures and the CPU baseline use.
DEFAULT_SIZES = [(4, 4), (6, 4), (8, 8), (16, 16), (64, 64), (1024, 1024), (2048, 2048)]
# sizes that also get the bounded-CG "sample" build used for CPU timing
SAMPLE_SIZES = [(16, 16), (64, 64), (1024, 1024), (2048, 2048)]
# variant name -> compile definitions
VARIANTS = {
    "fixed_apx": dict(REF_ADJ_SIGN=-1, REF_ADJ_MUSIGN=-1, REF_PERIODIC_X=0),  # reference BCs, true adjoint
    "fixed_px": dict(REF_ADJ_SIGN=-1, REF_ADJ_MUSIGN=-1, REF_PERIODIC_X=1),   # periodic x, true adjoint
    "exact_apx": dict(REF_ADJ_SIGN=1, REF_ADJ_MUSIGN=1, REF_PERIODIC_X=0),    # as shipped
    "sample_px": dict(REF_ADJ_SIGN=-1, REF_ADJ_MUSIGN=-1, REF_PERIODIC_X=1, REF_CG_MAX_ITER=21),
}
DEFAULT_CG_MAX_ITER = 100000


def _sub(pattern: str, repl: str, text: str, count_expected: int, flags=0) -> str:
    new, n = re.subn(pattern, repl, text, flags=flags)
    if n != count_expected:
        raise RuntimeError(f"make_ref: pattern {pattern!r} matched {n} times, expected {count_expected}")
    return new


def _patch_x_boundary(text: str) -> str:
    """Make the x-boundary branches switchable.  After ``x2 = xup[x]`` the test
    ``x2 > x`` means "interior" (the periodic case always takes it); after
    ``x2 = xdn[x]`` it means "wrapped" (the periodic case never takes it)."""
    out, last, n_up, n_dn = [], None, 0, 0
    for line in text.split("\n"):
        if re.search(r"\bx2 = xup\[x\]", line):
            last = "up"
        elif re.search(r"\bx2 = xdn\[x\]", line):
            last = "dn"
        if re.search(r"\bx2 > x\b", line):
            if last == "up":
                line, k = re.subn(r"\bx2 > x\b", "(x2 > x || REF_PERIODIC_X)", line)
                n_up += k
            elif last == "dn":
                line, k = re.subn(r"\bx2 > x\b", "(x2 > x && !REF_PERIODIC_X)", line)
                n_dn += k
            else:
                raise RuntimeError("make_ref: x-boundary test with no preceding x2 assignment")
        out.append(line)
    if (n_up, n_dn) != (7, 3):
        raise RuntimeError(f"make_ref: patched {n_up} forward / {n_dn} backward x-boundary tests, expected 7 / 3")
    return "\n".join(out)


def generate() -> str:
    """Write oracle/_ref/src/hmc_patched.c (+ RNG files, lapacke stub)."""
    os.makedirs(SRC, exist_ok=True)
    with open(os.path.join(REF_ROOT, "hmc.c")) as f:
        text = f.read()
    text = _sub(r"^#define NT 32\s*$", "#define NT REF_NT", text, 1, re.M)
    text = _sub(r"^#define NX 32\s*$", "#define NX REF_NX", text, 1, re.M)
    text = _sub(r"\bint main\(void\)", "int hmc_reference_main(void)", text, 1)
    text = _sub(r"^#define CG_MAX_ITER 100000\s*$", "#define CG_MAX_ITER REF_CG_MAX_ITER", text, 1, re.M)
    # fm_conjugate_mul body: from its signature to the first line that is "}".
    start = text.index("void fm_conjugate_mul(_Complex double ** v_in")
    end = text.index("\n}\n", start) + 3
    body = text[start:end]
    body = _sub(r"expmu = exp\(mu\);", "expmu = exp(REF_ADJ_MUSIGN*mu);", body, 1)
    body = _sub(r"expmmu = exp\(-mu\);", "expmmu = exp(-REF_ADJ_MUSIGN*mu);", body, 1)
    body = _sub(r"v \+= 0\.5 \*", "v += REF_ADJ_SIGN * 0.5 *", body, 4)
    body = _sub(r"v -= 0\.5 \*", "v -= REF_ADJ_SIGN * 0.5 *", body, 4)
    text = text[:start] + body + text[end:]
    text = _patch_x_boundary(text)
    header = ("/* GENERATED by oracle/make_ref.py from rantahar/Thirring2D hmc.c -- do not edit,\n"
              " * do not commit.  Test-oracle build only. */\n")
    with open(os.path.join(SRC, "hmc_patched.c"), "w") as f:
        f.write(header + text)
    for name in ("mersenne_inline.c", "mersenne.h"):
        with open(os.path.join(REF_ROOT, name)) as fi, open(os.path.join(SRC, name), "w") as fo:
            fo.write(fi.read())
    # hmc.c includes <lapacke.h> for determinant(), which main never calls.
    with open(os.path.join(SRC, "lapacke.h"), "w") as f:
        f.write("/* stub: declares the one LAPACK routine hmc.c names; ref_driver.c defines it to abort() */\n"
                "void LAPACK_zgetrf(int* m, int* n, _Complex double* a, int* lda, int* ipiv, int* info);\n")
    return os.path.join(SRC, "hmc_patched.c")


VSRC = os.path.join(SRC, "vecops")
VEC_SIZES = [(8, 8), (6, 4), (16, 16)]


# declarations of the LAPACK routines the reference names; oracle/lapack_lu.c
# (own code) defines the two real ones where a build links them
LAPACKE_STUB = ("/* stub lapacke.h: declares the LAPACK routines the reference names */\n"
                "void LAPACK_zgetrf(int* m, int* n, _Complex double* a, int* lda, int* ipiv, int* info);\n"
                "void LAPACK_dgetrf(int* m, int* n, double* a, int* lda, int* ipiv, int* info);\n"
                "void LAPACK_dgetri(int* n, double* a, int* lda, int* ipiv, double* work, int* lwork, int* info);\n")


def generate_vecops() -> None:
    """The fermion-bag sources: vec_ops.c, fermion_matrix.c and full_determinant.c
    unchanged, next to a copy of Thirring.h with these edits (every file
    includes "Thirring.h" from its own directory, so all sit in
    oracle/_ref/src/vecops/):

      * ``#define NT 64`` / ``#define NX 64``  ->  REF_NT / REF_NX;
      * ``#define ANTISYMMETRIC`` is kept unless REF_OPENX is set, which selects
        the file's own OPENX boundary instead (open x, antisymmetric t);
      * ``#define FLUCTUATION_MATRIX`` is kept unless REF_NO_FLUCTUATION_MATRIX
        is set: full_determinant.c compiles its determinant_mu only without it
        (full_determinant.c:15).
    """
    os.makedirs(VSRC, exist_ok=True)
    with open(os.path.join(REF_ROOT, "Thirring.h")) as f:
        text = f.read()
    text = _sub(r"^#define NT 64\s*$", "#define NT REF_NT", text, 1, re.M)
    text = _sub(r"^#define NX 64\s*$", "#define NX REF_NX", text, 1, re.M)
    text = _sub(r"^#define ANTISYMMETRIC //Antisymmetric boundaries\s*$",
                "#if REF_OPENX\n#define OPENX\n#else\n#define ANTISYMMETRIC //Antisymmetric boundaries\n#endif",
                text, 1, re.M)
    text = _sub(r"^#define FLUCTUATION_MATRIX\s*$",
                "#ifndef REF_NO_FLUCTUATION_MATRIX\n#define FLUCTUATION_MATRIX\n#endif", text, 1, re.M)
    with open(os.path.join(VSRC, "Thirring.h"), "w") as f:
        f.write("/* GENERATED by oracle/make_ref.py from rantahar/Thirring2D Thirring.h -- do not commit. */\n" + text)
    for name in ("vec_ops.c", "fermion_matrix.c", "full_determinant.c", "mersenne_inline.c", "mersenne.h"):
        with open(os.path.join(REF_ROOT, name)) as fi, open(os.path.join(VSRC, name), "w") as fo:
            fo.write(fi.read())
    with open(os.path.join(VSRC, "lapacke.h"), "w") as f:
        f.write(LAPACKE_STUB)


BSRC = os.path.join(SRC, "brute")


def generate_brute() -> None:
    """tests/thirring_brute.c, the reference's brute-force enumeration of the
    fermion-bag partition function on 4 x 4 with open x (its header fixes the
    size and boundary), with two edits:

      * ``#include "test_thirring.h"`` -> ``#include "thirring_brute.h"``: the
        header the repository ships under that other name (thirring_brute.c:10);
      * the final table's ``%g`` -> ``%.17g`` (five fields of one printf), so the
        sums come out at full precision.

    thirring_brute.h is copied unchanged; its ``#include "../mersenne.h"``
    finds oracle/_ref/src/mersenne.h, and its <lapacke.h> the stub here.
    """
    os.makedirs(BSRC, exist_ok=True)
    with open(os.path.join(REF_ROOT, "tests", "thirring_brute.c")) as f:
        text = f.read()
    text = _sub(r'#include "test_thirring\.h"', '#include "thirring_brute.h"', text, 1)
    lines = text.split("\n")
    hits = [i for i, ln in enumerate(lines) if 'printf(" Links %d Monomers %d det %g' in ln]
    if len(hits) != 1:
        raise RuntimeError(f"make_ref: brute-force table printf found {len(hits)} times, expected 1")
    lines[hits[0]] = _sub(r"%g", "%.17g", lines[hits[0]], 5)
    with open(os.path.join(BSRC, "thirring_brute.c"), "w") as f:
        f.write("/* GENERATED by oracle/make_ref.py from rantahar/Thirring2D tests/thirring_brute.c -- do not "
                "commit. */\n" + "\n".join(lines))
    with open(os.path.join(REF_ROOT, "tests", "thirring_brute.h")) as fi, \
            open(os.path.join(BSRC, "thirring_brute.h"), "w") as fo:
        fo.write(fi.read())
    with open(os.path.join(BSRC, "lapacke.h"), "w") as f:
        f.write(LAPACKE_STUB)


def brute_path() -> str:
    return os.path.join(OUT, "thirring_brute_T4X4")


def build_brute() -> str:
    """The brute-force program (reads its parameters from stdin as the
    reference's does), with vec_ops.c at 4 x 4 and open x for its
    measure_charge, and oracle/lapack_lu.c for dgetrf/dgetri."""
    out = brute_path()
    srcs = [os.path.join(BSRC, "thirring_brute.c"), os.path.join(VSRC, "vec_ops.c"),
            os.path.join(SRC, "mersenne_inline.c"), os.path.join(HERE, "lapack_lu.c")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    cmd = (["gcc", "-O2", "-std=gnu99", "-w", "-fcommon", f"-I{BSRC}", f"-I{VSRC}", "-DREF_NT=4", "-DREF_NX=4",
            "-DREF_OPENX=1", "-o", out] + srcs + ["-lm"])
    subprocess.run(cmd, check=True)
    return out


DET_SIZES = [(4, 4)]


def det_lib_path(nt: int, nx: int, openx: bool) -> str:
    return os.path.join(OUT, f"libdetref_T{nt}X{nx}_{'openx' if openx else 'apx'}.so")


def build_det_one(nt: int, nx: int, openx: bool) -> str:
    """full_determinant.c's determinant_mu with fermion_matrix.c's fM_index
    (mass on the diagonal), FLUCTUATION_MATRIX undefined, driven by
    oracle/det_driver.c; fermion_matrix.c and the driver both define the
    neighbour tables, hence -fcommon."""
    out = det_lib_path(nt, nx, openx)
    srcs = [os.path.join(HERE, "det_driver.c"), os.path.join(VSRC, "full_determinant.c"),
            os.path.join(VSRC, "fermion_matrix.c"), os.path.join(HERE, "lapack_lu.c")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    cmd = (["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-w", "-fcommon", "-Wl,-Bsymbolic", f"-I{VSRC}",
            f"-DREF_NT={nt}", f"-DREF_NX={nx}", f"-DREF_OPENX={1 if openx else 0}", "-DREF_NO_FLUCTUATION_MATRIX",
            "-o", out] + srcs + ["-lm"])
    subprocess.run(cmd, check=True)
    return out


def vec_lib_path(nt: int, nx: int) -> str:
    return os.path.join(OUT, f"libvecopsref_T{nt}X{nx}.so")


def build_vec_one(nt: int, nx: int) -> str:
    out = vec_lib_path(nt, nx)
    driver = os.path.join(HERE, "vecops_driver.c")
    srcs = [driver, os.path.join(VSRC, "vec_ops.c"), os.path.join(VSRC, "mersenne_inline.c")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    cmd = (["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-w", "-Wl,-Bsymbolic", f"-I{VSRC}",
            f"-DREF_NT={nt}", f"-DREF_NX={nx}", "-o", out] + srcs + ["-lm"])
    subprocess.run(cmd, check=True)
    return out


PROP_SIZES = [(8, 8), (6, 4)]


def prop_lib_path(nt: int, nx: int) -> str:
    return os.path.join(OUT, f"libpropref_T{nt}X{nx}.so")


def build_prop_one(nt: int, nx: int) -> str:
    """vec_ops.c + fermion_matrix.c with PROPAGATOR_MATRIX and WITH_MASS_MONOMERS:
    the reference's calc_Dinv (fermion_matrix.c:189-351).  fermion_matrix.c and
    Thirring.h both define the neighbour tables, hence -fcommon."""
    out = prop_lib_path(nt, nx)
    driver = os.path.join(HERE, "vecops_driver.c")
    srcs = [driver, os.path.join(VSRC, "vec_ops.c"), os.path.join(VSRC, "fermion_matrix.c"),
            os.path.join(VSRC, "mersenne_inline.c")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    cmd = (["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-w", "-fcommon", "-Wl,-Bsymbolic", f"-I{VSRC}",
            f"-DREF_NT={nt}", f"-DREF_NX={nx}", "-DPROPAGATOR_MATRIX", "-DWITH_MASS_MONOMERS", "-o", out]
           + srcs + ["-lm"])
    subprocess.run(cmd, check=True)
    return out


def lib_path(nt: int, nx: int, variant: str) -> str:
    return os.path.join(OUT, f"libhmcref_T{nt}X{nx}_{variant}.so")


def build_one(nt: int, nx: int, variant: str) -> str:
    out = lib_path(nt, nx, variant)
    driver = os.path.join(HERE, "ref_driver.c")
    srcs = [driver, os.path.join(SRC, "hmc_patched.c"), os.path.join(SRC, "mersenne_inline.c")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    var = dict(REF_CG_MAX_ITER=DEFAULT_CG_MAX_ITER, **{k: v for k, v in VARIANTS[variant].items()
                                                      if k != "REF_CG_MAX_ITER"})
    if "REF_CG_MAX_ITER" in VARIANTS[variant]:
        var["REF_CG_MAX_ITER"] = VARIANTS[variant]["REF_CG_MAX_ITER"]
    defs = [f"-DREF_NT={nt}", f"-DREF_NX={nx}"] + [f"-D{k}={v}" for k, v in var.items()]
    cmd = (["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-w", "-Wl,-Bsymbolic", f"-I{SRC}"] + defs
           + ["-o", out, driver, os.path.join(SRC, "mersenne_inline.c"), "-lm"])
    subprocess.run(cmd, check=True)
    return out


def available() -> bool:
    return os.path.exists(os.path.join(SRC, "hmc_patched.c")) or os.path.exists(os.path.join(REF_ROOT, "hmc.c"))


def build(sizes=None, variants=None) -> list[str]:
    """Generate (if the reference tree is present) and compile the oracle/_ref libraries."""
    if os.path.exists(os.path.join(REF_ROOT, "hmc.c")):
        generate()
        generate_vecops()
        generate_brute()
    elif not os.path.exists(os.path.join(SRC, "hmc_patched.c")):
        return []
    sizes = sizes or DEFAULT_SIZES
    variants = variants or [v for v in VARIANTS if not v.startswith("sample")]
    jobs = [(nt, nx, v) for (nt, nx) in sizes for v in variants]
    jobs += [(nt, nx, "sample_px") for (nt, nx) in SAMPLE_SIZES if (nt, nx) in sizes]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        libs = list(ex.map(lambda j: build_one(*j), jobs))
        if os.path.exists(os.path.join(VSRC, "vec_ops.c")):
            libs += list(ex.map(lambda j: build_vec_one(*j), VEC_SIZES))
        if os.path.exists(os.path.join(VSRC, "fermion_matrix.c")):
            libs += list(ex.map(lambda j: build_prop_one(*j), PROP_SIZES))
        if os.path.exists(os.path.join(VSRC, "full_determinant.c")):
            libs += list(ex.map(lambda j: build_det_one(*j), [(nt, nx, o) for (nt, nx) in DET_SIZES
                                                              for o in (False, True)]))
        if os.path.exists(os.path.join(BSRC, "thirring_brute.c")):
            libs.append(build_brute())
    return libs


if __name__ == "__main__":
    sizes = None
    if len(sys.argv) > 1:
        sizes = [tuple(int(v) for v in a.lower().split("x")) for a in sys.argv[1:]]
    for p in build(sizes):
        print(p)
