"""The drop-in `hmc` program (reference-signature layer libthirring_hmc.so on the
CUDA library) reproduces the reference hmc.c run: same stdin parameters, same
random stream, same printed lines, checked against the CPU oracle replaying
hmc.c's main (seed, 543210 warm-up draws, 100 pure-gauge sweeps, then
update_gauge and measure per loop)."""
import os
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HMC = os.path.join(ROOT, "bin", "hmc")


def run_hmc(stdin: str, nt: int, nx: int, extra_env=None) -> str:
    env = dict(os.environ, HMC_NT=str(nt), HMC_NX=str(nx))
    env.update(extra_env or {})
    r = subprocess.run([HMC], input=stdin, text=True, capture_output=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def oracle_replay(oracle_lib, nt, nx, n_loops, n_measure, m, g, mu, seed, bc_x=-1):
    o = oracle_lib.Oracle(nt, nx, m, g, mu, -1, bc_x)
    mt = oracle_lib.MT(seed, 543210)
    A = np.zeros((nt, nx, 2))
    for _ in range(100):
        o.puregauge_sweep(A, mt)
    out = []
    for i in range(1, n_loops + 1):
        s, st, _ = o.trajectory(A, mt, 10, 1.0, 1, True)
        out.append(("traj", s))
        if i % n_measure == 0:
            mt.gaussian_field(nt, nx)             # test_conjugate's vector (hmc.c:764)
            mag = A.sum() / (nt * nx)
            im = 0.0
            for _ in range(20):                   # fermion_phase, hmc.c:794-815
                c, _ = mt.gaussian_field(nt, nx)
                mdc = o.Mdag(A, c)
                im += float((c.real * mdc.imag - c.imag * mdc.real).sum())
            out.append(("measure", (mag, im / 20)))
    return out


def close(a: float, b: float, rel=2e-5, abs_=1e-9) -> bool:
    return abs(a - b) <= rel * abs(b) + abs_


@pytest.mark.parametrize("nt,nx,params", [(8, 8, "3 1 0.5 0.5 0.0 12345"), (6, 4, "2 2 0.4 1.0 0.2 77")])
def test_hmc_program_matches_oracle(oracle_lib, nt, nx, params):
    n_loops, n_measure, m, g, mu, seed = params.split()
    text = run_hmc(params + "\n", nt, nx)
    assert f"( {nt} , {nx} ) lattice" in text
    ends = [tuple(float(v) for v in re.findall(r"[-+0-9.e]+", line.split("dS", 1)[1]))
            for line in text.splitlines() if line.startswith("HMC End")]
    acc = [line.strip() for line in text.splitlines() if line.startswith("HMC ACC") or line.startswith("HMC REJ")]
    mags = [float(line.split()[1]) for line in text.splitlines() if line.startswith("Magnetisation")]
    phases = [float(line.split()[1]) for line in text.splitlines() if line.startswith("Phase")]
    want = oracle_replay(oracle_lib, nt, nx, int(n_loops), int(n_measure), float(m), float(g), float(mu), int(seed))
    trajs = [s for k, s in want if k == "traj"]
    meas = [v for k, v in want if k == "measure"]
    assert len(ends) == len(trajs) == len(acc)
    for got, s, a in zip(ends, trajs, acc):
        assert close(got[0], s[0], abs_=1e-6), (got, s[0])        # dS, printed with %g
        assert close(got[1], s[5]) and close(got[2], s[6])         # Sg, Smdm at the end
        assert a == ("HMC ACCEPTED" if s[9] else "HMC REJECTED")
    assert len(mags) == len(meas) == len(phases)
    for mg, ph, (wm, wp) in zip(mags, phases, meas):
        assert close(mg, wm, abs_=1e-6) and close(ph, wp, abs_=1e-5)


def test_hmc_program_jsonl_log(tmp_path):
    """HMC_JSONL appends one JSON line per trajectory; with HMC_VERBOSE=1 the
    printed dS lines carry every digit and agree with the log exactly."""
    import json
    log = tmp_path / "traj.jsonl"
    out = run_hmc("3 3 0.5 0.5 0.0 4242", 8, 8, {"HMC_JSONL": str(log), "HMC_VERBOSE": "1"})
    rows = [json.loads(line) for line in log.read_text().splitlines()]
    assert [r["trajectory"] for r in rows] == [1, 2, 3]
    printed = [float(x) for x in re.findall(r"HMC End, dS ([-+0-9.eE]+),", out)]
    decisions = re.findall(r"HMC (ACCEPTED|REJECTED)", out)
    assert printed == [r["dH"] for r in rows]
    assert decisions == ["ACCEPTED" if r["accepted"] else "REJECTED" for r in rows]
    assert all(r["cg_solves"] == 11 and r["cg_iterations"] > 0 and r["cg_ms"] > 0 for r in rows)


DENSE_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include <complex.h>
#include "thirring_hmc.h"
/* argv: nt nx m mu A.bin out.bin -- A double[nt][nx][2]; out: M as hmc.c stores
 * it (V*V complex, M[i + j*V]) then det M (re, im) */
int main(int argc, char** argv) {
  if (argc != 7) return 2;
  int nt = atoi(argv[1]), nx = atoi(argv[2]);
  m = atof(argv[3]);
  mu = atof(argv[4]);
  g = 0.5;
  thirring_hmc_set_lattice(nt, nx);
  FILE* f = fopen(argv[5], "rb");
  if (!f) return 3;
  A = malloc(nt * sizeof(double**));
  for (int t = 0; t < nt; t++) {
    A[t] = malloc((nx + 1) * sizeof(double*));
    for (int x = 0; x < nx + 1; x++) {
      A[t][x] = calloc(2, sizeof(double));
      if (x < nx && fread(A[t][x], sizeof(double), 2, f) != 2) return 4;
    }
  }
  fclose(f);
  int V = nt * nx;
  _Complex double* M = malloc((size_t)V * V * sizeof(_Complex double));
  fermion_matrix(M);
  _Complex double d = determinant();
  double dd[2] = {creal(d), cimag(d)};
  FILE* o = fopen(argv[6], "wb");
  fwrite(M, sizeof(_Complex double), (size_t)V * V, o);
  fwrite(dd, sizeof(double), 2, o);
  fclose(o);
  return 0;
}
"""


@pytest.mark.parametrize("name", ["det_4x4_apx", "det_4x4_px", "det_6x4_apx"])
def test_compat_fermion_matrix_and_determinant(tmp_path, name):
    """fermion_matrix(M) and determinant() of the reference-signature layer
    (hmc.c:269-336, for the global A) against the reference's own dense matrix
    and its log-determinant (tests/golden/det_*), called from plain C."""
    from helpers import golden
    d = golden(name)
    nt, nx = int(d["nt"]), int(d["nx"])
    src = tmp_path / "dense.c"
    src.write_text(DENSE_PROGRAM)
    lib_dir = os.path.join(ROOT, "thirring2d_gb300")
    exe = tmp_path / "dense"
    r = subprocess.run(["gcc", "-std=c99", "-O1", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(exe),
                        f"-L{lib_dir}", "-lthirring_hmc", f"-Wl,-rpath,{lib_dir}", "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    np.ascontiguousarray(d["A"], dtype=np.float64).tofile(tmp_path / "A.bin")
    env = dict(os.environ, HMC_BC_X="periodic" if int(d["bc_x"]) == 1 else "antiperiodic")
    r = subprocess.run([str(exe), str(nt), str(nx), repr(float(d["m"])), repr(float(d["mu"])),
                        str(tmp_path / "A.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       env=env, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
    V = nt * nx
    M = (out[:2 * V * V:2] + 1j * out[1:2 * V * V:2]).reshape(V, V).T   # hmc.c's M[i + j*V]
    assert np.abs(M - d["M"]).max() < 1e-14
    det = out[2 * V * V] + 1j * out[2 * V * V + 1]
    want = np.exp(float(d["logabsdet"])) * complex(d["phase"])
    assert abs(det - want) <= 1e-10 * abs(want)
