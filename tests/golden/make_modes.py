"""Generates tests/golden/modes_*.npz from the REFERENCE port-mode solver.

Writes one Med layer and an input.txt per case, runs the stock Mcalc
(ModeCalc/Mcalc.c compiled into oracle/_ref/Mcalc_ref by oracle.build(),
with LAPACK from scipy's bundled OpenBLAS, one thread) and keeps what it
wrote: every theta of the _bMode.dat file, the leading Xi columns (forward
and backward) of _bXi.dat, N_real, and the diagnostics it prints.  The
layers are seeded synthetic cross-sections from
smatranem_gb300.workloads.port_layer.

Usage (needs the reference sources, i.e. runs only where they are mounted):
    python tests/golden/make_modes.py
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from smatranem_gb300 import decks, workloads as W  # noqa: E402

WAVELENGTH = 1.55e-6
K0 = 1.0e7          # 1/k0 = 100 nm per unit cell
KEEP = 12           # leading Xi columns kept per direction

# (name, L0, L1, BoundC, port_layer kwargs)
CASES = [
    ("modes_strip_pec", 12, 10, (0, 0), dict(core=(4, 3), eps_core=12.11, eps_clad=2.085, seed=1)),
    ("modes_rib_mixed", 11, 9, (1, -1), dict(core=(5, 2), eps_core=12.11, eps_clad=2.085, seed=2, jitter=0.3)),
    ("modes_uniform_periodic", 6, 6, (1, 1), dict(core=(0, 0), eps_core=2.085, eps_clad=2.085, seed=3)),
    ("modes_metric_pec", 10, 8, (0, 0), dict(core=(3, 3), eps_core=12.11, eps_clad=1.0, seed=4, metric=0.2)),
]
# A lossy port layer is not a case: the reference exits in sortXi's final check
# (Mcalc.c:620-626) for any complex mode whose theta has a real part, so the
# reference mode solver serves lossless port media only.


def read_mode_file(path, N):
    nr = None
    theta = np.zeros(2 * N, np.complex128)
    info = {}
    pat = re.compile(r"theta\[(\d+)\]=\(([^,]+), ([^)]+)\), theta\[(\d+)\]=\(([^,]+), ([^)]+)\)")
    with open(path) as f:
        for line in f:
            if line.startswith("# Eigen-value"):
                nr = int(re.search(r"real num\./2 = (\d+)", line).group(1))
            elif line.startswith("# Check of solutions"):
                info["norm"] = float(line.split("=")[-1])
            elif line.startswith("# Check of bi-ortho"):
                info["check"] = float(line.split("=")[-1])
            elif line.startswith("# Matrix info"):
                info["real_matrix"] = "real" in line.split(":")[1] and "complex" not in line
            m = pat.match(line)
            if m:
                a, b = int(m.group(1)), int(m.group(4))
                theta[a] = complex(float(m.group(2)), float(m.group(3)))
                theta[b] = complex(float(m.group(5)), float(m.group(6)))
    return nr, theta, info


def read_xi_file(path, N, keep):
    fwd = np.zeros((2 * N, keep), np.complex128)
    bwd = np.zeros((2 * N, keep), np.complex128)
    with open(path) as f:
        f.readline()
        f.readline()
        for j in range(N):
            f.readline()
            rows = [f.readline() for _ in range(2 * N)]
            if j < keep:
                a = np.array([r.split() for r in rows], np.float64)
                fwd[:, j] = a[:, 0] + 1j * a[:, 1]
                bwd[:, j] = a[:, 2] + 1j * a[:, 3]
    return fwd, bwd


def run_case(name, L0, L1, bc, kw):
    med = W.port_layer(L0, L1, **kw)
    N = 2 * L0 * L1
    keep = min(KEEP, N)
    with tempfile.TemporaryDirectory() as tmp:
        os.makedirs(os.path.join(tmp, "Data"))
        decks.write_layer(os.path.join(tmp, "Data", "port_MedB1.dat"), med, (L0, L1), wavelength_m=WAVELENGTH, k0=K0)
        with open(os.path.join(tmp, "input.txt"), "w") as f:
            f.write(f"\tinv_k0 = {1.0 / K0:.20e} m\n")
            f.write(f"\tMediumPara: wavelength= {WAVELENGTH:.20e} m, temperature= 25 degC\n")
            f.write("\tPrefix = ./Data/port\n")
            f.write(f"\tBoundaryCondition: B0 = {bc[0]}, B1 = {bc[1]}, B2 = 0\n")
            f.write("\tModeP: Xi output = y, Internal precision = D, 1st = B1, 2nd = B1\n")
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
        r = subprocess.run([oracle.MCALC_BIN, "input.txt"], cwd=tmp, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{name}: Mcalc failed\n{r.stderr}")
        nr, theta, info = read_mode_file(os.path.join(tmp, "Data", "port_bMode.dat"), N)
        fwd, bwd = read_xi_file(os.path.join(tmp, "Data", "port_bXi.dat"), N, keep)
    degen = [tuple(int(x) for x in m.groups()) for m in
             re.finditer(r"theta_m\[(\d+)\]-theta_m\[(\d+)\]\)/", r.stderr)]
    omega = decks.omega_of(WAVELENGTH, K0)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), L0=L0, L1=L1, bc=np.array(bc), omega=omega, med=med,
                        theta=theta, num_real=nr, xi_fwd=fwd, xi_bwd=bwd, norm=info["norm"], check=info["check"],
                        real_matrix=info["real_matrix"], degenerate=np.array(degen, np.int64).reshape(-1, 2))
    print(f"{name}: L={L0}x{L1} bc={bc} N_real={nr} real={info['real_matrix']} check={info['check']:.3e} "
          f"theta0={theta[0]:.6f} degenerate pairs={len(degen)}")


if __name__ == "__main__":
    oracle.build()
    if not oracle.mcalc_available():
        sys.exit("oracle/_ref/Mcalc_ref is missing (needs the reference sources and scipy's OpenBLAS)")
    for case in CASES:
        run_case(*case)
