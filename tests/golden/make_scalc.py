"""Generates tests/golden/scalc_*.npz from the REFERENCE S-matrix program.

For each case: write a deck (smatranem_gb300.decks), compute its port modes
with the stock Mcalc (oracle/_ref/Mcalc_ref), then run the stock Scalc
(oracle/_ref/Scalc_ref, Smat/Scalc.c with zgesv/zgemm from scipy's OpenBLAS,
one thread) in both directions, and keep its inputs as arrays (the Med values
of layers iB..iT, the full Xi matrices of both port layers, N_real, omega)
with the S matrix it wrote to <prefix>_Smatrix.dat.

Usage (needs the reference sources, i.e. runs only where they are mounted):
    python tests/golden/make_scalc.py
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

# (name, (L0, L1, L2, L3), BoundC, defect (j0 range, j1 range, eps) or None, seed, ModeP targets);
# the targets must lie outside the 2-layer z-PML (Mcalc rejects a lossy layer)
CASES = [
    ("scalc_straight", (5, 4, 14, 4), (0, 0, 0), None, 51, ("B2", "T1")),
    ("scalc_defect", (6, 5, 12, 3), (1, 0, 0), ((1, 4), (0, 2), 6.5), 61, ("B2", "T0")),
]


def read_full_xi(path, NA):
    Xi = np.zeros((2 * NA, 2 * NA), np.complex128)
    with open(path) as f:
        f.readline()
        f.readline()
        for j in range(NA):
            f.readline()
            a = np.array([f.readline().split() for _ in range(2 * NA)], np.float64)
            Xi[:, j] = a[:, 0] + 1j * a[:, 1]
            Xi[:, j + NA] = a[:, 2] + 1j * a[:, 3]
    return Xi


def read_smatrix(path):
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#"):
                continue
            m, n, re_, im_, _ = line.split()
            rows.append((int(m), int(n), float(re_) + 1j * float(im_)))
    N = max(r[0] for r in rows) + 1
    S = np.zeros((N, N), np.complex128)
    for m, n, v in rows:
        S[m, n] = v
    return S


def run_case(name, L, bc, defect, seed, targets):
    L0, L1, L2, L3 = L
    om = decks.omega_of(1.55e-6, 1.0e7)
    med = W.port_layer(L0, L1, core=(2, 2), eps_core=12.11, eps_clad=2.085, seed=seed, jitter=0.25)
    s = W.waveguide_structure(med, L0, L1, L2, L3, omega=om, pml_z=2, iBc=bc)
    if defect:
        (a0, a1), (b0, b1), eps = defect
        pl = L0 * L1
        ep = s.epsi.reshape(L2, pl, 3)
        for z in range(L3, L2 - L3):
            for j1 in range(b0, b1):
                for j0 in range(a0, a1):
                    ep[z, j0 + L0 * j1, :] = eps
    NA = 2 * L0 * L1
    with tempfile.TemporaryDirectory() as root:
        decks.write_deck(root, s, seed=seed, time_period=(1, 2, 6), inci_point="B3", inci_mode=1,
                         targets=targets, nreal=(1, 1),
                         extra_lines=("\tinv_k0 = 1.00000000000000000000e-07 m",
                                      "\tMediumPara: wavelength= 1.55000000000000000000e-06 m, temperature= 25 degC",
                                      "\tSmatrix: both-ways = y, LAPACK solver = y"))
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
        for exe in (oracle.MCALC_BIN, oracle.SCALC_BIN):
            r = subprocess.run([exe, "input.txt"], cwd=root, capture_output=True, text=True, env=env)
            if r.returncode != 0:
                raise RuntimeError(f"{name}: {os.path.basename(exe)} failed\n{r.stderr[-2000:]}")
        pfx = os.path.join(root, "Data", "deck")
        nreal = []
        for side in "bt":
            txt = open(f"{pfx}_{side}Mode.dat").read()
            nreal.append(int(re.search(r"real num\./2 = (\d+)", txt).group(1)))
        XiB = read_full_xi(f"{pfx}_bXi.dat", NA)
        XiT = read_full_xi(f"{pfx}_tXi.dat", NA)
        S = read_smatrix(f"{pfx}_Smatrix.dat")
        resid = re.search(r"unitarity = (\S+), transpose = (\S+)", open(f"{pfx}_Smatrix.dat").read())
    iB, iT = int(targets[0][1:]), L2 - L3 + int(targets[1][1:])
    pl = L0 * L1
    mu = s.mu.reshape(L2, pl, 3)
    ep = s.epsi.reshape(L2, pl, 3)
    meds = np.stack([np.stack([mu[z][:, 0], mu[z][:, 1], ep[z][:, 2], ep[z][:, 1], ep[z][:, 0], mu[z][:, 2]])
                     for z in range(iB, iT + 1)])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), L=np.array(L), bc=np.array(bc[:2]), omega=om,
                        iB=iB, iT=iT, meds=meds, XiB=XiB, XiT=XiT, nreal=np.array(nreal), S=S,
                        unitarity=float(resid.group(1)), transpose=float(resid.group(2)))
    print(f"{name}: L={L} bc={bc[:2]} N_real={nreal} |S|^2=\n{np.round(np.abs(S) ** 2, 6)}")


if __name__ == "__main__":
    oracle.build()
    if not (oracle.mcalc_available() and oracle.scalc_available()):
        sys.exit("oracle/_ref/Mcalc_ref or Scalc_ref missing (needs the reference sources and scipy's OpenBLAS)")
    for case in CASES:
        run_case(*case)
