"""Generates the golden fixtures in tests/golden/ from the REFERENCE FDTD.

Runs the reference's own code, compiled from FDTDcalc/FDTDsplitfieldMetal.c
into oracle/_ref/libref_fdtd.so (oracle.build()), on seeded synthetic
structures: set_sigma -> remove_sigma -> set_address -> set_tau, then the
reference time loop (main :153-167) driving the reference main_calc with the
reference set_env envelope.  The coefficients fed to main_calc come from the
oracle port (the reference builds them inside main(), which is not callable);
they are pinned separately by the deck-level fixture below, where the stock
reference binary runs end to end.

The deck fixtures (tests/golden/decks/) are written by smatranem_gb300.decks
and run through the stock reference binary oracle/_ref/FDTD_ref; its stderr
(the |S|^2 report) is kept beside each deck.

Usage (needs the reference sources, i.e. runs only where they are mounted):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from smatranem_gb300 import workloads as W  # noqa: E402

# (name, L, seed, structure kwargs, iBTIin, time_period, nsteps)
CASES = [
    ("zpml_plain", (8, 7, 14, 3), 11, dict(pml=(0, 0, 3), pml_z_only=True), (3, 10, 5, 1), (1, 1, 3), 40),
    ("zpml_metal", (10, 9, 16, 3), 12, dict(pml=(0, 0, 3), pml_z_only=True, metals=0.06, lossy=0.05),
     (4, 11, 6, -2), (1, 1, 3), 12),
    ("allpml_metal", (12, 11, 13, 2), 13, dict(pml=(2, 2, 2), metals=0.05, lossy=0.05, iBc=(-1, 0, 1)),
     (4, 8, 6, 1), (1, 2, 4), 12),
    ("periodic_bc", (6, 9, 10, 2), 14, dict(pml=(0, 0, 2), pml_z_only=True, iBc=(1, -1, 0)), (3, 6, 4, 3),
     (1, 1, 2), 30),
]


def run_case(ref, port, name, L, seed, kw, iBTIin, tp, nsteps):
    s = W.random_structure(L, seed=seed, **kw)
    mu = np.ascontiguousarray(s.mu.reshape(-1))
    ep = np.ascontiguousarray(s.epsi.reshape(-1))
    sig = ref.set_sigma(L, mu, ep)
    m2, e2 = ref.remove_sigma(L, mu, ep, sig)
    cont, addr, ln = ref.set_address(L, sig, m2, e2)
    n2pi, iR, iI = ref.set_tau(s.omega, s.min_dt)
    Ah, Bh, Ae, Be = port.coefficients(L, ln, sig, m2, e2, cont, addr, iR, iI)
    n3 = L[0] * L[1] * L[2]
    pl = L[0] * L[1]
    H, E = W.random_fields(n3, ln, seed=seed + 100, scale=1e-3)
    Hinc, Einc = W.random_incident(pl, seed=seed + 200)
    H0, E0 = H.copy(), E.copy()
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    before = ref.exit_calls.value
    ref.time_loop(L, Ah, Bh, Ae, Be, s.iBc, H, E, iBTIin, Hinc, Einc, n2pi, tp, 0, nsteps, *mons, cont, addr)
    exits = ref.exit_calls.value - before
    env = np.array([[ref.set_env(n2pi, tp, jh, jt, jp) for jh in (0, 1) for jt in (0, n2pi // 3, n2pi - 1)]
                    for jp in range(tp[2])])
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"),
        L=np.array(L), seed=seed, iBc=np.array(s.iBc), iBTIin=np.array(iBTIin), time_period=np.array(tp),
        nsteps=nsteps, omega=s.omega, min_dt=s.min_dt, mu_in=mu, epsi_in=ep,
        sigma=sig, mu=m2, epsi=e2, cont=cont, addr=addr, lnotn=ln, n2pi=n2pi, invtau_R=iR, invtau_I=iI,
        Ah=Ah, Bh=Bh, Ae=Ae, Be=Be, H0=H0, E0=E0, Hinc=Hinc, Einc=Einc,
        H=H, E=E, HB=mons[0], EB=mons[1], HT=mons[2], ET=mons[3], ref_exits=exits, env=env)
    print(f"{name}: L={L} Lnotn={ln} classes={ {chr(k): int(np.sum(cont == k)) for k in np.unique(cont)} } "
          f"N_2pi={n2pi} steps={nsteps} exits={exits} max|H|={np.abs(H).max():.3e}")


# decks for the drop-in program: (name, L, seed, structure kwargs, deck kwargs)
DECKS = [
    ("deck_periodic", (3, 3, 12, 3), 41, dict(pml=(0, 0, 1), pml_z_only=True, iBc=(1, 1, 1)),
     dict(time_period=(1, 1, 3), inci_point="B2", inci_mode=1, targets=("B1", "T1"), nreal=(3, 2))),
    ("deck_lossy", (4, 3, 12, 3), 42, dict(pml=(0, 0, 1), pml_z_only=True, lossy=0.2, iBc=(-1, 0, 1)),
     dict(time_period=(1, 2, 4), inci_point="T0", inci_mode=-2, targets=("B1", "T1"), nreal=(2, 3))),
    # the top monitor plane lies in the z-PML: the reference aborts (:320)
    ("deck_pml_monitor", (3, 3, 12, 3), 43, dict(pml=(0, 0, 1), pml_z_only=True),
     dict(time_period=(1, 1, 2), inci_point="B2", inci_mode=1, targets=("B1", "T2"), nreal=(2, 2))),
]


def make_deck(name, L, seed, kw, dkw):
    """Write a deck with the repository's writer, run the stock reference FDTD
    binary on it, keep the deck and the reference's stderr."""
    import shutil
    import subprocess
    from smatranem_gb300 import decks
    root = os.path.join(HERE, "decks", name)
    shutil.rmtree(root, ignore_errors=True)
    s = W.random_structure(L, seed=seed, omega=decks.omega_of(1.55e-6, 1.0e7), **kw)
    decks.write_deck(root, s, seed=seed, **dkw)
    r = subprocess.run([oracle.REF_BIN, "input.txt"], cwd=root, capture_output=True, text=True)
    with open(os.path.join(root, "reference_stderr.txt"), "w") as f:
        f.write(r.stderr)
    with open(os.path.join(root, "reference_status.txt"), "w") as f:
        f.write(f"{r.returncode}\n")
    np.savez_compressed(os.path.join(root, "media.npz"), mu=s.mu.reshape(-1), epsi=s.epsi.reshape(-1),
                        min_dt=s.min_dt)
    print(f"{name}: " + r.stderr.strip().splitlines()[-1])


def make_mode_deck(name="deck_modes", L=(5, 4, 14, 4), seed=51):
    """A guide with a dielectric block beside the core, whose Mode / Xi files
    are the stock reference mode solver's (oracle/_ref/Mcalc_ref) for the two
    monitor layers; then the stock FDTD and the stock S-matrix program
    (oracle/_ref/Scalc_ref) run on it: the Mcalc -> FDTD / Scalc chains of
    the reference end to end.  The drop-ins check their outputs against
    reference_stderr.txt (FDTD, reading these files or solving the port modes
    itself) and reference_Smatrix.dat (Scalc)."""
    import shutil
    import subprocess
    from smatranem_gb300 import decks
    root = os.path.join(HERE, "decks", name)
    shutil.rmtree(root, ignore_errors=True)
    L0, L1, L2, L3 = L
    om = decks.omega_of(1.55e-6, 1.0e7)
    med = W.port_layer(L0, L1, core=(2, 2), eps_core=12.11, eps_clad=2.085, seed=seed, jitter=0.25)
    s = W.waveguide_structure(med, L0, L1, L2, L3, omega=om, pml_z=2)
    pl = L0 * L1
    ep = s.epsi.reshape(L2, pl, 3)
    for z in range(L3 + 1, L2 - L3 - 1):  # a dielectric block beside the core in the scatterer layers
        for j1 in range(0, 2):
            for j0 in range(3, 5):
                ep[z, j0 + L0 * j1, :] = 6.5
    decks.write_deck(root, s, seed=seed, time_period=(1, 2, 6), inci_point="B3", inci_mode=1,
                     targets=("B2", "T1"), nreal=(1, 1),
                     extra_lines=("\tinv_k0 = 1.00000000000000000000e-07 m",
                                  "\tMediumPara: wavelength= 1.55000000000000000000e-06 m, temperature= 25 degC",
                                  "\tSmatrix: both-ways = y, LAPACK solver = y"))
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
    r = subprocess.run([oracle.MCALC_BIN, "input.txt"], cwd=root, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"{name}: Mcalc failed\n{r.stderr}")
    r = subprocess.run([oracle.SCALC_BIN, "input.txt"], cwd=root, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"{name}: Scalc failed\n{r.stderr}")
    os.replace(os.path.join(root, "Data", "deck_Smatrix.dat"), os.path.join(root, "reference_Smatrix.dat"))
    r = subprocess.run([oracle.REF_BIN, "input.txt"], cwd=root, capture_output=True, text=True)
    with open(os.path.join(root, "reference_stderr.txt"), "w") as f:
        f.write(r.stderr)
    with open(os.path.join(root, "reference_status.txt"), "w") as f:
        f.write(f"{r.returncode}\n")
    np.savez_compressed(os.path.join(root, "media.npz"), mu=s.mu.reshape(-1), epsi=s.epsi.reshape(-1),
                        min_dt=s.min_dt, port_med=med)
    print(f"{name}: " + " | ".join(r.stderr.strip().splitlines()[-6:]))


def main():
    oracle.build(with_reference=True)
    ref, port = oracle.Oracle("reference"), oracle.Oracle("port")
    for case in CASES:
        run_case(ref, port, *case)
    for deck in DECKS:
        make_deck(*deck)
    make_mode_deck()


if __name__ == "__main__":
    if sys.argv[1:] == ["modes"]:
        oracle.build(with_reference=True)
        make_mode_deck()
    else:
        main()
