"""Writing FDTD input decks in the formats of the SMatrAnEM mesher chain.

A deck is input.txt plus <prefix>_Med{B<k>,<k>,T<k>}.dat (one per z layer),
<prefix>_{b,t}Mode.dat and <prefix>_{b,t}Xi.dat -- the files the reference
FDTD reads (FDTDcalc/FDTDsplitfieldMetal.c main :44-99).  Line formats follow
the writers of the chain: Med3DSi (header lines, Medium3DSi/Med3DSi.c:222-225),
PMLgen (the "PML num / min Dt^2" header tail, PMLset/PMLcalc.c:331), Mcalc (Mode
and Xi files, ModeCalc/Mcalc.c:186-229).  Values are synthetic (seeded); the Xi
matrix is a random matrix whose E rows are real, as the reference requires of an
incident column (:503).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import fdtd
from .workloads import Structure


def omega_of(wavelength_m: float, k0: float) -> float:
    """omega = 2 pi / (lambda k0) evaluated exactly as the FDTD does (long double
    2 pi, input_Lf :740), so the Mode file's Omega line passes its == check."""
    lib = fdtd.lib()
    f = lib.smat_omega
    f.restype = C.c_double
    f.argtypes = [C.c_double, C.c_double]
    return float(f(wavelength_m, k0))


def layer_name(prefix, L, z):
    L2, L3 = L[2], L[3]
    if z < L3:
        return f"{prefix}_MedB{z}.dat"
    if z < L2 - L3:
        return f"{prefix}_Med{z - L3}.dat"
    return f"{prefix}_MedT{z - (L2 - L3)}.dat"


def write_layer(path: str, med, L, *, wavelength_m=1.55e-6, k0=1.0e7, u2=0.0, min_sqdt=1.0, factors=None):
    """One Med layer file as the mesher chain writes it: a comment line, the
    wavelength / k_0 / lattice header (Medium3DSi/Med3DSi.c:222-227 with
    PMLgen's "PML num / min Dt^2" tail, PMLset/PMLcalc.c:331), then
    2*L0*L1 lines "l m j2 Re Im Re Im Re Im fx fx fx".  med is (6, L0*L1)
    complex in the file's column order (j2 = 0: mu00, mu11, eps22; j2 = 1:
    eps11, eps00, mu22); factors (same shape, real) default to 1."""
    L0, L1 = L[0], L[1]
    L2 = L[2] if len(L) > 2 else 1
    L3 = L[3] if len(L) > 3 else 0
    med = np.asarray(med, np.complex128).reshape(6, L0 * L1)
    fx = np.ones((6, L0 * L1)) if factors is None else np.asarray(factors, np.float64).reshape(6, L0 * L1)
    lines = ["# Created by smatranem_gb300.decks",
             f"# wavelength [m] = {wavelength_m:.20e}, temp. [K] = {298.15:.20e}, sinc_rad = 0",
             f"# k_0 * u_2  = {u2:.20e} ; {u2 + 0.05:.20e} ; {u2 + 0.1:.20e}, k_0[m^-1] = {k0:.20e}",
             f"# l < {L0}, m < {L1}, n + 2*outer < {L2}, media_no < 2, outer = {L3}, PML num = 1, "
             f"min Dt^2 = {min_sqdt:.20e}",
             "# l m 0 mu_u mu_v ep_w",
             "# l m 1 ep_v ep_u mu_w"]
    for j1 in range(L1):
        for j0 in range(L0):
            p = j0 + L0 * j1
            for j2 in (0, 1):
                vals = med[3 * j2:3 * j2 + 3, p]
                nums = " ".join(f"{v.real:.20e} {v.imag:.20e}" for v in vals)
                fs = " ".join(f"{x:.20e}" for x in fx[3 * j2:3 * j2 + 3, p])
                lines.append(f"{j0} {j1} {j2} {nums} {fs}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_deck(root: str, s: Structure, *, prefix="Data/deck", wavelength_m=1.55e-6, k0=1.0e7, time_period=(1, 1, 3),
               inci_point="B2", inci_mode=1, targets=("B1", "T1"), nreal=(3, 3), seed=0, extra_lines=()):
    """Write a deck for structure s under directory root; returns input.txt's path."""
    L = s.L
    L0, L1, L2, L3 = L
    pl = L0 * L1
    os.makedirs(os.path.join(root, os.path.dirname(prefix)), exist_ok=True)
    pfx = os.path.join(root, prefix)
    omega = omega_of(wavelength_m, k0)
    sq = s.min_dt ** 2  # the header holds min_Dt squared; the FDTD takes its square root
    mu = s.mu.reshape(L2, pl, 3)
    ep = s.epsi.reshape(L2, pl, 3)
    for z in range(L2):
        m, e = mu[z], ep[z]
        med = np.stack([m[:, 0], m[:, 1], e[:, 2], e[:, 1], e[:, 0], m[:, 2]])
        write_layer(layer_name(pfx, L, z), med, L, wavelength_m=wavelength_m, k0=k0, u2=z * 0.1, min_sqdt=sq)
    rng = np.random.default_rng(seed)
    NA = 2 * pl
    for side, nr in zip("bt", nreal):
        with open(f"{pfx}_{side}Mode.dat", "w") as f:
            f.write(f"# This file          : ' {pfx}_{side}Mode.dat '\n")
            f.write(f"# Omega              : k/k_0 = {omega:.20e}\n")
            f.write(f"# Lattice numbers    : L0 = {L0}, L1 = {L1}\n")
            f.write(f"# Eigen-value info.  : real num./2 = {nr}, comp. num./2 = {NA - nr}\n")
            for j in range(NA):
                a, b = rng.standard_normal(2)
                c, d = rng.standard_normal(2)
                f.write(f"theta[{j}]=({a:.20e}, {b:.20e}), theta[{j + NA}]=({c:.20e}, {d:.20e})\n")
        xi = rng.standard_normal((2 * NA, 2 * NA)) + 1j * rng.standard_normal((2 * NA, 2 * NA))
        xi[NA:, :] = xi[NA:, :].real  # real E rows: any column may be an incident one
        xi /= np.sqrt(2 * NA)
        with open(f"{pfx}_{side}Xi.dat", "w") as f:
            f.write(f"# This file      : ' {pfx}_{side}Xi.dat '\n")
            f.write(f"# Reference file : ' {pfx}_{side}Mode.dat '\n")
            for j in range(NA):
                f.write(f"ReXi[{j}] ImXi[{j}] ReXi[{j + NA}] ImXi[{j + NA}]\n")
                for r in range(2 * NA):
                    a, b = xi[r, j], xi[r, j + NA]
                    f.write(f"{a.real:.20e} {a.imag:.20e} {b.real:.20e} {b.imag:.20e}\n")
    path = os.path.join(root, "input.txt")
    bc = s.iBc
    with open(path, "w") as f:
        f.write(f"\tPrefix = ./{prefix}\n")
        f.write(f"\tBoundaryCondition: B0 = {bc[0]}, B1 = {bc[1]}, B2 = {bc[2]}\n")
        f.write(f"\tModeP: Xi output = y, Internal precision = D, 1st = {targets[0]}, 2nd = {targets[1]}\n")
        f.write(f"\tFDTD: ramp-period = {time_period[0]}, cw-period = {time_period[1]}, "
                f"stop-period = {time_period[2]}, incident-point = {inci_point}, incident-mode = {inci_mode:+d}, "
                f"Dt_factor = 1., stable_factor = 2.\n")
        for line in extra_lines:
            f.write(line + "\n")
    return path


def _open(input_txt: str):
    lib = fdtd.lib()
    lib.smat_deck_load.argtypes = [C.c_char_p, C.c_void_p]
    lib.smat_deck_free.argtypes = [C.c_void_p]
    lib.smat_deck_info.argtypes = [C.c_void_p] * 9
    lib.smat_deck_arrays.argtypes = [C.c_void_p] * 5
    lib.smat_deck_from_cache.argtypes = [C.c_void_p]
    lib.smat_deck_smatrix.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    h = C.c_void_p()
    # the Prefix of input.txt is relative to the directory the FDTD runs in
    cwd = os.getcwd()
    os.chdir(os.path.dirname(os.path.abspath(input_txt)))
    try:
        rc = lib.smat_deck_load(os.path.basename(input_txt).encode(), C.byref(h))
    finally:
        os.chdir(cwd)
    if rc != 0:
        raise fdtd.FdtdError(rc, lib.smat_last_error().decode())
    return lib, h


def smatrix(input_txt: str, which: int, HB, EB):
    """S_calc of the deck's bottom (which = 0) or top (1) plane for monitor
    planes HB, EB (2*L0*L1 complex each): 2*N_real complex values."""
    lib, h = _open(input_txt)
    try:
        nr = (C.c_int * 2)()
        lib.smat_deck_info(h, None, None, None, None, None, None, None, nr)
        S = np.zeros(2 * nr[which], np.complex128)
        HB = np.ascontiguousarray(HB, np.complex128)
        EB = np.ascontiguousarray(EB, np.complex128)
        rc = lib.smat_deck_smatrix(h, which, HB.ctypes.data_as(C.c_void_p), EB.ctypes.data_as(C.c_void_p),
                                   S.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise fdtd.FdtdError(rc, lib.smat_last_error().decode())
        return S
    finally:
        lib.smat_deck_free(h)


def load(input_txt: str):
    """Read a deck through the library: a dict of its numbers and arrays."""
    lib, h = _open(input_txt)
    try:
        L = (C.c_int * 4)()
        bti = (C.c_int * 4)()
        bc = (C.c_int * 3)()
        tp = (C.c_int * 3)()
        om, mdt, dtf = C.c_double(), C.c_double(), C.c_double()
        nr = (C.c_int * 2)()
        lib.smat_deck_info(h, L, bti, bc, tp, C.byref(om), C.byref(mdt), C.byref(dtf), nr)
        n3, pl = L[0] * L[1] * L[2], L[0] * L[1]
        mu = np.zeros(3 * n3, np.complex128)
        ep = np.zeros(3 * n3, np.complex128)
        Hi = np.zeros(2 * pl, np.complex128)
        Ei = np.zeros(2 * pl, np.complex128)
        lib.smat_deck_arrays(h, mu.ctypes.data_as(C.c_void_p), ep.ctypes.data_as(C.c_void_p),
                             Hi.ctypes.data_as(C.c_void_p), Ei.ctypes.data_as(C.c_void_p))
        return dict(L=tuple(L), iBTIin=tuple(bti), iBc=tuple(bc), time_period=tuple(tp), omega=om.value,
                    min_dt=mdt.value, dt_factor=dtf.value, nreal=tuple(nr), mu=mu, epsi=ep, Hinc=Hi, Einc=Ei,
                    from_cache=bool(lib.smat_deck_from_cache(h)))
    finally:
        lib.smat_deck_free(h)
