"""CPU restatement of the reference S-matrix program -- TEST INFRASTRUCTURE ONLY.

Follows Smat/Scalc.c: the frequency-domain layer transfer from one port layer
to the other (initial_calc :183-223, scattering_calc :227-261, final_calc
:269-306), the elimination step inv_process (:316-400, its zgesv branch) and
the assembly of the S matrix (Smat_calc :144-172).  Dense numpy / LAPACK
(scipy.linalg.solve is zgesv), for cross-sections of a few hundred unknowns.
Inputs are arrays instead of files: the per-layer Med values (as set_V reads
them) and the full Xi matrices of the two port layers (as Mcalc writes them:
column j forward, column j + NA backward).  Pinned against the stock Scalc
(oracle/_ref/Scalc_ref) by tests/golden/make_scalc.py.
"""
from __future__ import annotations

import numpy as np

from . import mode_oracle as MO


def set_Phi(Xi, iway):
    """set_Phi (:521-551): iway = 1 keeps Xi; iway = -1 rotates the rows by
    half and exchanges the forward and backward halves of the columns."""
    NA = Xi.shape[0] // 2
    if iway == 1:
        return Xi.copy()
    P = np.empty_like(Xi)
    rot = np.roll(np.arange(2 * NA), NA)  # row r of the file goes to (r + NA) % 2NA
    P[rot, :NA] = Xi[:, NA:]
    P[rot, NA:] = Xi[:, :NA]
    return P


def set_tilPhi(Xi, iway, Nimag):
    """set_tilPhi (:555-595): the dual columns (makePsi's pairing) for the
    first Nimag (real) modes, the complex-mode pairing for the rest."""
    NA = Xi.shape[0] // 2
    T = np.empty_like(Xi)
    rot = np.roll(np.arange(2 * NA), NA)
    first, second = Xi[:, :NA], Xi[:, NA:]
    real = np.arange(NA) < Nimag
    if iway == 1:
        T[np.ix_(rot, np.flatnonzero(real))] = first[:, real]
        T[np.ix_(rot, NA + np.flatnonzero(real))] = -second[:, real]
        T[np.ix_(rot, NA + np.flatnonzero(~real))] = first[:, ~real]
        T[np.ix_(rot, np.flatnonzero(~real))] = second[:, ~real]
    else:
        T[:, np.flatnonzero(real)] = -second[:, real]
        T[:, NA + np.flatnonzero(real)] = first[:, real]
        T[:, np.flatnonzero(~real)] = first[:, ~real]
        T[:, NA + np.flatnonzero(~real)] = second[:, ~real]
    return T


class _State:
    """F01 ((Noffset+NA) x Noffset), B01 ((Noffset+NA) x NA), F2 (NA x Noffset), B2 (NA x NA)."""

    def __init__(self, NA, Noffset):
        self.NA, self.No = NA, Noffset
        self.F01 = np.zeros((Noffset + NA, Noffset), np.complex128)
        self.B01 = np.zeros((Noffset + NA, NA), np.complex128)
        self.F2 = np.zeros((NA, Noffset), np.complex128)
        self.B2 = np.zeros((NA, NA), np.complex128)

    def inv_process(self):
        """:316-400 (zgesv branch): B01 <- B01 B2^{-1}, F01 <- F01 - B01 F2,
        then F2 = 0, B2 = 1."""
        import scipy.linalg as sl
        self.B01 = sl.solve(self.B2.T, self.B01.T, check_finite=False).T
        self.F01 = self.F01 - self.B01 @ self.F2
        self.F2[:] = 0.0
        self.B2 = np.eye(self.NA, dtype=np.complex128)

    def shift(self):
        """move the field rows of F01 into F2 (the next constraint)"""
        No = self.No
        self.F2 = self.F01[No:, :].copy()
        self.F01[No:, :] = 0.0

    def step(self, M, iway):
        """B2 <- field rows of B01 + i*iway*M; the field rows of B01 become 1;
        eliminate (the half-layer transfer of :207-221, :241-257, :286-296)"""
        No = self.No
        self.B2 = self.B01[No:, :] + (1j * float(iway)) * M
        self.B01[No:, :] = 0.0
        self.B01[No + np.arange(self.NA), np.arange(self.NA)] = 1.0
        self.inv_process()


def set_V(med, omega):
    """Scalc's set_V (:838-880): like Mcalc's, but rows 2 and 5 inverted as
    conj(z)/|z|^2 (:873-876)."""
    V = np.array(med, dtype=np.complex128, copy=True) * omega
    for r in (2, 5):
        z = V[r]
        V[r] = np.conj(z) / (z.real * z.real + z.imag * z.imag)
    return V, int(np.count_nonzero(V.imag != 0.0))


def _matrices(med, omega, L0, L1, bc):
    V, comp = set_V(med, omega)
    maa, mbb = MO.set_M(bc, L0, L1, V)
    return maa, mbb, comp


def one_way(iway, meds, omega, L0, L1, bc, Xi_start, Xi_end, Noffset, Nimag):
    """One direction of main :74-94: meds are the Med values of layers istart,
    istart + iway, ..., iend (in that order)."""
    NA = 2 * L0 * L1
    st = _State(NA, Noffset)
    # set_iniMat :407-458
    Phi = set_Phi(Xi_start, iway)
    st.B01[np.arange(Noffset), np.arange(Noffset)] = 1.0
    st.F01[Noffset:, :] = Phi[:NA, :Noffset]
    st.F2[:, :] = Phi[NA:, :Noffset]
    st.B01[Noffset:, :] = Phi[:NA, NA:]
    st.B2[:, :] = Phi[NA:, NA:]
    st.inv_process()
    # initial_calc :192-221
    st.shift()
    maa, mbb, comp = _matrices(meds[0], omega, L0, L1, bc)
    if comp != 0:
        raise ValueError("V is not real in initial_calc")
    st.step(mbb if iway > 0 else maa, iway)
    # scattering_calc :227-261 for the layers in between
    for med in meds[1:-1]:
        maa, mbb, _ = _matrices(med, omega, L0, L1, bc)
        for sub in range(2):
            st.shift()
            i_shift = ((1 - iway) // 2 + sub) % 2
            st.step((maa, mbb)[i_shift], iway)
    # final_calc :269-306
    st.shift()
    maa, mbb, comp = _matrices(meds[-1], omega, L0, L1, bc)
    if comp != 0:
        raise ValueError("V is not real in final_calc")
    st.step(maa if iway > 0 else mbb, iway)
    # set_finMat :461-517
    tilPhi = set_tilPhi(Xi_end, iway, Nimag)
    FB = np.zeros((2 * NA, Noffset + NA), np.complex128)
    FB[:NA, :Noffset] = st.F01[Noffset:, :]
    FB[NA:, :Noffset] = st.F2
    FB[:NA, Noffset:] = st.B01[Noffset:, :]
    FB[NA:, Noffset:] = st.B2
    Cm = tilPhi.conj().T @ FB
    st.F01[Noffset:, :] = Cm[:NA, :Noffset]
    st.F2 = Cm[NA:, :Noffset].copy()
    st.B01[Noffset:, :] = Cm[:NA, Noffset:]
    st.B2 = Cm[NA:, Noffset:].copy()
    st.inv_process()
    return st


def smatrix(meds, omega, L0, L1, bc, XiB, nB, XiT, nT, both_ways=True):
    """The S matrix of Scalc's main (:74-96) and Smat_calc (:144-172):
    (nB + nT) x (nB + nT) complex, meds the layers iB..iT in z order, XiB /
    XiT the full Xi of the bottom / top port layer."""
    N = nB + nT
    S = np.zeros((N, N), np.complex128)
    st = one_way(1, meds, omega, L0, L1, bc, XiB, XiT, nB, nT)
    S[:, :nB] = st.F01[:N, :]
    S[:, nB:] = st.B01[:N, :nT]
    if both_ways:
        st = one_way(-1, meds[::-1], omega, L0, L1, bc, XiT, XiB, nT, nB)
        S[nB:, nB:] = st.F01[:nT, :]
        S[:nB, nB:] = st.F01[nT:nT + nB, :]
    return S


def check_smat(S):
    """check_Smat's two residual norms are printed by the reference; here the
    unitarity residual ||S^H S - 1||_F and the transpose residual ||S - S^T||_F."""
    n = S.shape[0]
    return float(np.linalg.norm(S.conj().T @ S - np.eye(n))), float(np.linalg.norm(S - S.T))
