"""CPU restatement of the reference port-mode solver -- TEST INFRASTRUCTURE ONLY.

Follows calc_Xi of ModeCalc/Mcalc.c (:256-347): the dense eigenproblem of
mbb*maa on one z layer (2*L0*L1 unknowns) and the post-processing that turns
its eigenvectors into the biorthogonal mode matrix Xi.  Dense numpy/scipy,
for cross-sections of a few hundred points; it is the checker of the GPU
few-mode solver, never part of the product.  Each function names the
reference lines it restates.  Mcalc includes <tgmath.h>, so its sqrt, asin,
exp and fabs of complex arguments are csqrt, casin, cexp and cabs; the
numpy calls below are the same principal branches.

Pinned against the stock reference (oracle/_ref/Mcalc_ref, fixtures in
tests/golden/modes_*.npz written by tests/golden/make_modes.py).
"""
from __future__ import annotations

import numpy as np

DBL_EPSILON = np.finfo(np.float64).eps
FLT_EPSILON = float(np.finfo(np.float32).eps)


def set_V(med, omega):
    """Mcalc.c:1123-1160.  med: (6, L0*L1) complex Med values (value*factor) in
    the file's column order -- j2=0: mu00, mu11, eps22; j2=1: eps11, eps00,
    mu22.  Returns (Vcomp, comp_count): Vcomp = omega*med with rows 2 and 5
    inverted; comp_count = entries with a nonzero imaginary part."""
    V = np.array(med, dtype=np.complex128, copy=True) * omega
    V[2] = 1.0 / V[2]
    V[5] = 1.0 / V[5]
    return V, int(np.count_nonzero(V.imag != 0.0))


def set_D(bc, L0, L1):
    """Mcalc.c:1088-1121: forward differences with the wrap factor BoundC at
    the last column/row; Ddown = -Dup^T."""
    n = L0 * L1
    Dup0 = np.zeros((n, n))
    Dup1 = np.zeros((n, n))
    for i1 in range(L1):
        sw1 = (i1 + 1) // L1
        i1a = (i1 + 1) % L1
        for i0 in range(L0):
            sw0 = (i0 + 1) // L0
            i0a = (i0 + 1) % L0
            p = i0 + L0 * i1
            Dup0[p, p] = -1.0
            Dup0[p, i0a + L0 * i1] = float((1 - sw0) + sw0 * bc[0])
            Dup1[p, p] = -1.0
            Dup1[p, i0 + L0 * i1a] = float((1 - sw1) + sw1 * bc[1])
    return Dup0, Dup1, -Dup0.T, -Dup1.T


def set_M(bc, L0, L1, V):
    """Mcalc.c:990-1066: maa = diag(V0, V1) + Ddown (V2) Dup curl terms,
    mbb = diag(V3, V4) + Dup (V5) Ddown gradient terms."""
    n = L0 * L1
    Dup0, Dup1, Ddown0, Ddown1 = set_D(bc, L0, L1)
    maa = np.zeros((2 * n, 2 * n), np.complex128)
    mbb = np.zeros((2 * n, 2 * n), np.complex128)
    idx = np.arange(n)
    maa[idx, idx] = V[0]
    maa[idx + n, idx + n] = V[1]
    mbb[idx, idx] = V[3]
    mbb[idx + n, idx + n] = V[4]
    D1V = Ddown1 * V[2][None, :]
    D0V = Ddown0 * V[2][None, :]
    maa[:n, :n] += D1V @ Dup1
    maa[:n, n:] = -(D1V @ Dup0)
    maa[n:, :n] = -(D0V @ Dup1)
    maa[n:, n:] += D0V @ Dup0
    D0V = Dup0 * V[5][None, :]
    D1V = Dup1 * V[5][None, :]
    mbb[:n, :n] += D0V @ Ddown0
    mbb[:n, n:] = D0V @ Ddown1
    mbb[n:, :n] = D1V @ Ddown0
    mbb[n:, n:] += D1V @ Ddown1
    return maa, mbb


def eigen(A, real):
    """ReigenVcalc (:861-935, dgeev of the real part; conjugate pairs expanded)
    or eigenVcalc (:937-988, zgeev, then near-real/near-imaginary cleanup)."""
    import scipy.linalg as sl
    if real:
        w, v = sl.eig(A.real, check_finite=False)
        return w.astype(np.complex128), v.astype(np.complex128)
    w, v = sl.eig(A, check_finite=False)
    w = w.astype(np.complex128)
    for j in range(len(w)):
        re, im = w[j].real, w[j].imag
        if re * re / (im * im) <= DBL_EPSILON if im != 0 else False:
            w[j] = complex(0.0, im)
        re, im = w[j].real, w[j].imag
        if im * im / (re * re) <= DBL_EPSILON if re != 0 else im == 0:
            w[j] = complex(re, 0.0)
    return w, v


def realize_H(eiSin2, H):
    """realizeH (:833-859): for a real eigenvalue, rotate the vector so that its
    largest entry is real (or take the imaginary parts if that entry is
    purely imaginary)."""
    for j in range(len(eiSin2)):
        if eiSin2[j].imag != 0.0:
            continue
        col = H[:, j]
        a = np.abs(col)
        i = int(np.argmax(a))  # first maximum, as the strict > scan finds
        if col[i].real == 0.0:
            H[:, j] = col.imag.astype(np.complex128)
        elif col[i].imag != 0.0:
            H[:, j] = (a[i] / col[i]) * col


def make_sin(eiSin2):
    """makeSin (:821-831): the root with Re >= 0, flipped when its imaginary
    part is below -FLT_EPSILON*|Re|."""
    z = np.sqrt(eiSin2)
    if np.any(z.real < 0.0):
        raise ValueError("sqrt error in Ecalc")
    flip = z.imag < -FLT_EPSILON * np.abs(z.real)
    z[flip] = -z[flip]
    return z


def sort_sin(eiSin, H):
    """sortSin (:759-819): classify real roots, move them to the front, sort
    them by descending value and the rest by ascending imaginary part.  Same
    exchange sequence as the reference (selection-style swaps)."""
    eiSin = eiSin.copy()
    N = len(eiSin)
    count_real = 0
    for j in range(N):
        re, im = eiSin[j].real, eiSin[j].imag
        r1 = (im * im) / (re * re) if re != 0 else (np.inf if im != 0 else np.nan)
        if r1 <= DBL_EPSILON:
            eiSin[j] = complex(re, 0.0)
            count_real += 1
        else:
            r2 = (re * re) / (im * im) if im != 0 else (np.inf if re != 0 else np.nan)
            if r2 <= DBL_EPSILON:
                eiSin[j] = complex(0.0, im)

    def swap(a, b):
        eiSin[[a, b]] = eiSin[[b, a]]
        H[:, [a, b]] = H[:, [b, a]]

    for t in range(count_real):
        if eiSin[t].imag != 0.0:
            for j in range(t + 1, N):
                if eiSin[j].imag == 0.0:
                    # the reference stores the real part of eiSin[j] into eiSin[t]
                    d = eiSin[j].real
                    eiSin[j] = eiSin[t]
                    eiSin[t] = complex(d, 0.0)
                    H[:, [j, t]] = H[:, [t, j]]
    for t in range(count_real - 1):
        for j in range(t + 1, count_real):
            if eiSin[j].real > eiSin[t].real:
                d = eiSin[j].real
                eiSin[j] = eiSin[t]
                eiSin[t] = complex(d, 0.0)
                H[:, [j, t]] = H[:, [t, j]]
    for t in range(count_real, N - 1):
        for j in range(t + 1, N):
            if eiSin[j].imag < eiSin[t].imag:
                swap(j, t)
    return eiSin, count_real


def make_E(maa, eiSin, H):
    """makeE (:731-757): E = maa H / eiSin per column."""
    return (maa @ H) * (np.conj(eiSin) / (eiSin.real ** 2 + eiSin.imag ** 2))[None, :]


def make_Xi(eiSin, H, E):
    """makeXi (:645-666): theta = 2 asin(eiSin/2); forward column
    [e^{-i theta/2} H; E], backward column [e^{+i theta/2} H; -E]."""
    N = len(eiSin)
    theta = np.zeros(2 * N, np.complex128)
    theta[:N] = 2.0 * np.arcsin(0.5 * eiSin)
    theta[N:] = -theta[:N]
    Xi = np.zeros((2 * N, 2 * N), np.complex128)
    ph = np.exp(0.5j * theta[:N])[None, :]
    Xi[:N, N:] = ph * H
    Xi[:N, :N] = np.exp(-0.5j * theta[:N])[None, :] * H
    Xi[N:, :N] = E
    Xi[N:, N:] = -E
    return theta, Xi


def _swap_cols(theta, Xi, i, j):
    theta[[i, j]] = theta[[j, i]]
    Xi[:, [i, j]] = Xi[:, [j, i]]


def sort_Xi(N, num_real, theta, Xi):
    """sortXi (:563-630): pair complex-conjugate backward columns, order real
    modes by descending Re theta and complex ones by ascending Im theta.  The
    reference's consistency checks (which exit) raise here."""
    F = FLT_EPSILON
    for c in range(num_real, N - 1):
        if abs(theta[c + N].real) > F and abs((theta[c] + theta[c + N]).real) < F:
            for s in range(c + 1, N):
                if abs((theta[s + N] - theta[c]).real) < F and abs((theta[s + N] + theta[c]).imag) < F:
                    _swap_cols(theta, Xi, c + N, s + N)
                    break
    for c in range(num_real - 1):
        for s in range(c + 1, num_real):
            if theta[s].real > theta[c].real + F:
                _swap_cols(theta, Xi, c, s)
                _swap_cols(theta, Xi, c + N, s + N)
    for c in range(num_real, N - 1):
        for s in range(c + 1, N):
            if theta[s].imag + F < theta[c].imag:
                _swap_cols(theta, Xi, c, s)
                _swap_cols(theta, Xi, c + N, s + N)
    for c in range(num_real, N):
        if abs(theta[c] - np.conj(theta[c + N])) > F:
            for j in range(c + 1, N):
                if abs(theta[c] - np.conj(theta[j + N])) <= F:
                    _swap_cols(theta, Xi, c + N, j + N)
                    break
    for c in range(num_real - 1):
        if theta[c + 1].real > theta[c].real + F:
            raise ValueError("sortXi: real modes out of order")
    for c in range(num_real):
        if abs(theta[c].imag) > DBL_EPSILON or abs(theta[c + N].real + theta[c].real) > F:
            raise ValueError("sortXi: real mode without its backward partner")
    for c in range(num_real, N - 1):
        if theta[c + 1].imag + F < theta[c].imag:
            raise ValueError("sortXi: complex modes out of order")
    for c in range(num_real, N):
        if theta[c].imag < DBL_EPSILON or abs(theta[c] - np.conj(theta[c + N])) > F:
            raise ValueError(f"sortXi: complex mode {c} is not paired with its conjugate (lossy port media)")


def norm_Xi(N, num_real, c, Xi):
    """normXi (:529-561): unit power flow for a real mode's forward and
    backward columns; for a complex mode, the pair scaled so that the cross
    flow is 1."""
    if c < num_real:
        for fb in range(2):
            col = Xi[:, c + fb * N]
            nz = np.sum(np.conj(col[:N]) * col[N:]) + np.sum(np.conj(col[N:]) * col[:N])
            if (0.5 - fb) * nz.real < 0.0:
                raise ValueError(f"flow direction error in normXi at column {c}, fb={fb}")
            Xi[:, c + fb * N] = col * (1.0 / np.sqrt(abs(nz.real)))
    else:
        a, b = Xi[:, c], Xi[:, c + N]
        nz = np.sum(np.conj(b[:N]) * a[N:]) + np.sum(np.conj(b[N:]) * a[:N])
        nz = np.sqrt(nz)
        nz = np.conj(nz) / (nz.real ** 2 + nz.imag ** 2)
        Xi[:, c] = a * nz
        Xi[:, c + N] = b * np.conj(nz)


def psi_column(N, num_real, m, Xi):
    """makePsi (:505-527) for one mode: the dual columns (m, m+N) of tilde-Xi."""
    P0 = np.empty(2 * N, np.complex128)
    P1 = np.empty(2 * N, np.complex128)
    if m < num_real:
        P0[:N], P0[N:] = Xi[N:, m], Xi[:N, m]
        P1[:N], P1[N:] = -Xi[N:, m + N], -Xi[:N, m + N]
    else:
        P1[:N], P1[N:] = Xi[N:, m], Xi[:N, m]
        P0[:N], P0[N:] = Xi[N:, m + N], Xi[:N, m + N]
    return P0, P1


def dual(N, num_real, Xi):
    """The full tilde-Xi whose columns makePsi builds (checkXi :237-240)."""
    T = np.empty_like(Xi)
    for m in range(N):
        T[:, m], T[:, m + N] = psi_column(N, num_real, m, Xi)
    return T


def degene_Xi(N, num_real, theta, Xi, log=None):
    """degeneXi (:417-467): for modes whose thetas agree to FLT_EPSILON
    (relative), remove from the later one its component along the earlier one
    in the tilde-Xi pairing, then renormalise."""
    for j in range(N - 1):
        for i in range(j + 1, N):
            if abs((theta[j] - theta[i]) / (theta[j] + theta[i])) < FLT_EPSILON:
                Pi0, PiN = psi_column(N, num_real, i, Xi)
                s_ij0 = np.sum(np.conj(Pi0) * Xi[:, j])
                s_ijN = np.sum(np.conj(PiN) * Xi[:, j + N])
                Pj0, PjN = psi_column(N, num_real, j, Xi)
                s_ji0 = np.sum(np.conj(Pj0) * Xi[:, i])
                s_jiN = np.sum(np.conj(PjN) * Xi[:, i + N])
                a0 = 1.0 / np.sqrt(abs(1.0 - s_ji0 * s_ij0))
                aN = 1.0 / np.sqrt(abs(1.0 - s_jiN * s_ijN))
                Xi[:, i] = a0 * Xi[:, i] + (-a0 * s_ji0) * Xi[:, j]
                Xi[:, i + N] = aN * Xi[:, i + N] + (-aN * s_jiN) * Xi[:, j + N]
                norm_Xi(N, num_real, i, Xi)
                if log is not None:
                    log.append((j, i, abs(s_ji0)))


def check_Xi(N, num_real, Xi):
    """checkXi (:237-280): ||tilde-Xi^H Xi - 1||_F."""
    C = dual(N, num_real, Xi).conj().T @ Xi
    C[np.diag_indices_from(C)] -= 1.0
    return float(np.linalg.norm(C))


def calc_Xi(med, omega, L0, L1, bc):
    """calc_Xi (:256-347) with InPrecision "D".  Returns a dict with theta
    (2N), Xi (2N x 2N, columns [forward 0..N-1, backward 0..N-1]), num_real,
    eiSin2 (the eigenvalues of mbb*maa in the order makeXi saw them), the
    real-matrix flag and the two diagnostics Mcalc prints."""
    N = 2 * L0 * L1
    V, comp = set_V(med, omega)
    maa, mbb = set_M(bc, L0, L1, V)
    A = mbb @ maa
    real = comp == 0
    eiSin2, H = eigen(A, real)
    if real:
        realize_H(eiSin2, H)
    eiSin = make_sin(eiSin2)
    eiSin, num_real = sort_sin(eiSin, H)
    E = make_E(maa, eiSin, H)
    resid_num = np.linalg.norm((mbb @ E) / eiSin[None, :] - H)
    norm = resid_num / (np.linalg.norm((mbb @ E) / eiSin[None, :]) + np.linalg.norm(E))
    theta, Xi = make_Xi(eiSin, H, E)
    sort_Xi(N, num_real, theta, Xi)
    for c in range(N):
        norm_Xi(N, num_real, c, Xi)
    log = []
    degene_Xi(N, num_real, theta, Xi, log)
    return dict(theta=theta, Xi=Xi, num_real=num_real, real_matrix=real, maa=maa, mbb=mbb,
                check=check_Xi(N, num_real, Xi), norm=norm, degenerate=log)
