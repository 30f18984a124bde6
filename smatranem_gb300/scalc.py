"""Frequency-domain S matrix by layer transfer on the GPU: the reference's
S-matrix program (Smat/Scalc.c) through smat_scalc of include/smatran_fdtd.h.

``smatrix`` takes arrays where Scalc reads files: the Med values of the
layers between the two port layers and the full Xi matrices of the ports
(``read_xi`` parses Mcalc's Xi file).  The CUDA library is required; there is
no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import fdtd

_P = C.c_void_p


class ScalcInfo(C.Structure):
    _fields_ = [("ms", C.c_double), ("solves", C.c_int), ("unitarity", C.c_double), ("transpose", C.c_double)]


def _lib():
    L = fdtd.lib()
    if not getattr(L, "_scalc_bound", False):
        L.smat_scalc.argtypes = [C.c_int, C.c_int, _P, C.c_double, C.c_int, _P, _P, C.c_int, _P, C.c_int, C.c_int,
                                 _P, _P]
        L.smat_zgesv.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P]
        L.smat_zgemm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, C.c_int, _P, C.c_int, _P, C.c_int]
        L.smat_dense_mode.argtypes = [C.c_int]
        L.smat_zgemm_wait_test.argtypes = [_P]
        L.smat_zgemm_time.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]
        L._scalc_bound = True
    return L


def smatrix(meds, omega, L0, L1, bc, XiB, nB, XiT, nT, both_ways=True):
    """S ((nB+nT) x (nB+nT) complex) and the call's info dict.  meds: layers
    iB..iT, each (6, L0*L1) complex; XiB / XiT: (4*L0*L1, 4*L0*L1) complex."""
    m = np.ascontiguousarray(np.asarray(meds, np.complex128).reshape(len(meds), 6 * L0 * L1))
    xb = np.asfortranarray(np.asarray(XiB, np.complex128))
    xt = np.asfortranarray(np.asarray(XiT, np.complex128))
    bcv = np.ascontiguousarray(bc, np.int32)
    N = nB + nT
    S = np.zeros((N, N), np.complex128, order="F")
    info = ScalcInfo()
    fdtd._check(_lib().smat_scalc(L0, L1, bcv.ctypes.data_as(_P), float(omega), m.shape[0], m.ctypes.data_as(_P),
                                  xb.ctypes.data_as(_P), nB, xt.ctypes.data_as(_P), nT, 1 if both_ways else 0,
                                  S.ctypes.data_as(_P), C.byref(info)))
    return np.array(S), {f: getattr(info, f) for f, _ in ScalcInfo._fields_}


def zgesv(A, B):
    """X = A^{-1} B on the GPU (the LU solve behind smatrix); returns (X, info)."""
    A = np.asfortranarray(np.asarray(A, np.complex128))
    B = np.asarray(B, np.complex128)
    one = B.ndim == 1
    B = np.asfortranarray(B.reshape(B.shape[0], -1))
    X = np.zeros_like(B, order="F")
    info = C.c_int(0)
    fdtd._check(_lib().smat_zgesv(A.shape[0], B.shape[1], A.ctypes.data_as(_P), B.ctypes.data_as(_P),
                                  X.ctypes.data_as(_P), C.byref(info)))
    return (X[:, 0] if one else np.array(X)), info.value


def dense_mode(mode):
    """How smatrix and zgesv multiply: 1 (the default) FP64-accurate products
    on the tensor cores, 0 the FP64 multiply-add kernel."""
    fdtd._check(_lib().smat_dense_mode(int(mode)))


def zgemm(A, B, C=None, alpha=1.0, mode=1):
    """C + alpha * A @ B on the GPU (the products of smatrix): mode 1 on the
    tensor cores, 0 with the FP64 kernel."""
    A = np.asfortranarray(np.asarray(A, np.complex128))
    B = np.asfortranarray(np.asarray(B, np.complex128))
    m, k = A.shape
    n = B.shape[1]
    if B.shape[0] != k:
        raise ValueError(f"zgemm: A is {m} x {k}, B has {B.shape[0]} rows")
    out = np.zeros((m, n), np.complex128, order="F") if C is None else np.array(C, np.complex128, order="F")
    al = np.array([complex(alpha).real, complex(alpha).imag])
    fdtd._check(_lib().smat_zgemm(int(mode), m, n, k, al.ctypes.data_as(_P), A.ctypes.data_as(_P), m,
                                  B.ctypes.data_as(_P), k, out.ctypes.data_as(_P), m))
    return out


def zgemm_time(mode, m, n, k, reps=10):
    """Device milliseconds of one C += A B product of these sizes (operands
    seeded on the device; mode 1 tensor cores, 0 the FP64 kernel)."""
    ms = C.c_double()
    fdtd._check(_lib().smat_zgemm_time(int(mode), int(m), int(n), int(k), int(reps), C.byref(ms)))
    return ms.value


def zgemm_wait_test():
    """The error code the tensor-core product records when one of its operand
    loads never arrives (its bounded waits give up): 1 expected."""
    flag = C.c_int(-1)
    fdtd._check(_lib().smat_zgemm_wait_test(C.byref(flag)))
    return flag.value


def read_xi(path, NA=None):
    """Mcalc's Xi file (Mcalc.c:186-199) as the full (2NA x 2NA) matrix."""
    with open(path) as f:
        lines = f.readlines()
    if NA is None:
        NA = sum(1 for l in lines if l.startswith("ReXi["))
    Xi = np.zeros((2 * NA, 2 * NA), np.complex128)
    pos = 2
    for j in range(NA):
        pos += 1
        a = np.array([lines[pos + r].split() for r in range(2 * NA)], np.float64)
        pos += 2 * NA
        Xi[:, j] = a[:, 0] + 1j * a[:, 1]
        Xi[:, j + NA] = a[:, 2] + 1j * a[:, 3]
    return Xi
