"""Port eigenmodes on the GPU: the few-mode counterpart of the reference mode
solver (ModeCalc/Mcalc.c), through smat_mode_solve of include/smatran_fdtd.h.

``solve`` returns the propagating modes of one lossless z layer as Mcalc
writes them (theta and the columns of Xi), ``incident`` turns a column into
the source sheets the FDTD injects (FDTDsplitfieldMetal.c set_incident
:497-510) and ``dual`` into the overlap column S_calc projects on (set_tilXi
:598-628 / makePsi, Mcalc.c:505-527).  The CUDA library is required; there is
no CPU path.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import fdtd

_P = C.c_void_p


class ModeOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("degree", C.c_int), ("guard", C.c_int), ("max_iter", C.c_int),
                ("seed", C.c_ulonglong), ("precision", C.c_int)]


class ModeInfo(C.Structure):
    _fields_ = [("n_found", C.c_int), ("iterations", C.c_int), ("degenerate_pairs", C.c_int), ("block", C.c_int),
                ("matvecs", C.c_longlong), ("max_residual", C.c_double), ("spectral_radius", C.c_double),
                ("ms", C.c_double), ("matvecs_fp32", C.c_longlong)]


def _lib():
    L = fdtd.lib()
    if not getattr(L, "_modes_bound", False):
        L.smat_mode_solve.argtypes = [C.c_int, C.c_int, _P, C.c_double, _P, C.c_int, _P, _P, _P, _P]
        L.smat_mode_apply.argtypes = [C.c_int, C.c_int, _P, C.c_double, _P, C.c_int, C.c_int, _P, _P]
        L._modes_bound = True
    return L


@dataclasses.dataclass
class Modes:
    """The propagating modes of one layer, in Mcalc's conventions."""
    L0: int
    L1: int
    theta: np.ndarray   # (2*nmodes,) complex: theta[j], theta[nmodes + j] = -theta[j]
    Xi: np.ndarray      # (4*L0*L1, 2*nmodes) complex: forward j, backward nmodes + j
    info: dict

    @property
    def nmodes(self):
        return self.theta.shape[0] // 2

    @property
    def n_found(self):
        return self.info["n_found"]

    def column(self, inci_mode: int) -> np.ndarray:
        """Xi column of a signed 1-based mode number, as set_incident picks it
        (:497-499): +m forward column m-1, -m backward column."""
        if inci_mode == 0 or abs(inci_mode) > self.n_found:
            raise ValueError(f"inci_mode = {inci_mode} outside 1..{self.n_found}")
        j = abs(inci_mode) - 1
        return self.Xi[:, j if inci_mode > 0 else self.nmodes + j]

    def incident(self, inci_mode: int):
        """(Hinc, Einc) sheets, 2*L0*L1 complex each (component v of pixel p at
        v + 2p), for FDTD Plan.set_incident."""
        return incident(self.column(inci_mode), self.L0, self.L1)

    def dual(self, inci_mode: int) -> np.ndarray:
        """The tilde-Xi column S_calc projects on for this mode (4*L0*L1
        complex), for Plan.overlap / smat_overlap."""
        j = abs(inci_mode) - 1
        if inci_mode > 0:
            return dual_column(self.Xi[:, j], forward=True)
        return dual_column(self.Xi[:, self.nmodes + j], forward=False)


def _med(med, L0, L1):
    m = np.ascontiguousarray(np.asarray(med, np.complex128).reshape(6, L0 * L1))
    return m


def solve(med, omega: float, L0: int, L1: int, bc=(0, 0), nmodes: int = 4, *, tol: float = 0.0, degree: int = 0,
          guard: int = 0, max_iter: int = 0, seed: int = 0, fp64_only: bool = False) -> Modes:
    """The nmodes propagating modes of one z layer (smat_mode_solve).

    med: (6, L0*L1) complex Med values (mu00, mu11, eps22, eps11, eps00,
    mu22; value times metric factor), imaginary parts zero.  omega = k/k0 of
    the Mode file (2 pi / (lambda k0)); bc = (BoundC[0], BoundC[1]).
    fp64_only keeps every filter pass in FP64 (default: FP32 passes until the
    wanted residuals reach 1e-6, FP64 passes after)."""
    m = _med(med, L0, L1)
    bcv = np.ascontiguousarray(bc, np.int32)
    n = 2 * L0 * L1
    theta = np.zeros(2 * nmodes, np.complex128)
    Xi = np.zeros((2 * nmodes, 2 * n), np.complex128)  # column-major (4*L0*L1) x (2*nmodes)
    opts = ModeOpts(tol, degree, guard, max_iter, seed, 1 if fp64_only else 0)
    info = ModeInfo()
    fdtd._check(_lib().smat_mode_solve(L0, L1, bcv.ctypes.data_as(_P), float(omega), m.ctypes.data_as(_P), nmodes,
                                       C.byref(opts), theta.ctypes.data_as(_P), Xi.ctypes.data_as(_P),
                                       C.byref(info)))
    d = {f: getattr(info, f) for f, _ in ModeInfo._fields_}
    return Modes(L0=L0, L1=L1, theta=theta, Xi=Xi.T, info=d)


def apply(med, omega: float, L0: int, L1: int, bc, which: int, X) -> np.ndarray:
    """maa (which 0), mbb (1) or mbb*maa (2) applied on the GPU to the columns
    of X ((2*L0*L1,) or (2*L0*L1, m) real)."""
    m = _med(med, L0, L1)
    bcv = np.ascontiguousarray(bc, np.int32)
    Xa = np.asarray(X, np.float64)
    one = Xa.ndim == 1
    Xc = np.ascontiguousarray(Xa.reshape(Xa.shape[0], -1).T)  # columns contiguous
    Y = np.zeros_like(Xc)
    fdtd._check(_lib().smat_mode_apply(L0, L1, bcv.ctypes.data_as(_P), float(omega), m.ctypes.data_as(_P), which,
                                       Xc.shape[0], Xc.ctypes.data_as(_P), Y.ctypes.data_as(_P)))
    return Y[0] if one else Y.T


def incident(col, L0: int, L1: int):
    """set_incident's mapping (FDTDsplitfieldMetal.c:503-510) of one Xi column
    to the H and E source sheets; rejects a column whose E rows are not real
    (:503), as the reference does."""
    col = np.asarray(col, np.complex128)
    pl = L0 * L1
    NA = 2 * pl
    if np.any(col[NA:].imag != 0.0):
        raise ValueError("incident wave is not real number!")
    Hinc = np.zeros(2 * pl, np.complex128)
    Einc = np.zeros(2 * pl, np.complex128)
    Hinc[0::2] = col[0:pl]
    Hinc[1::2] = col[pl:2 * pl]
    Einc[1::2] = -col[2 * pl:3 * pl]
    Einc[0::2] = col[3 * pl:4 * pl]
    return Hinc, Einc


def dual_column(col, forward: bool = True) -> np.ndarray:
    """The tilde-Xi column of a real mode: set_tilXi (FDTDsplitfieldMetal.c
    :617-619) stores Xi's rows rotated by half, negated for a backward column."""
    col = np.asarray(col, np.complex128)
    NA = col.shape[0] // 2
    t = np.concatenate([col[NA:], col[:NA]])
    return t if forward else -t


def layer_media(s, z: int) -> np.ndarray:
    """(6, L0*L1) Med values of layer z of a Structure (its mu, epsi as read
    from the Med files), in the Med file's column order."""
    L0, L1 = s.L[0], s.L[1]
    pl = L0 * L1
    mu = np.asarray(s.mu).reshape(-1, pl, 3)[z]
    ep = np.asarray(s.epsi).reshape(-1, pl, 3)[z]
    return np.stack([mu[:, 0], mu[:, 1], ep[:, 2], ep[:, 1], ep[:, 0], mu[:, 2]])
