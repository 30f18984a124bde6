"""CPU oracle for the split-field FDTD time loop -- TEST INFRASTRUCTURE ONLY.

ctypes access to two CPU builds of the reference algorithm
(FDTDcalc/FDTDsplitfieldMetal.c):

* ``Oracle("port")`` -- ``_build/liboracle_fdtd.so``, this repository's C
  restatement (fdtd_oracle.c).  Builds anywhere gcc exists.
* ``Oracle("reference")`` -- ``_ref/libref_fdtd.so``, the reference itself
  compiled from its own sources (Makefile target ``ref``); exists only where
  the reference sources were present at build time.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
import this package.  It is the checker, never part of the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle_fdtd.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_fdtd.so")
REF_BIN = os.path.join(HERE, "_ref", "FDTD_ref")
MCALC_BIN = os.path.join(HERE, "_ref", "Mcalc_ref")
SCALC_BIN = os.path.join(HERE, "_ref", "Scalc_ref")


def reference_dir() -> str:
    """Where the reference sources are read from: $SMATRAN_REFERENCE_DIR, else
    the directory named ``reference`` beside this repository's directory."""
    env = os.environ.get("SMATRAN_REFERENCE_DIR")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


_P = C.c_void_p


# The reference's own flags (FDTDcalc/comp.sh:3: -O2 -std=c11) plus
# -ffp-contract=off, so that no fused multiply-add changes the rounding on hosts
# whose compilers contract by default (aarch64).
CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fPIC"]


def _newer(target, deps):
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target) for d in deps)


def build(with_reference: bool | None = None) -> None:
    """Compile the port (always) and the reference (when its sources exist).

    The reference is compiled from its own file under reference_dir(): a
    shared object with main renamed and exit()
    made non-fatal (ref_prelude.h), and the stock command-line binary.
    Nothing from the reference tree is copied; outputs go to _ref/ only."""
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    src = os.path.join(HERE, "fdtd_oracle.c")
    if _newer(PORT_LIB, [src, os.path.join(HERE, "fdtd_oracle.h")]):
        subprocess.run(["gcc", *CFLAGS, "-Wall", "-shared", src, "-o", PORT_LIB, "-lm"], check=True)
    ref_dir = reference_dir()
    ref_src = os.path.join(ref_dir, "FDTDcalc", "FDTDsplitfieldMetal.c")
    if with_reference is None:
        with_reference = os.path.isfile(ref_src)
    if not with_reference:
        return
    os.makedirs(os.path.join(HERE, "_ref"), exist_ok=True)
    shim = os.path.join(HERE, "blas_shim.c")
    prelude = os.path.join(HERE, "ref_prelude.h")
    if _newer(REF_LIB, [ref_src, shim, prelude]):
        subprocess.run(["gcc", *CFLAGS, "-w", "-shared", "-Dmain=ref_main", "-include", prelude, ref_src, shim,
                        "-o", REF_LIB, "-lm"], check=True)
    if _newer(REF_BIN, [ref_src, shim]):
        subprocess.run(["gcc", *CFLAGS, "-w", ref_src, shim, "-o", REF_BIN, "-lm"], check=True)
    _build_mcalc(ref_dir, shim)
    _build_scalc(ref_dir)


def _openblas():
    """scipy's bundled OpenBLAS (the only LAPACK in this image), or None."""
    import glob
    try:
        import scipy
    except ImportError:
        return None
    libs = glob.glob(os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs",
                                  "libscipy_openblas-*.so"))
    return libs[0] if libs else None


def _build_mcalc(ref_dir, blas_shim):
    """The stock reference mode solver (ModeCalc: Mcalc.c with its long-double
    eigen solvers) linked against scipy's OpenBLAS through lapack_shim.c.
    Skipped where the sources or that library are absent."""
    mdir = os.path.join(ref_dir, "ModeCalc")
    srcs = [os.path.join(mdir, f) for f in ("Mcalc.c", "ldgeev20160825.c", "lzgeev20181003.c")]
    blas = _openblas()
    if not all(os.path.isfile(s) for s in srcs) or blas is None:
        return
    lshim = os.path.join(HERE, "lapack_shim.c")
    if _newer(MCALC_BIN, srcs + [lshim, blas_shim]):
        subprocess.run(["gcc", "-O2", "-std=c11", "-w", *srcs, lshim, blas_shim, blas,
                        "-Wl,-rpath," + os.path.dirname(blas), "-o", MCALC_BIN, "-lm"], check=True)


def _build_scalc(ref_dir):
    """The stock reference S-matrix program (Smat/Scalc.c) with zgesv_ from
    lapack_shim.c and zgemm_/dznrm2_ from blas_fwd.c, both on scipy's OpenBLAS."""
    src = os.path.join(ref_dir, "Smat", "Scalc.c")
    blas = _openblas()
    if not os.path.isfile(src) or blas is None:
        return
    deps = [src, os.path.join(HERE, "lapack_shim.c"), os.path.join(HERE, "blas_fwd.c")]
    if _newer(SCALC_BIN, deps):
        subprocess.run(["gcc", "-O2", "-std=c11", "-w", *deps, blas, "-Wl,-rpath," + os.path.dirname(blas),
                        "-o", SCALC_BIN, "-lm"], check=True)


def scalc_available() -> bool:
    return os.path.isfile(SCALC_BIN)


def mcalc_available() -> bool:
    return os.path.isfile(MCALC_BIN)


def reference_available() -> bool:
    return os.path.isfile(REF_LIB)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


class Oracle:
    """Uniform wrapper over the port and the reference builds."""

    def __init__(self, kind: str = "port"):
        self.kind = kind
        path = PORT_LIB if kind == "port" else REF_LIB
        if not os.path.isfile(path):
            raise FileNotFoundError(f"oracle library missing: {path} (run oracle.build())")
        self.lib = C.CDLL(path)
        lib = self.lib
        pre = "orc_" if kind == "port" else ""
        self._f = {}
        for name in ("set_sigma", "remove_sigma", "set_address", "set_tau", "set_env", "main_calc"):
            self._f[name] = getattr(lib, pre + name)
        self._f["set_env"].restype = C.c_double
        if kind != "port":
            self.exit_calls = C.c_int.in_dll(lib, "ref_exit_calls")
        self._f["set_env"].argtypes = [C.c_int, _P, C.c_int, C.c_int, C.c_int]
        self._f["set_tau"].argtypes = [C.c_double, C.c_double, _P, _P, _P]
        if kind == "port":
            lib.orc_coefficients.argtypes = [_P, C.c_int, _P, _P, _P, _P, _P, C.c_double, C.c_double, _P, _P, _P, _P]
            lib.orc_time_loop.argtypes = [_P] * 11 + [C.c_int, _P, C.c_int, C.c_int] + [_P] * 6
            lib.orc_overlap.argtypes = [_P, C.c_int, _P, _P, _P, _P]
            lib.orc_expn_table.argtypes = [C.c_int, _P]
            self._f["set_address"].restype = C.c_int
            self._f["remove_sigma"].restype = C.c_int
            self._f["main_calc"].restype = C.c_int
            lib.orc_time_loop.restype = C.c_int

    # -- precompute -------------------------------------------------------
    @staticmethod
    def _L(L):
        return np.ascontiguousarray(L, dtype=np.int32)

    def set_sigma(self, L, mu, epsi):
        L = self._L(L)
        sigma = np.zeros(2 * int(L[0] + L[1] + L[2]), dtype=np.float64)
        self._f["set_sigma"](_ptr(L), _ptr(mu), _ptr(epsi), _ptr(sigma))
        return sigma

    def remove_sigma(self, L, mu, epsi, sigma):
        """In place on copies; returns (mu, epsi)."""
        L = self._L(L)
        mu = np.array(mu, dtype=np.complex128, copy=True)
        epsi = np.array(epsi, dtype=np.complex128, copy=True)
        rc = self._f["remove_sigma"](_ptr(L), _ptr(mu), _ptr(epsi), _ptr(sigma))
        if self.kind == "port" and rc != 0:
            raise ValueError("remove_sigma: media inconsistent with the PML stretch")
        return mu, epsi

    def set_address(self, L, sigma, mu, epsi):
        L = self._L(L)
        n3 = int(L[0]) * int(L[1]) * int(L[2])
        cont = np.zeros(n3, dtype=np.uint8)
        addr = np.zeros(n3, dtype=np.int32)
        if self.kind == "port":
            lnotn = self._f["set_address"](_ptr(L), _ptr(sigma), _ptr(mu), _ptr(epsi), _ptr(cont), _ptr(addr))
        else:
            ln = C.c_int(0)
            self._f["set_address"](_ptr(L), _ptr(sigma), _ptr(mu), _ptr(epsi), _ptr(cont), C.byref(ln), _ptr(addr))
            lnotn = ln.value
        return cont, addr, int(lnotn)

    def coefficients(self, L, lnotn, sigma, mu, epsi, cont, addr, inv_r, inv_i):
        if self.kind != "port":
            raise NotImplementedError("the reference builds coefficients inside main()")
        L = self._L(L)
        n = 3 * (int(L[0]) * int(L[1]) * int(L[2]) + lnotn)
        out = [np.zeros(n, dtype=np.float64) for _ in range(4)]
        self.lib.orc_coefficients(_ptr(L), lnotn, _ptr(sigma), _ptr(mu), _ptr(epsi), _ptr(cont), _ptr(addr),
                                  inv_r, inv_i, *[_ptr(a) for a in out])
        return tuple(out)

    def set_tau(self, omega, min_dt):
        n = C.c_int(0)
        r = C.c_double(0)
        i = C.c_double(0)
        self._f["set_tau"](omega, min_dt, C.byref(n), C.byref(r), C.byref(i))
        return n.value, r.value, i.value

    def set_env(self, n2pi, tp, jh, jt, jp):
        tp = np.ascontiguousarray(tp, dtype=np.int32)
        return self._f["set_env"](n2pi, _ptr(tp), jh, jt, jp)

    # -- the step ---------------------------------------------------------
    def main_calc(self, L, Ah, Bh, Ae, Be, iBc, H, E, iBTIin, Hi, Ei, expn2, HB, EB, HT, ET, cont, addr):
        """One Yee step in place on H, E, HB, EB, HT, ET (reference argument order)."""
        L = self._L(L)
        iBc = np.ascontiguousarray(iBc, dtype=np.int32)
        iBTIin = np.ascontiguousarray(iBTIin, dtype=np.int32)
        expn2 = np.ascontiguousarray(expn2, dtype=np.complex128)
        rc = self._f["main_calc"](_ptr(L), _ptr(Ah), _ptr(Bh), _ptr(Ae), _ptr(Be), _ptr(iBc), _ptr(H), _ptr(E),
                                  _ptr(iBTIin), _ptr(Hi), _ptr(Ei), _ptr(expn2), _ptr(HB), _ptr(EB), _ptr(HT),
                                  _ptr(ET), _ptr(cont), _ptr(addr))
        return 0 if self.kind != "port" else int(rc)

    def time_loop(self, L, Ah, Bh, Ae, Be, iBc, H, E, iBTIin, Hinc, Einc, n2pi, tp, k_begin, k_end,
                  HB, EB, HT, ET, cont, addr):
        """The reference time loop over global steps [k_begin, k_end), in place."""
        if self.kind == "port":
            L = self._L(L)
            iBc = np.ascontiguousarray(iBc, dtype=np.int32)
            iBTIin = np.ascontiguousarray(iBTIin, dtype=np.int32)
            tp = np.ascontiguousarray(tp, dtype=np.int32)
            rc = self.lib.orc_time_loop(_ptr(L), _ptr(Ah), _ptr(Bh), _ptr(Ae), _ptr(Be), _ptr(iBc), _ptr(H), _ptr(E),
                                        _ptr(iBTIin), _ptr(Hinc), _ptr(Einc), n2pi, _ptr(tp), k_begin, k_end,
                                        _ptr(HB), _ptr(EB), _ptr(HT), _ptr(ET), _ptr(cont), _ptr(addr))
            if rc == -2:
                raise MemoryError("oracle time loop: out of host memory")
            return rc  # -1: a monitor plane held a PML cell (the reference would exit)
        # the reference exposes no loop: drive its main_calc exactly as main :153-167 does
        expn = expn_table(n2pi)
        for k in range(k_begin, k_end):
            jp, jt = divmod(k, n2pi)
            jn = (jt + 1) % n2pi
            sE = 2.0 * self.set_env(n2pi, tp, 1, jt, jp)
            sH = 2.0 * self.set_env(n2pi, tp, 0, jt + 1, jp)
            # creal(conj(z)*w) = zr*wr - (-zi)*wi with one rounding per operation,
            # as C evaluates it; numpy's complex multiply may fuse (FMA) and differ
            zE, zH = expn[1 + 2 * jt], expn[0 + 2 * jn]
            Einc_c, Hinc_c = np.asarray(Einc, np.complex128), np.asarray(Hinc, np.complex128)
            Ei = sE * (zE.real * Einc_c.real - (-zE.imag) * Einc_c.imag)
            Hi = sH * (zH.real * Hinc_c.real - (-zH.imag) * Hinc_c.imag)
            self.main_calc(L, Ah, Bh, Ae, Be, iBc, H, E, iBTIin, Hi, Ei, expn[2 * jn:2 * jn + 2],
                           HB, EB, HT, ET, cont, addr)

    def overlap(self, L, tilxi_cols, HB, EB):
        L = self._L(L)
        t = np.ascontiguousarray(tilxi_cols, dtype=np.complex128)
        ncol = t.shape[0]
        S = np.zeros(ncol, dtype=np.complex128)
        self.lib.orc_overlap(_ptr(L), ncol, _ptr(t), _ptr(HB), _ptr(EB), _ptr(S))
        return S


def prepare(L, mu, epsi, omega, min_dt, dt_factor=1.0):
    """The reference precompute of main :62-143 through the port alone, for a
    process that must not load the CUDA library (the CPU timing workers):
    set_sigma, remove_sigma, set_address, set_tau (with min_Dt divided by
    dt_factor, as main :92 divides it by Dt_factor) and the coefficient arrays.
    mu, epsi: the stretched media as the Med files hold them, complex (n3*3,).
    Returns a dict of sigma, mu, epsi, cont, addr, lnotn, n2pi, invtau_R,
    invtau_I, Ah, Bh, Ae, Be."""
    o = Oracle("port")
    mu = np.ascontiguousarray(np.asarray(mu, np.complex128).reshape(-1))
    epsi = np.ascontiguousarray(np.asarray(epsi, np.complex128).reshape(-1))
    sigma = o.set_sigma(L, mu, epsi)
    mu2, ep2 = o.remove_sigma(L, mu, epsi, sigma)
    cont, addr, lnotn = o.set_address(L, sigma, mu2, ep2)
    n2pi, inv_r, inv_i = o.set_tau(omega, min_dt / dt_factor)
    Ah, Bh, Ae, Be = o.coefficients(L, lnotn, sigma, mu2, ep2, cont, addr, inv_r, inv_i)
    return {"sigma": sigma, "mu": mu2, "epsi": ep2, "cont": cont, "addr": addr, "lnotn": lnotn, "n2pi": n2pi,
            "invtau_R": inv_r, "invtau_I": inv_i, "Ah": Ah, "Bh": Bh, "Ae": Ae, "Be": Be}


def expn_table(n2pi: int) -> np.ndarray:
    """exp(i*phi) at whole and half steps, computed by the port (main :93-99)."""
    lib = C.CDLL(PORT_LIB)
    lib.orc_expn_table.argtypes = [C.c_int, _P]
    out = np.zeros(2 * n2pi, dtype=np.complex128)
    lib.orc_expn_table(n2pi, _ptr(out))
    return out
