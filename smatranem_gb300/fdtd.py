"""Python view of the C ABI in include/smatran_fdtd.h (ctypes, numpy arrays).

Mirrors the reference's FDTD interface (FDTDcalc/FDTDsplitfieldMetal.c):
``set_sigma``, ``remove_sigma``, ``set_address``, ``coefficients``,
``set_tau``, ``set_env`` and ``main_calc`` keep the reference names, argument
meaning and array layouts; ``Plan`` is the resident, many-steps-per-call form.
Errors raise ``FdtdError`` carrying the library's message (the reference would
print it and exit).

The CUDA library is required: loading fails loudly when it is missing or
cannot be loaded; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsmatran_fdtd.so")

FP64 = 0
FP32 = 1

_P = C.c_void_p
_lib = None


class FdtdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"smatran_fdtd error {code}: {msg}")
        self.code = code


class Desc(C.Structure):
    _fields_ = [("L", C.c_int * 4), ("iBc", C.c_int * 3), ("iBTIin", C.c_int * 4),
                ("invtau_R", C.c_double), ("invtau_I", C.c_double),
                ("mu", _P), ("epsi", _P), ("sigma", _P), ("pec", _P),
                ("precision", C.c_int), ("batch", C.c_int)]


def lib():
    """The loaded C library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise FdtdError(-100, f"{LIB_PATH} missing: run `python -m smatranem_gb300.build`")
        L = C.CDLL(LIB_PATH)
        L.smat_last_error.restype = C.c_char_p
        L.smat_set_env.restype = C.c_double
        L.smat_set_env.argtypes = [C.c_int, _P, C.c_int, C.c_int, C.c_int]
        L.smat_set_tau.argtypes = [C.c_double, C.c_double, _P, _P, _P]
        L.smat_coefficients.argtypes = [_P, C.c_int, _P, _P, _P, _P, _P, C.c_double, C.c_double, _P, _P, _P, _P]
        L.smat_fdtd_create.argtypes = [_P, _P, _P]
        L.smat_fdtd_create_from_coeffs.argtypes = [_P] * 8 + [C.c_int, _P, C.c_int, _P, _P]
        L.smat_fdtd_set_fields.argtypes = [_P, C.c_int, _P, _P]
        L.smat_fdtd_save_state.argtypes = [_P, C.c_char_p]
        L.smat_fdtd_load_state.argtypes = [_P, C.c_char_p]
        L.smat_fdtd_get_fields.argtypes = [_P, C.c_int, _P, _P]
        L.smat_fdtd_set_incident.argtypes = [_P, C.c_int, _P, _P]
        L.smat_fdtd_set_cw_schedule.argtypes = [_P, C.c_int, _P]
        L.smat_fdtd_set_source_plane.argtypes = [_P, C.c_int, C.c_int, C.c_int]
        L.smat_fdtd_set_schedule.argtypes = [_P, C.c_int, _P, C.c_int, C.c_int, _P, _P]
        L.smat_fdtd_run.argtypes = [_P, C.c_int, C.c_int]
        L.smat_fdtd_step.argtypes = [_P, _P, _P, _P]
        L.smat_fdtd_get_monitor.argtypes = [_P, C.c_int, _P, _P, _P, _P]
        L.smat_fdtd_get_dft.argtypes = [_P, C.c_int, C.c_int, C.c_int, _P]
        L.smat_fdtd_check_finite.argtypes = [_P, _P, _P]
        L.smat_fdtd_device_bytes.restype = C.c_longlong
        L.smat_fdtd_device_bytes.argtypes = [_P]
        L.smat_fdtd_destroy.argtypes = [_P]
        L.smat_fdtd_sync.argtypes = [_P]
        L.smat_fdtd_copy_bytes.argtypes = [_P, _P, _P]
        L.smat_fdtd_info.argtypes = [_P, _P, _P, _P, _P]
        L.smat_fdtd_time_kernels.argtypes = [_P, C.c_int, C.c_int, _P]
        L.smat_fdtd_set_tuning.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.smat_fdtd_get_tuning.argtypes = [_P, _P]
        L.smat_device_info.argtypes = [_P, C.c_int, _P, _P]
        L.smat_fdtd_autotune.argtypes = [_P, C.c_int, _P, _P]
        L.smat_fdtd_overlap.argtypes = [_P, C.c_int, C.c_int, C.c_int, _P, _P]
        L.smat_fdtd_dft_count.argtypes = [_P, _P, _P]
        L.smat_fdtd_dft_device.argtypes = [_P, C.c_int, C.c_int, C.c_int, _P, _P]
        L.smat_overlap.argtypes = [C.c_int, C.c_int, C.c_int, C.c_longlong, _P, _P, _P, _P]
        L.smat_fdtd_adjoint_grad.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P]
        L.smat_fdtd_group_create.argtypes = [_P, C.c_int, _P]
        L.smat_fdtd_group_destroy.argtypes = [_P]
        L.smat_fdtd_group_set_tuning.argtypes = [_P, C.c_int, C.c_int]
        L.smat_fdtd_group_autotune.argtypes = [_P, C.c_int, _P, _P]
        L.smat_fdtd_group_run.argtypes = [_P, C.c_int, C.c_int]
        L.smat_fdtd_group_sync.argtypes = [_P]
        L.smat_row32_pieces.argtypes = [C.c_int] * 6 + [_P, C.c_int, _P]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise FdtdError(rc, lib().smat_last_error().decode(errors="replace"))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


# -- host precompute: the reference's names (main :62-143) ------------------

def set_sigma(L, mu, epsi):
    """sigma[2*(L0+L1+L2)] from stretched media (set_sigma :858-926)."""
    L = _i32(L)
    sigma = np.zeros(2 * int(L[0] + L[1] + L[2]))
    _check(lib().smat_set_sigma(_ptr(L), _ptr(_c128(mu)), _ptr(_c128(epsi)), _ptr(sigma)))
    return sigma


def remove_sigma(L, mu, epsi, sigma):
    """Copies of mu, epsi with the PML stretch divided out (remove_sigma :822-853)."""
    L = _i32(L)
    mu = np.array(mu, dtype=np.complex128, copy=True)
    epsi = np.array(epsi, dtype=np.complex128, copy=True)
    _check(lib().smat_remove_sigma(_ptr(L), _ptr(mu), _ptr(epsi), _ptr(np.ascontiguousarray(sigma, np.float64))))
    return mu, epsi


def set_address(L, sigma, mu, epsi):
    """(Cont as uint8 codes of 'n','a','h','e','b', address_notn, Lnotn) (set_address :188-233)."""
    L = _i32(L)
    n3 = int(L[0]) * int(L[1]) * int(L[2])
    cont = np.zeros(n3, dtype=np.uint8)
    addr = np.zeros(n3, dtype=np.int32)
    ln = C.c_int(0)
    _check(lib().smat_set_address(_ptr(L), _ptr(np.ascontiguousarray(sigma, np.float64)), _ptr(_c128(mu)),
                                  _ptr(_c128(epsi)), _ptr(cont), C.byref(ln), _ptr(addr)))
    return cont, addr, ln.value


def coefficients(L, lnotn, sigma, mu, epsi, cont, addr, invtau_R, invtau_I):
    """(Ah, Bh, Ae, Be), 3*(L3D+Lnotn) doubles each (main :106-143)."""
    L = _i32(L)
    n = 3 * (int(L[0]) * int(L[1]) * int(L[2]) + lnotn)
    out = [np.zeros(n) for _ in range(4)]
    _check(lib().smat_coefficients(_ptr(L), lnotn, _ptr(np.ascontiguousarray(sigma, np.float64)), _ptr(_c128(mu)),
                                   _ptr(_c128(epsi)), _ptr(np.ascontiguousarray(cont, np.uint8)), _ptr(_i32(addr)),
                                   invtau_R, invtau_I, *[_ptr(a) for a in out]))
    return tuple(out)


def set_tau(omega, min_dt):
    """(N_2pi, invtau_R, invtau_I) (set_tau :515-524)."""
    n, r, i = C.c_int(0), C.c_double(0), C.c_double(0)
    _check(lib().smat_set_tau(omega, min_dt, C.byref(n), C.byref(r), C.byref(i)))
    return n.value, r.value, i.value


def set_env(n2pi, time_period, j_half, j_time, j_period):
    """Envelope value (set_env :452-475); NaN where the reference exits."""
    return lib().smat_set_env(n2pi, _ptr(_i32(time_period)), j_half, j_time, j_period)


def main_calc(L, Ah, Bh, Ae, Be, iBc, H_t, E_t, iBTIin, Hi, Ei, ExpN2, HB, EB, HT, ET, Cont, address_notn):
    """One step on the GPU with main_calc's arguments; updates H_t..ET in place."""
    for a in (H_t, E_t, HB, EB, HT, ET):
        if not a.flags["C_CONTIGUOUS"] or not a.flags["WRITEABLE"]:
            raise ValueError("in/out arrays must be writeable and C-contiguous")
    _check(lib().smat_main_calc(_ptr(_i32(L)), _ptr(Ah), _ptr(Bh), _ptr(Ae), _ptr(Be), _ptr(_i32(iBc)), _ptr(H_t),
                                _ptr(E_t), _ptr(_i32(iBTIin)), _ptr(np.ascontiguousarray(Hi, np.float64)),
                                _ptr(np.ascontiguousarray(Ei, np.float64)), _ptr(_c128(ExpN2)), _ptr(HB), _ptr(EB),
                                _ptr(HT), _ptr(ET), _ptr(np.ascontiguousarray(Cont, np.uint8)),
                                _ptr(_i32(address_notn))))


# -- plans ------------------------------------------------------------------

TUNING_CACHE = os.environ.get("SMATRAN_TUNING_CACHE", os.path.join(_HERE, "_build", "tuning_cache.json"))


def _load_cache():
    try:
        with open(TUNING_CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def device_info():
    """(name, SM count, compute capability) of the current CUDA device."""
    name = C.create_string_buffer(128)
    sms, cc = C.c_int(0), C.c_int(0)
    _check(lib().smat_device_info(name, 128, C.byref(sms), C.byref(cc)))
    return name.value.decode(), sms.value, cc.value


def row32_pieces(L1, L2, tile_y, z_chunk, ngroups, gidx):
    """The pieces (row tile, z0, z1) that CTA group (or item) gidx of the
    whole-row fused step marches: the kernel's own schedule, run on the host
    (smat_row32_pieces; no GPU needed)."""
    cap = 4 * (L1 + 4) + 16
    out = np.zeros(3 * cap, np.int32)
    n = C.c_int(0)
    _check(lib().smat_row32_pieces(L1, L2, tile_y, z_chunk, ngroups, gidx, _ptr(out), cap, C.byref(n)))
    return [tuple(int(v) for v in out[3 * i:3 * i + 3]) for i in range(n.value)]


class Plan:
    """A structure and its excitations resident on the GPU (smat_fdtd_* API)."""

    def __init__(self, handle, keep=()):
        self._h = handle
        self._keep = keep
        info = [(C.c_int * 4)(), C.c_int(), C.c_int(), C.c_int()]
        _check(lib().smat_fdtd_info(self._h, info[0], C.byref(info[1]), C.byref(info[2]), C.byref(info[3])))
        self.L = tuple(info[0])
        self.lnotn, self.precision, self.batch = info[1].value, info[2].value, info[3].value
        self.n3 = self.L[0] * self.L[1] * self.L[2]
        self.pl = self.L[0] * self.L[1]

    @classmethod
    def create(cls, L, iBc, iBTIin, invtau_R, invtau_I, mu, epsi, sigma, precision=FP64, batch=1, pec=None,
               stream=None):
        """From media after remove_sigma (complex 3*L3D each) and sigma."""
        mu, epsi = _c128(mu), _c128(epsi)
        sigma = np.ascontiguousarray(sigma, np.float64)
        pec_a = None if pec is None else np.ascontiguousarray(pec, np.uint8)
        d = Desc()
        d.L[:] = list(L)
        d.iBc[:] = list(iBc)
        d.iBTIin[:] = list(iBTIin)
        d.invtau_R, d.invtau_I = invtau_R, invtau_I
        d.mu, d.epsi, d.sigma, d.pec = _ptr(mu), _ptr(epsi), _ptr(sigma), _ptr(pec_a)
        d.precision, d.batch = precision, batch
        h = _P()
        _check(lib().smat_fdtd_create(C.byref(d), _P(stream) if stream else None, C.byref(h)))
        return cls(h)

    @classmethod
    def from_coeffs(cls, L, Ah, Bh, Ae, Be, iBc, Cont, address_notn, Lnotn, iBTIin, batch=1, stream=None):
        h = _P()
        _check(lib().smat_fdtd_create_from_coeffs(
            _ptr(_i32(L)), _ptr(Ah), _ptr(Bh), _ptr(Ae), _ptr(Be), _ptr(_i32(iBc)),
            _ptr(np.ascontiguousarray(Cont, np.uint8)), _ptr(_i32(address_notn)), Lnotn, _ptr(_i32(iBTIin)), batch,
            _P(stream) if stream else None, C.byref(h)))
        return cls(h)

    def close(self):
        if self._h:
            lib().smat_fdtd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def field_len(self):
        return 3 * (self.n3 + self.lnotn + 1)

    @property
    def device_bytes(self):
        return lib().smat_fdtd_device_bytes(self._h)

    def set_fields(self, b, H_t, E_t):
        _check(lib().smat_fdtd_set_fields(self._h, b, _ptr(np.ascontiguousarray(H_t, np.float64)),
                                          _ptr(np.ascontiguousarray(E_t, np.float64))))

    def get_fields(self, b=0):
        H = np.zeros(self.field_len)
        E = np.zeros(self.field_len)
        _check(lib().smat_fdtd_get_fields(self._h, b, _ptr(H), _ptr(E)))
        return H, E

    def set_incident(self, b, Hinc, Einc):
        _check(lib().smat_fdtd_set_incident(self._h, b, _ptr(_c128(Hinc)), _ptr(_c128(Einc))))

    def set_source_plane(self, b, iI, inci_mode):
        _check(lib().smat_fdtd_set_source_plane(self._h, b, iI, inci_mode))

    def set_cw_schedule(self, n2pi, time_period):
        _check(lib().smat_fdtd_set_cw_schedule(self._h, n2pi, _ptr(_i32(time_period))))

    def set_schedule(self, src, planes=(), phase=None):
        src = np.ascontiguousarray(src, np.float64).reshape(-1, 6)
        nsteps = src.shape[0]
        if phase is None:
            nfreq, planes_a, ph = 0, None, None
        else:
            ph = np.ascontiguousarray(phase, np.float64).reshape(nsteps, -1, 4)
            nfreq = ph.shape[1]
            planes_a = _i32(planes)
        _check(lib().smat_fdtd_set_schedule(self._h, nsteps, _ptr(src), nfreq,
                                            0 if planes_a is None else len(planes_a), _ptr(planes_a), _ptr(ph)))

    def step(self, Hi, Ei, ExpN2):
        _check(lib().smat_fdtd_step(self._h, _ptr(np.ascontiguousarray(Hi, np.float64)),
                                    _ptr(np.ascontiguousarray(Ei, np.float64)), _ptr(_c128(ExpN2))))

    def run(self, k_begin, k_end, sync=True):
        _check(lib().smat_fdtd_run(self._h, k_begin, k_end))
        if sync:
            self.sync()

    def sync(self):
        _check(lib().smat_fdtd_sync(self._h))

    def copy_bytes(self):
        """(host->device, device->host) bytes copied for this plan so far
        (smat_fdtd_copy_bytes)."""
        h, d = C.c_longlong(0), C.c_longlong(0)
        _check(lib().smat_fdtd_copy_bytes(self._h, C.byref(h), C.byref(d)))
        return h.value, d.value

    def get_monitor(self, b=0):
        out = [np.zeros(2 * self.pl, dtype=np.complex128) for _ in range(4)]
        _check(lib().smat_fdtd_get_monitor(self._h, b, *[_ptr(a) for a in out]))
        return tuple(out)

    def get_dft(self, b, f, q):
        out = np.zeros(4 * self.pl, dtype=np.complex128)
        _check(lib().smat_fdtd_get_dft(self._h, b, f, q, _ptr(out)))
        return out.reshape(4, self.pl)

    def time_kernels(self, k_begin, nsteps):
        ms = np.zeros(3)
        _check(lib().smat_fdtd_time_kernels(self._h, k_begin, nsteps, _ptr(ms)))
        return ms

    def save_state(self, path):
        """Fields, aux slots and DFT accumulators to a file (smat_fdtd_save_state)."""
        _check(lib().smat_fdtd_save_state(self._h, os.fsencode(path)))

    def load_state(self, path):
        """Restore a state saved from a plan of the same setup (smat_fdtd_load_state);
        run(k, ...) then continues from step k."""
        _check(lib().smat_fdtd_load_state(self._h, os.fsencode(path)))

    def set_tuning(self, fused=2, tile_y=1, z_chunk=0, ctas_per_sm=0, slots=4):
        _check(lib().smat_fdtd_set_tuning(self._h, fused, tile_y, z_chunk, ctas_per_sm, slots))

    def autotune(self, nsteps=4, cache=True):
        """Pick the fastest FP32 configuration (smat_fdtd_autotune).  With cache,
        the choice is remembered per (grid, batch, precision, GPU model, SM
        count) in TUNING_CACHE and reused without timing."""
        key = None
        if cache:
            key = json.dumps([list(self.L), self.batch, self.precision, *device_info()])
            entry = _load_cache().get(key)
            if entry:
                try:
                    self.set_tuning(*entry["tuning"])
                    return tuple(entry["tuning"]), entry["ms"]
                except FdtdError:
                    pass
        best = (C.c_int * 5)()
        ms = C.c_double(0)
        _check(lib().smat_fdtd_autotune(self._h, nsteps, best, C.byref(ms)))
        if key is not None:
            c = _load_cache()
            c[key] = {"tuning": list(best), "ms": ms.value}
            try:
                with open(TUNING_CACHE, "w") as f:
                    json.dump(c, f, indent=1)
            except OSError:
                pass
        return tuple(best), ms.value

    def get_tuning(self):
        out = (C.c_int * 5)()
        _check(lib().smat_fdtd_get_tuning(self._h, out))
        return tuple(out)

    def dft_count(self):
        """(DFT frequencies, DFT planes) of the schedule."""
        nf, nq = C.c_int(0), C.c_int(0)
        _check(lib().smat_fdtd_dft_count(self._h, C.byref(nf), C.byref(nq)))
        return nf.value, nq.value

    def overlap(self, b, q, tilxi_cols):
        """S for every DFT frequency of plane q: (nfreq, ncols) complex (GPU, FP64)."""
        t = _c128(tilxi_cols)
        ncols = t.shape[0]
        nf = C.c_int(0)
        _check(lib().smat_fdtd_dft_count(self._h, C.byref(nf), None))
        S = np.zeros((nf.value, ncols), np.complex128)
        _check(lib().smat_fdtd_overlap(self._h, b, q, ncols, _ptr(t), _ptr(S)))
        return S

    def adjoint_grad(self, nsteps, K, f, q, tilxi_cols, box):
        """J = sum_b |S_b|^2 of mode columns tilxi_cols (4*L0*L1 complex: one
        column for every excitation, or a (batch, 4*L0*L1) array, row b for
        excitation b) on DFT plane slot q at frequency f, and dJ/ds for every
        cell of box (x0, x1, y0, y1, z0, z1), s scaling the cell's permittivity
        by (1 + s) (smat_fdtd_adjoint_grad).  Returns (J, grad [nz, ny, nx],
        grad_c [3, nz, ny, nx])."""
        t = _c128(tilxi_cols)
        ncols = 1 if t.ndim == 1 else t.shape[0]
        t = t.reshape(-1)
        bx = _i32(box)
        shape = (int(bx[5] - bx[4]), int(bx[3] - bx[2]), int(bx[1] - bx[0]))
        g = np.zeros(shape)
        gc = np.zeros((3,) + shape)
        J = C.c_double(0)
        _check(lib().smat_fdtd_adjoint_grad(self._h, nsteps, K, f, q, ncols, _ptr(t), _ptr(bx), _ptr(g), _ptr(gc),
                                            C.byref(J)))
        return J.value, g, gc

    def check_finite(self):
        ok, m = C.c_int(0), C.c_double(0)
        _check(lib().smat_fdtd_check_finite(self._h, C.byref(ok), C.byref(m)))
        return bool(ok.value), m.value


class Group:
    """Several FP32 plans stepped together, one launch per sweep for all
    (smat_fdtd_group_*).  The plans stay owned by the caller and must outlive
    the group."""

    def __init__(self, plans):
        self.plans = list(plans)
        arr = (_P * len(self.plans))(*[p._h for p in self.plans])
        h = _P()
        _check(lib().smat_fdtd_group_create(arr, len(self.plans), C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            lib().smat_fdtd_group_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_tuning(self, mode, block_y):
        """mode 0: one grouped launch per sweep; 1: members' own sweep launches;
        2: members' own launch forms (their set_tuning / autotune); 3: one
        persistent whole-row fused launch per step for every member (the
        resident CTAs shared out among the members).  block_y: rows per sweep
        block (modes 0, 1); mode 3: 1 = CTAs of 384 threads, 2 = of 192 (two
        per SM, smaller tiles)."""
        _check(lib().smat_fdtd_group_set_tuning(self._h, mode, block_y))

    def autotune(self, nsteps=4):
        """((mode, block_y), ms per step) of the fastest form."""
        best, ms = (C.c_int * 2)(), C.c_double(0)
        _check(lib().smat_fdtd_group_autotune(self._h, nsteps, best, C.byref(ms)))
        return (best[0], best[1]), ms.value

    def run(self, k_begin, k_end, sync=True):
        _check(lib().smat_fdtd_group_run(self._h, k_begin, k_end))
        if sync:
            self.sync()

    def sync(self):
        _check(lib().smat_fdtd_group_sync(self._h))


def cw_schedule(n2pi, time_period):
    """The reference CW run as (src [nsteps,6], phase [nsteps,1,4]) (main :153-167)."""
    tp = _i32(time_period)
    nsteps = int(tp[2]) * n2pi
    src = np.zeros((nsteps, 6))
    ph = np.zeros((nsteps, 1, 4))
    _check(lib().smat_cw_schedule(n2pi, _ptr(tp), _ptr(src), _ptr(ph)))
    return src, ph
