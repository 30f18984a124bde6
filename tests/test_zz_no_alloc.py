"""The allocation-free S extraction, smat_overlap_noalloc, through the C ABI.

For callers that cannot allocate device memory when they extract S
parameters (under a framework that owns the device's memory pool, in a loop
that must not fail on memory after start-up).  Checked against
smat_overlap, the allocating entry point, on the same device inputs, on two
calls in a row (the static scratch keeps the previous call's contents): bit
for bit, since both reduce over the same grid of blocks, a function of npix
alone; and against a host evaluation of the projection with the tolerance the
overlap tests use (1e-12 relative).  Runs last so that a run
stopping at its first failure has run everything else; it passes alone in a
fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.float64)).to("cuda")


def test_noalloc_overlap_matches_allocating_overlap(built):
    torch = pytest.importorskip("torch")
    from smatranem_gb300 import fdtd
    lib = fdtd.lib()
    lib.smat_overlap_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(11)
    npix, ncols, nvec = 48 * 40, 6, 5
    stride = 4 * npix + 16  # planes need not be packed
    results = []
    for call in range(2):
        t = rng.standard_normal((ncols, 4 * npix)) + 1j * rng.standard_normal((ncols, 4 * npix))
        d = np.zeros(nvec * stride, np.complex128)
        for v in range(nvec):
            d[v * stride:v * stride + 4 * npix] = rng.standard_normal(4 * npix) + 1j * rng.standard_normal(4 * npix)
        dt, dd = _dev(t, torch), _dev(d, torch)
        s_ref = torch.zeros(2 * nvec * ncols, dtype=torch.float64, device="cuda")
        s_new = torch.full((2 * nvec * ncols,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        assert lib.smat_overlap(npix, ncols, nvec, stride, C.c_void_p(dt.data_ptr()), C.c_void_p(dd.data_ptr()),
                                C.c_void_p(s_ref.data_ptr()), None) == 0
        assert lib.smat_overlap_noalloc(npix, ncols, nvec, stride, C.c_void_p(dt.data_ptr()),
                                        C.c_void_p(dd.data_ptr()), C.c_void_p(s_new.data_ptr()), None) == 0
        torch.cuda.synchronize()
        a = s_ref.cpu().numpy().view(np.complex128)
        b = s_new.cpu().numpy().view(np.complex128)
        assert np.all(np.isfinite(b))
        assert np.array_equal(a, b)
        # and against the host reference of the projection
        ref = np.array([[np.sum(np.conj(t[c]) * np.concatenate(
            [d[v * stride:v * stride + npix], d[v * stride + npix:v * stride + 2 * npix],
             -d[v * stride + 3 * npix:v * stride + 4 * npix], d[v * stride + 2 * npix:v * stride + 3 * npix]]))
            for c in range(ncols)] for v in range(nvec)]).reshape(-1)
        assert np.max(np.abs(b - ref)) <= 1e-12 * np.max(np.abs(ref))
        results.append(b)
    assert not np.array_equal(results[0], results[1])  # two different problems, two answers


def test_noalloc_overlap_rejects_oversized_requests(built):
    pytest.importorskip("torch")
    from smatranem_gb300 import fdtd
    lib = fdtd.lib()
    lib.smat_overlap_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p]
    # 64 blocks x 2000 columns x 1 plane > 65536 partial sums: refused before any launch
    rc = lib.smat_overlap_noalloc(1 << 20, 2000, 1, 4 << 20, C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), None)
    assert rc == -1
    assert b"static scratch" in lib.smat_last_error()
