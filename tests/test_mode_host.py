"""Host parts of the port-mode solver that need no GPU: the small Schur
eigen solver of its Rayleigh-Ritz step (smat_mode_small_eig) against
numpy, and the argument checks of smat_mode_solve / smat_mode_apply."""
import ctypes as C

import numpy as np
import pytest

from smatranem_gb300 import fdtd, modes, workloads as W

_P = C.c_void_p


def small_eig(B):
    L = fdtd.lib()
    L.smat_mode_small_eig.argtypes = [C.c_int, _P, _P, _P]
    B = np.ascontiguousarray(B, np.complex128)
    m = B.shape[0]
    w = np.zeros(m, np.complex128)
    V = np.zeros((m, m), np.complex128)
    fdtd._check(L.smat_mode_small_eig(m, B.ctypes.data_as(_P), w.ctypes.data_as(_P), V.ctypes.data_as(_P)))
    return w, V


def _match(w, ref):
    """greedy pairing of two eigenvalue lists"""
    ref = list(ref)
    err = 0.0
    for x in w:
        k = int(np.argmin([abs(x - r) for r in ref]))
        err = max(err, abs(x - ref.pop(k)))
    return err


@pytest.mark.parametrize("m,kind", [(1, "c"), (2, "r"), (5, "c"), (16, "r"), (40, "c"), (64, "r")])
def test_small_eig_matches_numpy(m, kind):
    rng = np.random.default_rng(m)
    B = rng.standard_normal((m, m))
    if kind == "c":
        B = B + 1j * rng.standard_normal((m, m))
    w, V = small_eig(B)
    scale = np.abs(np.linalg.eigvals(B)).max()
    assert _match(w, np.linalg.eigvals(B)) < 1e-11 * scale
    # each column an eigenvector of unit norm
    np.testing.assert_allclose(np.linalg.norm(V, axis=0), 1.0, rtol=1e-12)
    assert np.abs(B @ V - V * w[None, :]).max() < 1e-10 * scale


def test_small_eig_triangular_and_repeated():
    B = np.triu(np.arange(1, 26, dtype=float).reshape(5, 5))
    w, V = small_eig(B)
    np.testing.assert_allclose(np.sort(w.real), np.sort(np.diag(B)), rtol=1e-13)
    D = np.diag([3.0, 3.0, 1.0, -2.0])  # repeated eigenvalue, normal matrix
    w, V = small_eig(D)
    np.testing.assert_allclose(np.sort(w.real), [-2.0, 1.0, 3.0, 3.0], atol=1e-14)
    assert np.abs(D @ V - V * w[None, :]).max() < 1e-13


def test_solve_rejects_lossy_and_bad_arguments():
    med = W.port_layer(6, 5, core=(2, 2), loss=0.05, seed=5)
    with pytest.raises(fdtd.FdtdError) as e:
        modes.solve(med, 0.4, 6, 5, (0, 0), 2)
    assert e.value.code == -1 and "lossless" in str(e.value)
    med = W.port_layer(6, 5, core=(2, 2), seed=5)
    for kw in (dict(bc=(2, 0)), dict(nmodes=0), dict(nmodes=61)):
        args = dict(bc=(0, 0), nmodes=2)
        args.update(kw)
        with pytest.raises(fdtd.FdtdError) as e:
            modes.solve(med, 0.4, 6, 5, args["bc"], args["nmodes"])
        assert e.value.code == -1
    with pytest.raises(fdtd.FdtdError):
        modes.solve(med, -1.0, 6, 5, (0, 0), 2)


def test_incident_and_dual_mappings():
    """set_incident (:503-510) and set_tilXi (:617-619) index maps."""
    L0, L1 = 3, 2
    pl = L0 * L1
    col = np.arange(4 * pl) + 0j
    Hinc, Einc = modes.incident(col, L0, L1)
    np.testing.assert_array_equal(Hinc[0::2].real, np.arange(pl))
    np.testing.assert_array_equal(Hinc[1::2].real, pl + np.arange(pl))
    np.testing.assert_array_equal(Einc[1::2].real, -(2 * pl + np.arange(pl)))
    np.testing.assert_array_equal(Einc[0::2].real, 3 * pl + np.arange(pl))
    bad = col.copy()
    bad[3 * pl] += 1e-30j
    with pytest.raises(ValueError):
        modes.incident(bad, L0, L1)
    t = modes.dual_column(col)
    np.testing.assert_array_equal(t[:2 * pl], col[2 * pl:])
    np.testing.assert_array_equal(modes.dual_column(col, forward=False), -t)
