"""The library's host precompute (product code) against the golden vectors."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden

CASES = golden_cases()


@pytest.mark.parametrize("name", CASES)
def test_library_precompute_matches_golden(built, name):
    from smatranem_gb300 import fdtd
    g = load_golden(name)
    L = g["L"]
    sig = fdtd.set_sigma(L, g["mu_in"], g["epsi_in"])
    assert np.array_equal(sig, g["sigma"])
    mu, ep = fdtd.remove_sigma(L, g["mu_in"], g["epsi_in"], sig)
    assert np.array_equal(mu, g["mu"]) and np.array_equal(ep, g["epsi"])
    cont, addr, ln = fdtd.set_address(L, sig, mu, ep)
    assert np.array_equal(cont, g["cont"]) and np.array_equal(addr, g["addr"]) and ln == int(g["lnotn"])
    n2, r, i = fdtd.set_tau(float(g["omega"]), float(g["min_dt"]))
    assert (n2, r, i) == (int(g["n2pi"]), float(g["invtau_R"]), float(g["invtau_I"]))
    coef = fdtd.coefficients(L, ln, sig, mu, ep, cont, addr, r, i)
    for a, key in zip(coef, ("Ah", "Bh", "Ae", "Be")):
        assert np.array_equal(a, g[key])
    tp = g["time_period"]
    env = np.array([[fdtd.set_env(n2, tp, jh, jt, jp) for jh in (0, 1) for jt in (0, n2 // 3, n2 - 1)]
                    for jp in range(int(tp[2]))])
    assert np.array_equal(env, g["env"])


def test_cw_schedule_matches_oracle_loop(built, port):
    """The schedule table reproduces the reference loop's Ei/Hi and phases."""
    import oracle
    from smatranem_gb300 import fdtd
    n2, tp = 37, (2, 1, 5)
    src, ph = fdtd.cw_schedule(n2, tp)
    expn = oracle.expn_table(n2)
    for k in (0, 5, n2 - 1, n2, 3 * n2 + 7, 5 * n2 - 1):
        jp, jt = divmod(k, n2)
        jn = (jt + 1) % n2
        assert src[k, 0] == 2.0 * port.set_env(n2, tp, 1, jt, jp)
        assert src[k, 3] == 2.0 * port.set_env(n2, tp, 0, jt + 1, jp)
        assert (src[k, 1], src[k, 2]) == (expn[1 + 2 * jt].real, expn[1 + 2 * jt].imag)
        assert (src[k, 4], src[k, 5]) == (expn[2 * jn].real, expn[2 * jn].imag)
        assert tuple(ph[k, 0]) == (expn[2 * jn].real, expn[2 * jn].imag, expn[2 * jn + 1].real,
                                   expn[2 * jn + 1].imag)


def test_precompute_errors(built):
    from smatranem_gb300 import fdtd
    with pytest.raises(fdtd.FdtdError):
        fdtd.set_tau(-1.0, 0.1)
    assert np.isnan(fdtd.set_env(10, (1, 1, 3), 0, 0, 3))  # beyond stop-period: the reference exits
    # media that the sigma profile does not explain: remove_sigma refuses (the reference exits)
    L = (4, 4, 6, 1)
    mu = np.ones(3 * 96, np.complex128)
    ep = np.ones(3 * 96, np.complex128)
    sig = np.zeros(2 * 14)
    sig[2 * 8 + 0] = 3.0
    with pytest.raises(fdtd.FdtdError):
        fdtd.remove_sigma(L, mu, ep, sig)


def test_precompute_independent_of_host_threads(built, monkeypatch):
    """set_address and the coefficient build split their planes over host
    worker threads: cell classes, addresses and coefficients are the same
    bits for every thread count (every cell class, ragged plane splits, more
    threads than planes)."""
    from smatranem_gb300 import fdtd
    from smatranem_gb300 import workloads as W
    s = W.random_structure((23, 17, 29, 2), seed=7, pml=(3, 3, 4), metals=0.04, lossy=0.05, pec=0.02)
    pr = W.prepare(s)
    out = {}
    for nt in (1, 2, 5, 29, 64):
        monkeypatch.setenv("SMATRAN_HOST_THREADS", str(nt))
        cont, addr, ln = fdtd.set_address(s.L, pr.sigma, pr.mu, pr.epsi)
        coef = fdtd.coefficients(s.L, ln, pr.sigma, pr.mu, pr.epsi, cont, addr, pr.invtau_R, pr.invtau_I)
        out[nt] = (cont, addr, ln, coef)
    assert set(np.unique(out[1][0])) >= {ord(c) for c in "naheb"}
    for nt in (2, 5, 29, 64):
        assert np.array_equal(out[1][0], out[nt][0]) and np.array_equal(out[1][1], out[nt][1])
        assert out[1][2] == out[nt][2]
        for a, b in zip(out[1][3], out[nt][3]):
            assert np.array_equal(a, b), nt


def test_host_threads_setting(built, monkeypatch):
    """SMATRAN_HOST_THREADS sets the precompute's worker threads (1..64);
    unset or out of range, small grids take one thread and large ones one per
    core, at most 16."""
    import ctypes
    import os
    from smatranem_gb300 import fdtd
    ht = fdtd.lib().host_threads
    ht.argtypes = [ctypes.c_longlong]
    ht.restype = ctypes.c_int
    for v, small in (("1", 1), ("5", 5), ("64", 64)):
        monkeypatch.setenv("SMATRAN_HOST_THREADS", v)
        assert ht(10) == small and ht(1 << 22) == small
    cores = min(os.cpu_count() or 1, 16)
    for v in ("65", "0", "x"):
        monkeypatch.setenv("SMATRAN_HOST_THREADS", v)
        assert ht(10) == 1 and 1 <= ht(1 << 22) <= 16
    monkeypatch.delenv("SMATRAN_HOST_THREADS")
    assert ht(10) == 1 and ht(1 << 22) == cores


def test_host_parallel_for_covers_each_index_once(built):
    """The precompute's range splitter: for any count and thread count
    (more threads than items, none, past the cap) every index of [0, n) is
    handed out exactly once, in contiguous ranges."""
    import ctypes
    from smatranem_gb300 import fdtd
    fn_t = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong)
    pf = fdtd.lib().host_parallel_for
    pf.argtypes = [ctypes.c_longlong, ctypes.c_int, fn_t, ctypes.c_void_p]
    pf.restype = None
    for n, nt in [(0, 4), (1, 1), (1, 8), (7, 3), (100, 16), (5, 64), (1000, 100), (33, 0), (33, -2)]:
        seen = np.zeros(n, np.int64)
        ranges = []

        def cb(ctx, lo, hi):
            ranges.append((lo, hi))
            seen[lo:hi] += 1

        pf(n, nt, fn_t(cb), None)
        assert np.all(seen == 1), (n, nt)
        assert all(lo < hi for lo, hi in ranges) and len(ranges) <= max(1, min(nt, 64, n))
