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
