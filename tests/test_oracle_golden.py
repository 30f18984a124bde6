"""The oracle port against the reference: golden vectors and live runs.

Golden vectors (tests/golden/*.npz) were produced by the reference's own code
(tests/golden/make_golden.py).  Live comparisons need the reference sources and
are skipped where they are absent.  Bit-for-bit: the port keeps the
reference's operation order and is compiled with the same flags.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden

CASES = golden_cases()


@pytest.mark.parametrize("name", CASES)
def test_port_precompute_matches_golden(port, name):
    g = load_golden(name)
    L = g["L"]
    sig = port.set_sigma(L, g["mu_in"], g["epsi_in"])
    assert np.array_equal(sig, g["sigma"])
    mu, ep = port.remove_sigma(L, g["mu_in"], g["epsi_in"], sig)
    assert np.array_equal(mu, g["mu"]) and np.array_equal(ep, g["epsi"])
    cont, addr, ln = port.set_address(L, sig, mu, ep)
    assert np.array_equal(cont, g["cont"]) and np.array_equal(addr, g["addr"]) and ln == int(g["lnotn"])
    n2, r, i = port.set_tau(float(g["omega"]), float(g["min_dt"]))
    assert (n2, r, i) == (int(g["n2pi"]), float(g["invtau_R"]), float(g["invtau_I"]))


@pytest.mark.parametrize("name", CASES)
def test_port_envelope_matches_golden(port, name):
    g = load_golden(name)
    n2, tp = int(g["n2pi"]), g["time_period"]
    env = np.array([[port.set_env(n2, tp, jh, jt, jp) for jh in (0, 1) for jt in (0, n2 // 3, n2 - 1)]
                    for jp in range(int(tp[2]))])
    assert np.array_equal(env, g["env"])


@pytest.mark.parametrize("name", CASES)
def test_port_time_loop_matches_golden(port, name):
    g = load_golden(name)
    H, E = g["H0"].copy(), g["E0"].copy()
    mons = [np.zeros_like(g["HB"]) for _ in range(4)]
    rc = port.time_loop(g["L"], g["Ah"], g["Bh"], g["Ae"], g["Be"], g["iBc"], H, E, g["iBTIin"], g["Hinc"],
                        g["Einc"], int(g["n2pi"]), g["time_period"], 0, int(g["nsteps"]), *mons, g["cont"],
                        g["addr"])
    assert (rc != 0) == (int(g["ref_exits"]) > 0)  # a PML cell on a monitor plane
    assert np.array_equal(H, g["H"])
    assert np.array_equal(E, g["E"])
    for m, key in zip(mons, ("HB", "EB", "HT", "ET")):
        assert np.array_equal(m, g[key])


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_port_main_calc_matches_reference_live(port, reference, seed):
    from smatranem_gb300 import workloads as W
    L = (9, 8, 11, 2)
    s = W.random_structure(L, seed=seed, pml=(2, 2, 2), metals=0.05, lossy=0.05, iBc=(seed % 3 - 1, 1, 0))
    mu = np.ascontiguousarray(s.mu.reshape(-1))
    ep = np.ascontiguousarray(s.epsi.reshape(-1))
    out = []
    for o in (port, reference):
        sig = o.set_sigma(L, mu, ep)
        m2, e2 = o.remove_sigma(L, mu, ep, sig)
        cont, addr, ln = o.set_address(L, sig, m2, e2)
        n2, r, i = o.set_tau(s.omega, s.min_dt)
        out.append((sig, m2, e2, cont, addr, ln, n2, r, i))
    for a, b in zip(*out):
        assert np.array_equal(a, b)
    sig, m2, e2, cont, addr, ln, n2, r, i = out[0]
    coef = port.coefficients(L, ln, sig, m2, e2, cont, addr, r, i)
    n3, pl = L[0] * L[1] * L[2], L[0] * L[1]
    H0, E0 = W.random_fields(n3, ln, seed=seed)
    rng = np.random.default_rng(seed)
    Hi, Ei = rng.standard_normal(2 * pl), rng.standard_normal(2 * pl)
    expn2 = np.exp(1j * rng.uniform(0, 6.28, 2))
    res = []
    for o in (port, reference):
        H, E = H0.copy(), E0.copy()
        mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
        for _ in range(3):
            o.main_calc(L, *coef, s.iBc, H, E, (3, 7, 5, -1), Hi, Ei, expn2, *mons, cont, addr)
        res.append((H, E, *mons))
    for a, b in zip(*res):
        assert np.array_equal(a, b)
