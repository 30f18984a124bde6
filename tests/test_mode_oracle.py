"""The mode-solver oracle (oracle/mode_oracle.py, a numpy restatement of
ModeCalc/Mcalc.c calc_Xi) against the stock reference Mcalc's own output
(tests/golden/modes_*.npz, written by tests/golden/make_modes.py)."""
import glob
import os

import numpy as np
import pytest

from oracle import mode_oracle as MO

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "modes_*.npz")))


def _fit_sign(a, b):
    """a scaled by the unit factor that best matches b (eigenvector gauge)."""
    ph = np.vdot(a, b) / np.vdot(a, a)
    return a * (ph / abs(ph))


@pytest.fixture(scope="module", params=FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def case(request):
    g = dict(np.load(request.param))
    L0, L1 = int(g["L0"]), int(g["L1"])
    r = MO.calc_Xi(g["med"], float(g["omega"]), L0, L1, tuple(int(x) for x in g["bc"]))
    return g, r


def test_fixtures_exist():
    assert len(FIXTURES) >= 4


def test_real_modes_and_thetas(case):
    g, r = case
    N = 2 * int(g["L0"]) * int(g["L1"])
    nr = int(g["num_real"])
    assert r["num_real"] == nr and r["real_matrix"] == bool(g["real_matrix"])
    th, ref = r["theta"], g["theta"]
    # propagating modes: same order (descending theta), same values
    np.testing.assert_allclose(th[:nr], ref[:nr], rtol=0, atol=1e-12)
    np.testing.assert_allclose(th[N:N + nr], ref[N:N + nr], rtol=0, atol=1e-12)
    # evanescent ones: the same multiset (near-ties may be ordered differently)
    key = lambda z: np.lexsort((np.round(z.real, 9), np.round(z.imag, 9)))  # noqa: E731
    a, b = th[nr:N], ref[nr:N]
    np.testing.assert_allclose(a[key(a)], b[key(b)], rtol=0, atol=1e-9)


def test_xi_columns_of_real_modes(case):
    g, r = case
    N = 2 * int(g["L0"]) * int(g["L1"])
    nr = int(g["num_real"])
    K = min(g["xi_fwd"].shape[1], nr)
    for j in range(K):
        for mine, ref in ((r["Xi"][:, j], g["xi_fwd"][:, j]), (r["Xi"][:, N + j], g["xi_bwd"][:, j])):
            err = np.abs(_fit_sign(mine, ref) - ref).max() / np.abs(ref).max()
            assert err < 1e-9, (j, err)
        # an incident column must have exactly real E rows (FDTD set_incident :503);
        # degeneXi's complex mixing (the later mode of a degenerate pair) leaves
        # rounding-level imaginary parts there, in the reference too
        mixed = {i for _, i in g["degenerate"]}
        imag = np.abs(r["Xi"][N:, j].imag).max()
        assert imag == 0.0 if j not in mixed else imag < 1e-15 * np.abs(r["Xi"][N:, j]).max()


def test_biorthogonality(case):
    g, r = case
    assert r["check"] < 1e-9 and float(g["check"]) < 1e-9


def test_degenerate_pairs_are_reported_alike(case):
    g, r = case
    ref_pairs = {tuple(p) for p in g["degenerate"]}
    mine = {(j, i) for j, i, _ in r["degenerate"]}
    assert mine == ref_pairs


def test_lossy_layer_is_rejected_like_the_reference():
    from smatranem_gb300 import workloads as W
    med = W.port_layer(6, 5, core=(2, 2), loss=0.05, seed=5)
    with pytest.raises(ValueError):
        MO.calc_Xi(med, 0.4, 6, 5, (0, 0))
