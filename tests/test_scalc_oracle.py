"""The S-matrix oracle (oracle/scalc_oracle.py, a numpy restatement of
Smat/Scalc.c) against the stock Scalc's own output (tests/golden/scalc_*.npz,
written by tests/golden/make_scalc.py from decks whose port modes come from
the stock Mcalc)."""
import glob
import os

import numpy as np
import pytest

from oracle import scalc_oracle as SO

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "scalc_*.npz")))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_smatrix_matches_stock_scalc(path):
    g = np.load(path)
    L = g["L"]
    nB, nT = (int(x) for x in g["nreal"])
    S = SO.smatrix(list(g["meds"]), float(g["omega"]), int(L[0]), int(L[1]), tuple(int(x) for x in g["bc"]),
                   g["XiB"], nB, g["XiT"], nT)
    assert np.abs(S - g["S"]).max() < 1e-12
    u, t = SO.check_smat(S)
    assert u < 1e-12 and t < 1e-12  # a lossless reciprocal structure: unitary and symmetric


def test_fixtures_exist():
    assert len(FIXTURES) >= 2


def test_forward_only_fills_the_first_columns():
    g = np.load(FIXTURES[0])
    L = g["L"]
    nB, nT = (int(x) for x in g["nreal"])
    S1 = SO.smatrix(list(g["meds"]), float(g["omega"]), int(L[0]), int(L[1]), tuple(int(x) for x in g["bc"]),
                    g["XiB"], nB, g["XiT"], nT, both_ways=False)
    np.testing.assert_allclose(S1[:, :nB], g["S"][:, :nB], atol=1e-12)
