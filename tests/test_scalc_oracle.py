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


@pytest.mark.parametrize("L0,L1,eps,om", [(6, 5, 2.085, 0.405), (8, 8, 1.0, 0.7), (5, 7, 4.0, 0.3)])
def test_plane_wave_basis_is_mcalcs_basis(L0, L1, eps, om):
    """The closed-form port basis of a uniform periodic layer (workloads.plane_wave_basis)
    against the dense reference algorithm (mode_oracle.calc_Xi): the same thetas, a
    biorthonormal Xi, and S matrices with the same singular values (the basis inside a
    degenerate group is free)."""
    from oracle import mode_oracle as MO
    from smatranem_gb300 import workloads as W
    th, Xi, nr = W.plane_wave_basis(L0, L1, eps, om)
    med = W.port_layer(L0, L1, core=(0, 0), eps_core=eps, eps_clad=eps)
    ref = MO.calc_Xi(med, om, L0, L1, (1, 1))
    N = 2 * L0 * L1
    assert nr == ref["num_real"]
    assert np.abs(np.sort_complex(th) - np.sort_complex(ref["theta"])).max() < 1e-12
    assert MO.check_Xi(N, nr, Xi) < 1e-12
    meds = W.grating_layers(L0, L1, 5, eps_port=eps, seed=3)
    S = SO.smatrix(list(meds), om, L0, L1, (1, 1), Xi, nr, Xi, nr)
    S2 = SO.smatrix(list(meds), om, L0, L1, (1, 1), ref["Xi"], nr, ref["Xi"], nr)
    assert SO.check_smat(S)[0] < 1e-11
    sv = np.sort(np.linalg.svd(S, compute_uv=False))
    assert np.abs(sv - np.sort(np.linalg.svd(S2, compute_uv=False))).max() < 1e-11
