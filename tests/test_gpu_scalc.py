"""GPU layer-transfer S matrix (smat_scalc) against the reference S-matrix
program (Smat/Scalc.c).

* the LU solve behind it (smat_zgesv) against numpy on random, pivoting-heavy
  and singular systems (block sizes straddling the 32-column panels);
* the S matrix against the stock Scalc's own output on its fixtures
  (tests/golden/scalc_*.npz) and against the oracle restatement on larger
  seeded structures (lossy inner layers, every BoundC);
* the tensor-core product (smat_zgemm mode 1: FP64-accurate complex products
  from bf16 slices, Ozaki scheme) against an extended-precision product, per
  entry within its error bound, on ragged sizes, wide dynamic ranges, zero
  rows and columns; the stock-Scalc comparisons in both dense modes;
* the argument checks.
Tolerance: 1e-10 absolute on S entries (|S| <= 1); the reference's own
unitarity residual is 2e-14 on these cases.
"""
import glob
import os

import numpy as np
import pytest

from oracle import scalc_oracle as SO
from smatranem_gb300 import fdtd, scalc, workloads as W

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "scalc_*.npz")))


@pytest.mark.parametrize("n,nrhs", [(1, 1), (5, 3), (31, 7), (32, 32), (33, 40), (100, 64), (257, 300)])
def test_zgesv_matches_numpy(dense, n, nrhs):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A[np.arange(n), np.arange(n)] *= 1e-3  # small diagonal: every column pivots
    B = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    X, info = scalc.zgesv(A, B)
    assert info == 0
    ref = np.linalg.solve(A, B)
    assert np.abs(X - ref).max() <= 1e-10 * np.abs(ref).max()
    assert np.abs(A @ X - B).max() <= 1e-11 * np.abs(A).max() * np.abs(X).max() * n


def test_zgesv_reports_a_zero_pivot(built):
    A = np.eye(6, dtype=complex)
    A[3, 3] = 0.0
    _, info = scalc.zgesv(A, np.ones(6))
    assert info == 4  # 1-based, as LAPACK's INFO


def _zgemm_case(rng, m, n, k, spread):
    A = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))) * 10.0 ** rng.uniform(-spread, spread, (m, 1))
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))) * 10.0 ** rng.uniform(-spread, spread, (1, n))
    if spread:  # entries far below their row's / column's largest, zero rows and columns
        A *= 10.0 ** rng.uniform(-6, 0, (m, k))
        A[m // 3, :] = 0
        B[:, n // 2] = 0
    return A, B


@pytest.mark.parametrize("m,n,k,spread", [(1, 1, 1, 0), (128, 32, 32, 0), (129, 33, 31, 0), (300, 70, 17, 3),
                                          (500, 260, 100, 0), (77, 500, 64, 8), (300, 40, 2048, 0)])
def test_zgemm_tensor_cores_within_bound(built, m, n, k, spread):
    """Per entry: |C - exact| <= 2e-15 k max|A row| max|B col| + 4 ulp of |C0| + |C|
    (the slices keep 55 bits of each scaled entry; the dropped slice pairs and
    the FP64 sums stay below that), the FP64 kernel on the same inputs."""
    rng = np.random.default_rng(m + 7 * n + 13 * k)
    A, B = _zgemm_case(rng, m, n, k, spread)
    C0 = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    alpha = 0.3 - 0.7j
    exact = C0.astype(np.clongdouble) + alpha * (A.astype(np.clongdouble) @ B.astype(np.clongdouble))
    rm = np.abs(np.concatenate([A.real, A.imag], axis=1)).max(axis=1, keepdims=True)
    cm = np.abs(np.concatenate([B.real, B.imag], axis=0)).max(axis=0, keepdims=True)
    for mode in (1, 0):
        got = scalc.zgemm(A, B, C0, alpha, mode=mode)
        err = np.abs(got - exact).astype(np.float64)
        bound = 2e-15 * k * abs(alpha) * rm * cm + 9e-16 * (np.abs(C0) + np.abs(got))
        assert np.all(err <= bound), (mode, float((err / bound).max()))


def test_zgemm_bounded_wait_gives_up(built):
    """A tensor-core product whose slice pair never arrives: its waits run out,
    it records error 1 and returns (no hang, no fault), and the next product
    on the device is right."""
    assert scalc.zgemm_wait_test() == 1
    rng = np.random.default_rng(5)
    A = rng.standard_normal((130, 20)) + 1j * rng.standard_normal((130, 20))
    B = rng.standard_normal((20, 40)) + 1j * rng.standard_normal((20, 40))
    got = scalc.zgemm(A, B, mode=1)
    assert np.abs(got - A @ B).max() <= 1e-13 * np.abs(A).max() * np.abs(B).max() * 20


def test_zgemm_argument_checks(built):
    with pytest.raises(ValueError):
        scalc.zgemm(np.ones((3, 2)), np.ones((3, 2)))  # inner sizes differ
    with pytest.raises(fdtd.FdtdError):
        scalc.zgemm(np.ones((3, 2)), np.ones((2, 2)), mode=2)
    with pytest.raises(fdtd.FdtdError):
        scalc.dense_mode(5)


@pytest.fixture(params=[1, 0], ids=["tensor_cores", "fp64_kernel"])
def dense(request, built):
    scalc.dense_mode(request.param)
    yield request.param
    scalc.dense_mode(1)


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_smatrix_matches_stock_scalc(dense, path):
    g = np.load(path)
    L = g["L"]
    nB, nT = (int(x) for x in g["nreal"])
    S, info = scalc.smatrix(g["meds"], float(g["omega"]), int(L[0]), int(L[1]), tuple(int(x) for x in g["bc"]),
                            g["XiB"], nB, g["XiT"], nT)
    assert np.abs(S - g["S"]).max() < 1e-10
    assert abs(info["unitarity"] - float(g["unitarity"])) < 1e-11
    nl = len(g["meds"])
    assert info["solves"] == 2 * (2 + 2 * (nl - 2) + 2)  # per direction: set_iniMat, 2 per layer... as Scalc


def _case(L0, L1, nl, bc, seed, lossy):
    from oracle import mode_oracle as MO
    om = 0.405
    med = W.port_layer(L0, L1, core=(3, 2), eps_core=12.11, eps_clad=2.085, seed=seed, jitter=0.2)
    port = MO.calc_Xi(med, om, L0, L1, bc)
    rng = np.random.default_rng(seed)
    meds = [med]
    for _ in range(nl - 2):
        m = med.copy()
        k = rng.integers(0, L0 * L1, size=max(1, L0 * L1 // 6))
        for r in (2, 3, 4):
            m[r, k] = rng.uniform(2.0, 12.0, size=k.size) + (1j * rng.uniform(0.0, 0.3, size=k.size) if lossy else 0)
        meds.append(m)
    meds.append(med)
    return om, np.array(meds), port["Xi"], port["num_real"]


@pytest.mark.parametrize("L0,L1,nl,bc,lossy", [(8, 6, 6, (0, 0), False), (7, 7, 5, (1, -1), True),
                                               (9, 5, 4, (-1, 1), False), (6, 6, 2, (1, 1), False)])
def test_smatrix_matches_oracle(dense, L0, L1, nl, bc, lossy):
    om, meds, Xi, nr = _case(L0, L1, nl, bc, L0 + 10 * L1, lossy)
    ref = SO.smatrix(list(meds), om, L0, L1, bc, Xi, nr, Xi, nr)
    S, info = scalc.smatrix(meds, om, L0, L1, bc, Xi, nr, Xi, nr)
    assert np.abs(S - ref).max() < 1e-10
    if not lossy:
        assert info["unitarity"] < 1e-10
    one, _ = scalc.smatrix(meds, om, L0, L1, bc, Xi, nr, Xi, nr, both_ways=False)
    assert np.abs(one[:, :nr] - ref[:, :nr]).max() < 1e-10


def test_smatrix_argument_checks(built):
    g = np.load(FIXTURES[0])
    L = g["L"]
    nB, nT = (int(x) for x in g["nreal"])
    meds = g["meds"].copy()
    meds[0, 2, 0] += 0.1j  # a lossy port layer: "V is not real in initial_calc"
    with pytest.raises(fdtd.FdtdError) as e:
        scalc.smatrix(meds, float(g["omega"]), int(L[0]), int(L[1]), (0, 0), g["XiB"], nB, g["XiT"], nT)
    assert e.value.code == -1
    with pytest.raises(fdtd.FdtdError):
        scalc.smatrix(g["meds"][:1], float(g["omega"]), int(L[0]), int(L[1]), (0, 0), g["XiB"], nB, g["XiT"], nT)


def test_grating_with_plane_wave_ports(built):
    """The bench's workload form at a small size: closed-form port basis, seeded grating."""
    L0, L1, om = 10, 8, 0.405
    th, Xi, nr = W.plane_wave_basis(L0, L1, omega=om)
    meds = W.grating_layers(L0, L1, 6, seed=7)
    ref = SO.smatrix(list(meds), om, L0, L1, (1, 1), Xi, nr, Xi, nr)
    S, info = scalc.smatrix(meds, om, L0, L1, (1, 1), Xi, nr, Xi, nr)
    assert np.abs(S - ref).max() < 1e-10
    assert info["unitarity"] < 1e-10
