"""GPU port-mode solver (smat_mode_solve) against the reference mode solver.

* the maa / mbb stencils against Mcalc's dense set_M matrices (oracle);
* the returned modes against the stock Mcalc's own output (golden fixtures,
  tests/golden/modes_*.npz) and against the oracle restatement on layers too
  large for a fixture, including degenerate clusters (compared as subspaces);
* a 128 x 96 uniform periodic layer against its closed-form spectrum;
* the 256 x 192 bend port (the FDTD workload's cross-section): convergence,
  biorthogonality, physical effective indices;
* an FDTD run excited and projected with the solver's modes gives the same
  |S|^2 as the run with the oracle's modes.
Tolerances: theta 1e-10 absolute (the reference's dgeev is accurate to about
1e-14 here, the iterative solve to its 1e-12 residual), Xi columns 1e-8
relative after the sign gauge, |S|^2 1e-9 relative.
"""
import glob
import os

import numpy as np
import pytest

from oracle import mode_oracle as MO
from smatranem_gb300 import fdtd as f, modes, workloads as W

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "modes_*.npz")))


def _fit_sign(a, b):
    ph = np.vdot(a, b) / np.vdot(a, a)
    return a * (ph / abs(ph))


def _span_residual(A, B):
    """largest relative distance of A's columns from span(B)"""
    c, *_ = np.linalg.lstsq(B, A, rcond=None)
    return (np.linalg.norm(A - B @ c, axis=0) / np.linalg.norm(A, axis=0)).max()


def _biortho(ms: modes.Modes):
    """||tilde-Xi^H Xi - 1|| over the returned modes (checkXi :237-280 restricted)"""
    k, K = ms.n_found, ms.nmodes
    cols = list(range(k)) + [K + j for j in range(k)]
    Xi = ms.Xi[:, cols]
    T = np.stack([modes.dual_column(ms.Xi[:, j]) for j in range(k)] +
                 [modes.dual_column(ms.Xi[:, K + j], forward=False) for j in range(k)], axis=1)
    C = T.conj().T @ Xi
    return np.abs(C - np.eye(2 * k)).max()


@pytest.mark.parametrize("L0,L1,bc", [(7, 5, (0, 0)), (6, 4, (1, -1)), (5, 6, (-1, 1)), (1, 6, (1, 0)),
                                      (6, 1, (0, 1)), (1, 1, (1, -1)), (33, 17, (1, 1))])
def test_stencils_match_mcalc_matrices(built, L0, L1, bc):
    med = W.port_layer(L0, L1, core=(min(3, L0), min(2, L1)), metric=0.2, seed=L0 + 7 * L1)
    om = 0.37
    V, _ = MO.set_V(med, om)
    maa, mbb = MO.set_M(bc, L0, L1, V)
    X = np.random.default_rng(1).standard_normal((2 * L0 * L1, 3))
    for which, M in ((0, maa.real), (1, mbb.real), (2, (mbb @ maa).real)):
        Y = modes.apply(med, om, L0, L1, bc, which, X)
        ref = M @ X
        assert np.abs(Y - ref).max() <= 1e-13 * np.abs(ref).max(), which


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_modes_match_stock_mcalc(built, path):
    g = np.load(path)
    L0, L1 = int(g["L0"]), int(g["L1"])
    N = 2 * L0 * L1
    nr = int(g["num_real"])
    k = min(nr, g["xi_fwd"].shape[1], 8)
    ms = modes.solve(g["med"], float(g["omega"]), L0, L1, tuple(int(x) for x in g["bc"]), k)
    assert ms.n_found == k, ms.info
    np.testing.assert_allclose(ms.theta[:k], g["theta"][:k], rtol=0, atol=1e-10)
    np.testing.assert_allclose(ms.theta[k:2 * k], g["theta"][N:N + k], rtol=0, atol=1e-10)
    degenerate = {i for p in g["degenerate"] for i in p if i < k}
    for j in range(k):
        fw, bw = ms.Xi[:, j], ms.Xi[:, k + j]
        assert np.all(fw[N:].imag == 0.0) or j in degenerate  # an incident column (set_incident :503)
        if j in degenerate:
            continue
        for mine, ref in ((fw, g["xi_fwd"][:, j]), (bw, g["xi_bwd"][:, j])):
            assert np.abs(_fit_sign(mine, ref) - ref).max() <= 1e-8 * np.abs(ref).max(), j
    if degenerate:
        idx = sorted(degenerate)
        assert _span_residual(ms.Xi[:, idx], g["xi_fwd"][:, idx]) < 1e-8
        assert _span_residual(ms.Xi[:, [k + i for i in idx]], g["xi_bwd"][:, idx]) < 1e-8
    assert _biortho(ms) < 1e-9


@pytest.mark.parametrize("L0,L1,bc,kw,om,k", [
    (24, 18, (0, 0), dict(core=(8, 5), eps_core=12.11, eps_clad=2.085, seed=11, metric=0.15), 0.405, 6),
    (26, 20, (1, -1), dict(core=(9, 4), eps_core=12.11, eps_clad=2.085, seed=12, jitter=0.2), 0.2, 5),
    (30, 22, (0, 0), dict(core=(10, 6), eps_core=12.11, eps_clad=2.085, seed=13), 0.1, 4),
    (20, 20, (1, 1), dict(core=(0, 0), eps_core=2.085, eps_clad=2.085, seed=14), 0.405, 6),
])
def test_modes_match_oracle(built, L0, L1, bc, kw, om, k):
    med = W.port_layer(L0, L1, **kw)
    ref = MO.calc_Xi(med, om, L0, L1, bc)
    N = 2 * L0 * L1
    k = min(k, ref["num_real"])
    ms = modes.solve(med, om, L0, L1, bc, k)
    assert ms.n_found == k, ms.info
    np.testing.assert_allclose(ms.theta[:k], ref["theta"][:k], rtol=0, atol=1e-10)
    # clusters (relative theta gap below 1e-6) compared as subspaces
    th = ref["theta"][:k].real
    groups, cur = [], [0]
    for j in range(1, k):
        if abs(th[j] - th[j - 1]) <= 1e-6 * abs(th[j]):
            cur.append(j)
        else:
            groups.append(cur)
            cur = [j]
    groups.append(cur)
    for grp in groups:
        if len(grp) == 1:
            j = grp[0]
            for mine, r in ((ms.Xi[:, j], ref["Xi"][:, j]), (ms.Xi[:, k + j], ref["Xi"][:, N + j])):
                assert np.abs(_fit_sign(mine, r) - r).max() <= 1e-8 * np.abs(r).max(), j
        elif grp[-1] + 1 < k or ref["theta"][k].real < th[grp[-1]] * (1 - 1e-6):
            assert _span_residual(ms.Xi[:, grp], ref["Xi"][:, grp]) < 1e-8
    assert _biortho(ms) < 1e-9


def test_uniform_periodic_layer_closed_form(built):
    """Uniform isotropic medium, periodic: mbb*maa = w^2 eps mu - (C^T C + G G^T),
    eigenvalues w^2 eps mu - 4 sin^2(pi p/L0) - 4 sin^2(pi q/L1), each twice."""
    L0, L1, eps, om = 128, 96, 2.085, 0.4
    med = W.port_layer(L0, L1, core=(0, 0), eps_core=eps, eps_clad=eps)
    p = np.arange(L0)[:, None]
    q = np.arange(L1)[None, :]
    lam = np.sort((om * om * eps - 4 * np.sin(np.pi * p / L0) ** 2 - 4 * np.sin(np.pi * q / L1) ** 2).ravel())[::-1]
    lam = np.repeat(lam, 2)
    k = 6  # clusters of 2 and 4: the block boundary falls between clusters
    ms = modes.solve(med, om, L0, L1, (1, 1), k)
    assert ms.n_found == k, ms.info
    theta = 2 * np.arcsin(np.sqrt(lam[:k]) / 2)
    np.testing.assert_allclose(ms.theta[:k].real, theta, rtol=0, atol=1e-10)
    assert ms.info["degenerate_pairs"] >= 1 + 6  # pairs within the two clusters
    assert _biortho(ms) < 1e-9


def test_bend_port_modes(built):
    """The 256 x 192 port of the bend workload: TE0/TM0-like guided modes with
    effective indices between the cladding and the core."""
    b = W.bend_structure(shape=(256, 192, 48))
    med = b.port_med
    ms = modes.solve(med, b.s.omega, 256, 192, (0, 0), 4)
    assert ms.n_found == 4, ms.info
    assert ms.info["max_residual"] <= 1e-12
    th = ms.theta[:4].real
    assert np.all(np.diff(th) <= 0)
    assert _biortho(ms) < 1e-9
    for j in range(4):
        assert np.all(ms.Xi[2 * 256 * 192:, j].imag == 0.0)


def _guide_run(s, ms, iB, iT, iI, nper=(2, 6, 10)):
    """FP64 CW run excited by forward mode 1 of ms; |S|^2 of every returned
    mode at the two monitor planes (S_calc :437-445 with ms's dual columns)."""
    pr = W.prepare(s)
    L = s.L
    with f.Plan.create(L, s.iBc, (iB, iT, iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma) as p:
        Hinc, Einc = ms.incident(1)
        p.set_incident(0, Hinc, Einc)
        p.set_cw_schedule(pr.n2pi, nper)
        p.run(0, pr.n2pi * nper[2])
        HB, EB, HT, ET = p.get_monitor(0)
    out = []
    for Hm, Em in ((HB, EB), (HT, ET)):
        v = np.concatenate([Hm[0::2], Hm[1::2], -Em[1::2], Em[0::2]])
        for m in range(1, ms.n_found + 1):
            for sgn in (1, -1):
                out.append(abs(np.vdot(ms.dual(sgn * m), v)) ** 2)
    return np.array(out)


def test_fdtd_with_solver_modes_matches_oracle_modes(built):
    L0, L1, L2, L3 = 14, 12, 22, 6
    med = W.port_layer(L0, L1, core=(5, 3), eps_core=12.11, eps_clad=2.085, seed=21)
    om = 0.405
    s = W.waveguide_structure(med, L0, L1, L2, L3, omega=om, pml_z=3)
    ref = MO.calc_Xi(med, om, L0, L1, (0, 0))
    k = min(3, ref["num_real"])
    mine = modes.solve(med, om, L0, L1, (0, 0), k)
    N = 2 * L0 * L1
    cols = list(range(k)) + [N + j for j in range(k)]
    theirs = modes.Modes(L0=L0, L1=L1, theta=ref["theta"][cols], Xi=ref["Xi"][:, cols], info={"n_found": k})
    iB, iT, iI = 4, L2 - 5, 5
    s1 = _guide_run(s, mine, iB, iT, iI)
    s2 = _guide_run(s, theirs, iB, iT, iI)
    assert np.abs(s1 - s2).max() <= 1e-9 * s2.max()
    # the excited mode carries most of the transmitted power
    assert s1[2 * k] > 10 * max(s1[2 * k + 2:].max(), 1e-30), s1


@pytest.mark.parametrize("k", [2, 3, 16, 40])
def test_fewer_propagating_modes_than_asked(built, k):
    """A 5 x 4 layer with two propagating modes (the golden mode deck's port):
    asking for more returns those two; a block as large as the space works."""
    g = np.load(os.path.join(HERE, "golden", "decks", "deck_modes", "media.npz"))
    med = g["port_med"]
    om = 2 * np.pi / (1.55e-6 * 1.0e7)
    ref = MO.calc_Xi(med, om, 5, 4, (0, 0))
    assert ref["num_real"] == 2
    ms = modes.solve(med, om, 5, 4, (0, 0), k)
    assert ms.n_found == 2, ms.info
    np.testing.assert_allclose(ms.theta[:2], ref["theta"][:2], rtol=0, atol=1e-10)
    assert np.all(ms.Xi[:, 2:k] == 0) and np.all(ms.Xi[:, k + 2:] == 0)


def test_fp32_filter_passes_give_the_fp64_result(built):
    """The default FP32 filter passes (until the residuals reach 1e-6) end at the
    same eigenpairs as FP64 passes throughout."""
    med = W.port_layer(24, 18, core=(8, 5), eps_core=12.11, eps_clad=2.085, seed=11, metric=0.15)
    a = modes.solve(med, 0.405, 24, 18, (0, 0), 5)
    b = modes.solve(med, 0.405, 24, 18, (0, 0), 5, fp64_only=True)
    assert a.info["matvecs_fp32"] > 0 and b.info["matvecs_fp32"] == 0
    np.testing.assert_allclose(a.theta, b.theta, rtol=0, atol=1e-12)
    for j in range(5):
        assert np.abs(_fit_sign(a.Xi[:, j], b.Xi[:, j]) - b.Xi[:, j]).max() < 1e-9


def test_one_and_two_pass_stencils_agree_bit_for_bit(built):
    """The two-pass stencils (curl / divergence once per point, the default)
    and the one-pass ones (SMATRAN_MODE_ONE_PASS=1) evaluate the same
    expressions: identical eigenpairs."""
    import subprocess
    import sys
    code = ("import numpy as np, sys; sys.path.insert(0, %r); from smatranem_gb300 import modes, workloads as W; "
            "med = W.port_layer(20, 16, core=(6, 4), seed=3, metric=0.1); "
            "ms = modes.solve(med, 0.405, 20, 16, (1, 0), 4); np.save(sys.argv[1], ms.Xi)") % os.path.dirname(HERE)
    out = {}
    for flag in ("0", "1"):
        path = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"xi_pass{flag}_{os.getpid()}.npy")
        env = dict(os.environ, SMATRAN_MODE_ONE_PASS=flag)
        subprocess.run([sys.executable, "-c", code, path], check=True, env=env)
        out[flag] = np.load(path)
        os.remove(path)
    assert np.array_equal(out["0"], out["1"])
