"""Adjoint gradient (smat_fdtd_adjoint_grad) against central finite differences.

The finite differences use the FP64 plan, whose forward run is bit-identical
to the reference main_calc; one case also pins the objective itself to the
oracle's reference loop on the CPU.  Tolerances: FP64 adjoint vs FD 1e-5, FP32
adjoint vs FD and vs the FP64 adjoint 1e-3 (of the largest gradient entry).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mods():
    from smatranem_gb300 import fdtd as F
    from smatranem_gb300 import workloads as W
    return F, W


def _design(pml_xy, shape=(40, 36, 48), design=(10, 10, 5), pml=8, seed=3):
    _, W = _mods()
    return W.design_structure(shape=shape, design=design, pml=pml, seed=seed, pml_xy=pml_xy)


def _column(mode):
    Hinc, Einc = mode
    return np.concatenate([Hinc[0::2], Hinc[1::2], -Einc[1::2], Einc[0::2]])


def _plan(d, eps, precision, schedule):
    F, W = _mods()
    s = d.with_eps(eps)
    pr = W.prepare(s, dt_factor=1.0 / 0.99)
    p = F.Plan.create(s.L, s.iBc, (d.iB, d.iT, d.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                      precision=precision, batch=1)
    Hinc, Einc = W.mode_profiles(d, n_modes=1)[0]
    p.set_incident(0, Hinc, Einc)
    if schedule == "cw":
        p.set_cw_schedule(pr.n2pi, (1, 1, 4))
        nsteps = 4 * pr.n2pi
    else:
        nsteps = 8 * pr.n2pi
        src, ph = W.pulse_schedule(nsteps, pr.dt, bandwidth=0.5, lams_um=[1.55])
        p.set_schedule(src, planes=(d.iB, d.iT), phase=ph)
    return p, pr, nsteps


def _objective(d, eps, precision, schedule):
    """J of a plain forward run (no adjoint): |S|^2 at the output plane."""
    F, W = _mods()
    p, _, nsteps = _plan(d, eps, precision, schedule)
    with p:
        p.run(0, nsteps)
        x = p.get_dft(0, 0, 1)
    Hinc, Einc = W.mode_profiles(d, n_modes=1)[0]
    S = W.overlap(x, Hinc, Einc)
    return abs(S) ** 2


def _adjoint(d, eps, precision, schedule, K=64, tuning=None):
    F, W = _mods()
    p, _, nsteps = _plan(d, eps, precision, schedule)
    with p:
        if tuning:
            p.set_tuning(*tuning)
        J, g, gc = p.adjoint_grad(nsteps, K, 0, 1, _column(W.mode_profiles(d, n_modes=1)[0]), d.box)
    return J, g / eps, gc


def _fd_cells(d, n, seed):
    rng = np.random.default_rng(seed)
    nz, ny, nx = d.eps.shape
    flat = rng.choice(nx * ny * nz, size=n, replace=False)
    return [np.unravel_index(i, d.eps.shape) for i in flat]


def _central_fd(d, cells, precision, schedule, h=1e-3):
    out = []
    for c in cells:
        ep = d.eps.copy()
        ep[c] += h
        jp = _objective(d, ep, precision, schedule)
        ep[c] -= 2 * h
        jm = _objective(d, ep, precision, schedule)
        out.append((jp - jm) / (2 * h))
    return np.array(out)


def test_adjoint_fp64_matches_fd_of_the_reference_loop(built, port):
    """CW schedule (the reference's own source and DFT, main :153-167) on a
    z-PML waveguide: J from the adjoint call equals J of the oracle's
    restatement of the reference loop, and the FP64 adjoint gradient matches
    central differences (delta eps_r = 1e-3) of the bit-exact FP64 forward to
    1e-5."""
    F, W = _mods()
    d = _design(pml_xy=False)
    J, g, _ = _adjoint(d, d.eps, F.FP64, "cw")
    # the objective of the reference loop itself (CPU oracle)
    p, pr, nsteps = _plan(d, d.eps, F.FP64, "cw")
    p.close()
    s = d.s
    Ah, Bh, Ae, Be = pr.coefficients()
    H = np.zeros(3 * (s.n3 + pr.lnotn + 1))
    E = np.zeros_like(H)
    pl = s.L[0] * s.L[1]
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    Hinc, Einc = W.mode_profiles(d, n_modes=1)[0]
    rc = port.time_loop(s.L, Ah, Bh, Ae, Be, s.iBc, H, E, (d.iB, d.iT, d.iI, 1), Hinc, Einc, pr.n2pi, (1, 1, 4),
                        0, nsteps, *mons, pr.cont, pr.addr)
    assert rc == 0
    HT, ET = mons[2], mons[3]
    x = np.stack([HT[0::2], HT[1::2], ET[0::2], ET[1::2]])
    J_ref = abs(W.overlap(x, Hinc, Einc)) ** 2
    assert J == pytest.approx(J_ref, rel=1e-12)
    cells = _fd_cells(d, 4, seed=1)
    fd = _central_fd(d, cells, F.FP64, "cw")
    adj = np.array([g[c] for c in cells])
    assert np.max(np.abs(adj - fd)) <= 1e-5 * np.max(np.abs(fd)), (adj, fd)


def test_adjoint_fp32_matches_fd_and_fp64_adjoint(built):
    """Split PML on all six faces, Gaussian pulse, DFT at 1.55 um, checkpoints
    every 64 steps: FP32 adjoint within 1e-3 of central differences of the
    FP64 forward and of the FP64 adjoint over the whole design box."""
    F, W = _mods()
    d = _design(pml_xy=True)
    J32, g32, _ = _adjoint(d, d.eps, F.FP32, "pulse")
    J64, g64, _ = _adjoint(d, d.eps, F.FP64, "pulse")
    assert J32 == pytest.approx(J64, rel=1e-4)
    scale = np.max(np.abs(g64))
    assert scale > 0
    assert np.max(np.abs(g32 - g64)) <= 1e-3 * scale
    cells = _fd_cells(d, 6, seed=2)
    fd = _central_fd(d, cells, F.FP64, "pulse")
    a64 = np.array([g64[c] for c in cells])
    a32 = np.array([g32[c] for c in cells])
    fscale = np.max(np.abs(fd))
    assert np.max(np.abs(a64 - fd)) <= 1e-5 * fscale, (a64, fd)
    assert np.max(np.abs(a32 - fd)) <= 1e-3 * fscale, (a32, fd)


def test_adjoint_checkpoint_interval_does_not_change_the_gradient(built):
    """The recompute from checkpoints reproduces the forward exactly: in FP64,
    K = 1, 7 and 1000 (one segment) give the same bits.  In FP32 the DFT ring
    is folded into FP64 at the end of every forward segment, so the FP32 sum
    grouping (and J, in its last digits) depends on K: 1e-6 there."""
    F, _ = _mods()
    d = _design(pml_xy=True, shape=(24, 20, 28), design=(6, 5, 4), pml=6)
    res = [_adjoint(d, d.eps, F.FP64, "pulse", K=K) for K in (1000, 7, 1)]
    for J, g, gc in res[1:]:
        assert J == res[0][0]
        assert np.array_equal(g, res[0][1]) and np.array_equal(gc, res[0][2])
    res = [_adjoint(d, d.eps, F.FP32, "pulse", K=K) for K in (1000, 7)]
    assert res[1][0] == pytest.approx(res[0][0], rel=1e-6)
    assert np.max(np.abs(res[1][1] - res[0][1])) <= 1e-5 * np.max(np.abs(res[0][1]))


def test_autograd_function_returns_the_adjoint_gradient(built):
    """PortOverlap (torch.autograd.Function) carries J forward and dJ/d eps_r
    backward, the same numbers as the C ABI."""
    torch = pytest.importorskip("torch")
    F, W = _mods()
    from smatranem_gb300 import autograd as A
    d = _design(pml_xy=True, shape=(24, 20, 28), design=(6, 5, 4), pml=6)
    pr = W.prepare(d.s, dt_factor=1.0 / 0.99)
    nsteps = 6 * pr.n2pi
    src, ph = W.pulse_schedule(nsteps, pr.dt, bandwidth=0.5, lams_um=[1.55])
    mode = W.mode_profiles(d, n_modes=1)[0]
    kw = dict(precision=F.FP32, nsteps=nsteps, K=32, mode=mode, src=src, phase=ph)
    eps = torch.tensor(d.eps, dtype=torch.float64, requires_grad=True)
    J = A.PortOverlap.apply(eps, d, kw)
    J.backward()
    J0, g0 = A.objective_and_grad(d, d.eps, **kw)
    assert float(J.detach()) == J0
    assert np.array_equal(eps.grad.numpy(), g0)


def test_adjoint_rejects_bad_requests(built):
    F, W = _mods()
    d = _design(pml_xy=True, shape=(24, 20, 28), design=(6, 5, 4), pml=6)
    p, pr, nsteps = _plan(d, d.eps, F.FP32, "pulse")
    col = _column(W.mode_profiles(d, n_modes=1)[0])
    with p:
        with pytest.raises(F.FdtdError):  # box outside the grid
            p.adjoint_grad(nsteps, 64, 0, 1, col, (0, 30, 0, 5, 0, 5))
        with pytest.raises(F.FdtdError):  # design cells in the PML
            p.adjoint_grad(nsteps, 64, 0, 1, col, (0, 4, 0, 4, 0, 4))
        with pytest.raises(F.FdtdError):  # frequency not in the schedule
            p.adjoint_grad(nsteps, 64, 3, 1, col, d.box)
        with pytest.raises(F.FdtdError):  # more steps than scheduled
            p.adjoint_grad(nsteps + 1, 64, 0, 1, col, d.box)


def test_adjoint_sums_over_the_batch(built):
    """J = sum_b |S_b|^2: a batch of two identical excitations gives exactly
    twice J and twice the gradient of one (FP64)."""
    F, W = _mods()
    d = _design(pml_xy=True, shape=(24, 20, 28), design=(6, 5, 4), pml=6)
    J1, g1, _ = _adjoint(d, d.eps, F.FP64, "pulse", K=32)
    s = d.with_eps(d.eps)
    pr = W.prepare(s, dt_factor=1.0 / 0.99)
    mode = W.mode_profiles(d, n_modes=1)[0]
    nsteps = 8 * pr.n2pi
    src, ph = W.pulse_schedule(nsteps, pr.dt, bandwidth=0.5, lams_um=[1.55])
    with F.Plan.create(s.L, s.iBc, (d.iB, d.iT, d.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                       precision=F.FP64, batch=2) as p:
        for b in range(2):
            p.set_incident(b, *mode)
        p.set_schedule(src, planes=(d.iB, d.iT), phase=ph)
        J2, g2, _ = p.adjoint_grad(nsteps, 32, 0, 1, _column(mode), d.box)
    assert J2 == 2 * J1
    assert np.array_equal(g2 / d.eps, 2 * g1)


def test_vectorised_fp32_adjoint_matches_the_scalar_one(built, monkeypatch):
    """The float4 adjoint kernels (four x-cells per thread) against the
    one-cell-per-thread ones on the all-face PML case: same J, gradients
    within 1e-6 of the largest entry (the two may contract multiply-adds
    differently)."""
    F, _ = _mods()
    d = _design(pml_xy=True)
    Jv, gv, _ = _adjoint(d, d.eps, F.FP32, "pulse")
    monkeypatch.setenv("SMATRAN_ADJOINT_SCALAR", "1")
    Js, gs, _ = _adjoint(d, d.eps, F.FP32, "pulse")
    assert Jv == Js
    assert np.max(np.abs(gv - gs)) <= 1e-6 * np.max(np.abs(gs))


@pytest.mark.parametrize("tuning", [(6, 2, 0, 1, 0), (6, 3, 7, 1, 0), (6, 1, 0, 2, 0)])
def test_adjoint_with_the_fused_forward(built, tuning):
    """The forward and the recompute from checkpoints in the whole-row fused
    step (kernel 6: it swaps the field sets each step; persistent and chunked)
    give the bits of the sweeps' forward: the same J and gradient."""
    F, _ = _mods()
    d = _design(pml_xy=True, shape=(24, 20, 28), design=(6, 5, 4), pml=6)
    ref = _adjoint(d, d.eps, F.FP32, "pulse", K=7, tuning=(2, 1, 0, 0, 4))
    got = _adjoint(d, d.eps, F.FP32, "pulse", K=7, tuning=tuning)
    assert got[0] == ref[0]
    assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])


def test_adjoint_with_a_column_per_excitation(built):
    """One objective column per excitation: the same source twice, the second
    projected on twice the mode column, gives J and the gradient 5 times those
    of the first alone (|2 S|^2 = 4 |S|^2; FP64)."""
    F, W = _mods()
    d = _design(pml_xy=True, shape=(24, 20, 28), design=(6, 5, 4), pml=6)
    J1, g1, _ = _adjoint(d, d.eps, F.FP64, "pulse", K=32)
    s = d.with_eps(d.eps)
    pr = W.prepare(s, dt_factor=1.0 / 0.99)
    mode = W.mode_profiles(d, n_modes=1)[0]
    nsteps = 8 * pr.n2pi
    src, ph = W.pulse_schedule(nsteps, pr.dt, bandwidth=0.5, lams_um=[1.55])
    col = _column(mode)
    with F.Plan.create(s.L, s.iBc, (d.iB, d.iT, d.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                       precision=F.FP64, batch=2) as p:
        for b in range(2):
            p.set_incident(b, *mode)
        p.set_schedule(src, planes=(d.iB, d.iT), phase=ph)
        J2, g2, _ = p.adjoint_grad(nsteps, 32, 0, 1, np.stack([col, 2 * col]), d.box)
        with pytest.raises(F.FdtdError):  # three columns for two excitations
            p.adjoint_grad(nsteps, 32, 0, 1, np.stack([col, col, col]), d.box)
    assert J2 == pytest.approx(5 * J1, rel=1e-13)
    assert np.allclose(g2 / d.eps, 5 * g1, rtol=1e-12, atol=1e-12 * np.max(np.abs(g1)))


def test_adjoint_at_the_design_workload_shape(built):
    """The adjoint workload's own shape: 160 x 160 x 120 cells, a 60 x 60 x 20
    design box of seeded eps_r ~ U[2.085, 12.11] between two single-mode strip
    ports, 12-cell split PML on all six faces, objective |TE0 overlap of the
    output-port DFT at 1.55 um|^2, FP32 forward and adjoint with a checkpoint
    every 64 steps, through the torch.autograd wrapper.  A Gaussian pulse of
    50 % bandwidth over 1600 steps (the workload runs 6000; the pulse has
    crossed the design box by 1600) keeps the finite differences affordable.
    Against central differences (delta eps_r = 1e-3) of the FP64 forward --
    bit-identical to the reference loop -- on 8 seeded design cells: within
    1e-3 of the largest difference quotient; against the FP64 adjoint over
    all 72,000 design cells: within 1e-3 of its largest entry."""
    torch = pytest.importorskip("torch")
    F, W = _mods()
    from smatranem_gb300 import autograd as A
    d = W.design_structure(shape=(160, 160, 120), design=(60, 60, 20), pml=12, seed=0)
    assert d.eps.shape == (20, 60, 60)
    pr = W.prepare(d.s, dt_factor=1.0 / 0.99)
    nsteps = 1600
    src, ph = W.pulse_schedule(nsteps, pr.dt, bandwidth=0.5, lams_um=[1.55])
    mode = W.mode_profiles(d, n_modes=1)[0]
    kw = dict(nsteps=nsteps, K=64, mode=mode, src=src, phase=ph)
    eps = torch.tensor(d.eps, dtype=torch.float64, requires_grad=True)
    J32 = A.PortOverlap.apply(eps, d, dict(kw, precision=F.FP32))
    J32.backward()
    g32 = eps.grad.numpy()
    J64, g64 = A.objective_and_grad(d, d.eps, precision=F.FP64, **kw)
    assert float(J32.detach()) == pytest.approx(J64, rel=1e-4)
    assert np.max(np.abs(g32 - g64)) <= 1e-3 * np.max(np.abs(g64))

    def objective(e):
        s = d.with_eps(e)
        prx = W.prepare(s, dt_factor=1.0 / 0.99)
        with F.Plan.create(s.L, s.iBc, (d.iB, d.iT, d.iI, 1), prx.invtau_R, prx.invtau_I, prx.mu, prx.epsi,
                           prx.sigma, precision=F.FP64, batch=1) as p:
            p.set_incident(0, *mode)
            p.set_schedule(src, planes=(d.iB, d.iT), phase=ph)
            p.run(0, nsteps)
            return abs(W.overlap(p.get_dft(0, 0, 1), *mode)) ** 2

    cells = _fd_cells(d, 8, seed=7)
    fd = []
    for c in cells:
        e = d.eps.copy()
        e[c] += 1e-3
        jp = objective(e)
        e[c] -= 2e-3
        fd.append((jp - objective(e)) / 2e-3)
    fd = np.array(fd)
    a32 = np.array([g32[c] for c in cells])
    a64 = np.array([g64[c] for c in cells])
    fscale = np.max(np.abs(fd))
    assert fscale > 0
    assert np.max(np.abs(a64 - fd)) <= 1e-5 * fscale, (a64, fd)
    assert np.max(np.abs(a32 - fd)) <= 1e-3 * fscale, (a32, fd)
