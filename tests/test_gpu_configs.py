"""The structures of the benchmark configurations, built by the same generators
at reduced size: the curvilinear strip bend (graded cells, bend curvature:
distinct coefficients in every cell), a slab with random inclusions (the
batched-structures members) and the large-domain PEC patch array on a curved
substrate (PEC record cells).

FP64 plans reproduce the reference loop (the oracle) bit for bit; every FP32
launch form that applies gives the scalar sweeps' bits; FP32 stays within a
stated tolerance of FP64 over a pulse."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    "bend": lambda W: W.bend_structure(shape=(64, 48, 48), pml=8, L3=12, core_cell0=20),
    "slab": lambda W: W.slab_structure((64, 56, 40), seed=3, pml=8),
    "patches": lambda W: W.large_structure(shape=(96, 80, 48), pml=8, period=16, patch=8),
}


def _case(name):
    from smatranem_gb300 import workloads as W
    b = CASES[name](W)
    return b, W.prepare(b.s, dt_factor=1.0 / 0.99)


def _oracle_coefficients(pr, pec):
    """The reference's coefficient arrays; PEC cells get Ae = Be = 0 on their
    E components, as the plan's pec mask does."""
    Ah, Bh, Ae, Be = pr.coefficients()
    if pec is not None:
        Ae, Be = Ae.copy(), Be.copy()
        cells = np.flatnonzero(pec)
        for c in range(3):
            Ae[3 * cells + c] = 0.0
            Be[3 * cells + c] = 0.0
    return Ah, Bh, Ae, Be


@pytest.mark.parametrize("name", sorted(CASES))
def test_config_structure_fp64_bit_identical(built, port, name):
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    b, pr = _case(name)
    s = b.s
    n3, pl = s.n3, s.L[0] * s.L[1]
    iBTIin = (b.iB, b.iT, b.iI, 1)
    H0, E0 = W.random_fields(n3, pr.lnotn, seed=21, scale=1e-2)
    Hinc, Einc = W.random_incident(pl, seed=22)
    tp, nsteps = (1, 1, 3), 12
    src, ph = f.cw_schedule(pr.n2pi, tp)
    with f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma, pec=s.pec) as p:
        p.set_fields(0, H0, E0)
        p.set_incident(0, Hinc, Einc)
        p.set_schedule(src, planes=(b.iB, b.iT), phase=ph)
        p.run(0, nsteps)
        Hg, Eg = p.get_fields(0)
    H, E = H0.copy(), E0.copy()
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    port.time_loop(s.L, *_oracle_coefficients(pr, s.pec), s.iBc, H, E, iBTIin, Hinc, Einc, pr.n2pi, tp, 0, nsteps,
                   *mons, pr.cont, pr.addr)
    assert np.array_equal(Hg, H) and np.array_equal(Eg, E)


def _run32(b, pr, tuning, nsteps, src, ph, batch=2):
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    s = b.s
    pl = s.L[0] * s.L[1]
    with f.Plan.create(s.L, s.iBc, (b.iB, b.iT, b.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                       precision=f.FP32, batch=batch, pec=s.pec) as p:
        p.set_tuning(*tuning)
        for e in range(batch):
            p.set_incident(e, *W.random_incident(pl, seed=30 + e))
            p.set_source_plane(e, b.iI + e, 1 - 2 * e)
        p.set_schedule(src, planes=(b.iB, b.iT), phase=ph)
        p.run(0, nsteps // 2)
        p.run(nsteps // 2, nsteps)
        return [(*p.get_fields(e), p.get_dft(e, 0, 0), p.get_dft(e, 0, 1)) for e in range(batch)]


@pytest.mark.parametrize("name", sorted(CASES))
def test_config_structure_fp32_forms_bit_identical(built, name):
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    b, pr = _case(name)
    nsteps = 41
    src, ph = W.pulse_schedule(nsteps, pr.dt, lams_um=[1.55])
    ref = _run32(b, pr, (0, 4, 0, 0, 4), nsteps, src, ph)
    tunings = [(2, 1, 0, 0, 4), (2, 2, 5, 0, 4), (6, 5, 0, 1, 0), (6, 2, 7, 1, 0), (6, 4, 20, 1, 0)]
    for tuning in tunings:
        got = _run32(b, pr, tuning, nsteps, src, ph)
        for rb, gb in zip(ref, got):
            for a, b_ in zip(rb, gb):
                assert np.array_equal(a, b_), tuning


@pytest.mark.parametrize("name", sorted(CASES))
def test_config_structure_fp32_within_tolerance_of_fp64(built, name):
    """A Gaussian pulse through the structure's port sheet, DFT at 3
    wavelengths on both monitor planes after 600 steps: the autotuned FP32
    plan within 1e-5 of the largest DFT value of the FP64 plan."""
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    b, pr = _case(name)
    s = b.s
    nsteps = 600
    lams = [1.50, 1.55, 1.60]
    src, ph = W.pulse_schedule(nsteps, pr.dt, lams_um=lams)
    Hinc, Einc = W.mode_profiles(b, n_modes=1)[0]
    out = {}
    for prec in (f.FP64, f.FP32):
        with f.Plan.create(s.L, s.iBc, (b.iB, b.iT, b.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                           precision=prec, pec=s.pec) as p:
            if prec == f.FP32:
                p.autotune(2, cache=False)
            p.set_incident(0, Hinc, Einc)
            p.set_schedule(src, planes=(b.iB, b.iT), phase=ph)
            p.run(0, nsteps)
            out[prec] = np.array([[p.get_dft(0, fi, q) for q in range(2)] for fi in range(len(lams))])
    a, c = out[f.FP32], out[f.FP64]
    assert np.all(np.isfinite(a)) and np.max(np.abs(c)) > 0
    assert np.max(np.abs(a - c)) <= 1e-5 * np.max(np.abs(c))
