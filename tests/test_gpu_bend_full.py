"""The headline workload at its full size: the curvilinear strip-waveguide
bend, 256 x 192 x 160 cells with non-uniform metric factors on every cell,
12-cell split PML on all six faces (2,563,584 split cells).

The FP64 plan reproduces the reference loop (the oracle's restatement of
main_calc, FDTDsplitfieldMetal.c:242-329) bit for bit over a few steps from a
random state, and the FP32 whole-row fused step (the bench's launch form)
reproduces the FP32 sweeps bit for bit on the same grid, so the chain
reference -> FP64 plan -> FP32 sweeps -> fused step holds at the size the
throughput and the FP32-vs-FP64 errors are measured on."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bend():
    from smatranem_gb300 import workloads as W
    b = W.bend_structure()
    return b, W.prepare(b.s, dt_factor=1.0 / 0.99)


def test_full_bend_fp64_bit_identical_to_the_reference_loop(built, port, bend):
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    b, pr = bend
    s = b.s
    L, n3 = s.L, s.n3
    pl = L[0] * L[1]
    assert (n3, pr.lnotn) == (7864320, 2563584)
    iBTIin = (b.iB, b.iT, b.iI, 1)
    Hinc, Einc = W.mode_profiles(b, n_modes=1)[0]
    tp, nsteps = (1, 1, 3), 3
    H0, E0 = W.random_fields(n3, pr.lnotn, seed=21, scale=1e-2)
    src, ph = f.cw_schedule(pr.n2pi, tp)
    with f.Plan.create(L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma) as p:
        p.set_fields(0, H0, E0)
        p.set_incident(0, Hinc, Einc)
        p.set_schedule(src, planes=(b.iB, b.iT), phase=ph)
        p.run(0, nsteps)
        Hg, Eg = p.get_fields(0)
    H, E = H0.copy(), E0.copy()
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    Ah, Bh, Ae, Be = pr.coefficients()
    port.time_loop(L, Ah, Bh, Ae, Be, s.iBc, H, E, iBTIin, Hinc, Einc, pr.n2pi, tp, 0, nsteps, *mons, pr.cont,
                   pr.addr)
    assert np.array_equal(Hg, H) and np.array_equal(Eg, E)


def test_full_bend_fp32_fused_step_bit_identical_to_the_sweeps(built, bend):
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    b, pr = bend
    s = b.s
    iBTIin = (b.iB, b.iT, b.iI, 1)
    sheets = W.mode_profiles(b, n_modes=2)
    src, ph = W.pulse_schedule(6, pr.dt, lams_um=[1.5, 1.55, 1.6])
    H0, E0 = W.random_fields(s.n3, pr.lnotn, seed=22, scale=1e-2)
    out = []
    for tuning in ((2, 1, 0, 0, 4), (6, 5, 0, 1, 0)):
        with f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                           precision=f.FP32, batch=2) as p:
            p.set_tuning(*tuning)
            for e in range(2):
                p.set_fields(e, H0, E0)
                p.set_incident(e, *sheets[e])
            p.set_schedule(src, planes=(b.iB, b.iT), phase=ph)
            p.run(0, 6)
            out.append([(*p.get_fields(e), *[p.get_dft(e, fi, q) for fi in range(3) for q in range(2)])
                        for e in range(2)])
    for ra, rb in zip(*out):
        for x, y in zip(ra, rb):
            assert np.array_equal(x, y)
