"""The plain FP64 benchmark case at its full size: 96^3 cells in vacuum, a
centred 30^3 dielectric block (eps 12.11), a 40x40 one-cell PEC plate 15 cells
below it, 10-cell split PML on all six faces, an x point source.

FP64 plans must reproduce the reference loop (the oracle's restatement of
main_calc) bit for bit -- fields and the monitor DFT -- and FP32 plans stay
within a stated tolerance of FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cube():
    from smatranem_gb300 import workloads as W
    c = W.cube_structure()
    return c, W.prepare(c.s, dt_factor=1.0 / 0.99)


def _pec_coefficients(pr, pec):
    """The coefficient arrays of the reference with the PEC plate: Ae = Be = 0
    on the E components of the plate's (ordinary) cells, as the plan's pec
    mask does."""
    Ah, Bh, Ae, Be = pr.coefficients()
    Ae, Be = Ae.copy(), Be.copy()
    cells = np.flatnonzero(pec)
    for c in range(3):
        Ae[3 * cells + c] = 0.0
        Be[3 * cells + c] = 0.0
    return Ah, Bh, Ae, Be


def test_cube_fp64_bit_identical_to_the_reference_loop(built, port):
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    c, pr = _cube()
    L, n3 = c.s.L, c.s.n3
    pl = L[0] * L[1]
    assert pr.lnotn == 445760  # the split cells of the 10-cell PML on six faces
    iBTIin = (c.iM, c.iI + 4, c.iI, 1)
    Hinc, Einc = W.point_source(c)
    tp, nsteps = (1, 1, 3), 20
    H0, E0 = W.random_fields(n3, pr.lnotn, seed=11, scale=1e-2)
    # every plane crosses the x and y PML, which the reference's own monitor
    # refuses (:320): the reference's CW envelope through the general schedule,
    # whose DFT planes may hold PML cells
    src, ph = f.cw_schedule(pr.n2pi, tp)
    with f.Plan.create(L, c.s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                       pec=c.s.pec) as p:
        p.set_fields(0, H0, E0)
        p.set_incident(0, Hinc, Einc)
        p.set_schedule(src, planes=(iBTIin[0], iBTIin[1]), phase=ph)
        p.run(0, nsteps)
        Hg, Eg = p.get_fields(0)
        dft = [p.get_dft(0, 0, q) for q in range(2)]
    H, E = H0.copy(), E0.copy()
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    rc = port.time_loop(L, *_pec_coefficients(pr, c.s.pec), c.s.iBc, H, E, iBTIin, Hinc, Einc, pr.n2pi, tp, 0,
                        nsteps, *mons, pr.cont, pr.addr)
    assert rc == -1  # the oracle reports the PML cells on the monitor planes and accumulates on
    assert np.array_equal(Hg, H) and np.array_equal(Eg, E)
    # the running DFT of the monitor planes (HB, EB at iB; HT, ET at iT) on
    # their ordinary cells: in a split (PML) cell the reference samples the
    # main slot, the general DFT the total field
    cont = np.frombuffer(np.asarray(pr.cont).tobytes(), np.uint8)
    for q in range(2):
        z = iBTIin[q]
        plain = cont[z * pl:(z + 1) * pl] == ord("n")
        assert plain.sum() > pl // 2
        Hm, Em = mons[2 * q], mons[2 * q + 1]
        ref = np.array([Hm[0::2], Hm[1::2], Em[0::2], Em[1::2]])
        assert np.max(np.abs(dft[q][:, plain] - ref[:, plain])) <= 1e-12 * np.max(np.abs(ref[:, plain]))


def test_cube_fp32_pulse_within_tolerance_of_fp64(built):
    """A Gaussian-modulated pulse (20 % bandwidth at 1.55 um), DFT at 11
    wavelengths on the monitor plane: the autotuned FP32 plan (PEC record
    cells) against the FP64 plan after 1500 steps."""
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    c, pr = _cube()
    nsteps = 1500
    lams = list(np.linspace(1.55 * 0.9, 1.55 * 1.1, 11))
    src, ph = W.pulse_schedule(nsteps, pr.dt, lam0_um=1.55, bandwidth=0.2, lams_um=lams)
    Hinc, Einc = W.point_source(c)
    out = {}
    for prec in (f.FP64, f.FP32):
        with f.Plan.create(c.s.L, c.s.iBc, (c.iM, c.iM, c.iI, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi,
                           pr.sigma, precision=prec, pec=c.s.pec) as p:
            if prec == f.FP32:
                p.autotune(2, cache=False)
            p.set_incident(0, Hinc, Einc)
            p.set_schedule(src, planes=(c.iM,), phase=ph)
            p.run(0, nsteps)
            out[prec] = np.array([p.get_dft(0, fi, 0) for fi in range(len(lams))])
    a, b = out[f.FP32], out[f.FP64]
    assert np.all(np.isfinite(a)) and np.max(np.abs(b)) > 0
    assert np.max(np.abs(a - b)) <= 1e-5 * np.max(np.abs(b))
