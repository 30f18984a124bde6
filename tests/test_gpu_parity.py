"""GPU parity: the CUDA path through the C ABI against the oracle and the goldens.

FP64 plans must reproduce the reference bit for bit (np.array_equal).  FP32
plans are compared with a relative tolerance stated per test: the error of a
field after n steps in FP32 against the FP64 result, measured as
max|x32 - x64| / max|x64| over the array.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu

CASES = golden_cases()


def _fdtd():
    from smatranem_gb300 import fdtd
    return fdtd


def _plan_from_golden(g, precision, batch=1):
    f = _fdtd()
    return f.Plan.create(g["L"], g["iBc"], g["iBTIin"], float(g["invtau_R"]), float(g["invtau_I"]), g["mu"],
                         g["epsi"], g["sigma"], precision=precision, batch=batch)


def _relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", CASES)
def test_fp64_run_is_bit_identical_to_reference(built, name):
    g = load_golden(name)
    f = _fdtd()
    n2, tp, nsteps = int(g["n2pi"]), g["time_period"], int(g["nsteps"])
    with _plan_from_golden(g, f.FP64) as p:
        p.set_fields(0, g["H0"], g["E0"])
        p.set_incident(0, g["Hinc"], g["Einc"])
        if int(g["ref_exits"]) > 0:
            # a monitor plane holds a PML cell: the reference exits, so does the CW schedule
            with pytest.raises(f.FdtdError) as ei:
                p.set_cw_schedule(n2, tp)
            assert ei.value.code == -4
            src, ph = f.cw_schedule(n2, tp)
            p.set_schedule(src, planes=(int(g["iBTIin"][0]), int(g["iBTIin"][1])), phase=ph)
        else:
            p.set_cw_schedule(n2, tp)
        p.run(0, nsteps)
        H, E = p.get_fields(0)
        assert np.array_equal(H, g["H"])
        assert np.array_equal(E, g["E"])
        if int(g["ref_exits"]) == 0:
            HB, EB, HT, ET = p.get_monitor(0)
            for m, key in zip((HB, EB, HT, ET), ("HB", "EB", "HT", "ET")):
                assert np.array_equal(m, g[key]), key


@pytest.mark.parametrize("name", CASES)
def test_fp64_chunking_does_not_change_results(built, name):
    """Graph-captured chunks, remainders and split run() calls give identical bits."""
    g = load_golden(name)
    f = _fdtd()
    n2, tp = int(g["n2pi"]), g["time_period"]
    src, ph = f.cw_schedule(n2, tp)
    nsteps = min(75, src.shape[0])
    planes = (int(g["iBTIin"][0]), int(g["iBTIin"][1]))
    out = []
    for cuts in ((0, nsteps), (0, 7, 40, nsteps)):
        with _plan_from_golden(g, f.FP64) as p:
            p.set_fields(0, g["H0"] * 1e-3, g["E0"] * 1e-3)
            p.set_incident(0, g["Hinc"], g["Einc"])
            p.set_schedule(src, planes=planes, phase=ph)
            for a, b in zip(cuts[:-1], cuts[1:]):
                p.run(a, b)
            out.append((*p.get_fields(0), p.get_dft(0, 0, 0), p.get_dft(0, 0, 1)))
    for a, b in zip(*out):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["zpml_plain", "zpml_metal", "periodic_bc"])
def test_step_api_and_main_calc_are_bit_identical(built, port, name):
    """smat_fdtd_step (explicit Hi/Ei) and the stateless smat_main_calc."""
    g = load_golden(name)
    f = _fdtd()
    L = g["L"]
    pl = int(L[0] * L[1])
    rng = np.random.default_rng(7)
    steps = [(rng.standard_normal(2 * pl), rng.standard_normal(2 * pl), np.exp(1j * rng.uniform(0, 6, 2)))
             for _ in range(3)]
    coef = (g["Ah"], g["Bh"], g["Ae"], g["Be"])
    # oracle
    H, E = g["H0"].copy(), g["E0"].copy()
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    for Hi, Ei, z in steps:
        assert port.main_calc(L, *coef, g["iBc"], H, E, g["iBTIin"], Hi, Ei, z, *mons, g["cont"], g["addr"]) == 0
    # plan step API
    with _plan_from_golden(g, f.FP64) as p:
        p.set_fields(0, g["H0"], g["E0"])
        for Hi, Ei, z in steps:
            p.step(Hi, Ei, z)
        H2, E2 = p.get_fields(0)
        m2 = p.get_monitor(0)
    assert np.array_equal(H2, H) and np.array_equal(E2, E)
    for a, b in zip(m2, mons):
        assert np.array_equal(a, b)
    # stateless main_calc, same signature as the reference
    H3, E3 = g["H0"].copy(), g["E0"].copy()
    m3 = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    for Hi, Ei, z in steps:
        f.main_calc(L, *coef, g["iBc"], H3, E3, g["iBTIin"], Hi, Ei, z, *m3, g["cont"], g["addr"])
    assert np.array_equal(H3, H) and np.array_equal(E3, E)
    for a, b in zip(m3, mons):
        assert np.array_equal(a, b)


def test_from_coeffs_plan_and_batch(built, port):
    """A plan built from main_calc's arrays; three excitations in one batch each
    equal their own oracle run."""
    g = load_golden("zpml_plain")
    f = _fdtd()
    from smatranem_gb300 import workloads as W
    L, n2, tp = g["L"], int(g["n2pi"]), g["time_period"]
    pl = int(L[0] * L[1])
    n3 = int(np.prod(L[:3]))
    ln = int(g["lnotn"])
    coef = (g["Ah"], g["Bh"], g["Ae"], g["Be"])
    nsteps = 45
    excit = []
    for b in range(3):
        H0, E0 = W.random_fields(n3, ln, seed=30 + b, scale=1e-3)
        Hinc, Einc = W.random_incident(pl, seed=40 + b)
        excit.append((H0, E0, Hinc, Einc))
    with f.Plan.from_coeffs(L, *coef, g["iBc"], g["cont"], g["addr"], ln, g["iBTIin"], batch=3) as p:
        for b, (H0, E0, Hinc, Einc) in enumerate(excit):
            p.set_fields(b, H0, E0)
            p.set_incident(b, Hinc, Einc)
        p.set_cw_schedule(n2, tp)
        p.run(0, nsteps)
        got = [(*p.get_fields(b), *p.get_monitor(b)) for b in range(3)]
    for b, (H0, E0, Hinc, Einc) in enumerate(excit):
        H, E = H0.copy(), E0.copy()
        mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
        port.time_loop(L, *coef, g["iBc"], H, E, g["iBTIin"], Hinc, Einc, n2, tp, 0, nsteps, *mons, g["cont"],
                       g["addr"])
        for a, r in zip(got[b], (H, E, *mons)):
            assert np.array_equal(a, r)


def test_general_dft_matches_oracle_fields(built, port):
    """Multi-frequency DFT on three planes, one cutting the x/y PML, against a
    DFT of the oracle's fields (total field on split cells)."""
    f = _fdtd()
    from smatranem_gb300 import workloads as W
    L = (10, 9, 12, 2)
    s = W.random_structure(L, seed=5, pml=(2, 2, 2))
    pr = W.prepare(s)
    coef = pr.coefficients()
    n3, pl = s.n3, L[0] * L[1]
    tp = (1, 1, 3)
    src, _ = f.cw_schedule(pr.n2pi, tp)
    nsteps = 20
    src = src[:nsteps]
    rng = np.random.default_rng(3)
    nf = 3
    wdt = rng.uniform(0.05, 0.4, nf)
    k = np.arange(nsteps)[:, None]
    ph = np.stack([np.cos(wdt * (k + 1)), np.sin(wdt * (k + 1)), np.cos(wdt * (k + 1.5)), np.sin(wdt * (k + 1.5))],
                  axis=-1)
    planes = (3, 6, 0)  # plane 0 lies in the z-PML; all cut the x/y PML
    H0, E0 = W.random_fields(n3, pr.lnotn, seed=9, scale=1e-2)
    Hinc, Einc = W.random_incident(pl, seed=8)
    iBTIin = (3, 6, 5, 1)
    with f.Plan.create(L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma) as p:
        p.set_fields(0, H0, E0)
        p.set_incident(0, Hinc, Einc)
        p.set_schedule(src, planes=planes, phase=ph)
        p.run(0, nsteps)
        got = [[p.get_dft(0, fi, q) for q in range(3)] for fi in range(nf)]
        Hg, Eg = p.get_fields(0)
    H, E = H0.copy(), E0.copy()
    acc = np.zeros((nf, 3, 4, pl, 2))
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    cont, addr = pr.cont, pr.addr
    for kk in range(nsteps):
        port.time_loop(L, *coef, s.iBc, H, E, iBTIin, Hinc, Einc, pr.n2pi, tp, kk, kk + 1, *mons, cont, addr)
        for q, z in enumerate(planes):
            cells = np.arange(pl) + pl * z
            x = []
            for F in (H, E):
                for v in range(2):
                    val = F[v + 3 * cells].copy()
                    split = cont[cells] == ord("a")
                    val[split] = val[split] + F[v + 3 * (n3 + addr[cells[split]])]
                    x.append(val)
            for fi in range(nf):
                for v in range(4):
                    pr_, pi_ = (ph[kk, fi, 0], ph[kk, fi, 1]) if v < 2 else (ph[kk, fi, 2], ph[kk, fi, 3])
                    acc[fi, q, v, :, 0] = acc[fi, q, v, :, 0] + pr_ * x[v]
                    acc[fi, q, v, :, 1] = acc[fi, q, v, :, 1] + pi_ * x[v]
    assert np.array_equal(Hg, H) and np.array_equal(Eg, E)
    for fi in range(nf):
        for q in range(3):
            ref = acc[fi, q, :, :, 0] + 1j * acc[fi, q, :, :, 1]
            assert np.array_equal(got[fi][q], ref)


# ---- FP32 -----------------------------------------------------------------

FP32_TOL_FIELDS = 2e-5  # relative, after <= 45 steps of a bounded case


@pytest.mark.parametrize("name", ["zpml_plain", "periodic_bc"])
def test_fp32_run_within_tolerance_of_fp64(built, name):
    g = load_golden(name)
    f = _fdtd()
    with _plan_from_golden(g, f.FP32) as p:
        p.set_fields(0, g["H0"], g["E0"])
        p.set_incident(0, g["Hinc"], g["Einc"])
        p.set_cw_schedule(int(g["n2pi"]), g["time_period"])
        p.run(0, int(g["nsteps"]))
        H, E = p.get_fields(0)
        mons = p.get_monitor(0)
    assert _relerr(H, g["H"]) < FP32_TOL_FIELDS
    assert _relerr(E, g["E"]) < FP32_TOL_FIELDS
    for m, key in zip(mons, ("HB", "EB", "HT", "ET")):
        assert _relerr(m, g[key]) < FP32_TOL_FIELDS, key


@pytest.mark.parametrize("seed", [1, 2])
def test_fp32_general_cells_within_tolerance(built, port, seed):
    """Lossy, PEC, metallic ('h','e','b') and split cells, x/y/z PML, FP32 vs FP64."""
    f = _fdtd()
    from smatranem_gb300 import workloads as W
    L = (14, 12, 13, 2)
    s = W.random_structure(L, seed=seed, pml=(3, 3, 3), metals=0.04, lossy=0.08, pec=0.05, iBc=(1, -1, 0))
    pr = W.prepare(s)
    n3, pl = s.n3, L[0] * L[1]
    H0, E0 = W.random_fields(n3, pr.lnotn, seed=seed, scale=1e-2)
    Hinc, Einc = W.random_incident(pl, seed=seed)
    src, ph = f.cw_schedule(pr.n2pi, (1, 1, 3))
    iBTIin = (4, 9, 6, 1)
    res = {}
    for prec in (f.FP64, f.FP32):
        with f.Plan.create(L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma, precision=prec,
                           pec=s.pec) as p:
            p.set_fields(0, H0, E0)
            p.set_incident(0, Hinc, Einc)
            p.set_schedule(src, planes=(4, 9), phase=ph)
            p.run(0, 6)
            res[prec] = (*p.get_fields(0), p.get_dft(0, 0, 0), p.get_dft(0, 0, 1))
    # the FP64 plan is the oracle's bit pattern (PEC applied to the coefficients)
    Ah, Bh, Ae, Be = pr.coefficients()
    pec = np.flatnonzero(s.pec)
    for c in range(3):
        Ae[c + 3 * pec] = 0.0
        Be[c + 3 * pec] = 0.0
    H, E = H0.copy(), E0.copy()
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    port.time_loop(L, Ah, Bh, Ae, Be, s.iBc, H, E, iBTIin, Hinc, Einc, pr.n2pi, (1, 1, 3), 0, 6, *mons, pr.cont,
                   pr.addr)
    assert np.array_equal(res[f.FP64][0], H) and np.array_equal(res[f.FP64][1], E)
    for a, b in zip(res[f.FP32], res[f.FP64]):
        assert _relerr(a, b) < 1e-5


def test_fp32_batch_members_are_independent(built):
    g = load_golden("zpml_plain")
    f = _fdtd()
    from smatranem_gb300 import workloads as W
    L = g["L"]
    n3, pl, ln = int(np.prod(L[:3])), int(L[0] * L[1]), int(g["lnotn"])
    ex = [(*W.random_fields(n3, ln, seed=60 + b, scale=1e-3), *W.random_incident(pl, seed=70 + b)) for b in range(4)]
    outs = []
    with _plan_from_golden(g, f.FP32, batch=4) as p:
        for b, (H0, E0, Hi, Ei) in enumerate(ex):
            p.set_fields(b, H0, E0)
            p.set_incident(b, Hi, Ei)
        p.set_cw_schedule(int(g["n2pi"]), g["time_period"])
        p.run(0, 40)
        batch = [p.get_fields(b) for b in range(4)]
    for b, (H0, E0, Hi, Ei) in enumerate(ex):
        with _plan_from_golden(g, f.FP32) as p:
            p.set_fields(0, H0, E0)
            p.set_incident(0, Hi, Ei)
            p.set_cw_schedule(int(g["n2pi"]), g["time_period"])
            p.run(0, 40)
            single = p.get_fields(0)
        assert np.array_equal(batch[b][0], single[0]) and np.array_equal(batch[b][1], single[1])


def test_finite_check_and_errors(built):
    g = load_golden("zpml_plain")
    f = _fdtd()
    with _plan_from_golden(g, f.FP32) as p:
        ok, m = p.check_finite()
        assert ok and m == 0.0
        with pytest.raises(f.FdtdError):
            p.run(0, 10)  # no schedule yet
        p.set_cw_schedule(int(g["n2pi"]), g["time_period"])
        with pytest.raises(f.FdtdError):
            p.run(0, 10 ** 6)  # beyond the schedule
        H = g["H0"].copy()
        H[5] = np.inf
        p.set_fields(0, H, g["E0"])
        ok, m = p.check_finite()
        assert not ok


# ---- FP32 launch forms ---------------------------------------------------------

FUSED_CASES = [
    # (L, seed, structure kwargs, iBTIin)
    ((37, 13, 15, 2), 21, dict(pml=(3, 2, 3), metals=0.03, lossy=0.05, pec=0.04, iBc=(-1, 0, 1)), (4, 10, 6, 1)),
    ((40, 17, 19, 3), 22, dict(pml=(4, 4, 4), lossy=0.05, iBc=(1, 1, -1)), (5, 13, 7, -1)),
    ((33, 9, 12, 2), 23, dict(pml=(0, 0, 2), pml_z_only=True, iBc=(0, -1, 0)), (3, 8, 5, 1)),
    ((64, 24, 20, 3), 24, dict(pml=(5, 5, 4), metals=0.02, iBc=(0, 0, 0)), (5, 14, 7, 1)),
    # rows of 34 quads, lossy and PEC records
    ((136, 13, 17, 2), 25, dict(pml=(4, 3, 3), lossy=0.05, pec=0.03, iBc=(0, 0, 0)), (4, 12, 6, 1)),
]


def _run_fp32(s, pr, iBTIin, tuning, nsteps, batch=2, seed=0):
    f = _fdtd()
    from smatranem_gb300 import workloads as W
    n3, pl = s.n3, s.L[0] * s.L[1]
    src, ph = f.cw_schedule(pr.n2pi, (1, 1, 3))
    with f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma, precision=f.FP32,
                       batch=batch, pec=s.pec) as p:
        p.set_tuning(*tuning)
        for b in range(batch):
            H0, E0 = W.random_fields(n3, pr.lnotn, seed=seed + b, scale=1e-2)
            Hinc, Einc = W.random_incident(pl, seed=seed + 10 + b)
            p.set_fields(b, H0, E0)
            p.set_incident(b, Hinc, Einc)
            p.set_source_plane(b, iBTIin[2] + b, 1 - 2 * b)
        p.set_schedule(src, planes=(iBTIin[0], iBTIin[1], 0), phase=ph)
        p.run(0, nsteps // 2)
        p.run(nsteps // 2, nsteps)  # an odd split exercises both field sets
        return [(*p.get_fields(b), *[p.get_dft(b, 0, q) for q in range(3)]) for b in range(batch)]


@pytest.mark.parametrize("case", range(len(FUSED_CASES)))
def test_sweep_forms_fp32_are_bit_identical(built, case):
    """The vectorised and z-chunked sweeps reproduce the scalar two-sweep FP32
    kernels bit for bit, for every block shape, z chunk, register bound and
    grid size, across field-set swaps, iBc = -1/0/1 wraps, PML on all faces,
    lossy/PEC/metal cells and per-excitation source planes."""
    from smatranem_gb300 import workloads as W
    L, seed, kw, iBTIin = FUSED_CASES[case]
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    nsteps = 9 if kw.get("metals") else 37
    ref = _run_fp32(s, pr, iBTIin, (0, 4, 0, 0, 4), nsteps)
    # z_chunk of the sweeps (kernels 0, 2): planes per H/E chunk, 0 = whole grid
    tunings = [(0, 4, 1, 0, 4), (0, 2, 3, 0, 4), (0, 8, 0, 6, 4), (0, 1, 5, 8, 4)]
    if L[0] % 4 == 0:
        tunings += [(2, 1, 0, 0, 4), (2, 2, 1, 0, 4), (2, 4, 3, 0, 4), (2, 1, 5, 0, 4), (2, 2, 16, 0, 4),
                    (2, 1, 0, 6, 4), (2, 2, 0, 8, 4), (2, 1, 0, -3, 4), (2, 2, 3, -3, 4)]
    for tuning in tunings:
        got = _run_fp32(s, pr, iBTIin, tuning, nsteps)
        for rb, gb in zip(ref, got):
            for a, b_ in zip(rb, gb):
                assert np.array_equal(a, b_), tuning


ROW_CASES = [
    # record-free structures (launch form 6): (L, seed, structure kwargs, iBTIin)
    ((40, 17, 19, 3), 31, dict(pml=(4, 4, 4), iBc=(1, 1, -1)), (5, 13, 7, -1)),
    ((36, 9, 12, 2), 32, dict(pml=(0, 0, 2), pml_z_only=True, iBc=(0, -1, 0)), (3, 8, 5, 1)),
    ((64, 24, 20, 3), 33, dict(pml=(5, 5, 4), iBc=(0, 0, 0)), (5, 14, 7, 1)),
    # rows of two warps with idle lanes (34 quads), odd row count
    ((136, 13, 17, 2), 34, dict(pml=(4, 3, 3), iBc=(-1, 1, 1)), (4, 12, 6, 1)),
    ((8, 5, 3, 1), 35, dict(pml=(0, 0, 0), iBc=(1, -1, 1)), (0, 2, 1, 1)),
]


def _row_fits(L0, ty, mb, zc):
    """Kernel 6 launch shape: a thread per quad of tile_y + 1 rows (whole
    warps), staging rings in shared memory (at most 227 KB per CTA)."""
    nq = L0 // 4
    threads = ((nq * (ty + 1) + 31) // 32) * 32
    smem = 16 * (27 * nq * (ty + 1) + 4 * nq + 2 * (zc + 1))
    return threads <= {1: 1024, 2: 384, 3: 256}[mb] and smem <= 232448


@pytest.mark.parametrize("case", range(len(ROW_CASES)))
def test_row_fused_fp32_is_bit_identical_to_the_sweeps(built, case):
    """The whole-row fused step (kernel 6) reproduces the scalar FP32 sweeps
    bit for bit: partial last row tiles, z chunks of 1 plane to the whole
    grid, persistent CTAs (whole tiles in rounds, the leftover tiles' planes
    shared out in pieces of a few planes), every register bound, iBc = -1/0/1
    wraps on each axis (the halo row and closing plane hold iBc * H_new),
    split PML on all faces, per-excitation source planes and DFT planes,
    across field-set swaps."""
    from smatranem_gb300 import workloads as W
    L, seed, kw, iBTIin = ROW_CASES[case]
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    nsteps = 37
    ref = _run_fp32(s, pr, iBTIin, (0, 4, 0, 0, 4), nsteps)
    # the fifth value: the warp order (1: the last two warps trade places with
    # the two before them, in blocks of a multiple of 128 threads, >= 256)
    tunings = [(6, ty, zc, mb, wo) for ty, zc, mb, wo in
               [(1, L[2], 1, 0), (2, 5, 2, 0), (4, 3, 1, 0), (3, 1, 3, 0), (4, 7, 2, 0), (8, 40, 1, 0), (2, 2, 3, 0),
                (5, L[2], 1, 0), (1, 4, 3, 0), (1, 2, 2, 0), (1, 0, 1, 0), (2, 0, 2, 0), (5, 0, 1, 0), (3, 0, 3, 0),
                (15, 0, 1, 1), (15, 7, 1, 1), (5, 0, 1, 1)]
               if _row_fits(L[0], ty, mb, min(zc, L[2]) if zc else L[2])]
    assert len(tunings) >= 5
    for tuning in tunings:
        got = _run_fp32(s, pr, iBTIin, tuning, nsteps)
        for rb, gb in zip(ref, got):
            for a, b_ in zip(rb, gb):
                assert np.array_equal(a, b_), tuning


ROW_REC_CASES = [
    # record cells other than metal: lossy and PEC ordinary cells, split cells
    # with lossy media
    ((40, 17, 19, 3), 41, dict(pml=(4, 4, 4), lossy=0.05, iBc=(1, 1, -1)), (5, 13, 7, -1)),
    ((48, 19, 21, 3), 44, dict(pml=(4, 4, 4), lossy=0.03, lossy_pml=0.2, iBc=(1, -1, 1)), (5, 15, 8, 1)),
    ((36, 10, 16, 2), 45, dict(pml=(0, 0, 4), pml_z_only=True, lossy_pml=0.3, pec=0.03, iBc=(0, 0, -1)),
     (5, 11, 8, -1)),
    ((136, 13, 17, 2), 42, dict(pml=(4, 3, 3), lossy=0.05, pec=0.03, iBc=(0, 0, 0)), (4, 12, 6, 1)),
    ((36, 9, 12, 2), 43, dict(pml=(0, 0, 3), pml_z_only=True, pec=0.05, iBc=(0, -1, 0)), (4, 8, 5, 1)),
]


@pytest.mark.parametrize("case", range(len(ROW_REC_CASES)))
def test_row_fused_record_cells_bit_identical(built, case):
    """Record cells in kernel 6 (the sweeps' general-cell update, out of
    line): lossy and PEC ordinary cells and split cells with lossy media, bit
    for bit as the scalar sweeps, chunked and persistent."""
    from smatranem_gb300 import workloads as W
    L, seed, kw, iBTIin = ROW_REC_CASES[case]
    kw = dict(kw)
    lossy_pml = kw.pop("lossy_pml", 0.0)
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    if lossy_pml:
        # absorbing media in a share of the split cells (the reference's
        # remove_sigma refuses such decks; the plan API takes them)
        rng = np.random.default_rng(seed)
        cells = np.flatnonzero(np.asarray(pr.cont).view(np.uint8) == ord("a"))
        pick = rng.choice(cells, size=max(1, int(lossy_pml * cells.size)), replace=False)
        for c in range(3):
            pr.epsi[3 * pick + c] += 1j * np.abs(pr.epsi[3 * pick + c].real) * rng.uniform(0.01, 0.3, pick.size)
    nsteps = 33
    ref = _run_fp32(s, pr, iBTIin, (0, 4, 0, 0, 4), nsteps)
    # plans with record cells run kernel 6 at one CTA per SM only
    tunings = [(6, ty, zc, 1, 0) for ty, zc in [(2, 5), (5, 0), (1, 3), (3, 0), (4, L[2])]
               if _row_fits(L[0], ty, 1, min(zc, L[2]) if zc else L[2])]
    assert len(tunings) >= 4
    for tuning in tunings:
        got = _run_fp32(s, pr, iBTIin, tuning, nsteps)
        for rb, gb in zip(ref, got):
            for a, b_ in zip(rb, gb):
                assert np.array_equal(a, b_), tuning


def test_fp32_plan_independent_of_host_threads(built, monkeypatch):
    """FP32 plan creation packs the coefficients and numbers the record cells
    on host worker threads: plans made with 1, 3 and 16 threads step to the
    same bits (every record kind: metal, lossy, PEC, lossy split cells)."""
    from smatranem_gb300 import workloads as W
    L, seed, kw, iBTIin = (40, 17, 19, 3), 46, dict(pml=(4, 4, 4), metals=0.03, lossy=0.05, pec=0.02), (5, 13, 7, 1)
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    rng = np.random.default_rng(seed)
    cells = np.flatnonzero(np.asarray(pr.cont).view(np.uint8) == ord("a"))
    pick = rng.choice(cells, size=cells.size // 5, replace=False)
    for c in range(3):
        pr.epsi[3 * pick + c] += 1j * np.abs(pr.epsi[3 * pick + c].real) * rng.uniform(0.01, 0.3, pick.size)
    runs = []
    for nt in (1, 3, 16):
        monkeypatch.setenv("SMATRAN_HOST_THREADS", str(nt))
        runs.append(_run_fp32(s, pr, iBTIin, (0, 4, 0, 0, 4), 9))
    for got in runs[1:]:
        for rb, gb in zip(runs[0], got):
            for a, b_ in zip(rb, gb):
                assert np.array_equal(a, b_)


ROW_METAL_CASES = [
    # metal cells ('h', 'e', 'b': stable-form and frozen components) with lossy
    # and PEC cells; monitor planes through the metal; iBc wraps on every axis
    ((40, 17, 19, 3), 47, dict(pml=(4, 4, 4), metals=0.04, lossy=0.03, pec=0.02, iBc=(1, -1, 1)), (6, 12, 8, 1)),
    ((36, 14, 16, 2), 48, dict(pml=(0, 0, 3), pml_z_only=True, metals=0.05, iBc=(-1, 1, -1)), (4, 9, 6, -1)),
    ((64, 12, 14, 2), 49, dict(pml=(5, 3, 3), metals=0.03, pec=0.03, iBc=(0, 0, 0)), (4, 9, 5, 1)),
]


@pytest.mark.parametrize("case", range(len(ROW_METAL_CASES)))
def test_row_fused_metal_cells_bit_identical(built, case):
    """Metal cells in kernel 6: the H stable-form update in the march (the
    backward curl of E's main slot from the old set), the E stable-form update
    and the monitor samples of stable-form and frozen components in the second
    launch after the step -- bit for bit as the scalar sweeps, for whole
    grids, z chunks and persistent CTAs, across field-set swaps."""
    from smatranem_gb300 import workloads as W
    L, seed, kw, iBTIin = ROW_METAL_CASES[case]
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    cont = np.asarray(pr.cont).view(np.uint8)
    pl = L[0] * L[1]
    metal = np.isin(cont, [ord("e"), ord("h"), ord("b")])
    assert metal.any() and any(metal[z * pl:(z + 1) * pl].any() for z in iBTIin[:2])
    nsteps = 9  # the stable form is not unconditionally stable: few steps
    ref = _run_fp32(s, pr, iBTIin, (0, 4, 0, 0, 4), nsteps)
    tunings = [(6, ty, zc, 1, 0) for ty, zc in [(2, 5), (5, 0), (1, 3), (3, 0), (4, L[2])]
               if _row_fits(L[0], ty, 1, min(zc, L[2]) if zc else L[2])]
    assert len(tunings) >= 4
    for tuning in tunings:
        got = _run_fp32(s, pr, iBTIin, tuning, nsteps)
        for rb, gb in zip(ref, got):
            for a, b_ in zip(rb, gb):
                assert np.all(np.isfinite(a)) and np.array_equal(a, b_), tuning


def test_row_fused_refuses_bad_tunings(built):
    """Kernel 6's arguments out of range are refused and leave the plan's
    launch form as it was."""
    from smatranem_gb300 import workloads as W
    f = _fdtd()
    L, seed, kw, iBTIin = ROW_CASES[0]
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    with f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                       precision=f.FP32) as p:
        p.set_tuning(6, 2, 0, 1, 0)
        assert tuple(p.get_tuning())[:4] == (6, 2, 0, 1)
        for bad in [(6, 0, 0, 1, 0), (6, 17, 0, 1, 0), (6, 2, -1, 1, 0), (6, 2, 0, 0, 0), (6, 2, 0, 4, 0),
                    (6, 200, 0, 1, 0), (6, 2, 0, 1, 2), (6, 2, 0, 1, -1), (7, 2, 0, 1, 0), (-1, 2, 0, 1, 0),
                    (1, 8, 40, 0, 5), (3, 8, 40, 0, 5), (4, 2, 2, 0, 0), (5, 4, 40, 1, 4)]:
            with pytest.raises(f.FdtdError):
                p.set_tuning(*bad)
            assert tuple(p.get_tuning())[:4] == (6, 2, 0, 1)


def test_fused_fp32_within_tolerance_of_fp64_long_run(built):
    """A 300-step run with PML on all faces: FP32 (fused) vs the FP64 plan."""
    f = _fdtd()
    from smatranem_gb300 import workloads as W
    L = (48, 40, 36, 4)
    s = W.random_structure(L, seed=31, pml=(6, 6, 6), lossy=0.02)
    pr = W.prepare(s)
    n3, pl = s.n3, L[0] * L[1]
    src, ph = f.cw_schedule(pr.n2pi, (2, 2, 6))
    Hinc, Einc = W.random_incident(pl, seed=3)
    out = {}
    for prec in (f.FP64, f.FP32):
        with f.Plan.create(L, s.iBc, (8, 27, 10, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                           precision=prec) as p:
            p.set_incident(0, Hinc, Einc)
            p.set_schedule(src, planes=(8, 27), phase=ph)
            p.run(0, 300)
            out[prec] = (*p.get_fields(0), p.get_dft(0, 0, 0), p.get_dft(0, 0, 1))
    for a, b in zip(out[f.FP32], out[f.FP64]):
        assert _relerr(a, b) < 2e-5


def test_autotune_keeps_state_and_results(built):
    """The autotuner leaves a zero-state plan unchanged; the tuned plan gives the
    same bits as the two-sweep configuration."""
    from smatranem_gb300 import workloads as W
    f = _fdtd()
    L, seed, kw, iBTIin = FUSED_CASES[1]
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    with f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                       precision=f.FP32) as p:
        best, ms = p.autotune(2, cache=False)
        assert ms > 0 and p.get_tuning() == best
        ok, mx = p.check_finite()
        assert ok and mx == 0.0
    ref = _run_fp32(s, pr, iBTIin, (0, 4, 1, 0, 4), 21)
    got = _run_fp32(s, pr, iBTIin, tuple(best[:4]) + (best[4],), 21)
    for rb, gb in zip(ref, got):
        for a, b_ in zip(rb, gb):
            assert np.array_equal(a, b_)


def test_gpu_overlap_matches_oracle_s_calc(built, port):
    """GPU mode-overlap projection vs the oracle's S_calc (reference order), FP64,
    relative tolerance 1e-12 (the GPU sums rows in blocks)."""
    f = _fdtd()
    from smatranem_gb300 import workloads as W
    L = (20, 14, 16, 3)
    s = W.random_structure(L, seed=8, pml=(3, 3, 3))
    pr = W.prepare(s)
    pl = L[0] * L[1]
    src, _ = f.cw_schedule(pr.n2pi, (1, 1, 3))
    nsteps = 30
    k = np.arange(nsteps)[:, None]
    wdt = np.array([0.11, 0.23, 0.31])
    ph = np.stack([np.cos(wdt * (k + 1)), np.sin(wdt * (k + 1)), np.cos(wdt * (k + 1.5)), np.sin(wdt * (k + 1.5))],
                  axis=-1)
    rng = np.random.default_rng(2)
    ncols = 5
    tilxi = rng.standard_normal((ncols, 4 * pl)) + 1j * rng.standard_normal((ncols, 4 * pl))
    Hinc, Einc = W.random_incident(pl, seed=4)
    with f.Plan.create(L, s.iBc, (4, 11, 6, 1), pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma) as p:
        p.set_incident(0, Hinc, Einc)
        p.set_schedule(src[:nsteps], planes=(4, 11), phase=ph)
        p.run(0, nsteps)
        for q in range(2):
            S = p.overlap(0, q, tilxi)
            for fi in range(3):
                d = p.get_dft(0, fi, q)
                HB = np.empty(2 * pl, np.complex128)
                EB = np.empty(2 * pl, np.complex128)
                HB[0::2], HB[1::2] = d[0], d[1]
                EB[0::2], EB[1::2] = d[2], d[3]
                ref = port.overlap(L, tilxi, HB, EB)
                assert np.max(np.abs(S[fi] - ref)) <= 1e-12 * np.max(np.abs(ref))


# ---- degenerate grids -------------------------------------------------------

DEGENERATE = [
    # (L, iBc, iBTIin): a dimension of 1 or 2 wraps onto itself / its neighbour
    ((1, 1, 6, 1), (1, 1, 1), (0, 5, 2, 1)),
    ((2, 3, 5, 1), (-1, 0, 1), (0, 4, 1, -1)),
    ((4, 1, 7, 2), (0, -1, -1), (1, 6, 3, 1)),
    ((1, 5, 4, 1), (1, -1, 0), (0, 3, 2, 1)),
    ((8, 2, 2, 0), (1, 1, -1), (0, 1, 1, 1)),
]


@pytest.mark.parametrize("case", range(len(DEGENERATE)))
def test_degenerate_grids(built, port, case):
    """Grids with a dimension of 1 or 2 (every curl neighbour wraps onto the
    cell itself or its only neighbour, with each boundary factor): FP64
    bit-identical to the oracle's reference loop, every FP32 tuning
    bit-identical to the scalar sweeps and within 2e-5 of FP64."""
    f = _fdtd()
    from smatranem_gb300 import workloads as W
    L, iBc, iBTIin = DEGENERATE[case]
    s = W.random_structure(L, seed=40 + case, pml=(0, 0, 0), iBc=iBc)
    pr = W.prepare(s)
    coef = pr.coefficients()
    n3, pl = s.n3, L[0] * L[1]
    tp = (1, 1, 3)
    nsteps = 25
    H0, E0 = W.random_fields(n3, pr.lnotn, seed=7, scale=1e-2)
    Hinc, Einc = W.random_incident(pl, seed=6)
    with f.Plan.create(L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma) as p:
        p.set_fields(0, H0, E0)
        p.set_incident(0, Hinc, Einc)
        p.set_cw_schedule(pr.n2pi, tp)
        p.run(0, nsteps)
        Hg, Eg = p.get_fields(0)
        mon = p.get_monitor(0)
    H, E = H0.copy(), E0.copy()
    mons = [np.zeros(2 * pl, np.complex128) for _ in range(4)]
    assert port.time_loop(L, *coef, s.iBc, H, E, iBTIin, Hinc, Einc, pr.n2pi, tp, 0, nsteps, *mons, pr.cont,
                          pr.addr) == 0
    assert np.array_equal(Hg, H) and np.array_equal(Eg, E)
    for a, b_ in zip(mon, mons):
        assert np.array_equal(a, b_)
    # FP32: all tunings that apply give the scalar sweeps' bits
    fp32_planes = (iBTIin[0], iBTIin[1], 0, 1)
    ref = _run_fp32(s, pr, fp32_planes, (0, 4, 0, 0, 4), 20, batch=1)
    tunings = [(0, 1, 0, 0, 4), (0, 2, 1, 0, 4), (0, 8, 3, 0, 4)]
    if L[0] % 4 == 0:
        tunings += [(2, 1, 0, 0, 4), (2, 2, 1, 0, 4), (2, 1, 0, -3, 4), (6, 1, 1, 1, 0), (6, 2, 2, 2, 0),
                    (6, 1, L[2], 3, 0)]
    for tuning in tunings:
        got = _run_fp32(s, pr, fp32_planes, tuning, 20, batch=1)
        for rb, gb in zip(ref, got):
            for a, b_ in zip(rb, gb):
                assert np.array_equal(a, b_), tuning


@pytest.mark.parametrize("precision", ["FP64", "FP32"])
def test_checkpoint_and_resume(built, tmp_path, precision):
    """save_state after a run, then a new plan of the same setup (and FP32
    launch form) that loads it continues with the bits of the uninterrupted
    run (fields, aux slots and the DFT); a plan of another setup refuses the
    file."""
    from smatranem_gb300 import workloads as W
    f = _fdtd()
    L, seed, kw, iBTIin = FUSED_CASES[1]
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    prec = getattr(f, precision)
    n3, pl = s.n3, L[0] * L[1]
    src, ph = f.cw_schedule(pr.n2pi, (1, 1, 3))

    def plan(batch=2):
        p = f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma, precision=prec,
                          batch=batch, pec=s.pec)
        for b in range(batch):
            p.set_incident(b, *W.random_incident(pl, seed=50 + b))
            p.set_source_plane(b, iBTIin[2] + b, 1 - 2 * b)
        p.set_schedule(src, planes=(iBTIin[0], iBTIin[1], 0), phase=ph)
        return p

    path = str(tmp_path / "state.bin")
    with plan() as p:
        if prec == f.FP32:
            p.set_tuning(6, 2, 0, 1, 0)  # the fused step, which swaps field sets every step
        for b in range(2):
            p.set_fields(b, *W.random_fields(n3, pr.lnotn, seed=60 + b, scale=1e-2))
        p.run(0, 25)
        p.save_state(path)
        p.run(25, 60)
        ref = [(*p.get_fields(b), *[p.get_dft(b, 0, q) for q in range(3)]) for b in range(2)]
    with plan() as p:
        if prec == f.FP32:
            p.set_tuning(6, 2, 0, 1, 0)  # the same launch form: the same DFT sum grouping
        p.load_state(path)
        p.run(25, 60)
        got = [(*p.get_fields(b), *[p.get_dft(b, 0, q) for q in range(3)]) for b in range(2)]
    for rb, gb in zip(ref, got):
        for a, b_ in zip(rb, gb):
            assert np.array_equal(a, b_)
    with plan(batch=1) as p:
        with pytest.raises(f.FdtdError):
            p.load_state(path)


# runs of the FP32 plan: each is cut into windows of 32 steps from its start,
# the last one partial (6, 29, 31, 25 and 8 steps: every flush instantiation)
FLUSH_RUNS = [[(0, 70)], [(0, 29), (29, 90)], [(0, 31), (31, 56), (56, 81), (81, 89)]]


@pytest.mark.parametrize("runs", FLUSH_RUNS)
def test_fp32_dft_flush_is_compensated(built, runs):
    """The FP32 running DFT (ring of field samples folded into FP64
    accumulators, the reference's DFT of :318-328 on FP32 samples) is summed
    in compensated FP32: against the exact FP64 sum of the same samples with
    the same FP64 phases, its error stays under 2 units of 2^-24 of the
    summed magnitudes and its RMS under half that of a plain FP32 sum of the
    window (FP32 phases, one fused multiply-add per sample, as an
    uncompensated flush would do), for full and partial windows of every
    length class.  The samples come from a twin plan stepped one step per run
    (the field updates do not depend on how steps are grouped); its monitor
    planes hold no split cell, so a sample is the cell's field itself."""
    from smatranem_gb300 import workloads as W
    f = _fdtd()
    L = (16, 12, 24, 2)
    s = W.random_structure(L, seed=5, pml=(0, 0, 3), pml_z_only=True, iBc=(1, 1, 0))
    pr = W.prepare(s)
    planes = (7, 15)
    iBTIin = (7, 15, 10, 1)
    nsteps = runs[-1][1]
    windows = [(w0, min(w0 + 32, r1)) for r0, r1 in runs for w0 in range(r0, r1, 32)]
    src, ph = W.pulse_schedule(nsteps, pr.dt, lams_um=[1.3, 1.55, 1.9])
    H0, E0 = W.random_fields(s.n3, pr.lnotn, seed=3, scale=1e-2)
    Hinc, Einc = W.random_incident(L[0] * L[1], seed=4)

    def plan():
        p = f.Plan.create(L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma, precision=f.FP32)
        p.set_tuning(2, 1, 0, 0, 4)
        p.set_fields(0, H0, E0)
        p.set_incident(0, Hinc, Einc)
        p.set_schedule(src, planes=planes, phase=ph)
        return p

    pl = L[0] * L[1]
    with plan() as a, plan() as b:
        for r0, r1 in runs:
            a.run(r0, r1)
        got = np.array([[a.get_dft(0, fi, q) for q in range(2)] for fi in range(3)])  # [f][q][Hx,Hy,Ex,Ey][px]
        samples = np.zeros((nsteps, 2, 4, pl))
        for k in range(nsteps):
            b.run(k, k + 1)
            H, E = b.get_fields(0)
            for qi, z in enumerate(planes):
                cells = np.arange(pl) + pl * z
                for c in range(2):
                    samples[k, qi, c] = H[c + 3 * cells]
                    samples[k, qi, 2 + c] = E[c + 3 * cells]
    # phases: H samples at [0] + i[1], E samples at [2] + i[3]
    phz = np.stack([ph[:, :, 0] + 1j * ph[:, :, 1], ph[:, :, 2] + 1j * ph[:, :, 3]], axis=-1)  # [k][f][half]
    exact = np.zeros((3, 2, 4, pl), np.complex128)
    plain = np.zeros_like(exact)
    scale = np.zeros((3, 2, 4, pl))
    for w0, w1 in windows:
        for fi in range(3):
            for v in range(4):
                z = phz[w0:w1, fi, v // 2]
                x = samples[w0:w1, :, v, :]                                   # [k][q][px]
                exact[fi, :, v] += np.einsum("k,kqp->qp", z, x)
                scale[fi, :, v] += np.abs(x).sum(axis=0)
                zr = z.real.astype(np.float32).astype(np.float64)
                zi = z.imag.astype(np.float32).astype(np.float64)
                sr = np.zeros((2, pl), np.float32)
                si = np.zeros((2, pl), np.float32)
                for k in range(w1 - w0):  # fl(ph*x + s): one rounding per fused multiply-add
                    sr = (zr[k] * x[k] + sr.astype(np.float64)).astype(np.float32)
                    si = (zi[k] * x[k] + si.astype(np.float64)).astype(np.float32)
                plain[fi, :, v] += sr.astype(np.float64) + 1j * si.astype(np.float64)
    err = np.abs(got - exact)
    err_plain = np.abs(plain - exact)
    u = 2.0 ** -24
    assert np.max(err / scale) < 2 * u
    assert np.sqrt(np.mean(err ** 2)) < 0.5 * np.sqrt(np.mean(err_plain ** 2))
