"""Groups: structures of uneven size stepped together (smat_fdtd_group_*).

Every member of a group must end bit-identical -- fields and DFT -- to the same
plan stepped alone with the vectorised sweeps, whatever the group's launch form."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (L, seed, structure kwargs, iBTIin, batch)
MEMBERS = [
    ((40, 17, 19, 3), 31, dict(pml=(4, 4, 4), lossy=0.05, iBc=(1, 1, -1)), (5, 13, 7, 1), 2),
    ((64, 24, 20, 3), 32, dict(pml=(5, 5, 4), pec=0.03, lossy=0.04, iBc=(0, 0, 0)), (5, 14, 7, 1), 1),
    ((32, 12, 16, 2), 33, dict(pml=(0, 0, 3), pml_z_only=True, iBc=(-1, 0, 0)), (4, 11, 6, -1), 3),
    ((136, 9, 12, 2), 34, dict(pml=(3, 2, 3)), (3, 8, 5, 1), 1),
]


def _setup(f, W, s, pr, iBTIin, batch, seed, nsteps):
    n3, pl = s.n3, s.L[0] * s.L[1]
    src, ph = f.cw_schedule(pr.n2pi, (1, 1, 3))
    p = f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma, precision=f.FP32,
                      batch=batch, pec=s.pec)
    for b in range(batch):
        H0, E0 = W.random_fields(n3, pr.lnotn, seed=seed + b, scale=1e-2)
        Hinc, Einc = W.random_incident(pl, seed=seed + 10 + b)
        p.set_fields(b, H0, E0)
        p.set_incident(b, Hinc, Einc)
        p.set_source_plane(b, iBTIin[2] + b % 2, 1 - 2 * (b % 2))
    p.set_schedule(src[:nsteps], planes=(iBTIin[0], iBTIin[1], 0), phase=ph[:nsteps])
    return p


def _result(p, batch):
    return [(*p.get_fields(b), *[p.get_dft(b, 0, q) for q in range(3)]) for b in range(batch)]


@pytest.mark.parametrize("mode,block_y", [(0, 1), (0, 2), (0, 4), (1, 1), (1, 2)])
def test_group_members_match_plans_stepped_alone(built, mode, block_y):
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    nsteps = 60  # windows of 20 and 40 steps: the second holds a captured 32-step chunk
    structs = []
    for L, seed, kw, iBTIin, batch in MEMBERS:
        s = W.random_structure(L, seed=seed, **kw)
        structs.append((s, W.prepare(s), iBTIin, batch, seed))
    alone = []
    for s, pr, iBTIin, batch, seed in structs:
        with _setup(f, W, s, pr, iBTIin, batch, seed, nsteps) as p:
            p.set_tuning(2, block_y, 0, 0, 4)
            # the same run() windows as the group: the FP32 DFT ring is folded
            # into the FP64 sums at the end of each window
            p.run(0, 20)
            p.run(20, nsteps)
            alone.append(_result(p, batch))
    plans = [_setup(f, W, s, pr, iBTIin, batch, seed, nsteps) for s, pr, iBTIin, batch, seed in structs]
    try:
        with f.Group(plans) as g:
            g.set_tuning(mode, block_y)
            g.run(0, 20)
            g.run(20, nsteps)
        for p, ref, (_, _, _, batch, _) in zip(plans, alone, structs):
            got = _result(p, batch)
            for rb, gb in zip(ref, got):
                for a, b_ in zip(rb, gb):
                    assert np.all(np.isfinite(a)) and np.array_equal(a, b_)
    finally:
        for p in plans:
            p.close()


def test_group_members_own_launch_forms(built):
    """Mode 2: every member in its own launch form -- the whole-row fused step
    (kernel 6: chunked or persistent, with and without record cells) or the
    sweeps -- gives the bits of the member stepped alone with the sweeps, over
    run windows that leave the fused members on either field set."""
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    nsteps = 60
    windows = [(0, 20), (20, 53), (53, nsteps)]  # 33 steps: a captured 32-step chunk and one more
    own = [(6, 2, 0, 1, 0), (6, 4, 7, 1, 0), (2, 1, 0, 0, 4), (6, 1, 0, 2, 0)]
    structs = []
    for L, seed, kw, iBTIin, batch in MEMBERS:
        s = W.random_structure(L, seed=seed, **kw)
        structs.append((s, W.prepare(s), iBTIin, batch, seed))
    alone = []
    for s, pr, iBTIin, batch, seed in structs:
        with _setup(f, W, s, pr, iBTIin, batch, seed, nsteps) as p:
            p.set_tuning(2, 1, 0, 0, 4)
            for a, b in windows:
                p.run(a, b)
            alone.append(_result(p, batch))
    plans = [_setup(f, W, s, pr, iBTIin, batch, seed, nsteps) for s, pr, iBTIin, batch, seed in structs]
    try:
        for p, t in zip(plans, own):
            p.set_tuning(*t)
        with f.Group(plans) as g:
            g.set_tuning(2, 1)
            for a, b in windows:
                g.run(a, b)
        for p, ref, (_, _, _, batch, _) in zip(plans, alone, structs):
            got = _result(p, batch)
            for rb, gb in zip(ref, got):
                for a, b_ in zip(rb, gb):
                    assert np.all(np.isfinite(a)) and np.array_equal(a, b_)
    finally:
        for p in plans:
            p.close()


@pytest.mark.parametrize("order,shape", [((0, 1, 2, 3), 1), ((3, 2, 1, 0), 2), ((2,), 1), ((1, 3), 2),
                                         ((0, 1, 2, 3), 2)])
def test_group_one_persistent_launch(built, order, shape):
    """Mode 3: one persistent launch of the whole-row fused step per step over
    every member (tiles of up to 16 whole rows per member, the resident CTAs
    shared out among the members, each marching its member's own schedule;
    members with lossy and PEC record cells) gives each member the bits of the
    member stepped alone with the sweeps, over run windows that leave the
    members on either field set and across re-captured graphs."""
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    nsteps = 60
    windows = [(0, 20), (20, 53), (53, nsteps)]
    structs = []
    for L, seed, kw, iBTIin, batch in [MEMBERS[i] for i in order]:
        s = W.random_structure(L, seed=seed, **kw)
        structs.append((s, W.prepare(s), iBTIin, batch, seed))
    alone = []
    for s, pr, iBTIin, batch, seed in structs:
        with _setup(f, W, s, pr, iBTIin, batch, seed, nsteps) as p:
            p.set_tuning(2, 1, 0, 0, 4)
            for a, b in windows:
                p.run(a, b)
            alone.append(_result(p, batch))
    plans = [_setup(f, W, s, pr, iBTIin, batch, seed, nsteps) for s, pr, iBTIin, batch, seed in structs]
    try:
        with f.Group(plans) as g:
            g.set_tuning(3, shape)
            for a, b in windows:
                g.run(a, b)
        for p, ref, (_, _, _, batch, _) in zip(plans, alone, structs):
            got = _result(p, batch)
            for rb, gb in zip(ref, got):
                for a, b_ in zip(rb, gb):
                    assert np.all(np.isfinite(a)) and np.array_equal(a, b_)
    finally:
        for p in plans:
            p.close()


@pytest.mark.parametrize("shape", [1, 2])
def test_group_one_persistent_launch_mixed_tiles(built, shape):
    """Mode 3 with members whose tiles differ: 256-cell rows (5-row tiles) and
    128-cell rows (11-row tiles), batches 2 and 3, a PML-free member with
    wrapped boundaries -- each member ends with the bits of the member stepped
    alone."""
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    members = [
        ((256, 13, 10, 2), 41, dict(pml=(4, 3, 3)), (3, 7, 5, 1), 2),
        ((128, 24, 12, 2), 42, dict(pml=(5, 5, 3), lossy=0.03), (4, 8, 6, -1), 3),
        ((64, 7, 9, 1), 43, dict(pml=(0, 0, 0), iBc=(1, -1, 1)), (2, 6, 4, 1), 1),
    ]
    nsteps = 45
    windows = [(0, 7), (7, 45)]
    structs = []
    for L, seed, kw, iBTIin, batch in members:
        s = W.random_structure(L, seed=seed, **kw)
        structs.append((s, W.prepare(s), iBTIin, batch, seed))
    alone = []
    for s, pr, iBTIin, batch, seed in structs:
        with _setup(f, W, s, pr, iBTIin, batch, seed, nsteps) as p:
            p.set_tuning(2, 1, 0, 0, 4)
            for a, b in windows:
                p.run(a, b)
            alone.append(_result(p, batch))
    plans = [_setup(f, W, s, pr, iBTIin, batch, seed, nsteps) for s, pr, iBTIin, batch, seed in structs]
    try:
        with f.Group(plans) as g:
            g.set_tuning(3, shape)
            for a, b in windows:
                g.run(a, b)
        for p, ref, (_, _, _, batch, _) in zip(plans, alone, structs):
            got = _result(p, batch)
            for rb, gb in zip(ref, got):
                for a, b_ in zip(rb, gb):
                    assert np.all(np.isfinite(a)) and np.array_equal(a, b_)
    finally:
        for p in plans:
            p.close()


def test_group_persistent_launch_needs_a_cta_per_excitation(built):
    """Mode 3 gives every excitation its own CTA: 160 excitations exceed the
    152 resident CTAs of 384 threads (refused, the group keeps its form) but
    fit the 304 of 192 threads, where the members still end with the bits of
    the plans stepped alone."""
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    _, sms, _ = f.device_info()
    L, seed, kw, iBTIin = (16, 6, 8, 1), 51, dict(pml=(2, 2, 2)), (2, 5, 3, 1)
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    batch = sms + 8
    nsteps = 12
    with _setup(f, W, s, pr, iBTIin, batch, seed, nsteps) as ref:
        ref.set_tuning(2, 1, 0, 0, 4)
        ref.run(0, nsteps)
        picks = (0, 1, sms - 1, batch - 1)  # CTAs at both ends of the member's range
        want = [(*ref.get_fields(b), *[ref.get_dft(b, 0, q) for q in range(3)]) for b in picks]
    with _setup(f, W, s, pr, iBTIin, batch, seed, nsteps) as p:
        with f.Group([p]) as g:
            g.set_tuning(1, 1)
            with pytest.raises(f.FdtdError):
                g.set_tuning(3, 1)
            g.set_tuning(3, 2)
            g.run(0, nsteps)
        got = [(*p.get_fields(b), *[p.get_dft(b, 0, q) for q in range(3)]) for b in picks]
    for rb, gb in zip(want, got):
        for a, b_ in zip(rb, gb):
            assert np.array_equal(a, b_)


def test_group_persistent_launch_with_metal_member(built):
    """Mode 3 with a member holding metal cells (its stable-form E update and
    metal monitor samples in a second launch after the group's step) and a
    record-free member: each ends with the bits of the member stepped alone;
    an out-of-range shape is refused and the group keeps its form."""
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    members = [
        ((40, 17, 19, 3), 7, dict(pml=(4, 4, 4), metals=0.03, pec=0.02, iBc=(1, 1, -1)), (6, 12, 8, 1), 2),
        MEMBERS[3],
    ]
    nsteps = 9
    windows = [(0, 4), (4, 9)]
    structs = []
    for L, seed, kw, iBTIin, batch in members:
        s = W.random_structure(L, seed=seed, **kw)
        structs.append((s, W.prepare(s), iBTIin, batch, seed))
    alone = []
    for s, pr, iBTIin, batch, seed in structs:
        with _setup(f, W, s, pr, iBTIin, batch, seed, nsteps) as p:
            p.set_tuning(0, 4, 0, 0, 4)
            for a, b in windows:
                p.run(a, b)
            alone.append(_result(p, batch))
    plans = [_setup(f, W, s, pr, iBTIin, batch, seed, nsteps) for s, pr, iBTIin, batch, seed in structs]
    try:
        with f.Group(plans) as g:
            with pytest.raises(f.FdtdError):
                g.set_tuning(3, 3)
            g.set_tuning(3, 1)
            for a, b in windows:
                g.run(a, b)
        for p, ref, (_, _, _, batch, _) in zip(plans, alone, structs):
            got = _result(p, batch)
            for rb, gb in zip(ref, got):
                for a, b_ in zip(rb, gb):
                    assert np.all(np.isfinite(a)) and np.array_equal(a, b_)
    finally:
        for p in plans:
            p.close()


def test_group_autotune_and_errors(built):
    from smatranem_gb300 import fdtd as f
    from smatranem_gb300 import workloads as W
    L, seed, kw, iBTIin, batch = MEMBERS[0]
    s = W.random_structure(L, seed=seed, **kw)
    pr = W.prepare(s)
    src, ph = f.cw_schedule(pr.n2pi, (1, 1, 3))
    with f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                       precision=f.FP32, batch=2) as p, \
            f.Plan.create(s.L, s.iBc, iBTIin, pr.invtau_R, pr.invtau_I, pr.mu, pr.epsi, pr.sigma,
                          precision=f.FP64) as p64:
        p.set_schedule(src, planes=(iBTIin[0], iBTIin[1]), phase=ph)
        with f.Group([p]) as g:
            (mode, by), ms = g.autotune(2)
            assert mode in (0, 1, 2, 3) and by in (1, 2, 4) and ms > 0
            assert p.check_finite() == (True, 0.0)  # left at the zero state
            with pytest.raises(f.FdtdError):
                g.run(0, src.shape[0] + 1)  # beyond the schedule
        with pytest.raises(f.FdtdError):
            f.Group([p, p64])  # FP64 member
        with pytest.raises(f.FdtdError):
            f.Group([p, p])  # the same plan twice
