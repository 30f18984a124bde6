"""The drop-in's deck reader (CPU): input.txt and the Med/Mode/Xi files of the
golden decks, against the arrays they were written from and the reference
FDTD's own report of the same deck (tests/golden/decks/*/reference_stderr.txt)."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN

DECKS = sorted(d for d in os.listdir(os.path.join(GOLDEN, "decks")))


def _ref_lines(name):
    with open(os.path.join(GOLDEN, "decks", name, "reference_stderr.txt")) as f:
        return f.read().splitlines()


@pytest.mark.parametrize("name", DECKS)
def test_deck_reader_matches_written_arrays(built, name):
    from smatranem_gb300 import decks
    root = os.path.join(GOLDEN, "decks", name)
    d = decks.load(os.path.join(root, "input.txt"))
    with np.load(os.path.join(root, "media.npz")) as z:
        assert np.array_equal(d["mu"], z["mu"]) and np.array_equal(d["epsi"], z["epsi"])
        assert d["min_dt"] == float(z["min_dt"])
    lines = _ref_lines(name)
    start = [l for l in lines if l.startswith("Start = ")][0]
    iB, iI, mode, iT = (int(x) for x in re.findall(r"= ([+-]?\d+)", start))
    assert d["iBTIin"] == (iB, iT, iI, mode)
    L3d = [l for l in lines if l.startswith("L3d")]
    if L3d:
        assert int(re.findall(r"L3d = (\d+)", L3d[0])[0]) == d["L"][0] * d["L"][1] * d["L"][2]


@pytest.mark.parametrize("name", DECKS)
def test_precompute_report_matches_reference(built, name):
    """sigma lines, set_tau line and the cell census as the reference prints them."""
    from smatranem_gb300 import decks, fdtd
    root = os.path.join(GOLDEN, "decks", name)
    d = decks.load(os.path.join(root, "input.txt"))
    L = d["L"]
    sig = fdtd.set_sigma(L, d["mu"], d["epsi"])
    mine = []
    off = (0, 2 * L[0], 2 * (L[0] + L[1]))
    for a in range(3):
        for j in range(L[a]):
            for h in range(2):
                v = sig[off[a] + h + 2 * j]
                if v != 0.0:
                    mine.append(f"l{a} = {j}.{5 if h else 0}, sigma = {v:.5e}")
    ref = [l for l in _ref_lines(name) if re.match(r"l\d = ", l)]
    assert mine == ref
    n, iR, iI = fdtd.set_tau(d["omega"], d["min_dt"] / d["dt_factor"])
    import math
    dphi = 2 * math.pi / n
    line = [l for l in _ref_lines(name) if l.startswith("omega = ")][0]
    assert f"N_2pi = {n}," in line
    assert f"tau_R = {1 / iR:.5e}, tau_I = {1 / iI:.5e}" in line
    mu2, ep2 = fdtd.remove_sigma(L, d["mu"], d["epsi"], sig)
    cont, addr, ln = fdtd.set_address(L, sig, mu2, ep2)
    census = [l for l in _ref_lines(name) if l.startswith("L3d")]
    if census:
        assert census[0] == f"L3d = {L[0] * L[1] * L[2]}, Lnotn = {ln}"


def test_deck_reader_errors(built, tmp_path):
    from smatranem_gb300 import decks, fdtd
    p = tmp_path / "input.txt"
    p.write_text("Prefix = ./nowhere\n")
    with pytest.raises(fdtd.FdtdError, match="4 control commands"):
        decks.load(str(p))
    p.write_text("Prefix = ./nowhere\nBoundaryCondition: B0 = 1, B1 = 1, B2 = 1\n"
                 "ModeP: a = y, b = D, 1st = B1, 2nd = T1\n"
                 "FDTD: ramp-period = 1, cw-period = 1, stop-period = 3, incident-point = B2, incident-mode = +1, "
                 "Dt_factor = 1.\n")
    with pytest.raises(fdtd.FdtdError, match="open error"):
        decks.load(str(p))


def test_deck_binary_cache(built, tmp_path):
    """"FDTD_GPU: cache = y" keeps the parsed deck in <prefix>.smatdeck: a second
    load reads it (same arrays and tilde-Xi columns, bit for bit); touching a
    data file or dropping the key makes the loader parse the text again."""
    import shutil
    from smatranem_gb300 import decks
    for name in DECKS:
        dst = tmp_path / name
        shutil.copytree(os.path.join(GOLDEN, "decks", name), dst)
        txt = str(dst / "input.txt")
        with open(txt) as f:
            plain = f.read()
        with open(txt, "a") as f:
            f.write("\tFDTD_GPU: cache = y\n")
        a = decks.load(txt)
        b = decks.load(txt)
        assert not a["from_cache"] and b["from_cache"]
        for k in ("mu", "epsi", "Hinc", "Einc"):
            assert np.array_equal(a[k], b[k])
        for k in ("L", "iBTIin", "min_dt", "nreal", "omega", "time_period"):
            assert a[k] == b[k]
        rng = np.random.default_rng(1)
        pl = a["L"][0] * a["L"][1]
        HB, EB = (rng.standard_normal(2 * pl) + 1j * rng.standard_normal(2 * pl) for _ in range(2))
        for which in (0, 1):
            s_parse = decks.smatrix(txt, which, HB, EB)  # from the cache now
            with open(txt, "w") as f:
                f.write(plain)
            s_text = decks.smatrix(txt, which, HB, EB)
            assert np.array_equal(s_parse, s_text)
            with open(txt, "a") as f:
                f.write("\tFDTD_GPU: cache = y\n")
        med = sorted((dst / "Data").glob("*_Med*.dat"))[0]
        st = os.stat(med)
        os.utime(med, ns=(st.st_atime_ns, st.st_mtime_ns + 1_000_000))
        c = decks.load(txt)
        assert not c["from_cache"] and np.array_equal(c["mu"], a["mu"])
        assert decks.load(txt)["from_cache"]
