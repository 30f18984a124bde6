"""The drop-in `FDTD` executable on the golden decks, against the reference
FDTD's report of the same decks.  FP64 is bit-identical, so every line of the
|S|^2 table (printed with %.20e) must match exactly.  The lines that differ by
design: the start-time stamp, and the check_Xi diagnostic (||tilXi^H Xi - I||)
which needs the whole Xi matrix the drop-in does not read."""
import os
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "smatranem_gb300", "_build", "FDTD")
DECKS = sorted(os.listdir(os.path.join(GOLDEN, "decks")))


def _comparable(text):
    return [l for l in text.splitlines() if l and not l.startswith("# Start time") and not l.startswith("tilXi^+ Xi")]


@pytest.mark.parametrize("name", DECKS)
def test_dropin_report_matches_reference(built, tmp_path, name):
    src = os.path.join(GOLDEN, "decks", name)
    work = tmp_path / name
    shutil.copytree(src, work)
    r = subprocess.run([EXE, "input.txt"], cwd=work, capture_output=True, text=True, timeout=600)
    ref = open(os.path.join(src, "reference_stderr.txt")).read()
    ref_status = int(open(os.path.join(src, "reference_status.txt")).read())
    if ref_status != 0:
        # the reference aborts (a PML cell on a monitor plane); so does the drop-in, without running
        assert r.returncode != 0
        assert "monitor plane" in r.stderr
        return
    assert r.returncode == 0, r.stderr
    mine, theirs = _comparable(r.stderr), _comparable(ref)
    table = theirs.index(next(l for l in theirs if l.startswith("Bottom |S_")))
    assert mine[mine.index(theirs[table]):] == theirs[table:]  # the |S|^2 tables, byte for byte
    assert mine == theirs  # and every other line of the report


def test_dropin_fp32_within_tolerance(built, tmp_path):
    """The optional FP32 mode ("FDTD_GPU: precision = FP32" in input.txt, a key the
    reference ignores): |S|^2 within 1e-4 relative of the reference."""
    name = "deck_periodic"
    src = os.path.join(GOLDEN, "decks", name)
    work = tmp_path / name
    shutil.copytree(src, work)
    with open(work / "input.txt", "a") as f:
        f.write("\tFDTD_GPU: precision = FP32\n")
    r = subprocess.run([EXE, "input.txt"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr

    def table(text):
        vals = []
        for l in text.splitlines():
            parts = [p.strip() for p in l.split(",")]
            if len(parts) == 4 and parts[0][:1] in "+-":
                vals += [float(parts[1]), float(parts[3])]
        return vals
    a, b = table(r.stderr), table(open(os.path.join(src, "reference_stderr.txt")).read())
    assert len(a) == len(b) > 0
    big = max(b)
    for x, y in zip(a, b):
        assert abs(x - y) <= 1e-4 * big


@pytest.mark.parametrize("name", DECKS)
def test_dropin_with_deck_cache(built, tmp_path, name):
    """With "FDTD_GPU: cache = y" the first run writes <prefix>.smatdeck and the
    second reads it; both print the reference's report."""
    src = os.path.join(GOLDEN, "decks", name)
    if int(open(os.path.join(src, "reference_status.txt")).read()) != 0:
        pytest.skip("a deck the reference rejects")
    work = tmp_path / name
    shutil.copytree(src, work)
    with open(work / "input.txt", "a") as f:
        f.write("\tFDTD_GPU: cache = y\n")
    ref = _comparable(open(os.path.join(src, "reference_stderr.txt")).read())
    for run in range(2):
        r = subprocess.run([EXE, "input.txt"], cwd=work, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        assert _comparable(r.stderr) == ref, run
        assert any(p.name.endswith(".smatdeck") for p in (work / "Data").iterdir())


def _table(text):
    rows = []
    for l in text.splitlines():
        parts = [p.strip() for p in l.split(",")]
        if len(parts) == 4 and parts[0][:1] in "+-":
            rows.append((parts[0], float(parts[1]), parts[2], float(parts[3])))
    return rows


def test_dropin_solves_port_modes(built, tmp_path):
    """"FDTD_GPU: modes = solve": the drop-in computes the port modes of the two
    monitor layers with the GPU mode solver instead of reading the Mode / Xi
    files (deleted here), and reports the same |S|^2 as the reference FDTD fed
    with the stock Mcalc's files -- same modes, same N_real, values within
    1e-8 relative (the modes agree to the solver's residual, not bit for bit)."""
    name = "deck_modes"
    src = os.path.join(GOLDEN, "decks", name)
    work = tmp_path / name
    shutil.copytree(src, work)
    for fn in os.listdir(work / "Data"):
        if fn.endswith(("Mode.dat", "Xi.dat")):
            os.remove(work / "Data" / fn)
    with open(work / "input.txt", "a") as f:
        f.write("\tFDTD_GPU: modes = solve, nmodes = 16\n")
    r = subprocess.run([EXE, "input.txt"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    a, b = _table(r.stderr), _table(open(os.path.join(src, "reference_stderr.txt")).read())
    assert len(a) == len(b) == 4
    big = max(max(x[1], x[3]) for x in b)
    for x, y in zip(a, b):
        assert x[0] == y[0] and x[2] == y[2]
        assert abs(x[1] - y[1]) <= 1e-8 * big and abs(x[3] - y[3]) <= 1e-8 * big


SCALC_EXE = os.path.join(ROOT, "smatranem_gb300", "_build", "Scalc")


def _smatrix_file(path):
    rows = {}
    header = {}
    for line in open(path):
        if line.startswith("# Mode numbers") or line.startswith("# Target layers") or line.startswith("# Omega"):
            header[line.split(":")[0].strip()] = line.split(":", 1)[1].strip()
        if line.startswith("#"):
            continue
        m, n, re_, im_, a2 = line.split()
        rows[(int(m), int(n))] = (float(re_), float(im_), float(a2))
    return header, rows


def test_scalc_dropin_matches_reference(built, tmp_path):
    """The drop-in `Scalc input.txt` on the golden mode deck (Mode / Xi files from
    the stock Mcalc): the same header facts and every S entry of the stock
    Scalc's <prefix>_Smatrix.dat within 1e-10."""
    src = os.path.join(GOLDEN, "decks", "deck_modes")
    work = tmp_path / "deck_modes"
    shutil.copytree(src, work)
    r = subprocess.run([SCALC_EXE, "input.txt"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    h1, s1 = _smatrix_file(work / "Data" / "deck_Smatrix.dat")
    h2, s2 = _smatrix_file(os.path.join(src, "reference_Smatrix.dat"))
    assert h1 == h2
    assert s1.keys() == s2.keys() and len(s1) == 16
    for k in s2:
        assert all(abs(a - b) < 1e-10 for a, b in zip(s1[k], s2[k])), (k, s1[k], s2[k])


def test_scalc_dropin_errors(built, tmp_path):
    src = os.path.join(GOLDEN, "decks", "deck_modes")
    work = tmp_path / "deck_modes"
    shutil.copytree(src, work)
    os.remove(work / "Data" / "deck_tXi.dat")
    r = subprocess.run([SCALC_EXE, "input.txt"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and "open error" in r.stderr
    r = subprocess.run([SCALC_EXE], cwd=work, capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
    r = subprocess.run([SCALC_EXE, "-v"], cwd=work, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "scattering matrix" in r.stderr
