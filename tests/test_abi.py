"""The C ABI library loads and exports every symbol include/smatran_fdtd.h declares."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "smatran_fdtd.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(smat_\w+)\s*\(", text)))


def test_header_declares_the_api():
    names = declared_symbols()
    for required in ("smat_main_calc", "smat_fdtd_create", "smat_fdtd_run", "smat_fdtd_get_monitor",
                     "smat_set_sigma", "smat_remove_sigma", "smat_set_address", "smat_coefficients"):
        assert required in names


def test_library_exports_every_declared_symbol(built):
    from smatranem_gb300 import fdtd
    lib = ctypes.CDLL(fdtd.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_error_message_is_reported(built):
    from smatranem_gb300 import fdtd
    lib = fdtd.lib()
    n = ctypes.c_int()
    r = ctypes.c_double()
    i = ctypes.c_double()
    assert lib.smat_set_tau(ctypes.c_double(0.0), ctypes.c_double(1.0), ctypes.byref(n), ctypes.byref(r),
                            ctypes.byref(i)) == -1
    assert b"positive" in lib.smat_last_error()


@pytest.mark.parametrize("L,batch,msg", [
    ((1000, 1000, 1000, 1), 1, b"too large"),   # 3*L3D past 32-bit reference indices
    ((0, 4, 4, 1), 1, b"positive"),
    ((4, 4, -1, 1), 1, b"positive"),
    ((4, 4, 4, 1), 0, b"batch"),
])
def test_create_rejects_bad_shapes(built, L, batch, msg):
    """Plan creation checks the grid before touching the GPU or the arrays."""
    from smatranem_gb300 import fdtd
    dummy = np.zeros(8, np.complex128)
    with pytest.raises(fdtd.FdtdError) as e:
        fdtd.Plan.create(L, (0, 0, 0), (0, 1, 0, 1), 1.0, 0.0, dummy, dummy, np.zeros(8), batch=batch)
    assert e.value.code == -1 and msg in str(e.value).encode()
