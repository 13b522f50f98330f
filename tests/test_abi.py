"""The C ABI library (no GPU needed): it loads, exports every entry point
include/qbg.h declares, builds the reference's basis bit for bit, and
rejects bad arguments with status codes instead of crashing."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden
import qball_gb300 as Q


def header_symbols():
    text = open(os.path.join(ROOT, "include", "qbg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qbg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(Q.LIBPATH)
    syms = header_symbols()
    assert len(syms) >= 16
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the python mirror binds exactly the declared set
    assert sorted(Q.ABI) == syms


def test_version_and_error_string():
    assert b"sm_103a" in Q.lib().qbg_version()
    assert isinstance(Q.lib().qbg_last_error(), bytes)


@pytest.mark.parametrize("name", ["l12_e10", "l20_e10_g48", "l30_e25", "l40_e20"])
def test_product_basis_matches_reference(name):
    g = load_golden(name)
    b = Q.Basis(g["a"], float(g["ecut"]))
    assert (b.ngw, b.nrods) == (int(g["ngw"]), int(g["nrods"]))
    assert tuple(b.np) == tuple(g["np"])
    for k in ("rod_h", "rod_k", "rod_lmin", "rod_size"):
        assert np.array_equal(getattr(b, k), g[k]), k
    sel = g["g_sel"]
    assert np.array_equal(b.kpg2[sel], g["kpg2_sel"])
    assert np.array_equal(b.kpgx.reshape(3, -1)[:, sel], g["kpgx_sel"])


def test_product_basis_matches_oracle_noncubic():
    from oracle import oracle as O
    a = np.array([11.0, 0.3, 0.0, -0.2, 12.5, 0.1, 0.4, 0.0, 9.5])
    b, o = Q.Basis(a, 8.0), O.Basis(a, 8.0)
    for k in ("rod_h", "rod_k", "rod_lmin", "rod_size", "idx", "kpg2", "kpgx"):
        assert np.array_equal(getattr(b, k), getattr(o, k)), k


def test_invalid_arguments_return_status():
    L = Q.lib()
    info = np.zeros(12, np.int32)
    assert L.qbg_basis_dims(None, 1.0, info.ctypes.data_as(ctypes.c_void_p)) == 1
    assert L.qbg_basis_dims(np.zeros(9).ctypes.data_as(ctypes.c_void_p), -1.0,
                            info.ctypes.data_as(ctypes.c_void_p)) == 1
    assert L.qbg_plan_create(None, 8, 8, 8, 0, None) == 1
    assert b"invalid" in L.qbg_last_error()
    assert L.qbg_plan_destroy(None) == 0
    assert L.qbg_hpsi(None, None, 0, None, 0, None, None, None) == 1
    assert L.qbg_etrs_step(None, None, 0, 0, None, 0.1, None, None, None, None, None) == 1
