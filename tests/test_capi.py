"""The C-ABI library: loads without a GPU, exports every function declared in
include/hsspack_gb300.h, and handles argument checks and workspace queries
(LAPACK conventions of SRC/mdstedc.f90:186-245) on the host."""
import ctypes
import os
import re

import numpy as np

import hsspack_gb300 as hp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "hsspack_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    return sorted(set(n for n in names if n not in ("if", "sizeof")))


def test_library_exports_every_declared_symbol():
    L = hp.load()
    names = declared_functions()
    assert "mdstedc_" in names and "hss_mdstedc_dev" in names
    for n in names:
        assert hasattr(L, n), n
        assert n in hp.SIGNATURES, n


def test_config_roundtrip():
    old = hp.set_config(hss_leaf=64, tol=1e-14)
    try:
        c = hp.get_config()
        assert c.hss_leaf == 64 and c.tol == 1e-14
    finally:
        hp.restore_config(old)
    assert hp.get_config().hss_leaf == old.hss_leaf


def _call(compz, n, ldz, lwork, liwork):
    d = np.zeros(max(n, 1)); e = np.zeros(max(n, 1)); z = np.zeros((max(ldz, 1), max(n, 1)), order="F")
    work = np.zeros(1); iwork = np.zeros(1, dtype=np.int32)
    info = hp.mdstedc(compz, n, d, e, z, ldz, work, lwork, iwork, liwork)
    return info, work[0], iwork[0]


def test_mdstedc_workspace_query():
    n = 1000
    info, lw, liw = _call("I", n, n, -1, -1)
    assert info == 0
    assert lw == 1 + 4 * n + n * n and liw == 3 + 5 * n
    info, lw, liw = _call("I", 20, 20, -1, -1)  # N <= SMLSIZ
    assert info == 0 and lw == 2 * 19 and liw == 1
    # COMPZ = 'V' (SRC/mdstedc.f90:222-224), LGN = ceil(log2 N)
    info, lw, liw = _call("V", n, n, -1, -1)
    assert info == 0
    assert lw == 1 + 3 * n + 2 * n * 10 + 4 * n * n and liw == 6 + 6 * n + 5 * n * 10
    info, lw, liw = _call("V", 1024, 1024, -1, -1)
    assert lw == 1 + 3 * 1024 + 2 * 1024 * 10 + 4 * 1024 * 1024
    # the reference's SMLSIZ (25) decides the small case, whatever the GPU's leaf size
    old = hp.set_config(smlsiz=12)
    try:
        info, lw, liw = _call("I", 20, 20, -1, -1)
    finally:
        hp.restore_config(old)
    assert info == 0 and lw == 2 * 19 and liw == 1


def test_mdstedc_argument_errors():
    assert _call("X", 10, 10, 1000, 1000)[0] == -1
    assert _call("V", 10, 5, 1000, 1000)[0] == -6
    assert _call("V", 100, 100, 1 + 4 * 100 + 100 * 100, 10000)[0] == -8  # 'I' size is short
    assert _call("I", -1, 10, 1000, 1000)[0] == -2
    assert _call("I", 10, 5, 1000, 1000)[0] == -6
    assert _call("I", 100, 100, 10, 10000)[0] == -8
    assert _call("I", 100, 100, 100000, 10)[0] == -10


def test_mdstedc_quick_returns_without_gpu():
    assert _call("I", 0, 1, 1, 1)[0] == 0
    d = np.array([3.0]); e = np.zeros(1); z = np.zeros((1, 1), order="F")
    info = hp.mdstedc("I", 1, d, e, z, 1, np.zeros(1), 1, np.zeros(1, dtype=np.int32), 1)
    assert info == 0 and z[0, 0] == 1.0 and d[0] == 3.0


def _band_call(fn, c1, uplo, n, kd, ldab, ldz, lwork, liwork):
    ab = np.zeros((max(ldab, 1), max(n, 1)), order="F")
    w = np.zeros(max(n, 1))
    z = np.zeros((max(ldz, 1), max(n, 1)), order="F")
    work, iwork = np.zeros(1), np.zeros(1, dtype=np.int32)
    info = fn(c1, uplo, n, kd, ab, ldab, w, z, ldz, work, lwork, iwork, liwork)
    return info, work[0], iwork[0]


def test_mdsbedc_arguments_and_workspace():
    # argument numbering and workspace sizes of SRC/mdsbedc.f90:190-228
    n = 300
    assert _band_call(hp.mdsbedc, "X", "U", n, 4, 5, n, -1, -1)[0] == -1
    assert _band_call(hp.mdsbedc, "V", "X", n, 4, 5, n, -1, -1)[0] == -2
    assert _band_call(hp.mdsbedc, "V", "U", -1, 4, 5, n, -1, -1)[0] == -3
    assert _band_call(hp.mdsbedc, "V", "U", n, -1, 5, n, -1, -1)[0] == -4
    assert _band_call(hp.mdsbedc, "V", "U", n, 4, 4, n, -1, -1)[0] == -6
    assert _band_call(hp.mdsbedc, "V", "U", n, 4, 5, n - 1, -1, -1)[0] == -9
    info, lw, liw = _band_call(hp.mdsbedc, "V", "U", n, 4, 5, n, -1, -1)
    assert info == 0 and lw == 1 + 5 * n + 2 * n * n and liw == 3 + 5 * n
    info, lw, liw = _band_call(hp.mdsbedc, "N", "L", n, 4, 5, 1, -1, -1)
    assert info == 0 and lw == 2 * n and liw == 1
    assert _band_call(hp.mdsbedc, "V", "U", n, 4, 5, n, 10, 10)[0] == -11
    # wide bands are accepted (reduced to tridiagonal form on the device)
    assert _band_call(hp.mdsbedc, "V", "U", n, 40, 41, n, -1, -1)[0] == 0
    assert _band_call(hp.mdsbedc, "V", "U", n, 40, 40, n, -1, -1)[0] == -6


def test_mdsbevd_arguments_and_workspace():
    # SRC/mdsbevd.f90:228-263 (its own numbering: -1, -2, -6, -8, -10)
    n = 300
    assert _band_call(hp.mdsbevd, "X", "U", n, 4, 5, n, -1, -1)[0] == -1
    assert _band_call(hp.mdsbevd, "I", "U", -1, 4, 5, n, -1, -1)[0] == -2
    assert _band_call(hp.mdsbevd, "I", "U", n, 4, 5, n - 1, -1, -1)[0] == -6
    info, lw, liw = _band_call(hp.mdsbevd, "I", "U", n, 4, 5, n, -1, -1)
    assert info == 0 and lw == 1 + 4 * n + n * n and liw == 3 + 5 * n
    assert _band_call(hp.mdsbevd, "I", "U", n, 4, 5, n, 10, 10)[0] == -8


def test_dhssmm_arguments_without_gpu():
    # argument checks and the N = 0 quick return happen on the host
    A = np.zeros((4, 4), order="F")
    B = np.zeros((4, 3), order="F")
    assert hp.dhssmm(A, B, 2, 1e-11, m=3)[0] == -3                      # M != N
    assert hp.dhssmm(A, np.zeros((3, 2), order="F"), 2, 1e-11)[0] == -6  # LDB < N
    assert hp.dhssmm(A, B, 0, 1e-11)[0] == -10                          # ni < 1
    assert hp.dhssmm(A, B, 2, 1e-11, ncol=0)[0] == -11                  # ncol < 1
    assert hp.dhssmml(A, np.zeros((3, 4), order="F"), 2, 1e-11, ncol=0)[0] == -11
    A0 = np.zeros((1, 0), order="F")
    B0 = np.zeros((1, 0), order="F")
    assert hp.dhssmm(A0, B0, 2, 1e-11)[0] == 0
