"""CPU oracle for the HSS divide-and-conquer merge -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package; it is the checker, never the product path.

It wraps ``_build/libhss_oracle.so`` (built from hss_oracle.cpp by build.py), a
C++ restatement of HSSPACK's MDSTEDC/MDLAED0-3/DHSSEVC chain that calls LAPACK
from SciPy's bundled OpenBLAS.
"""
import ctypes
import glob
import os

import numpy as np

from . import build as _build

_lib = None


class HsoConfig(ctypes.Structure):
    _fields_ = [("hss_leaf", ctypes.c_int), ("bsmlz", ctypes.c_int),
                ("tol", ctypes.c_double), ("smlsiz", ctypes.c_int)]


class HsoStats(ctypes.Structure):
    _fields_ = [("n_merges", ctypes.c_int), ("n_hss_merges", ctypes.c_int),
                ("n_dense_merges", ctypes.c_int), ("max_k", ctypes.c_int),
                ("max_rank", ctypes.c_int), ("total_k", ctypes.c_longlong),
                ("n_swaps", ctypes.c_longlong)]


def openblas_path():
    import scipy
    base = os.path.dirname(scipy.__file__)
    cands = sorted(glob.glob(os.path.join(base, "..", "scipy.libs", "libscipy_openblas*.so")))
    if not cands:
        cands = sorted(glob.glob(os.path.join(base, ".libs", "libscipy_openblas*.so")))
    if not cands:
        raise RuntimeError("SciPy's bundled OpenBLAS was not found")
    return os.path.realpath(cands[0])


_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.hso_init.argtypes = [ctypes.c_char_p]
        L.hso_set_threads.argtypes = [ctypes.c_int]
        L.hso_mdstedc.argtypes = [ctypes.c_char, ctypes.c_int, _D, _D, _D, ctypes.c_int,
                                  ctypes.POINTER(HsoConfig)]
        L.hso_dstedc_lapack.argtypes = [ctypes.c_int, _D, _D, _D, ctypes.c_int]
        L.hso_secular.argtypes = [ctypes.c_int, _D, _D, ctypes.c_double, _D, _D, _D]
        L.hso_lowner.argtypes = [ctypes.c_int, _D, _D, _D, _D, _D]
        L.hso_cauchy_eig_dense.argtypes = [ctypes.c_int, _D, _D, _D, _D, _D, _D]
        L.hso_dhssevc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, _D, _D, _D,
                                  _D, _D, _D, _D, ctypes.c_int, ctypes.c_int, _I]
        L.hso_cauchylike.argtypes = [_D, _D, _D, _D, _D, ctypes.c_int, ctypes.c_int]
        L.hso_get_stats.argtypes = [ctypes.POINTER(HsoStats)]
        L.hso_cauchyhssmm.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_int,
                                      ctypes.c_double, _D, ctypes.c_int, ctypes.c_int]
        L.hso_cauchyhssmm.restype = ctypes.c_int
        rc = L.hso_init(openblas_path().encode())
        if rc != 0:
            raise RuntimeError("oracle: cannot load LAPACK (rc=%d)" % rc)
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_D)


def set_threads(n):
    lib().hso_set_threads(int(n))


def config(hss_leaf=200, bsmlz=1500, tol=1e-17, smlsiz=25):
    return HsoConfig(hss_leaf, bsmlz, tol, smlsiz)


def stats():
    s = HsoStats()
    lib().hso_get_stats(ctypes.byref(s))
    return {k: getattr(s, k) for k, _ in HsoStats._fields_}


def eigh_tridiagonal(d, e, hss_leaf=200, bsmlz=1500, tol=1e-17, smlsiz=25):
    """Oracle MDSTEDC('I'): returns (w, Q) with Q an (n, n) float64 array whose
    columns are the eigenvectors (Fortran order in memory)."""
    n = len(d)
    dd = np.array(d, dtype=np.float64, copy=True)
    ee = np.zeros(max(n, 1), dtype=np.float64)
    ee[: max(n - 1, 0)] = np.asarray(e, dtype=np.float64)[: max(n - 1, 0)]
    Z = np.zeros((n, n), dtype=np.float64, order="F")
    cfg = config(hss_leaf, bsmlz, tol, smlsiz)
    info = lib().hso_mdstedc(b"I", n, _p(dd), _p(ee), _p(Z), max(n, 1), ctypes.byref(cfg))
    if info != 0:
        raise RuntimeError("oracle mdstedc info=%d" % info)
    return dd, Z


def dstedc_lapack(d, e):
    """LAPACK DSTEDC('I') from OpenBLAS: the accuracy oracle."""
    n = len(d)
    dd = np.array(d, dtype=np.float64, copy=True)
    ee = np.zeros(max(n, 1), dtype=np.float64)
    ee[: max(n - 1, 0)] = np.asarray(e, dtype=np.float64)[: max(n - 1, 0)]
    Z = np.zeros((n, n), dtype=np.float64, order="F")
    info = lib().hso_dstedc_lapack(n, _p(dd), _p(ee), _p(Z), max(n, 1))
    if info != 0:
        raise RuntimeError("dstedc info=%d" % info)
    return dd, Z


def secular(dlamda, z, rho):
    """All roots of 1 + rho*sum z_i^2/(d_i - x) by LAPACK DLAED4.
    Returns (lam, difl, difr)."""
    k = len(dlamda)
    dl = np.ascontiguousarray(dlamda, dtype=np.float64)
    zz = np.ascontiguousarray(z, dtype=np.float64)
    lam = np.zeros(k); difl = np.zeros(k); difr = np.zeros(k)
    info = lib().hso_secular(k, _p(dl), _p(zz), float(rho), _p(lam), _p(difl), _p(difr))
    if info != 0:
        raise RuntimeError("dlaed4 failed at root %d" % info)
    return lam, difl, difr


def lowner(dlamda, difl, difr, z):
    """Loewner z-hat and column scalings alpha (MDLAED3's steps)."""
    k = len(dlamda)
    dl = np.ascontiguousarray(dlamda, dtype=np.float64)
    zz = np.array(z, dtype=np.float64, copy=True)
    alpha = np.zeros(k)
    lib().hso_lowner(k, _p(dl), _p(np.ascontiguousarray(difl, dtype=np.float64)),
                     _p(np.ascontiguousarray(difr, dtype=np.float64)), _p(zz), _p(alpha))
    return zz, alpha


def cauchy_eig_dense(F, u, v, difl, difr):
    k = len(F)
    C = np.zeros((k, k), dtype=np.float64, order="F")
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (F, u, v, difl, difr)]
    lib().hso_cauchy_eig_dense(k, *[_p(a) for a in args], _p(C))
    return C


def dhssevc(F, u, v, difl, difr, Q, ni=200, tol=1e-17):
    """Q (nrows x K, Fortran order) <- Q @ C through the HSS compression."""
    k = len(F)
    Q = np.asfortranarray(np.array(Q, dtype=np.float64, copy=True))
    nrows = Q.shape[0]
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (F, F, u, v, difl, difr)]
    mr = ctypes.c_int(0)
    rc = lib().hso_dhssevc(k, ni, tol, *[_p(a) for a in args], _p(Q), max(nrows, 1), nrows,
                           ctypes.byref(mr))
    if rc != 0:
        raise RuntimeError("dhssevc rc=%d" % rc)
    return Q, mr.value


def cauchyhssmm(D, F, U, V, B, ni, tol):
    """CauchyHssMM (SRC/cauchyhssmm.f90) restated with the VP2 module: returns
    (C @ B, max generator rank) for C(i,j) = U_i V_j / (D_i - F_j)."""
    n = len(D)
    args = [np.array(a, dtype=np.float64, copy=True) for a in (D, F, U, V)]
    Bf = np.array(B, dtype=np.float64, order="F", copy=True)
    r = lib().hso_cauchyhssmm(n, *[_p(a) for a in args], int(ni), float(tol), _p(Bf),
                              Bf.shape[0], Bf.shape[1])
    return Bf, r
