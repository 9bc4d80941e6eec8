"""hsspack_gb300 -- GB300 (sm_103a) HSS-accelerated divide-and-conquer eigensolver.

Python mirror of HSSPACK's Fortran interface for the DC merge path, over the
C ABI of ``_lib/libhsspack_gb300.so`` (declared in include/hsspack_gb300.h).
The compute runs in hand-written CUDA kernels; there is no CPU fallback: if the
library cannot be loaded every entry point raises.

Host-array entry points follow the Fortran argument meaning and LAPACK error
convention (INFO = -i for a bad i-th argument, INFO > 0 for a numerical
failure):

* :func:`mdstedc` -- ``MDSTEDC(COMPZ,N,D,E,Z,LDZ,WORK,LWORK,IWORK,LIWORK,INFO)``
  (SRC/mdstedc.f90:139).
* :func:`cauchylike` -- ``Cauchylike(A,D,F,u,v,M,N)`` (SRC/Cauchylike.f90:1).

Device entry points take torch CUDA tensors (torch is used only to hold device
memory and streams): :func:`mdstedc_dev`, :func:`mdstedc_batch_dev`
(many problems of uneven sizes in one call), :func:`secular_dev`,
:func:`lowner_dev`, :func:`dhssevc_dev`, :func:`cauchy_eig_dev`.
"""
import ctypes
import math
import os

import numpy as np

from . import build as _build

__all__ = [
    "Config", "Stats", "load", "get_config", "set_config", "get_stats", "finalize",
    "mdstedc", "eigh_tridiagonal", "cauchylike", "mdstedc_dev", "mdstedc_batch_dev",
    "batch_offsets", "secular_dev",
    "lowner_dev", "dhssevc_dev", "cauchy_eig_dev", "HssError",
]


class HssError(RuntimeError):
    pass


class Config(ctypes.Structure):
    _fields_ = [("hss_leaf", ctypes.c_int), ("bsmlz", ctypes.c_int), ("tol", ctypes.c_double),
                ("smlsiz", ctypes.c_int), ("precision", ctypes.c_int),
                ("predictor", ctypes.c_int), ("batched", ctypes.c_int),
                ("profile", ctypes.c_int), ("sec_terms", ctypes.c_int),
                ("split_min_log2", ctypes.c_int), ("small_nk", ctypes.c_int),
                ("split_min_m", ctypes.c_int), ("sec_threads", ctypes.c_int),
                ("gemm_path", ctypes.c_int), ("reserved", ctypes.c_int * 2)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Stats(ctypes.Structure):
    _fields_ = [("n_levels", ctypes.c_int), ("n_merges", ctypes.c_int),
                ("n_hss_merges", ctypes.c_int), ("n_dense_merges", ctypes.c_int),
                ("max_k", ctypes.c_int), ("max_rank", ctypes.c_int),
                ("total_k", ctypes.c_longlong), ("secular_iters", ctypes.c_longlong),
                ("secular_roots", ctypes.c_longlong), ("predictor_fallbacks", ctypes.c_longlong),
                ("kernel_launches", ctypes.c_longlong), ("ms_total", ctypes.c_double),
                ("stage_ms", ctypes.c_double * 16), ("stage_calls", ctypes.c_longlong * 16),
                ("stage_bytes", ctypes.c_longlong * 16), ("stage_flops", ctypes.c_double * 16),
                ("host_h2d_bytes", ctypes.c_longlong), ("host_d2h_bytes", ctypes.c_longlong),
                ("reserved", ctypes.c_int * 4)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}
        for k in ("stage_ms", "stage_calls", "stage_bytes", "stage_flops"):
            d[k] = {STAGES[i]: d[k][i] for i in range(len(STAGES))}
        return d


STAGES = ["leaf", "prepare", "givens", "secular", "lowner", "build_S", "gather", "gemm",
          "scatter", "finish", "final_gather", "hss_build", "hss_multiply", "other", "predict"]


_lib = None
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_V = ctypes.c_void_p

# exported symbol -> (restype, argtypes); must match include/hsspack_gb300.h
SIGNATURES = {
    "hss_default_config": (None, [ctypes.POINTER(Config)]),
    "hss_set_config": (None, [ctypes.POINTER(Config)]),
    "hss_get_config": (None, [ctypes.POINTER(Config)]),
    "hss_get_stats": (None, [ctypes.POINTER(Stats)]),
    "hss_last_error": (ctypes.c_char_p, []),
    "hss_finalize": (ctypes.c_int, []),
    "mdstedc_": (None, [ctypes.c_char_p, _I, _D, _D, _D, _I, _D, _I, _I, _I, _I, ctypes.c_size_t]),
    "cauchylike_": (None, [_D, _D, _D, _D, _D, _I, _I]),
    "mdsbevd_": (None, [ctypes.c_char_p, ctypes.c_char_p, _I, _I, _D, _I, _D, _D, _I, _D, _I, _I,
                        _I, _I, ctypes.c_size_t, ctypes.c_size_t]),
    "mdsbedc_": (None, [ctypes.c_char_p, ctypes.c_char_p, _I, _I, _D, _I, _D, _D, _I, _D, _I, _I,
                        _I, _I, ctypes.c_size_t, ctypes.c_size_t]),
    "hss_mdsbevd_dev": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _V, ctypes.c_int, _V, _V,
                                       ctypes.c_int, _V]),
    "mdbdsdc_": (None, [ctypes.c_char_p, ctypes.c_char_p, _I, _D, _D, _D, _I, _D, _I, _D, _I, _D,
                        _I, _I, ctypes.c_size_t, ctypes.c_size_t]),
    "hss_mdbdsdc_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, ctypes.c_int, _V, ctypes.c_int,
                                       _V]),
    "mdbdsvd_": (None, [_I, _I, _D, _I, _D, _D, _D, _I, _D, _I, _I, _D, _I, _I, _I]),
    "hss_mdbdsvd_dev": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _V, ctypes.c_int, _V, _V,
                                       ctypes.c_int, _V, ctypes.c_int, ctypes.c_int, _V]),
    "cauchyhssmm_": (None, [_D, _D, _D, _D, _I, _I, _D, _I, _D, _I, _D]),
    "hss_cauchyhssmm_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, _V, ctypes.c_int,
                                           ctypes.c_double, _V, ctypes.c_int, ctypes.c_int, _V,
                                           _V]),
    "dhssmm_": (None, [_D, _I, _I, _I, _D, _I, _I, _D, _I, _I, _I, _D, _I]),
    "dhssmml_": (None, [_D, _I, _I, _I, _D, _I, _I, _D, _I, _I, _I, _D, _I]),
    "hss_dhssmm_dev": (ctypes.c_int, [ctypes.c_int, _V, ctypes.c_int, _V, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      _V, _V]),
    "svdhssupdat_": (None, [_D, _D, _D, _D, _I, _D, _I]),
    "hss_svdhssupdat_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, _V, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_int, _V, _V]),
    "hss_svdupd_deflate": (ctypes.c_int, [ctypes.c_int, _D, _D, _I, _I]),
    "hss_bsvd_tree": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _I, _I, _I]),
    "hsscholsolver_": (None, [ctypes.c_char_p, ctypes.c_char_p, _D, _I, _D, _I, _D, _I, _I, _D,
                              _I, _I, ctypes.c_size_t, ctypes.c_size_t]),
    "hss_chol_factor_dev": (ctypes.c_int, [ctypes.c_int, _V, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_int, ctypes.c_int, _V, _V]),
    "hss_chol_solve_dev": (ctypes.c_int, [_V, _V, ctypes.c_int, ctypes.c_int, _V]),
    "hss_chol_pcg_dev": (ctypes.c_int, [_V, ctypes.c_int, _V, ctypes.c_int, _V, _V,
                                        ctypes.c_double, ctypes.c_int, _V, _V, _V]),
    "hss_chol_info": (ctypes.c_int, [_V, _V, _V, _V, _V, _V]),
    "hss_chol_free": (None, [_V]),
    "hss_rcp_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V]),
    "hss_fp64_fma_rate": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _V, _V, _V]),
    "hss_mdstedc_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, ctypes.c_int, _V]),
    "hss_mdstedc_v_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, ctypes.c_int, _V]),
    "hss_mdstedc_batch_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, _V, _V]),
    "hss_secular_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, ctypes.c_double, _V, _V, _V, _V, _V]),
    "hss_lowner_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, _V, _V, _V]),
    "hss_lowner_noalloc_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, _V, _V, _V]),
    "hss_dhssevc_dev": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double, _V, _V, _V, _V,
                                       _V, _V, ctypes.c_int, ctypes.c_int, _V]),
    "hss_cauchy_eig_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, _V, _V, _V, _V]),
    "hss_predictor_nparam": (ctypes.c_int, []),
    "hss_predictor_nfeat": (ctypes.c_int, []),
    "hss_predictor_set": (ctypes.c_int, [_V, _V]),
    "hss_predictor_features_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, ctypes.c_double, _V, _V,
                                                  _V, _V, _V]),
    "hss_predictor_grad_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, _V, _V, _V, _V, _V]),
    "hss_predictor_adam_dev": (ctypes.c_int, [_V, _V, _V, _V, ctypes.c_float, ctypes.c_int, _V]),
    "hss_predict_dev": (ctypes.c_int, [ctypes.c_int, _V, _V, ctypes.c_double, _V, _V]),
    "hss_gemm_dev": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _V, ctypes.c_int,
                                    _V, ctypes.c_int, _V, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, _V]),
}


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library; raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise HssError("libhsspack_gb300.so is not built: run hsspack_gb300/build.py")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _err():
    return load().hss_last_error().decode(errors="replace")


def get_config():
    c = Config()
    load().hss_get_config(ctypes.byref(c))
    return c


def set_config(**kw):
    """Update the process-wide configuration; returns the previous one."""
    old = get_config()
    c = Config()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(old), ctypes.sizeof(Config))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    load().hss_set_config(ctypes.byref(c))
    return old


def restore_config(c):
    load().hss_set_config(ctypes.byref(c))


def get_stats():
    s = Stats()
    load().hss_get_stats(ctypes.byref(s))
    return s.as_dict()


def finalize():
    return load().hss_finalize()


def _pd(a):
    return a.ctypes.data_as(_D)


def mdstedc(compz, n, d, e, z, ldz, work, lwork, iwork, liwork):
    """MDSTEDC with the Fortran argument list; arrays are numpy, modified in
    place (d: eigenvalues, z: eigenvectors in Fortran order).  Returns INFO."""
    L = load()
    info = ctypes.c_int(0)
    n_, ldz_, lw_, liw_ = (ctypes.c_int(int(x)) for x in (n, ldz, lwork, liwork))
    for a, dt in ((d, np.float64), (e, np.float64), (z, np.float64), (work, np.float64),
                  (iwork, np.int32)):
        if a.dtype != dt:
            raise TypeError("array dtype must be %s" % dt)
    if z.ndim == 2 and not z.flags.f_contiguous:
        raise ValueError("z must be Fortran ordered")
    L.mdstedc_(compz.encode() if isinstance(compz, str) else compz, ctypes.byref(n_), _pd(d), _pd(e),
               _pd(z), ctypes.byref(ldz_), _pd(work), ctypes.byref(lw_),
               iwork.ctypes.data_as(_I), ctypes.byref(liw_), ctypes.byref(info), 1)
    return info.value


def eigh_tridiagonal(d, e):
    """Eigenvalues (ascending) and eigenvectors of the symmetric tridiagonal
    (d, e) through MDSTEDC('I').  Returns (w, Z) with Z Fortran ordered."""
    n = len(d)
    dd = np.array(d, dtype=np.float64, copy=True)
    ee = np.zeros(max(n, 1), dtype=np.float64)
    ee[: max(n - 1, 0)] = np.asarray(e, dtype=np.float64)[: max(n - 1, 0)]
    Z = np.zeros((n, n), dtype=np.float64, order="F")
    work = np.zeros(1)
    iwork = np.zeros(1, dtype=np.int32)
    info = mdstedc("I", n, dd, ee, Z, max(1, n), work, -1, iwork, -1)
    if info != 0:
        raise HssError("MDSTEDC workspace query: INFO=%d" % info)
    lw, liw = int(work[0]), int(iwork[0])
    # The GPU implementation keeps its workspace in device memory and touches
    # only WORK(1) and IWORK(1), so one-element arrays declared with the
    # queried sizes are passed instead of LWORK = 1 + 4N + N^2 doubles.
    info = mdstedc("I", n, dd, ee, Z, max(1, n), work, lw, iwork, liw)
    if info != 0:
        raise HssError("MDSTEDC INFO=%d: %s" % (info, _err()))
    return dd, Z


def _band_call(name, c1, uplo, n, kd, ab, ldab, w, z, ldz, work, lwork, iwork, liwork):
    for a, dt in ((ab, np.float64), (w, np.float64), (z, np.float64), (work, np.float64),
                  (iwork, np.int32)):
        if a.dtype != dt:
            raise TypeError("array dtype must be %s" % dt)
    for a in (ab, z):
        if a.ndim == 2 and not a.flags.f_contiguous:
            raise ValueError("band and eigenvector arrays must be Fortran ordered")
    info = ctypes.c_int(0)
    ints = [ctypes.c_int(int(x)) for x in (n, kd, ldab, ldz, lwork, liwork)]
    getattr(load(), name)(c1.encode(), uplo.encode(), ctypes.byref(ints[0]), ctypes.byref(ints[1]),
                          _pd(ab), ctypes.byref(ints[2]), _pd(w), _pd(z), ctypes.byref(ints[3]),
                          _pd(work), ctypes.byref(ints[4]), iwork.ctypes.data_as(_I),
                          ctypes.byref(ints[5]), ctypes.byref(info), 1, 1)
    return info.value


def mdsbevd(compz, uplo, n, kd, ab, ldab, d, q, ldq, work, lwork, iwork, liwork):
    """MDSBEVD with the Fortran argument list (SRC/mdsbevd.f90:183); numpy
    arrays, ab and q Fortran ordered.  Returns INFO."""
    return _band_call("mdsbevd_", compz, uplo, n, kd, ab, ldab, d, q, ldq, work, lwork, iwork,
                      liwork)


def mdsbedc(jobz, uplo, n, kd, ab, ldab, w, z, ldz, work, lwork, iwork, liwork):
    """MDSBEDC with the Fortran argument list (SRC/mdsbedc.f90:166).  Returns INFO."""
    return _band_call("mdsbedc_", jobz, uplo, n, kd, ab, ldab, w, z, ldz, work, lwork, iwork,
                      liwork)


def eigh_banded(ab, lower=False):
    """Eigenvalues (ascending) and eigenvectors of the symmetric band matrix in
    LAPACK band storage ab (kd + 1, n) through MDSBEDC('V').  Returns (w, Z)."""
    ab = np.asfortranarray(ab, dtype=np.float64)
    kd, n = ab.shape[0] - 1, ab.shape[1]
    w = np.zeros(n)
    Z = np.zeros((n, n), order="F")
    work = np.zeros(1)
    iwork = np.zeros(1, dtype=np.int32)
    uplo = "L" if lower else "U"
    info = mdsbedc("V", uplo, n, kd, ab, kd + 1, w, Z, max(1, n), work, -1, iwork, -1)
    if info != 0:
        raise HssError("MDSBEDC workspace query: INFO=%d" % info)
    # the GPU path keeps its workspace in HBM; only WORK(1), IWORK(1) are touched
    info = mdsbedc("V", uplo, n, kd, ab, kd + 1, w, Z, max(1, n), work, int(work[0]), iwork,
                   int(iwork[0]))
    if info != 0:
        raise HssError("MDSBEDC INFO=%d: %s" % (info, _err()))
    return w, Z


def mdsbevd_dev(kd, ab, w, z, stream=None):
    """Device band eigensolve: ab (n, kd + 1) tensor whose memory is the
    column-major (kd + 1) x n upper band storage; w (n,), z (n, n) column-major."""
    n = w.numel()
    info = load().hss_mdsbevd_dev(n, kd, _ptr(ab), kd + 1, _ptr(w), _ptr(z), max(1, n),
                                  _stream(stream))
    if info != 0:
        raise HssError("hss_mdsbevd_dev INFO=%d: %s" % (info, _err()))
    return info


def mdbdsdc(uplo, compq, n, d, e, u, ldu, vt, ldvt, q, iq, work, iwork):
    """MDBDSDC with the Fortran argument list (SRC/mdbdsdc.f90:1); numpy arrays,
    u and vt Fortran ordered.  Returns INFO."""
    for a, dt in ((d, np.float64), (e, np.float64), (u, np.float64), (vt, np.float64),
                  (q, np.float64), (work, np.float64), (iq, np.int32), (iwork, np.int32)):
        if a.dtype != dt:
            raise TypeError("array dtype must be %s" % dt)
    for a in (u, vt):
        if a.ndim == 2 and not a.flags.f_contiguous:
            raise ValueError("u and vt must be Fortran ordered")
    info = ctypes.c_int(0)
    n_, ldu_, ldvt_ = (ctypes.c_int(int(x)) for x in (n, ldu, ldvt))
    load().mdbdsdc_(uplo.encode(), compq.encode(), ctypes.byref(n_), _pd(d), _pd(e), _pd(u),
                    ctypes.byref(ldu_), _pd(vt), ctypes.byref(ldvt_), _pd(q),
                    iq.ctypes.data_as(_I), _pd(work), iwork.ctypes.data_as(_I),
                    ctypes.byref(info), 1, 1)
    return info.value


def svd_bidiagonal(d, e, lower=False):
    """(s descending, U, VT) of the square bidiagonal (d, e) through MDBDSDC('I')."""
    n = len(d)
    dd = np.array(d, dtype=np.float64, copy=True)
    ee = np.zeros(max(n, 1))
    ee[:max(n - 1, 0)] = np.asarray(e, dtype=np.float64)[:max(n - 1, 0)]
    U = np.zeros((n, n), order="F")
    VT = np.zeros((n, n), order="F")
    one = np.zeros(1)
    ione = np.zeros(1, dtype=np.int32)
    info = mdbdsdc("L" if lower else "U", "I", n, dd, ee, U, max(1, n), VT, max(1, n), one, ione,
                   one, ione)
    if info != 0:
        raise HssError("MDBDSDC INFO=%d: %s" % (info, _err()))
    return dd, U, VT


def mdbdsdc_dev(d, e, u, vt, stream=None):
    """Device bidiagonal SVD: d (n,) -> singular values (descending), u and vt
    (n, n) column-major storage."""
    n = d.numel()
    info = load().hss_mdbdsdc_dev(n, _ptr(d), _ptr(e), _ptr(u), max(1, n), _ptr(vt), max(1, n),
                                  _stream(stream))
    if info != 0:
        raise HssError("hss_mdbdsdc_dev INFO=%d: %s" % (info, _err()))
    return info


def mdbdsvd(n, sb, ab, ldab, a, s, u, ldu, vt, ldvt, smlsiz, work, lwork, iwork):
    """MDBDSVD with the Fortran argument list (SRC/mdbdsvd.f90:1); numpy arrays,
    ab (LDAB x N), u and vt Fortran ordered.  Returns (INFO, SMLSIZ on exit)."""
    for x, dt in ((ab, np.float64), (a, np.float64), (s, np.float64), (u, np.float64),
                  (vt, np.float64), (work, np.float64), (iwork, np.int32)):
        if x.dtype != dt:
            raise TypeError("array dtype must be %s" % dt)
    for x in (ab, u, vt):
        if x.ndim == 2 and not x.flags.f_contiguous:
            raise ValueError("ab, u and vt must be Fortran ordered")
    info = ctypes.c_int(0)
    ints = [ctypes.c_int(int(x)) for x in (n, sb, ldab, ldu, ldvt, smlsiz, lwork)]
    load().mdbdsvd_(ctypes.byref(ints[0]), ctypes.byref(ints[1]), _pd(ab), ctypes.byref(ints[2]),
                    _pd(a), _pd(s), _pd(u), ctypes.byref(ints[3]), _pd(vt), ctypes.byref(ints[4]),
                    ctypes.byref(ints[5]), _pd(work), ctypes.byref(ints[6]),
                    iwork.ctypes.data_as(_I), ctypes.byref(info))
    return info.value, ints[5].value


def svd_banded(ab, sb, smlsiz=25):
    """(s descending, U, VT) of the upper banded n x n matrix in upper band
    storage ab ((sb + 1) x n, row sb the diagonal) through MDBDSVD."""
    ab = np.asfortranarray(ab, dtype=np.float64)
    n = ab.shape[1]
    s = np.zeros(n)
    U = np.zeros((n, n), order="F")
    VT = np.zeros((n, n), order="F")
    one = np.zeros(1)
    info, _ = mdbdsvd(n, sb, ab, ab.shape[0], one, s, U, max(1, n), VT, max(1, n), smlsiz, one, 1,
                      np.zeros(1, dtype=np.int32))
    if info != 0:
        raise HssError("MDBDSVD INFO=%d: %s" % (info, _err()))
    return s, U, VT


def bsvd_tree(n, sb, smlsiz=25):
    """The banded SVD's leaves (host logic, no GPU): (merge levels, [(first row,
    rows, columns), ...]); raises HssError for arguments the library rejects."""
    st, rw, cl = (np.zeros(max(n, 1), dtype=np.int32) for _ in range(3))
    nl = ctypes.c_int(0)
    depth = load().hss_bsvd_tree(int(n), int(sb), int(smlsiz), st.ctypes.data_as(_I),
                                 rw.ctypes.data_as(_I), cl.ctypes.data_as(_I), ctypes.byref(nl))
    if depth < 0:
        raise HssError("hss_bsvd_tree rc=%d" % depth)
    return depth, [(int(a), int(b), int(c)) for a, b, c in zip(st[:nl.value], rw[:nl.value],
                                                              cl[:nl.value])]


def mdbdsvd_dev(sb, ab, s, u, vt, smlsiz=25, stream=None):
    """Device banded SVD: ab a tensor whose memory is the column-major
    (sb + 1) x n upper band storage; s (n,) singular values descending, u and vt
    (n, n) column-major storage."""
    n = s.numel()
    info = load().hss_mdbdsvd_dev(n, sb, _ptr(ab), sb + 1, _ptr(s), _ptr(u), max(1, n), _ptr(vt),
                                  max(1, n), int(smlsiz), _stream(stream))
    if info != 0:
        raise HssError("hss_mdbdsvd_dev INFO=%d: %s" % (info, _err()))
    return info


def cauchyhssmm(D, F, U, V, B, ni, tol, ncol=None):
    """CauchyHssMM (SRC/cauchyhssmm.f90:1): B <- C B in place (B Fortran-ordered
    n x n), C(i,j) = U_i V_j / (D_i - F_j) in HSS form.  Returns time(1:2)."""
    D, F, U, V = (np.ascontiguousarray(x, dtype=np.float64) for x in (D, F, U, V))
    n = len(D)
    if B.dtype != np.float64 or not B.flags.f_contiguous:
        raise ValueError("B must be a Fortran-ordered float64 array")
    t = np.zeros(2)
    ints = [ctypes.c_int(int(x)) for x in (n, ni, ncol or n, B.shape[0])]
    load().cauchyhssmm_(_pd(D), _pd(F), _pd(U), _pd(V), ctypes.byref(ints[0]),
                        ctypes.byref(ints[1]), ctypes.byref(ctypes.c_double(tol)),
                        ctypes.byref(ints[2]), _pd(B), ctypes.byref(ints[3]), _pd(t))
    return t


def cauchyhssmm_dev(D, F, u, v, B, ni, tol, stream=None):
    """B (tensor whose memory is column-major n x ncb) <- C B on the device;
    returns (construction ms, multiply ms)."""
    n = D.numel()
    ncb = B.numel() // max(n, 1)
    t = (ctypes.c_float * 2)()
    rc = load().hss_cauchyhssmm_dev(n, _ptr(D), _ptr(F), _ptr(u), _ptr(v), int(ni), float(tol),
                                    _ptr(B), max(1, n), ncb, ctypes.cast(t, ctypes.c_void_p),
                                    _stream(stream))
    if rc != 0:
        raise HssError("hss_cauchyhssmm_dev rc=%d: %s" % (rc, _err()))
    return t[0], t[1]


def svdhssupdat(F, Z, V, tol, ni):
    """SvdHssUpdat (SRC/SvdHssUpdat.f90:1) through the Fortran entry point.
    F (n, ascending) and Z = V^T a are copied; V (n x n, Fortran-ordered, rows =
    right singular vectors) is updated in place.  Returns (D, F, Z) as the
    routine leaves them (D[:K] the new singular values, ascending)."""
    F = np.array(F, dtype=np.float64)
    Z = np.array(Z, dtype=np.float64)
    n = len(F)
    if V.dtype != np.float64 or not V.flags.f_contiguous or V.shape != (n, n):
        raise ValueError("V must be a Fortran-ordered float64 n x n array")
    D = np.zeros(n)
    ints = [ctypes.c_int(int(x)) for x in (n, ni)]
    load().svdhssupdat_(_pd(D), _pd(F), _pd(Z), _pd(V), ctypes.byref(ints[0]),
                        ctypes.byref(ctypes.c_double(tol)), ctypes.byref(ints[1]))
    msg = _err()  # the entry point clears it on entry; non-empty means it failed
    if msg:
        raise HssError(msg)
    return D, F, Z


def svdhssupdat_dev(d, f, z, vt, tol, ni, stream=None):
    """SvdHssUpdat on device tensors (vt: memory column-major n x n, rows = right
    singular vectors); returns K."""
    n = f.numel()
    k = ctypes.c_int(0)
    rc = load().hss_svdhssupdat_dev(n, _ptr(d), _ptr(f), _ptr(z), _ptr(vt), max(1, n), float(tol),
                                    int(ni), ctypes.cast(ctypes.pointer(k), ctypes.c_void_p),
                                    _stream(stream))
    if rc != 0:
        raise HssError("hss_svdhssupdat_dev rc=%d: %s" % (rc, _err()))
    return k.value


def hsscholsolver(rs, wpcg, A, b, ni, tol, prank, pp=5, tau=1e-13, maxit=30):
    """HssCholSolver (SRC/HssCholSolver.f90:1) through the Fortran entry point:
    returns (x, INFO) for the SPD matrix A (n x n, any float64 layout; symmetric)."""
    A = np.asfortranarray(A, dtype=np.float64)
    x = np.array(b, dtype=np.float64)
    n = A.shape[0]
    info = ctypes.c_int(0)
    ints = [ctypes.c_int(int(v)) for v in (n, ni, prank, pp, maxit)]
    load().hsscholsolver_(rs.encode(), wpcg.encode(), _pd(A), ctypes.byref(ints[0]), _pd(x),
                          ctypes.byref(ints[1]), ctypes.byref(ctypes.c_double(tol)),
                          ctypes.byref(ints[2]), ctypes.byref(ints[3]),
                          ctypes.byref(ctypes.c_double(tau)), ctypes.byref(ints[4]),
                          ctypes.byref(info), 1, 1)
    return x, info.value


class HssChol:
    """An HSS Cholesky factor of a device matrix (hss_chol_factor_dev)."""

    def __init__(self, A, ni, tol, prank, ps=0, stream=None):
        """A: device tensor holding the n x n matrix column-major (any shape)."""
        n = math.isqrt(A.numel())
        if n * n != A.numel():
            raise ValueError("A must hold an n x n matrix")
        h = ctypes.c_void_p()
        rc = load().hss_chol_factor_dev(n, _ptr(A), n, int(ni), float(tol), int(prank), int(ps),
                                        ctypes.cast(ctypes.pointer(h), ctypes.c_void_p),
                                        _stream(stream))
        if rc != 0:
            raise HssError("hss_chol_factor_dev rc=%d: %s" % (rc, _err()))
        self.h, self.n = h, n

    def info(self):
        v = [ctypes.c_int(0) for _ in range(4)]
        b = ctypes.c_longlong(0)
        load().hss_chol_info(self.h, *[ctypes.cast(ctypes.pointer(x), ctypes.c_void_p) for x in v],
                             ctypes.cast(ctypes.pointer(b), ctypes.c_void_p))
        return {"n": v[0].value, "max_rank": v[1].value, "levels": v[2].value,
                "root": v[3].value, "bytes": b.value}

    def solve(self, B, stream=None):
        """B: device tensor whose memory is column-major n x nrhs (solved in place)."""
        nrhs = B.numel() // self.n
        rc = load().hss_chol_solve_dev(self.h, _ptr(B), self.n, nrhs, _stream(stream))
        if rc != 0:
            raise HssError("hss_chol_solve_dev rc=%d: %s" % (rc, _err()))

    def pcg(self, A, b, x, tau, maxit, precondition=True, stream=None):
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        rc = load().hss_chol_pcg_dev(self.h if precondition else None, self.n, _ptr(A), self.n,
                                     _ptr(b), _ptr(x), float(tau), int(maxit),
                                     ctypes.cast(ctypes.pointer(it), ctypes.c_void_p),
                                     ctypes.cast(ctypes.pointer(rr), ctypes.c_void_p),
                                     _stream(stream))
        if rc != 0:
            raise HssError("hss_chol_pcg_dev rc=%d: %s" % (rc, _err()))
        return it.value, rr.value

    def free(self):
        if self.h:
            load().hss_chol_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def svdupd_deflate(f, z):
    """MDLASD20's deflation on the host (no GPU): returns (K, f, z, idxp, nrot)."""
    f = np.array(f, dtype=np.float64)
    z = np.array(z, dtype=np.float64)
    n = len(f)
    idxp = np.zeros(n, dtype=np.int32)
    nrot = ctypes.c_int(0)
    K = load().hss_svdupd_deflate(n, _pd(f), _pd(z),
                                  idxp.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                  ctypes.byref(nrot))
    return K, f, z, idxp, nrot.value


def _dhssmm_call(fn, A, B, ni, tol, prank, ncol, m=None):
    if A.dtype != np.float64 or not A.flags.f_contiguous:
        raise ValueError("A must be a Fortran-ordered float64 array")
    if B.dtype != np.float64 or not B.flags.f_contiguous:
        raise ValueError("B must be a Fortran-ordered float64 array")
    n = A.shape[1]
    k = B.shape[1] if fn == "dhssmm_" else B.shape[0]
    if fn == "dhssmml_" and B.shape[1] < n:
        raise ValueError("DHSSMML: B must have N columns")
    t = np.zeros(2)
    info = ctypes.c_int(0)
    ints = [ctypes.c_int(int(x)) for x in (A.shape[0], n if m is None else m, n, B.shape[0], k,
                                           prank, ni, ncol)]
    getattr(load(), fn)(_pd(A), ctypes.byref(ints[0]), ctypes.byref(ints[1]),
                        ctypes.byref(ints[2]), _pd(B), ctypes.byref(ints[3]),
                        ctypes.byref(ints[4]), ctypes.byref(ctypes.c_double(tol)),
                        ctypes.byref(ints[5]), ctypes.byref(ints[6]), ctypes.byref(ints[7]),
                        _pd(t), ctypes.byref(info))
    return info.value, t


def dhssmm(A, B, ni, tol, prank=0, ncol=100, m=None):
    """DHSSMM (SRC/DHSSMM.f90:1): B(n x k) <- A_hss B in place (A, B
    Fortran-ordered float64; A is not modified).  Returns (INFO, time(1:2))."""
    return _dhssmm_call("dhssmm_", A, B, ni, tol, prank, ncol, m)


def dhssmml(A, B, ni, tol, prank=0, ncol=100, m=None):
    """DHSSMML (SRC/DHSSMML.f90:2): B(k x n) <- B A_hss in place.  Returns
    (INFO, time(1:2))."""
    return _dhssmm_call("dhssmml_", A, B, ni, tol, prank, ncol, m)


def dhssmm_dev(A, B, ni, tol, side=0, stream=None):
    """Device DHSSMM (side 0: B (n x k) <- A_hss B) or DHSSMML (side 1: B (k x n)
    <- B A_hss).  A: tensor whose memory is column-major n x n; B: column-major
    with leading dimension n (side 0) or k (side 1).  Returns (construction ms,
    multiply ms)."""
    n = int(round(A.numel() ** 0.5))
    k = B.numel() // max(n, 1)
    t = (ctypes.c_float * 2)()
    rc = load().hss_dhssmm_dev(n, _ptr(A), max(1, n), _ptr(B), max(1, n if side == 0 else k), k,
                               float(tol), int(ni), int(side), ctypes.cast(t, ctypes.c_void_p),
                               _stream(stream))
    if rc != 0:
        raise HssError("hss_dhssmm_dev rc=%d: %s" % (rc, _err()))
    return t[0], t[1]


def cauchylike(D, F, u, v):
    """A(i,j) = u_i v_j / (D_i - F_j) computed on the GPU (Cauchylike.f90:1)."""
    D, F, u, v = (np.ascontiguousarray(x, dtype=np.float64) for x in (D, F, u, v))
    m, n = len(D), len(F)
    A = np.zeros((m, n), dtype=np.float64, order="F")
    load().cauchylike_(_pd(A), _pd(D), _pd(F), _pd(u), _pd(v), ctypes.byref(ctypes.c_int(m)),
                       ctypes.byref(ctypes.c_int(n)))
    return A


# ------------------------------------------------------------ device API ----
def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda:
        raise HssError("device entry points take CUDA tensors")
    if not t.is_contiguous():
        raise HssError("tensor must be contiguous")
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def mdstedc_dev(d, e, z, stream=None):
    """Device MDSTEDC('I'): d (n,) -> eigenvalues, z (n, n) column-major
    storage, i.e. a tensor whose memory is Fortran order (use z.T for rows)."""
    n = d.numel()
    info = load().hss_mdstedc_dev(n, _ptr(d), _ptr(e), _ptr(z), max(1, n), _stream(stream))
    if info != 0:
        raise HssError("hss_mdstedc_dev INFO=%d: %s" % (info, _err()))
    return info


def mdstedc_v_dev(d, e, z, stream=None):
    """Device MDSTEDC('V'): z (n x n column-major storage) holds Q0 on entry and
    Q0 times the tridiagonal's eigenvectors on exit; d -> eigenvalues."""
    n = d.numel()
    info = load().hss_mdstedc_v_dev(n, _ptr(d), _ptr(e), _ptr(z), max(1, n), _stream(stream))
    if info != 0:
        raise HssError("hss_mdstedc_v_dev INFO=%d: %s" % (info, _err()))
    return info


def batch_offsets(sizes):
    """Offsets of each problem in the packed d/e (sum n) and z (sum n^2) arrays."""
    sizes = np.asarray(sizes, dtype=np.int64)
    o = np.concatenate([[0], np.cumsum(sizes)])
    oz = np.concatenate([[0], np.cumsum(sizes * sizes)])
    return o, oz


def mdstedc_batch_dev(sizes, d, e, z, stream=None):
    """Batched device MDSTEDC('I') over packed problems (see
    :func:`batch_offsets`): d (sum n) -> eigenvalues, e (sum n; problem p's
    off-diagonals at its offset), z (sum n^2; problem p column-major n_p x n_p)."""
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    info = load().hss_mdstedc_batch_dev(len(sizes), sizes.ctypes.data_as(ctypes.c_void_p), _ptr(d),
                                        _ptr(e), _ptr(z), _stream(stream))
    if info != 0:
        raise HssError("hss_mdstedc_batch_dev INFO=%d: %s" % (info, _err()))
    return info


def pack_batch(problems):
    """Packed host arrays (sizes, d, e) of a list of (d, e) numpy pairs."""
    sizes = np.array([len(d) for d, _ in problems], dtype=np.int32)
    o, _ = batch_offsets(sizes)
    D = np.zeros(int(o[-1]))
    E = np.zeros(int(o[-1]))
    for p, (d, e) in enumerate(problems):
        D[o[p]:o[p + 1]] = d
        E[o[p]:o[p] + len(e)] = e
    return sizes, D, E


def eigh_tridiagonal_batch(problems, stream=None):
    """[(w, Q)] for a list of (d, e) problems, solved in one batched call."""
    import torch
    sizes, D, E = pack_batch(problems)
    o, oz = batch_offsets(sizes)
    d = torch.tensor(D, device="cuda")
    e = torch.tensor(E, device="cuda")
    z = torch.empty(int(oz[-1]), dtype=torch.float64, device="cuda")
    mdstedc_batch_dev(sizes, d, e, z, stream)
    w, zh = d.cpu().numpy(), z.cpu().numpy()
    return [(w[o[p]:o[p + 1]].copy(),
             zh[oz[p]:oz[p + 1]].reshape(int(sizes[p]), int(sizes[p])).T.copy())
            for p in range(len(sizes))]


def secular_dev(dlamda, z, rho, lam, difl, difr, iters=None, stream=None):
    k = dlamda.numel()
    rc = load().hss_secular_dev(k, _ptr(dlamda), _ptr(z), float(rho), _ptr(lam), _ptr(difl),
                                _ptr(difr), _ptr(iters), _stream(stream))
    if rc != 0:
        raise HssError("hss_secular_dev rc=%d: %s" % (rc, _err()))
    return rc


def lowner_dev(dlamda, difl, difr, z, alpha, stream=None):
    k = dlamda.numel()
    rc = load().hss_lowner_dev(k, _ptr(dlamda), _ptr(difl), _ptr(difr), _ptr(z), _ptr(alpha),
                               _stream(stream))
    if rc != 0:
        raise HssError("hss_lowner_dev rc=%d: %s" % (rc, _err()))
    return rc


def cauchy_eig_dev(F, u, v, difl, difr, C, stream=None):
    k = F.numel()
    rc = load().hss_cauchy_eig_dev(k, _ptr(F), _ptr(u), _ptr(v), _ptr(difl), _ptr(difr), _ptr(C),
                                   _stream(stream))
    if rc != 0:
        raise HssError("hss_cauchy_eig_dev rc=%d: %s" % (rc, _err()))
    return rc


def gemm_dev(A, B, C, m, n, k, lda, ldb, ldc, beta=0, precision=0, stream=None):
    """C = A @ B (+ C) on column-major device buffers (FP64 or split-BF16)."""
    rc = load().hss_gemm_dev(int(m), int(n), int(k), _ptr(A), int(lda), _ptr(B), int(ldb), _ptr(C),
                             int(ldc), int(beta), int(precision), _stream(stream))
    if rc != 0:
        raise HssError("hss_gemm_dev rc=%d: %s" % (rc, _err()))
    return rc


def fp64_fma_rate(blocks=152 * 8, iters=8192, stream=None):
    """The GPU's FP64 FMA rate in TFLOP/s, measured by one timed launch
    (:c:func:`hss_fp64_fma_rate`); returns (tflops, ms)."""
    ms = ctypes.c_float(0.0)
    tf = ctypes.c_double(0.0)
    rc = load().hss_fp64_fma_rate(int(blocks), int(iters), ctypes.byref(ms), ctypes.byref(tf),
                                  _stream(stream))
    if rc != 0:
        raise HssError("hss_fp64_fma_rate rc=%d" % rc)
    return tf.value, ms.value


def dhssevc_dev(F, u, v, difl, difr, Q, ldq, nrows, ni=200, tol=1e-17, stream=None):
    """Q(0:nrows, 0:K) <- Q @ C in place (Q column-major, leading dim ldq)."""
    k = F.numel()
    rc = load().hss_dhssevc_dev(k, int(ni), float(tol), _ptr(F), _ptr(u), _ptr(v), _ptr(difl),
                                _ptr(difr), _ptr(Q), int(ldq), int(nrows), _stream(stream))
    if rc != 0:
        raise HssError("hss_dhssevc_dev rc=%d: %s" % (rc, _err()))
    return rc
