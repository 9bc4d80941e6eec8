"""hss_lowner_noalloc_dev (Loewner stage with static device scratch, no
allocation) against hss_lowner_dev on the same inputs, through the C ABI.

Collected last on purpose: it must pass both in a fresh process (where its
first call does the per-device set-up) and after every other test has used
the library's buffer pool."""
import ctypes

import numpy as np
import pytest
import torch

import hsspack_gb300 as hp
from helpers import secular_problem

pytestmark = pytest.mark.gpu

MAX_K = 65536


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _inputs(k, seed):
    d, z, rho = secular_problem(k, seed)
    dd, zz = _dev(d), _dev(z)
    lam, difl, difr = (torch.zeros(k, dtype=torch.float64, device="cuda") for _ in range(3))
    hp.secular_dev(dd, zz, rho, lam, difl, difr)
    return dd, zz, difl, difr


def _run(fn, dd, zz, difl, difr):
    k = dd.numel()
    z = zz.clone()
    alpha = torch.zeros(k, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = fn(k, hp._ptr(dd), hp._ptr(difl), hp._ptr(difr), hp._ptr(z), hp._ptr(alpha),
            hp._stream(None))
    return rc, z.cpu().numpy(), alpha.cpu().numpy()


def _compare(k, seed):
    L = hp.load()
    args = _inputs(k, seed)
    rc0, z0, a0 = _run(L.hss_lowner_dev, *args)
    rc1, z1, a1 = _run(L.hss_lowner_noalloc_dev, *args)
    assert rc0 == 0 and rc1 == 0, (rc0, rc1, hp.load().hss_last_error())
    # same kernels on the same inputs: agreement to the Loewner tests' 1e-12 bound
    # (in practice bitwise)
    assert np.all(np.isfinite(z1)) and np.all(np.isfinite(a1))
    assert np.max(np.abs(z1 - z0) / np.abs(z0)) <= 1e-12
    assert np.max(np.abs(a1 - a0) / np.abs(a0)) <= 1e-12


def test_noalloc_matches_pool_version_two_calls():
    # the second call is smaller, so the scratch still holds the first call's
    # values past k; they must not leak into the result
    _compare(4000, 41)
    _compare(700, 42)


def test_noalloc_leaves_free_device_memory_unchanged():
    # after a first (set-up) call, a call must not change the device's free
    # memory: everything it needs is in the static scratch and the caller's
    # buffers, all allocated before the measurement
    L = hp.load()
    dd, zz, difl, difr = _inputs(3000, 44)
    k = dd.numel()
    z = zz.clone()
    alpha = torch.zeros(k, dtype=torch.float64, device="cuda")
    args = (k, hp._ptr(dd), hp._ptr(difl), hp._ptr(difr), hp._ptr(z), hp._ptr(alpha),
            hp._stream(None))
    z.copy_(zz)
    assert L.hss_lowner_noalloc_dev(*args) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        z.copy_(zz)
        assert L.hss_lowner_noalloc_dev(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_limit():
    _compare(MAX_K, 43)
    L = hp.load()
    dummy = ctypes.c_void_p(0)
    rc = L.hss_lowner_noalloc_dev(MAX_K + 1, dummy, dummy, dummy, dummy, dummy, dummy)
    assert rc == -1
    assert b"65536" in L.hss_last_error()
