"""ads_residual_noalloc (the entry point that allocates no device memory)
against ads_apply_mass, through the C-ABI.

Collected last on purpose: the entry point keeps its scratch in a fixed
device array shared by all calls, so it must give the same answers in a fresh
process and after every other test has run on the same device.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _abi():
    import ads_mpi_gb300 as A
    lib = A.ads.load()
    f = lib.ads_residual_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    return A, lib, f


def _call(lib, f, g, dF, du, dr):
    norms = (ctypes.c_double * 3)()
    st = f(g.h, dF.data_ptr() if dF is not None else None, du.data_ptr(), dr.data_ptr(), norms)
    assert st == 0, lib.ads_last_error(g.h)
    return np.array(norms[:])


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("E,p", [((30, 20, 24), 2), ((17, 24, 9), 3)])
def test_noalloc_residual_matches_apply_mass_twice(E, p):
    torch = pytest.importorskip("torch")
    A, lib, f = _abi()
    n = tuple(e + p - 1 for e in (E if isinstance(E, tuple) else (E,) * 3))
    g = A.ADS(n, (p, p, p))
    rng = np.random.default_rng(41)
    for call in range(2):  # two calls in a row: the second sees the first's scratch contents
        u = rng.standard_normal(g.N)
        F = rng.standard_normal(g.N)
        Mu = g.apply_mass(u)
        du = torch.from_numpy(u).cuda()
        dF = torch.from_numpy(F).cuda()
        dr = torch.empty_like(du)
        norms = _call(lib, f, g, dF, du, dr)
        torch.cuda.synchronize()
        r = dr.cpu().numpy()
        expect = F - Mu
        assert _rel(r, expect) < FP64_TOL, call
        assert abs(norms[0] - np.dot(expect, expect)) < FP64_TOL * np.dot(expect, expect)
        assert abs(norms[1] - np.dot(F, F)) < FP64_TOL * np.dot(F, F)
        assert norms[2] == np.abs(r).max()
        # without F: the plain mass product
        dm = torch.empty_like(du)
        norms = _call(lib, f, g, None, du, dm)
        torch.cuda.synchronize()
        assert _rel(dm.cpu().numpy(), Mu) < FP64_TOL, call
        assert norms[1] == 0.0
        assert abs(norms[0] - np.dot(Mu, Mu)) < FP64_TOL * np.dot(Mu, Mu)
    g.cleanup()


def test_noalloc_calls_allocate_no_device_memory():
    """After a first call (which looks up the scratch address), further calls
    leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    A, lib, f = _abi()
    g = A.ADS((25, 22, 19), (2, 2, 2))
    rng = np.random.default_rng(43)
    du = torch.from_numpy(rng.standard_normal(g.N)).cuda()
    dF = torch.from_numpy(rng.standard_normal(g.N)).cuda()
    dr = torch.empty_like(du)
    _call(lib, f, g, dF, du, dr)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        _call(lib, f, g, dF, du, dr)
        _call(lib, f, g, None, du, dr)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    g.cleanup()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    """448 x 448 x 352 DOFs need 14 x 56 x 11 = 8624 residual tiles of
    32 x 8 x 32 DOFs, more than the fixed scratch's 8192 CTAs: the call
    returns ADS_ERR_ARG before any launch."""
    torch = pytest.importorskip("torch")
    A, lib, f = _abi()
    g = A.ADS((447, 447, 351), (2, 2, 2))
    du = torch.zeros(8, dtype=torch.float64, device="cuda")  # never read: the call is refused first
    norms = (ctypes.c_double * 3)()
    st = f(g.h, None, du.data_ptr(), du.data_ptr(), norms)
    assert st == 1  # ADS_ERR_ARG
    assert b"scratch" in lib.ads_last_error(g.h)
    g.cleanup()
