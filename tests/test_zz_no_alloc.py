"""The allocation-free residual entry point against the context one.

lbm_gpu_residual_noalloc serves callers that cannot call cudaMalloc (their
device memory comes from another allocator, or they cannot afford its
implicit synchronisation).  Here the caller's device memory comes from
PyTorch's caching allocator; the library itself allocates nothing.  Its result
must match lbm_gpu_residual (which uses the context's own scratch) on two
calls in a row over different states.  This file is collected last so that a
run that stops at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_case
from lbm_gb300._lib import load
from lbm_gb300.solver import TableSolver

pytestmark = pytest.mark.gpu


def _soa(aos: np.ndarray, n: int, nvar: int) -> np.ndarray:
    return np.ascontiguousarray(aos.reshape(n, nvar).T)


def test_noalloc_residual_matches_context_residual_twice():
    torch = pytest.importorskip("torch")
    meta, solver, grid, out, consts, bnds, forcing = load_case("poiseuille_50")
    g = TableSolver(consts, grid, bnds, forcing)
    g.initial_condition()
    lib = load()
    stream = torch.cuda.current_stream()
    for steps in (17, 40):
        g.step(steps)
        expect = g.residual()  # the existing entry point
        n, nvar = grid.ncells, g.nvar
        v = torch.from_numpy(_soa(g.vars(), n, nvar)).cuda()
        vo = torch.from_numpy(_soa(g.varsold(), n, nvar)).cuda()
        res = torch.full((nvar,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.lbm_gpu_residual_noalloc(C.c_void_p(v.data_ptr()), C.c_void_p(vo.data_ptr()), n, nvar,
                                          C.c_void_p(res.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        got = res.cpu().numpy()
        assert np.allclose(got, expect, rtol=1e-12, atol=0), (got, expect)


def test_noalloc_rejects_too_many_variables():
    torch = pytest.importorskip("torch")
    lib = load()
    a = torch.zeros(9 * 16, dtype=torch.float64, device="cuda")
    res = torch.zeros(9, dtype=torch.float64, device="cuda")
    rc = lib.lbm_gpu_residual_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), 16, 9, C.c_void_p(res.data_ptr()), None)
    assert rc == -1


def test_noalloc_residual_full_scratch_three_calls():
    """Enough cells that the first pass runs the full 304 blocks, with the
    full 8 variables: every slot of the fixed scratch array is written.  The
    calls alternate between that size and a smaller one (fewer blocks), each
    on fresh data, so a partial left over from an earlier call would show."""
    torch = pytest.importorskip("torch")
    lib = load()
    stream = torch.cuda.current_stream()
    gen = torch.Generator(device="cuda").manual_seed(7)
    for n, scale in ((700_001, 1.0), (100_003, 3.0), (700_001, 0.25)):
        nvar = 8
        a = torch.randn((nvar, n), dtype=torch.float64, device="cuda", generator=gen) * scale
        b = torch.randn((nvar, n), dtype=torch.float64, device="cuda", generator=gen)
        res = torch.full((nvar,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.lbm_gpu_residual_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), n, nvar,
                                          C.c_void_p(res.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        expect = (a - b).abs().sum(dim=1).cpu().numpy()
        got = res.cpu().numpy()
        assert np.allclose(got, expect, rtol=1e-12, atol=0), (n, got, expect)
