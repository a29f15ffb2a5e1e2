"""pdg_dot_noalloc: the dot product for callers that cannot allocate.

Callers that record work by CUDA stream capture, or host solvers that own
every device buffer, cannot let the library call cudaMalloc when they ask
for a dot product.  pdg_dot_noalloc keeps its reduction scratch in a
file-scope device array instead.  This test calls it through the C ABI and
checks it against the context-based pdg_dot (same vectors, FP64 tolerance
1e-12 relative to sum |a_i b_i|) on two calls in a row, so a second call
that saw stale scratch from the first would fail.  It also checks that a
length beyond the scratch limit is refused before anything runs.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pdg():
    import __graft_entry__
    __graft_entry__.build()
    import pdg as m
    return m


def _check_pair(pdg, torch, go, n, seed):
    lib = pdg.load()
    gen = torch.Generator(device="cuda").manual_seed(seed)
    result = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    for call in range(2):
        a = torch.rand(n, dtype=torch.float64, device="cuda", generator=gen) - 0.5
        b = torch.rand(n, dtype=torch.float64, device="cuda", generator=gen) - 0.5
        st = lib.pdg_dot_noalloc(n, a.data_ptr(), b.data_ptr(), result.data_ptr(), None)
        assert st == pdg.PDG_OK, lib.pdg_last_error()
        torch.cuda.synchronize()
        ref = go.dot(a[:go.ndof], b[:go.ndof]) if n == go.ndof else float((a * b).sum())
        scale = float((a * b).abs().sum())
        assert abs(result.item() - ref) <= 1e-12 * scale, (call, result.item(), ref)


def test_dot_noalloc_matches_dot(pdg):
    import torch
    # 24^3 cells of Q2: 373,248 DoF = 6 reduction chunks, the last one partial
    go = pdg.GridOperator(3, 2, (24, 24, 24))
    _check_pair(pdg, torch, go, go.ndof, seed=0)
    go.close()
    # a single partial chunk
    go = pdg.GridOperator(2, 1, (10, 25))
    _check_pair(pdg, torch, go, go.ndof, seed=1)
    go.close()


def test_dot_noalloc_rejects_oversize(pdg):
    import torch
    lib = pdg.load()
    a = torch.zeros(4, dtype=torch.float64, device="cuda")
    r = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = lib.pdg_dot_noalloc(ctypes.c_long(67108864 + 1), a.data_ptr(), a.data_ptr(),
                             r.data_ptr(), None)
    assert st == pdg.PDG_EINVAL
    assert b"PDG_DOT_NOALLOC_MAX_N" in lib.pdg_last_error()


def test_dot_noalloc_empty_and_host_pointers(pdg):
    import numpy as np
    import torch
    lib = pdg.load()
    a = torch.ones(4, dtype=torch.float64, device="cuda")
    r = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    # n = 0: the sum over nothing is zero, written over the NaN
    st = lib.pdg_dot_noalloc(ctypes.c_long(0), a.data_ptr(), a.data_ptr(), r.data_ptr(), None)
    assert st == pdg.PDG_OK, lib.pdg_last_error()
    torch.cuda.synchronize()
    assert r.item() == 0.0
    # host memory is refused before anything runs
    h = np.ones(4)
    st = lib.pdg_dot_noalloc(ctypes.c_long(4), h.ctypes.data, a.data_ptr(), r.data_ptr(), None)
    assert st == pdg.PDG_EINVAL
    assert b"device pointers" in lib.pdg_last_error()
