"""Host-buffer applies: the library copies host vectors in and out slab by
slab, overlapping the copies with the operator kernel.  The result must be
bit-identical to the same apply on device vectors (every cell is computed by
the same arithmetic in either path), for ragged slab splits, 2D and 3D,
accumulate / overwrite / scaled / residual / transposed forms and with
upwind convection."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import __graft_entry__
    __graft_entry__.build()
    import pdg
    import torch
    return pdg, torch


def _go(pdg, dim, k, cells, seed, conv=False):
    rng = np.random.default_rng(seed)
    go = pdg.GridOperator(dim, k, cells, alpha=3.0)
    go.set_permeability(rng.standard_normal(go.ncell), is_log=True)
    if conv:
        go.set_reaction(np.ones(go.ncell))
        go.set_velocity_modes(pdg.fourier_velocity_modes(seed))
    go.set_source(fc=rng.standard_normal(go.ncell))
    return go, rng


# (dim, degree, cells): 2, 4, 4 (ragged: 10,10,10,7 planes) and 3 (67,67,66)
# slabs of at least 16384 cells
CASES = [(3, 1, (32, 32, 32)), (3, 2, (64, 64, 16)), (3, 1, (48, 40, 37)),
         (2, 2, (256, 200))]


@pytest.mark.parametrize("dim,k,cells", CASES)
def test_host_apply_bitwise_equals_device(env, dim, k, cells):
    pdg, torch = env
    go, rng = _go(pdg, dim, k, cells, seed=k + len(cells))
    dev = torch.device("cuda", 0)
    x = rng.uniform(-1, 1, go.ndof)
    y0 = rng.uniform(-1, 1, go.ndof)
    xd = torch.tensor(x, device=dev)
    torch.cuda.synchronize()
    op = pdg.OnTheFlyOperator(go)
    forms = {
        "jacobian_apply": lambda a, b: go.jacobian_apply(a, b),
        "apply": lambda a, b: op.apply(a, b),
        "applyscaleadd": lambda a, b: op.applyscaleadd(-0.75, a, b),
        "residual": lambda a, b: go.residual(a, b),
        "transpose": lambda a, b: go.jacobian_apply_transpose(a, b),
    }
    for name, f in forms.items():
        yh = y0.copy()
        f(x, yh)                                   # host x, host y (pipelined)
        yd = torch.tensor(y0, device=dev)
        torch.cuda.synchronize()
        f(xd, yd)                                  # device x, device y
        torch.cuda.synchronize()
        assert np.array_equal(yh, yd.cpu().numpy()), name
        ym = torch.tensor(y0, device=dev)
        torch.cuda.synchronize()
        f(x, ym)                                   # host x, device y
        torch.cuda.synchronize()
        assert np.array_equal(ym.cpu().numpy(), yh), name + " (host x, device y)"
        yo = y0.copy()
        f(xd, yo)                                  # device x, host y
        assert np.array_equal(yo, yh), name + " (device x, host y)"
    go.close()


def test_host_apply_pinned_and_convection(env):
    pdg, torch = env
    go, rng = _go(pdg, 3, 2, (40, 40, 24), seed=9, conv=True)
    dev = torch.device("cuda", 0)
    x = torch.tensor(rng.uniform(-1, 1, go.ndof)).pin_memory()
    y = torch.zeros(go.ndof, dtype=torch.float64).pin_memory()
    op = pdg.OnTheFlyOperator(go)
    for _ in range(3):                              # repeated calls reuse the streams
        op.apply(x, y)
    yd = torch.zeros(go.ndof, dtype=torch.float64, device=dev)
    xd = x.to(dev)
    torch.cuda.synchronize()
    op.apply(xd, yd)
    torch.cuda.synchronize()
    assert torch.equal(y, yd.cpu())
    go.close()


def test_device_calls_follow_torch_current_stream(env):
    """Device tensors produced on torch's current stream behind a long kernel
    (a bounded GPU sleep of ~20 ms) are read only once they are written, and
    torch reads the results only after the call's work: the binding orders the
    context's stream against torch's current stream with events, without an
    explicit synchronisation in the caller."""
    pdg, torch = env
    go, rng = _go(pdg, 3, 2, (24, 24, 24), seed=4)
    dev = torch.device("cuda", 0)
    base = torch.tensor(rng.uniform(-1, 1, go.ndof), device=dev)
    ref = torch.zeros_like(base)
    torch.cuda.synchronize()
    go.jacobian_apply(base, ref)
    torch.cuda.synchronize()
    for stream in (None, torch.cuda.Stream(dev)):
        ctx = torch.cuda.stream(stream) if stream is not None else torch.cuda.stream(
            torch.cuda.current_stream(dev))
        with ctx:
            torch.cuda._sleep(40_000_000)
            x = base * 1.0                      # written after the sleep
            y = torch.zeros_like(base)
            go.jacobian_apply(x, y)
            out = y.clone()                     # read on torch's stream
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
    # an explicitly bound stream is the caller's to order
    s = torch.cuda.Stream(dev)
    go.set_stream(s)
    with torch.cuda.stream(s):
        y = torch.zeros_like(base)
        go.jacobian_apply(base, y)
    s.synchronize()
    assert torch.equal(y, ref)
    go.set_stream(None)
    go.close()
