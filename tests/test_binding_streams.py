"""Host logic of the Python binding's stream ordering, on CPU with fakes.

Calls that can touch device buffers are ordered between torch's current
stream and the context's stream: before the call the context's stream waits
for torch's, after it (also when the call raises) torch's waits for the
context's.  Nothing happens while torch has not initialised CUDA, and an
explicitly bound stream turns the ordering off.  The GPU-side behaviour is
tested in test_gpu_host_pipeline.test_device_calls_follow_torch_current_stream.
"""
import ctypes
import sys
import types

import pytest


class _Stream:
    def __init__(self, name, log):
        self.name, self.log = name, log

    def wait_stream(self, other):
        self.log.append(f"{self.name} waits {other.name}")


def _fake_torch(log, initialised=True):
    cuda = types.SimpleNamespace(
        is_initialized=lambda: initialised,
        ExternalStream=lambda ptr, device=None: _Stream(f"lib@{ptr:#x}", log),
        current_stream=lambda device=None: _Stream("torch", log))
    return types.SimpleNamespace(cuda=cuda, device=lambda *a: a)


class _FakeLib:
    def __init__(self, ptr):
        self.ptr = ptr

    def pdg_get_stream(self, h, out):
        out._obj.value = self.ptr
        return 0


@pytest.fixture
def env(monkeypatch):
    import pdg
    log = []
    lib = _FakeLib(0x1000)
    monkeypatch.setattr(pdg, "load", lambda *a: lib)
    monkeypatch.setitem(sys.modules, "torch", _fake_torch(log))
    go = types.SimpleNamespace(_h=ctypes.c_void_p(1), _explicit_stream=False, _lib_stream=None,
                               cfg=types.SimpleNamespace(device=0))

    class Op:                      # a binding class that holds the context as .go
        def __init__(self):
            self.go = go

        @pdg._stream_ordered
        def apply(self, fail=False):
            log.append("call")
            if fail:
                raise RuntimeError("boom")
            return 7

    return pdg, log, lib, go, Op()


def test_call_is_ordered_both_ways(env):
    pdg, log, lib, go, op = env
    assert op.apply() == 7
    assert log == ["lib@0x1000 waits torch", "call", "torch waits lib@0x1000"]


def test_torch_waits_even_when_the_call_raises(env):
    pdg, log, lib, go, op = env
    with pytest.raises(RuntimeError):
        op.apply(fail=True)
    assert log[-1] == "torch waits lib@0x1000"


def test_follows_a_new_context_stream(env):
    pdg, log, lib, go, op = env
    op.apply()
    lib.ptr = 0x2000               # the context was bound to another stream
    log.clear()
    op.apply()
    assert log[0] == "lib@0x2000 waits torch"


def test_explicit_stream_and_uninitialised_cuda_skip_the_ordering(env, monkeypatch):
    pdg, log, lib, go, op = env
    go._explicit_stream = True
    op.apply()
    assert log == ["call"]
    go._explicit_stream = False
    log.clear()
    monkeypatch.setitem(sys.modules, "torch", _fake_torch(log, initialised=False))
    op.apply()
    assert log == ["call"]


def test_closed_context_skips_the_ordering(env):
    pdg, log, lib, go, op = env
    go._h = None
    op.apply()
    assert log == ["call"]
