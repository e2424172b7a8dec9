"""Objects made on a context (batches, networks) are closed before the
context is destroyed, whatever order the interpreter finalises them in
(host logic only: a recording stand-in replaces the native library)."""
import gc

import axonexa_gb300._native as N
from axonexa_gb300.acquisition import Device


class _Recorder:
    def __init__(self):
        self.calls = []

    def axx_destroy(self, h):
        self.calls.append(("ctx", h))

    def axx_batch_destroy(self, h):
        self.calls.append(("batch", h))


class _Child:
    """A handle holder as Batch and MLP are: close() frees its handle once."""

    def __init__(self, rec, dev, h):
        self.rec, self.dev, self.h = rec, dev, h
        dev.adopt(self)

    def close(self):
        if self.h is not None:
            self.rec.axx_batch_destroy(self.h)
            self.h = None


def _device(rec, h):
    d = Device.__new__(Device)  # no native context: the handle is a token
    d.h, d.device = h, 0
    import weakref
    d._children = weakref.WeakSet()
    return d


def test_context_closes_its_objects_first(monkeypatch):
    rec = _Recorder()
    monkeypatch.setattr(N, "lib", lambda: rec)
    d = _device(rec, "ctx0")
    a, b = _Child(rec, d, "b1"), _Child(rec, d, "b2")
    d.close()
    assert rec.calls[-1] == ("ctx", "ctx0")
    assert sorted(rec.calls[:-1]) == [("batch", "b1"), ("batch", "b2")]
    # closing the objects later does nothing more, and neither does the context
    a.close()
    b.close()
    d.close()
    assert len(rec.calls) == 3


def test_objects_in_a_reference_cycle_with_their_context(monkeypatch):
    rec = _Recorder()
    monkeypatch.setattr(N, "lib", lambda: rec)
    d = _device(rec, "ctx1")
    c = _Child(rec, d, "b3")
    c.cycle = c  # unreachable only through the cycle collector
    d.close()
    del c
    gc.collect()
    assert rec.calls == [("batch", "b3"), ("ctx", "ctx1")]
