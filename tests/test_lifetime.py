"""The Python wrapper frees a context's pipelines, servers and batches before
the context, whatever order they are closed or finalised in. Checked on the
CPU against a fake library that records the free calls."""
import ctypes as C
import gc

import libcraw_gb300 as L


class FakeLib:
    def __init__(self):
        self.log = []
        self.next = 0x1000

    def _new(self, ref, kind):
        self.next += 16
        ref._obj.value = self.next
        self.log.append(("create", kind, self.next))
        return 0

    def _free(self, ref, kind):
        box = ref._obj
        if box.value:
            self.log.append(("free", kind, box.value))
            box.value = None

    def craw_context_create(self, ref, params, opts):
        return self._new(ref, "context")

    def craw_pipeline_create(self, ctx, params, ref):
        return self._new(ref, "pipeline")

    def craw_server_create(self, ctx, params, ref):
        return self._new(ref, "server")

    def craw_batch_create(self, ctx, params, ref):
        return self._new(ref, "batch")

    def craw_context_free(self, ref):
        self._free(ref, "context")

    def craw_pipeline_free(self, ref):
        self._free(ref, "pipeline")

    def craw_server_free(self, ref):
        self._free(ref, "server")

    def craw_batch_free(self, ref):
        self._free(ref, "batch")


def _frees(fake):
    return [(k, h) for op, k, h in fake.log if op == "free"]


def _check_order(fake):
    frees = _frees(fake)
    handles = [h for _, h in frees]
    assert len(handles) == len(set(handles)), "a handle freed twice"
    created = {h for op, _, h in fake.log if op == "create"}
    assert set(handles) == created, "a handle never freed"
    ctx_at = [i for i, (k, _) in enumerate(frees) if k == "context"]
    assert ctx_at and ctx_at[-1] == len(frees) - 1, "the context freed before a child"


def test_close_orders(monkeypatch):
    fake = FakeLib()
    monkeypatch.setattr(L, "_lib", fake)
    # Context first: it frees the children, whose own close is then a no-op.
    c = L.Context(0)
    p = L.Pipeline(c, L.PipelineParams())
    s = L.Server(c, L.ServerParams())
    b = L.Batch(c, L.BatchParams())
    c.close()
    p.close(), s.close(), b.close()
    _check_order(fake)
    # Children first.
    fake.log.clear()
    c = L.Context(0)
    p = L.Pipeline(c, L.PipelineParams())
    p.close()
    p2 = L.Pipeline(c, L.PipelineParams())
    c.close()
    p2.close()
    _check_order(fake)
    assert len(c._children) == 0


def test_cycle_collected(monkeypatch):
    fake = FakeLib()
    monkeypatch.setattr(L, "_lib", fake)
    gc.collect()
    for _ in range(8):
        c = L.Context(0)
        ps = [L.Pipeline(c, L.PipelineParams()) for _ in range(3)]
        cyc = [c, *ps]
        cyc.append(cyc)
        for p in ps:
            p.cycle = cyc
        del c, ps, p, cyc
        gc.collect()
        _check_order(fake)
        fake.log.clear()
