"""Host logic of engine.Resident that needs no GPU: the per-network workspace cache."""
import ctypes

import torch

from graddft_gb300 import engine


class _Net:
    def __init__(self, key, nbytes):
        self.key, self.nbytes = key, nbytes
        self.desc = ctypes.c_int(0)


def _resident():
    r = object.__new__(engine.Resident)  # no device buffers: only the cache is exercised
    r.desc = ctypes.c_int(0)
    r.device = torch.device("cpu")
    return r


def test_network_workspaces_cached_per_key():
    """Alternating networks (the DM21 inputs' default network beside a functional's own) keep one zeroed
    workspace each instead of reallocating on every switch; the oldest goes beyond the kept count."""
    r = _resident()
    calls = []
    nets = {}

    def size_fn(desc, net_desc, out):
        net = nets[id(net_desc._obj)]
        calls.append(net.key)
        out._obj.value = net.nbytes
        return 0

    a, b = _Net(("a",), 64), _Net(("b",), 32)
    for n in (a, b):
        nets[id(n.desc)] = n
    wa = r._cached_ws("_nws", a, size_fn)
    wb = r._cached_ws("_nws", b, size_fn)
    for _ in range(3):
        assert r._cached_ws("_nws", a, size_fn) is wa
        assert r._cached_ws("_nws", b, size_fn) is wb
    assert calls == [("a",), ("b",)]
    assert wa.numel() == 64 and int(wa.sum()) == 0 and wb.numel() == 32
    extra = [_Net((f"n{i}",), 8) for i in range(engine.Resident._WS_KEEP)]
    for n in extra:
        nets[id(n.desc)] = n
        r._cached_ws("_nws", n, size_fn)
    assert len(r._nws) == engine.Resident._WS_KEEP and ("a",) not in r._nws
