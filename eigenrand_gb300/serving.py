"""Serving loop over per-client device-resident engines (gr_server_* in
include/gpurand.h): requests of mixed kinds and sizes are admitted by stream
slots and a device-memory budget, run concurrently, and complete out of order;
each client's requests run in order on its own Vmt19937_64, so every result
equals the client's plain call sequence run alone.

    srv = Server(nclients=256, seeds=[1000 + c for c in range(256)], budget_bytes=40 << 30)
    t = srv.submit(client=3, kind="GAMMA", dtype=torch.float32, count=10**6, a=0.5, b=1.0)
    for c in srv.progress(): ...   # dicts with ticket, latency, ...
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import KINDS, GR_SERVE_MVNORMAL

_L = _lib.load()
_DT = {torch.float32: _lib.F32, torch.float64: _lib.F64, torch.int32: _lib.I32}
_NP = {_lib.F32: np.float32, _lib.F64: np.float64, _lib.I32: np.int32}


def now():
    return _L.gr_server_now()


class Server:
    def __init__(self, nclients, seeds, budget_bytes, slots=32):
        arr = (ctypes.c_uint64 * nclients)(*[int(s) for s in seeds])
        h = ctypes.c_void_p()
        _lib.check(_L.gr_server_create(ctypes.byref(h), nclients, arr, int(budget_bytes), slots))
        self._h = h
        self.nclients = nclients
        self._cap = 4096
        self._buf = (_lib.Completion * self._cap)()
        self._dtype = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _L is not None:
            _L.gr_server_destroy(h)
            self._h = None

    def set_mvnormal(self, mean, cov):
        mean = np.asarray(mean, dtype=np.float64)
        cov = np.asarray(cov, dtype=np.float64)
        d = mean.size
        m = (ctypes.c_double * d)(*mean.tolist())
        c = (ctypes.c_double * (d * d))(*cov.reshape(-1, order="F").tolist())
        _lib.check(_L.gr_server_set_mvnormal(self._h, d, m, c))

    def submit(self, client, kind, dtype, count, a=0.0, b=0.0, trials=0, arrival=-1.0):
        r = _lib.Request()
        r.client = client
        r.kind = GR_SERVE_MVNORMAL if kind == "MVNORMAL" else KINDS[kind]
        r.dtype = _DT[dtype]
        r.trials = int(trials)
        r.a = float(a)
        r.b = float(b)
        r.count = int(count)
        r.arrival = float(arrival)
        t = ctypes.c_uint64()
        _lib.check(_L.gr_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)))
        self._dtype[t.value] = r.dtype
        return t.value

    def progress(self):
        n = ctypes.c_size_t()
        _lib.check(_L.gr_server_progress(self._h, self._buf, self._cap, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            c = self._buf[i]
            out.append(dict(ticket=c.ticket, status=c.status, client=c.client, count=c.count, bytes=c.bytes,
                            arrival=c.arrival, admitted=c.admitted, completed=c.completed))
        return out

    def read(self, ticket, count=None):
        """Copy a finished result to a numpy array (synchronous)."""
        dt = _NP[self._dtype[ticket]]
        n = count
        a = np.empty(n, dtype=dt)
        _lib.check(_L.gr_server_read(self._h, ticket, ctypes.c_void_p(a.ctypes.data), a.nbytes))
        return a

    def release(self, ticket):
        _lib.check(_L.gr_server_release(self._h, ticket))
        self._dtype.pop(ticket, None)

    def cancel(self, ticket):
        """Cancel a request not reported yet: queued ones never run, running ones
        finish on the GPU and are freed; reported later with status
        GR_ERR_CANCELLED and ended by release() like any other."""
        _lib.check(_L.gr_server_cancel(self._h, ticket))

    def cancel_client(self, client):
        """Cancel every unreported request of a client (a client that went away)."""
        _lib.check(_L.gr_server_cancel_client(self._h, client))

    def fail_allocs(self, n):
        """Test hook: the next n result allocations fail (GR_ERR_NOMEM completions)."""
        _lib.check(_L.gr_server_fail_allocs(self._h, n))

    def pending(self):
        q, r, b = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        _lib.check(_L.gr_server_pending(self._h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(b)))
        return q.value, r.value, b.value
