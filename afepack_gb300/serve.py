"""Python front end of the solve server (afp_server_* in the C ABI).

    with Server(workers=8) as srv:
        t = srv.submit(workload)          # afepack_gb300.workloads.Workload
        x, result = srv.wait(t)
        srv.stats()                       # p50/p99 latency, solves/s
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


class Server:
    def __init__(self, device: int = 0, workers: int = 8, precision: int = N.AFP_PRECISION_MIXED, tol: float = 1e-10,
                 maxit: int = 500, hbm_budget_bytes: int = 0, dense_tail: int = -1):
        o = N.ServerOpts()
        N.lib().afp_server_default_opts(C.byref(o))
        o.workers, o.precision, o.tol, o.maxit = workers, precision, tol, maxit
        o.hbm_budget_bytes, o.dense_tail = hbm_budget_bytes, dense_tail
        h = C.c_void_p()
        N.call("afp_server_create", device, C.byref(o), C.byref(h))
        self.handle = h
        self._n = {}

    def submit(self, wl) -> int:
        """Queue one request; its arrays are copied, so wl may be dropped."""
        sp, mesh = wl.space, wl.mesh
        coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
        cells = np.ascontiguousarray(mesh.cells, dtype=np.int32)
        ed = np.ascontiguousarray(sp.elem_dof, dtype=np.int32)
        dirichlet = (sp.dof_bmark != 0).astype(np.int32)
        f = np.ascontiguousarray(wl.f, dtype=np.float64)
        coef = None if wl.coef is None else np.ascontiguousarray(wl.coef, dtype=np.float64)
        r = N.Request(mesh.dim, sp.degree, wl.acc_stiff, wl.acc_mass, mesh.n_vertex, coords.ctypes.data, mesh.n_cell,
                      cells.ctypes.data, sp.n_dof, ed.ctypes.data, dirichlet.ctypes.data,
                      None if coef is None else coef.ctypes.data, f.ctypes.data)
        t = C.c_int64()
        N.call("afp_server_submit", self.handle, C.byref(r), C.byref(t))
        self._n[t.value] = sp.n_dof
        return t.value

    def wait(self, ticket: int):
        x = np.empty(self._n.pop(ticket))
        res = N.RequestResult()
        N.call("afp_server_wait", self.handle, ticket, x.ctypes.data, C.byref(res))
        return x, res.as_dict()

    def done(self, ticket: int) -> bool:
        d = C.c_int()
        N.call("afp_server_poll", self.handle, ticket, C.byref(d))
        return bool(d.value)

    def stats(self):
        s = N.ServerStats()
        N.call("afp_server_get_stats", self.handle, C.byref(s))
        return s.as_dict()

    def reset_stats(self):
        N.call("afp_server_reset_stats", self.handle)

    def close(self):
        if self.handle:
            N.lib().afp_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchServer:
    """Continuous batching of right-hand sides against one resident hierarchy
    (afp_batch_server_* in the C ABI): `width` CG columns stay in flight;
    requests join free columns between CG iterations and leave when solved.

        with BatchServer(amg, width=32) as srv:
            t = srv.submit(b)            # numpy array, n doubles
            x, result = srv.wait(t)
    """

    def __init__(self, amg, width: int = 32, tol: float = 1e-10, maxit: int = 500):
        o = N.BatchOpts()
        N.lib().afp_batch_default_opts(C.byref(o))
        o.width, o.tol, o.maxit = width, tol, maxit
        h = C.c_void_p()
        N.call("afp_batch_server_create", amg.handle, C.byref(o), C.byref(h))
        self.handle = h
        self.amg = amg  # keeps the hierarchy alive
        self.n = amg.level_info(0)[0]

    def submit(self, b) -> int:
        b = np.ascontiguousarray(b, dtype=np.float64)
        assert b.shape == (self.n,)
        t = C.c_int64()
        N.call("afp_batch_server_submit", self.handle, b.ctypes.data, C.byref(t))
        return t.value

    def wait(self, ticket: int):
        x = np.empty(self.n)
        res = N.RequestResult()
        N.call("afp_batch_server_wait", self.handle, ticket, x.ctypes.data, C.byref(res))
        return x, res.as_dict()

    def stats(self):
        s = N.ServerStats()
        N.call("afp_batch_server_get_stats", self.handle, C.byref(s))
        return s.as_dict()

    def reset_stats(self):
        N.call("afp_batch_server_reset_stats", self.handle)

    def close(self):
        if self.handle:
            N.lib().afp_batch_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
