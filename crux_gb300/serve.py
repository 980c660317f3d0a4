"""Serving loop front end: cxgServer* of include/cxlik_gpu.h.

``Server(precision, hbm_budget, max_active)`` starts the library's request
loop; ``submit(request)`` copies a request and returns a ticket;
``wait(ticket)`` returns (lnL, latency_ms).  ``request_from_case`` turns a
synthetic case (tree + compressed alignment + model) into a request.
"""
import ctypes

import numpy as np

from . import _native
from .mc3 import tree_arrays

LNL, MC3 = 0, 1


class ServerConfig(ctypes.Structure):
    _fields_ = [("max_active", ctypes.c_uint),
                ("hbm_budget", ctypes.c_ulonglong),
                ("precision", ctypes.c_int)]


class Request(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("ntaxa", ctypes.c_uint),
        ("npat", ctypes.c_uint),
        ("masks", ctypes.POINTER(ctypes.c_uint8)),
        ("pattern_freqs", ctypes.POINTER(ctypes.c_uint32)),
        ("parent", ctypes.POINTER(ctypes.c_int32)),
        ("len", ctypes.POINTER(ctypes.c_double)),
        ("root", ctypes.c_uint),
        ("rates", ctypes.c_double * 6),
        ("freqs", ctypes.c_double * 4),
        ("alpha", ctypes.c_double),
        ("ncat", ctypes.c_uint),
        ("pinv", ctypes.c_double),
        ("mc3_gens", ctypes.c_uint),
        ("mc3_chains", ctypes.c_uint),
        ("mc3_heat_delta", ctypes.c_double),
        ("seed", ctypes.c_ulonglong),
        ("session", ctypes.c_ulonglong),
        ("dataset", ctypes.c_ulonglong),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_ulonglong),
                ("batches", ctypes.c_ulonglong),
                ("max_batch", ctypes.c_ulonglong),
                ("bytes_peak", ctypes.c_ulonglong),
                ("bytes_budget", ctypes.c_ulonglong),
                ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double),
                ("wall_s", ctypes.c_double),
                ("updates", ctypes.c_double),
                ("deferrals", ctypes.c_ulonglong)]


def declare(lib):
    P, vp = ctypes.POINTER, ctypes.c_void_p
    lib.cxgServerCreate.argtypes = [P(ServerConfig), P(vp)]
    lib.cxgServerCreate.restype = ctypes.c_int
    lib.cxgServerSubmit.argtypes = [vp, P(Request), P(ctypes.c_ulonglong)]
    lib.cxgServerSubmit.restype = ctypes.c_int
    lib.cxgServerWait.argtypes = [vp, ctypes.c_ulonglong, ctypes.c_double,
                                  P(ctypes.c_double), P(ctypes.c_double)]
    lib.cxgServerWait.restype = ctypes.c_int
    lib.cxgServerAddDataset.argtypes = [vp, ctypes.c_ulonglong, ctypes.c_uint,
                                        ctypes.c_uint, P(ctypes.c_uint8),
                                        P(ctypes.c_uint32)]
    lib.cxgServerAddDataset.restype = ctypes.c_int
    lib.cxgServerAddDatasetRaw.argtypes = [
        vp, ctypes.c_ulonglong, ctypes.c_uint, ctypes.c_uint, P(ctypes.c_uint8),
        P(ctypes.c_uint8), P(ctypes.c_uint8), ctypes.c_uint8, P(ctypes.c_uint)]
    lib.cxgServerAddDatasetRaw.restype = ctypes.c_int
    lib.cxgServerDropDataset.argtypes = [vp, ctypes.c_ulonglong]
    lib.cxgServerDropDataset.restype = ctypes.c_int
    lib.cxgServerStats.argtypes = [vp, P(ServerStats)]
    lib.cxgServerStats.restype = ctypes.c_int
    lib.cxgServerResetStats.argtypes = [vp]
    lib.cxgServerResetStats.restype = ctypes.c_int
    lib.cxgServerDestroy.argtypes = [vp]
    lib.cxgServerDestroy.restype = ctypes.c_int


class PreparedRequest:
    """Host arrays of one request, kept alive while it is submitted."""

    def __init__(self, case, kind=LNL, mc3_gens=10, mc3_chains=4, seed=1,
                 session=0, alignment=None, dataset=0):
        aln = alignment if alignment is not None else case.alignment()
        self.alignment = aln
        self.case = case
        tree = case.tree(aln.taxaMap)
        self.parent, self.length, self.root = tree_arrays(tree, aln.taxaMap)
        ch = aln.charType.get()
        self.masks = np.ascontiguousarray(ch.val_table[aln.rows], dtype=np.uint8)
        self.freqs = np.ascontiguousarray(aln.freqs, dtype=np.uint32)
        r = Request()
        r.kind = kind
        r.ntaxa = aln.ntaxa
        r.npat = aln.nchars
        r.masks = self.masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        r.pattern_freqs = self.freqs.ctypes.data_as(
            ctypes.POINTER(ctypes.c_uint32))
        r.parent = self.parent.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        r.len = self.length.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        r.root = self.root
        for i in range(6):
            r.rates[i] = float(case.params["rates"][i])
        for i in range(4):
            r.freqs[i] = float(case.params["freqs"][i])
        r.alpha = float(case.alpha) if case.alpha is not None else 1.0
        r.ncat = case.ncat if case.alpha is not None else 1
        r.pinv = float(case.pinv)
        r.mc3_gens = mc3_gens
        r.mc3_chains = mc3_chains
        r.mc3_heat_delta = 0.1
        r.seed = seed
        r.session = session
        r.dataset = dataset
        self.req = r
        self.updates = (aln.ntaxa - 2) * aln.nchars

    def oracle_lik(self, lib):
        """The same likelihood as a Lik on `lib` (for checks)."""
        return self.case.lik(lib=lib, alignment=self.case.alignment())


class Server:
    def __init__(self, precision="fp32", hbm_budget=0, max_active=256,
                 lib=None):
        self.lib = lib or _native.load()
        declare(self.lib)
        c = ServerConfig(max_active, hbm_budget,
                         1 if precision == "fp32" else 0)
        self.h = ctypes.c_void_p()
        rc = self.lib.cxgServerCreate(ctypes.byref(c), ctypes.byref(self.h))
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgServerCreate")
        self._keep = {}

    def submit(self, prepared):
        t = ctypes.c_ulonglong()
        rc = self.lib.cxgServerSubmit(self.h, ctypes.byref(prepared.req),
                                      ctypes.byref(t))
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgServerSubmit")
        return t.value

    def add_dataset(self, ident, prepared):
        """Keep `prepared`'s patterns on the device under `ident`; requests
        built with ``dataset=ident`` then send no patterns."""
        rc = self.lib.cxgServerAddDataset(
            self.h, ident, prepared.req.ntaxa, prepared.req.npat,
            prepared.req.masks, prepared.req.pattern_freqs)
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgServerAddDataset")

    def add_dataset_raw(self, ident, alignment):
        """Keep a raw (uncompacted) alignment's patterns on the device under
        `ident`; the server compacts it there.  Returns the pattern count
        (that of Alignment.compact, in the same order)."""
        ch = alignment.charType.get()
        rows = np.ascontiguousarray(alignment.rows, dtype=np.uint8)
        canon = np.ascontiguousarray(ch.canon_table, dtype=np.uint8)
        val = np.ascontiguousarray(np.where(ch.val_table < 0, 0, ch.val_table),
                                   dtype=np.uint8)
        u8 = ctypes.POINTER(ctypes.c_uint8)
        npat = ctypes.c_uint()
        rc = self.lib.cxgServerAddDatasetRaw(
            self.h, ident, rows.shape[0], rows.shape[1],
            rows.ctypes.data_as(u8), canon.ctypes.data_as(u8),
            val.ctypes.data_as(u8), ch.any, ctypes.byref(npat))
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgServerAddDatasetRaw")
        return npat.value

    def drop_dataset(self, ident):
        rc = self.lib.cxgServerDropDataset(self.h, ident)
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgServerDropDataset")

    def wait(self, ticket, timeout=120.0):
        v, lat = ctypes.c_double(), ctypes.c_double()
        rc = self.lib.cxgServerWait(self.h, ticket, timeout, ctypes.byref(v),
                                    ctypes.byref(lat))
        if rc != 0:
            raise _native.error(self.lib, rc, "cxgServerWait")
        return v.value, lat.value

    def stats(self):
        s = ServerStats()
        self.lib.cxgServerStats(self.h, ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def reset_stats(self):
        self.lib.cxgServerResetStats(self.h)

    def close(self):
        if self.h:
            self.lib.cxgServerDestroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
