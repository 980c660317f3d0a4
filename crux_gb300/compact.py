"""Pattern compression on the GPU: ``cxgCompact`` (include/cxlik_gpu.h).

``compact(alignment)`` does what ``Alignment.compact`` does on the host
(pkg/Crux/CTMatrix.pyx:949-1031): canonical codes, sorted unique columns,
summed frequencies.  It also returns the leaf-tip state masks that the
likelihood walker reads (Lik.pyx:1466-1475: 0 -> all states).
"""
import ctypes

import numpy as np

from . import _native


def declare(lib):
    P = ctypes.POINTER
    lib.cxgCompact.argtypes = [P(ctypes.c_uint8), ctypes.c_uint, ctypes.c_uint,
                               P(ctypes.c_uint32), P(ctypes.c_uint8),
                               P(ctypes.c_uint8), ctypes.c_uint8,
                               P(ctypes.c_uint8), P(ctypes.c_uint32),
                               P(ctypes.c_uint8), P(ctypes.c_uint)]
    lib.cxgCompact.restype = ctypes.c_int


def _u8(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def compact(alignment, lib=None, masks=True):
    """(rows [ntaxa][npat] canonical codes, freqs [npat] uint32,
    masks [ntaxa][npat] uint8 or None) of `alignment`, computed on the GPU."""
    lib = lib or _native.load()
    declare(lib)
    ch = alignment.charType.get()
    rows = np.ascontiguousarray(alignment.rows, dtype=np.uint8)
    ntaxa, nsites = rows.shape
    freqs = np.ascontiguousarray(alignment.freqs, dtype=np.uint32)
    canon = np.ascontiguousarray(ch.canon_table, dtype=np.uint8)
    val = np.ascontiguousarray(np.where(ch.val_table < 0, 0, ch.val_table),
                               dtype=np.uint8)
    out_rows = np.zeros(ntaxa * max(nsites, 1), dtype=np.uint8)
    out_freqs = np.zeros(max(nsites, 1), dtype=np.uint32)
    out_masks = np.zeros(ntaxa * max(nsites, 1), dtype=np.uint8) if masks else None
    npat = ctypes.c_uint()
    rc = lib.cxgCompact(_u8(rows), ntaxa, nsites,
                        freqs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                        _u8(canon), _u8(val), ch.any, _u8(out_rows),
                        out_freqs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                        _u8(out_masks) if masks else None, ctypes.byref(npat))
    if rc != 0:
        raise _native.error(lib, rc, "cxgCompact")
    n = npat.value
    r = out_rows[:ntaxa * n].reshape(ntaxa, n)
    m = out_masks[:ntaxa * n].reshape(ntaxa, n) if masks else None
    return r, out_freqs[:n].copy(), m


def compact_alignment(alignment, lib=None):
    """Compact `alignment` in place on the GPU (as Alignment.compact)."""
    rows, freqs, _ = compact(alignment, lib, masks=False)
    alignment.rows = np.ascontiguousarray(rows)
    alignment.freqs = freqs
    return 0
