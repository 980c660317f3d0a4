"""The ``Lik`` likelihood object: model state, execution planning, lnL.

Python-3 restatement of pkg/Crux/Tree/Lik.pyx (the reference is Python-2
Cython).  ``Lik`` owns a ``CxtLik`` (include/cxlik_gpu.h, the ABI of
lib/Crux/Tree/CxLik.h) and per-ring conditional-likelihood (CL) caches, plans
the post-order step list with the reference's cache-validity rule, and hands
the plan to a C library exporting ``CxLikExecute``.  By default that library
is the GB300 one (crux_gb300/_lib/libcxlik_gpu.so); the ``lib=`` argument
accepts any library with the same three entry points, which is how the tests
run the same plans through the CPU oracles.

Method map to the reference:
  constructor / stripes    Lik.pyx:200-250     model alloc/init/decomp 388-475
  dup / clone              Lik.pyx:587-660, 835-883
  model API                Lik.pyx:885-1393    (weights, rates, freqs, alpha,
                                                +I, mixtures)
  _planAppend/_planRecurse/_plan  Lik.pyx:1395-1601
  prep (weightScaled, wNorm)      Lik.pyx:1603-1665
  lnL / siteLnLs / flush          Lik.pyx:1687-1787
"""
import ctypes
import math
import os
import struct
import weakref

import numpy as np

from . import _abi, _native
from .cxmath import gamma_rates

CACHE_LINE = 64
MQ_MULT = 8  # CxmLikMqMult (CxLik.h:277)

# Counts changes to CL buffers and CL mirrors made outside a planner run
# (prepare, buffer release, flush).  A flattened traversal kept for the
# native planner is valid only while this count and the tree's serial
# number are what they were when it was built.
_epoch = [0]


def _bump():
    _epoch[0] += 1


class Config:
    """Striping policy inputs (pkg/Crux/Config.py; Cx.c:7, 63-66)."""
    threaded = True
    ncpus = os.cpu_count() or 1


def _tokens(nbytes=16):
    return np.empty(max(nbytes // 8, 2), dtype=np.float64)


class CL:
    """CL cache of one ring, two polarities (Lik.pyx:32-108).

    With a device library the host buffers are 16-byte identity tokens (the
    device holds the data); with a host library they are real arrays.
    """
    __slots__ = ("c", "ptr", "addr", "bufs", "lib", "device", "forget",
                 "leaf", "valid", "cvalid", "parent", "nSibs", "edgeLen",
                 "__weakref__")

    def __init__(self, lib, device):
        self.c = (_abi.CxtLikCL(), _abi.CxtLikCL())
        # Pointers to the two structs, made once (plans store them).
        self.ptr = (ctypes.pointer(self.c[0]), ctypes.pointer(self.c[1]))
        self.addr = (ctypes.addressof(self.c[0]), ctypes.addressof(self.c[1]))
        self.bufs = [None, None]
        self.lib = lib
        self.device = device
        # A GPU library caches device copies keyed by the host pointer:
        # tell it when a host buffer goes away (also in drop-in mode).
        self.forget = hasattr(lib, "cxgLikClForget")
        self.leaf = False
        # Python mirrors of the CxtLikCL cache-key fields, per polarity.
        # The planner works on the mirrors; the struct's valid field is
        # brought up to date at the end of each plan (sync_valid), and
        # cvalid is what the struct holds.
        self.valid = [False, False]
        self.cvalid = [False, False]
        self.parent = [None, None]
        self.nSibs = [0, 0]
        self.edgeLen = [0.0, 0.0]

    def prepare(self, polarity, nchars, dim, ncomp):
        if self.bufs[polarity] is None:
            _bump()
            if self.device:
                mat, lsc = _tokens(), _tokens()
            else:
                mat = np.zeros(nchars * dim * ncomp, dtype=np.float64)
                lsc = np.zeros(nchars, dtype=np.float64)
            self.bufs[polarity] = (mat, lsc)
            self.c[polarity].cLMat = _abi.dptr(mat)
            self.c[polarity].lnScale = _abi.dptr(lsc)

    def resize(self, polarity, nchars, dim, ncomp):
        self.flush_buffers(polarity)
        self.prepare(polarity, nchars, dim, ncomp)

    def flush_buffers(self, polarity):
        b = self.bufs[polarity]
        if b is not None:
            _bump()
            if self.forget:
                self.lib.cxgLikClForget(_abi.dptr(b[0]))
            self.bufs[polarity] = None
            self.c[polarity].cLMat = None
            self.c[polarity].lnScale = None

    def flush(self, polarity):
        self.flush_buffers(polarity)
        if self.valid[polarity] or self.cvalid[polarity] or \
                self.parent[polarity] is not None:
            _bump()
        self.c[polarity].valid = False
        self.c[polarity].parent = None
        self.valid[polarity] = False
        self.cvalid[polarity] = False
        self.parent[polarity] = None

    def set_valid(self, polarity, v):
        self.valid[polarity] = v

    def sync_valid(self, polarity):
        v = self.valid[polarity]
        if self.cvalid[polarity] != v:
            self.c[polarity].valid = v
            self.cvalid[polarity] = v

    def release(self):
        for p in (0, 1):
            self.flush_buffers(p)

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class _Model:
    """Host copy of one CxtLikModel with its arrays (Lik.pyx:388-466)."""

    def __init__(self, dim, rlen):
        self.s = _abi.CxtLikModel()
        self.rclass = np.zeros(rlen, dtype=np.uint32)
        self.rTri = np.ones(rlen, dtype=np.float64)
        self.piDiag = np.full(dim, 1.0 / dim, dtype=np.float64)
        self.piDiagNorm = np.zeros(dim, dtype=np.float64)
        self.cube = np.zeros(dim * dim * dim, dtype=np.float64)
        self.eig = np.zeros(dim, dtype=np.float64)
        s = self.s
        s.rclass = _abi.uptr(self.rclass)
        s.rTri = _abi.dptr(self.rTri)
        s.piDiag = _abi.dptr(self.piDiag)
        s.piDiagNorm = _abi.dptr(self.piDiagNorm)
        s.qEigVecCube = _abi.dptr(self.cube)
        s.qEigVals = _abi.dptr(self.eig)


def default_library():
    from . import _native
    return _native.load()


_planner = []


def planner_library():
    """The library exporting cxgPlanSnapRun (the GB300 library; loading it
    makes no CUDA call), or None where it has not been built.  Host-only
    libraries given as `lib=` (the CPU oracles) plan through it too."""
    if not _planner:
        try:
            from . import _native
            _planner.append(_native.load())
        except Exception:
            _planner.append(None)
    return _planner[0]


def _lik_unpickled(precision, dropin):
    """An empty Lik for pickle to fill (Lik.__setstate__); its library is
    set by Lik.unpickle."""
    ret = Lik.__new__(Lik)
    ret.lib = None
    ret.dropin = dropin
    ret.device = False
    ret.precision = precision
    ret.lik = None
    ret.mate = None
    ret._models = []
    ret._snap = None
    ret._pyKey = None
    ret._compsKey = None
    return ret


class _Snap:
    """A flattened rooted traversal for cxgPlanSnapRun (see Lik._snapBuild)."""


class Lik:
    """Tree likelihood over an alignment and a mixture of models."""

    def __init__(self, tree=None, alignment=None, nmodels=1, ncat=1,
                 catMedian=False, invar=False, lib=None, precision="fp64",
                 dropin=False):
        """`lib`: library exporting the CxLik entry points (default: the
        GB300 one).  `precision`: "fp64" (plain) or "fp32" (scaled form).
        `dropin`: drive the library exactly as Lik.pyx does -- host CL
        buffers with leaf rows of 4 doubles, CxLikExecute, and the stripe
        sum -- instead of the device-resident cxg* path."""
        self.dropin = dropin
        self._set_lib(lib if lib is not None else default_library())
        self.precision = precision
        self.lik = None
        self.mate = None
        self._models = []
        self._snap = None
        self._pyKey = None
        self._compsKey = None
        if alignment is not None:
            self._init0(tree)
            nchars = alignment.nchars
            npad = self._computeNpad(nchars, self._computeStripeWidth(nchars))
            char_ = alignment.charType.get()
            if npad != 0:
                alignment.pad(char_.val2code(char_.any), npad)
                nchars += npad
            self._init1(tree, nchars, char_.nstates, 0)
            self._init2(alignment, char_)
            for _ in range(nmodels):
                self.addModel(1.0, ncat, catMedian, invar)

    def _set_lib(self, lib):
        self.lib = lib
        # A host library that sets plan_natively = False is planned by the
        # Python restatement alone and never maps the GB300 library.
        if not getattr(lib, "plan_natively", True):
            self.native_plan = False
        self.device = hasattr(lib, "cxgLikClForget") and not self.dropin

    # -- construction (Lik.pyx:221-324) ------------------------------------
    @staticmethod
    def _computeStripeWidth(nchars):
        if Config.threaded:
            quantum = CACHE_LINE // (4 * 8)
            width = quantum
            nstripes = -(-nchars // width)
            while nstripes > Config.ncpus * MQ_MULT:
                width += quantum
                nstripes = -(-nchars // width)
            return width
        return nchars

    @staticmethod
    def _computeNpad(nchars, width):
        return (width - nchars % width) if nchars % width else 0

    def _init0(self, tree):
        if tree.rooted:
            raise ValueError("Tree must be unrooted")
        tree.clearAux()

    def _init1(self, tree, nchars, dim, polarity):
        self.mate = None
        self._snap = None
        self._pyKey = None
        self._compsKey = None
        self.tree = tree
        L = self.lik = _abi.CxtLik()
        L.polarity = polarity
        L.dim = dim
        L.rlen = dim * (dim - 1) // 2
        L.cbase = 0
        L.nchars = nchars
        L.mschars = nchars
        L.stripeWidth = self._computeStripeWidth(nchars)
        L.nstripes = L.mschars // L.stripeWidth
        assert L.nstripes * L.stripeWidth == L.mschars
        L.invalidate = False
        L.resize = False
        L.reweight = False
        L.wNorm = 0.0
        self._models = []
        self._comps = []          # per component: [model, cweight, cmult]
        self._compsArr = None
        self._modelsArr = None
        self.siteLnLBuf = np.zeros(nchars, dtype=np.float64)
        self.stripeLnLBuf = np.zeros(L.nstripes, dtype=np.float64)
        L.siteLnL = _abi.dptr(self.siteLnLBuf)
        L.stripeLnL = _abi.dptr(self.stripeLnLBuf)

    def _init2(self, alignment, char_):
        self.char_ = char_
        self.alignment = alignment
        L = self.lik
        L.npad = alignment.npad
        self._freqs = np.ascontiguousarray(alignment.freqs, dtype=np.uint32)
        L.charFreqs = _abi.uptr(self._freqs)
        if self.device and hasattr(self.lib, "cxgLikSetPatternWeights"):
            # The weights of a compacted alignment do not change: register
            # them once (the library then skips comparing them per call) and
            # forget them when this Lik goes away.
            n = int(L.mschars)
            rc = self.lib.cxgLikSetPatternWeights(L.charFreqs, n)
            if rc != 0:
                raise _native.error(self.lib, rc, "cxgLikSetPatternWeights")
            fin = weakref.finalize(self, self.lib.cxgLikForgetPatternWeights,
                                   _abi.uptr(self._freqs), n)
            fin.atexit = False  # the process's exit releases the device copy
        stepsMax = 2 * alignment.ntaxa - 2
        self._steps = (_abi.CxtLikStep * max(stepsMax, 1))()
        L.steps = ctypes.cast(self._steps, ctypes.POINTER(_abi.CxtLikStep))
        L.stepsLen = 0
        L.stepsMax = stepsMax
        self.rootCL = CL(self.lib, self.device)
        L.rootCLC = ctypes.pointer(self.rootCL.c[L.polarity])

    # -- component array maintenance ----------------------------------------
    def _sync_comps(self):
        """Rebuild the C comps/models arrays from the Python-side lists, unless
        they already hold exactly these models and values (the key keeps the
        model objects themselves, so a replaced model never matches)."""
        key = (tuple((c["model"], c["weightScaled"], c["cweight"], c["cmult"])
                     for c in self._comps),
               tuple((m, m.comp0, m.clen) for m in self._models))
        if key == self._compsKey:
            return
        self._compsKey = key
        n = len(self._comps)
        arr = (_abi.CxtLikComp * max(n, 1))()
        for i, c in enumerate(self._comps):
            arr[i].model = ctypes.pointer(c["model"].s)
            arr[i].weightScaled = c["weightScaled"]
            arr[i].cweight = c["cweight"]
            arr[i].cmult = c["cmult"]
        self._compsArr = arr
        self.lik.comps = ctypes.cast(arr, ctypes.POINTER(_abi.CxtLikComp))
        self.lik.compsLen = n
        self.lik.compsMax = max(n, 1)
        m = len(self._models)
        marr = (ctypes.POINTER(_abi.CxtLikModel) * max(m, 1))()
        for i, mod in enumerate(self._models):
            marr[i] = ctypes.pointer(mod.s)
            mod.s.comp0 = mod.comp0
            mod.s.clen = mod.clen
        self._modelsArr = marr
        self.lik.models = ctypes.cast(
            marr, ctypes.POINTER(ctypes.POINTER(_abi.CxtLikModel)))
        self.lik.modelsLen = m
        self.lik.modelsMax = max(m, 1)

    # -- models (Lik.pyx:388-509, 885-1393) ----------------------------------
    def _model(self, i):
        assert i < len(self._models)
        return self._models[i]

    def addModel(self, weight, ncat=1, catMedian=False, invar=False):
        assert ncat > 0
        L = self.lik
        mod = _Model(L.dim, L.rlen)
        ncomp = ncat + (1 if invar else 0)
        mod.comp0 = len(self._comps)
        mod.clen = ncomp
        s = mod.s
        s.decomp = True
        s.weight = weight
        s.rmult = 1.0
        s.alpha = math.inf
        s.catMedian = catMedian
        s.invar = invar
        for i in range(ncomp):
            self._comps.append({"model": mod, "cweight": 1.0 if i == 0 else 0.0,
                                "cmult": 1.0 if i == 0 else 0.0,
                                "weightScaled": 0.0})
        self._models.append(mod)
        self._sync_comps()
        L.resize = True
        return len(self._models) - 1

    def delModel(self, model):
        assert model < len(self._models)
        if len(self._models) == 0:
            raise ValueError("No models remain")
        mod = self._models[model]
        del self._comps[mod.comp0:mod.comp0 + mod.clen]
        for later in self._models[model + 1:]:
            later.comp0 -= mod.clen
        del self._models[model]
        self._sync_comps()
        self.lik.resize = True

    def nmodels(self):
        return len(self._models)

    def getWNorm(self):
        return self.lik.wNorm

    def getWeight(self, model):
        return self._model(model).s.weight

    def setWeight(self, model, weight):
        assert weight >= 0.0
        self._model(model).s.weight = weight
        self.lik.reweight = True

    def getRmult(self, model):
        return self._model(model).s.rmult

    def setRmult(self, model, rmult):
        assert rmult >= 0.0
        self._model(model).s.rmult = rmult
        self.lik.reweight = True

    def getRclass(self, model):
        return [int(x) for x in self._model(model).rclass]

    def setRclass(self, model, rclass, rates=None):
        mod = self._model(model)
        rmax = 0
        for r in rclass:
            if r == rmax + 1:
                rmax += 1
            elif r > rmax + 1:
                raise ValueError("Invalid rclass specification")
        mod.rclass[:] = rclass
        if rates is None:
            mod.rTri[:] = 1.0
        else:
            if len(rates) != rmax + 1:
                raise ValueError("Incorrect rates list length")
            for i in range(self.lik.rlen):
                if not isinstance(rates[rclass[i]], float):
                    raise ValueError("Incorrect type for rate %d" % i)
            for i in range(self.lik.rlen):
                mod.rTri[i] = rates[rclass[i]]
        mod.s.decomp = True

    def getNrates(self, model):
        return int(self._model(model).rclass.max()) + 1

    def getRate(self, model, i):
        mod = self._model(model)
        for j in range(self.lik.rlen):
            if mod.rclass[j] == i:
                return float(mod.rTri[j])
        raise ValueError("Invalid rate class index")

    def setRate(self, model, i, rate):
        mod = self._model(model)
        assert rate >= 0.0
        found = False
        decomp = False
        for j in range(self.lik.rlen):
            if mod.rclass[j] == i:
                if mod.rTri[j] != rate:
                    decomp = True
                mod.rTri[j] = rate
                found = True
        if not found:
            raise ValueError("Invalid rate class index")
        if decomp:
            mod.s.decomp = True

    def getFreq(self, model, i):
        return float(self._model(model).piDiag[i])

    def setFreq(self, model, i, freq):
        mod = self._model(model)
        assert freq > 0.0
        if mod.piDiag[i] != freq:
            mod.piDiag[i] = freq
            mod.s.decomp = True

    def getAlpha(self, model):
        return self._model(model).s.alpha

    def _ncat(self, mod):
        return mod.clen - (1 if mod.s.invar else 0)

    def setAlpha(self, model, alpha):
        mod = self._model(model)
        ncat = self._ncat(mod)
        assert ncat > 1
        if mod.s.alpha == alpha:
            return
        mod.s.alpha = alpha
        comps = self._comps[mod.comp0:mod.comp0 + ncat]
        if alpha != math.inf:
            rates = gamma_rates(alpha, ncat, bool(mod.s.catMedian))
            for c, r in zip(comps, rates):
                c["cmult"] = r
            cw = sum(c["cweight"] for c in comps) / ncat
            for c in comps:
                c["cweight"] = cw
        else:
            cw = sum(c["cweight"] for c in comps)
            comps[0]["cweight"] = cw
            comps[0]["cmult"] = 1.0
            for c in comps[1:]:
                c["cweight"] = 0.0
                c["cmult"] = 0.0
        self._sync_comps()
        self.lik.invalidate = True

    def getNcat(self, model):
        return self._ncat(self._model(model))

    def getCatMedian(self, model):
        return bool(self._model(model).s.catMedian)

    def getInvar(self, model):
        return bool(self._model(model).s.invar)

    def getWVar(self, model):
        mod = self._model(model)
        if mod.s.alpha == math.inf:
            return self._comps[mod.comp0]["cweight"]
        return sum(c["cweight"] for c in
                   self._comps[mod.comp0:mod.comp0 + self._ncat(mod)])

    def setWVar(self, model, wVar):
        mod = self._model(model)
        assert wVar >= 0.0
        if mod.s.alpha == math.inf:
            self._comps[mod.comp0]["cweight"] = wVar
        else:
            n = self._ncat(mod)
            for c in self._comps[mod.comp0:mod.comp0 + n]:
                c["cweight"] = wVar / n
        self._sync_comps()
        self.lik.reweight = True

    def getWInvar(self, model):
        mod = self._model(model)
        if not mod.s.invar:
            return 0.0
        return self._comps[mod.comp0 + mod.clen - 1]["cweight"]

    def setWInvar(self, model, wInvar):
        mod = self._model(model)
        if not mod.s.invar and wInvar != 0.0:
            raise ValueError("Model does not support invariable sites.")
        assert wInvar >= 0.0
        self._comps[mod.comp0 + mod.clen - 1]["cweight"] = wInvar
        self._sync_comps()
        self.lik.reweight = True

    # -- pickling (Lik.pyx:326-386, 573-585) ---------------------------------
    def __reduce__(self):
        return (_lik_unpickled, (self.precision, self.dropin), self.__getstate__())

    def __getstate__(self):
        """(tree, nchars, dim) and one tuple per model: weight, rmult,
        rclass, rates, freqs, alpha, ncat, catMedian, invar, wVar, wInvar.
        The alignment is not part of the state: ``unpickle`` takes it from
        the Lik it is called on."""
        init_args = (self.tree, self.lik.nchars, self.lik.dim)
        models = []
        for i in range(len(self._models)):
            models.append((self.getWeight(i), self.getRmult(i), self.getRclass(i),
                           [self.getRate(i, j) for j in range(self.getNrates(i))],
                           [self.getFreq(i, j) for j in range(self.lik.dim)],
                           self.getAlpha(i), self.getNcat(i), self.getCatMedian(i),
                           self.getInvar(i), self.getWVar(i), self.getWInvar(i)))
        return (init_args, models)

    def __setstate__(self, data):
        init_args, models = data
        tree, nchars, dim = init_args
        self._init0(tree)
        self._init1(tree, nchars, dim, 0)
        for i, (weight, rmult, rclass, rates, freqs, alpha, ncat, catMedian,
                invar, wVar, wInvar) in enumerate(models):
            self.addModel(weight, ncat, catMedian, invar)
            self.setRmult(i, rmult)
            self.setRclass(i, rclass, rates)
            assert len(freqs) == self.lik.dim
            for j in range(self.lik.dim):
                self.setFreq(i, j, freqs[j])
            if alpha != math.inf:
                self.setAlpha(i, alpha)
            if invar:
                self.setWVar(i, wVar)
                self.setWInvar(i, wInvar)

    def unpickle(self, data):
        """The partial Lik pickled in `data` (bytes), completed with this
        Lik's alignment, library, precision and drop-in mode."""
        import pickle
        ret = pickle.loads(data)
        ret.dropin = self.dropin
        ret._set_lib(self.lib)
        ret._init2(self.alignment, self.char_)
        return ret

    # -- simulation (Lik.pyx:662-833) ---------------------------------------
    def simulate(self, nchars=0, rng=None):
        """A duplicate of this Lik (see dup) whose alignment holds sequences
        simulated under the current models, tree and branch lengths: nchars
        sites (default: as many as this alignment's unpadded sites), padded
        to the stripe width as a new Lik would be, uncompacted.  Draws come
        from `rng` (a random.Random; default: the random module), in the
        reference's order: the root sequence component by component, then
        each child edge depth-first in ring order."""
        import random
        from .alignment import Alignment
        rng = rng if rng is not None else random
        ret = Lik(lib=self.lib, precision=self.precision, dropin=self.dropin)
        tree = self.tree.dup()
        if nchars == 0:
            nchars = self.alignment.nchars - self.alignment.npad
        aln = Alignment(taxaMap=self.alignment.taxaMap, nchars=nchars,
                        charType=self.alignment.charType)
        npad = self._computeNpad(nchars, self._computeStripeWidth(nchars))
        if npad != 0:
            aln.pad(self.char_.val2code(self.char_.any), npad)
            nchars += npad
        ret._init0(tree)
        ret._init1(tree, nchars, self.lik.dim, 0)
        ret._init2(aln, self.char_)
        self._dup(ret)
        ret._simulate(rng)
        return ret

    def _simulate(self, rng):
        L = self.lik
        dim = L.dim
        i2c = "".join(self.char_.pcodes())
        self.prep()
        # Breaks between the sites simulated under each component, by
        # weightScaled (Lik.pyx:760-776).
        nsim = self.alignment.nchars - self.alignment.npad
        brks = []
        wsum = 0.0
        for i in range(L.compsLen - 1):
            wsum += L.comps[i].weightScaled
            if wsum > 1.0:
                wsum = 1.0
            brks.append(int(math.ceil(wsum * float(nsim))))
        brks.append(nsim)

        def cdf_of(row):
            cdf, cum = [], 0.0
            for j in range(dim - 1):
                cum += row[j]
                if cum > 1.0:
                    cum = 1.0
                cdf.append(cum)
            cdf.append(1.0)
            return cdf

        def draw(cdf):
            u = rng.random()
            for j in range(dim):
                if cdf[j] >= u:
                    return j
            raise AssertionError("CDF does not reach 1")

        def root_seq():
            seq, c = [], 0
            for comp in range(L.compsLen):
                m = L.comps[comp].model.contents
                cdf = cdf_of([m.piDiagNorm[j] for j in range(dim)])
                while c < brks[comp]:
                    seq.append(draw(cdf))
                    c += 1
            return seq

        P = np.zeros(dim * dim, dtype=np.float64)

        def child_seq(par, brlen):
            seq, c = [], 0
            for comp in range(L.compsLen):
                m = L.comps[comp].model.contents
                self.lib.CxLikPt(dim, _abi.dptr(P), m.qEigVecCube, m.qEigVals,
                                 brlen)
                cdfs = [cdf_of(P[i * dim:(i + 1) * dim]) for i in range(dim)]
                while c < brks[comp]:
                    seq.append(draw(cdfs[par[c]]))
                    c += 1
            return seq

        def put(node, seq):
            if node.getTaxon() is not None:
                self.alignment.setSeq(
                    self.alignment.taxaMap.indGet(node.getTaxon()), 0,
                    "".join(i2c[x] for x in seq))

        base = self.tree.getBase()
        seq = root_seq()
        put(base, seq)
        if base.ring is None:
            return
        stack = [(r.other, seq) for r in reversed(list(base.ring))]
        while stack:
            ring, par = stack.pop()
            s = child_seq(par, ring.edge.length)
            put(ring.node, s)
            for r in reversed(list(ring.siblings())):
                stack.append((r.other, s))

    # -- copies (Lik.pyx:587-660, 835-883) ------------------------------------
    def _dup(self, other):
        assert len(other._models) == 0
        for fr in self._models:
            ncat = fr.clen - (1 if fr.s.invar else 0)
            m = other.addModel(fr.s.weight, ncat, bool(fr.s.catMedian),
                               bool(fr.s.invar))
            to = other._models[m]
            to.s.rmult = fr.s.rmult
            to.rclass[:] = fr.rclass
            to.rTri[:] = fr.rTri
            to.piDiag[:] = fr.piDiag
            to.piDiagNorm[:] = fr.piDiagNorm
            to.s.alpha = fr.s.alpha
            to.s.catMedian = fr.s.catMedian
        for i, c in enumerate(self._comps):
            other._comps[i]["cweight"] = c["cweight"]
            other._comps[i]["cmult"] = c["cmult"]
        other._sync_comps()

    def dup(self):
        """Independent Lik on a duplicated tree; no cached CLs."""
        ret = Lik(lib=self.lib, precision=self.precision, dropin=self.dropin)
        tree = self.tree.dup()
        ret._init0(tree)
        ret._init1(tree, self.lik.nchars, self.lik.dim, 0)
        ret._init2(self.alignment, self.char_)
        self._dup(ret)
        return ret

    def clone(self):
        """Mate Lik with the other CL polarity, sharing the tree."""
        if self.mate is not None:
            ret = self.mate
            ret.lik.invalidate = True
            resize = len(ret._comps) != len(self._comps)
            for i in range(len(ret._models) - 1, -1, -1):
                ret.delModel(i)
        else:
            assert self.lik.polarity == 0
            resize = False
            ret = Lik(lib=self.lib, precision=self.precision,
                      dropin=self.dropin)
            ret._init1(self.tree, self.lik.nchars, self.lik.dim, 1)
            ret._init2(self.alignment, self.char_)
            ret.mate = weakref.proxy(self)
            self.mate = ret
        self._dup(ret)
        ret.lik.resize = resize
        ret.lik.reweight = True
        return ret

    # -- planning (Lik.pyx:1395-1601) ----------------------------------------
    def _planAppend(self, variant, ntrail, parentCL, childCL, edgeLen):
        # Steps are collected here and written into the CxtLikStep array by
        # _flushSteps at the end of _plan.
        assert ntrail != 0 or variant in (_abi.MergeL, _abi.MergeI)
        pol = self._pol
        if childCL.bufs[1] is None:
            assert childCL.bufs[0] is not None
            child = childCL.addr[0]
        else:
            child = childCL.addr[pol]
        if edgeLen < 0.0:
            raise ValueError("Negative branch length")
        self._pending.append((variant, ntrail, parentCL.addr[pol], child,
                              edgeLen))
        self._plan_refs.append((parentCL, childCL))

    def _flushSteps(self):
        L = self.lik
        n = len(self._pending)
        if n:
            view = np.frombuffer(self._steps, dtype=_abi.STEP_DTYPE)
            view[L.stepsLen:L.stepsLen + n] = np.array(self._pending,
                                                        dtype=_abi.STEP_DTYPE)
            L.stepsLen += n
        self._pending = []

    def _leafInit(self, ring):
        L = self.lik
        taxon = ring.node.taxon
        if taxon is None:
            raise ValueError("Leaf node missing taxon")
        cl = CL(self.lib, self.device)
        cl.leaf = True
        cl.prepare(0, L.mschars, L.dim, 1)
        ind = self.alignment.taxaMap.indGet(taxon)
        if ind == -1:
            raise ValueError("Taxon %r missing from alignment's taxa map"
                             % taxon)
        row = self.alignment.getRow(ind)[L.cbase:L.cbase + L.mschars]
        vals = self.char_.val_table[row]
        if (vals < 0).any():
            bad = row[vals < 0][0]
            raise ValueError("State not defined: %r" % chr(bad))
        vals = np.where(vals == 0, self.char_.any, vals)
        if self.device:
            masks = np.ascontiguousarray(vals, dtype=np.uint8)
            rc = self.lib.cxgLikClSetLeafMasks(
                ctypes.pointer(cl.c[0]),
                masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                L.mschars)
            if rc != 0:
                raise _native.error(self.lib, rc, "cxgLikClSetLeafMasks")
        else:
            mat = cl.bufs[0][0].reshape(L.mschars, L.dim)
            for j in range(L.dim):
                mat[:, j] = ((vals >> j) & 1).astype(np.float64)
            cl.bufs[0][1][:] = 0.0
        ring.aux = cl
        return cl

    def _planRecurse(self, ring, parent, nSibs, edgeLen):
        # self._pol, self._inval, self._resize and self._dims are the
        # polarity, invalidate and resize flags and the CL shape, read from
        # the CxtLik once per plan by _plan (they do not change during it).
        pol = self._pol
        inval = self._inval
        cL = ring.aux
        degree = ring.node.getDegree()
        if degree == 1:
            if cL is None:
                cL = self._leafInit(ring)
        else:
            if cL is None:
                cL = CL(self.lib, self.device)
                cL.prepare(pol, *self._dims)
                ring.aux = cL
            elif self._resize:
                cL.resize(pol, *self._dims)
            elif cL.bufs[pol] is None:
                cL.prepare(pol, *self._dims)

        r = ring.next
        while r is not ring:
            nxt = r.next
            if inval:
                f = r.aux
                if f is not None:
                    f.flush(pol)
            self._planRecurse(r.other, cL, degree, r.edge.length)
            r = nxt

        if inval or cL.parent[pol] is not parent \
                or cL.nSibs[pol] != nSibs or cL.edgeLen[pol] != edgeLen:
            parent.valid[pol] = False
            # The struct fields follow the mirrors; a full re-plan of an
            # unchanged tree writes none of them.
            cLC = cL.c[pol]
            if cL.parent[pol] is not parent:
                cL.parent[pol] = parent
                cLC.parent = parent.ptr[pol]
            if cL.nSibs[pol] != nSibs:
                cL.nSibs[pol] = nSibs
                cLC.nSibs = nSibs
            if cL.edgeLen[pol] != edgeLen:
                cL.edgeLen[pol] = edgeLen
                cLC.edgeLen = edgeLen

        if degree != 1:
            if inval or not cL.valid[pol]:
                r = ring.next
                for j in range(1, degree):
                    if r.other.node.getDegree() > 1:
                        variant = _abi.ComputeI if j == 1 else _abi.MergeI
                    else:
                        variant = _abi.ComputeL if j == 1 else _abi.MergeL
                    self._planAppend(variant, degree - j - 1, cL, r.other.aux,
                                     r.edge.length)
                    r = r.next
                cL.valid[pol] = True
                parent.valid[pol] = False
        self._touched.append(cL)

    # -- native planner (cxgPlanSnapRun) ---------------------------------------
    # The recursion above runs once per topology, root and set of CL buffers;
    # _snapBuild then flattens the traversal it took, and later plans of the
    # same traversal run natively.  Every rule (what is dirty, which steps,
    # which struct fields change) is the one _planRecurse applies.
    native_plan = True

    def _snapBuild(self, root, key):
        pol = self._pol
        vis = []          # (CL, parent CL, nSibs, edge index, kids or None)
        opp = []          # CLs an invalidating plan would flush
        edges, eidx = [], {}
        ok = [True]

        def eid(e):
            if e is None:
                return -1
            i = eidx.get(id(e))
            if i is None:
                i = eidx[id(e)] = len(edges)
                edges.append(e)
            return i

        def kid(r, internal=None):
            c = r.other.aux
            addr = c.addr[0] if c.bufs[1] is None else c.addr[pol]
            if internal is None:
                internal = r.other.node.getDegree() > 1
            return (addr, internal, eid(r.edge))

        def rec(ring, parent, nSibs, edge):
            cL = ring.aux
            degree = ring.node.getDegree()
            if cL is None or degree == 2 or \
                    (degree != 1 and cL.bufs[pol] is None):
                ok[0] = False
                return
            r = ring.next
            while r is not ring:
                if r.aux is not None:
                    opp.append(r.aux)
                rec(r.other, cL, degree, r.edge)
                if not ok[0]:
                    return
                r = r.next
            kids = None
            if degree != 1:
                kids = []
                r = ring.next
                for _ in range(1, degree):
                    kids.append(kid(r))
                    r = r.next
            vis.append((cL, parent, nSibs, eid(edge), kids))

        degree = root.getDegree()
        ring = root.ring
        if degree == 1:
            rec(ring.other, self.rootCL, 2, ring.edge)
            if ok[0]:
                rec(ring, self.rootCL, 2, None)
            if ok[0]:
                c = ring.aux
                leaf = (c.addr[0] if c.bufs[1] is None else c.addr[pol],
                        False, -1)
                rkids = [kid(ring), leaf]
        else:
            for r in ring:
                if r.aux is not None:
                    opp.append(r.aux)
                rec(r.other, self.rootCL, degree, r.edge)
                if not ok[0]:
                    break
            if ok[0]:
                rkids = [kid(r) for r in ring]
        if not ok[0]:
            return None
        vis.append((self.rootCL, None, 0, -1, rkids))
        index = {id(v[0]): i for i, v in enumerate(vis)}
        if len(index) != len(vis):
            return None
        n = len(vis)
        sn = _Snap()
        sn.key = key
        sn.objs = [v[0] for v in vis]
        sn.up_obj = [v[1] for v in vis]
        sn.edges = edges
        sn.opp_clean = all(
            f.bufs[pol] is None and not f.valid[pol] and not f.cvalid[pol]
            and f.parent[pol] is None for f in opp)
        u32, i32 = np.uint32, np.int32
        sn.cl = np.array([v[0].addr[pol] for v in vis], dtype=np.uint64)
        sn.up = np.array([-1 if v[1] is None else index[id(v[1])]
                          for v in vis], dtype=i32)
        sn.nsibs = np.array([v[2] for v in vis], dtype=u32)
        sn.edge = np.array([v[3] for v in vis], dtype=i32)
        kids = [v[4] or [] for v in vis]
        sn.nkids = np.array([len(k) for k in kids], dtype=u32)
        sn.kid0 = np.zeros(n, dtype=u32)
        if n > 1:
            sn.kid0[1:] = np.cumsum(sn.nkids[:-1])
        flat = [k for ks in kids for k in ks]
        sn.kid_cl = np.array([k[0] for k in flat], dtype=np.uint64)
        sn.kid_int = np.array([1 if k[1] else 0 for k in flat], dtype=np.uint8)
        sn.kid_edge = np.array([k[2] for k in flat], dtype=i32)
        sn.valid = np.array([v[0].valid[pol] for v in vis], dtype=np.uint8)
        sn.cvalid = np.array([v[0].cvalid[pol] for v in vis], dtype=np.uint8)
        sn.m_parent = np.array(
            [0 if v[0].parent[pol] is None else v[0].parent[pol].addr[pol]
             for v in vis], dtype=np.uint64)
        sn.m_nsibs = np.array([v[0].nSibs[pol] for v in vis], dtype=u32)
        sn.m_elen = np.array([v[0].edgeLen[pol] for v in vis],
                             dtype=np.float64)
        sn.lens = np.zeros(max(len(edges), 1), dtype=np.float64)
        # Packs the edges' lengths into sn.lens in one C loop (a numpy slice
        # assignment from a list converts element by element).
        sn.lens_pack = struct.Struct("%dd" % len(edges)).pack_into
        sn.changed = np.zeros(n, dtype=u32)
        c = sn.c = _abi.CxgPlanSnap()
        c.nvis = n
        c.nkid = len(flat)
        for f in ("cl", "up", "nsibs", "edge", "kid0", "nkids", "kid_cl",
                  "kid_int", "kid_edge", "valid", "cvalid", "m_parent",
                  "m_nsibs", "m_elen"):
            setattr(c, f, getattr(sn, f).ctypes.data)
        sn.cref = ctypes.byref(c)
        sn.lens_p = _abi.dptr(sn.lens)
        sn.nsteps = ctypes.c_uint32()
        sn.nchanged = ctypes.c_uint32()
        sn.nsteps_p = ctypes.byref(sn.nsteps)
        sn.nchanged_p = ctypes.byref(sn.nchanged)
        sn.changed_p = sn.changed.ctypes.data_as(
            ctypes.POINTER(ctypes.c_uint32))
        return sn

    def _snapSync(self, sn, idx):
        """Copy the native mirrors of visits `idx` into the CL objects."""
        pol = self._pol
        for v in idx:
            cl = sn.objs[v]
            cl.valid[pol] = bool(sn.valid[v])
            cl.cvalid[pol] = bool(sn.cvalid[v])
            cl.nSibs[pol] = int(sn.m_nsibs[v])
            cl.edgeLen[pol] = float(sn.m_elen[v])
            if sn.up_obj[v] is not None and \
                    sn.m_parent[v] == sn.up_obj[v].addr[pol]:
                cl.parent[pol] = sn.up_obj[v]

    def _nativePlan(self, root):
        """Plan natively if this Lik's traversal is unchanged since the last
        plan; False when the Python planner must run."""
        L = self.lik
        if not self.native_plan or L.resize:
            return False
        key = (self.tree.sn, _epoch[0], self._pol, root)
        sn = self._snap
        if sn is None or sn.key != key:
            if self._pyKey != key:
                return False
            lib = planner_library()
            if lib is None:
                return False
            sn = self._snapBuild(root, key)
            self._pyKey = None
            if sn is None:
                return False
            sn.lib = lib
            self._snap = sn
        inval = bool(L.invalidate)
        if inval and not sn.opp_clean:
            return False
        sn.lens_pack(sn.lens, 0, *[e.length for e in sn.edges])
        rc = sn.lib.cxgPlanSnapRun(sn.cref, sn.lens_p, inval, self._steps,
                                   L.stepsMax, sn.nsteps_p, sn.changed_p,
                                   sn.nchanged_p)
        nc = sn.nchanged.value
        if nc:
            self._snapSync(sn, sn.changed[:nc].tolist())
        if rc != 0:
            self._snap = None
            self._snapSync(sn, range(len(sn.objs)))
            if rc == 1:
                raise ValueError("Negative branch length")
            raise RuntimeError("cxgPlanSnapRun: %s"
                               % sn.lib.cxgLastError().decode())
        L.stepsLen = sn.nsteps.value
        self._plan_refs = sn.objs
        L.resize = False
        L.invalidate = False
        return True

    def _plan(self, root):
        L = self.lik
        pol = L.polarity
        self._pol = pol
        self._pending = []
        self._touched = [self.rootCL]
        self._inval = bool(L.invalidate)
        self._resize = bool(L.resize)
        self._dims = (L.mschars, L.dim, L.compsLen)
        if L.resize:
            self.rootCL.resize(pol, L.mschars, L.dim, L.compsLen)
        else:
            self.rootCL.prepare(pol, L.mschars, L.dim, L.compsLen)
        L.rootCLC = self.rootCL.ptr[pol]
        if root is None:
            root = self.tree.base
        if self._nativePlan(root):
            return
        self._snap = None
        self._planPython(root)
        self._pyKey = (self.tree.sn, _epoch[0], pol, root)

    def _planPython(self, root):
        L = self.lik
        pol = self._pol
        degree = root.getDegree()
        ring = root.ring
        if degree == 1:
            self._planRecurse(ring.other, self.rootCL, 2, ring.edge.length)
            self._planRecurse(ring, self.rootCL, 2, 0.0)
            if L.invalidate or not self.rootCL.valid[pol]:
                variant = (_abi.ComputeI if ring.other.node.getDegree() > 1
                           else _abi.ComputeL)
                self._planAppend(variant, 1, self.rootCL, ring.other.aux,
                                 ring.edge.length)
                self._planAppend(_abi.MergeL, 0, self.rootCL, ring.aux, 0.0)
                self.rootCL.set_valid(pol, True)
        else:
            for r in ring:
                if L.invalidate:
                    f = r.aux
                    if f is not None:
                        f.flush(pol)
                self._planRecurse(r.other, self.rootCL, degree, r.edge.length)
            if L.invalidate or not self.rootCL.valid[pol]:
                variant = (_abi.ComputeI if ring.other.node.getDegree() > 1
                           else _abi.ComputeL)
                ntrail = degree - 1
                self._planAppend(variant, ntrail, self.rootCL, ring.other.aux,
                                 ring.edge.length)
                for r in ring.siblings():
                    variant = (_abi.MergeI if r.other.node.getDegree() > 1
                               else _abi.MergeL)
                    ntrail -= 1
                    self._planAppend(variant, ntrail, self.rootCL,
                                     r.other.aux, r.edge.length)
                self.rootCL.set_valid(pol, True)
        self._flushSteps()
        for cl in self._touched:
            cl.sync_valid(pol)
        self._touched = []
        L.resize = False
        L.invalidate = False

    # -- preparation (Lik.pyx:1603-1685) -------------------------------------
    def prep(self):
        L = self.lik
        if len(self._models) == 0:
            raise ValueError("Empty model mixture")
        if L.resize:
            L.reweight = True
        if L.reweight:
            wsum = sum(m.s.weight for m in self._models)
            if wsum == 0.0:
                raise ValueError("At least one model must have non-zero "
                                 "weight")
            for m in self._models:
                comps = self._comps[m.comp0:m.comp0 + m.clen]
                wsumc = sum(c["cweight"] for c in comps)
                assert wsumc > 0.0
                for c in comps:
                    c["weightScaled"] = (m.s.weight / wsum) * \
                        (c["cweight"] / wsumc)
            L.invalidate = True
            L.reweight = False
        for m in self._models:
            if m.s.decomp:
                self._decompModel(m)
        qmean = 0.0
        for c in self._comps:
            if c["weightScaled"] != 0.0 and c["cmult"] != 0.0:
                m = c["model"]
                qmean += c["weightScaled"] * (m.s.rmult / m.s.qNorm)
        wnorm = 1.0 / qmean if qmean != 0.0 else math.inf
        if wnorm != L.wNorm:
            L.invalidate = True
            L.wNorm = wnorm
        self._sync_comps()

    def _decompModel(self, m):
        qnorm = ctypes.c_double()
        if self.lib.CxLikQDecomp(self.lik.dim, _abi.dptr(m.rTri),
                                 _abi.dptr(m.piDiag), _abi.dptr(m.piDiagNorm),
                                 ctypes.byref(qnorm), _abi.dptr(m.cube),
                                 _abi.dptr(m.eig)):
            raise ValueError("Error decomposing Q")
        m.s.qNorm = qnorm.value
        m.s.decomp = False

    def _prep(self, root):
        self.prep()
        L = self.lik
        stepsMax = 2 * self.alignment.ntaxa - 2
        if L.stepsMax < stepsMax:
            self._steps = (_abi.CxtLikStep * stepsMax)()
            L.steps = ctypes.cast(self._steps,
                                  ctypes.POINTER(_abi.CxtLikStep))
            L.stepsMax = stepsMax
        L.stepsLen = 0
        self._plan_refs = []
        self._plan(root)

    # -- evaluation (Lik.pyx:1687-1763) ---------------------------------------
    def _precision_code(self):
        return 1 if self.precision == "fp32" else 0

    def _failed(self, rc):
        """The exception for a failed evaluation.  The plan marked its CLs
        valid before the run, which did not complete (an allocation failed,
        or a bounded device wait gave up), so the next plan recomputes
        every CL."""
        self.lik.invalidate = True
        return _native.error(self.lib, rc, "cxgLikExecuteLnL")

    def lnL(self, root=None):
        """Log-likelihood, rooted at `root` (default: the tree's base)."""
        self._prep(root)
        if self.device:
            out = ctypes.c_double()
            rc = self.lib.cxgLikExecuteLnL(ctypes.byref(self.lik),
                                           self._precision_code(),
                                           ctypes.byref(out), None)
            if rc != 0:
                raise self._failed(rc)
            return out.value
        self.lib.CxLikExecute(ctypes.byref(self.lik))
        ret = 0.0
        for i in range(self.lik.nstripes):
            ret += self.stripeLnLBuf[i]
        return ret

    def siteLnLs(self, root=None):
        """Per-site lnL (pad sites excluded)."""
        self._prep(root)
        if self.device:
            out = ctypes.c_double()
            rc = self.lib.cxgLikExecuteLnL(ctypes.byref(self.lik),
                                           self._precision_code(),
                                           ctypes.byref(out),
                                           _abi.dptr(self.siteLnLBuf))
            if rc != 0:
                raise self._failed(rc)
        else:
            self.lib.CxLikExecute(ctypes.byref(self.lik))
        n = self.lik.nchars - self.lik.npad
        return [float(x) for x in self.siteLnLBuf[:n]]

    def execute_dropin(self, root=None):
        """Plan, then run the library's drop-in CxLikExecute; return the
        stripe sum the way Lik.lnL does (Lik.pyx:1697-1712)."""
        self._prep(root)
        self.lib.CxLikExecute(ctypes.byref(self.lik))
        ret = 0.0
        for i in range(self.lik.nstripes):
            ret += self.stripeLnLBuf[i]
        return ret

    def prepare_plan(self, root=None, full=True):
        """Plan without executing (for plans and batches run elsewhere);
        `full` re-plans every CL, as after a model change."""
        if full:
            self.lik.invalidate = True
        self._prep(root)
        return self.lik.stepsLen

    def flush(self):
        """Drop all cached CLs of this polarity (Lik.pyx:1765-1787)."""
        pol = self.lik.polarity
        for e in self.tree.edges:
            for ring in (e.ring, e.ring.other):
                if ring.node.getDegree() > 1 and ring.aux is not None:
                    ring.aux.flush(pol)

    @property
    def nsteps(self):
        return self.lik.stepsLen

    def steps(self):
        """The current plan as (variant, ntrail, edgeLen) tuples."""
        return [(self._steps[i].variant, self._steps[i].ntrail,
                 self._steps[i].edgeLen) for i in range(self.lik.stepsLen)]
