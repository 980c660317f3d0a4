"""Character codes, taxa, FASTA matrices and pattern-compressed alignments.

Host-side restatement of the data model the likelihood consumes:

* ``Dna``: state bitmasks A=1, C=2, G=4, T=8, IUPAC ambiguities, ``-`` = 0
  and the lower-case/RNA aliases (pkg/Crux/Character.pyx:129-185).
* ``TaxaMap``: taxon label <-> row index (pkg/Crux/Taxa.pyx:64-129).
* ``CTMatrix``: FASTA text -> per-taxon sequences, taxa in order of first
  appearance (pkg/Crux/Fasta.pyx:66-96, 179-223).
* ``Alignment``: row-major uint8 matrix plus uint32 column frequencies with
  ``pad`` (CTMatrix.pyx:610-662), ``canonize`` (856-887) and ``compact``
  (949-1031): columns are canonicalised, sorted bytewise and equal columns
  merged with summed frequencies, which is the order a Python-2 sort of
  ``[column string, freq]`` pairs produces; the Fitch variants
  (``_fitchCanonize`` :785-854, ``_fitchCompact`` :890-947) and ``render``
  (:1040-1145), whose text the reference's own compaction tests print.
"""
import re

import numpy as np


class Character:
    """State-code table: code -> bitmask value, value -> primary code."""

    def __init__(self, states, ambiguities, aliases):
        self.any = 0
        self.nstates = len(states)
        self._val = {}
        self._code = {}
        for i, s in enumerate(states):
            v = 1 << i
            self._val[s] = v
            self._code.setdefault(v, s)
            self.any |= v
        for code, members in ambiguities:
            v = 0
            for m in members:
                v |= self._val[m]
            self._val[code] = v
            self._code.setdefault(v, code)
        for code, target in aliases:
            v = self._val[target]
            self._val[code] = v
            self._code.setdefault(v, code)
        # Byte -> value and byte -> canonical byte tables.
        self.val_table = np.full(256, -1, dtype=np.int32)
        self.canon_table = np.arange(256, dtype=np.uint8)
        for code, v in self._val.items():
            self.val_table[ord(code)] = v
            self.canon_table[ord(code)] = ord(self._code[v])

    def codes(self):
        return list(self._val.keys())

    def pcodes(self):
        return [self._code[1 << i] for i in range(self.nstates)]

    def code2val(self, code):
        if code not in self._val:
            raise ValueError("State not defined: %r" % code)
        return self._val[code]

    def val2code(self, val):
        if val not in self._code:
            raise ValueError("Value not defined: %r" % val)
        return self._code[val]


_DNA = None
_PROTEIN = None


class Dna:
    """Singleton DNA/RNA code table (Character.pyx:129-185)."""

    @staticmethod
    def get():
        global _DNA
        if _DNA is None:
            _DNA = Character(
                ["A", "C", "G", "T"],
                [("K", "GT"), ("Y", "CT"), ("S", "CG"), ("B", "CGT"),
                 ("W", "AT"), ("R", "AG"), ("D", "AGT"), ("M", "AC"),
                 ("H", "ACT"), ("V", "ACG"), ("N", "ACGT"), ("-", "")],
                [("U", "T"), ("u", "T"), ("t", "T"), ("g", "G"), ("k", "K"),
                 ("c", "C"), ("y", "Y"), ("s", "S"), ("b", "B"), ("a", "A"),
                 ("w", "W"), ("r", "R"), ("d", "D"), ("m", "M"), ("h", "H"),
                 ("v", "V"), ("n", "N"), ("?", "N"), (".", "-")])
        return _DNA


class Protein:
    """Singleton amino-acid code table (Character.pyx:190-254)."""

    @staticmethod
    def get():
        global _PROTEIN
        if _PROTEIN is None:
            st = list("ACDEFGHIKLMNPQRSTUVWY*")
            lower = [(c.lower(), c) for c in "ABCDEFGHIKLMNPQRSTUVWXYZ"]
            _PROTEIN = Character(
                st, [("B", "DN"), ("Z", "EQ"), ("X", "".join(st)), ("-", "")],
                lower + [("?", "X"), (".", "-")])
        return _PROTEIN


class TaxaMap:
    """Ordered taxon labels with index lookup (Taxa.pyx:64-129)."""

    def __init__(self, taxa=None):
        self._ind = {}
        self._tax = []
        for t in taxa or []:
            self.map(t)

    def map(self, label, ind=None):
        if label in self._ind:
            raise ValueError("Taxon %r already mapped" % label)
        self._ind[label] = len(self._tax)
        self._tax.append(label)

    @property
    def ntaxa(self):
        return len(self._tax)

    @property
    def taxa(self):
        return list(self._tax)

    def indGet(self, label):
        return self._ind.get(label, -1)

    def taxonGet(self, ind):
        return self._tax[ind] if 0 <= ind < len(self._tax) else None


class CTMatrix:
    """Per-taxon character strings parsed from FASTA text."""

    def __init__(self, fasta=None, charType=Dna):
        self.charType = charType
        self.taxaMap = TaxaMap()
        self._data = {}
        if fasta is not None:
            self._parse(fasta)

    def _parse(self, text):
        label = None
        chunks = []

        def flush():
            if label is not None:
                if self.taxaMap.indGet(label) == -1:
                    self.taxaMap.map(label)
                self._data[label] = "".join(chunks)

        for line in text.splitlines():
            if line.startswith(">"):
                flush()
                m = re.match(r">(\S+)", line)
                if m is None:
                    raise SyntaxError("Invalid FASTA description: %r" % line)
                label = m.group(1).replace("_", " ")
                chunks = []
            elif line.strip() == "":
                continue
            else:
                if label is None:
                    raise SyntaxError("Characters before first description")
                chunks.append(re.sub(r"[ \t\r\n]+", "", line))
        flush()

    def dataGet(self, label):
        return self._data.get(label)

    def dataSet(self, label, data):
        if self.taxaMap.indGet(label) == -1:
            self.taxaMap.map(label)
        self._data[label] = data


class Alignment:
    """Row-major alignment with per-column frequencies.

    ``rows`` is a uint8 array [ntaxa, nchars] of character codes and
    ``freqs`` a uint32 array [nchars].
    """

    def __init__(self, matrix=None, taxaMap=None, nchars=-1, charType=Dna,
                 rows=None):
        if matrix is not None:
            self.charType = matrix.charType
            self.taxaMap = TaxaMap(matrix.taxaMap.taxa)
            seqs = [matrix.dataGet(t) for t in self.taxaMap.taxa]
            n = len(seqs[0])
            if n == 0:
                raise ValueError("Invalid alignment size: %dx0" % len(seqs))
            for s in seqs:
                if len(s) != n:
                    raise ValueError("Inconsistent sequence lengths (%d vs. %d)"
                                     % (n, len(s)))
            self.rows = np.frombuffer("".join(seqs).encode("ascii"),
                                      dtype=np.uint8).reshape(len(seqs), n).copy()
        else:
            if taxaMap is None:
                raise ValueError("Specify matrix or taxaMap")
            self.charType = charType
            self.taxaMap = TaxaMap(taxaMap.taxa)
            if rows is not None:
                self.rows = np.ascontiguousarray(rows, dtype=np.uint8)
            else:
                if nchars <= 0:
                    raise ValueError("Invalid alignment size")
                self.rows = np.full((self.taxaMap.ntaxa, nchars), ord("-"),
                                    dtype=np.uint8)
        self.freqs = np.ones(self.rows.shape[1], dtype=np.uint32)
        self.npad = 0

    @property
    def ntaxa(self):
        return self.rows.shape[0]

    @property
    def nchars(self):
        return self.rows.shape[1]

    def getRow(self, ind):
        return self.rows[ind]

    def getSeq(self, ind):
        return self.rows[ind].tobytes().decode("ascii")

    def setSeq(self, ind, col, chars):
        b = np.frombuffer(chars.encode("ascii"), dtype=np.uint8)
        self.rows[ind, col:col + len(b)] = b

    def getChar(self, col):
        return self.rows[:, col].tobytes().decode("ascii")

    def pad(self, code, npad):
        """Append npad columns of `code` with frequency 1 (CTMatrix.pyx:610)."""
        assert npad > 0
        extra = np.full((self.ntaxa, npad), ord(code), dtype=np.uint8)
        self.rows = np.ascontiguousarray(np.concatenate([self.rows, extra], 1))
        self.freqs = np.concatenate([self.freqs,
                                     np.ones(npad, dtype=np.uint32)])
        self.npad += npad

    def canonize(self, fitch=False):
        """Map aliases to primary codes (CTMatrix.pyx:856-887).

        With ``fitch``, also relabel each column's states in order of first
        appearance down the column (``_fitchCanonize``, :785-854), so that
        columns equal up to a renaming of states become equal.
        """
        self.rows = self.charType.get().canon_table[self.rows]
        if fitch:
            self._fitch_canonize()

    @staticmethod
    def _bits(v):
        """State indices of bitmask `v`, lowest first (the ffs order)."""
        out = []
        while v:
            low = v & -v
            out.append(low.bit_length() - 1)
            v ^= low
        return out

    def _fitch_canonize(self):
        ch = self.charType.get()
        n = ch.nstates
        codes = ch.codes()
        for j in range(self.nchars):
            col = self.rows[:, j]
            ftrans = [-1] * n
            seen = 0
            for b in col:
                if seen == n:
                    break
                for bit in self._bits(int(ch.val_table[b])):
                    if ftrans[bit] == -1:
                        ftrans[bit] = 1 << seen
                        seen += 1
                        if seen == n:
                            break
            i = 0
            while seen < n:
                if ftrans[i] == -1:
                    ftrans[i] = 1 << seen
                    seen += 1
                i += 1
            trans = np.arange(256, dtype=np.uint8)
            for code in codes:
                r = 0
                for bit in self._bits(ch.code2val(code)):
                    r |= ftrans[bit]
                trans[ord(code)] = ord(ch.val2code(r))
            self.rows[:, j] = trans[col]

    def _fitch_informative(self, col):
        """(informative, states seen) of one column (CTMatrix.pyx:890-947):
        more than two states, or two states that each occur twice."""
        ch = self.charType.get()
        n = ch.nstates
        freqs = [0] * n
        seen = 0
        for b in col:
            for bit in self._bits(int(ch.val_table[b])):
                freqs[bit] += 1
                if freqs[bit] == 1:
                    seen += 1
                    if seen > 2:
                        return True, seen
        if seen == 2:
            mult = 0
            for i in range(n):
                if mult >= 2:
                    break
                if freqs[i] != 0:
                    if freqs[i] == 1:
                        break
                    mult += 1
            if mult == 2:
                return True, seen
        return False, seen

    def compact(self, fitch=False):
        """Merge identical columns, sorted bytewise (CTMatrix.pyx:949-1031).

        With ``fitch``, the columns are Fitch-canonized first and
        parsimony-uninformative patterns are dropped afterwards; the return
        value is then the number of changes dropped (one per unit of
        frequency of each dropped two-state pattern), else 0.
        """
        self.canonize(fitch)
        cols = np.ascontiguousarray(self.rows.T)
        key = cols.view(np.dtype((np.void, cols.shape[1]))).ravel()
        order = np.argsort(key, kind="stable")
        skey = key[order]
        first = np.ones(len(skey), dtype=bool)
        first[1:] = skey[1:] != skey[:-1]
        group = np.cumsum(first) - 1
        freqs = np.zeros(int(first.sum()), dtype=np.uint64)
        np.add.at(freqs, group, self.freqs[order].astype(np.uint64))
        ucols = cols[order[first]]
        freqs = freqs.astype(np.uint32)
        ret = 0
        if fitch:
            keep = np.zeros(len(ucols), dtype=bool)
            for j, col in enumerate(ucols):
                informative, seen = self._fitch_informative(col)
                keep[j] = informative
                if not informative and seen == 2:
                    ret += int(freqs[j])
            ucols, freqs = ucols[keep], freqs[keep]
        self.rows = np.ascontiguousarray(ucols.T).reshape(self.ntaxa,
                                                          len(ucols))
        self.freqs = freqs
        return ret

    def render(self, interleave=50, pad=False):
        """Human-readable alignment with site frequencies, as
        ``Alignment.render`` prints it (CTMatrix.pyx:1040-1145): blocks of
        `interleave` columns (rounded up to a multiple of 5; 0 = one
        block), a frequency line (``(f)`` for f >= 10), ``=`` rules and
        column offsets.  Padding columns are shown only with ``pad``."""
        taxa = self.taxaMap.taxa
        nchars = self.nchars if pad else self.nchars - self.npad
        lines = []
        if nchars > 0:
            w = max(len(t) for t in taxa)
            if interleave == 0:
                interleave = nchars
            elif interleave % 5 != 0:
                interleave += 5 - interleave % 5
            seqs = [self.getSeq(k) for k in range(len(taxa))]
            if not pad and self.npad > 0:
                seqs = [s[:-self.npad] for s in seqs]
            for i in range(0, nchars, interleave):
                lim = min(i + interleave, nchars)
                if i > 0:
                    lines.append("\n")
                head = ["%-*s" % (w, "")]
                for j in range(i, lim):
                    if j % 5 == 0:
                        head.append(" ")
                    f = int(self.freqs[j])
                    head.append("%d" % f if f < 10 else "(%d)" % f)
                lines.append("".join(head) + "\n")
                rule = "%-*s " % (w, "") + "=" * ((lim - i) + (lim - 1 - i) // 5)
                lines.append(rule + "\n")
                for label, seq in zip(taxa, seqs):
                    lines.append("%-*s" % (w, label) + "".join(
                        " %s" % seq[j:j + 5] for j in range(i, lim, 5)) + "\n")
                lines.append(rule + "\n")
                offs = "%-*s " % (w, "") + "".join(
                    "%-6d" % j for j in range(i, lim, 5))
                lines.append(offs.rstrip() + "\n")
        else:
            for label in taxa:
                lines.append("%s\n" % label)
        text = "".join(lines)
        return text[:-1] if text.endswith("\n") else text
