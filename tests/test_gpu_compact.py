"""Pattern compression on the GPU is bit-exact with Alignment.compact (the
host restatement of CTMatrix.pyx:949-1031): the same sorted unique columns
and summed frequencies, including ambiguity codes, aliases (lower case, U,
'?', '.'), gaps, many duplicate columns, one taxon, one site and wide
alignments; the leaf-tip masks equal the value table (0 -> all states)."""
import numpy as np
import pytest

from crux_gb300 import compact as gc
from crux_gb300.alignment import Alignment, Dna, TaxaMap

pytestmark = pytest.mark.gpu

CODES = np.frombuffer(b"ACGTACGTACGTNRY-acgtuU?.KMSWBDHV", dtype=np.uint8)


def random_alignment(rng, ntaxa, nsites, pool=None, codes=CODES):
    if pool:
        base = rng.choice(codes, size=(ntaxa, pool))
        rows = base[:, rng.integers(pool, size=nsites)]
    else:
        rows = rng.choice(codes, size=(ntaxa, nsites))
    aln = Alignment(taxaMap=TaxaMap(["t%d" % i for i in range(ntaxa)]),
                    rows=rows)
    aln.freqs = rng.integers(1, 4, size=nsites).astype(np.uint32)
    return aln


def host_compact(aln):
    h = Alignment(taxaMap=aln.taxaMap, rows=aln.rows.copy())
    h.freqs = aln.freqs.copy()
    h.compact()
    return h


@pytest.mark.parametrize("ntaxa,nsites,pool", [
    (1, 1, None), (1, 40, 5), (3, 1, None), (8, 300, 20), (16, 5000, None),
    (64, 20000, 900), (300, 3000, 50), (1030, 2000, 400)])
def test_compact_matches_host(gpu, ntaxa, nsites, pool):
    rng = np.random.default_rng(ntaxa * 1000 + nsites)
    aln = random_alignment(rng, ntaxa, nsites, pool)
    want = host_compact(aln)
    rows, freqs, masks = gc.compact(aln, gpu)
    assert rows.shape == want.rows.shape
    assert np.array_equal(rows, want.rows)
    assert np.array_equal(freqs, want.freqs)
    ch = Dna.get()
    v = ch.val_table[want.rows]
    assert np.array_equal(masks, np.where(v == 0, ch.any, v).astype(np.uint8))


def test_compact_dna_only_and_identical_columns(gpu):
    rng = np.random.default_rng(3)
    aln = random_alignment(rng, 40, 10000, pool=1,
                           codes=np.frombuffer(b"ACGT", dtype=np.uint8))
    rows, freqs, _ = gc.compact(aln, gpu)
    assert rows.shape == (40, 1) and freqs[0] == aln.freqs.sum()
    aln2 = random_alignment(rng, 24, 6000, codes=np.frombuffer(b"ACGT", dtype=np.uint8))
    want = host_compact(aln2)
    rows2, freqs2, _ = gc.compact(aln2, gpu)
    assert np.array_equal(rows2, want.rows) and np.array_equal(freqs2, want.freqs)


def test_compact_alignment_feeds_the_likelihood(gpu, port):
    """A GPU-compacted alignment gives the same lnL as a host-compacted one."""
    from crux_gb300 import synth
    case = synth.Case(20, 3000, 0.1, 44, gap_frac=0.01)
    a_host = case.alignment()
    from crux_gb300.alignment import CTMatrix
    a_gpu = Alignment(CTMatrix(case.fasta))
    gc.compact_alignment(a_gpu, gpu)
    assert np.array_equal(a_gpu.rows, a_host.rows)
    assert np.array_equal(a_gpu.freqs, a_host.freqs)
    assert case.lik(lib=port, alignment=a_gpu).lnL() == \
        case.lik(lib=port, alignment=a_host).lnL()


def _kat():
    import json
    import os
    return json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                       "compaction_kat.json")))


def test_compact_matches_reference_kats(gpu):
    """cxgCompact prints the reference's own compaction answers byte for
    byte: rinehart.fasta (test/Alignment_a.cx.exp) and the "# Compact"
    blocks of test/CTMatrix_e.cx.exp, then pads as the reference does."""
    from crux_gb300.alignment import CTMatrix
    kat = _kat()
    aln = Alignment(CTMatrix(kat["rinehart_fasta"]))
    gc.compact_alignment(aln, gpu)
    assert aln.render() == kat["alignment_a"]
    for case in kat["ctmatrix_e"]:
        aln = Alignment(CTMatrix(case["fasta"]))
        rows, freqs, masks = gc.compact(aln, gpu)
        want = host_compact(aln)
        assert np.array_equal(rows, want.rows)
        assert np.array_equal(freqs, want.freqs)
        aln.rows, aln.freqs = np.ascontiguousarray(rows), freqs
        assert aln.render(pad=True) == case["Compact"]
        aln.pad("-", 4)
        assert aln.render() == case["Compact"]
