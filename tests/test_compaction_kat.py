"""Pattern compression against the reference's own known answers.

The fixture ``tests/golden/compaction_kat.json`` holds the reference's
test inputs and printed outputs (written by ``make_compaction_kat.py``):
``test/Alignment_a.cx`` compacts ``rinehart.fasta`` (22 taxa, 327
patterns) and ``test/CTMatrix_e.cx`` renders four small DNA matrices with
IUPAC codes, aliases, ``-`` and ``N`` as read, compacted, Fitch-compacted
and padded.  The host restatement (``Alignment``, CTMatrix.pyx:610-662,
785-1031, 1040-1145) must print the same text byte for byte."""
import json
import os

import pytest

from crux_gb300.alignment import Alignment, CTMatrix

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                  "compaction_kat.json")))


def test_rinehart_compacts_as_the_reference():
    aln = Alignment(CTMatrix(KAT["rinehart_fasta"]))
    assert aln.compact() == 0
    assert aln.render() == KAT["alignment_a"]


@pytest.mark.parametrize("i", range(len(KAT["ctmatrix_e"])))
def test_ctmatrix_e_blocks(i):
    case = KAT["ctmatrix_e"][i]
    aln = Alignment(CTMatrix(case["fasta"]))
    assert aln.render(pad=True) == case["Basic"]
    assert aln.compact() == 0
    assert aln.render(pad=True) == case["Compact"]
    aln.compact(fitch=True)
    assert aln.render(pad=True) == case["Fitch compact"]
    aln.pad("-", 4)
    assert aln.render(pad=True) == case["Fitch compact plus pad"]
    assert aln.npad == 4


def test_render_hides_padding_unless_asked():
    case = KAT["ctmatrix_e"][0]
    aln = Alignment(CTMatrix(case["fasta"]))
    aln.compact()
    aln.pad("N", 3)
    assert aln.render() == case["Compact"]
    assert aln.render(pad=True) != case["Compact"]


def test_fitch_compact_counts_dropped_changes():
    """Two-state patterns dropped by the Fitch compaction count one change
    per unit of frequency (CTMatrix.pyx:935-940); constant ones count 0."""
    fasta = ">a\nAAAACG\n>b\nAAAACG\n>c\nAACCAG\n>d\nAATCAT\n"
    aln = Alignment(CTMatrix(fasta))
    aln.compact()
    # Columns: AAAA (x2), AACT (informative? A twice, C, T: 3 states),
    # AACC (x1, two states each twice: informative), CCAA, GGGT.
    changes = aln.compact(fitch=True)
    # After Fitch relabelling: AAAA x2 (constant, 0 changes); AACC and CCAA
    # merge into AACC x2 (informative); AACT (3 states, informative);
    # GGGT -> AAAC (two states, one singleton: 1 change).
    assert changes == 1
    assert sorted(aln.freqs.tolist()) == [1, 2]
