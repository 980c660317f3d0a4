"""Extract the reference's pattern-compression known answers into a fixture.

Test infrastructure, run once where the reference tree exists:

    python tests/golden/make_compaction_kat.py /root/reference/crux

It reads, as text, the reference's own tests of ``Alignment.compact``:

* ``test/Alignment_a.cx``: ``rinehart.fasta`` compacted and rendered; the
  answer is ``test/Alignment_a.cx.exp`` between "Test begin" and "Test end".
* ``test/CTMatrix_e.cx``: four FASTA strings, each rendered as read
  ("# Basic"), compacted ("# Compact"), Fitch-compacted ("# Fitch compact")
  and padded with four '-' columns ("# Fitch compact plus pad"); the
  answers are the blocks of ``test/CTMatrix_e.cx.exp``.

and writes ``tests/golden/compaction_kat.json`` with the inputs and the
expected text of every block.  Nothing is computed here: the fixture holds
only the reference's own inputs and printed answers.
"""
import ast
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "compaction_kat.json")
BLOCKS = ["Basic", "Compact", "Fitch compact", "Fitch compact plus pad"]


def between_markers(text):
    lines = text.split("\n")
    a = lines.index("Test begin")
    b = lines.index("Test end")
    return lines[a + 1:b]


def ctmatrix_e(test_dir):
    src = open(os.path.join(test_dir, "CTMatrix_e.cx")).read()
    m = re.search(r"dnaTestStrs = (\(.*?\n\))\n", src, re.S)
    strings = ast.literal_eval(m.group(1))
    body = between_markers(open(os.path.join(test_dir,
                                             "CTMatrix_e.cx.exp")).read())
    blocks, cur = [], None
    for line in body:
        if line.startswith("# ") and line[2:] in BLOCKS:
            cur = [line[2:], []]
            blocks.append(cur)
        else:
            cur[1].append(line)
    assert len(blocks) == 4 * len(strings), len(blocks)
    cases = []
    for i, fasta in enumerate(strings):
        case = {"fasta": fasta}
        for name, lines in blocks[4 * i:4 * i + 4]:
            case[name] = "\n".join(lines)
        assert list(case) == ["fasta"] + BLOCKS
        cases.append(case)
    return cases


def main(ref):
    test_dir = os.path.join(ref, "test")
    fasta = open(os.path.join(test_dir, "rinehart.fasta")).read()
    render = between_markers(open(os.path.join(test_dir,
                                               "Alignment_a.cx.exp")).read())
    out = {
        "source": "crux test/Alignment_a.cx(.exp), test/rinehart.fasta, "
                  "test/CTMatrix_e.cx(.exp)",
        "rinehart_fasta": fasta,
        "alignment_a": "\n".join(render),
        "ctmatrix_e": ctmatrix_e(test_dir),
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_compaction_kat.py <crux source tree>")
    main(sys.argv[1])
