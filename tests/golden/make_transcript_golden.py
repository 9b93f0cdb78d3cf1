"""Generate ``tests/golden/transcripts.json`` from the reference's
``test_read_transcript`` (snapatac2-core/src/genome.rs:599-643): its GFF3 and
GTF inputs, the expected first transcript, and the GTF line whose quoted
value holds ';' that must parse.  Rust string literals are unescaped
(``\\n\\`` continuations, ``\\t``, ``\\"``).

Run from the repository root:  python tests/golden/make_transcript_golden.py
"""
from __future__ import annotations

import json
import os
import re

# root of the SnapATAC2 source tree the fixtures are cut from: the first
# command-line argument, else $SNAPATAC2_REFERENCE
import sys  # noqa: E402
REFERENCE_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SNAPATAC2_REFERENCE", "")
if not REFERENCE_ROOT:
    sys.exit("usage: python " + os.path.basename(__file__) + " <SnapATAC2 source root> (or set SNAPATAC2_REFERENCE)")

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.path.join(REFERENCE_ROOT, "snapatac2-core/src/genome.rs")


def rust_str(src: str, name: str) -> str:
    m = re.search(r'let ' + name + r' = "(.*?)(?<!\\)";', src, re.S)
    s = re.sub(r"\\\n\s*", "", m.group(1))
    return s.replace("\\n", "\n").replace("\\t", "\t").replace('\\"', '"')


def main() -> None:
    src = open(REF).read()
    body = src[src.index("fn test_read_transcript()"):]
    exp = body[body.index("let expected = Transcript {"):body.index("};")]
    field = lambda k: re.search(k + r': (?:Some\()?"([^"]*)"', exp).group(1)  # noqa: E731
    num = lambda k: int(re.search(k + r": Position::try_from\((\d+)\)", exp).group(1))  # noqa: E731
    out = {
        "gff": rust_str(body, "gff"),
        "gtf": rust_str(body, "gtf"),
        "worked": rust_str(body, "worked"),
        "expected": {"transcript_name": field("transcript_name"), "transcript_id": field("transcript_id"),
                     "gene_name": field("gene_name"), "gene_id": field("gene_id"), "chrom": field("chrom"),
                     "left": num("left"), "right": num("right"),
                     "strand": "+" if "Strand::Forward" in exp else "-"},
    }
    with open(os.path.join(ROOT, "tests", "golden", "transcripts.json"), "w") as fh:
        json.dump(out, fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
