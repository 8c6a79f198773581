"""Writes the golden fixtures of tests/golden/ (run in a checkout that has the
reference tree; the GPU machine never runs this).

  bibd_histograms.json  |Aut| histograms of complete BIBD enumerations, parsed
                        from the reference's Results/BIBDs/V = v/<v>_<k>_<lambda>.txt
  k10_canonical.txt     the 396 canonical 1-factorizations of K10 with |Aut(M)|,
                        parsed from k-Factorization/Results/Complete_graphs/10/
                        10x9x2/K_OrderedMatrices.txt
  sts15_canonical.txt   the 80 canonical STS(15) (one per isomorphism class) as
                        built by the oracle's orderly enumeration; pinned by the
                        reference's STS(15) |Aut| histogram (checked here)

Usage: python tests/golden/make_fixtures.py [REFERENCE_ROOT]
"""
import collections
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

BIBD_PARAMS = [  # (v, b, r, k, lambda)
    (7, 7, 3, 3, 1), (7, 14, 6, 3, 2), (9, 12, 4, 3, 1), (13, 26, 6, 3, 1),
    (15, 35, 7, 3, 1), (8, 14, 7, 4, 3), (11, 11, 5, 5, 2), (9, 18, 8, 4, 3),
    (10, 15, 6, 4, 2),
]


def parse_bibd_histogram(path):
    hist = {}
    with open(path, encoding="latin-1") as f:
        lines = f.read().splitlines()
    start = next(i for i, l in enumerate(lines) if "|Aut(D)|" in l)
    i = start + 2
    while not lines[i].strip().startswith("_"):
        parts = lines[i].split()
        hist[int(parts[0])] = int(parts[1])
        i += 1
    return hist


def parse_k10(path):
    txt = open(path, encoding="latin-1").read().splitlines()
    out = []
    i = 0
    while i < len(txt):
        m = re.match(r"\s*(\d+): \|Aut\(M\)\| =\s*(\d+)", txt[i])
        if m:
            rows = [txt[i + j].strip().strip('"').split() for j in range(1, 10)]
            out.append((int(m.group(2)), [" ".join(r) for r in rows]))
            i += 10
        else:
            i += 1
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    hists = {}
    for (v, b, r, k, lam) in BIBD_PARAMS:
        path = os.path.join(ref, "Results", "BIBDs", "V = %3d" % v, "%d_%d_%d.txt" % (v, k, lam))
        hists["%d,%d,%d,%d,%d" % (v, b, r, k, lam)] = parse_bibd_histogram(path)
    with open(os.path.join(HERE, "bibd_histograms.json"), "w") as f:
        json.dump(hists, f, indent=1, sort_keys=True)

    k10 = parse_k10(os.path.join(ref, "k-Factorization", "Results", "Complete_graphs", "10",
                                 "10x9x2", "K_OrderedMatrices.txt"))
    assert len(k10) == 396
    with open(os.path.join(HERE, "k10_canonical.txt"), "w") as f:
        f.write("# 396 canonical 1-factorizations of K10: |Aut| then 9 rounds of 10 players\n")
        for aut, rows in k10:
            f.write("%d %s\n" % (aut, " | ".join(rows)))

    import oracle  # noqa: E402  (CPU oracle, test infrastructure)
    found, _ = oracle.bibd_enumerate(15, 35, 7, 3, 1)
    hist = collections.Counter(a for _, a in found)
    assert dict(hist) == {int(k): v for k, v in hists["15,35,7,3,1"].items()}, hist
    with open(os.path.join(HERE, "sts15_canonical.txt"), "w") as f:
        f.write("# 80 canonical STS(15) (oracle orderly enumeration): |Aut| then 15 rows of 35 bits\n")
        for M, aut in found:
            f.write("%d %s\n" % (aut, " ".join("".join(str(x) for x in row) for row in M)))


if __name__ == "__main__":
    main()
