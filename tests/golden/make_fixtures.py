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
  bibd_result_tables.json  the |Aut(D)| tables (Nd, Ns, Ndt, Nst per group order,
                        totals) of every BIBD result file with v <= 16 and
                        b <= 63, and for files in the current layout the exact
                        text from the BIBD( line to the "fully constructed" line
  k10_results_table.txt the |Aut(M)| x cycles table of K_Results.txt for K10
  kts15_canonical.txt   the 7 canonical Kirkman triple systems on 15 points (groups of
                        3, 7 rounds) with |Aut(M)|, parsed from
                        k-Factorization/Results/Complete_graphs/15/15x7x3/K_OrderedMatrices.txt

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


def parse_k10(path, nrows=9):
    """(|Aut(M)|, rounds) of every matrix of a K_OrderedMatrices.txt file with nrows rounds."""
    txt = open(path, encoding="latin-1").read().splitlines()
    out = []
    i = 0
    while i < len(txt):
        m = re.match(r"\s*(\d+): \|Aut\(M\)\| =\s*(\d+)", txt[i])
        if m:
            rows = [txt[i + j].strip().strip('"').split() for j in range(1, nrows + 1)]
            out.append((int(m.group(2)), [" ".join(r) for r in rows]))
            i += nrows + 1
        else:
            i += 1
    return out


def parse_bibd_table(path):
    lines = open(path, encoding="latin-1").read().splitlines()
    t = next(i for i, l in enumerate(lines) if l.startswith("BIBD("))
    h = next(i for i, l in enumerate(lines) if "|Aut(D)|" in l)
    rows, i = [], h + 2
    while not lines[i].strip().startswith("_"):
        rows.append([int(x) for x in lines[i].split()[:5]])
        i += 1
    entry = dict(rows=rows, total=[int(x) for x in lines[i + 1].split()[1:5]],
                 wide="Nd:             Ns:" in lines[h])
    if entry["wide"]:
        end = next(j for j in range(i, len(lines)) if "fully constructed" in lines[j])
        entry["text"] = "\n".join(lines[t:end + 1]) + "\n"
        secs = next(l for l in lines[i:end] if "constructed in" in l)
        entry["seconds"] = float(re.search(r"constructed in\s+([\d.]+)", secs).group(1))
        entry["fully_constructed"] = int(lines[end].split()[0])
    return entry


def bibd_result_tables(ref):
    tables = {}
    base = os.path.join(ref, "Results", "BIBDs")
    for d in sorted(os.listdir(base)):
        if not d.startswith("V ="):
            continue
        for f in sorted(os.listdir(os.path.join(base, d))):
            m = re.fullmatch(r"(\d+)_(\d+)_(\d+)\.txt", f)
            if not m:
                continue
            path = os.path.join(base, d, f)
            text = open(path, encoding="latin-1").read()
            title = next(l for l in text.splitlines() if l.startswith("BIBD("))
            v, b, r, k, lam = map(int, re.findall(r"\d+", title)[:5])
            if v <= 16 and b <= 63 and "|Aut(D)|" in text:      # runs that finished
                tables["%d,%d,%d,%d,%d" % (v, b, r, k, lam)] = parse_bibd_table(path)
    return tables


def k10_results_table(path):
    lines = open(path, encoding="latin-1").read().splitlines()
    t = next(i for i, l in enumerate(lines) if "Factorization of K(10)" in l)
    end = next(i for i in range(t, len(lines)) if "Total:" in lines[i]) + 1
    return "\n".join(lines[t:end + 1]) + "\n\n\n"


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

    kts = parse_k10(os.path.join(ref, "k-Factorization", "Results", "Complete_graphs", "15",
                                 "15x7x3", "K_OrderedMatrices.txt"), nrows=7)
    assert len(kts) == 7
    with open(os.path.join(HERE, "kts15_canonical.txt"), "w") as f:
        f.write("# 7 canonical Kirkman triple systems on 15 points: |Aut| then 7 rounds of 15 players "
                "(groups of 3)\n")
        for aut, rows in kts:
            f.write("%d %s\n" % (aut, " | ".join(rows)))

    with open(os.path.join(HERE, "bibd_result_tables.json"), "w") as f:
        json.dump(bibd_result_tables(ref), f, indent=1, sort_keys=True)
    kdir = os.path.join(ref, "k-Factorization", "Results", "Complete_graphs", "10", "10x9x2")
    with open(os.path.join(HERE, "k10_results_table.txt"), "w") as f:
        f.write(k10_results_table(os.path.join(kdir, "K_Results.txt")))

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
