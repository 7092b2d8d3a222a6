"""Regenerate the golden fixtures from the reference's example data.

Run in a checkout where the reference project is available:

    python tests/golden/make_golden.py /path/to/Whale.jl

Writes, next to this script:
  example1/*.ale      the 12 CCDs of example/example-1/ale, re-serialised with
                      the two sections the likelihood never reads blanked
                      (constructor_string -> "(omitted)", Bip_bls -> 0)
  example1_tree.nw    extree (src/Whale.jl:34-37) with the two WGDs of
                      test/runtests.jl:10-11 inserted halfway up the branches
                      above ATHA and above LCA(ATHA, ATRI), each new node
                      appended to its parent's children (insertnode!)
  example5/*.ale      example/example-5 CCDs, same treatment; example5_tree.nw
  example4/*.ale      example/example-4/cytp450.ale (one family of 95 genes,
                      4,916 clades), same treatment; example4_tree.nw
  landplant/*.ale     docs/data/landplant/100fams (100 families), same
                      treatment; landplant_tree.nw (its speciestree.nw)
  golden.json         the reference's own pinned values (test/runtests.jl:19,
                      :32) and the settings they were computed with
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def normalise(text: str) -> str:
    parts = text.split("#")
    out = [parts[0]]
    for sec in parts[1:]:
        head, _, body = sec.partition("\n")
        if head.strip() == "constructor_string":
            sec = head + "\n(omitted)\n"
        elif head.strip() == "Bip_bls":
            lines = [l for l in body.split("\n") if l.strip()]
            sec = head + "\n" + "".join(l.split()[0] + "\t0\n" for l in lines)
        out.append(sec)
    return "#".join(out)


def main(ref: str) -> None:
    for sub, dst in (("example/example-1/ale", "example1"), ("example/example-5", "example5"),
                     ("example/example-4", "example4"), ("docs/data/landplant/100fams", "landplant")):
        src = os.path.join(ref, sub)
        os.makedirs(os.path.join(HERE, dst), exist_ok=True)
        for f in sorted(os.listdir(src)):
            if not f.endswith(".ale"):
                continue
            with open(os.path.join(src, f)) as fh:
                txt = normalise(fh.read())
            with open(os.path.join(HERE, dst, f), "w") as fh:
                fh.write(txt)
    # extree with wgd_1 above ATHA and wgd_2 above LCA(ATHA, ATRI)
    tree1 = ("((MPOL:4.752,PPAT:4.752):0.292,(SMOE:4.457,((GBIL:3.178,PABI:3.178):0.34,"
             "(((OSAT:1.555,(CPAP:0.5548,(ATHA:0.2774)wgd_1:0.2774):1.0002):0.738,ATRI:2.293):0.6125)"
             "wgd_2:0.6125):0.939):0.587);")
    with open(os.path.join(HERE, "example1_tree.nw"), "w") as fh:
        fh.write(tree1 + "\n")
    with open(os.path.join(ref, "example/example-5/tree.nw")) as fh:
        t5 = fh.readline().strip()
    with open(os.path.join(HERE, "example5_tree.nw"), "w") as fh:
        fh.write(t5 + "\n")
    for src, dst in (("example/example-4/tree.nw", "example4_tree.nw"),
                     ("docs/data/landplant/speciestree.nw", "landplant_tree.nw")):
        with open(os.path.join(ref, src)) as fh:
            t = fh.readline().strip()
        with open(os.path.join(HERE, dst), "w") as fh:
            fh.write(t + "\n")
    golden = {
        "source": "test/runtests.jl of Whale.jl v2.1.0",
        "single_family": {"file": "OG0004512.fasta.nex.treesample.ale", "dt": 0.05, "maxn": 5,
                          "lambda_log": 1.0, "mu_log": 1.0, "n_rates": 17, "q": [0.2, 0.1], "eta": 0.9,
                          "logpdf": -60.96367806571888, "cite": "test/runtests.jl:15-19"},
        "twelve_families": {"dt": 0.05, "maxn": 10000, "lambda_log": 1.0, "mu_log": 1.0, "n_rates": 17,
                            "q": [0.2, 0.1], "eta": 0.9, "condition": "root", "logpdf": -592.0185620440255,
                            "cite": "test/runtests.jl:21-34"},
    }
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(golden, fh, indent=1)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("WHALE_REFERENCE_DIR", "")
    if not src:
        sys.exit("usage: make_golden.py <reference checkout> (or set WHALE_REFERENCE_DIR)")
    main(src)
