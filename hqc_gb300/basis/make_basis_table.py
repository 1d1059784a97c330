"""Build ``gth_h.json``: the hydrogen entries of the reference's basis files.

The reference reads CP2K-format ``.dat`` files at factory time
(``hqc/basis/parse.py:32-64``: split on '#BASIS SET', take the first block
whose text starts with the element symbol).  The GPU hosts do not carry the
reference checkout, so this script extracts, with that same rule, the
hydrogen block of every ``gth-raw`` and ``gth-test`` file into one JSON table
keyed by basis name.  The data are the published GTH basis sets of CP2K
(VandeVondele & Hutter, J. Chem. Phys. 127, 114105 (2007); CP2K data,
GPL-2.0-or-later), copied verbatim because the numbers must be identical.

    python hqc_gb300/basis/make_basis_table.py [/path/to/reference]

The checkout defaults to ``$HQC_REFERENCE`` (or /root/reference when unset).
The licence notice of the extracted data is ``NOTICE`` beside the table.
"""
import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref=None):
    ref = ref or os.environ.get("HQC_REFERENCE", "/root/reference")
    table = {}
    for sub in ("gth-raw", "gth-test"):
        for path in sorted(glob.glob(os.path.join(ref, "hqc", "basis", sub, "*.dat"))):
            name = os.path.basename(path)[:-4]
            if name in table:
                continue
            blocks = open(path).read().split("#BASIS SET\n")
            for b in blocks:
                if b[:1] == "H":
                    table[name] = "#BASIS SET\n" + b
                    break
    with open(os.path.join(HERE, "gth_h.json"), "w") as fh:
        json.dump(table, fh, indent=0, sort_keys=True)
    print(len(table), "basis entries")


if __name__ == "__main__":
    main(*sys.argv[1:])
