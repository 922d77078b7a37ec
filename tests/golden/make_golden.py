"""Regenerate the golden fixtures in this folder from the reference checkout.

Run once where the NuclearToolkit.jl sources are available, with the path of
that checkout as the only argument:

    python tests/golden/make_golden.py <NuclearToolkit.jl checkout>

Copies
the interaction files the reference's own ShellModel tests use and records the
reference's known-answer values next to them (golden.json).  Tests read only
the files written here, never the reference tree.
"""
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    src = os.path.join(ref, "test", "interaction_file")
    for f in ("ckpot.snt", "usdb.snt"):
        shutil.copyfile(os.path.join(src, f), os.path.join(HERE, f))
    golden = {
        # test/ShellModel_test.jl:8-15 — main_sm("ckpot.snt","Be8",10,[]; q=2, is_block=true)
        "ckpot_Be8": {
            "source": "test/ShellModel_test.jl:10",
            "energies": [-31.119, -27.300, -19.162, -18.249, -16.722, -14.925, -14.517, -14.017, -13.951, -13.478],
            "tolerance_sq": 1.0e-6,
        },
        # example/log_sample_script.txt:323 — 24Mg in the sd shell (16O core)
        "sd_Mg24_mdim": {"source": "example/log_sample_script.txt:323", "mdim": 28503},
    }
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <NuclearToolkit.jl checkout>")
    main(sys.argv[1])
