"""Copies the reference's graph-build golden fixtures into tests/golden/.

The fixtures are the inputs and expected text dumps of the genomix-hyracks graph-build
tests: BatchTestFilesTest (8 single-end k=3 pairs under data/sequence/) and
StepByStepTest's paired-end case (data/input/smalltest.txt ->
data/expected/smalltest-graph-result.txt).  They are data, copied byte for byte so the
parity tests can run where the reference tree is absent.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SUB = "genomix/genomix-hyracks/src/test/resources/data"

# (name, input, expected, k): k comes from the `_k(\d+)` file-name rule of
# GraphBuildingTestSetting.java:12-19; smalltest is run with k=3 by StepByStepTest.
CASES = [
    ("Random100_k3", "sequence/random/Random100_k3.test.txt", "sequence/random/Random100_k3.expected.txt", 3),
    ("Synthetic_k3", "sequence/pathmerge/Synthetic_k3.test.txt", "sequence/pathmerge/Synthetic_k3.expected.txt", 3),
    ("HighSplitRepeat_k3", "sequence/splitrepeat/HighSplitRepeat_k3.test.txt",
     "sequence/splitrepeat/HighSplitRepeat_k3.expected.txt", 3),
    ("MidSplitRepeat_k3", "sequence/splitrepeat/MidSplitRepeat_k3.test.txt",
     "sequence/splitrepeat/MidSplitRepeat_k3.expected.txt", 3),
    ("LowSplitRepeat_k3", "sequence/splitrepeat/LowSplitRepeat_k3.test.txt",
     "sequence/splitrepeat/LowSplitRepeat_k3.expected.txt", 3),
    ("MultiTandemRepeat_k3", "sequence/multi_tandem_repeat/MultiTandemRepeat_k3.test.txt",
     "sequence/multi_tandem_repeat/MultiTandemRepeat_k3.expected.txt", 3),
    ("MultiTandemRepeat2_k3", "sequence/multi_tandem_repeat/MultiTandemRepeat2_k3.test.txt",
     "sequence/multi_tandem_repeat/MultiTandemRepeat2_k3.expected.txt", 3),
    ("MultiTandemRepeat3_k3", "sequence/multi_tandem_repeat/MultiTandemRepeat3_k3.test.txt",
     "sequence/multi_tandem_repeat/MultiTandemRepeat3_k3.expected.txt", 3),
    ("smalltest_paired_k3", "input/smalltest.txt", "expected/smalltest-graph-result.txt", 3),
]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    src = os.path.join(ref, SUB)
    index = []
    for name, inp, exp, k in CASES:
        for rel, suffix in ((inp, ".input.txt"), (exp, ".expected.txt")):
            shutil.copyfile(os.path.join(src, rel), os.path.join(HERE, name + suffix))
        index.append({"name": name, "k": k, "source_input": f"{SUB}/{inp}", "source_expected": f"{SUB}/{exp}"})
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1)
        f.write("\n")
    print(f"copied {len(CASES)} fixture pairs to {HERE}")


if __name__ == "__main__":
    main()
