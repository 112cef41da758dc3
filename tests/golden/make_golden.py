"""Regenerate tests/golden/ref_random.json from the reference's own random.hpp.

Builds oracle/_ref/ref_golden (oracle/Makefile target `ref`, which compiles
the reference's random.hpp from the reference source tree given as REF, or
in the environment variable MINIPIC_REFERENCE) and stores its JSON output.
Run from the repository root:

    python tests/golden/make_golden.py [REF]
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MINIPIC_REFERENCE", "")
    if not ref:
        sys.exit("usage: make_golden.py REF (or set MINIPIC_REFERENCE to the MiniPIC source tree)")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + ref])
    out = subprocess.check_output([os.path.join(ROOT, "oracle", "_ref", "ref_golden")], text=True)
    data = json.loads(out)
    data["generated_by"] = "tests/golden/make_golden.py from random.hpp of the reference tree"
    with open(os.path.join(ROOT, "tests", "golden", "ref_random.json"), "w") as f:
        json.dump(data, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
