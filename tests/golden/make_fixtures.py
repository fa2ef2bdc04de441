"""Copies the reference's golden C++ trajectories into this directory.

The 14 files ``oracle3d/scene-{0..13}.json`` are the avbd-demo3d C++ solver's double-precision
output (positions and quaternions of every body at frames 1, 10, 60, 120 and 180, plus the
force count), shipped by the reference as
``reference/three-avbd/tests/fixtures/oracle3d/scene-*.json``. They are copied unchanged so
the tests can run where the reference is not present.

Usage: python tests/golden/make_fixtures.py <path-to-reference-checkout>
"""
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    src = os.path.join(ref_root, "reference", "three-avbd", "tests", "fixtures", "oracle3d")
    dst = os.path.join(HERE, "oracle3d")
    os.makedirs(dst, exist_ok=True)
    for i in range(14):
        name = f"scene-{i}.json"
        shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
        json.load(open(os.path.join(dst, name)))  # well-formed
    print(f"copied 14 fixtures to {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path-to-reference-checkout>")
    main(sys.argv[1])
