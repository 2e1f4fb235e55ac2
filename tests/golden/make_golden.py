"""Regenerate the golden fixtures in this folder from the reference itself.

Builds oracle/_ref/ref_driver (the reference's own sources, compiled as they
lie in the reference checkout, with oracle/refshim standing in for the
FFTW3 / GSL / Boost / Armadillo libraries that are not installed) and packs
each driver case into <case>.npz. Run from the repository root:

    python tests/golden/make_golden.py [/path/to/reference] [--cases c1,c2,...]

The fixtures are committed; the GPU machines never run this script.
"""
import os
import shutil
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASES = ["weights", "phi", "bulk", "eval_models16", "eval_hs32", "eval_lj", "fire_hs32", "fire_lj24",
         "ddft_lj16", "ddft_adapt16", "coex", "hessian", "files", "ao"]
# cases that also leave files next to their output: copied here as <case>.<suffix>
FILE_OUTPUTS = {"files": [".a.vtk", ".b.vtk"]}


def read_driver_output(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    o = 0
    while o < len(data):
        (nl,) = struct.unpack_from("<I", data, o)
        o += 4
        name = data[o:o + nl].decode()
        o += nl
        (n,) = struct.unpack_from("<Q", data, o)
        o += 8
        out[name] = np.frombuffer(data, dtype="<f8", count=n, offset=o).copy()
        o += 8 * n
    return out


def main():
    args = sys.argv[1:]
    cases = CASES
    if "--cases" in args:
        i = args.index("--cases")
        cases = args[i + 1].split(",")
        del args[i:i + 2]
    ref = args[0] if args else "/root/reference"
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + ref])
    drv = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
    with tempfile.TemporaryDirectory() as tmp:  # FIRE writes snapshot files into the cwd
        for case in cases:
            out = os.path.join(tmp, case + ".bin")
            subprocess.check_call([drv, case, out], cwd=tmp)
            arrays = read_driver_output(out)
            np.savez_compressed(os.path.join(HERE, case + ".npz"), **arrays)
            for suffix in FILE_OUTPUTS.get(case, []):
                shutil.copyfile(out + suffix, os.path.join(HERE, case + suffix))
            print(case, len(arrays), "arrays")


if __name__ == "__main__":
    main()
