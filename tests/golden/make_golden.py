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
         "ddft_lj16", "ddft_adapt16", "coex", "hessian", "files", "ao", "spectral", "boundary"]
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


def spectral_post(arrays):
    """The dense Hessians the driver wrote (column j = matrix_dot_v1 of the j-th unit
    vector) are replaced by what the spectral-driver tests compare with: every
    eigenvalue (LAPACK, of the symmetrised matrix), the asymmetry, the eigenvectors of
    the isolated extreme eigenvalues, and the extreme eigenvalues of H + vshift vshift^T / 2
    (Eigenvalues::calculate_gradients, src/Eigenvalues.cpp) for a seeded vshift."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    # the DDFT dynamical matrix g.H: not symmetric, but similar to a symmetric matrix on
    # the range of the mobility, so its eigenvalues are real; every eigenvalue (sorted),
    # the largest imaginary part LAPACK leaves, and the unit eigenvectors of the two
    # eigenvalues of largest magnitude
    G = arrays.pop("sp16.G")
    n = int(round(np.sqrt(G.size)))
    G = G.reshape(n, n).T
    w, V = np.linalg.eig(G)
    order = np.argsort(w.real)
    arrays["sp16.G.eig"] = w.real[order]
    arrays["sp16.G.eig_imag_max"] = np.array([np.abs(w.imag).max()])
    top = np.argsort(-np.abs(w.real))[:2]
    for j, i in enumerate(top):
        v = V[:, i].real
        v = v / np.linalg.norm(v)
        arrays["sp16.G.evec_top%d" % j] = v * np.sign(v[np.argmax(np.abs(v))])
    for tag in ("sp16", "splj16"):
        H = arrays.pop(tag + ".H")
        n = int(round(np.sqrt(H.size)))
        H = H.reshape(n, n).T
        arrays[tag + ".asym"] = np.array([np.abs(H - H.T).max()])
        Hs = 0.5 * (H + H.T)
        w, V = np.linalg.eigh(Hs)
        arrays[tag + ".eig"] = w
        for name, i in (("evec_min", 0), ("evec_max", n - 1)):
            v = V[:, i] * np.sign(V[np.argmax(np.abs(V[:, i])), i])
            arrays[tag + "." + name] = v
        s = pyoracle.fill_noise((16, 16, 16), 1.0, 1.0, 31).ravel() - 1.0
        s *= np.sqrt(2 * 0.01) / np.linalg.norm(s)
        arrays[tag + ".vshift"] = s
        ws = np.linalg.eigvalsh(Hs + 0.5 * np.outer(s, s))
        arrays[tag + ".eig_vshift"] = np.concatenate([ws[:8], ws[-8:]])
    return arrays


POST = {"spectral": spectral_post}


def main():
    args = sys.argv[1:]
    cases = CASES
    if "--cases" in args:
        i = args.index("--cases")
        cases = args[i + 1].split(",")
        del args[i:i + 2]
    # the reference checkout: the first argument, else $CDFT_REFERENCE_DIR, else its usual mount point
    ref = args[0] if args else os.environ.get("CDFT_REFERENCE_DIR", "/root/reference")
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + ref])
    drv = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
    with tempfile.TemporaryDirectory() as tmp:  # FIRE writes snapshot files into the cwd
        for case in cases:
            out = os.path.join(tmp, case + ".bin")
            subprocess.check_call([drv, case, out], cwd=tmp)
            arrays = read_driver_output(out)
            if case in POST:
                arrays = POST[case](arrays)
            np.savez_compressed(os.path.join(HERE, case + ".npz"), **arrays)
            for suffix in FILE_OUTPUTS.get(case, []):
                shutil.copyfile(out + suffix, os.path.join(HERE, case + suffix))
            print(case, len(arrays), "arrays")


if __name__ == "__main__":
    main()
