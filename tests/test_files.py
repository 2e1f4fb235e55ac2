"""Density files of the reference (no GPU): the VTK writer byte for byte against
files the reference itself wrote (Density::write_VTK_File through its VisIt
writer, tests/golden/files.*.vtk from oracle/ref_driver), and the Armadillo
binary snapshot (Density::writeDensity / readDensity) by its published layout
and a round trip."""
import os

import numpy as np
import pytest

from conftest import golden

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def cd():
    import classicaldft_gb300 as cd
    cd.lib()
    return cd


@pytest.mark.parametrize("tag", ["a", "b"])
def test_vtk_matches_reference_bytes(cd, tmp_path, tag):
    g = golden("files")
    shape = tuple(int(x) for x in g["files.%s.shape" % tag])
    rho = g["files.%s.rho" % tag].reshape(shape)
    out = tmp_path / ("d_%s" % tag)  # ".vtk" is appended, as the reference does
    cd.write_vtk(str(out), rho)
    mine = (tmp_path / ("d_%s.vtk" % tag)).read_bytes()
    ref = open(os.path.join(HERE, "golden", "files.%s.vtk" % tag), "rb").read()
    assert mine == ref


def test_arma_binary_layout_and_round_trip(cd, tmp_path):
    rng = np.random.default_rng(5)
    rho = rng.uniform(0.01, 0.9, size=(6, 5, 4))
    p = tmp_path / "snap.dat"
    cd.write_density(str(p), rho)
    raw = p.read_bytes()
    head = b"ARMA_MAT_BIN_FN008\n120 1\n"
    assert raw[:len(head)] == head and len(raw) == len(head) + 8 * rho.size
    assert np.array_equal(np.frombuffer(raw[len(head):], dtype="<f8"), rho.ravel())
    back = cd.read_density(str(p), rho.shape)
    assert np.array_equal(back, rho)
    with pytest.raises(cd.CDFTError):
        cd.read_density(str(p), (6, 5, 5))  # wrong size
    with pytest.raises(cd.CDFTError):
        cd.read_density(str(tmp_path / "missing.dat"), rho.shape)
