"""The reference's C++ class API over the C ABI (include/classicaldft_gb300.hpp):
a reference-style app compiles and links here; on a GPU it reproduces the
reference's config-1 evaluation and FIRE2 trajectory."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden

APP = os.path.join(ROOT, "tests", "cpp", "reference_style_app.cpp")


def build_app(out):
    import classicaldft_gb300 as cd
    if not os.path.exists(cd.LIB_PATH):
        from classicaldft_gb300 import build
        build.build()
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), APP, "-o", out,
           "-L", os.path.dirname(cd.LIB_PATH), "-lcdft", "-Wl,-rpath," + os.path.dirname(cd.LIB_PATH),
           "-L/usr/local/cuda/lib64", "-lcudart"]
    subprocess.check_call(cmd)


def test_reference_style_app_builds(tmp_path):
    build_app(str(tmp_path / "app"))
    assert os.path.exists(str(tmp_path / "app"))


@pytest.mark.gpu
def test_reference_style_app_runs_config1(tmp_path):
    exe = str(tmp_path / "app")
    build_app(exe)
    import classicaldft_gb300 as cd
    ao = golden("ao")
    cd.write_density(str(tmp_path / "ao_rho.dat"), ao["ao16.WhiteBearI.rho"])
    out = subprocess.check_output([exe, "20", str(tmp_path / "ao_rho.dat")], text=True, cwd=str(tmp_path)).split()
    F, Fhs, mu, steps, Ffin = float(out[0]), float(out[1]), float(out[2]), int(out[3]), float(out[4])
    g = golden("eval_hs32")
    assert abs(F - g["hs32.Omega"][0]) <= 1e-12 * abs(F)
    assert abs(Fhs - g["hs32.F_hs"][0]) <= 1e-12 * abs(Fhs)
    fire = golden("fire_hs32")
    assert steps == 20
    assert abs(Ffin - fire["fire32.F"][19]) <= 1e-12 * abs(Ffin)
    # Hessian . v through the C++ mirror, against the oracle at the same density
    from oracle import pyoracle
    shape = (32, 32, 32)
    rho = pyoracle.fill_noise(shape, 0.7, 0.05, 20240601)
    v = 0.3 * (pyoracle.fill_noise(shape, 1.0, 1.0, 77) - 1.0)
    o = pyoracle.Oracle(32, 0.2, "WhiteBearI", hsd=1.0)
    hv = o.hessian_dot_v(rho, v)
    hsum, habs = float(out[5]), float(out[6])
    assert abs(habs - np.abs(hv).sum()) <= 1e-11 * np.abs(hv).sum()
    assert abs(hsum - hv.sum()) <= 1e-11 * np.abs(hv).sum()
    # Density::writeDensity / readDensity round trip and write_VTK_File through the mirror
    assert float(out[7]) == 0.0
    assert (tmp_path / "snapshot.vtk").read_bytes().startswith(b"# vtk DataFile Version 2.0\nWritten using VisIt writer\nASCII\n")
    # FMT_AO_Species through the mirror, on a density handed over as a reference snapshot file
    assert abs(float(out[8]) - ao["ao16.WhiteBearI.Omega"][0]) <= 1e-12 * abs(ao["ao16.WhiteBearI.Omega"][0])
    # Log_Det and Eigenvalues through the mirror, at the starting density: the log det
    # against the oracle's restatement (same probes), the largest eigenvalue against the
    # Python binding's
    ref_ld, _ = o.log_det(rho, 6, 0.2, 0.005, 1234, 1)
    assert abs(float(out[9]) - ref_ld) <= 1e-10 * abs(ref_ld)
    c = cd.Context(32, 0.2, cd.WHITEBEAR_I, hsd=1.0)
    c.set_density(rho)
    lam, _, _ = c.eigenvalue(tol=1e-10, change_sign=True)
    c.close()
    assert abs(float(out[10]) - lam) <= 1e-9 * lam
    # getDF(0) is a DFT_Vec: its inf_norm and accu against the reference's dF
    dV = 0.2 ** 3
    assert abs(float(out[11]) - g["hs32.dF.absmax"][0]) <= 1e-10 * dV
    assert abs(float(out[12]) - g["hs32.dF.sum"][0]) <= 1e-10 * dV * 32 ** 3
    # the state saved after 20 steps and resumed by a second minimizer: steps 21-30 of the
    # reference's trajectory
    assert int(out[14]) == 30
    assert abs(float(out[13]) - fire["fire32.F"][29]) <= 1e-12 * abs(float(out[13]))
    # snapshot_s0.dat: written by the 1st and 11th steps (the reference's every tenth call),
    # so it holds the density after step 11
    snap = cd.read_density(str(tmp_path / "snapshot_s0.dat"), shape)
    c = cd.Context(32, 0.2, cd.WHITEBEAR_I, hsd=1.0)
    c.set_chem_potential(c.bulk(0.7)["mu"])
    c.set_density(rho)
    c.fire_init(force_limit=0.0)
    c.fire_step(11)
    np.testing.assert_allclose(snap, c.get_density(), rtol=1e-12, atol=0)
    c.close()
