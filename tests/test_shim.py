"""The C++ shim with the reference's task signatures (include/phx_parthenon_shim.hpp).

CPU: the shim and its driver compile and link against the library.
GPU: an RK stage run through fluid::PrimitiveToConserved, ConservedToPrimitive,
CalculateFluidSourceTerms, CalculateFluxes, FluxCT and EstimateTimestepBlock
(the C++ host path a phoebus build would take) is bit-identical to the oracle.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from phoebus_gb300 import abi, states

ROOT = Path(__file__).resolve().parent.parent
CUDA = Path("/usr/local/cuda")


def build_driver(tmp, exact=True):
    lib = "phx_fluid_exact" if exact else "phx_fluid"
    exe = tmp / "shim_stage"
    cmd = ["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
           str(ROOT / "tests" / "cpp" / "shim_stage.cpp"), "-o", str(exe), "-L", str(ROOT / "phoebus_gb300" / "_lib"),
           f"-l{lib}", f"-Wl,-rpath,{ROOT / 'phoebus_gb300' / '_lib'}", "-L", str(CUDA / "lib64"), "-lcudart",
           f"-Wl,-rpath,{CUDA / 'lib64'}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.skipif(not shutil.which("g++"), reason="needs g++")
def test_shim_compiles_and_links(built, tmp_path):
    exe = build_driver(tmp_path)
    assert exe.exists()


@pytest.mark.gpu
def test_shim_stage_matches_oracle(built, oracle, tmp_path):
    exe = build_driver(tmp_path, exact=True)
    n, ng = 12, 4
    hb, par = states.kelvin_helmholtz(n=n, seed=31)
    (tmp_path / "in.bin").write_bytes(np.ascontiguousarray(hb["prim"]).tobytes())
    dt = 2.0e-4
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(n), str(ng),
                        str(abi.RECON["weno5z"]), str(abi.RIEMANN["hll"]), repr(5.0 / 3.0), repr(dt)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    p = abi.default_params(Gamma=5.0 / 3.0, recon="weno5z", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100, cfl=0.4)
    oracle.Initialize(p, hb)
    dt0 = oracle.EstimateTimestepBlock(p, hb, False)
    out = np.zeros_like(hb["cons"])
    oracle.Stage(p, hb, hb["cons"], out, 1.0, dt)
    dt1 = oracle.EstimateTimestepBlock(p, hb, True)
    lines = dict(l.split() for l in r.stdout.splitlines() if l.startswith("dt"))
    assert float(lines["dt0"]) == dt0 and float(lines["dt1"]) == dt1
    data = np.frombuffer((tmp_path / "out.bin").read_bytes(), dtype=np.float64)
    N = hb.N
    prim = data[:12 * N].reshape(hb["prim"].shape)
    cons = data[12 * N:].reshape(hb["cons"].shape)
    assert np.array_equal(prim, hb["prim"])
    ks, js, is_ = hb.isl()
    assert np.array_equal(cons, out)


def build_rad_driver(tmp, exact=True):
    lib = "phx_fluid_exact" if exact else "phx_fluid"
    exe = tmp / "shim_rad_stage"
    cmd = ["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
           str(ROOT / "tests" / "cpp" / "shim_rad_stage.cpp"), "-o", str(exe), "-L",
           str(ROOT / "phoebus_gb300" / "_lib"), f"-l{lib}", f"-Wl,-rpath,{ROOT / 'phoebus_gb300' / '_lib'}", "-L",
           str(CUDA / "lib64"), "-lcudart", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.skipif(not shutil.which("g++"), reason="needs g++")
def test_shim_radiation_compiles_and_links(built, tmp_path):
    assert build_rad_driver(tmp_path).exists()


@pytest.mark.gpu
def test_shim_radiation_stage_matches_oracle(built, tmp_path):
    """radiation::MomentPrim2Con, MomentCon2Prim, MomentCalculateOpacities,
    ReconstructEdgeStates, CalculateFluxes, CalculateGeometricSource,
    MomentFluidSource and EstimateTimestepBlock through the shim (C++ host
    path), one stage of a random periodic 3D block, against the oracle
    running the same task sequence: bit for bit (exact build)."""
    from oracle.oracle import RadOracle
    from tests.util import random_rad_block

    exe = build_rad_driver(tmp_path, exact=True)
    n, ng, dt, ks_, ka, jbb = 12, 4, 2.0e-3, 30.0, 2.0, 0.5
    hb = random_rad_block((n, n, n), 3, seed=41, vmax=0.3)
    (tmp_path / "in.bin").write_bytes(np.ascontiguousarray(hb["prim"]).tobytes() +
                                      np.ascontiguousarray(hb["rprim"]).tobytes())
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(n), str(ng), repr(dt),
                        repr(ks_), repr(ka), repr(jbb)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    o = RadOracle()
    p = abi.default_params(Cv=1.0)
    rp = abi.default_rad_params(cfl=0.5, kappa_s=ks_, kappa_a=ka, jbb_coeff=jbb)
    o.MomentPrim2Con(rp, p, hb)
    o.Initialize(rp, p, hb)
    o.MomentCalculateOpacities(rp, p, hb)
    o.CalculateFluxes(rp, p, hb)
    out = np.zeros_like(hb["rcons"])
    o.Update(rp, hb, hb["rcons"].copy(), out, 1.0, dt)
    hb.arrays["rcons"] = out
    o.MomentCon2Prim(rp, p, hb)
    o.MomentFluidSource(rp, p, hb, dt)
    o.FillGhostsPeriodic(hb)
    o.MomentCon2Prim(rp, p, hb)
    dtn = o.EstimateTimestepBlock(rp, p, hb)
    data = np.frombuffer((tmp_path / "out.bin").read_bytes(), dtype=np.float64)
    N = hb.N
    cons = data[:4 * N].reshape(hb["rcons"].shape)
    prim = data[4 * N:14 * N].reshape(hb["rprim"].shape)
    assert np.array_equal(cons, hb["rcons"])
    assert np.array_equal(prim[:abi.RFAIL + 1], hb["rprim"][:abi.RFAIL + 1])
    assert data[14 * N] == dtn
