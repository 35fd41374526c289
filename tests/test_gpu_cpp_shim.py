"""A compiled C++ caller of the C ABI: the GpuSPH Physics package
(include/sphgpu_spheral.hh), built with g++ against include/sphgpu.h and
stand-in Spheral headers (tests/cpp/stub), linked with libsphgpu.so.

The driver (tests/cpp/physics_shim_main.cc) goes through the Physics
interface as a Spheral integrator does (registerState, registerDerivatives,
initializeProblemStartupDependencies, evaluateDerivatives, dt) and then takes
three device-resident CheapSynchronousRK2 steps.  On a 1,728-node periodic box
its derivative FieldLists match the oracle to 1e-12 normwise, the dt vote to
1e-12, and the state after three steps to 1e-11."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from spheral_gb300 import problems

from _parity import rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NSTEPS = 3


def _compile(native_lib, out_dir):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ is not available")
    libdir = os.path.join(ROOT, "spheral_gb300")
    exe = os.path.join(out_dir, "physics_shim")
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "tests", "cpp", "stub"), os.path.join(ROOT, "tests", "cpp", "physics_shim_main.cc"),
           "-L", libdir, "-lsphgpu", "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _write_problem(p, path):
    c = p.config
    nl = p.nodelists[0]
    head = [p.n, NSTEPS, len(p.boundaries), c["cfl"], int(c["compatible_energy"]), int(c["gradh_correction"]),
            int(c["xsph"]), int(c["correct_velocity_gradient"]), c["Cl"], c["Cq"], c["dt_min"], c["dt_max"],
            c["dt_growth"], c["last_dt"], 0, 0,
            nl["nPerh"], nl["hmin"], nl["hmax"], nl["rhoMin"], nl["rhoMax"], nl["gamma"]]
    for b in p.boundaries:
        head += [b["type"], b["axis"], b["lo"], b["hi"], b.get("wall_high", 0)]
    data = np.concatenate([np.array(head, dtype=np.float64), p.pos.ravel(), p.vel.ravel(), p.mass, p.rho, p.eps,
                           p.H.ravel()])
    data.tofile(path)


def test_cpp_shim_compiles_and_links(native_lib, tmp_path):
    # no GPU needed: the package header, the C ABI and the library agree
    _compile(native_lib, str(tmp_path))


@pytest.mark.gpu
def test_cpp_physics_package_matches_oracle(native_lib, oracle_mod, tmp_path):
    p = problems.random_box(n_side=12, seed=41, boundaries="periodic")
    exe = _compile(native_lib, str(tmp_path))
    prob_path = os.path.join(str(tmp_path), "problem.bin")
    _write_problem(p, prob_path)
    prefix = os.path.join(str(tmp_path), "out")
    r = subprocess.run([exe, prob_path, prefix], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "label GpuSPH" in r.stdout
    n = p.n
    d = np.fromfile(prefix + "_derivs.bin", dtype=np.float64)
    sizes = [("DvDt", 3), ("DepsDt", 1), ("DvDx", 9), ("massDensitySum", 1), ("Hideal", 6), ("DHDt", 6),
             ("maxViscousPressure", 1), ("pressure", 1)]
    assert d.size == n * sum(s for _, s in sizes) + 1
    orc = oracle_mod.Oracle(p)
    orc.initialize()
    orc.evaluate_derivatives()
    q = 0
    for name, nc in sizes:
        got = d[q:q + n * nc].reshape(n, nc) if nc > 1 else d[q:q + n]
        q += n * nc
        assert rel_err(got, orc.field(name)) <= 1e-12, name
    dt_orc = orc.hydro_dt()
    assert abs(d[-1] - dt_orc) <= 1e-12 * dt_orc
    for _ in range(NSTEPS):
        orc.step()
    s = np.fromfile(prefix + "_state.bin", dtype=np.float64)
    assert abs(s[0] - orc.time) <= 1e-12 * orc.time
    q = 1
    for name, nc in [("position", 3), ("velocity", 3), ("massDensity", 1), ("specificThermalEnergy", 1), ("H", 6),
                     ("pressure", 1)]:
        got = s[q:q + n * nc].reshape(n, nc) if nc > 1 else s[q:q + n]
        q += n * nc
        assert rel_err(got, orc.field(name)) <= 1e-11, name
