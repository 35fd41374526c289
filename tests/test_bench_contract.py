"""The benchmark's reference arm on the CPU: `bench.py --impl reference`
times the FP64 oracle on the host cores and prints one JSON line with the
contract's keys (metric, value, unit, step counts, dtype, the reference
marker, a cpu_baseline describing the run and an e2e record of the same
value with no host-device copies), for each workload name, on a small
sample so the check takes seconds.  Also the KH generator's interface
smoothing (the CRKSPH benchmark's initial conditions)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload,extra", [("kh", ["--cpu-n1", "12"]), ("crksph", ["--cpu-n1", "12"]),
                                            ("sod", ["--cpu-n1", "16"])])
def test_reference_arm_prints_the_contract_line(workload, extra):
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", workload,
                        "--steps", "1", "--warmup", "1"] + extra,
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_kelvin_helmholtz_interface_smoothing():
    from spheral_gb300 import problems
    sharp = problems.kelvin_helmholtz(n1=16)
    smooth = problems.kelvin_helmholtz(n1=16, smooth=0.025)
    assert np.array_equal(sharp.pos, smooth.pos)
    # pressure equilibrium everywhere, P = 2.5
    gamma = 5.0 / 3.0
    np.testing.assert_allclose((gamma - 1.0) * smooth.rho * smooth.eps, 2.5, rtol=1e-14)
    # densities and shear velocities between the two slabs' values, relaxed
    # towards the mean near the interfaces and untouched far from them
    assert smooth.rho.min() >= 1.0 and smooth.rho.max() <= 2.0
    d = np.minimum(np.abs(smooth.pos[:, 1] - 0.25), np.abs(smooth.pos[:, 1] - 0.75))
    far = d > 0.2   # exp(-0.2 / 0.025) / 2 = 1.7e-4 of the jump at most
    assert far.sum() > 0.1 * len(d)
    np.testing.assert_allclose(smooth.rho[far], sharp.rho[far], rtol=2e-4)
    np.testing.assert_allclose(smooth.vel[far, 0], sharp.vel[far, 0], atol=2e-4)
    near = d < 0.04   # the layers next to an interface move towards the mean density
    assert near.sum() > 0
    assert np.all(smooth.rho[near & (sharp.rho == 1.0)] > 1.05)
    assert np.all(smooth.rho[near & (sharp.rho == 2.0)] < 1.95)
    # masses follow the density (same volume per node)
    np.testing.assert_allclose(smooth.mass / smooth.rho, sharp.mass / sharp.rho, rtol=1e-14)
