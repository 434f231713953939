"""Pin the oracle's total-variation solver against gratopy's golden values.

gratopy's tests/test_fanbeam.py:1249-1382 run 2000 TV iterations on the
walnut sinogram (400^2, fan beam) and compare control numbers with
0.251590 (mu = 1e8, exact data) and 0.038413 (mu = 20, data + 0.2 N(0,1)
noise from default_rng(1)).  At 2000 iterations the CPU oracle needs a few
minutes per run, too slow for the unit-test suite, so this script runs the
two pins once and records the outcome in tests/golden/oracle_solver_pins.json
(the Landweber and CG pins run in tests/test_oracle_pins.py).

    python -m oracle.pin_solvers
"""

from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))

import configs  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.helpers import control_number, host_settings, walnut_sinogram  # noqa: E402


def main():
    ps = host_settings(configs.configs()["fan_walnut400"])
    walnut = walnut_sinogram("float32")
    walnut = walnut / np.mean(walnut)
    rng = np.random.default_rng(1)
    noisy = walnut + rng.normal(0, 1, walnut.shape) * 0.2
    dims = (400, 400, 328, 120, 1)
    nrm = O.normest(ps)
    out = {"normest": nrm}
    for name, data, mu, golden in (("exact_mu1e8", walnut, 1e8, 0.251590),
                                    ("noisy_mu20", noisy, 20.0, 0.038413)):
        t0 = time.time()
        sino = np.require(data, np.float32, "F")
        U = O.total_variation(sino, ps, mu, 2000, slice_thickness=0, stepsize_weighting=10,
                              norm_estimate=nrm)
        val = float(control_number(U, dims, "img"))
        out[name] = {"control_number": val, "golden": golden,
                     "rel_err": abs(val - golden) / abs(golden), "seconds": time.time() - t0}
        print(name, out[name], flush=True)
    path = ROOT / "tests" / "golden" / "oracle_solver_pins.json"
    path.write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
