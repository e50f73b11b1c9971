"""Batched replicas at dense states against the reference algorithm's own
chain: N = 2048 (8^3 FCC start) at rho = 0.75 and 0.85, 16 GPU replicas per
density under the persistent batched schedule, 2000 sweeps from the lattice,
then the virial contact histogram every 20 sweeps for 10^4 sweeps.  The
straight-line contact fit (python/hsmc_pressure.py:11-41) of the replicas
must agree with the oracle chains' (tests/golden/make_dense_stats.py) within
3 combined standard errors (each replica and each chain one block).  The
departure of both from Carnahan-Starling is printed: it is the fit's, the
same for both chains."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "dense_oracle_stats.npz")
REPS = 16


def contact_z(counts, samples, n, rho, bin_=0.01):
    nb = len(counts)
    r1 = 1.0 + bin_ * np.arange(nb)
    g = counts / samples / (4 * np.pi / 3 * ((r1 + bin_) ** 3 - r1**3) * rho * n)
    b1, b0 = np.polyfit(r1 + bin_ / 2, g, 1)
    return 1 + 2 * np.pi / 3 * rho * (b0 + b1)


def test_dense_replica_pressure_matches_reference_chain(gpu_lib):
    from hsmc_gb300.batch import ReplicaBatch, carnahan_starling

    ref = np.load(FIX)
    cells, dr = int(ref["cells"]), float(ref["dr_max"])
    equil, samples, every = int(ref["equil"]), int(ref["samples"]), int(ref["every"])
    n = 4 * cells**3
    rhos = [float(r) for r in ref["rhos"]]
    systems = [(rho, cells, dr, 900 + 100 * k + j) for k, rho in enumerate(rhos) for j in range(REPS)]
    b = ReplicaBatch(systems)
    b.set_schedule(1, 2, 2)
    b.sweeps(equil)
    nb, bin_ = 5, 0.01
    acc = np.zeros((len(systems), nb))
    for _ in range(samples):
        b.sweeps(every)
        acc += b.pressv_counts(bin_, 1.0 + nb * bin_, nb)
    report, bad = [], []
    for k, rho in enumerate(rhos):
        zg = np.array([contact_z(acc[k * REPS + j], samples, n, rho) for j in range(REPS)])
        zr = np.array([contact_z(pv, samples, n, rho) for pv in ref["pv"][k]])
        mg, eg = zg.mean(), zg.std(ddof=1) / math.sqrt(len(zg))
        mr, er = zr.mean(), zr.std(ddof=1) / math.sqrt(len(zr))
        s = math.hypot(eg, er)
        zcs = carnahan_starling(rho)
        report.append(f"rho {rho}: Z gpu {mg:.4f} +- {eg:.4f}, reference chain {mr:.4f} +- {er:.4f} "
                      f"({(mg - mr) / s:+.2f} sigma); Carnahan-Starling {zcs:.4f}: gpu {(mg - zcs) / zcs:+.3%}, "
                      f"reference chain {(mr - zcs) / zcs:+.3%}")
        if abs(mg - mr) > 3 * s:
            bad.append(rho)
    print("\n" + "\n".join(report))
    assert not bad, "\n".join(report)
