"""Statistical gate at the large NVT fluid state: N = 256,000 (40^3 FCC
start), rho = 0.85, dr_max 0.1635 (the benchmarked state).

The GPU chain (checkerboard sweeps) and the reference algorithm's chain
(random-particle moves, the CPU oracle; eight chains recorded by
tests/golden/make_c2_stats.py) sample the same ensemble.  Every observable
must agree within 3 combined blocking standard errors, and each error is
printed:
  - Z from the reference's contact fit: a straight line through the five
    0.01 bins of g(r) on [1, 1.05) extrapolated to contact,
    Z = 1 + 2 pi/3 rho g(1) (python/hsmc_pressure.py:11-41);
  - g(r) on five ranges of r up to 5 (bins of 0.01);
  - beta mu_ex from Widom insertions, 10 x 10^4 per sample;
  - the global q6 with bond cutoff 1.5.
beta mu_ex must also agree with Carnahan-Starling within 3 standard errors.
Z from the straight-line contact fit sits about 0.7 % below
Carnahan-Starling at this density: the line's bias (g(r) is convex near
contact) plus Carnahan-Starling's own error are both far larger than the
statistical error of 256,000 spheres.  The test requires the GPU's and the
reference chain's deviations from Carnahan-Starling to be the same within 3
standard errors (the chain-to-chain gate above) and prints them.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "c2_oracle_stats.npz")
RHO, CELLS, DR = 0.85, 40, 0.1635
N = 4 * CELLS**3
EQUIL, SAMPLES, EVERY, RDF_EVERY, BLOCKS = 1500, 200, 100, 5, 10
BIN, NB_PV, NB_RDF = 0.01, 5, 400
RANGES = [(1.0, 1.1), (1.1, 1.3), (1.3, 1.6), (1.6, 2.2), (2.2, 5.0)]


def shell_volumes(nb, bin_):
    r1 = 1.0 + bin_ * np.arange(nb)
    return 4 * np.pi / 3 * ((r1 + bin_) ** 3 - r1**3)


def g_of(counts, samples):
    return counts / (shell_volumes(len(counts), BIN) * RHO * N * samples)


def contact_z(g5):
    r = 1.0 + BIN * (np.arange(NB_PV) + 0.5)
    b1, b0 = np.polyfit(r, g5, 1)
    return 1 + 2 * np.pi / 3 * RHO * (b0 + b1)


def g_ranges(g):
    r = 1.0 + BIN * (np.arange(NB_RDF) + 0.5)
    return np.array([g[(r >= a) & (r < b)].mean() for a, b in RANGES])


def mean_se(x):
    x = np.asarray(x, dtype=float)
    return x.mean(axis=0), x.std(axis=0, ddof=1) / math.sqrt(len(x))


def cs(eta):
    z = (1 + eta + eta**2 - eta**3) / (1 - eta) ** 3
    mu = (8 * eta - 9 * eta**2 + 3 * eta**3) / (1 - eta) ** 3
    return z, mu


def test_large_fluid_observables_agree_with_reference_chain(gpu_lib):
    ref = np.load(FIX)
    assert float(ref["rho"]) == RHO and int(ref["cells"]) == CELLS and float(ref["dr_max"]) == DR
    # the reference chains: one block each
    ref_samples = int(ref["samples"])
    ref_z = [contact_z(g_of(pv, ref_samples)) for pv in ref["pv"]]
    ref_g = [g_ranges(g_of(rd, n)) for rd, n in zip(ref["rdf"], ref["n_rdf"])]
    ref_q6 = ref["q6"]
    p_ref = ref["widom_ok"] / ref["widom_n"]

    g = gpu_lib.HardSphereSystem(rho=RHO, cells=CELLS, dr_max=DR, seed=77)
    g.sweep_nvt(EQUIL)
    per = SAMPLES // BLOCKS
    pv = np.zeros((BLOCKS, NB_PV))
    rdf = np.zeros((BLOCKS, NB_RDF))
    n_rdf = np.zeros(BLOCKS)
    q6 = np.zeros(BLOCKS)
    ok = np.zeros(BLOCKS)
    n_ins = np.zeros(BLOCKS)
    for k in range(SAMPLES):
        b = k // per
        g.sweep_nvt(EVERY)
        pv[b] += g.compute_pressv_counts(BIN, 1.0 + NB_PV * BIN, NB_PV)
        q6[b] += g.global_ql(6, 1.5) / per
        for _ in range(10):
            ok[b] += g.widom_insertion(10_000)
            n_ins[b] += 10_000
        if k % RDF_EVERY == 0:
            rdf[b] += g.compute_rdf_counts(BIN, 1.0 + NB_RDF * BIN, NB_RDF)
            n_rdf[b] += 1
    acc = g.get_moves_counters()
    g.close()
    gpu_z = [contact_z(g_of(pv[b], per)) for b in range(BLOCKS)]
    gpu_g = [g_ranges(g_of(rdf[b], n_rdf[b])) for b in range(BLOCKS)]

    report, failures = [], []

    def gate(name, a, b):
        (ma, ea), (mb, eb) = mean_se(a), mean_se(b)
        ma, ea, mb, eb = np.atleast_1d(ma), np.atleast_1d(ea), np.atleast_1d(mb), np.atleast_1d(eb)
        for k in range(len(ma)):
            s = math.hypot(ea[k], eb[k])
            dev = (ma[k] - mb[k]) / s if s > 0 else 0.0
            label = f"{name}[{k}]" if len(ma) > 1 else name
            report.append(f"{label}: gpu {ma[k]:.6f} +- {ea[k]:.6f}  reference {mb[k]:.6f} +- {eb[k]:.6f}  "
                          f"({dev:+.2f} sigma)")
            if abs(dev) > 3.0:
                failures.append(label)

    gate("Z (contact fit)", gpu_z, ref_z)
    gate("g(r) on " + ", ".join(f"[{a},{b})" for a, b in RANGES), gpu_g, ref_g)
    gate("q6", q6, ref_q6)
    # Widom: the pooled insertion probability, its error from the blocks
    p_gpu = ok / n_ins
    (mp_g, ep_g), (mp_r, ep_r) = mean_se(p_gpu), mean_se(p_ref)
    mu_g, emu_g = -math.log(mp_g), ep_g / mp_g
    mu_r, emu_r = -math.log(mp_r), ep_r / mp_r
    s_mu = math.hypot(emu_g, emu_r)
    report.append(f"beta mu_ex: gpu {mu_g:.4f} +- {emu_g:.4f} ({int(ok.sum())} of {int(n_ins.sum())})  reference "
                  f"{mu_r:.4f} +- {emu_r:.4f} ({int(ref['widom_ok'].sum())} of {int(ref['widom_n'].sum())})  "
                  f"({(mu_g - mu_r) / s_mu:+.2f} sigma)")
    if abs(mu_g - mu_r) > 3 * s_mu:
        failures.append("beta mu_ex")
    z_cs, mu_cs = cs(math.pi * RHO / 6)
    report.append(f"beta mu_ex vs Carnahan-Starling {mu_cs:.4f}: {(mu_g - mu_cs) / emu_g:+.2f} sigma")
    if abs(mu_g - mu_cs) > 3 * emu_g:
        failures.append("beta mu_ex vs Carnahan-Starling")
    mz_g, ez_g = mean_se(gpu_z)
    mz_r, ez_r = mean_se(ref_z)
    report.append(f"Z - Z_CS ({z_cs:.5f}): gpu {mz_g - z_cs:+.5f} +- {ez_g:.5f} ({(mz_g - z_cs) / z_cs:+.3%}), "
                  f"reference {mz_r - z_cs:+.5f} +- {ez_r:.5f} ({(mz_r - z_cs) / z_cs:+.3%})")
    report.append(f"acceptance: gpu {acc[1] / acc[0]:.4f} (checkerboard, with cell-boundary rejections), "
                  f"reference {float(np.mean(ref['acc'])):.4f}")
    print("\n" + "\n".join(report))
    assert not failures, "\n".join(report)
