"""The C analysis tool against the reference's own analysis modules
(tests/golden/stat_ref/, made by tests/golden/make_stat_golden.py from the
reference program's outputs), and on synthetic files with known answers.

Tolerance: the reference fits its contact line with scipy's iterative
least-squares, the tool in closed form; the two agree to ~1e-8 relative, so
printed numbers are compared with a relative tolerance of 1e-6."""
import math
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def stat_exe():
    import sys

    sys.path.insert(0, ROOT)
    from hsmc_gb300 import build

    return build.build_stat()


def _run(exe, *args):
    r = subprocess.run([exe] + list(args), capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _same(got: str, want: str):
    gl, wl = got.strip().splitlines(), want.strip().splitlines()
    assert len(gl) == len(wl), (got, want)
    for a, b in zip(gl, wl):
        ta, tb = a.split(), b.split()
        assert len(ta) == len(tb), (a, b)
        for x, y in zip(ta, tb):
            try:
                fx, fy = float(x.rstrip(":")), float(y.rstrip(":"))
            except ValueError:
                assert x == y, (a, b)
                continue
            assert math.isclose(fx, fy, rel_tol=1e-6, abs_tol=1e-8), (a, b)


CASES = {
    "nvt_pressv": ("nvt_small", [], ["pressv"]),
    "nvt_pressv_b2": ("nvt_small", ["-b", "2"], ["pressv"]),
    "nvt_mu": ("nvt_small", [], ["mu"]),
    "nvt_op": ("nvt_small", [], ["op"]),
    "npt_op": ("npt_small", [], ["op"]),
    "npt_density": ("npt_small", [], ["density"]),
    "npt_density_jk": ("npt_small", ["-j"], ["density"]),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_matches_reference_analysis(stat_exe, case):
    sub, opts, cmds = CASES[case]
    want = open(os.path.join(GOLD, "stat_ref", case + ".txt")).read()
    got = _run(stat_exe, "-d", os.path.join(GOLD, "host_ref", sub), *opts, *cmds)
    _same(got, want)


def _write_thermo(d, n_part, vol, samples, slope, offset, n_bins=8, dxi=1e-3, zero_bin=None):
    with open(os.path.join(d, "press_thermo.dat"), "w") as fh:
        for s in range(samples):
            fh.write("#" * 38 + "\n# Bins, volume, number of particles\n" + "#" * 38 + "\n")
            fh.write(f"{n_bins} {vol:.8e} {n_part}\n")
            fh.write("#" * 38 + "\n# abs(xi), exp(-beta*U)\n" + "#" * 38 + "\n")
            for k in range(n_bins):
                xi = (k + 1) * dxi
                v = 0.0 if (zero_bin is not None and k == zero_bin and s == 0) else \
                    math.exp(-(offset + slope[s] * xi))
                fh.write(f"{xi:.8e} {v:.8e}\n")


def test_thermo_pressure_from_the_slope(stat_exe, tmp_path):
    """-ln(non-overlap fraction) linear in xi with slope N p_ex: the tool
    recovers P = rho (1 + p_ex) per block; a zero bin is dropped, not fatal."""
    n_part, vol = 500, 1000.0
    slopes = [n_part * (1.5 + 0.1 * k) for k in range(6)]
    _write_thermo(tmp_path, n_part, vol, 6, slopes, 0.0, zero_bin=3)
    out = _run(stat_exe, "-d", str(tmp_path), "presst").splitlines()
    n, ave, std, ave_iso, std_iso = out[2].split()
    rho = n_part / vol
    p = [rho * (1 + s / n_part) for s in slopes]
    assert int(n) == 6
    assert float(ave) == pytest.approx(sum(p) / 6, rel=1e-6)
    assert float(ave_iso) == pytest.approx(sum(p) / 6 / rho, rel=1e-6)
    assert float(std) > 0


def test_thermo_pressure_npt_uses_sample_densities(stat_exe, tmp_path):
    n_part, vol = 256, 512.0
    slopes = [n_part * 2.0] * 4
    _write_thermo(tmp_path, n_part, vol, 4, slopes, 0.0)
    dens = [0.50, 0.52, 0.48, 0.54]
    with open(os.path.join(tmp_path, "density.dat"), "w") as fh:
        fh.write("#" * 38 + "\n# Density (each line is one sample)\n" + "#" * 38 + "\n")
        for v in dens:
            fh.write(f"{v:.8e}\n")
    out = _run(stat_exe, "-d", str(tmp_path), "presst-npt").splitlines()
    assert float(out[2].split()[1]) == pytest.approx(sum(d * 3.0 for d in dens) / 4, rel=1e-6)
    assert float(out[5].split()[1]) == pytest.approx(sum(dens) / 4, rel=1e-6)


def test_bad_usage_fails_loudly(stat_exe, tmp_path):
    r = subprocess.run([stat_exe, "-d", str(tmp_path), "mu"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "cannot open" in r.stderr
    r = subprocess.run([stat_exe, "nonsense"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
