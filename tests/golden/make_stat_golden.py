"""Record what the reference's own analysis modules print for the reference
program's outputs in tests/golden/host_ref/, as the golden answers for the
C analysis tool (hsmc_gb300/bin/hsmc_stat).

The modules (python/hsmc_pressure.py, hsmc_chem_pot.py, hsmc_op.py,
hsmc_density.py, hsmc_stat.py of the reference) are imported from the
reference sources with a do-nothing stand-in for matplotlib, whose plots play
no part in the numbers.  Cases where the reference's analysis itself raises
are listed in stat_ref/reference_failures.txt instead of being recorded (its
thermodynamic-pressure reader overruns its coefficient array when a block's
fit is undefined; its NpT path also reads past the end of density.dat).  Run
where the reference sources are present:

    python tests/golden/make_stat_golden.py
"""
from __future__ import annotations

import contextlib
import io
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.oracle import REF_ROOT  # noqa: E402  ($HSMC_REFERENCE, else ../reference)

REF_PY = os.path.normpath(os.path.join(REF_ROOT, "python"))
OUT = os.path.join(HERE, "stat_ref")


def _stub_matplotlib():
    class _Noop:
        def __getattr__(self, name):
            return lambda *a, **k: None

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    plt.__getattr__ = _Noop().__getattr__  # type: ignore[attr-defined]
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt


def main() -> None:
    _stub_matplotlib()
    sys.path.insert(0, REF_PY)
    import hsmc_chem_pot
    import hsmc_density
    import hsmc_op
    import hsmc_pressure

    nvt = os.path.join(HERE, "host_ref", "nvt_small")
    npt = os.path.join(HERE, "host_ref", "npt_small")
    cases = {
        "nvt_pressv": lambda: hsmc_pressure.pressure_virial(nvt),
        "nvt_pressv_b2": lambda: hsmc_pressure.pressure_virial(nvt, samples_block=2),
        "nvt_presst": lambda: hsmc_pressure.pressure_thermo(nvt),
        "nvt_mu": lambda: (hsmc_chem_pot.ave(nvt, plot=False), hsmc_chem_pot.std(nvt)),
        "nvt_op": lambda: (hsmc_op.ave(nvt, plot=False), hsmc_op.std(nvt, plot=False)),
        "npt_op": lambda: (hsmc_op.ave(npt, plot=False), hsmc_op.std(npt, plot=False)),
        "npt_density": lambda: (hsmc_density.ave(npt, plot=False), hsmc_density.std(npt, plot=False)),
        "npt_density_jk": lambda: (hsmc_density.ave(npt, plot=False),
                                   hsmc_density.std(npt, plot=False, jackknife=True)),
    }
    os.makedirs(OUT, exist_ok=True)
    failed = []
    for name, fn in cases.items():
        buf = io.StringIO()
        try:
            with contextlib.redirect_stdout(buf):
                fn()
        except Exception as exc:  # the reference's own analysis fails on this input
            failed.append(f"{name}: {type(exc).__name__}: {exc}")
            continue
        with open(os.path.join(OUT, name + ".txt"), "w") as fh:
            fh.write(buf.getvalue())
        print(name, "->", len(buf.getvalue().splitlines()), "lines")
    with open(os.path.join(OUT, "reference_failures.txt"), "w") as fh:
        fh.write("\n".join(failed) + ("\n" if failed else ""))
    for f in failed:
        print("reference analysis failed:", f)


if __name__ == "__main__":
    main()
