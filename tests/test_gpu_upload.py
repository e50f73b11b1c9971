"""hsmc_gpu_upload_config checks the configuration on the device after the
copy: ids 0..N-1 (HSMC_ERR_INVALID_ARG) and coordinates in [0, L]
(HSMC_ERR_OUT_OF_BOX, NaN included).  A configuration that fails leaves the
context without one, so the sweeps refuse to run, and a valid upload after
it continues the chain as if the failed ones had not happened."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INVALID_ARG, OUT_OF_BOX = 1, 8


def test_upload_checks_and_recovery(gpu_lib):
    from hsmc_gb300.system import HsmcError

    g = gpu_lib.HardSphereSystem(rho=0.5, cells=5, dr_max=0.2, seed=3)
    good = g.download()
    L = g.get_box()[0]
    cases = []
    c = good.copy()
    c[7, 0] = 8.0
    cases.append((c, INVALID_ARG))
    c = good.copy()
    c[3, 2] = -1e-12
    cases.append((c, OUT_OF_BOX))
    c = good.copy()
    c[5, 3] = math.nextafter(L, math.inf)
    cases.append((c, OUT_OF_BOX))
    c = good.copy()
    c[9, 1] = float("nan")
    cases.append((c, OUT_OF_BOX))
    c = good.copy()
    c[2, 0] = 9.0
    c[4, 1] = 2 * L
    cases.append((c, INVALID_ARG))  # a bad id is reported before a bad coordinate
    for conf, code in cases:
        with pytest.raises(HsmcError) as err:
            g.upload(conf)
        assert err.value.code == code
        with pytest.raises(HsmcError) as err:
            g.sweep_nvt(1)
        assert err.value.code == INVALID_ARG
    edge = good.copy()
    edge[0, 1], edge[1, 2] = 0.0, L  # the box's own faces are inside
    g.upload(edge)
    g.upload(good)
    g.sweep_nvt(5)
    ref = gpu_lib.HardSphereSystem(rho=0.5, cells=5, dr_max=0.2, seed=3)
    ref.sweep_nvt(5)
    assert np.array_equal(g.download(), ref.download())
    g.close()
    ref.close()
