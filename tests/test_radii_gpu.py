"""setCutoffRadii on the device against the oracle (src/particle.h:1320-1456,
src/particle.h:704-730): the radial velocity-dispersion bins, the Gaussian
smoothing of the bins at every body and the radii.  The device computes the
Gaussian weights near each body's bin with exp and the rest by a recurrence
(factors shrinking by e^-2 per bin), and its exp and pow are CUDA's: the
results agree with the oracle's bin-by-bin libm arithmetic to 1e-13
relative."""
import numpy as np
import pytest

from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.p3t import GpuSystem
from oracle import harness as H

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mk", [lambda: make_disk(65536, 1e-10 * 16, 0.5, 1.5, seed=31),
                                lambda: make_disk(20000, 1e-9, 0.95, 1.05, ecc_hill=6.0, inc_hill=3.0, seed=32)],
                         ids=["65k wide disk", "20k ring"])
def test_radii_match_oracle(gpu, mk):
    d = mk()
    P = P3TParams()
    orc, g = H.CpuSystem("orc", P), GpuSystem(P)
    orc.load(d)
    orc.f("set_r_planet")()
    orc.prepare()
    g.load(d)
    g.set_r_planet()
    g.prepare()
    for k in ("v_disp", "r_out", "r_search", "r_out_inv"):
        a, b = g.get(k), orc.get(k)
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=0, err_msg=k)
