"""CPU checks of the sea-state generator's host restatement
(cfdwavemaker_gb300/seastate.py), which the GPU generator
(cfdwm_spectrum_components) is tested against:

* SplitMix64 against the published outputs of its reference implementation
  for state 1234567;
* the generated sea has the requested Hs (4 sqrt(m0), m0 = sum A^2 / 2), the
  spreading weights sum to one, the phases lie in [0, 2 pi) and the
  wavenumbers solve the dispersion relation.
"""
import math

import numpy as np

from cfdwavemaker_gb300 import seastate as ss


def test_splitmix64_known_answers():
    got = [int(v) for v in ss.splitmix64(1234567, 5)]
    assert got == [6457827717110365317, 3203168211198807973, 9817491932198370423, 4593380528125082431,
                   16408922859458223821]


def test_splitmix_sea_properties():
    c = ss.irregular_components(5.0, 11.0, 2.2, 40, 0.3, 1.8, 70.0, 99, ndir=7, spreading_s=6.0,
                                phase_rng="splitmix")
    m0 = 0.5 * np.sum(c["A"] ** 2)
    assert abs(4.0 * math.sqrt(m0) - 5.0) < 1e-12
    assert np.all((c["phase"] >= 0.0) & (c["phase"] < 2 * math.pi))
    w, k = c["omega"], c["k"]
    assert np.max(np.abs(9.81 * k * np.tanh(k * 70.0) - w * w) / (w * w)) < 1e-13
    th = np.unique(c["theta"])
    assert th.size == 7 and abs(th[0] + math.pi / 2) < 1e-15 and abs(th[-1] - math.pi / 2) < 1e-15
    # a different seed gives different phases, the same seed the same
    c2 = ss.irregular_components(5.0, 11.0, 2.2, 40, 0.3, 1.8, 70.0, 99, ndir=7, spreading_s=6.0,
                                 phase_rng="splitmix")
    c3 = ss.irregular_components(5.0, 11.0, 2.2, 40, 0.3, 1.8, 70.0, 100, ndir=7, spreading_s=6.0,
                                 phase_rng="splitmix")
    np.testing.assert_array_equal(c["phase"], c2["phase"])
    assert np.all(c["phase"] != c3["phase"])
