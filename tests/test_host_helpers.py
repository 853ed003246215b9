"""Host-side helpers of the drop-in modules, no GPU: the frequency and MAS-index
helpers against the compiled reference (where it is built), the mode-count
checks against the reference's definition (Pk_library.pyx:90-117), and the
bispectrum's integer shell bounds against a brute-force scan."""
import math

import numpy as np
import pytest

import build_ref
from pylians_gb300 import Pk_library as P


@pytest.fixture(scope='module')
def ref():
    if not build_ref.built():
        pytest.skip('compiled reference not built here')
    return build_ref.load_reference()[1]


@pytest.mark.parametrize('dims', [1, 2, 31, 32, 33, 128, 1000, 1024])
def test_frequencies_match_reference(ref, dims):
    assert P.frequencies(1000.0, dims) == tuple(ref.frequencies(1000.0, dims))
    assert P.frequencies_2D(250.0, dims) == tuple(ref.frequencies_2D(250.0, dims))


def test_mas_index_matches_reference(ref):
    for mas in ('NGP', 'CIC', 'TSC', 'PCS', 'None', None, 'cic'):
        assert P.MAS_function(mas) == ref.MAS_function(mas), mas


@pytest.mark.parametrize('dims', [4, 5, 16, 17])
def test_mode_count_checks(dims):
    own3 = 1 if dims % 2 else 8
    own2 = 1 if dims % 2 else 4
    n3 = (dims ** 3 - own3) // 2 + own3
    n2 = (dims ** 2 - own2) // 2 + own2
    P.check_number_modes(np.array([n3 - 5, 5]), dims)
    P.check_number_modes_2D(np.array([n2]), dims)
    with pytest.raises(RuntimeError):
        P.check_number_modes(np.array([n3 + 1]), dims)
    with pytest.raises(RuntimeError):
        P.check_number_modes_2D(np.array([n2 - 1]), dims)


@pytest.mark.parametrize('k_min,k_max', [(0.0, 1.0), (0.5, 1.5), (1.0, 3.0), (5.2, 7.2),
                                         (math.sqrt(50.0), math.sqrt(72.0)), (12.3, 14.3)])
def test_shell_bounds_are_exact(k_min, k_max):
    """[lo, hi) holds exactly the integer k^2 whose float64 square root lies in
    [k_min, k_max), the test the reference applies per mode."""
    lo, hi = P.shell_k2_bounds(k_min, k_max)
    for c in range(0, int(k_max * k_max) + 40):
        inside = k_min <= np.sqrt(np.float64(c)) < k_max
        assert inside == (lo <= c < hi), (c, lo, hi)
