"""Queue order of the persistent kernel (host logic; results do not depend on it)."""
import numpy as np

from discoeb_gb300.perturbations import K_STEP_PEAK, schedule_order


def test_heuristic_order_is_a_permutation_starting_at_the_step_peak():
    k = np.geomspace(1e-4, 10.0, 512)
    o = schedule_order(k)
    assert o.dtype == np.int32 and np.array_equal(np.sort(o), np.arange(512))
    d = np.abs(np.log(k[o] / K_STEP_PEAK))
    assert (np.diff(d) >= 0).all()


def test_cost_order_is_longest_first_and_stable():
    cost = np.array([5, 900, 5, 40, 900, 1])
    o = schedule_order(None, cost)
    assert o.tolist() == [1, 4, 3, 0, 2, 5]


def test_invalid_k_goes_last_without_warnings():
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("error")
        o = schedule_order(np.array([0.1, -1.0, np.nan, 1.0, 0.0]))
    assert o.tolist()[:2] == [0, 3] and sorted(o.tolist()[2:]) == [1, 2, 4]
