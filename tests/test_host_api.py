"""Host-side mirror of the reference API (CPU only): the pool task split and
the multi-survey design matrix."""
import numpy as np
import pytest


def test_batch_tasks_split_like_the_reference():
    """utils.batch_tasks (:22-72): n_batches runs, the first n % n_batches
    one longer; one run when there are fewer tasks than batches (also for
    zero tasks)."""
    from thejoker_gb300.sampler import batch_tasks
    arr = np.arange(100, 110)
    got = batch_tasks(10, 3, arr)
    assert [len(g) for g in got] == [4, 3, 3]
    np.testing.assert_array_equal(np.concatenate(got), arr)
    got = batch_tasks(2, 5, arr[:2])
    assert len(got) == 1 and list(got[0]) == [100, 101]
    got = batch_tasks(0, 1, arr[:0])
    assert len(got) == 1 and len(got[0]) == 0
    got = batch_tasks(7, 7, arr[:7])
    assert [len(g) for g in got] == [1] * 7


def _reference_trend(data_list, poly_trend):
    """validate_prepare_data + get_trend_design_matrix of the reference
    (data_helpers.py:56-133, likelihood_helpers.py:8-37) restated: the epochs
    sorted by time, the ids left in concatenation order."""
    t = np.concatenate([d[0] for d in data_list])
    ids = np.concatenate([[k] * len(d[0]) for k, d in enumerate(data_list)])
    ts = np.sort(t, kind="stable")
    unq = np.unique(ids)
    const = np.zeros((len(t), len(unq)))
    const[:, 0] = 1.0
    for j, id_ in enumerate(unq[1:]):
        const[ids == id_, j + 1] = 1.0
    dt = ts - ts.min()
    return np.hstack((const, np.vander(dt, N=poly_trend, increasing=True)[:, 1:]))


@pytest.mark.parametrize("poly_trend", [1, 2])
def test_multi_survey_offsets_follow_the_reference_ids_order(poly_trend):
    """Interleaved surveys: the offset column follows the ids in concatenation
    order, as the reference builds it; ref_ids_order=False gives each epoch
    its own survey's column."""
    from thejoker_gb300.data import RVData, validate_prepare_data
    rng = np.random.default_rng(3)
    a = (np.sort(rng.uniform(0, 100, 7)) + 56000, rng.normal(0, 5, 7), np.full(7, 0.3))
    b = (np.sort(rng.uniform(0, 100, 5)) + 56000, rng.normal(0, 5, 5), np.full(5, 0.5))
    data = [RVData(*a), RVData(*b)]
    all_data, ids, trend = validate_prepare_data(data, poly_trend, 1)
    np.testing.assert_array_equal(trend, _reference_trend([a, b], poly_trend))
    np.testing.assert_array_equal(ids, [0] * 7 + [1] * 5)
    _, ids2, trend2 = validate_prepare_data(data, poly_trend, 1, ref_ids_order=False)
    t = np.concatenate([a[0], b[0]])
    own = np.concatenate([[0] * 7, [1] * 5])[np.argsort(t, kind="stable")]
    np.testing.assert_array_equal(ids2, own)
    np.testing.assert_array_equal(trend2[:, 1], (own == 1).astype(float))
    # the sorted epochs carry the velocities of their own survey
    np.testing.assert_array_equal(all_data.rv, np.concatenate([a[1], b[1]])[np.argsort(t)])
