"""The oracle reproduces the committed golden vectors (tests/golden/)."""
import numpy as np
import pytest


def test_assign_golden(oracle, golden):
    lab, dist = oracle.assign(golden["assign_X"], golden["assign_C"], return_dist=True)
    np.testing.assert_array_equal(lab, golden["assign_labels"])
    np.testing.assert_array_equal(dist, golden["assign_dist"])


def test_wide_golden(oracle, golden):
    np.testing.assert_array_equal(oracle.assign(golden["wide_X"], golden["wide_C"]), golden["wide_labels"])


def test_ties_golden(oracle, golden):
    np.testing.assert_array_equal(oracle.assign(golden["tie_X"], golden["tie_C"]), golden["tie_labels"])
    np.testing.assert_array_equal(golden["tie_labels"], [0, 4, 1, 0, 3, 1, 0, 4])


def test_blobs_golden(oracle, golden):
    np.testing.assert_array_equal(oracle.assign(golden["blobs_X"], golden["blobs_C"]),
                                  np.arange(5000) // 1000)


def test_update_golden(oracle, golden):
    Cn, counts, cost, _ = oracle.update(golden["assign_X"], golden["assign_labels"], golden["assign_C"])
    np.testing.assert_array_equal(Cn, golden["update_C"])
    np.testing.assert_array_equal(counts, golden["update_counts"])
    assert cost == golden["update_cost"][0]


def test_lloyd_golden(oracle, golden):
    r = oracle.lloyd(golden["lloyd_X"], golden["lloyd_C0"], 100, 1e-5)
    assert r["n_iter"] == golden["lloyd_n_iter"][0]
    assert int(r["converged"]) == golden["lloyd_converged"][0]
    np.testing.assert_array_equal(r["centers"], golden["lloyd_C"])
    np.testing.assert_array_equal(r["labels"], golden["lloyd_labels"])
    np.testing.assert_array_equal(r["inertias"], golden["lloyd_inertias"])


def test_kmpp_golden(oracle, golden):
    C, idx = oracle.kmpp(golden["kmpp_X"], 20, int(golden["kmpp_seed"][0]))
    np.testing.assert_array_equal(idx, golden["kmpp_idx"])
    np.testing.assert_array_equal(C, golden["kmpp_X"][idx])


def test_make_golden_reproduces_the_fixtures(oracle, golden, monkeypatch):
    # the committed generator, run again, gives the committed arrays
    pytest.importorskip("sklearn")
    import os
    import runpy
    captured = {}
    monkeypatch.setattr(np, "savez_compressed", lambda path, **kw: captured.update(kw))
    root = os.path.dirname(os.path.abspath(__file__))
    runpy.run_path(os.path.join(root, "golden", "make_golden.py"), run_name="__main__")
    assert set(captured) == set(golden)
    for key, value in golden.items():
        np.testing.assert_array_equal(captured[key], value, err_msg=key)
