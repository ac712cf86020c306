"""The benchmark's held-out metrics against upstream's metric values at given scores
(tests/fixtures/metrics, which crates/lgbm-core/tests/golden_metrics.rs checks for the
reference): the AUC of binary scores, the L2 of regression scores and the multi-class log loss
of 4-class raw scores (class-major), to 1e-12 relative (the benchmark sums in another order)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

METRICS = os.path.join(GOLDEN, "metrics")


def _case(name):
    d = os.path.join(METRICS, name)
    score = np.load(os.path.join(d, "score.npy")).astype(np.float64)
    label = np.load(os.path.join(d, "label.npy")).astype(np.float32)  # labels are f32 (metadata)
    expected = dict(json.load(open(os.path.join(d, "expected.json"))))
    return score, label, expected


@pytest.fixture(scope="module")
def bench():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_auc(bench):
    torch = pytest.importorskip("torch")
    score, label, want = _case("binary")
    got = bench._auc(torch.tensor(score), torch.tensor(label))
    assert abs(got - want["auc"]) <= 1e-12 * want["auc"]


def test_l2(bench):
    torch = pytest.importorskip("torch")
    score, label, want = _case("reg")
    got = bench._l2(torch.tensor(score), torch.tensor(label))
    assert abs(got - want["l2"]) <= 1e-12 * want["l2"]


def test_multi_logloss(bench):
    torch = pytest.importorskip("torch")
    score, label, want = _case("multiclass")
    K = 4
    got = bench._multi_logloss(torch.tensor(score.reshape(K, -1)), torch.tensor(label))
    assert abs(got - want["multi_logloss"]) <= 1e-12 * want["multi_logloss"]
