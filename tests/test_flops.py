"""The algorithmic operation counter (oracle/flops.py) behind the bench's
FP32 roofline: known answers on small expressions, and the per-ray count
frozen in profiles/trace_precision_1e8.json equal to a fresh count."""

import json
import pathlib

import numpy as np
import pytest

from optika_gb300 import configs
from oracle import flops as F

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _count(fn, *arrays):
    F.COUNTS.clear()
    fn(*(np.asarray(a, dtype=np.result_type(a, np.float64)).view(F.Counted) for a in arrays))
    out = dict(F.COUNTS)
    F.COUNTS.clear()
    return out


def test_trivial_operations_are_free():
    x = np.array([2.0, 3.0, 0.0, 1.0])
    c = _count(lambda a: a * 1.0 + 0.0, x)
    assert c.get("flops", 0) == 0
    c = _count(lambda a: a * 3.0 + 2.0, x)
    # products by 0 and 1 are free (2 count); so is the sum with the zero
    # product (3 count)
    assert c["flops"] == 2 + 3
    c = _count(lambda a, b: a * b, np.array([2.0, -1.0, 5.0]), np.array([3.0, 4.0, 0.0]))
    assert c["flops"] == 1


def test_complex_and_matrix_counts():
    a = np.array([1.5 + 2.0j])
    b = np.array([0.5 - 3.0j])
    assert _count(lambda x, y: x * y, a, b)["flops"] == 6
    assert _count(lambda x, y: x + y, a, b)["flops"] == 2
    c = _count(lambda x, y: x / y, a, b)
    assert c["flops"] == 9 and c["div"] == 2
    # a 2 x 2 product with the identity costs nothing
    m = np.array([[[1.5 + 1j, 2.0], [0.3j, 4.0 - 1j]]])
    eye = np.eye(2, dtype=complex)[None]
    assert _count(lambda x, y: x @ y, m, eye).get("flops", 0) == 0
    full = _count(lambda x, y: x @ y, m, m)["flops"]
    assert 0 < full <= 4 * (2 * 6 + 2)
    c = _count(lambda x: np.sqrt(x) + np.exp(x), np.array([2.0, 3.0]))
    assert c["special"] == 4 and c["flops"] == 2


def test_frozen_count_matches_the_counter():
    frozen = json.loads((ROOT / "profiles" / "trace_precision_1e8.json").read_text())
    c = F.count_rayfunction(configs.newtonian(coated=True), configs.precision_grid(20000))
    assert c["flops"] == pytest.approx(frozen["algorithmic_flops_per_ray"], rel=2e-3)
    assert c["div"] == pytest.approx(frozen["algorithmic_div_per_ray"], rel=2e-3)
    assert c["special"] == pytest.approx(frozen["algorithmic_special_per_ray"], rel=2e-3)


def test_count_does_not_change_the_oracle():
    from oracle import trace as O

    s = configs.newtonian(coated=True)
    g = configs.precision_grid(500)
    plain = O.rayfunction(s, **g)
    F.count_rayfunction(s, g)
    again = O.rayfunction(s, **g)
    for k in ("px", "py", "opl", "intensity"):
        assert np.array_equal(plain[k], again[k], equal_nan=True)


def test_frozen_workload_counts_match_the_counter():
    from oracle import freeze_counts

    frozen = json.loads((ROOT / "profiles" / "algorithmic_counts.json").read_text())
    for name, fresh in (("batched-spectrograph", freeze_counts.batched_counts(2, 1000)),
                        ("multilayer-periodic", freeze_counts.multilayer_counts(2, 1000))):
        for k in ("flops", "div", "special"):
            assert fresh[k] == pytest.approx(frozen[name][k], rel=1e-2), (name, k)
