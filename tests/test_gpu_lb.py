"""Lower-bound producers (DtwKeoghLowerBound, DtwKimLowerBound) on the GPU.

Parity: the reference's outputs (golden fixtures made by running it) and the
CPU oracle on larger seeded cases; bounds within 1e-12 relative (the
reference's operations in its order), and argmin_distance driven by the
bounds returns the oracle's indices exactly.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from tests import _golden  # noqa: E402
from wildboar_gb300.distance import argmin_distance  # noqa: E402
from wildboar_gb300.distance.lb import DtwKeoghLowerBound, DtwKimLowerBound  # noqa: E402

RTOL = 1e-12


def _cases(kind):
    cs = _golden.cases(kind)
    return pytest.mark.parametrize("case", cs, ids=[c["name"] for c in cs])


@_cases("lb_keogh")
def test_lb_keogh_golden(case):
    a, inp, out = case["args"], case["inputs"], case["outputs"]
    lbk = DtwKeoghLowerBound(r=a["r"], kind=a["kind"]).fit(inp["x"])
    np.testing.assert_array_equal(lbk.lower_, out["lower"])
    np.testing.assert_array_equal(lbk.upper_, out["upper"])
    np.testing.assert_allclose(lbk.transform(inp["q"]), out["out"], rtol=RTOL, atol=0)


@_cases("lb_kim")
def test_lb_kim_golden(case):
    inp = case["inputs"]
    got = DtwKimLowerBound().fit(inp["x"]).transform(inp["q"])
    np.testing.assert_allclose(got, case["outputs"]["out"], rtol=RTOL, atol=0)


@pytest.mark.parametrize("r,kind", [(0.1, "both"), (0.02, "left"), (0.5, "right"),
                                    (1.0, "both")])
def test_lb_keogh_vs_oracle(r, kind):
    rng = np.random.default_rng(12)
    X = np.cumsum(rng.standard_normal((333, 200)), axis=1)
    X[7, 50:90] = X[7, 50]
    Q = np.cumsum(rng.standard_normal((37, 200)), axis=1)
    got = DtwKeoghLowerBound(r=r, kind=kind).fit(X).transform(Q)
    np.testing.assert_allclose(got, O.lb_keogh(Q, X, r=r, kind=kind), rtol=RTOL, atol=0)


def test_lb_kim_vs_oracle():
    rng = np.random.default_rng(13)
    X = np.cumsum(rng.standard_normal((300, 64)), axis=1)
    Q = np.cumsum(rng.standard_normal((41, 64)), axis=1)
    got = DtwKimLowerBound().fit(X).transform(Q)
    np.testing.assert_allclose(got, O.lb_kim(Q, X), rtol=RTOL, atol=0)


def test_argmin_with_keogh_bound_vs_oracle():
    rng = np.random.default_rng(14)
    X = np.cumsum(rng.standard_normal((120, 80)), axis=1)
    Q = np.cumsum(rng.standard_normal((15, 80)), axis=1)
    lb = DtwKeoghLowerBound(r=0.1).fit(X).transform(Q)
    idx, dist = argmin_distance(Q, X, k=3, metric="dtw", metric_params={"r": 0.1},
                                lower_bound=lb, return_distance=True)
    oi, od = O.argmin(Q, X, k=3, metric="dtw", metric_params={"r": 0.1}, lower_bound=lb)
    np.testing.assert_array_equal(idx, oi)
    np.testing.assert_allclose(dist, od, rtol=RTOL, atol=0)
