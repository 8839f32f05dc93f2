"""The device forms of the logarithmic and Stolarsky means against exact values,
through the C ABI (tag_eval_means runs the kernels' own inline functions).

Every form is a series below a threshold of f2 = ((y-x)/(y+x))^2 and a closed
form above it; the fixture (tests/golden/means_exact.json) sweeps f2 over
[1e-14, 0.2] with clusters on both sides of each threshold (1e-4, 1e-2, 0.08,
0.09), so a form that were wrong or discontinuous at its switch would show
there.  Bounds: in a series range a few ulp (the series are exact to < 1e-17
there); above it the condition number of the closed form: log(y/x) / (y-x) has
1/|log(y/x)|, a difference of per-node logarithms log y - log x has
max(|log x|, |log y|) / |log(y/x)|, and the Stolarsky form's differences of
powers have about 1/t with t = |y-x|/(y+x)."""
import numpy as np
import pytest

from test_means import EPS, fixture, log_bound, rel

pytestmark = pytest.mark.gpu


def device(tg, kind, x, y, gamma):
    L = tg._lib.load()
    n = len(x)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    o1, o2 = np.zeros(n), np.zeros(n)
    dp = lambda a: a.ctypes.data_as(tg._lib._dp)  # noqa: E731
    tg._lib.check(L.tag_eval_means(kind, n, gamma[0], gamma[1], dp(x), dp(y), dp(o1), dp(o2)))
    return o1, o2


def node_log_bound(x, y, halved=False):
    lx, ly = np.log(0.5 * x if halved else x), np.log(0.5 * y if halved else y)
    return EPS * (6.0 + 2.0 * np.maximum(np.abs(lx), np.abs(ly)) / np.abs(ly - lx))


@pytest.mark.parametrize("kind,series_f2,node_logs", [(0, 1e-2, False), (1, 1e-2, True),
                                                      (2, 0.09, True), (3, 1e-2, False)])
def test_device_log_means_against_exact(tg, gpu_lib, orc, kind, series_f2, node_logs):
    F, gamma = fixture()
    x, y, f2 = F["x"], F["y"], F["f2"]
    ln, iln = device(tg, kind, x, y, gamma)
    series = f2 < series_f2
    for got, ex in ((ln, F["ln_mean"]), (iln, F["inv_ln_mean"])):
        assert np.all(rel(got[series], ex[series]) <= 6 * EPS), rel(got[series], ex[series]).max()
        bound = node_log_bound(x, y, kind == 2) if node_logs else log_bound(x, y, 6.0)
        assert np.all(rel(got[~series], ex[~series]) <= bound[~series])
    # where both are exact series, the device agrees with the oracle's
    # definitions (Trixi's four-term form) to a few ulp
    short = f2 < 1e-4
    o = np.array([orc.ln_mean(a, b) for a, b in zip(x[short], y[short])])
    oi = np.array([orc.inv_ln_mean(a, b) for a, b in zip(x[short], y[short])])
    assert rel(ln[short], o).max() <= 8 * EPS and rel(iln[short], oi).max() <= 8 * EPS


@pytest.mark.parametrize("kind", [5, 6])
def test_device_halved_means_take_separate_forms(tg, gpu_lib, kind):
    """The 3D kernel's halved pair form chooses each mean's form from that
    mean's own f2: with the other mean's pair equal (f2 = 0, the short form),
    the swept mean still meets its bounds on both sides of every threshold."""
    F, gamma = fixture()
    x, y, f2 = F["x"], F["y"], F["f2"]
    m, im = device(tg, kind, x, y, gamma)
    got, other, ex = (m, im, F["ln_mean"]) if kind == 5 else (im, m, F["inv_ln_mean"])
    series = f2 < 0.09
    assert np.all(rel(got[series], ex[series]) <= 6 * EPS), rel(got[series], ex[series]).max()
    bound = node_log_bound(x, y, True)
    assert np.all(rel(got[~series], ex[~series]) <= bound[~series])
    assert np.abs(other - 1.0).max() <= 2 * EPS


def test_device_stolarsky_mean_against_exact(tg, gpu_lib):
    F, gamma = fixture()
    st, _ = device(tg, 4, F["x"], F["y"], gamma)
    ex, f2 = F["stolarsky_mean"], F["f2"]
    series = f2 < 1e-2
    assert np.all(rel(st[series], ex[series]) <= 6 * EPS), rel(st[series], ex[series]).max()
    t = np.sqrt(f2[~series])
    assert np.all(rel(st[~series], ex[~series]) <= EPS * (8.0 + 8.0 / t))


def test_eval_means_rejects_bad_kind(tg, gpu_lib):
    L = tg._lib.load()
    z = np.zeros(1)
    dp = z.ctypes.data_as(tg._lib._dp)
    assert L.tag_eval_means(9, 1, 1004.0, 717.0, dp, dp, dp, dp) == tg._lib.TAG_E_INVALID
