"""The oracle's logarithmic and Stolarsky means against exact values (CPU).

tests/golden/means_exact.json (written by tests/golden/make_means_fixture.py in
50-digit arithmetic) holds value pairs swept over f2 = ((y-x)/(y+x))^2 in
[1e-14, 0.2], dense on both sides of every branch threshold, at three
magnitudes.  The reference's forms (Trixi's ln_mean / inv_ln_mean /
stolarsky_mean, imported at src/TrixiAtmo.jl:37) are exact series below their
threshold and closed forms above; a closed form loses accuracy as the two
values approach each other (the logarithm of a ratio near 1 has condition
number 1/|log(y/x)|), so every bound below is a few ulp plus that condition
term.  The device forms are checked against the same fixture in
tests/test_gpu_means.py."""
import json
import math
import os

import numpy as np

EPS = np.finfo(np.float64).eps
HERE = os.path.dirname(os.path.abspath(__file__))


def fixture():
    with open(os.path.join(HERE, "golden", "means_exact.json")) as f:
        d = json.load(f)
    r = np.asarray(d["rows"])
    return {k: r[:, i] for i, k in enumerate(d["columns"])}, d["gamma"]


def rel(a, b):
    return np.abs(a - b) / np.abs(b)


def log_bound(x, y, ulps=4.0):
    """ulps plus the condition term of a closed form log(y/x) / (y - x)."""
    return EPS * (ulps + 2.0 / np.abs(np.log(y / x)))


def test_fixture_covers_every_threshold():
    F, _ = fixture()
    for c in (1e-4, 1e-2, 0.08, 0.09):
        assert np.sum((F["f2"] > 0.98 * c) & (F["f2"] < c)) >= 30
        assert np.sum((F["f2"] >= c) & (F["f2"] < 1.02 * c)) >= 30
    assert F["f2"].min() < 1e-13 and F["f2"].max() > 0.19


def test_oracle_means_against_exact(orc):
    F, gamma = fixture()
    x, y = F["x"], F["y"]
    ln = np.array([orc.ln_mean(a, b) for a, b in zip(x, y)])
    iln = np.array([orc.inv_ln_mean(a, b) for a, b in zip(x, y)])
    short = F["f2"] < 1e-4
    assert np.all(rel(ln[short], F["ln_mean"][short]) <= 4 * EPS)
    assert np.all(rel(iln[short], F["inv_ln_mean"][short]) <= 4 * EPS)
    assert np.all(rel(ln, F["ln_mean"]) <= log_bound(x, y))
    assert np.all(rel(iln, F["inv_ln_mean"]) <= log_bound(x, y))
    g = gamma[0] / gamma[1]
    st = np.array([orc.stolarsky(a, b, g) for a, b in zip(x, y)])
    series = F["f2"] < 1e-2
    assert np.all(rel(st[series], F["stolarsky_mean"][series]) <= 4 * EPS)
    t = np.sqrt(F["f2"])
    assert np.all(rel(st[~series], F["stolarsky_mean"][~series]) <= EPS * (8 + 4 / t[~series]))
    # the closed forms the thresholds switch to are continuous with the series
    for c in (1e-4, 1e-2):
        below = (F["f2"] > 0.98 * c) & (F["f2"] < c)
        above = (F["f2"] >= c) & (F["f2"] < 1.02 * c)
        assert rel(ln[below], F["ln_mean"][below]).max() <= 4 * EPS + 2 * EPS / (2 * math.sqrt(c))
        assert rel(ln[above], F["ln_mean"][above]).max() <= 4 * EPS + 2 * EPS / (2 * math.sqrt(c))


def _device_polynomial(src, name):
    """Coefficients c0, c1, ... of `TAG_DEV double name(double f2)` in
    tag_common.cuh, written as Horner steps from the highest one down."""
    import re
    body = re.search(r"TAG_DEV double " + name + r"\(double f2\) \{(.*?)\n\}", src, re.S).group(1)
    nums = [float(v) for v in re.findall(r"(-?\d+\.\d+(?:e-?\d+)?)", body)]
    assert nums[-1] == 1.0  # the final fma(r, f2, 1.0)
    return nums[:-1][::-1]


def test_device_series_coefficients_are_the_economized_ones():
    """The polynomial forms of R(f2) = z/atanh z and Q(f2) = atanh z / z in
    csrc/tag_common.cuh are the Chebyshev economizations that
    csrc/log_mean_series.py computes, and each is exact to well below an ulp
    over its range (50-digit evaluation of the rounded coefficients)."""
    import importlib.util
    root = os.path.dirname(HERE)
    csrc = os.path.join(root, "trixiatmo.jl_gb300", "csrc")
    spec = importlib.util.spec_from_file_location("log_mean_series",
                                                  os.path.join(csrc, "log_mean_series.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    with open(os.path.join(csrc, "tag_common.cuh")) as f:
        src = f.read()
    names = {("R", "0.09"): "ln_series_R_long", ("Q", "0.09"): "ln_series_Q_long",
             ("R", "0.01"): "ln_series_R", ("Q", "0.01"): "ln_series_Q"}
    for _, fun, F, m in gen.FORMS:
        dev = _device_polynomial(src, names[(fun, F)])
        assert dev == gen.coefficients(fun, F, m), (fun, F)
        assert gen.max_rel_error(fun, F, dev, samples=400) < 4e-18
