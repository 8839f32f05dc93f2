"""Writes tests/golden/means_exact.json: value pairs (x, y) with the exact
logarithmic mean ln_mean(x, y) = (y - x) / log(y / x), its inverse, and the
Stolarsky mean (gamma - 1)/gamma (y^gamma - x^gamma) / (y^(gamma-1) - x^(gamma-1))
of the potential-temperature equations (gamma = 1004/717), each evaluated in
50-digit arithmetic from the exact double inputs and rounded to double.

The pairs sweep f2 = ((y - x)/(y + x))^2 over [1e-14, 0.2], log-spaced, with
dense clusters on both sides of every threshold the device forms branch at
(1e-4, 1e-2, 0.08, 0.09), at three magnitudes of x (a density ~1, an inverse
temperature-like rho/p ~ 1e-5, a weighted potential temperature ~ 300).
Needs mpmath (this container); the GPU machine only reads the JSON.

    python tests/golden/make_means_fixture.py
"""
import json
import os

import mpmath as mp
import numpy as np

mp.mp.dps = 50
GAMMA = mp.mpf(1004) / 717


def pairs():
    rng = np.random.default_rng(20261204)
    f2 = list(np.logspace(-14, np.log10(0.2), 240))
    for c in (1e-4, 1e-2, 0.08, 0.09):
        f2 += list(c * (1 + np.linspace(-0.02, 0.02, 41)))
    out = []
    for scale in (1.0, 1.3e-5, 300.0):
        for v in f2:
            x = float(scale * (0.5 + rng.random()))
            t = float(np.sqrt(v))
            y = x * (1 + t) / (1 - t)
            if rng.random() < 0.5:
                x, y = y, x
            out.append((x, y))
    return out


def exact(x, y):
    X, Y = mp.mpf(x), mp.mpf(y)
    ln = (Y - X) / mp.log(Y / X)
    st = (GAMMA - 1) / GAMMA * (Y ** GAMMA - X ** GAMMA) / (Y ** (GAMMA - 1) - X ** (GAMMA - 1))
    return float(ln), float(1 / ln), float(st)


def main():
    rows = []
    for x, y in pairs():
        ln, iln, st = exact(x, y)
        f2 = ((y - x) / (y + x)) ** 2
        rows.append([x, y, f2, ln, iln, st])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "means_exact.json")
    with open(path, "w") as f:
        json.dump({"gamma": [1004.0, 717.0], "columns": ["x", "y", "f2", "ln_mean", "inv_ln_mean",
                                                         "stolarsky_mean"], "rows": rows}, f)
    print(f"wrote {len(rows)} pairs to {path}")


if __name__ == "__main__":
    main()
