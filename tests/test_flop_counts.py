"""The algorithmic operation counts bench.py divides by the kernel time
(ALGORITHMIC_OPS) against a fresh counting run of the oracle (CPU only): the
warm-bubble member and the covariant members are recomputed exactly; the
headline shell row is checked on a 4 x 4 x 2 shell of the same kind, whose
counts per DOF·stage differ from the 16 x 16 x 8 shell's only through the share
of faces and of pairs that take the logarithmic branch."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fc(orc):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import flop_counts
    return flop_counts


def test_counting_scalar_counts_a_known_formula(orc):
    """flux_ranocha of the 2D oracle on one pair: what the counting run sees
    for the volume phase of a one-element mesh agrees with a hand count of a
    CK2N54 step's stage updates (3 flops per value: k = A k + dt du, u += B k)."""
    import numpy as np
    u = np.zeros((1, 4, 4, 5))
    u[..., 0] = 1.2
    u[..., 3] = 2.5e5
    c = orc.count_euler2d_step(3, 1, 1, 0.0, 1.0, 0.0, 1.0, u)
    upd = c["stage_update"]
    assert upd["add"] == 5 * 2 * u.size and upd["mul"] == 5 * 3 * u.size
    assert upd["div"] == 0 and c["volume"]["add"] > 0


def test_bubble_and_covariant_rows_match_bench(tg, orc, fc):
    import bench
    got = {"bubble": fc.summary(fc.bubble_members(tg))}
    for variant in ("weak", "ec"):
        for N in (3, 5, 7):
            got[f"swe_{variant}_{N}"] = fc.summary(fc.swe(tg, variant, N))
    for key, row in got.items():
        for k, v in row.items():
            assert abs(v - bench.ALGORITHMIC_OPS[key][k]) <= 1e-3 * max(1.0, abs(v)), (key, k, v)


def test_shell_row_consistent_with_a_small_shell(tg, orc, fc):
    import bench
    small = fc.summary(fc.shell(tg, trees=4, layers=2))
    ref = bench.ALGORITHMIC_OPS["shell"]
    for k in ("total", "element", "div"):
        assert abs(small[k] / ref[k] - 1) < 5e-3, (k, small[k], ref[k])
