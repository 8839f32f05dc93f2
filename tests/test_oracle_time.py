"""The oracle's SSP time integrators (SSPRK43, SSPRK33 in Shu-Osher form) are
third order: on the smooth dry convergence problem of the moist equations
(manufactured source, periodic unit square) the difference between runs at
dt, dt/2 and dt/4 shrinks by 2^3.  CarpenterKennedy2N54 is checked the same
way at fourth order.  These pin the stage coefficients the GPU integrators
are compared with."""
import numpy as np
import pytest


def _case(orc):
    return orc.Moist2D(3, 4, 4, 0.0, 2.0, 0.0, 2.0, True, True, weak_form=True, surface_kind=1,
                       source_kind=3, gravity=0.0, ic_kind=1)


def _run(orc, scheme, nsteps, t_end):
    c = _case(orc)
    u = np.ascontiguousarray(c.initial_condition(0.0))
    dt = t_end / nsteps
    if scheme == 0:
        t = c.ck_steps(u, np.zeros_like(u), 0.0, 1.0, nsteps, fixed_dt=dt)
    else:
        t = c.ssp_steps(u, 0.0, 1.0, nsteps, scheme, fixed_dt=dt)
    assert abs(t - t_end) < 1e-12
    return u


@pytest.mark.parametrize("scheme,order", [(1, 3), (2, 3), (0, 4)])
def test_time_integrator_order(orc, scheme, order):
    t_end = 0.05
    u = [_run(orc, scheme, m, t_end) for m in (8, 16, 32)]
    e1 = np.abs(u[0] - u[1]).max()
    e2 = np.abs(u[1] - u[2]).max()
    rate = np.log2(e1 / e2)
    assert abs(rate - order) < 0.35, rate


def test_ssp_steps_land_on_t_end(orc):
    """The last step is shortened to reach t_end exactly (OrdinaryDiffEq's
    tstops behaviour with a StepsizeCallback)."""
    c = _case(orc)
    u = np.ascontiguousarray(c.initial_condition(0.0))
    dt = c.max_dt(u)
    t_end = 2.5 * dt
    t = c.ssp_steps(u, 0.0, 1.0, 100, 1, t_end=t_end)
    assert t == t_end
