"""CPU self-check of the NumPy MLP restatement used to verify the CUDA
training kernels: analytic gradient against central finite differences."""
import numpy as np


def test_mlp_reference_gradient_matches_finite_differences(orc, tg):
    import mlp_ref
    lg = tg.learned_guess
    rng = np.random.default_rng(0)
    p = lg.init_params(3).astype(np.float64)
    X = rng.normal(size=(40, 5))
    T = rng.normal(size=40)
    loss, g = mlp_ref.loss_grad(p, X, T)
    h = 1e-6
    for k in list(range(0, lg.N_TRAIN, 97)) + [lg.N_TRAIN - 1]:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mlp_ref.loss_grad(pp, X, T)[0] - mlp_ref.loss_grad(pm, X, T)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])), (k, fd, g[k])
