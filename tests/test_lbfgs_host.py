"""The trainer's L-BFGS (aenet_gb300/lbfgs.py) on the host: convergence on
standard test functions, strong Wolfe steps, and a restart from the saved
state that continues the identical trajectory (train.restart semantics)."""
import numpy as np

from aenet_gb300.lbfgs import FTOL, GTOL, LBFGS


def rosenbrock(x):
    f = np.sum(100.0 * (x[1:] - x[:-1] ** 2) ** 2 + (1.0 - x[:-1]) ** 2)
    g = np.zeros_like(x)
    g[:-1] = -400.0 * x[:-1] * (x[1:] - x[:-1] ** 2) - 2.0 * (1.0 - x[:-1])
    g[1:] += 200.0 * (x[1:] - x[:-1] ** 2)
    return f, g


def test_converges_on_rosenbrock_and_quadratic():
    x0 = np.full(20, -1.2)
    x0[1::2] = 1.0
    opt = LBFGS(rosenbrock, x0, m=20)
    for _ in range(500):
        if np.abs(opt.g).max() < 1e-8 or not opt.step():
            break
    np.testing.assert_allclose(opt.x, 1.0, atol=1e-6)
    rng = np.random.default_rng(1)
    Q = rng.normal(size=(30, 30))
    A = Q @ Q.T + 30 * np.eye(30)
    b = rng.normal(size=30)
    opt = LBFGS(lambda x: (0.5 * x @ A @ x - b @ x, A @ x - b), np.zeros(30), m=5)
    for _ in range(200):
        if np.abs(opt.g).max() < 1e-10 or not opt.step():
            break
    np.testing.assert_allclose(opt.x, np.linalg.solve(A, b), atol=1e-8)


def test_steps_satisfy_the_strong_wolfe_conditions():
    x0 = np.linspace(-1, 1, 10)
    calls = []

    def fg(x):
        calls.append(x.copy())
        return rosenbrock(x)

    opt = LBFGS(fg, x0, m=7)
    for _ in range(15):
        x, f, g = opt.x.copy(), opt.f, opt.g.copy()
        d = opt.direction() if opt.S else -g
        assert opt.step()
        s = opt.x - x
        assert opt.f <= f + FTOL * (g @ s) + 1e-12
        assert abs(opt.g @ s) <= GTOL * abs(g @ s) + 1e-12
        assert np.linalg.norm(np.cross(s[:3], d[:3])) <= 1e-8 * np.linalg.norm(s) * np.linalg.norm(d) + 1e-14


def test_restart_continues_the_same_trajectory(tmp_path):
    x0 = np.full(12, 0.5)
    a = LBFGS(rosenbrock, x0, m=4)
    for _ in range(30):
        a.step()
    b = LBFGS(rosenbrock, x0, m=4)
    for _ in range(12):
        b.step()
    path = str(tmp_path / "train.restart")
    b.save(path)
    c = LBFGS.load(rosenbrock, path, m=4)
    for _ in range(18):
        c.step()
    assert c.k == a.k == 30
    np.testing.assert_array_equal(c.x, a.x)
    np.testing.assert_array_equal(c.g, a.g)
