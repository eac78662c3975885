"""The seeded case generator: sizes of the benchmark workloads, determinism, orientation."""
import numpy as np
import pytest

from cuteflow_gb300 import cases


def _signed_area(c):
    t = c.tri - 1
    x, y = c.x[t], c.y[t]
    return 0.5 * ((x[:, 1] - x[:, 0]) * (y[:, 2] - y[:, 0]) - (x[:, 2] - x[:, 0]) * (y[:, 1] - y[:, 0]))


def test_benchmark_sizes():
    assert cases.circular_dam_break().nelt == 80000
    f = cases.flooding(1000, 500)
    assert f.nelt == 1000000 and f.nnt == 1001 * 501


def test_ccw_and_jitter_bounds():
    c = cases.flooding(50, 25, seed=9)
    assert (_signed_area(c) > 0).all()
    dx = 2000.0 / 50
    gx = np.tile(np.arange(51), 26) * dx
    assert np.abs(c.x - gx).max() <= 0.2 * dx + 1e-9
    # boundary nodes stay on the rectangle
    assert np.isclose(c.x.min(), 0) and np.isclose(c.x.max(), 2000) and np.isclose(c.y.max(), 1000)


def test_deterministic():
    a = cases.flooding(40, 20, seed=3)
    b = cases.flooding(40, 20, seed=3)
    assert np.array_equal(a.x, b.x) and np.array_equal(a.tri, b.tri) and np.array_equal(a.manning, b.manning)
    c = cases.flooding(40, 20, seed=4)
    assert not np.array_equal(a.x, c.x)


def test_flooding_inputs_follow_the_spec():
    c = cases.flooding(200, 100, seed=2)
    assert 0.01 <= c.manning.min() and c.manning.max() <= 0.1
    assert abs(np.median(c.manning) - 0.03) < 0.003
    zc = cases.cell_bed(c.x, c.y, c.z, c.tri)
    wet = c.U0[:, 0] > 0
    assert np.allclose((c.U0[:, 0] + zc)[wet], 1.0)
    assert (zc[~wet] >= 1.0 - 1e-4).all()
    assert c.params["debitglob"][0] == 10.0 * 1000.0 and c.params["debitglob_start"][0] == 2.0 * 1000.0


def test_ensemble_members_are_flooding_cases():
    """Ensemble members come from the flooding generator: bathymetry (not flat), still water at
    1 m, an inflow ramp from 2 m^2/s to the member's peak in [2, 15] m^2/s, the fixed 1 m outflow."""
    for i in (0, 5, 17):
        c = cases.ensemble_member(i)
        ly = 2.0 * c.ny
        assert np.ptp(np.asarray(c.z)) > 0.1
        assert c.params["debitglob_start"][0] == 2.0 * ly
        assert 2.0 * ly <= c.params["debitglob"][0] <= 15.0 * ly
        assert c.params["h_sortie"] == [1.0] and c.params["iflux"] == 3
        h = c.U0[:, 0]
        assert h.max() <= 1.0 and (h > 0).any()


def test_ensemble_sizes_span_range():
    n = [cases.ensemble_member(i).nelt for i in range(0, 256, 16)]
    assert min(n) >= 15000 and max(n) <= 560000
    assert max(n) / min(n) > 5


def test_generator_functions_are_accurate_fixed_sequences():
    """det_exp / det_log / det_cos2pi (the generators' elementary functions: plain float64 operation
    sequences, so every machine builds the same inputs from a seed) within 4 ulp of the exact values
    (mpmath) over the ranges the generators use."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 120
    rng = np.random.default_rng(3)
    xe = np.concatenate([rng.uniform(-700.0, 0.0, 3000), rng.uniform(-3.0, 3.0, 3000)])
    xl = np.concatenate([10.0 ** rng.uniform(-300, 0, 3000), rng.uniform(0.5, 30.0, 3000)])
    xc = rng.uniform(0.0, 1.0, 6000)
    for f, xs, ref in ((cases.det_exp, xe, mpmath.exp), (cases.det_log, xl, mpmath.log),
                       (cases.det_cos2pi, xc, lambda u: mpmath.cos(2 * mpmath.pi * u))):
        got = f(xs)
        for x, g in zip(xs, got):
            r = float(ref(mpmath.mpf(float(x))))
            assert abs(g - r) <= 4 * np.spacing(max(abs(r), 1e-300)) + (1e-16 if f is cases.det_cos2pi else 0.0), (f, x, g, r)
    # the same value for an element wherever it sits in the array
    assert np.array_equal(cases.det_exp(xe)[::7], cases.det_exp(xe[::7].copy()))
