"""The GPU step's arithmetic (cuteflow_gb300/csrc/cf_flux.h, compiled here for the CPU
without FMA contraction, as the kernels are compiled with -fmad=false) against the oracle:
every (element, edge) flux and every full run must agree bit for bit."""
import numpy as np
import pytest

import harness as H
from cuteflow_gb300 import cases


def test_markstein_division_is_the_ieee_quotient():
    """The kernels replace a/d by Markstein's correction from y = RN(1/d) where 1/d is known;
    it must be the correctly rounded quotient, bit for bit, signed zeros included."""
    assert H.div_check(5_000_000, seed=1) == 0
    assert H.div_check(5_000_000, seed=2) == 0


def test_inverse_cube_root_is_the_oracles_and_within_an_ulp(oracle):
    """The friction term's h^(-1/3): the kernels' rcbrt (run here on the host) equals the
    oracle's bit for bit, and both are within 1 ulp of the exact power (mpmath, 130 bits) over
    the whole normal range, the depths a run meets, binade edges and the special values."""
    mpmath = pytest.importorskip("mpmath")
    rng = np.random.default_rng(11)
    n = 60_000
    bits = rng.integers(0, 1 << 52, n, dtype=np.uint64) | (
        rng.integers(1, 2047, n).astype(np.uint64) << np.uint64(52))
    x = np.concatenate([bits.view(np.float64), 10.0 ** rng.uniform(-7, 3, n),
                        2.0 ** np.arange(-1022, 1024, 1.0), np.nextafter(2.0 ** np.arange(-1000, 1000, 1.0), 0),
                        np.array([5e-324, 2.2e-308, 1e-310, 1.0, 8.0, 27.0, 0.125])])
    yk, yo = H.rcbrt(x), oracle.rcbrt(x)
    assert np.array_equal(yk.view(np.uint64), yo.view(np.uint64))
    mpmath.mp.prec = 130
    third = mpmath.mpf(-1) / 3
    worst = 0.0
    for xi, yi in zip(x[::3], yk[::3]):
        ex = mpmath.mpf(float(xi)) ** third
        worst = max(worst, float(abs(mpmath.mpf(float(yi)) - ex)) / np.spacing(float(ex)))
    assert worst <= 1.0, worst
    sp = np.array([0.0, -0.0, np.inf, -1.0, -np.inf, np.nan])
    for f in (H.rcbrt, oracle.rcbrt):
        got = f(sp)
        assert got[0] == np.inf and got[1] == -np.inf and got[2] == 0.0
        assert np.isnan(got[3:]).all()


def _state_after(oracle, case, n, params=None):
    r = oracle.run(case, n, params=params)
    return r["U"], r["dt_hist"][-1], r["t"]


@pytest.mark.parametrize("iflux", [1, 2, 3, 4])
@pytest.mark.parametrize("flux_mode", [0, 1])
def test_edge_fluxes_bitwise(oracle, iflux, flux_mode):
    c = cases.flooding(60, 30, seed=4, iflux=iflux)
    prm = dict(flux_mode=flux_mode)
    for n in (0, 25):
        U, dt, t = _state_after(oracle, c, n, prm) if n else (c.U0, 0.3, 0.0)
        fo = oracle.edge_fluxes(c, U, dt, t, params=prm)
        fh, _ = H.edge_fluxes(c, U, dt, t, params=prm)
        if flux_mode == 0:
            assert np.array_equal(fo, fh)
        else:
            # conservative mode: the element with the smaller index evaluates, the other negates
            bnd = oracle.setup(c)[0]
            own = (bnd[:, :, 0] <= 0) | (bnd[:, :, 0] - 1 > np.arange(c.nelt)[:, None])
            assert np.array_equal(fo[own], fh[own])


CASES = [
    ("dam_hllc", lambda: cases.circular_dam_break(30, 30, seed=3, iflux=1), 150, {}),
    ("dam_riadh", lambda: cases.circular_dam_break(30, 30, seed=3, iflux=2), 150, {}),
    ("dam_waf", lambda: cases.circular_dam_break(30, 30, seed=3, iflux=3), 150, {}),
    ("flood_hllc", lambda: cases.flooding(60, 30, seed=4, iflux=1), 200, {}),
    ("flood_riadh", lambda: cases.flooding(60, 30, seed=4, iflux=2), 200, {}),
    ("flood_waf", lambda: cases.flooding(60, 30, seed=4, iflux=3), 200, {}),
    ("flood_waf_conservative", lambda: cases.flooding(40, 20, seed=7, iflux=3), 150, dict(flux_mode=1)),
    ("waf_lim0", lambda: cases.flooding(40, 20, seed=6, iflux=3), 150, dict(ilimiteur=0)),
    ("waf_lim2", lambda: cases.flooding(40, 20, seed=6, iflux=3), 150, dict(ilimiteur=2)),
    ("waf_lim3", lambda: cases.flooding(40, 20, seed=6, iflux=3), 150, dict(ilimiteur=3)),
    ("waf_lim4", lambda: cases.flooding(40, 20, seed=6, iflux=3), 150, dict(ilimiteur=4)),
    ("dam_muscl", lambda: cases.circular_dam_break(30, 30, seed=3, iflux=4), 150, {}),
    ("flood_muscl", lambda: cases.flooding(60, 30, seed=4, iflux=4), 200, {}),
    ("muscl_lim0", lambda: cases.flooding(40, 20, seed=6, iflux=4), 150, dict(ilimiteur=0)),
    ("muscl_lim2", lambda: cases.flooding(40, 20, seed=6, iflux=4), 150, dict(ilimiteur=2)),
    ("muscl_lim3", lambda: cases.flooding(40, 20, seed=6, iflux=4), 150, dict(ilimiteur=3)),
    ("muscl_lim4_unset", lambda: cases.flooding(40, 20, seed=6, iflux=4), 100, dict(ilimiteur=4)),
    ("muscl_conservative", lambda: cases.flooding(40, 20, seed=7, iflux=4), 150, dict(flux_mode=1)),
    ("muscl_outlet_transm", lambda: cases.flooding(40, 20, seed=9, iflux=4), 120, dict(outlet=2)),
    ("lake_muscl", lambda: cases.lake_at_rest(30, 15, iflux=4), 100, {}),
    ("phys_inflow_hllc", lambda: cases.flooding(40, 20, seed=9, iflux=1), 150, dict(inlet=3)),
    ("phys_inflow_waf", lambda: cases.flooding(40, 20, seed=9, iflux=3), 150, dict(inlet=3)),
    ("phys_inflow_muscl", lambda: cases.flooding(40, 20, seed=9, iflux=4), 120, dict(inlet=3)),
    ("phys_inflow_dry_start", lambda: cases.flooding(18, 9, seed=22, lx=360.0, ly=180.0, iflux=3), 60,
     dict(inlet=3)),
    ("steady_stop_any", lambda: cases.channel(), 400, dict(tol_reg_perm=1.5, steady_count=30)),
    ("steady_stop_half", lambda: cases.channel(), 900, dict(tol_reg_perm=0.5, steady_count=20)),
    ("steady_stop_phys_inflow", lambda: cases.channel(inlet=3), 900, dict(tol_reg_perm=0.05, steady_count=50)),
    ("fric_explicit", lambda: cases.flooding(40, 20, seed=8, iflux=1), 120, dict(fricimplic=0)),
    ("fric_diag", lambda: cases.flooding(40, 20, seed=8, iflux=1), 120, dict(fricimplic=2)),
    ("no_friction", lambda: cases.flooding(40, 20, seed=8, iflux=3), 120, dict(friction=0)),
    ("inlet_transm_outlet_transm", lambda: cases.flooding(40, 20, seed=9, iflux=1), 120, dict(inlet=1, outlet=2)),
    ("outlet_transm_waf", lambda: cases.flooding(40, 20, seed=9, iflux=3), 120, dict(outlet=2)),
    ("constant_dt", lambda: cases.circular_dam_break(20, 20, seed=2, iflux=1), 60, dict(is_dt_constant=1, constant_dt=0.01)),
    ("lake_wet", lambda: cases.lake_at_rest(30, 15, iflux=3), 100, {}),
    # all dry at t=0: the first step runs with the 1e5 dt sentinel (the initial dt is not tested)
    ("dry_start_inflow", lambda: cases.flooding(18, 9, seed=22, lx=360.0, ly=180.0, iflux=3), 60, {}),
    ("lake_islands", lambda: cases.lake_at_rest(30, 15, iflux=3, wet=False), 100, {}),
]


@pytest.mark.parametrize("name,make,n,prm", CASES, ids=[c[0] for c in CASES])
def test_full_run_bitwise(oracle, name, make, n, prm):
    c = make()
    r1 = oracle.run(c, n, params=prm, check=False)
    r2 = H.run(c, n, params=prm)
    assert r2["nbhd_bad"] == 0
    assert r1["rc"] == r2["rc"]
    assert r1["steps"] == r2["steps"]
    assert np.array_equal(r1["dt_hist"], r2["dt_hist"])
    assert np.array_equal(r1["U"], r2["U"])
    assert r1["t"] == r2["t"]


XD_CASES = [c for c in CASES if c[0] in ("dam_hllc", "dam_riadh", "dam_waf", "flood_hllc", "flood_riadh", "flood_waf",
                                          "flood_waf_conservative", "waf_lim2", "waf_lim3", "outlet_transm_waf",
                                          "lake_wet", "dry_start_inflow", "phys_inflow_waf", "steady_stop_half",
                                          "dam_muscl", "flood_muscl", "muscl_lim2", "muscl_lim3",
                                          "muscl_conservative", "lake_muscl")]


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("name,make,n,prm", XD_CASES, ids=[c[0] for c in XD_CASES])
def test_full_run_bitwise_integer_pipes(oracle, name, make, n, prm, mode):
    """The edge arithmetic on GB300's integer pipes (exact integer comparisons, and exact integer
    products of the significands) runs the same IEEE operations: bit-identical runs."""
    c = make()
    r1 = oracle.run(c, n, params=prm, check=False)
    H.set_xd(mode)
    try:
        r2 = H.run(c, n, params=prm)
    finally:
        H.set_xd(0)
    assert r2["nbhd_bad"] == 0
    assert r1["rc"] == r2["rc"] and r1["steps"] == r2["steps"]
    assert np.array_equal(r1["dt_hist"], r2["dt_hist"])
    assert np.array_equal(r1["U"], r2["U"])
    assert r1["t"] == r2["t"]


@pytest.mark.parametrize("name", ["flood_waf", "flood_muscl", "flood_hllc", "dry_start_inflow", "lake_islands",
                                  "phys_inflow_waf"])
def test_dry_neighbourhood_shortcut_is_taken_and_exact(oracle, name):
    """The element kernel's shortcut for a dry element amid dry ones (its depth and its three
    neighbours' depths +0, three interior edges) skips reading its slots: on the wet/dry cases it
    is taken, every element that takes it has signed-zero slots (the general test passes on them),
    and the run is the oracle's bit for bit."""
    _, make, n, prm = next(c for c in CASES if c[0] == name)
    c = make()
    r1 = oracle.run(c, n, params=prm, check=False)
    r2 = H.run(c, n, params=prm)
    assert r2["nbhd_took"] > 0 and r2["nbhd_bad"] == 0
    assert np.array_equal(r1["U"], r2["U"]) and np.array_equal(r1["dt_hist"], r2["dt_hist"])


def test_integer_product_is_the_ieee_product():
    """em_mul (cf_xd.h) against the hardware product on adversarial operands: normal and
    near-overflow/underflow exponents, all-ones and near-all-ones significands, ties."""
    assert H.mul_check(2_000_000, seed=3) == 0


def test_dry_region_shortcuts_are_the_general_result():
    """The edge kernel's shortcut for two elements of depth +0 and the element kernel's shortcut
    for a dry element with zero slots return, bit for bit, what the general evaluation returns
    (signed zeros included) on adversarial inputs: random signs of g, nx, ny, len, beds with
    signed zeros, ties, infinities and NaN, wet upwind states, every scheme, limiter, flux mode,
    friction option and arithmetic type."""
    bad, took = H.dry_check(400_000, seed=7)
    assert took > 200_000
    assert bad == 0


def test_closed_form_hllc_reverse_edge_is_the_dual_derivative():
    """The reverse edge kernel's closed-form path for first-order HLLC (frame change, hydrostatic
    reconstruction, tangential velocities and bed sources by hand around a Dual<4> flux core)
    equals the edge differentiated in six Dual lanes, to round-off, on random wet, dry and nearly
    dry edges; nearly dry sides (raw and masked depths differ) are left to the six-lane path."""
    worst, took = H.adj_hllc_check(200_000, seed=11)
    assert took > 100_000
    assert worst < 1e-12, worst
