"""GPU step against the CPU oracle on the same seeded inputs, through the C ABI.

The bar stated for this path is max |h - h_ref| <= 1e-9 m and |hu|, |hv| <= 1e-9 m^2/s after
the stated step count.  The kernels evaluate the reference's operations in its order without
FMA contraction, so the tests require more: the GPU state, every dt and the time must equal
the oracle's bit for bit (TOL is only reported in the failure message).
"""
import ctypes as C

import numpy as np
import pytest

from cuteflow_gb300 import _abi, cases

pytestmark = pytest.mark.gpu

TOL = 1e-9


def run_gpu(case, nsteps, params=None, U0=None, chunks=(None,)):
    from cuteflow_gb300 import Solver
    with Solver(case, params) as s:
        s.set_state(case.U0 if U0 is None else U0)
        info = None
        done = 0
        sizes = [c for c in chunks if c] or [nsteps]
        i = 0
        while done < nsteps:
            k = min(sizes[i % len(sizes)], nsteps - done)
            info = s.step(k, check=False)
            done += k
            i += 1
        return s.get_state(), info


def compare_bitwise(case, nsteps, oracle, params=None, chunks=(None,)):
    U, info = run_gpu(case, nsteps, params, chunks=chunks)
    ref = oracle.run(case, nsteps, params=params, check=False)
    d = np.abs(U - ref["U"]).max(axis=0)
    assert info.steps == nsteps or ref["rc"] != 0
    assert np.array_equal(U, ref["U"]), f"{case.name}: max|dU| = {d} (bar {TOL})"
    assert info.t == ref["t"], (info.t, ref["t"])
    assert info.dt_next == ref["dt_hist"][info.steps]
    return U, ref, info


@pytest.mark.parametrize("iflux", [1, 2, 3, 4])
def test_dam_break(gpu_lib, oracle, iflux):
    compare_bitwise(cases.circular_dam_break(40, 40, seed=3, iflux=iflux), 200, oracle)


@pytest.mark.parametrize("iflux", [1, 2, 3, 4])
def test_flooding_wet_dry(gpu_lib, oracle, iflux):
    compare_bitwise(cases.flooding(80, 40, seed=4, iflux=iflux), 300, oracle, chunks=(7, 100, 1, 50))


@pytest.mark.parametrize("ilim", [0, 1, 2, 3, 4])
def test_waf_limiters(gpu_lib, oracle, ilim):
    compare_bitwise(cases.flooding(60, 30, seed=6, iflux=3), 200, oracle, params=dict(ilimiteur=ilim))


@pytest.mark.parametrize("ilim", [0, 1, 2, 3, 4])
def test_muscl_limiters(gpu_lib, oracle, ilim):
    """MUSCL-Hancock (iflux 4) with every simple_limiter; ilimiteur 4 leaves the reference's
    slope unset, defined as no slope on both sides."""
    compare_bitwise(cases.flooding(60, 30, seed=6, iflux=4), 200, oracle, params=dict(ilimiteur=ilim))


@pytest.mark.parametrize("iflux", [1, 3, 4])
def test_conservative_mode(gpu_lib, oracle, iflux):
    compare_bitwise(cases.flooding(60, 30, seed=7, iflux=iflux), 200, oracle, params=dict(flux_mode=1))


@pytest.mark.parametrize("prm", [dict(fricimplic=2), dict(friction=0), dict(inlet=1, outlet=2),
                                 dict(outlet=2), dict(is_dt_constant=1, constant_dt=0.05)],
                         ids=["fric_diag", "no_friction", "transm_in_out", "transm_out", "constant_dt"])
@pytest.mark.parametrize("iflux", [3, 4])
def test_options(gpu_lib, oracle, prm, iflux):
    compare_bitwise(cases.flooding(50, 25, seed=8, iflux=iflux), 150, oracle, params=prm)


def test_explicit_friction_stops_like_the_reference(gpu_lib, oracle):
    """Explicit friction (fricimplic=0) is unstable on this case: dt leaves the reference's
    sane range (cfl_condition.cuf:129-132).  Both stop at the same step with the same state."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(40, 20, seed=8, iflux=1)
    ref = oracle.run(c, 120, params=dict(fricimplic=0), check=False)
    assert ref["rc"] == -2
    with Solver(c, dict(fricimplic=0)) as s:
        s.set_state(c.U0)
        info = s.step(120, check=False)
        assert info.status & _abi.CF_STATUS_DT_RANGE
        U = s.get_state()
        with pytest.raises(Exception):
            s.step(1)
    assert np.array_equal(U, ref["U"])
    assert info.t == ref["t"]


def test_advance_chained_is_the_continuous_run(gpu_lib, oracle):
    """cf_advance (state in, steps, state out, one wait), chained as a coupling host would chain it
    (each call from the returned state at the returned time, in place or not): the continuous run,
    bit for bit."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(60, 30, seed=8, iflux=3)
    ref = oracle.run(c, 30)
    with Solver(c) as s:
        U, t = np.array(c.U0), 0.0
        for k in (7, 0, 13, 10):
            U, info = s.advance(U, t, k)
            t = info.t
        assert np.array_equal(U, ref["U"]) and t == ref["t"] and info.steps == 10


def test_advance_returns_a_stopped_state_like_the_three_calls(gpu_lib, oracle):
    """A member that stops inside cf_advance (the reference's dt-range test) returns the state where
    it stopped and the same code as cf_set_state + cf_step + cf_get_state: the state's buffer is
    chosen on the device."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(40, 20, seed=8, iflux=1)
    ref = oracle.run(c, 120, params=dict(fricimplic=0), check=False)
    with Solver(c, dict(fricimplic=0)) as s:
        U, info = s.advance(c.U0, 0.0, 120, check=False)
        rc = s._L.cf_advance(s._ctx, np.ascontiguousarray(c.U0).ctypes.data_as(C.POINTER(C.c_double)), 0.0, 120,
                             np.empty_like(c.U0).ctypes.data_as(C.POINTER(C.c_double)), None)
    assert rc == _abi.CF_EDT and info.status & _abi.CF_STATUS_DT_RANGE
    assert np.array_equal(U, ref["U"]) and info.t == ref["t"]


def test_advance_with_pinned_buffers_writes_the_last_step_or_the_stopped_state(gpu_lib, oracle):
    """cf_advance into pinned host memory: the last step's element kernel writes the caller's buffer
    itself; a member that stopped before it (the dt-range test) gets its stopped state from the
    store kernel instead; a call of zero steps returns the state it was given.  Each is the
    oracle's state bit for bit."""
    import ctypes
    torch = pytest.importorskip("torch")
    from cuteflow_gb300 import Solver
    dp = ctypes.POINTER(ctypes.c_double)
    c = cases.flooding(40, 20, seed=8, iflux=1)
    for prm, n in ((dict(fricimplic=0), 120), ({}, 35), ({}, 0)):
        ref = oracle.run(c, n, params=prm, check=False)
        with Solver(c, prm) as s:
            src = torch.from_numpy(np.ascontiguousarray(c.U0, dtype=np.float64)).pin_memory()
            dst = torch.full_like(src, float("nan")).pin_memory()
            info = _abi.CfStepInfo()
            rc = s._L.cf_advance(s._ctx, ctypes.cast(src.data_ptr(), dp), 0.0, n, ctypes.cast(dst.data_ptr(), dp),
                                 ctypes.byref(info))
            assert rc == (_abi.CF_EDT if prm else 0)
            assert np.array_equal(dst.numpy(), ref["U"]) and info.t == ref["t"], (prm, n)


@pytest.mark.parametrize("iflux", [3, 4])
def test_lake_at_rest(gpu_lib, oracle, iflux):
    c = cases.lake_at_rest(40, 20, iflux=iflux)
    U, ref, info = compare_bitwise(c, 200, oracle)
    zm = oracle.setup(c)[2]
    eta0 = c.U0[:, 0] + zm
    assert np.abs(U[:, 0] + zm - eta0).max() < 1e-12
    assert np.abs(U[:, 1:]).max() < 1e-12


def test_state_round_trip_and_reordering(gpu_lib):
    """cf_set_state / cf_get_state keep the reference's element order through the internal
    space-filling-curve renumbering, with and without renumbering."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(30, 15, seed=1, iflux=1)
    U = np.random.default_rng(0).uniform(0.1, 2.0, (c.nelt, 3))
    for reorder in (1, 0):
        with Solver(c, dict(reorder=reorder)) as s:
            s.set_state(U, t0=3.5)
            assert np.array_equal(s.get_state(), U)
            assert s.info().t == 3.5
    a, _ = run_gpu(c, 50, dict(reorder=1))
    b, _ = run_gpu(c, 50, dict(reorder=0))
    assert np.array_equal(a, b)


def test_initial_condition_matches_oracle(gpu_lib, oracle):
    from cuteflow_gb300 import Solver
    c = cases.flooding(40, 20, seed=2, iflux=1)
    for ic in (dict(eqlin_barrage=1, x1eqbar=500.001, x2eqbar=500.0, y1eqbar=0.0, y2eqbar=1000.0,
                    h_amont=3.0, u_amont=0.5, v_amont=0.1, h_aval=1.0),
               dict(plan=1, xplan=0.0, yplan=0.0, zplan=1.0, xpoint=0.0, ypoint=0.0, zpoint=1.5, u_aval=0.2)):
        ref = oracle.initial_condition(c, ic)
        with Solver(c) as s:
            s.set_initial_condition(ic)
            assert np.array_equal(s.get_state(), ref)


def test_deterministic_and_graph_equals_single_steps(gpu_lib):
    c = cases.flooding(60, 30, seed=5, iflux=3)
    a, ia = run_gpu(c, 120)                    # graph replay of step pairs
    b, ib = run_gpu(c, 120, chunks=(1,))       # one launch pair per call
    c2, _ = run_gpu(c, 120)
    assert np.array_equal(a, b) and np.array_equal(a, c2) and ia.t == ib.t


def test_discharge_diagnostics(gpu_lib, oracle):
    c = cases.flooding(60, 30, seed=4, iflux=3)
    U, info = run_gpu(c, 40)
    ref = oracle.run(c, 40)
    assert info.q_in == pytest.approx(ref["q_in"], rel=1e-12)
    assert info.q_out == pytest.approx(ref["q_out"], rel=1e-12, abs=1e-12)
    t_ramp = ref["t"] - ref["dt_hist"][39]  # time at the start of the last step
    assert info.q_in == pytest.approx(1000.0 * (2.0 + 8.0 * t_ramp / 600.0), rel=1e-9)


def test_config1_circular_dam_break_full(gpu_lib, oracle):
    """The CPU-runnable benchmark case: 80,000 triangles, HLLC, CFL 0.9, 500 steps."""
    c = cases.circular_dam_break(200, 200, seed=1, iflux=1)
    U, ref, info = compare_bitwise(c, 500, oracle)
    area = oracle.setup(c)[1]
    m0 = float((c.U0[:, 0] * area).sum())
    m1 = float((U[:, 0] * area).sum())
    assert abs(m1 - m0) <= 1e-12 * m0


def test_config2_flooding_1M_5000_steps(gpu_lib, oracle):
    """The benchmark workload at full size and length: 1,000,000 triangles, WAF, inflow ramp and
    fixed-level outflow, 5000 steps from the initial state, with the integer-pipe setting the
    bench's autotuner picks (int_compare 1, integer products, quotients and roots in every edge
    warp and in the element kernel).  Bit for bit the oracle's state, time and next dt (the
    tolerance of the target is 1e-9 m)."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(1000, 500, seed=2, iflux=3)
    ref = oracle.run(c, 5000, check=False)
    with Solver(c) as s:
        s.set_tuning(1, 0x1F)
        s.set_state(c.U0)
        info = s.step(5000)
        U = s.get_state()
    assert info.steps == 5000 and info.status == 0
    assert np.array_equal(U, ref["U"]), np.abs(U - ref["U"]).max(axis=0)
    assert info.t == ref["t"] and info.dt_next == ref["dt_hist"][5000]


@pytest.mark.parametrize("iflux", [1, 3, 4])
def test_phys_inflow(gpu_lib, oracle, iflux):
    """inlet 3 (phys_inflow): the per-step inlet sums of calcul_surf_entree on the device."""
    c = cases.flooding(50, 25, seed=9, iflux=iflux)
    U, ref, info = compare_bitwise(c, 150, oracle, params=dict(inlet=3), chunks=(7, 60, 1))
    assert abs(info.q_in - ref["q_in"]) <= 1e-12 * abs(ref["q_in"])


@pytest.mark.parametrize("tol,count", [(1.5, 30), (0.5, 20), (0.05, 50)])
@pytest.mark.parametrize("inlet", [2, 3])
def test_steady_state_stop(gpu_lib, oracle, tol, count, inlet):
    """The steady-state test runs on the device after every step; the member stops at the
    oracle's step with CF_STATUS_STEADY, cf_step reports success, and further calls do not
    step it."""
    from cuteflow_gb300 import Solver
    c = cases.channel(inlet=inlet)
    prm = dict(tol_reg_perm=tol, steady_count=count)
    ref = oracle.run(c, 1200, params=prm, check=False)
    assert ref["rc"] == 1
    with Solver(c, prm) as s:
        s.set_state(c.U0)
        info = s.step(1200)
        assert info.status & _abi.CF_STATUS_STEADY
        assert info.steps == ref["steps"]
        U = s.get_state()
        again = s.step(5)
        assert again.steps == info.steps and np.array_equal(s.get_state(), U)
    assert np.array_equal(U, ref["U"])
    assert info.t == ref["t"]


def _steps_to(dt_hist, ts, tc=0.0):
    """Steps the reference's loop (finite_volumes_method.cuf:123, :232) takes to reach ts:
    tc starts at t0 and adds the dt computed after every step."""
    tol = float(np.float32(1e-6))
    if not (tc - ts + 2 * tol < tol):
        return 0
    for k in range(1, len(dt_hist)):
        tc = tc + dt_hist[k]
        if not (tc - ts + 2 * tol < tol):
            return k
    raise AssertionError("ts not reached")


@pytest.mark.parametrize("iflux", [1, 3])
def test_run_until_ts(gpu_lib, oracle, iflux):
    """cf_run stops every member at the step where the reference's time loop ends, and a later
    cf_run with a larger ts continues from there."""
    from cuteflow_gb300 import Solver
    c = cases.channel(iflux=iflux)
    full = oracle.run(c, 1500)
    k1, k2 = _steps_to(full["dt_hist"], 60.0), _steps_to(full["dt_hist"], 97.5)
    assert 0 < k1 < k2 < 1500
    with Solver(c) as s:
        s.set_state(c.U0)
        info = s.run(60.0)
        assert info.status & _abi.CF_STATUS_END and info.steps == k1
        assert np.array_equal(s.get_state(), oracle.run(c, k1)["U"])
        info = s.run(97.5)
        assert info.status & _abi.CF_STATUS_END and info.steps == k2
        assert np.array_equal(s.get_state(), oracle.run(c, k2)["U"])
        info = s.run(97.5)
        assert info.steps == k2
        info = s.run(1e9, max_steps=10)
        assert info.steps == k2 + 10 and not info.status


def test_case_directory_runs_to_ts(gpu_lib, oracle, tmp_path):
    """A case directory in the reference's formats (namelist, ASCII mesh, initial condition
    file) read through cf_case_read and run to its ts equals the oracle on the same steps."""
    from cuteflow_gb300 import Solver, case_files
    c = cases.channel(inlet=3, iflux=3)
    case_files.write_case(c, str(tmp_path), ts=45.0)
    r = case_files.read_case(str(tmp_path))
    with Solver(r, r.params) as s:
        s.set_state(r.U0)
        info = s.run(r.ts)
        U = s.get_state()
    full = oracle.run(c, 1000)
    k = _steps_to(full["dt_hist"], 45.0)
    assert info.steps == k and info.status & _abi.CF_STATUS_END
    assert np.array_equal(U, oracle.run(c, k)["U"])


@pytest.mark.parametrize("iflux", [1, 2, 3, 4])
def test_integer_pipe_settings_are_bit_identical(gpu_lib, oracle, iflux):
    """Every setting of cf_set_tuning (comparisons, and products, quotients and roots on the
    integer pipes in some or all edge warps and in the element kernel) gives the oracle's run bit
    for bit."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(60, 30, seed=4, iflux=iflux)
    ref = oracle.run(c, 120)
    with Solver(c) as s:
        for cmp_, mask in ((1, 0), (1, 0xF), (1, 0x5), (1, 0x2), (1, 0x10), (1, 0x1F), (0, 0)):
            s.set_tuning(cmp_, mask)
            assert s.tuning() == (cmp_, mask)
            s.set_state(c.U0)
            info = s.step(120)
            assert np.array_equal(s.get_state(), ref["U"]), (cmp_, mask)
            assert info.t == ref["t"]
        with pytest.raises(Exception):
            s.set_tuning(0, 0xF)
        with pytest.raises(Exception):
            s.set_tuning(1, 0x20)


def test_autotune_leaves_the_run_unchanged(gpu_lib, oracle):
    """cf_autotune times the settings on the current state and restores it: the run continues
    exactly as without tuning."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(60, 30, seed=5, iflux=3)
    ref = oracle.run(c, 90)
    with Solver(c) as s:
        s.set_state(c.U0)
        s.step(40)
        before = s.get_state()
        info0 = s.info()
        cmp_, mask, ms = s.autotune(20)
        assert (cmp_, mask) == s.tuning() and ms > 0
        assert np.array_equal(s.get_state(), before)
        info1 = s.info()
        assert info1.steps == info0.steps and info1.t == info0.t and info1.dt_next == info0.dt_next
        info = s.step(50)
        assert np.array_equal(s.get_state(), ref["U"]) and info.t == ref["t"] and info.steps == 90
        eb, ept, cb = s.launch_shape()
        assert eb in (64, 128, 256) and ept in (1, 2) and cb in (128, 256)


@pytest.mark.parametrize("iflux", [1, 3, 4])
def test_every_launch_shape_and_element_order_is_bit_identical(gpu_lib, oracle, iflux):
    """The autotuner's search space: every edge-kernel shape (64, 128 or 256 threads per block, 1
    or 2 edges per thread), both element-kernel blocks (128, 256) and the three element orders
    (Hilbert, Morton, the caller's), with the integer-pipe arithmetic on and off, each run equal
    to the oracle bit for bit; cf_autotune_order picks one of the orders."""
    from cuteflow_gb300 import Solver, solver
    c = cases.flooding(50, 30, seed=21, iflux=iflux)
    ref = oracle.run(c, 40)
    shapes = [(eb, ept, cb) for eb in (64, 128, 256) for ept in (1, 2) for cb in (256, 128)]
    for reorder in (1, 2, 0):
        with Solver(c, dict(reorder=reorder)) as s:
            for k, shape in enumerate(shapes):
                if reorder != 1 and k % 3:
                    continue
                s.set_launch_shape(*shape)
                s.set_tuning(*((1, 0x1F) if k % 2 else (0, 0)))
                s.set_state(c.U0)
                info = s.step(40)
                assert s.launch_shape() == shape
                assert np.array_equal(s.get_state(), ref["U"]) and info.t == ref["t"], (reorder, shape)
    r, ms = solver.autotune_order(c, steps_per_trial=5)
    assert r in (0, 1, 2) and ms > 0


def test_set_state_consumes_a_pinned_buffer_before_returning(gpu_lib, oracle):
    """cf_set_state from pinned host memory (an asynchronous copy) returns once the buffer has been
    read: the caller overwrites it at once, and the run is still the oracle's."""
    import ctypes
    torch = pytest.importorskip("torch")
    from cuteflow_gb300 import Solver
    c = cases.flooding(60, 30, seed=3, iflux=3)
    ref = oracle.run(c, 40)
    buf = torch.from_numpy(np.ascontiguousarray(c.U0, dtype=np.float64)).pin_memory()
    with Solver(c) as s:
        rc = s._L.cf_set_state(s._ctx, ctypes.cast(buf.data_ptr(), ctypes.POINTER(ctypes.c_double)), 0.0)
        assert rc == 0
        buf.fill_(float("nan"))
        info = s.step(40)
        assert np.array_equal(s.get_state(), ref["U"]) and info.t == ref["t"]


@pytest.mark.parametrize("direct", [1, 0])
def test_state_buffers_of_every_kind_move_the_same_bytes(gpu_lib, oracle, direct):
    """cf_set_state / cf_get_state / cf_advance with pageable host memory, pinned host memory
    (read and written by the state kernels over the CPU link when direct access is on) and device
    memory, and cf_advance with one pinned buffer for input and output: every combination runs the
    oracle's trajectory bit for bit."""
    import ctypes
    torch = pytest.importorskip("torch")
    from cuteflow_gb300 import Solver
    c = cases.flooding(70, 40, seed=5, iflux=3)
    ref = oracle.run(c, 30)
    U0 = np.ascontiguousarray(c.U0, dtype=np.float64)
    dp = ctypes.POINTER(ctypes.c_double)
    with Solver(c) as s:
        s.set_direct_io(bool(direct))
        pinned = torch.from_numpy(U0.copy()).pin_memory()
        device = torch.from_numpy(U0.copy()).cuda()
        for kind in ("pageable", "pinned", "device"):
            if kind == "pageable":
                s.set_state(U0)
            elif kind == "pinned":
                assert s._L.cf_set_state(s._ctx, ctypes.cast(pinned.data_ptr(), dp), 0.0) == 0
            else:
                s.set_state_device(device.data_ptr())
            info = s.step(30)
            assert info.t == ref["t"]
            out_p = torch.zeros_like(pinned).pin_memory()
            out_d = torch.zeros_like(device)
            assert s._L.cf_get_state(s._ctx, ctypes.cast(out_p.data_ptr(), dp)) == 0
            s.get_state_device(out_d.data_ptr())
            torch.cuda.synchronize()
            assert np.array_equal(out_p.numpy(), ref["U"]), kind
            assert np.array_equal(out_d.cpu().numpy(), ref["U"]), kind
            assert np.array_equal(s.get_state(), ref["U"]), kind
        # cf_advance in place on one pinned buffer
        buf = torch.from_numpy(U0.copy()).pin_memory()
        info = _abi.CfStepInfo()
        ptr = ctypes.cast(buf.data_ptr(), dp)
        assert s._L.cf_advance(s._ctx, ptr, 0.0, 30, ptr, ctypes.byref(info)) == 0
        assert np.array_equal(buf.numpy(), ref["U"]) and info.t == ref["t"]


def test_fp64_probe_reports_a_plausible_rate(gpu_lib):
    """cf_probe_fp64 (the step's roofline denominator): GB300 issues ~2 FP64 instructions per
    clock per SM, ~6e11/s over 152 SMs at 2 GHz; the probe must land in that range and leave the
    context usable."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(20, 10, seed=1, iflux=1)
    with Solver(c) as s:
        r = s.probe_fp64()
        assert 1e11 < r < 5e12, r
        s.set_state(c.U0)
        assert s.step(3).status == 0


def test_integer_pipe_arithmetic_matches_the_fp64_unit(gpu_lib):
    """cf_selftest_xd: the device's integer products, quotients (float-seeded reciprocal,
    fixed-point refinement, exact remainder), scalings by 2^k, negation and comparisons give the
    FP64 unit's bits on 2^26 adversarial operand pairs per seed: whole exponent range, subnormals,
    zeros, infinities, NaN, all-ones significands and quotients next to rounding midpoints."""
    from cuteflow_gb300 import Solver
    c = cases.flooding(20, 10, seed=1, iflux=1)
    with Solver(c) as s:
        for seed in (1, 2, 3):
            assert s.selftest_xd(1 << 26, seed) == 0
        s.set_state(c.U0)
        assert s.step(3).status == 0


@pytest.mark.parametrize("iflux,nparts", [(1, 3), (3, 2), (3, 4), (4, 3)])
def test_decomposed_mesh_equals_the_whole(gpu_lib, oracle, iflux, nparts):
    """A mesh cut into parts (separate contexts, halos exchanged and the minimum dt applied after
    every step) evolves bit for bit as the undivided mesh."""
    from cuteflow_gb300 import domains
    c = cases.flooding(50, 25, seed=6, iflux=iflux)
    ref = oracle.run(c, 80)
    parts = domains.partition(c, nparts)
    with domains.Decomposed(parts) as d:
        d.set_state(c.U0)
        info = d.step(80)
        U = d.get_state()
    assert np.array_equal(U, ref["U"])
    assert info.t == ref["t"] and info.steps == 80
