"""Discrete adjoint (dt frozen) against central finite differences of the GPU forward and of
the CPU oracle forward, both replaying the recorded dt sequence.

Objective: J = <w_eta, eta> + <w_state, U^N> with seeded weights; eta = h + z of the gauge
elements after every step.  Checks: the recording forward is the plain step bit for bit; the
replayed forward repeats it; the gradient does not depend on the checkpoint interval; the
directional derivative along seeded Manning and initial-state directions and single-element
Manning derivatives agree with central differences to 1e-5 relative.
"""
import numpy as np
import pytest

import adjoint_cases as AC

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _setup(kind, nsteps=30, ngauges=7, interval=0):
    from cuteflow_gb300 import Solver
    from cuteflow_gb300.adjoint import Adjoint
    c, extra = AC.make(kind)
    s = Solver(c, extra)
    rng = np.random.default_rng(7)
    wet = np.flatnonzero(c.U0[:, 0] > 0.05)
    gauges = rng.choice(wet, ngauges, replace=False)
    adj = Adjoint(s, nsteps, gauges, interval)
    w_eta = rng.standard_normal((nsteps, ngauges))
    w_state = 0.01 * rng.standard_normal((c.nelt, 3))
    return c, extra, s, adj, w_eta, w_state


_J = AC.objective
KINDS = AC.KINDS


@pytest.mark.parametrize("kind", AC.ALL_KINDS)
def test_record_forward_is_the_step(gpu_lib, kind):
    c, extra, s, adj, w_eta, w_state = _setup(kind)
    with s, adj:
        s.set_state(c.U0)
        eta, UN = adj.forward()
        eta2, UN2 = adj.forward(replay=True)
        s.step(adj.nsteps)
        ref = s.get_state()
        zm = s.mesh_tables()[2]
    assert np.array_equal(UN, ref)
    assert np.array_equal(UN2, UN) and np.array_equal(eta2, eta)
    assert np.array_equal(eta[-1], ref[adj.gauges, 0] + zm[adj.gauges])


@pytest.mark.parametrize("kind", AC.FD_KINDS)
def test_gradient_matches_central_differences_gpu(gpu_lib, kind):
    c, extra, s, adj, w_eta, w_state = _setup(kind)
    rng = np.random.default_rng(11)
    n0 = c.manning.copy()
    with s, adj:
        s.set_manning(n0)
        s.set_state(c.U0)
        adj.forward()
        gU, gn = adj.backward(w_eta, w_state)

        def J(n, U0):
            s.set_manning(n)
            s.set_state(U0)
            return _J(*adj.forward(replay=True), w_eta, w_state)

        # Manning direction
        vn = n0 * rng.uniform(-1.0, 1.0, c.nelt)
        eps = 1e-6
        fd = (J(n0 + eps * vn, c.U0) - J(n0 - eps * vn, c.U0)) / (2 * eps)
        ad = float(np.dot(gn, vn))
        assert abs(fd - ad) <= RTOL * abs(ad), (fd, ad)
        # initial-state direction: depth and discharges of the clearly wet elements
        wet = c.U0[:, 0] > 0.05
        vU = np.zeros_like(c.U0)
        vU[wet, 0] = 0.01 * rng.uniform(-1.0, 1.0, wet.sum())
        vU[wet, 1:] = 0.01 * rng.uniform(-1.0, 1.0, (wet.sum(), 2))
        fd = (J(n0, c.U0 + eps * vU) - J(n0, c.U0 - eps * vU)) / (2 * eps)
        ad = float(np.sum(gU * vU))
        assert abs(fd - ad) <= RTOL * abs(ad), (fd, ad)
        # single elements: the largest Manning sensitivities
        for e in np.argsort(-np.abs(gn))[:4]:
            d = np.zeros(c.nelt)
            d[e] = n0[e]
            fd = (J(n0 + eps * d, c.U0) - J(n0 - eps * d, c.U0)) / (2 * eps)
            assert abs(fd - gn[e] * n0[e]) <= RTOL * abs(gn[e] * n0[e]), (e, fd, gn[e] * n0[e])


@pytest.mark.parametrize("kind", ["hllc_dam", "waf_flood"])
def test_gradient_matches_central_differences_oracle(gpu_lib, oracle, kind):
    c, extra, s, adj, w_eta, w_state = _setup(kind, nsteps=20)
    rng = np.random.default_rng(5)
    n0 = c.manning.copy()
    with s, adj:
        s.set_manning(n0)
        s.set_state(c.U0)
        eta_g, UN_g = adj.forward()
        _, gn = adj.backward(w_eta, w_state)
        dt, t = adj.dt_history()
        zm = s.mesh_tables()[2]
    eta_o, UN_o = AC.oracle_run(oracle, c, extra, c.U0, n0, dt, t, adj.gauges, zm)
    assert np.array_equal(eta_o, eta_g) and np.array_equal(UN_o, UN_g)
    vn = n0 * rng.uniform(-1.0, 1.0, c.nelt)
    eps = 1e-6
    Jp = _J(*AC.oracle_run(oracle, c, extra, c.U0, n0 + eps * vn, dt, t, adj.gauges, zm), w_eta, w_state)
    Jm = _J(*AC.oracle_run(oracle, c, extra, c.U0, n0 - eps * vn, dt, t, adj.gauges, zm), w_eta, w_state)
    fd = (Jp - Jm) / (2 * eps)
    ad = float(np.dot(gn, vn))
    assert abs(fd - ad) <= RTOL * abs(ad), (fd, ad)


@pytest.mark.parametrize("kind,frozen", [(k, False) for k in AC.ALL_KINDS] +
                         [("waf_flood", True), ("waf_superbee", True)])
def test_adjoint_is_the_transpose_of_the_tangent(gpu_lib, kind, frozen):
    """<dJ/dU0, dU0> + <dJ/dn, dn> from the adjoint equals the tangent-linear derivative of J
    along (dU0, dn) (CPU, same branches): exact up to summation order, on every case,
    including those whose WAF limiter or wet/dry switches make central differences
    unreliable."""
    import harness as H
    c, extra, s, adj, w_eta, w_state = _setup(kind)
    rng = np.random.default_rng(21)
    wet = c.U0[:, 0] > 0.05
    dU = np.zeros_like(c.U0)
    dU[wet] = 0.01 * rng.uniform(-1.0, 1.0, (wet.sum(), 3))
    dn = c.manning * rng.uniform(-1.0, 1.0, c.nelt)
    with s, adj:
        adj.set_linearization(frozen)
        s.set_manning(c.manning)
        s.set_state(c.U0)
        eta, UN = adj.forward()
        gU, gn = adj.backward(w_eta, w_state)
        dt, t = adj.dt_history()
    eta_t, deta, UN_t, dUN = H.tangent(c, extra, c.U0, dU, c.manning, dn, dt, t, adj.gauges, freeze_r=frozen)
    assert np.array_equal(eta_t, eta) and np.array_equal(UN_t, UN)
    terms = np.concatenate([(w_eta * deta).ravel(), (w_state * dUN).ravel()])
    tl = float(terms.sum())
    ad = float(np.sum(gU * dU) + np.sum(gn * dn))
    assert abs(ad - tl) <= 1e-9 * np.abs(terms).sum(), (ad, tl)


def test_gradient_independent_of_checkpoint_interval(gpu_lib):
    from cuteflow_gb300.adjoint import Adjoint
    c, extra, s, adj, w_eta, w_state = _setup("waf_flood", nsteps=23)
    out = []
    with s:
        adj.close()
        for k in (1, 4, 23, 0):
            with Adjoint(s, 23, adj.gauges, k) as a:
                s.set_state(c.U0)
                a.forward()
                out.append(a.backward(w_eta, w_state))
    for gU, gn in out[1:]:
        assert np.array_equal(gU, out[0][0]) and np.array_equal(gn, out[0][1])


@pytest.mark.parametrize("case", ["waf_flood", "hllc_dam"])
def test_gradient_independent_of_memory_budget(gpu_lib, case):
    """cf_adjoint_create_budget: the recording forward keeps the step records of the last steps
    that fit the budget (all of them, some, or none beyond the minimum), the backward replays only
    the rest; every schedule, with or without a checkpoint interval, gives the gradient of the
    plain sqrt(N) schedule bit for bit, and a budget below every schedule is CF_ENOMEM."""
    from cuteflow_gb300.adjoint import Adjoint
    from cuteflow_gb300.solver import CFError
    c, extra, s, adj, w_eta, w_state = _setup(case, nsteps=23)
    with s:
        adj.close()
        with Adjoint(s, 23, adj.gauges, 0) as a:
            s.set_state(c.U0)
            eta_ref, U_ref = a.forward()
            ref = a.backward(w_eta, w_state)
        with Adjoint(s, 23, adj.gauges, 0, budget_bytes=1 << 40) as a:
            full = a.device_bytes
            assert a.schedule["stored_steps"] == 23 and a.schedule["checkpoints"] == 0
        stored = set()
        for frac, k in ((1.0, 0), (0.8, 0), (0.6, 0), (0.45, 0), (0.6, 4), (0.3, 0)):
            try:
                a = Adjoint(s, 23, adj.gauges, k, budget_bytes=int(full * frac))
            except CFError as e:
                assert e.code == -3
                continue
            with a:
                assert a.device_bytes <= int(full * frac)
                sc = a.schedule
                rest = 23 - sc["stored_steps"]
                assert sc["checkpoints"] == (0 if rest == 0 else -(-rest // sc["checkpoint_interval"]))
                stored.add(sc["stored_steps"])
                s.set_state(c.U0)
                eta, U = a.forward()
                assert np.array_equal(eta, eta_ref) and np.array_equal(U, U_ref)
                gU, gn = a.backward(w_eta, w_state)
                assert np.array_equal(gU, ref[0]) and np.array_equal(gn, ref[1]), (frac, k, sc)
                # a second backward of the same forward (the records are still there)
                gU2, gn2 = a.backward(w_eta, w_state)
                assert np.array_equal(gU2, ref[0]) and np.array_equal(gn2, ref[1])
        assert 23 in stored and any(0 < t < 23 for t in stored)
        with pytest.raises(CFError) as e:
            Adjoint(s, 23, adj.gauges, 0, budget_bytes=1024)
        assert e.value.code == -3


@pytest.mark.parametrize("case", ["waf_flood", "hllc_dam"])
def test_gradient_independent_of_integer_pipe_setting(gpu_lib, case):
    """The recording forward and the segment replays run the step's kernels in the context's
    integer-pipe setting; every setting rounds identically, so the gradient is the same bit for bit."""
    from cuteflow_gb300.adjoint import Adjoint
    c, extra, s, adj, w_eta, w_state = _setup(case, nsteps=23)
    out = []
    with s:
        adj.close()
        for tuning in ((0, 0), (1, 0), (1, 0xF), (1, 0x5), (1, 0x1F)):
            s.set_tuning(*tuning)
            with Adjoint(s, 23, adj.gauges, 4) as a:
                s.set_state(c.U0)
                a.forward()
                out.append(a.backward(w_eta, w_state))
    for gU, gn in out[1:]:
        assert np.array_equal(gU, out[0][0]) and np.array_equal(gn, out[0][1])


def test_torch_function(gpu_lib):
    torch = pytest.importorskip("torch")
    from cuteflow_gb300.adjoint import gauge_run
    c, extra, s, adj, w_eta, w_state = _setup("waf_flood", nsteps=15)
    dev = torch.device("cuda:0")
    with s, adj:
        n = torch.tensor(c.manning, dtype=torch.float64, device=dev, requires_grad=True)
        U0 = torch.tensor(c.U0, dtype=torch.float64, device=dev, requires_grad=True)
        obs = torch.tensor(w_eta, dtype=torch.float64, device=dev)
        eta, UN = gauge_run(adj, n, U0)
        loss = ((eta - obs) ** 2).sum() + (UN[:, 0] ** 2).sum()
        loss.backward()
        # the same through the numpy interface
        s.set_manning(c.manning)
        s.set_state(c.U0)
        e2, U2 = adj.forward()
        w_s = np.zeros_like(U2)
        w_s[:, 0] = 2 * U2[:, 0]
        gU, gn = adj.backward(2 * (e2 - w_eta), w_s)
    assert np.array_equal(eta.detach().cpu().numpy(), e2)
    assert np.array_equal(n.grad.cpu().numpy(), gn)
    assert np.array_equal(U0.grad.cpu().numpy(), gU)


def _batch_members():
    ms = []
    for i, kind in enumerate(["hllc_flood", "hllc_dam", "hllc_flood"]):
        c, extra = AC.make(kind)
        if i == 2:
            c = AC.generic(c, 40)
        ms.append((c, extra))
    return ms


def test_batched_adjoint_equals_single_runs(gpu_lib):
    """A batch's adjoint (every member in the same launches, its own dt) gives each member the
    forward, the dt history and the gradients of that member's own adjoint, bit for bit."""
    from cuteflow_gb300 import Batch, Solver
    from cuteflow_gb300.adjoint import Adjoint
    ms = _batch_members()
    rng = np.random.default_rng(3)
    nsteps = 25
    gl = [rng.choice(np.flatnonzero(c.U0[:, 0] > 0.05), 4, replace=False) for c, _ in ms]
    singles = []
    for (c, extra), g in zip(ms, gl):
        with Solver(c, extra) as s, Adjoint(s, nsteps, g, 6) as adj:
            s.set_state(c.U0)
            eta, UN = adj.forward()
            w = np.linspace(-1.0, 1.0, eta.size).reshape(eta.shape)
            ws = 0.01 * np.ones((c.nelt, 3))
            gU, gn = adj.backward(w, ws)
            dt, t = adj.dt_history()
            singles.append((eta, UN, gU, gn, dt, w, ws))
    gm = np.concatenate([np.full(len(g), i, np.int32) for i, g in enumerate(gl)])
    gg = np.concatenate(gl).astype(np.int32)
    with Batch([c for c, _ in ms], [e for _, e in ms]) as b, Adjoint(b, nsteps, gg, 6, gauge_member=gm) as adj:
        for i, (c, _) in enumerate(ms):
            b.set_state(i, c.U0)
        eta, UN = adj.forward()
        w = np.concatenate([sg[5] for sg in singles], axis=1)
        ws = np.concatenate([sg[6] for sg in singles])
        gU, gn = adj.backward(w, ws)
        dt, t = adj.dt_history()
    off, col = 0, 0
    for i, ((c, _), sg) in enumerate(zip(ms, singles)):
        n, G = c.nelt, len(gl[i])
        assert np.array_equal(eta[:, col:col + G], sg[0]), i
        assert np.array_equal(UN[off:off + n], sg[1]), i
        assert np.array_equal(gU[off:off + n], sg[2]), i
        assert np.array_equal(gn[off:off + n], sg[3]), i
        assert np.array_equal(dt[:, i], sg[4]), i
        off += n
        col += G
    assert len({tuple(dt[:, i]) for i in range(len(ms))}) == len(ms)   # own dt per member


def test_zones_gradient_and_descent(gpu_lib):
    """Zone gradients are the per-zone sums of dJ/dn (fixed order on the device); a descent step
    moves the zone values by -lr g within [lo, hi] and writes them into the Manning field."""
    from cuteflow_gb300 import Solver
    from cuteflow_gb300.adjoint import Adjoint, Zones, zone_gradient
    c, extra = AC.make("hllc_flood")
    rng = np.random.default_rng(5)
    zones = rng.integers(0, 5, c.nelt).astype(np.int32)
    zones[:7] = -1
    g = rng.choice(np.flatnonzero(c.U0[:, 0] > 0.05), 5, replace=False)
    vals = np.array([0.02, 0.03, 0.04, 0.05, 0.06])
    with Solver(c, extra) as s, Adjoint(s, 20, g) as adj, Zones(s, zones, 5) as z:
        s.set_manning(c.manning)
        z.set(vals)
        s.set_state(c.U0)
        eta, _ = adj.forward()
        _, gn = adj.backward(np.ones_like(eta))
        gz = z.gradient(adj)
        ref = zone_gradient(gn[zones >= 0], zones[zones >= 0], 5)
        assert np.allclose(gz, ref, rtol=1e-12, atol=1e-300)
        z.descend(1e-4, 0.01, 0.1)
        v, gz2 = z.get()
        assert np.array_equal(gz2, gz)
        assert np.allclose(v, np.clip(vals - 1e-4 * gz, 0.01, 0.1), rtol=0, atol=1e-15)
        # the context now steps with those values: same run as an explicit Manning field
        s.set_state(c.U0)
        eta2, U2 = adj.forward()
    n_expl = c.manning.copy()
    n_expl[zones >= 0] = v[zones[zones >= 0]]
    with Solver(c, extra) as s2, Adjoint(s2, 20, g) as adj2:
        s2.set_manning(n_expl)
        s2.set_state(c.U0)
        eta3, U3 = adj2.forward()
    assert np.array_equal(eta2, eta3) and np.array_equal(U2, U3)


def test_batched_calibration_reduces_the_misfit(gpu_lib):
    """Two calibration instances in one batch: observations from their true zone fields, then
    gradient descent on the zone values from n = 0.035, entirely through the device-side zone
    gradient and descent: the gauge misfit falls."""
    from cuteflow_gb300 import Batch, cases
    from cuteflow_gb300.adjoint import Adjoint, Zones
    inst = [cases.calibration(60, 24, seed=20 + i, nzones=4, ngauges=12) for i in range(2)]
    zoff = np.cumsum([0] + [len(nz) for _, _, nz, _ in inst])
    zone_all = np.concatenate([z + zoff[i] for i, (_, z, _, _) in enumerate(inst)]).astype(np.int32)
    true_vals = np.concatenate([nz for _, _, nz, _ in inst])
    gm = np.concatenate([np.full(len(g), i, np.int32) for i, (_, _, _, g) in enumerate(inst)])
    gg = np.concatenate([g for *_, g in inst]).astype(np.int32)
    with Batch([c for c, *_ in inst]) as b, Adjoint(b, 150, gg, 0, gauge_member=gm) as adj, \
            Zones(b, zone_all, int(zoff[-1])) as zs:
        def start():
            for i, (c, *_) in enumerate(inst):
                b.set_state(i, c.U0)
        zs.set(true_vals)
        start()
        eta_obs, _ = adj.forward()
        zs.set(np.full(int(zoff[-1]), 0.035))
        misfit = []
        lr = None
        for it in range(8):
            start()
            eta, _ = adj.forward()
            r = eta - eta_obs
            misfit.append(float(np.sum(r * r)))
            adj.backward(2.0 * r)
            g = zs.gradient(adj)
            if lr is None:
                lr = 0.004 / np.abs(g).max()
            zs.descend(lr, 0.01, 0.1)
        start()
        eta, _ = adj.forward()
        misfit.append(float(np.sum((eta - eta_obs) ** 2)))
    assert misfit[-1] < 0.5 * misfit[0], misfit
