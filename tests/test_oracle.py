"""Known-answer checks of the oracle itself (no reference vectors are loadable for this path,
so the restatement is pinned by properties of the equations and of the scheme)."""
import numpy as np
import pytest

from cuteflow_gb300 import cases


@pytest.mark.parametrize("iflux,tol", [(1, 1e-7), (2, 1e-12), (3, 1e-12), (4, 1e-12)])
def test_lake_at_rest(oracle, iflux, tol):
    """Hydrostatic reconstruction keeps still water still (source_terms.cuf:90-97 with
    flux_riemann.cuf:176-181).  HLLC's eps = 1e-8 in the HLL denominator (flux_riemann.cuf:1005)
    makes it well-balanced only to ~1e-9, a property of the reference scheme."""
    c = cases.lake_at_rest(30, 15, iflux=iflux)
    zm = oracle.setup(c)[2]
    r = oracle.run(c, 100)
    eta0 = c.U0[:, 0] + zm
    eta = r["U"][:, 0] + zm
    assert np.abs(eta - eta0).max() < tol
    assert np.abs(r["U"][:, 1:]).max() < 20 * tol


def test_lake_with_islands(oracle):
    c = cases.lake_at_rest(30, 15, iflux=3, wet=False)
    zm = oracle.setup(c)[2]
    r = oracle.run(c, 100)
    wet = c.U0[:, 0] > 0
    assert np.array_equal(wet, r["U"][:, 0] > 0)
    assert np.abs((r["U"][:, 0] + zm)[wet] - (c.U0[:, 0] + zm)[wet]).max() < 1e-12


@pytest.mark.parametrize("iflux", [1, 2, 3])
def test_mass_conservation_walls(oracle, iflux):
    c = cases.circular_dam_break(40, 40, seed=5, iflux=iflux)
    area = oracle.setup(c)[1]
    r = oracle.run(c, 200)
    m0 = (c.U0[:, 0] * area).sum()
    m1 = (r["U"][:, 0] * area).sum()
    assert abs(m1 - m0) <= 1e-12 * m0


def test_once_per_edge_equals_two_sided_for_hllc(oracle):
    """The HLLC flux of the reference is antisymmetric to the bit, so evaluating each edge
    once gives the reference's two-sided result exactly."""
    c = cases.circular_dam_break(40, 40, seed=3, iflux=1)
    a = oracle.run(c, 100, params=dict(flux_mode=0))
    b = oracle.run(c, 100, params=dict(flux_mode=1))
    assert np.array_equal(a["U"], b["U"])


def test_waf_two_sided_is_not_conservative(oracle):
    """The reference's WAF evaluates r = dupw/(dloc + eps) from each side; where the
    reconstructed depths are equal to the bit the two sides disagree, so a once-per-edge
    evaluation differs from the reference (this is why the GPU keeps both sides)."""
    c = cases.flooding(60, 30, seed=2, iflux=3)
    a = oracle.run(c, 100, params=dict(flux_mode=0))
    b = oracle.run(c, 100, params=dict(flux_mode=1))
    assert np.abs(a["U"] - b["U"]).max() > 1e-9


def _symmetric_mesh_case(nx=40, ny=10):
    """A mesh symmetric under x -> Lx - x (no jitter, mirrored diagonals)."""
    lx, ly = float(nx), float(ny)
    x, y, tri = cases.grid_mesh(nx, ny, lx, ly, seed=1, jitter=0.0)
    qi = np.tile(np.arange(nx), ny)
    qj = np.repeat(np.arange(ny), nx)
    flip = ((qj % 2) == 0) ^ (qi >= nx // 2)
    a = qj * (nx + 1) + qi + 1
    b, d = a + 1, a + (nx + 1)
    cc = b + (nx + 1)
    t1 = np.where(flip[:, None], np.stack([a, b, d], 1), np.stack([a, b, cc], 1))
    t2 = np.where(flip[:, None], np.stack([b, cc, d], 1), np.stack([a, cc, d], 1))
    tri = np.empty((2 * nx * ny, 3), dtype=np.int32)
    tri[0::2] = t1
    tri[1::2] = t2
    c = cases.circular_dam_break(nx, ny, seed=1)
    c.x, c.y, c.tri = x, y, tri
    xc, yc = cases.cell_centroids(x, y, tri)
    c.U0 = np.zeros((tri.shape[0], 3))
    c.U0[:, 0] = np.where(np.abs(xc - lx / 2) < lx / 4, 2.0, 1.0)
    c.manning = np.full(tri.shape[0], 0.02)
    return c, xc, yc


@pytest.mark.parametrize("iflux", [1])
def test_mirror_symmetry(oracle, iflux):
    """HLLC keeps a mirror-symmetric dam break symmetric to round-off.  (IFLUX 2 and 3 do not:
    the star-state selection of flux_riemann.cuf:1160-1176 falls through to F(U_R) when
    s* == 0 exactly, as on a symmetry plane, and the WAF ratios of :876-878 change sign with
    one-ulp perturbations, so round-off grows to O(1) differences there.)"""
    c, xc, yc = _symmetric_mesh_case()
    c.params["iflux"] = iflux
    r = oracle.run(c, 80)
    # pair every element with its mirror image
    key = np.round(xc, 9) * 1e6 + np.round(yc, 9)
    mkey = np.round(c.nx - xc, 9) * 1e6 + np.round(yc, 9)
    order = np.argsort(key)
    mirror = order[np.searchsorted(key[order], mkey)]
    assert np.array_equal(key[mirror], mkey)
    U = r["U"]
    assert np.abs(U[:, 0] - U[mirror, 0]).max() < 1e-11
    assert np.abs(U[:, 1] + U[mirror, 1]).max() < 1e-11


def _stoker(x, t, hl, hr, x0, g):
    """Exact 1-D dam break on a wet bed (Stoker): rarefaction, constant middle state, shock."""
    from scipy.optimize import brentq
    cl, cr = np.sqrt(g * hl), np.sqrt(g * hr)

    # middle state from the standard cubic: solve for cm
    def g2(cm):
        hm = cm * cm / g
        um = 2 * (cl - cm)
        # shock: s = um*hm/(hm-hr) and momentum: hm*um^2 + g hm^2/2 - g hr^2/2 = s*hm*um
        s = um * hm / (hm - hr)
        return hm * um * um + 0.5 * g * hm * hm - 0.5 * g * hr * hr - s * hm * um
    cm = brentq(g2, cr * (1 + 1e-12), cl * (1 - 1e-12))
    hm = cm * cm / g
    um = 2 * (cl - cm)
    s = um * hm / (hm - hr)
    xi = (x - x0) / t
    h = np.where(xi <= -cl, hl, 0.0)
    fan = (xi > -cl) & (xi <= um - cm)
    h = np.where(fan, (2 * cl - xi) ** 2 / (9 * g), h)
    h = np.where((xi > um - cm) & (xi <= s), hm, h)
    h = np.where(xi > s, hr, h)
    return h


def test_dam_break_converges_to_stoker(oracle):
    """1-D wet-bed dam break in a 10 m x 1 m channel (the shape of the reference's Test_1-3
    validation cases): the L1 error against the exact solution shrinks with refinement."""
    errs = []
    for nx in (100, 200):
        ny = max(2, nx // 20)
        x, y, tri = cases.grid_mesh(nx, ny, 10.0, 1.0, seed=4)
        c = cases.circular_dam_break(nx, ny, seed=4, iflux=2)
        c.x, c.y, c.tri = x, y, tri
        c.z = np.zeros_like(x)
        xc, yc = cases.cell_centroids(x, y, tri)
        c.U0 = np.zeros((tri.shape[0], 3))
        c.U0[:, 0] = np.where(xc < 5.0, 1.0, 0.5)
        c.manning = np.zeros(tri.shape[0])
        c.params.update(friction=0)
        dt0 = oracle.run(c, 1)["dt_hist"][0]
        r = oracle.run(c, int(0.5 / dt0))
        t = r["t"]
        h_ex = _stoker(xc, t, 1.0, 0.5, 5.0, 9.81)
        area = oracle.setup(c)[1]
        errs.append((np.abs(r["U"][:, 0] - h_ex) * area).sum() / area.sum())
    assert errs[1] < 0.75 * errs[0]
    assert errs[1] < 0.02


@pytest.mark.parametrize("iflux", [1, 3])
def test_phys_inflow_delivers_the_discharge(oracle, iflux):
    """phys_inflow (flux_riemann.cuf:127-138) gives each inflow edge Q * h len / sum(h len):
    with one inflow edge per element the edges carry Q in total, spread in proportion to depth
    (calcul_surf_entree, maillage.cuf:1368-1421)."""
    c = cases.channel(iflux=iflux, inlet=3, q=1.5)
    Q = 1.5 * 120.0
    for n in (1, 40, 200):
        r = oracle.run(c, n)
        assert abs(r["q_in"] - Q) <= 1e-12 * Q, (n, r["q_in"])


def test_phys_inflow_shares_by_depth(oracle):
    """Against inlet 2 (uniform unit discharge Q/L), phys_inflow puts more of the same Q
    through the deeper inflow elements: on a cross-slope the deep side's momentum grows faster."""
    c = cases.channel(inlet=2, q=1.0)
    c.z = c.z + 0.004 * c.y          # deeper at small y
    from cuteflow_gb300.cases import cell_bed
    zc = cell_bed(c.x, c.y, c.z, c.tri)
    c.U0[:, 0] = np.where(1.0 - zc > 1e-4, 1.0 - zc, 0.0)
    a = oracle.run(c, 30)
    b = oracle.run(c, 30, params=dict(inlet=3))
    assert abs(a["q_in"] - b["q_in"]) <= 1e-12 * a["q_in"]
    xc, yc = cases.cell_centroids(c.x, c.y, c.tri)
    left = xc < 10.0
    deep, shallow = left & (yc < 30.0), left & (yc > 90.0)
    assert b["U"][deep, 1].mean() > a["U"][deep, 1].mean()
    assert b["U"][shallow, 1].mean() < a["U"][shallow, 1].mean()


def test_steady_state_stop(oracle):
    """check_steady_state (finite_volumes_method.cuf:370-393): the run stops after more than
    steady_count consecutive steps with |Q_in - Q_out| / Q_in < tol_reg_perm; a tolerance
    above 1 qualifies every step with inflow; 0 never stops."""
    c = cases.channel()
    r = oracle.run(c, 200, params=dict(tol_reg_perm=1.5, steady_count=30))
    assert r["rc"] == 1 and r["steps"] == 31
    r = oracle.run(c, 900, params=dict(tol_reg_perm=0.5, steady_count=20))
    assert r["rc"] == 1 and 20 < r["steps"] < 900
    assert abs(r["q_in"] - r["q_out"]) < 0.5 * r["q_in"]
    r = oracle.run(c, 300)
    assert r["rc"] == 0 and r["steps"] == 300
