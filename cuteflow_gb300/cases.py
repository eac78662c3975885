"""Seeded synthetic cases with the shapes of the benchmark workloads.

The reference's own meshes are not available (Git LFS stubs), so the workloads are built
here: an nx x ny grid of quads over an Lx x Ly rectangle, each quad split into two
counter-clockwise triangles along a diagonal chosen by a seeded coin flip, interior
vertices jittered uniformly by +/-0.2 of the grid spacing.  Inputs are the reference's own
inputs: node coordinates and bed elevation, 1-based connectivity in the reference's edge
order, per-element Manning n, and inflow / outflow / wall node lists with inlet and outlet
numbers (the tables ``lec_mail_tri`` reads, maillage.cuf:196-313).

Random numbers come from a counter-based splitmix64 stream, so a seed gives the same mesh
on every machine (the Gaussian bumps and the lognormal Manning field go through libm and
may differ in the last bit between machines).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, stream: int, n: int) -> np.ndarray:
    """n consecutive splitmix64 outputs of (seed, stream) as uint64."""
    base = np.uint64((seed * 0x2545F4914F6CDD1D + stream * 0x632BE59BD9B4E019) & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        z = base + (np.arange(1, n + 1, dtype=np.uint64) * _GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, stream: int, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    u = (splitmix64(seed, stream, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


# ---- elementary functions as fixed sequences of float64 operations --------------------------
#
# numpy's exp, log and cos are not correctly rounded and differ between its x86-64 and aarch64
# builds, so the same seed would give different inputs on different machines.  The generators use
# these instead: range reduction that is exact, then a truncated Taylor or atanh series by Horner's
# rule in plain IEEE additions and multiplications (a few ulp from the true value, identical on every
# machine).

_LN2_HI = float.fromhex("0x1.62e42fee00000p-1")   # ln 2 truncated to 32 bits: k * _LN2_HI is exact
_LN2_LO = float.fromhex("0x1.a39ef35793c76p-33")  # ln 2 - _LN2_HI
_INV_LN2 = float.fromhex("0x1.71547652b82fep+0")
_TWO_PI = float.fromhex("0x1.921fb54442d18p+2")
_INV_FACT = [1.0 / float(math.factorial(i)) for i in range(23)]


def det_exp(x) -> np.ndarray:
    """e^x: x = k ln 2 + r (Cody-Waite, |r| <= ln2 / 2), e^r by its Taylor series to r^13, 2^k exactly."""
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x * _INV_LN2)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.full_like(r, _INV_FACT[13])
    for i in range(12, -1, -1):
        p = p * r + _INV_FACT[i]
    return np.ldexp(p, np.clip(k, -2000, 2000).astype(np.int64))


def det_log(x) -> np.ndarray:
    """ln x for x > 0: x = m 2^e with m in [1/sqrt 2, sqrt 2), ln m = 2 atanh(s) with
    s = (m - 1) / (m + 1) (|s| <= 0.172) by its series to s^23."""
    m, e = np.frexp(np.asarray(x, dtype=np.float64))
    low = m < 0.7071067811865476
    m = np.where(low, m * 2.0, m)
    e = np.where(low, e - 1, e).astype(np.float64)
    s = (m - 1.0) / (m + 1.0)
    s2 = s * s
    p = np.full_like(s, 1.0 / 23.0)
    for j in range(21, 0, -2):
        p = p * s2 + 1.0 / j
    return e * _LN2_HI + (e * _LN2_LO + 2.0 * s * p)


def det_cos2pi(u) -> np.ndarray:
    """cos(2 pi u) for u in [0, 1): folded by symmetry (exact subtractions) to an angle in
    [0, pi/4], where the Taylor series of cos (to x^20) or of sin (to x^21) is summed."""
    u = np.asarray(u, dtype=np.float64)
    w = np.where(u > 0.5, 1.0 - u, u)                  # cos(2 pi u) = cos(2 pi (1 - u))
    neg = w > 0.25
    w = np.where(neg, 0.5 - w, w)                      # cos(2 pi w) = -cos(2 pi (1/2 - w))
    use_sin = w > 0.125
    a = _TWO_PI * np.where(use_sin, 0.25 - w, w)       # cos(2 pi w) = sin(2 pi (1/4 - w))
    a2 = a * a
    c = np.full_like(a, _INV_FACT[20])
    sn = np.full_like(a, _INV_FACT[21])
    for i in range(18, -1, -2):
        c = c * a2 * (-1.0) + _INV_FACT[i]
        sn = sn * a2 * (-1.0) + _INV_FACT[i + 1]
    v = np.where(use_sin, a * sn, c)
    return np.where(neg, -v, v)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """Box-Muller standard normals."""
    u1 = uniform(seed, stream, n)
    u2 = uniform(seed, stream + 1000003, n)
    u1 = np.maximum(u1, 1e-300)
    return np.sqrt(-2.0 * det_log(u1)) * det_cos2pi(u2)


@dataclasses.dataclass
class Case:
    """Reference inputs for one simulation (arrays follow the reference's mesh tables)."""

    x: np.ndarray            # [nnt] float64
    y: np.ndarray            # [nnt]
    z: np.ndarray            # [nnt] bed elevation at nodes
    tri: np.ndarray          # [nelt, 3] int32, 1-based node ids, counter-clockwise
    manning: np.ndarray      # [nelt] per-element Manning n
    ndinput: np.ndarray      # inflow node ids (1-based)
    numero_ndinput: np.ndarray
    ndoutput: np.ndarray
    numero_ndoutput: np.ndarray
    ndwall: np.ndarray
    nombre_entrees: int
    nombre_sorties: int
    params: dict             # cf_params fields that differ from the defaults
    U0: np.ndarray           # [nelt, 3] initial (h, hu, hv) per element
    name: str = ""
    nx: int = 0
    ny: int = 0

    @property
    def nelt(self) -> int:
        return int(self.tri.shape[0])

    @property
    def nnt(self) -> int:
        return int(self.x.shape[0])


def grid_mesh(nx: int, ny: int, lx: float, ly: float, seed: int, jitter: float = 0.2):
    """Jittered quad grid split into CCW triangles.  Returns x, y, tri (1-based)."""
    dx, dy = lx / nx, ly / ny
    i = np.arange(nx + 1, dtype=np.float64)
    j = np.arange(ny + 1, dtype=np.float64)
    X, Y = np.meshgrid(i * dx, j * dy)                    # [ny+1, nx+1]
    x = X.ravel().copy()
    y = Y.ravel().copy()
    nnt = (nx + 1) * (ny + 1)
    ii = np.tile(np.arange(nx + 1), ny + 1)
    jj = np.repeat(np.arange(ny + 1), nx + 1)
    interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
    jx = uniform(seed, 1, nnt, -jitter * dx, jitter * dx)
    jy = uniform(seed, 2, nnt, -jitter * dy, jitter * dy)
    x[interior] += jx[interior]
    y[interior] += jy[interior]
    qi = np.tile(np.arange(nx), ny)
    qj = np.repeat(np.arange(ny), nx)
    a = qj * (nx + 1) + qi + 1          # (i, j)
    b = a + 1                            # (i+1, j)
    c = b + (nx + 1)                     # (i+1, j+1)
    d = a + (nx + 1)                     # (i, j+1)
    flip = (splitmix64(seed, 3, nx * ny) >> np.uint64(63)).astype(bool)
    t1 = np.where(flip[:, None], np.stack([a, b, d], 1), np.stack([a, b, c], 1))
    t2 = np.where(flip[:, None], np.stack([b, c, d], 1), np.stack([a, c, d], 1))
    tri = np.empty((2 * nx * ny, 3), dtype=np.int32)
    tri[0::2] = t1
    tri[1::2] = t2
    return x, y, tri


def side_nodes(nx: int, ny: int):
    """1-based node ids on the left, right, bottom and top sides of the grid."""
    left = np.arange(ny + 1) * (nx + 1) + 1
    right = left + nx
    bottom = np.arange(nx + 1) + 1
    top = ny * (nx + 1) + np.arange(nx + 1) + 1
    return left.astype(np.int32), right.astype(np.int32), bottom.astype(np.int32), top.astype(np.int32)


def cell_centroids(x, y, tri):
    t = tri - 1
    return (x[t[:, 0]] + x[t[:, 1]] + x[t[:, 2]]) / 3, (y[t[:, 0]] + y[t[:, 1]] + y[t[:, 2]]) / 3


def cell_bed(x, y, z, tri):
    """Cell bed by the reference rule: centroid-distance-weighted vertex z (maillage.cuf:1319-1329)."""
    t = tri - 1
    xs, ys, zs = x[t], y[t], z[t]
    xg = (xs[:, 0] + xs[:, 1] + xs[:, 2]) / 3.0
    yg = (ys[:, 0] + ys[:, 1] + ys[:, 2]) / 3.0
    d = np.sqrt((xs - xg[:, None]) ** 2 + (ys - yg[:, None]) ** 2)
    return (d[:, 0] * zs[:, 0] + d[:, 1] * zs[:, 1] + d[:, 2] * zs[:, 2]) / (d[:, 0] + d[:, 1] + d[:, 2])


def _lognormal_manning(seed: int, stream: int, n: int, median=0.03, sigma=0.3, lo=0.01, hi=0.1):
    return np.clip(median * det_exp(sigma * normal(seed, stream, n)), lo, hi)


def circular_dam_break(nx: int = 200, ny: int = 200, seed: int = 1, lx: Optional[float] = None,
                       ly: Optional[float] = None, iflux: int = 1, manning: float = 0.025,
                       tolisec: float = 1e-5) -> Case:
    """Circular dam break on a flat bed with reflective walls.

    The benchmark case is 200 m x 200 m, 200x200 quads (80,000 triangles), z = 0,
    n = 0.025, h = 10 m inside a radius-50 m circle centred in the domain (by cell
    centroid) and 1 m outside, u = v = 0, CFL 0.9, first-order HLLC.
    """
    lx = float(nx) if lx is None else lx
    ly = float(ny) if ly is None else ly
    x, y, tri = grid_mesh(nx, ny, lx, ly, seed)
    z = np.zeros_like(x)
    xc, yc = cell_centroids(x, y, tri)
    r = min(lx, ly) * 0.25
    inside = (xc - lx / 2) ** 2 + (yc - ly / 2) ** 2 < r * r
    U0 = np.zeros((tri.shape[0], 3))
    U0[:, 0] = np.where(inside, 10.0, 1.0)
    left, right, bottom, top = side_nodes(nx, ny)
    walls = np.unique(np.concatenate([left, right, bottom, top])).astype(np.int32)
    e = np.zeros(0, dtype=np.int32)
    return Case(x=x, y=y, z=z, tri=tri, manning=np.full(tri.shape[0], manning), ndinput=e,
                numero_ndinput=e, ndoutput=e, numero_ndoutput=e, ndwall=walls, nombre_entrees=0,
                nombre_sorties=0,
                params=dict(iflux=iflux, tolisec=tolisec, cfl=0.9, friction=1, fricimplic=1,
                            is_override_manning=0),
                U0=U0, name=f"circular_dam_break_{nx}x{ny}", nx=nx, ny=ny)


def flooding(nx: int = 1000, ny: int = 500, seed: int = 2, lx: float = 2000.0, ly: float = 1000.0,
             iflux: int = 3, q0: float = 2.0, q1: float = 10.0, ramp: float = 600.0,
             out_level: float = 1.0, tolisec: float = 1e-4, nbumps: int = 8, bump_scale: float = 1.0) -> Case:
    """Wet/dry flooding over seeded bathymetry.

    The benchmark case is 2 km x 1 km, 1000x500 quads (1,000,000 triangles),
    z = 0.001 x + 8 Gaussian bumps (amplitude U(0.5,3) m, width U(30,150) m, centres uniform),
    per-element lognormal Manning (median 0.03, sigma_log 0.3, clipped to [0.01, 0.1]),
    still water at level 1.0 m where z < 1 m and dry elsewhere (dry threshold 1e-4 m),
    left-edge inflow ramping q = 2 -> 10 m^2/s over 600 s, fixed level 1.0 m at the right
    edge, walls top and bottom, CFL 0.9, second-order WAF.  bump_scale multiplies the bump
    widths (smaller domains with the same bathymetry statistics per area).
    """
    x, y, tri = grid_mesh(nx, ny, lx, ly, seed)
    cx = uniform(seed, 10, nbumps, 0.0, lx)
    cy = uniform(seed, 11, nbumps, 0.0, ly)
    amp = uniform(seed, 12, nbumps, 0.5, 3.0)
    wid = uniform(seed, 13, nbumps, 30.0, 150.0) * bump_scale
    z = 0.001 * x
    for k in range(nbumps):
        z = z + amp[k] * det_exp(-((x - cx[k]) ** 2 + (y - cy[k]) ** 2) / (2.0 * wid[k] ** 2))
    manning = _lognormal_manning(seed, 20, tri.shape[0])
    zc = cell_bed(x, y, z, tri)
    h = 1.0 - zc
    U0 = np.zeros((tri.shape[0], 3))
    U0[:, 0] = np.where(h > tolisec, h, 0.0)
    left, right, bottom, top = side_nodes(nx, ny)
    walls = np.unique(np.concatenate([bottom, top])).astype(np.int32)
    params = dict(iflux=iflux, ilimiteur=1, tolisec=tolisec, cfl=0.9, friction=1, fricimplic=1,
                  is_override_manning=0, inlet=2, outlet=1, ramp_time=ramp)
    params["debitglob"] = [q1 * ly]
    params["debitglob_start"] = [q0 * ly]
    params["h_sortie"] = [out_level]
    return Case(x=x, y=y, z=z, tri=tri, manning=manning, ndinput=left,
                numero_ndinput=np.ones_like(left), ndoutput=right,
                numero_ndoutput=np.ones_like(right), ndwall=walls, nombre_entrees=1,
                nombre_sorties=1, params=params, U0=U0, name=f"flooding_{nx}x{ny}", nx=nx, ny=ny)


def channel(nx: int = 60, ny: int = 12, seed: int = 6, lx: float = 600.0, ly: float = 120.0, iflux: int = 1,
            q: float = 1.0, slope: float = 0.001, out_level: float = 1.0, manning: float = 0.03,
            inlet: int = 2, tolisec: float = 1e-4) -> Case:
    """A sloping rectangular channel that settles towards a steady flow: bed z = slope * (lx - x),
    inflow of q m^2/s over the left edge (inlet 2 'inflow' or 3 'phys_inflow'), fixed level
    out_level at the right edge, walls top and bottom, uniform Manning n, still water at level
    out_level at t = 0 (dry where the bed is above it)."""
    x, y, tri = grid_mesh(nx, ny, lx, ly, seed)
    z = slope * (lx - x)
    zc = cell_bed(x, y, z, tri)
    h = out_level - zc
    U0 = np.zeros((tri.shape[0], 3))
    U0[:, 0] = np.where(h > tolisec, h, 0.0)
    left, right, bottom, top = side_nodes(nx, ny)
    walls = np.unique(np.concatenate([bottom, top])).astype(np.int32)
    params = dict(iflux=iflux, ilimiteur=1, tolisec=tolisec, cfl=0.9, friction=1, fricimplic=1,
                  is_override_manning=0, inlet=inlet, outlet=1, debitglob=[q * ly], h_sortie=[out_level])
    return Case(x=x, y=y, z=z, tri=tri, manning=np.full(tri.shape[0], manning), ndinput=left,
                numero_ndinput=np.ones_like(left), ndoutput=right, numero_ndoutput=np.ones_like(right),
                ndwall=walls, nombre_entrees=1, nombre_sorties=1, params=params, U0=U0,
                name=f"channel_{nx}x{ny}", nx=nx, ny=ny)


def lake_at_rest(nx: int = 40, ny: int = 20, seed: int = 5, depth: float = 0.5, iflux: int = 3,
                 wet: bool = True) -> Case:
    """Still water over the flooding bathymetry with walls only (well-balancedness).

    The free surface sits ``depth`` above the highest cell bed (fully wet), or with
    ``wet=False`` at the median cell bed so that the bumps emerge as dry islands."""
    c = flooding(nx, ny, seed=seed, lx=2.0 * nx, ly=2.0 * ny, iflux=iflux, tolisec=1e-4)
    zc = cell_bed(c.x, c.y, c.z, c.tri)
    level = (zc.max() + depth) if wet else float(np.median(zc))
    U0 = np.zeros((c.nelt, 3))
    U0[:, 0] = np.maximum(level - zc, 0.0)
    U0[U0[:, 0] <= 1e-4, 0] = 0.0
    left, right, bottom, top = side_nodes(nx, ny)
    e = np.zeros(0, dtype=np.int32)
    c.U0 = U0
    c.ndinput = c.numero_ndinput = c.ndoutput = c.numero_ndoutput = e
    c.ndwall = np.unique(np.concatenate([left, right, bottom, top])).astype(np.int32)
    c.nombre_entrees = c.nombre_sorties = 0
    c.params = dict(iflux=iflux, ilimiteur=1, tolisec=1e-4, cfl=0.9, friction=1, fricimplic=1,
                    is_override_manning=0)
    c.name = f"lake_at_rest_{nx}x{ny}"
    return c


def ensemble_member(index: int, seed: int = 3, n_min: int = 20000, n_max: int = 500000,
                    iflux: int = 3) -> Case:
    """One member of the batched ensemble: the flooding generator (seeded bathymetry, lognormal
    Manning field, still water at 1 m, inflow ramp on the left edge, fixed 1 m level on the right)
    with its own size (triangle count drawn unevenly in [n_min, n_max], aspect U(0.5, 2)) at the
    benchmark case's 2 m spacing, its own seed for the bumps and the Manning field, bumps in
    proportion to the area (8 per 2 km^2, at least one) with widths scaled by the square root of
    the area ratio (the benchmark's bumps on the benchmark's domain keep their size; a small domain
    is not covered by one hill and left dry), and an inflow ramping from 2 m^2/s to its own peak
    q ~ U(2, 15) m^2/s over 600 s."""
    u = uniform(seed, 100, index + 1)[index]
    target = n_min * float(det_exp(u * np.sqrt(u) * det_log(n_max / n_min)))   # uneven, skewed to small members
    aspect = uniform(seed, 101, index + 1, 0.5, 2.0)[index]
    ny = max(8, int(round(np.sqrt(target / 2.0 / aspect))))
    nx = max(8, int(round(target / 2.0 / ny)))
    peak = float(uniform(seed, 102, index + 1, 2.0, 15.0)[index])
    lx, ly = 2.0 * nx, 2.0 * ny
    nbumps = max(1, int(round(8.0 * lx * ly / 2.0e6)))
    c = flooding(nx, ny, seed=seed * 1000 + index, lx=lx, ly=ly, iflux=iflux, q0=2.0, q1=peak, nbumps=nbumps,
                 bump_scale=min(1.0, float(np.sqrt(lx * ly / 2.0e6))))
    c.name = f"member_{index}_{nx}x{ny}"
    return c


def calibration(nx: int = 500, ny: int = 200, seed: int = 4, nzones: int = 12, ngauges: int = 40,
                iflux: int = 1):
    """Manning calibration case: the circular dam break's bed and boundaries (flat bed z = 0,
    reflective walls) on an nx x ny quad grid at 2 m spacing (500x200 -> 200,000 triangles over
    1000 m x 400 m), h = 10 m inside a circle of radius a quarter of the shorter side centred in
    the domain and 1 m outside, u = v = 0; a true Manning field piecewise constant over
    ``nzones`` Voronoi zones of seeded sites with n ~ U(0.02, 0.06), and ``ngauges`` seeded gauge
    elements drawn uniformly over the mesh.  The dam-break wave crosses the whole domain within
    the calibration run, so the flow, and with it the friction of every zone, reaches the gauges.

    First-order HLLC by default: over thousands of steps the gauge misfit of the WAF scheme is
    not a differentiable function of n (its limiters jump when the local depth difference
    changes sign, superbee also at r = 0.5, 1, 2), while the first-order one is, so gradients
    and finite differences agree.

    Returns (case with the true field, zones [nelt] zone id of every element, true zone values
    [nzones], gauges [ngauges] element ids)."""
    lx, ly = 2.0 * nx, 2.0 * ny
    c = circular_dam_break(nx, ny, seed=seed, lx=lx, ly=ly, iflux=iflux)
    xc, yc = cell_centroids(c.x, c.y, c.tri)
    sx = uniform(seed, 30, nzones, 0.0, lx)
    sy = uniform(seed, 31, nzones, 0.0, ly)
    zones = np.argmin((xc[:, None] - sx[None, :]) ** 2 + (yc[:, None] - sy[None, :]) ** 2, axis=1).astype(np.int32)
    nz = uniform(seed, 32, nzones, 0.02, 0.06)
    c.manning = nz[zones]
    pick = np.floor(uniform(seed, 33, ngauges, 0.0, 1.0) * c.nelt).astype(np.int64)
    gauges = np.unique(pick)
    k = 34
    while gauges.size < ngauges:      # draw again on collisions
        extra = np.floor(uniform(seed, k, ngauges, 0.0, 1.0) * c.nelt).astype(np.int64)
        gauges = np.unique(np.concatenate([gauges, extra]))[:ngauges]
        k += 1
    c.name = f"calibration_{nx}x{ny}"
    return c, zones, nz, gauges.astype(np.int32)


def observation_steps(t_start: np.ndarray, dt: np.ndarray, every: float) -> np.ndarray:
    """Indices k of the steps after which an observation is taken: the first step whose end
    time t_start[k] + dt[k] reaches each multiple of ``every``."""
    t_end = t_start + dt
    marks = np.arange(every, t_end[-1] + 1e-9, every)
    return np.searchsorted(t_end, marks - 1e-9).astype(np.int64)
