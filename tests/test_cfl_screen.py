"""The element kernel's single-precision screening of the CFL minimum (k_cells, cfl_dt_f32): the
block minimum is exact only if the float value of every wet element lies within 7e-7 relative of
its FP64 value (the kernel selects elements within 4e-6 of the float minimum).  This restates the
float evaluation with numpy (float32 operations are correctly rounded, as __fdiv_rn / __fsqrt_rn
are) and checks the bound against the FP64 evaluation on adversarial inputs."""
import numpy as np


def _trunc_f32(x):
    b = np.asarray(x, dtype=np.float64).view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64) - 1023
    zero = (b << np.uint64(1)) == 0
    ok = ((e >= -126) & (e <= 127)) | zero
    sign = (b >> np.uint64(32)) & np.uint64(0x80000000)
    fb = (sign | (np.clip(e + 127, 0, 255).astype(np.uint64) << np.uint64(23))
          | ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)))
    fb = np.where(zero, sign, fb).astype(np.uint32)
    return fb.view(np.float32), ok


def _cfl_f64(L, h, hu, hv, g):
    vu, vv = hu / h, hv / h
    nv = np.sqrt(vu * vu + vv * vv)
    vmax = np.maximum(0.01, nv + np.sqrt(g * np.abs(h)))
    return np.minimum(L / vmax, 1e6)


def _cfl_f32(L, h, hu, hv, g):
    (hf, a), (huf, b), (hvf, c), (lf, d) = _trunc_f32(h), _trunc_f32(hu), _trunc_f32(hv), _trunc_f32(L)
    gf = _trunc_f32(np.array([g]))[0][0]
    with np.errstate(over="ignore", under="ignore"):
        vu, vv = huf / hf, hvf / hf
        nv = np.sqrt(vu * vu + vv * vv)
        cc = np.sqrt(gf * hf)
        vmax = np.maximum(np.float32(0.01), nv + cc)
        df = np.minimum(lf / vmax, np.float32(1e6))
    ok = a & b & c & d & (df > np.float32(1e-30)) & (df <= np.float32(1e6))
    return df.astype(np.float64), ok


def test_single_precision_cfl_is_within_the_screening_bound():
    rng = np.random.default_rng(5)
    n = 2_000_000
    g = 9.81
    h = 10.0 ** rng.uniform(-6, 2, n)
    vel = 10.0 ** rng.uniform(-12, 2, n) * rng.choice([-1.0, 1.0], n)
    hu = h * vel * rng.uniform(0.5, 1.5, n)
    hv = h * vel * rng.uniform(-1.5, 1.5, n)
    L = 10.0 ** rng.uniform(-2, 3, n)
    # significands near all-ones (the largest truncation errors)
    for arr in (h, hu, L):
        bits = arr[::5].view(np.uint64) | np.uint64((1 << 52) - (1 << 20))
        arr[::5] = bits.view(np.float64)
    hu[::7] = 0.0
    hv[::11] = 0.0
    exact = _cfl_f64(L, h, hu, hv, g)
    approx, ok = _cfl_f32(L, h, hu, hv, g)
    assert ok.mean() > 0.99
    rel = np.abs(approx[ok] - exact[ok]) / exact[ok]
    assert rel.max() <= 7e-7, rel.max()
    # the selection threshold covers both errors with room: (1 + 7e-7) / (1 - 7e-7) < 1.000004
    assert (1 + 7e-7) / (1 - 7e-7) * (1 + 2 ** -24) < 1.000004
