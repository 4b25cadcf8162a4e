"""Integer-pipe FP64 <-> FP32 conversions of the complex64 kernels against the
hardware conversions: bit-identical in the normal float range (round half to
even included), signed zero below 2^-126, inf on overflow, NaN kept."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(x):
    from effmass_gb300 import build
    from effmass_gb300._lib import load
    build.build()
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = x.size
    fb, fh = np.empty(n, np.float32), np.empty(n, np.float32)
    db, dh = np.empty(n), np.empty(n)
    rc = load().hpsi_selftest_convert(x.ctypes.data_as(C.POINTER(C.c_double)), n, fb.ctypes.data, fh.ctypes.data,
                                      db.ctypes.data, dh.ctypes.data)
    assert rc == 0
    return fb, fh, db, dh


def _cases():
    rng = np.random.default_rng(7)
    parts = [
        rng.standard_normal(200_000) * 10.0 ** rng.uniform(-30, 30, 200_000),
        # random bit patterns over the whole double range
        rng.integers(0, 1 << 63, 200_000, dtype=np.uint64).view(np.float64),
    ]
    # exact ties and neighbours: float32 values plus half an ulp, +- one double ulp
    f = (rng.standard_normal(50_000) * 10.0 ** rng.uniform(-20, 20, 50_000)).astype(np.float32).astype(np.float64)
    half = np.abs(f) * 2.0 ** -24
    tie = f + half
    parts += [tie, np.nextafter(tie, np.inf), np.nextafter(tie, -np.inf)]
    # range edges
    edges = np.array([0.0, -0.0, 2.0 ** -126, -(2.0 ** -126), 2.0 ** -127, 2.0 ** -150, np.finfo(np.float32).max,
                      -float(np.finfo(np.float32).max), 3.5e38, 1e300, -1e300, np.inf, -np.inf, np.nan, 1.0, -1.0])
    parts.append(edges)
    return np.concatenate(parts)


def test_double_to_float_and_back():
    x = _cases()
    fb, fh, db, dh = _run(x)
    finite = np.isfinite(x)
    normal_range = finite & (np.abs(fh) >= np.float32(2.0 ** -126))
    assert np.array_equal(fb[normal_range].view(np.uint32), fh[normal_range].view(np.uint32))
    # overflow and infinities
    big = finite & np.isinf(fh)
    assert np.array_equal(fb[big], fh[big])
    assert np.array_equal(fb[np.isinf(x)], fh[np.isinf(x)])
    assert np.isnan(fb[np.isnan(x)]).all()
    # below the normal float range: signed zero (the hardware may give a subnormal)
    tiny = finite & (np.abs(fh) < np.float32(2.0 ** -126))
    assert (np.abs(fb[tiny]) <= np.float32(2.0 ** -126)).all()
    assert np.array_equal(np.signbit(fb[tiny & (fb == 0)]), np.signbit(x[tiny & (fb == 0)]))
    # float -> double: exact for normal floats, inf and NaN
    ok = np.isfinite(fh) & (np.abs(fh) >= np.float32(2.0 ** -126)) | np.isinf(fh)
    assert np.array_equal(db[ok], dh[ok])
    assert np.isnan(db[np.isnan(fh)]).all()
    sub = np.isfinite(fh) & (np.abs(fh) < np.float32(2.0 ** -126))
    assert (db[sub] == 0).all()
