"""Known-answer and accuracy tests of the generator and of the portable FP64
functions that the replay kernels share with the CPU restatement.

Replay parity cannot catch an error in code that both sides compile, so these
pin it independently:
  * Philox-4x32-10 against the published known-answer vectors of Salmon et
    al., "Parallel random numbers: as easy as 1, 2, 3" (SC'11; the Random123
    distribution's kat_vectors), and against a plain Python restatement of
    the published round function on random counters and keys;
  * the portable exp / log / sin / cos against libm (Python's math module)
    and, where mpmath is importable, against correctly rounded values;
  * the portable Box-Muller pair against its formula.
The host forms run in the CPU suite; the device forms (the replay kernels'
and the MIXED kernel's round-key form) are checked on the GPU against the same
answers and, bit for bit, against the host forms.
"""
import ctypes as C
import math

import numpy as np
import pytest

from pdds_gb300 import _capi as capi

# counter (4 words), key (2 words) -> output (4 words)
PHILOX_KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF),
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85


def philox_py(ctr, key):
    """Philox-4x32-10 written out from the published round function."""
    c = list(ctr)
    k0, k1 = key
    for _ in range(10):
        p0, p1 = M0 * c[0], M1 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k0, p1 & 0xFFFFFFFF, (p0 >> 32) ^ c[3] ^ k1, p0 & 0xFFFFFFFF]
        k0, k1 = (k0 + W0) & 0xFFFFFFFF, (k1 + W1) & 0xFFFFFFFF
    return tuple(c)


def _u32(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _f64(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def lib_philox(device, form, ctr, key):
    L = capi.load()
    ctr = np.ascontiguousarray(ctr, np.uint32).reshape(-1)
    key = np.ascontiguousarray(key, np.uint32).reshape(-1)
    n = len(ctr) // 4
    out = np.zeros(4 * n, np.uint32)
    err = C.create_string_buffer(256)
    st = L.pdds_check_philox(device, form, _u32(ctr), _u32(key), n, _u32(out), err, 256)
    assert st == capi.OK, err.value
    return out.reshape(n, 4)


def lib_math(device, fn, x):
    L = capi.load()
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros_like(x)
    err = C.create_string_buffer(256)
    st = L.pdds_check_portable_math(device, fn, _f64(x), len(x), _f64(out), err, 256)
    assert st == capi.OK, err.value
    return out


def ulp_distance(a, b):
    """Distance in units in the last place between doubles (same sign side)."""
    ia = np.asarray(a, np.float64).view(np.int64)
    ib = np.asarray(b, np.float64).view(np.int64)
    ia = np.where(ia < 0, np.int64(-(2 ** 63)) - ia, ia)
    ib = np.where(ib < 0, np.int64(-(2 ** 63)) - ib, ib)
    return np.abs(ia - ib)


def kat_arrays():
    ctr = np.array([c for c, _, _ in PHILOX_KAT], np.uint32)
    key = np.array([k for _, k, _ in PHILOX_KAT], np.uint32)
    exp = np.array([o for _, _, o in PHILOX_KAT], np.uint32)
    return ctr, key, exp


def random_counters(n=256, seed=9):
    rng = np.random.default_rng(seed)
    ctr = rng.integers(0, 2 ** 32, size=(n, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2 ** 32, size=(n, 2), dtype=np.uint64).astype(np.uint32)
    exp = np.array([philox_py(tuple(int(v) for v in c), tuple(int(v) for v in k)) for c, k in zip(ctr, key)],
                   np.uint32)
    return ctr, key, exp


def sweep(name, n=20000, seed=3):
    rng = np.random.default_rng(seed)
    if name == "exp":
        return np.concatenate([rng.uniform(-1, 1, n), rng.uniform(-50, 50, n), rng.uniform(-700, 700, n // 4),
                               [0.0, -0.0, 1e-300, -1e-300, 709.0, -708.0]])
    if name == "log":
        return np.concatenate([rng.uniform(0.5, 2.0, n), np.exp(rng.uniform(-700, 700, n)),
                               rng.uniform(1e-12, 1.0, n // 4), [1.0, 2.0, 0.5, 1e-310, 1.7e308]])
    return np.concatenate([rng.uniform(-4, 4, n), rng.uniform(-1e5, 1e5, n), [0.0, math.pi / 4, math.pi / 2]])


FNS = [(capi.FN_EXP, "exp"), (capi.FN_LOG, "log"), (capi.FN_SIN, "sin"), (capi.FN_COS, "cos")]


# ------------------------------------------------------------------ host (CPU suite)
def test_python_restatement_matches_published_vectors():
    for ctr, key, out in PHILOX_KAT:
        assert philox_py(ctr, key) == out


def test_host_philox_known_answers():
    ctr, key, exp = kat_arrays()
    np.testing.assert_array_equal(lib_philox(-1, capi.PHILOX_PORTABLE, ctr, key), exp)
    ctr, key, exp = random_counters()
    np.testing.assert_array_equal(lib_philox(-1, capi.PHILOX_PORTABLE, ctr, key), exp)


@pytest.mark.parametrize("fn,name", FNS)
def test_host_portable_math_within_two_ulp_of_libm(fn, name):
    x = sweep(name)
    got = lib_math(-1, fn, x)
    ref = np.array([getattr(math, name)(v) for v in x])
    d = ulp_distance(got, ref)
    assert d.max() <= 2, (name, int(d.max()), x[np.argmax(d)])
    assert np.mean(d > 0) < 0.25


@pytest.mark.parametrize("fn,name", FNS)
def test_host_portable_math_against_correct_rounding(fn, name):
    mpmath = pytest.importorskip("mpmath")
    x = sweep(name, n=1500, seed=11)
    got = lib_math(-1, fn, x)
    with mpmath.workprec(160):
        ref = np.array([float(getattr(mpmath, name)(mpmath.mpf(float(v)))) for v in x])
    d = ulp_distance(got, ref)
    assert d.max() <= 2, (name, int(d.max()), x[np.argmax(d)])


def test_host_box_muller_formula():
    rng = np.random.default_rng(5)
    a = rng.integers(0, 2 ** 32, 5000, dtype=np.uint64)
    b = rng.integers(0, 2 ** 32, 5000, dtype=np.uint64)
    bits = (a | (b << np.uint64(32))).astype(np.uint64).view(np.float64)
    z0 = lib_math(-1, capi.FN_BOX_MULLER_Z0, bits)
    z1 = lib_math(-1, capi.FN_BOX_MULLER_Z1, bits)
    u0 = (a.astype(np.float64) + 0.5) * 2.0 ** -32
    u1 = (b.astype(np.float64) + 0.5) * 2.0 ** -32
    rho = np.sqrt(-2.0 * np.log(u0))
    np.testing.assert_allclose(z0, rho * np.cos(2 * np.pi * u1), rtol=0, atol=1e-13)
    np.testing.assert_allclose(z1, rho * np.sin(2 * np.pi * u1), rtol=0, atol=1e-13)


def test_check_entry_points_reject_bad_arguments():
    L = capi.load()
    err = C.create_string_buffer(128)
    z = np.zeros(8, np.uint32)
    assert L.pdds_check_philox(-1, 7, _u32(z), _u32(z), 1, _u32(z), err, 128) == capi.ERR_INVALID
    assert L.pdds_check_philox(-1, capi.PHILOX_ROUND_KEYS, _u32(z), _u32(z), 1, _u32(z), err, 128) == \
        capi.ERR_INVALID
    x = np.zeros(2)
    assert L.pdds_check_portable_math(-1, 99, _f64(x), 2, _f64(x), err, 128) == capi.ERR_INVALID


# ------------------------------------------------------------------ device
@pytest.mark.gpu
def test_device_philox_known_answers_both_forms():
    for ctr, key, exp in (kat_arrays(), random_counters(64)):
        for form in (capi.PHILOX_PORTABLE, capi.PHILOX_ROUND_KEYS):
            np.testing.assert_array_equal(lib_philox(0, form, ctr, key), exp)


@pytest.mark.gpu
@pytest.mark.parametrize("fn,name", FNS + [(capi.FN_BOX_MULLER_Z0, "bm0"), (capi.FN_BOX_MULLER_Z1, "bm1")])
def test_device_portable_math_equals_host_bit_for_bit(fn, name):
    if name.startswith("bm"):
        rng = np.random.default_rng(6)
        x = rng.integers(0, 2 ** 63, 20000, dtype=np.uint64).view(np.float64)
    else:
        x = sweep(name)
    dev = lib_math(0, fn, x)
    host = lib_math(-1, fn, x)
    assert np.array_equal(dev.view(np.int64), host.view(np.int64)), name
    if not name.startswith("bm"):
        ref = np.array([getattr(math, name)(v) for v in x])
        assert ulp_distance(dev, ref).max() <= 2
