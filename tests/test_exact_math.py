"""The GPU kernels' float emulation of the reference's double-rounded per-pixel steps
(cbclib_v2_gb300/csrc/exact.cuh) is compiled here as host C and compared bit for bit
with the oracle on random and adversarial inputs."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, 'cbclib_v2_gb300', 'csrc')


@pytest.fixture(scope='module')
def exact(tmp_path_factory):
    out = str(tmp_path_factory.mktemp('exact') / 'libexact_host.so')
    subprocess.run(['gcc', '-O2', '-std=c11', '-ffp-contract=off', '-fPIC', '-shared',
                    '-I', CSRC, os.path.join(ROOT, 'tests', 'native', 'exact_host.c'),
                    '-o', out, '-lm'], check=True)
    lib = ctypes.CDLL(out)
    P = ctypes.c_void_p
    lib.exact_profile_batch.argtypes = [ctypes.c_int, P, P, ctypes.c_int64]
    lib.exact_pixel_error_batch.argtypes = [P] * 5 + [ctypes.c_int64]
    lib.exact_pixel_error_r_batch.argtypes = [P] * 5 + [ctypes.c_int64]
    lib.exact_div_batch.argtypes = [P] * 3 + [ctypes.c_int64]
    lib.exact_ddiv_batch.argtypes = [P] * 3 + [ctypes.c_int64]
    lib.exact_normal_error3_batch.argtypes = [P] * 5 + [ctypes.c_int64, ctypes.c_int]
    lib.exact_take_slow_count.restype = ctypes.c_longlong
    return lib


@pytest.fixture(scope='module')
def olib():
    lib = oracle._load()
    P = ctypes.c_void_p
    lib.cbc_oracle_profile_batch_f32.argtypes = [ctypes.c_int, P, P, ctypes.c_int64]
    lib.cbc_oracle_pixel_error_batch_f32.argtypes = [P] * 5 + [ctypes.c_int64]
    return lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _xs(rng, n):
    near_one = np.arange(np.float32(0.9995).view(np.uint32), np.float32(1.0).view(np.uint32) + 1,
                         dtype=np.uint32).view(np.float32)
    return [rng.random(n, dtype=np.float32),
            np.sqrt(rng.random(n, dtype=np.float32)),
            (rng.random(n, dtype=np.float32) ** 8).astype(np.float32),
            (1 - rng.random(n, dtype=np.float32) * 1e-3).astype(np.float32),
            near_one, np.array([0.0, 1.0, 0.5, 1e-30, 1e-12], np.float32)]


@pytest.mark.parametrize("kernel", list(oracle.KERNELS))
def test_profiles_bit_exact(exact, olib, kernel):
    rng = np.random.default_rng(11)
    k = oracle.KERNELS[kernel]
    for x in _xs(rng, 400_000):
        x = np.ascontiguousarray(x)
        a = np.empty_like(x)
        b = np.empty_like(x)
        olib.cbc_oracle_profile_batch_f32(k, _p(x), _p(a), x.size)
        exact.exact_profile_batch(k, _p(x), _p(b), x.size)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("mode", ['body', 'caps', 'near_line'])
def test_pixel_error_bit_exact(exact, olib, mode):
    rng = np.random.default_rng({'body': 1, 'caps': 2, 'near_line': 3}[mode])
    m = 600_000
    ln = (rng.random(m) * 100 + 0.01).astype(np.float32)
    w = (rng.random(m) * 6 + 0.05).astype(np.float32)
    te = ((rng.random(m) * 1.4 - 0.2) * ln * ln).astype(np.float32)
    ne = ((rng.random(m) * 2 - 1) * w * ln * 1.2).astype(np.float32)
    if mode == 'caps':
        te = (ln * ln + (rng.random(m) * 2 - 1) * w * ln).astype(np.float32)
    if mode == 'near_line':
        ne = (ne * 1e-3).astype(np.float32)
        te = ((rng.random(m) * 2 - 1) * w * ln).astype(np.float32)
    a = np.empty(m, np.float32)
    b = np.empty(m, np.float32)
    c = np.empty(m, np.float32)
    olib.cbc_oracle_pixel_error_batch_f32(_p(te), _p(ne), _p(ln), _p(w), _p(a), m)
    exact.exact_pixel_error_batch(_p(te), _p(ne), _p(ln), _p(w), _p(b), m)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    exact.exact_pixel_error_r_batch(_p(te), _p(ne), _p(ln), _p(w), _p(c), m)
    fast = c != -1.0
    assert fast.mean() > 0.99
    assert np.array_equal(a[fast].view(np.uint32), c[fast].view(np.uint32))


def test_reciprocal_division(exact):
    """Markstein's correction from a correctly rounded reciprocal gives the IEEE
    quotient; outside [2^-60, 2^60] the helper defers to the IEEE division."""
    rng = np.random.default_rng(17)
    n = 2_000_000
    ea = rng.integers(-70, 70, n).astype(np.float32)
    eb = rng.integers(-59, 59, n).astype(np.float32)
    a = (rng.uniform(1, 2, n) * 2.0**ea * rng.choice([-1, 1], n)).astype(np.float32)
    b = (rng.uniform(1, 2, n) * 2.0**eb).astype(np.float32)
    a[:100] = 0.0
    got = np.empty(n, np.float32)
    exact.exact_div_batch(_p(a), _p(b), _p(got), n)
    want = a / b
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all()


def test_reciprocal_division_double(exact):
    """the double form: the IEEE quotient for b in [2^-400, 2^400], including quotients
    next to rounding ties (a = b * q + a tiny remainder)"""
    rng = np.random.default_rng(18)
    n = 2_000_000
    ea = rng.integers(-420, 420, n).astype(np.float64)
    eb = rng.integers(-399, 399, n).astype(np.float64)
    a = rng.uniform(1, 2, n) * 2.0 ** ea * rng.choice([-1, 1], n)
    b = rng.uniform(1, 2, n) * 2.0 ** eb
    a[:100] = 0.0
    # near ties: a = b * (q + half an ulp of q), rounded
    m = n // 4
    q = rng.uniform(1, 2, m)
    b[-m:] = rng.uniform(1, 2, m) * 2.0 ** rng.integers(-50, 50, m)
    a[-m:] = b[-m:] * (q + np.spacing(q) / 2)
    got = np.empty(n)
    exact.exact_ddiv_batch(_p(a), _p(b), _p(got), n)
    with np.errstate(over='ignore', under='ignore'):
        want = a / b
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


@pytest.mark.parametrize("kernel", ['biweight', 'gaussian', 'parabolic'])
def test_profiles_rarely_leave_fast_path(exact, kernel):
    """the float pair path decides all but a tiny fraction of random inputs (the double
    fallback is for near-ties only)"""
    rng = np.random.default_rng(5)
    x = np.ascontiguousarray(rng.random(1_000_000, dtype=np.float32))
    out = np.empty_like(x)
    exact.exact_take_slow_count()
    exact.exact_profile_batch(oracle.KERNELS[kernel], _p(x), _p(out), x.size)
    assert exact.exact_take_slow_count() < 1000     # under 0.1 %


def test_pixel_error_rarely_leaves_fast_path(exact):
    rng = np.random.default_rng(6)
    m = 1_000_000
    ln = (rng.random(m) * 100 + 1).astype(np.float32)
    w = (rng.random(m) * 6 + 0.5).astype(np.float32)
    te = (ln * ln + (rng.random(m) * 2 - 1) * w * ln).astype(np.float32)   # end caps
    ne = ((rng.random(m) * 2 - 1) * w * ln).astype(np.float32)
    out = np.empty_like(te)
    exact.exact_take_slow_count()
    exact.exact_pixel_error_r_batch(_p(te), _p(ne), _p(ln), _p(w), _p(out), m)
    assert exact.exact_take_slow_count() < 1000     # under 0.1 %


def _normal_error3_ref(n0, n1, n2, ln):
    """the reference's float accumulator: err += std::pow(ne / len, 2) through double"""
    err = np.zeros(ln.shape, np.float32)
    for ne in (n0, n1, n2):
        b = (ne / ln).astype(np.float32)
        err = (err.astype(np.float64) + b.astype(np.float64) ** 2).astype(np.float32)
    return err


@pytest.mark.parametrize("mode", ['body', 'near_axis', 'wide'])
def test_normal_error3_bit_exact(exact, mode):
    """the three-pair normal error of 3-D positions, float(double(err) + b^2) per pair,
    from float pairs with a double fallback near ties"""
    rng = np.random.default_rng({'body': 21, 'near_axis': 22, 'wide': 23}[mode])
    m = 1_000_000
    ln = (rng.random(m) * 100 + 0.01).astype(np.float32)
    w = (rng.random(m) * 6 + 0.05).astype(np.float32)
    ns = [((rng.random(m) * 2 - 1) * w * ln * 1.2).astype(np.float32) for _ in range(3)]
    if mode == 'near_axis':
        ns[1] = (ns[1] * 1e-4).astype(np.float32)
        ns[2][: m // 4] = 0.0
    if mode == 'wide':
        e = rng.integers(-40, 40, (3, m))
        ns = [(ns[k] * 2.0 ** e[k]).astype(np.float32) for k in range(3)]
    want = _normal_error3_ref(*ns, ln)
    for use_r in (0, 1):
        got = np.empty(m, np.float32)
        exact.exact_take_slow_count()
        exact.exact_normal_error3_batch(_p(ns[0]), _p(ns[1]), _p(ns[2]), _p(ln), _p(got), m,
                                        use_r)
        slow = exact.exact_take_slow_count()
        fast = got != -1.0 if use_r else np.ones(m, bool)
        assert fast.mean() > 0.99
        assert np.array_equal(want[fast].view(np.uint32), got[fast].view(np.uint32))
        if mode == 'body':
            assert slow < 2 * m // 1000     # under 0.1 % of the two accumulations


def test_normal_error3_ties(exact):
    """second squares of exactly half an ulp of the accumulator (and one float either
    side): the double sum sits on or next to a float rounding boundary"""
    rng = np.random.default_rng(24)
    m = 200_000
    n0 = (rng.random(m) * 50 + 0.5).astype(np.float32)
    err0 = (n0.astype(np.float64) ** 2).astype(np.float32)
    e = np.frexp(err0)[1].astype(np.int64) - 1            # err0 in [2^e, 2^(e+1))
    keep = (e - 24) % 2 == 0
    n0, e = n0[keep], e[keep]
    half = np.ldexp(np.float32(1.0), ((e - 24) // 2).astype(np.int32)).astype(np.float32)
    n1 = np.concatenate([half, np.nextafter(half, np.float32(0)),
                         np.nextafter(half, np.float32(np.inf))]).astype(np.float32)
    n0 = np.concatenate([n0] * 3)
    n2 = np.zeros_like(n0)
    ln = np.ones_like(n0)
    want = _normal_error3_ref(n0, n1, n2, ln)
    got = np.empty_like(want)
    exact.exact_normal_error3_batch(_p(n0), _p(n1), _p(n2), _p(ln), _p(got), n0.size, 1)
    assert np.array_equal(want.view(np.uint32), got.view(np.uint32))
