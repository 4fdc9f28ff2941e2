"""CPU checks of the ring-FFT planner (host code of the library, no GPU): every
ring length of the benchmark grids (L = 4 + 4 ri, complex length N = L/2 after
real packing, ri up to 1200) gets a direct Stockham plan or one Rader pass —
no Bluestein — whose radices multiply out to N, with direct prime passes only
up to the precision's limit and Rader inner convolutions zero-padded to a
smooth length exactly when p − 1 has a prime factor above the padding limit."""
import ctypes as C
import math

import pytest

import springsteel_gpu as S
from springsteel_gpu import abi


def _lpf(n):
    p, d = 1, 2
    while d * d <= n:
        while n % d == 0:
            p, n = max(p, d), n // d
        d += 1
    return max(p, n) if n > 1 else p


def _is_prime(n):
    return n > 1 and _lpf(n) == n


def _plan(lib, n, precision):
    info = abi.ss_fft_plan_info()
    assert lib.ss_fft_plan(n, precision, C.byref(info)) == abi.SS_OK
    return info


@pytest.mark.parametrize("precision", [abi.SS_PREC_F64, abi.SS_PREC_F32_REFINED, abi.SS_PREC_F64_FAST])
def test_every_ring_length_gets_a_direct_or_rader_plan(precision, monkeypatch):
    for var in ("SS_FFT_MAX_PRIME", "SS_FFT_RADER", "SS_FFT_RADER_PAD"):
        monkeypatch.delenv(var, raising=False)
    lib = S.load_library()
    kinds = {abi.FFT_DIRECT: 0, abi.FFT_RADER: 0, abi.FFT_BLUESTEIN: 0}
    for ri in range(1, 1201):
        n = 2 * (ri + 1)
        p = _plan(lib, n, precision)
        kinds[p.kind] += 1
        rad = list(p.rad[:p.nrad])
        assert math.prod(rad) == n, (n, rad)
        assert p.kind != abi.FFT_BLUESTEIN, (n, rad)
        limit = p.max_prime
        assert limit == (127 if precision == abi.SS_PREC_F32_REFINED else 67)
        direct = rad[1:] if p.kind == abi.FFT_RADER else rad
        for r in direct:
            assert r in (2, 3, 4, 5, 7, 11, 13) or (_is_prime(r) and r <= 199), (n, rad)
        if p.kind == abi.FFT_DIRECT:
            assert _lpf(n) <= limit, (n, rad)
            continue
        # one Rader pass for the largest prime factor, above the direct limit
        P = p.rader_p
        assert rad[0] == P == _lpf(n) and P > limit, (n, rad)
        inner = list(p.inner_rad[:p.inner_nrad])
        assert math.prod(inner) == p.rader_inner, (n, inner, p.rader_inner)
        if _lpf(P - 1) > p.pad_prime:
            # zero-padded: a smooth length that holds the linear convolution
            assert p.rader_inner >= 2 * (P - 1) - 1, (n, P, p.rader_inner)
            assert set(inner) <= {2, 3, 4, 5, 7}, (n, inner)
        else:
            assert p.rader_inner == P - 1, (n, P, p.rader_inner)
    assert kinds[abi.FFT_RADER] > 0 and kinds[abi.FFT_DIRECT] > 0


def test_padded_inner_length_is_the_smallest_smooth_one():
    lib = S.load_library()
    # ring ri = 382: N = 766 = 2 · 383, 382 = 2 · 191 → padded to 768 = 3 · 4^4
    p = _plan(lib, 766, abi.SS_PREC_F64)
    assert p.kind == abi.FFT_RADER and p.rader_p == 383 and p.rader_inner == 768
    # ri = 600: N = 1202 = 2 · 601, 600 = 2^3 · 3 · 5^2 → unpadded
    p = _plan(lib, 1202, abi.SS_PREC_F64)
    assert p.kind == abi.FFT_RADER and p.rader_p == 601 and p.rader_inner == 600


def test_tuning_overrides_change_the_plan(monkeypatch):
    lib = S.load_library()
    n = 2 * 61  # a direct 61-point pass by default (61 ≤ 67)
    assert _plan(lib, n, abi.SS_PREC_F64).kind == abi.FFT_DIRECT
    monkeypatch.setenv("SS_FFT_MAX_PRIME", "31")
    p = _plan(lib, n, abi.SS_PREC_F64)
    assert p.kind == abi.FFT_RADER and p.rader_p == 61 and p.max_prime == 31
    monkeypatch.setenv("SS_FFT_RADER", "0")
    p = _plan(lib, n, abi.SS_PREC_F64)
    assert p.kind == abi.FFT_BLUESTEIN and p.bluestein_m >= 2 * n - 1


def test_plan_rejects_bad_arguments():
    lib = S.load_library()
    info = abi.ss_fft_plan_info()
    assert lib.ss_fft_plan(0, abi.SS_PREC_F64, C.byref(info)) == abi.SS_BAD_ARG
    assert lib.ss_fft_plan(8, 7, C.byref(info)) == abi.SS_BAD_ARG
    assert lib.ss_fft_plan(8, abi.SS_PREC_F64, None) == abi.SS_BAD_ARG
