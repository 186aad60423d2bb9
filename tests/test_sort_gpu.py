"""sky_sort_pairs (device-pointer onesweep sort) against numpy's stable sort:
sizes around the 4096-key tile, 1..32 key bits, ties, sorted and reversed
input, and the implicit (index) payload."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(a.view(np.int32)).cuda()


def sort_gpu(sky, keys, vals, bits):
    L = sky.lib()
    kin = dev(keys)
    vin = dev(vals) if vals is not None else None
    kout = torch.empty_like(kin)
    vout = torch.empty_like(kin)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.sky_sort_pairs(C.c_void_p(kin.data_ptr()), C.c_void_p(vin.data_ptr()) if vin is not None else None,
                          C.c_void_p(kout.data_ptr()), C.c_void_p(vout.data_ptr()), keys.size, bits,
                          C.c_void_p(stream))
    sky._lib.check(rc)
    torch.cuda.synchronize()
    return (kout.cpu().numpy().view(np.uint32), vout.cpu().numpy().view(np.uint32))


def expect(keys, vals, bits):
    mask = np.uint32(0xFFFFFFFF) if bits == 32 else np.uint32((1 << bits) - 1)
    order = np.argsort(keys & mask, kind="stable")
    v = vals if vals is not None else np.arange(keys.size, dtype=np.uint32)
    return keys[order], v[order]


@pytest.mark.parametrize("n", [1, 2, 31, 4095, 4096, 4097, 8191, 100_003, 1_000_000])
@pytest.mark.parametrize("bits", [8, 24, 29, 32])
def test_random_keys(sky, n, bits):
    rng = np.random.default_rng(n * 131 + bits)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    keys &= np.uint32(0xFFFFFFFF if bits == 32 else (1 << bits) - 1)
    vals = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    ko, vo = sort_gpu(sky, keys, vals, bits)
    ke, ve = expect(keys, vals, bits)
    assert np.array_equal(ko, ke) and np.array_equal(vo, ve)


@pytest.mark.parametrize("bits", [1, 3, 7, 9, 15, 17, 31])
def test_odd_bit_widths_ignore_high_bits(sky, bits):
    rng = np.random.default_rng(bits)
    n = 50_000
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    ko, vo = sort_gpu(sky, keys, vals, bits)
    ke, ve = expect(keys, vals, bits)
    assert np.array_equal(vo, ve) and np.array_equal(ko, ke)


@pytest.mark.parametrize("kind", ["equal", "few", "sorted", "reversed", "depth_like"])
def test_structured_inputs_stable(sky, kind):
    n = 300_000
    rng = np.random.default_rng(7)
    if kind == "equal":
        keys = np.full(n, 12345, np.uint32)
    elif kind == "few":
        keys = rng.integers(0, 5, n).astype(np.uint32)
    elif kind == "sorted":
        keys = np.sort(rng.integers(0, 2**24, n)).astype(np.uint32)
    elif kind == "reversed":
        keys = np.sort(rng.integers(0, 2**24, n))[::-1].astype(np.uint32).copy()
    else:   # tile << 16 | small integer depth, the intersection keys' shape
        keys = ((rng.integers(0, 8160, n) << 16) | rng.integers(2, 7, n)).astype(np.uint32)
    ko, vo = sort_gpu(sky, keys, None, 29)
    ke, ve = expect(keys, None, 29)
    assert np.array_equal(ko, ke) and np.array_equal(vo, ve)


def test_zero_length_and_bad_arguments(sky):
    L = sky.lib()
    assert L.sky_sort_pairs(None, None, None, None, 0, 8, None) == sky._lib.SKY_ERR_ARG
    x = torch.zeros(16, dtype=torch.int32, device="cuda")
    y = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = C.c_void_p(x.data_ptr())
    q = C.c_void_p(y.data_ptr())
    assert L.sky_sort_pairs(p, None, q, q, 0, 8, None) == 0
    assert L.sky_sort_pairs(p, None, p, q, 16, 8, None) == sky._lib.SKY_ERR_ARG
    assert L.sky_sort_pairs(p, None, q, q, 16, 33, None) == sky._lib.SKY_ERR_ARG
