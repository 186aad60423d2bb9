"""sky_sort_pairs_noalloc, the sort entry point for callers that cannot let
the library allocate device memory (a host whose own pool or caching
allocator owns the GPU, or code that must not call cudaMalloc mid-work): it
must return exactly what sky_sort_pairs returns, on two calls in a row (its
one shared scratch array keeps the previous call's contents), and reject
sizes above its fixed maximum.  Collected last so that a failure here comes
after every other test has run; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def as_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def run(sky, fn, keys, vals, bits):
    kin = as_dev(keys)
    vin = as_dev(vals) if vals is not None else None
    kout = torch.empty_like(kin)
    vout = torch.empty_like(kin)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    sky._lib.check(getattr(sky.lib(), fn)(ptr(kin), ptr(vin), ptr(kout), ptr(vout), keys.size,
                                          bits, stream))
    torch.cuda.synchronize()
    return kout.cpu().numpy().view(np.uint32), vout.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_sky_sort_pairs_twice(sky):
    rng = np.random.default_rng(2024)
    cases = [
        (rng.integers(0, 2**32, 1_000_000, dtype=np.uint64).astype(np.uint32),
         rng.integers(0, 2**32, 1_000_000, dtype=np.uint64).astype(np.uint32), 32),
        (((rng.integers(0, 8160, 300_001) << 16) | rng.integers(2, 7, 300_001)).astype(np.uint32),
         None, 29),
        # exactly the maximum (256 full tiles of 4096 keys), a key width that
        # is not a multiple of 8, with values
        (rng.integers(0, 2**32, 1 << 20, dtype=np.uint64).astype(np.uint32),
         rng.integers(0, 2**32, 1 << 20, dtype=np.uint64).astype(np.uint32), 23),
    ]
    for keys, vals, bits in cases:        # two calls in a row through one scratch array
        k_ref, v_ref = run(sky, "sky_sort_pairs", keys, vals, bits)
        k_na, v_na = run(sky, "sky_sort_pairs_noalloc", keys, vals, bits)
        assert np.array_equal(k_na, k_ref) and np.array_equal(v_na, v_ref)
        order = np.argsort(keys & np.uint32(0xFFFFFFFF if bits == 32 else (1 << bits) - 1),
                           kind="stable")
        assert np.array_equal(k_na, keys[order])


def test_noalloc_sort_rejects_sizes_above_its_maximum(sky):
    L = sky.lib()
    n = (1 << 20) + 1
    x = torch.zeros(n, dtype=torch.int32, device="cuda")
    y = torch.zeros(n, dtype=torch.int32, device="cuda")
    z = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = L.sky_sort_pairs_noalloc(ptr(x), None, ptr(y), ptr(z), n, 32, None)
    assert rc == sky._lib.SKY_ERR_ARG
    assert b"SKY_SORT_NOALLOC_MAX_KEYS" in L.sky_last_error()
