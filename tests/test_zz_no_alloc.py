"""The allocation-free radix sort (sx_radix_sort_pairs_noalloc), for callers
that cannot allocate device memory when they sort -- hosts whose device memory
belongs to another allocator with a fixed budget, or loops that cannot take the
synchronisation a cudaMalloc may cause.  It is called through the C ABI and
compared with the workspace-taking sort on calls in a row (each call reuses the
library's fixed scratch array as the previous one left it).  The cases cover
even and odd pass counts (an odd count ends in the scratch array and copies
back), keys with bits set above `bits` (they take no part in the order), and
the claim that the call allocates nothing (free device memory unchanged)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 18


def _keys(n, bits, seed, high_bits=False):
    rng = np.random.default_rng(seed)
    k = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    if not high_bits and bits < 32:
        k &= np.uint32((1 << bits) - 1)
    k[: n // 3] = k[n // 3: 2 * (n // 3)]   # repeated keys: the sort must stay stable
    return k


@pytest.mark.parametrize("cases", [[(200003, 30, False), (MAX_KEYS, 32, False)],
                                   [(MAX_KEYS, 20, True), (150001, 8, True), (77777, 17, False)]])
def test_noalloc_sort_matches_workspace_sort(pkg, cases):
    from starlab_physics_gb300 import _lib

    L = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    for call, (n, bits, high) in enumerate(cases):
        keys = _keys(n, bits, seed=call, high_bits=high)
        vals = np.arange(n, dtype=np.int32)
        k_ws = torch.from_numpy(keys.view(np.int32)).cuda()
        v_ws = torch.from_numpy(vals).cuda()
        k_na, v_na = k_ws.clone(), v_ws.clone()
        ws = torch.empty(int(L.sx_radix_sort_workspace_bytes(n)), dtype=torch.uint8, device="cuda")
        assert L.sx_radix_sort_pairs(k_ws.data_ptr(), v_ws.data_ptr(), n, bits, ws.data_ptr(), ws.numel(),
                                     stream) == 0
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.sx_radix_sort_pairs_noalloc(k_na.data_ptr(), v_na.data_ptr(), n, bits, stream)
        assert rc == 0, L.sx_last_error()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before, "the no-alloc sort changed free device memory"
        assert torch.equal(k_na, k_ws) and torch.equal(v_na, v_ws)       # integer outputs: exact
        masked = keys & np.uint32((1 << bits) - 1) if bits < 32 else keys
        order = np.argsort(masked, kind="stable")
        assert np.array_equal(v_na.cpu().numpy(), order)
        assert np.array_equal(k_na.cpu().numpy().view(np.uint32), keys[order])


def test_noalloc_sort_rejects_oversize(pkg):
    from starlab_physics_gb300 import _lib

    L = _lib.load()
    k = torch.zeros(MAX_KEYS + 1, dtype=torch.int32, device="cuda")
    v = torch.zeros_like(k)
    rc = L.sx_radix_sort_pairs_noalloc(k.data_ptr(), v.data_ptr(), MAX_KEYS + 1, 30,
                                       torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.SX_ERR_ARG
    assert b"capacity" in L.sx_last_error()
