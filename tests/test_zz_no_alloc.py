"""The allocation-free entry point, emt6_simulate_noalloc.

It exists for callers that cannot call cudaMalloc themselves (code inside a
host application or framework whose allocator owns all device memory): they
pass device buffers they already own and the library
keeps the working state in a fixed 8 MiB device array.  This file is
collected last so that a failure here does not hide the other tests; it must
pass alone in a fresh process as well as after them.

The check: its living counts equal those of the regular batch entry points
(emt6_batch_create / emt6_batch_run / emt6_batch_counts) exactly -- integer
counts, the same tolerance (none) as the other parity tests -- on two calls in
a row, and requests beyond the array's capacity are refused."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(N, params, tumors_dev, H, W, st_dev, sp_dev, n, doses_dev, bins, steps, seed,
          counts_dev, stream):
    return N.lib().emt6_simulate_noalloc(
        ctypes.byref(params.native), ctypes.c_void_p(tumors_dev.data_ptr()), H, W,
        ctypes.c_void_p(st_dev.data_ptr()), ctypes.c_void_p(sp_dev.data_ptr()), n,
        ctypes.c_void_p(doses_dev.data_ptr()), bins, 300, 144_000, steps, seed,
        ctypes.c_void_p(counts_dev.data_ptr()), ctypes.c_void_p(stream))


def test_noalloc_matches_batch_on_two_calls():
    import torch
    from emt6ro import _native as N
    from emt6ro import workloads as wl
    from emt6ro.batch import Batch

    params = wl.default_parameters()
    tumors = [wl.disc_tumor(params, 9, seed=1), wl.disc_tumor(params, 12, seed=2),
              wl.disc_tumor(params, 16, seed=3)]  # the last one needs the wide kernel
    prots = [[(300, 2.0)], [(0, 1.25), (900, 1.25)]]
    n, steps, seed = 30, 1500, 4242
    st = (np.arange(n) % 3).astype(np.int32)
    sp = ((np.arange(n) // 3) % 2).astype(np.int32)

    ref = Batch(params, tumors, prots, st, sp, seed=seed)
    ref.run(steps)
    expected = ref.counts()

    bins = ref.bins
    dev = torch.device("cuda:0")
    stack = np.ascontiguousarray(np.stack([t.sites for t in tumors]))
    tumors_dev = torch.from_numpy(stack.view(np.uint8).reshape(-1)).to(dev)
    st_dev = torch.from_numpy(st).to(dev)
    sp_dev = torch.from_numpy(sp).to(dev)
    doses_dev = torch.from_numpy(np.ascontiguousarray(ref.doses)).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    H, W = stack.shape[1], stack.shape[2]
    for _ in range(2):
        counts_dev = torch.full((n,), 0xFFFF, dtype=torch.int32, device=dev)
        rc = _call(N, params, tumors_dev, H, W, st_dev, sp_dev, n, doses_dev, bins, steps,
                   seed, counts_dev, stream)
        assert rc == 0, N.lib().emt6_last_error()
        got = counts_dev.cpu().numpy().astype(np.uint32)
        assert (got == expected).all(), (got, expected)


def test_noalloc_rejects_requests_beyond_capacity():
    import torch
    from emt6ro import _native as N
    from emt6ro import workloads as wl

    params = wl.default_parameters()
    t = wl.disc_tumor(params, 5, seed=1).sites
    dev = torch.device("cuda:0")
    n = 48  # 47 default-size simulations fit in 8 MiB
    tumors_dev = torch.from_numpy(np.ascontiguousarray(t).view(np.uint8).reshape(-1)).to(dev)
    z = torch.zeros(n, dtype=torch.int32, device=dev)
    doses_dev = torch.zeros(480, dtype=torch.float32, device=dev)
    counts_dev = torch.zeros(n, dtype=torch.int32, device=dev)
    rc = _call(N, params, tumors_dev, 53, 53, z, z, n, doses_dev, 480, 10, 1, counts_dev,
               torch.cuda.current_stream(dev).cuda_stream)
    assert rc == N.EMT6_ERR_LIMIT if hasattr(N, "EMT6_ERR_LIMIT") else rc == 5
    assert "at most 47 simulations" in N.lib().emt6_last_error().decode()
