"""The allocation-free DVC entry point (uwg_dvc_weights_noalloc), called through
the C ABI, gives the same weights and centroids as uwg_dvc_weights.

Callers of this entry point cannot allocate device memory where they need the
weights (during CUDA-graph capture, or under a framework that owns all device
memory), so it keeps its scratch in a fixed device array.  Two calls in a row
check that the shared array's leftover contents from the first call do not
leak into the second.  Collected last (file name) so a stop-at-first-failure
run has run everything else first."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(dim, res, ppc, seed):
    from underworld2_gb300._core import Context, rng_seed
    c = Context(dim, res, (0.0,) * dim, (1.0,) * dim)
    x, owner, off, lst, _ = c.layout_random(ppc, rng_seed(seed))
    ip_xi = c.pic_map(x, off, lst)
    return c, off, ip_xi


def test_noalloc_matches_context_entry_point(gpu):
    from underworld2_gb300 import _native
    lib = _native.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    for dim, res, ppc, seed, grid in [(3, (6, 5, 4), 9, 5, 15), (2, (17, 11), 23, 8, 12)]:
        c, off, ip_xi = _case(dim, res, ppc, seed)
        xi_ref = ip_xi.clone()
        w_ref = c.dvc_weights(off, xi_ref, res=grid)
        xi = ip_xi.clone()
        w = torch.full_like(w_ref, -1.0)
        rc = lib.uwg_dvc_weights_noalloc(dim, grid, c.n_el, p(off), p(xi), p(w), stream)
        assert rc == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(w.cpu().numpy(), w_ref.cpu().numpy())
        np.testing.assert_array_equal(xi.cpu().numpy(), xi_ref.cpu().numpy())


def test_noalloc_rejects_bad_sizes(gpu):
    from underworld2_gb300 import _native
    lib = _native.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    off = torch.tensor([0, 1], dtype=torch.int32, device="cuda")
    xi = torch.zeros((1, 3), dtype=torch.float64, device="cuda")
    w = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.uwg_dvc_weights_noalloc(3, 17, 1, p(off), p(xi), p(w), stream) == -1   # res > 16
    assert lib.uwg_dvc_weights_noalloc(4, 8, 1, p(off), p(xi), p(w), stream) == -1
