"""The allocation-free DVC entry point (uwg_dvc_weights_noalloc), called through
the C ABI, gives the same weights and centroids as uwg_dvc_weights.

Callers of this entry point cannot allocate device memory where they need the
weights (a host framework that keeps all device memory in its own pool, or a
plugin host that gives out buffers but no allocator), so it keeps its scratch,
including its status word, in a fixed device array shared by every call.  The
tests make two calls in a row, and a failing call (an empty element) followed
by a valid one, to check that what one call leaves in the array does not leak
into the next.  Collected last (file name) so a stop-at-first-failure run has
run everything else first."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

UWG_ERR_ARG = -1
UWG_ERR_EMPTY_CELL = -4


def _case(dim, res, ppc, seed):
    from underworld2_gb300._core import Context, rng_seed
    c = Context(dim, res, (0.0,) * dim, (1.0,) * dim)
    x, owner, off, lst, _ = c.layout_random(ppc, rng_seed(seed))
    ip_xi = c.pic_map(x, off, lst)
    return c, off, ip_xi


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check_against_context(lib, dim, res, ppc, seed, grid):
    c, off, ip_xi = _case(dim, res, ppc, seed)
    xi_ref = ip_xi.clone()
    w_ref = c.dvc_weights(off, xi_ref, res=grid)
    xi = ip_xi.clone()
    w = torch.full_like(w_ref, -1.0)
    rc = lib.uwg_dvc_weights_noalloc(dim, grid, c.n_el, _ptr(off), _ptr(xi), _ptr(w), _stream())
    assert rc == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(w.cpu().numpy(), w_ref.cpu().numpy())
    np.testing.assert_array_equal(xi.cpu().numpy(), xi_ref.cpu().numpy())


def test_noalloc_matches_context_entry_point(gpu):
    from underworld2_gb300 import _native
    lib = _native.load()
    # two calls in a row on different meshes share the fixed scratch array
    for dim, res, ppc, seed, grid in [(3, (6, 5, 4), 9, 5, 15), (2, (17, 11), 23, 8, 12)]:
        _check_against_context(lib, dim, res, ppc, seed, grid)


def test_noalloc_error_then_valid_call(gpu):
    from underworld2_gb300 import _native
    lib = _native.load()
    # element 1 of 3 is empty: the call reports it ...
    off = torch.tensor([0, 2, 2, 4], dtype=torch.int32, device="cuda")
    xi = torch.tensor([[-0.5, 0.1], [0.4, -0.2], [0.0, 0.0], [0.3, 0.7]], dtype=torch.float64, device="cuda")
    w = torch.zeros(4, dtype=torch.float64, device="cuda")
    assert lib.uwg_dvc_weights_noalloc(2, 10, 3, _ptr(off), _ptr(xi), _ptr(w), _stream()) == UWG_ERR_EMPTY_CELL
    # ... and its error code, left in the shared status word, does not leak into the next call
    _check_against_context(lib, 2, (7, 9), 11, 3, 15)


def test_noalloc_rejects_bad_sizes(gpu):
    from underworld2_gb300 import _native
    lib = _native.load()
    off = torch.tensor([0, 1], dtype=torch.int32, device="cuda")
    xi = torch.zeros((1, 3), dtype=torch.float64, device="cuda")
    w = torch.zeros(1, dtype=torch.float64, device="cuda")
    s = _stream()
    assert lib.uwg_dvc_weights_noalloc(3, 17, 1, _ptr(off), _ptr(xi), _ptr(w), s) == UWG_ERR_ARG   # res > 16
    assert lib.uwg_dvc_weights_noalloc(4, 8, 1, _ptr(off), _ptr(xi), _ptr(w), s) == UWG_ERR_ARG    # dim 4
