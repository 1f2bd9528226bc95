"""The allocation-free product entry point (bse_op_matmul_device_noalloc).

It serves callers that cannot call cudaMalloc when they need a product (device
memory owned by another component's pool, or no allocation-induced
synchronisation allowed inside a pipelined solve).  Checked through the C ABI
against the ordinary device entry point, on two calls in a row (the static
scratch keeps the previous call's contents), and for the size limit.  This
file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-11  # same FP64 arithmetic, possibly different split-K summation order


def _ctx(v, c, naux, nmo, seed, precision=0, offdiag_hqp=False):
    from votca_gb300 import bse_operator as bo
    from votca_gb300.synthetic import Problem

    p = Problem(v=v, c=c, naux=naux, nmo=nmo, seed=seed)
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
    hqp = p.hqp
    if offdiag_hqp:  # symmetric off-diagonal couplings within the occupied and virtual blocks
        g = 0.05 * np.random.default_rng(seed + 100).standard_normal(hqp.shape)
        g[:v, v:] = 0.0
        g[v:, :v] = 0.0
        hqp = hqp + g + g.T
    return bo.GpuBSEContext(p.w, bo.TCMatrix_gwbse(p.mmn), hqp, opt, precision=precision)


def _products(ctx, coef, k, pad=0, ref_ctx=None):
    """The ordinary device product (on ref_ctx, default ctx) and two allocation-free products in a
    row, on buffers with leading dimension dim + pad whose padding rows hold a sentinel."""
    import torch

    from votca_gb300 import _lib

    L = _lib.load()
    dim = ctx.size
    ld = dim + pad
    X = torch.from_numpy(np.random.default_rng(4).standard_normal((k, ld))).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    Yref = torch.full_like(X, 7.0)
    rc = ref_ctx if ref_ctx is not None else ctx
    _lib.check(L.bse_op_matmul_device(rc.handle, *coef, ctypes.c_void_p(X.data_ptr()), ld, k,
                                      ctypes.c_void_p(Yref.data_ptr()), ld, stream))
    outs = []
    for _ in range(2):
        Y = torch.full_like(X, 7.0)
        Y[:, :dim] = float("nan")
        _lib.check(L.bse_op_matmul_device_noalloc(ctx.handle, *coef, ctypes.c_void_p(X.data_ptr()), ld, k,
                                                  ctypes.c_void_p(Y.data_ptr()), ld, stream))
        torch.cuda.synchronize()
        outs.append(Y.cpu().numpy())
    return Yref.cpu().numpy(), outs, dim


@pytest.mark.parametrize("coef", [(1, 2, 1, 0), (1, 0, 1, 0), (0, 2, 0, 1), (1, 0, 0, 0)])
def test_noalloc_matches_device_entry_point_twice(coef):
    import torch

    from votca_gb300 import _lib

    L = _lib.load()
    ctx = _ctx(8, 64, 256, 72, seed=1)
    dim, k = ctx.size, 11
    X = torch.from_numpy(np.random.default_rng(4).standard_normal((k, dim))).cuda()
    Yref = torch.empty_like(X)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(L.bse_op_matmul_device(ctx.handle, *coef, ctypes.c_void_p(X.data_ptr()), dim, k,
                                      ctypes.c_void_p(Yref.data_ptr()), dim, ctypes.c_void_p(stream)))
    outs = []
    for _ in range(2):
        Y = torch.full_like(X, float("nan"))
        _lib.check(L.bse_op_matmul_device_noalloc(ctx.handle, *coef, ctypes.c_void_p(X.data_ptr()), dim, k,
                                                  ctypes.c_void_p(Y.data_ptr()), dim, ctypes.c_void_p(stream)))
        torch.cuda.synchronize()
        outs.append(Y.cpu().numpy())
    ref = Yref.cpu().numpy()
    for y in outs:
        assert np.all(np.isfinite(y))
        assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < TOL


def test_noalloc_rejects_requests_beyond_the_scratch():
    import torch

    from votca_gb300 import _lib

    L = _lib.load()
    ctx = _ctx(4, 16, 64, 20, seed=2)
    dim = ctx.size
    k = (7 << 20) // 64 + 1  # Naux * k just above the static scratch
    X = torch.zeros((k, dim), dtype=torch.float64, device="cuda")
    Y = torch.zeros_like(X)
    rc = L.bse_op_matmul_device_noalloc(ctx.handle, 0, 1, 0, 0, ctypes.c_void_p(X.data_ptr()), dim, k,
                                        ctypes.c_void_p(Y.data_ptr()), dim, None)
    assert rc == 1
    assert b"static scratch" in L.bse_last_error()


@pytest.mark.parametrize("case", ["offdiag_hqp", "hd_chunks", "mixed_handle", "padded_ld"])
def test_noalloc_paths(case):
    """The branches a single small problem does not reach: Hqp with off-diagonal couplings (its
    two GEMMs), an Hd intermediate larger than the scratch holds for all columns (several column
    chunks), a handle created in split precision (the product is still FP64), and leading
    dimensions larger than the operator (padding rows left untouched)."""
    coefs = [(1, 2, 1, 0), (0, 2, 0, 1)]
    if case == "offdiag_hqp":
        ctx, k, pad, ref = _ctx(8, 64, 256, 72, seed=5, offdiag_hqp=True), 9, 0, None
        coefs = [(1, 2, 1, 0), (1, 0, 0, 0)]
    elif case == "hd_chunks":
        # Naux v c = 2^20 doubles per column: 7 columns per chunk of the 56 MiB region, 11 columns
        ctx, k, pad, ref = _ctx(16, 128, 512, 150, seed=6), 11, 0, None
        coefs = [(1, 2, 1, 0), (1, 0, 1, 0)]
    elif case == "mixed_handle":
        ctx = _ctx(8, 64, 256, 72, seed=7, precision=1)
        ref, k, pad = _ctx(8, 64, 256, 72, seed=7), 5, 0
    else:
        ctx, k, pad, ref = _ctx(8, 64, 256, 72, seed=8), 6, 3, None
    for coef in coefs:
        yref, outs, dim = _products(ctx, coef, k, pad, ref)
        for y in outs:
            assert np.all(np.isfinite(y[:, :dim]))
            err = np.linalg.norm(y[:, :dim] - yref[:, :dim]) / np.linalg.norm(yref[:, :dim])
            assert err < TOL, (case, coef, err)
            if pad:
                assert np.all(y[:, dim:] == 7.0), "padding rows were written"
